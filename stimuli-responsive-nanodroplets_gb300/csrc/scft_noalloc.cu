/*
 * scft_noalloc.cu — the propagator unit entry point without device allocation.
 *
 * scft_propagate() allocates its working buffers with cudaMalloc on every call.
 * Some callers cannot do that: a host that has already handed the device's
 * memory to its own pools (a serving process sized to the card), code that must
 * not trigger the implicit device synchronisation cudaMalloc/cudaFree can
 * cause, or code that must not fail on an allocation in the middle of a run.
 * scft_propagate_static() gives them the same computation with its working
 * buffers in one file-scope device array of fixed size, which every GPU that
 * loads this library holds until the process exits.
 *
 * Set-up: the device address of the array is looked up with
 * cudaGetSymbolAddress the first time the entry point runs on a device (with
 * that device current) and kept for the life of the process, so a device reset
 * (cudaDeviceReset, or the primary context torn down and created again) after
 * that first call is not supported. The function synchronises its stream and
 * copies into pageable host memory, so it cannot be called inside a stream
 * capture. Every call on a device reuses the same array and leaves the
 * previous call's data in it; each call writes every byte it later reads, so
 * nothing needs to start at zero. Calls that overlap on the GPU (other threads,
 * other contexts on the same device) race on the array and must be serialised
 * by the caller; every return, on success or error, comes after the call's own
 * GPU work has finished.
 */
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <atomic>

#include "scft_internal.h"

/* 32 MiB of working space per device: enough for 100 FP64 contour steps (or
 * 150 FP32 steps) on a 192 x 96 grid, i.e. one chain in the precision of the
 * context plus its FP64 staging, one intermediate and one Boltzmann slice. */
#define SCFT_STATIC_SCRATCH_BYTES (32u << 20)
#define SCFT_STATIC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_scratch[SCFT_STATIC_SCRATCH_BYTES];

/* per device: the array's device address, looked up once (atomic: first calls
 * from several threads may race to store the same value) */
static std::atomic<void *> g_scratch_addr[SCFT_STATIC_MAX_DEVICES];

static size_t up256(size_t b) { return (b + 255) / 256 * 256; }

extern "C" size_t scft_static_scratch_bytes(void) { return SCFT_STATIC_SCRATCH_BYTES; }

extern "C" int scft_propagate_static(scft_ctx *ctx, const double *q0, const double *w, int steps, double *q_out)
{
    if (!ctx || !q0 || !w || !q_out || steps < 0) return SCFT_ERR_PARAM;
    int dev = 0, prec = 0;
    long m = 0, sm = 0;
    double ds = 0.0;
    cudaStream_t st = nullptr;
    const InstOps *ops = nullptr;
    scft_ctx_info(ctx, &dev, &prec, &m, &sm, &ds, &st, &ops);
    if (dev < 0 || dev >= SCFT_STATIC_MAX_DEVICES) return SCFT_ERR_PARAM;
    const size_t psize = prec == SCFT_PREC_FP32 ? 4 : 8; /* FP64 or an FP32 pair */
    const size_t slices = (size_t)steps + 1;
    /* layout: descriptor | FP64 staging of q (slices) | q in the context precision
     * (slices) | intermediate slice | Boltzmann slice | FP64 staging of w */
    const size_t o_desc = 0;
    const size_t o_qd = up256(sizeof(ChainDesc));
    const size_t o_q = o_qd + up256(sizeof(double) * sm * slices);
    const size_t o_tmp = o_q + up256(psize * sm * slices);
    const size_t o_bz = o_tmp + up256(psize * sm);
    const size_t o_w = o_bz + up256(psize * sm);
    const size_t need = o_w + up256(sizeof(double) * sm);
    if (need > SCFT_STATIC_SCRATCH_BYTES) {
        char msg[256];
        snprintf(msg, sizeof(msg),
                 "scft_propagate_static: %d steps on %ld points need %zu bytes, above the fixed %u-byte working array",
                 steps, m, need, SCFT_STATIC_SCRATCH_BYTES);
        scft_set_error(msg);
        return SCFT_ERR_PARAM;
    }
    cudaError_t e = cudaSetDevice(dev);
    void *addr = g_scratch_addr[dev].load(std::memory_order_acquire);
    if (e == cudaSuccess && !addr) {
        e = cudaGetSymbolAddress(&addr, g_scratch);
        if (e == cudaSuccess) g_scratch_addr[dev].store(addr, std::memory_order_release);
    }
    if (e != cudaSuccess) {
        char msg[256];
        snprintf(msg, sizeof(msg), "scft_propagate_static: device set-up failed: %s", cudaGetErrorString(e));
        scft_set_error(msg);
        return SCFT_ERR_CUDA;
    }
    /* from here on work is queued on the stream: every return waits for it, so
     * no error path leaves a copy or kernel writing the shared array */
    auto fail = [&](cudaError_t err, int rc) {
        cudaStreamSynchronize(st);
        if (err != cudaSuccess) {
            char msg[256];
            snprintf(msg, sizeof(msg), "scft_propagate_static: %s", cudaGetErrorString(err));
            scft_set_error(msg);
        }
        return rc;
    };
    unsigned char *base = static_cast<unsigned char *>(addr);
    ChainDesc *desc = reinterpret_cast<ChainDesc *>(base + o_desc);
    double *qd = reinterpret_cast<double *>(base + o_qd);
    void *q = base + o_q;
    void *tmp = base + o_tmp;
    void *bz = base + o_bz;
    double *wd = reinterpret_cast<double *>(base + o_w);

    ChainDesc cd;
    memset(&cd, 0, sizeof(cd));
    cd.q = q;
    cd.tmp = tmp;
    cd.b0 = bz;
    cd.b1 = bz;
    cd.seg_end = steps + 1;
    cd.len = steps + 1;
    cd.ops = ops;
    e = cudaMemcpyAsync(desc, &cd, sizeof(cd), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(wd, w, sizeof(double) * m, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(qd, q0, sizeof(double) * m, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = scft_boltz_one(prec, wd, bz, ds, m, st);
    if (e == cudaSuccess) e = scft_convert(prec, qd, q, m, 1, st);
    if (e != cudaSuccess) return fail(e, SCFT_ERR_CUDA);
    int rc = scft_ctx_run_chain(ctx, desc, steps + 1);
    if (rc != SCFT_OK) return fail(cudaSuccess, rc);
    e = scft_convert(prec, static_cast<const double *>(q), qd, (long)(sm * slices), 0, st);
    for (size_t s = 0; s < slices && e == cudaSuccess; ++s)
        e = cudaMemcpyAsync(q_out + s * m, qd + s * sm, sizeof(double) * m, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(e, SCFT_ERR_CUDA);
    return SCFT_OK;
}
