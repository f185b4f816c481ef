/*
 * scft_ctx.cu — the C ABI of include/scft_gpu.h: context set-up, device
 * memory, the per-iteration launch sequence and host transfers.
 *
 * One iteration (SCFT.c:1090-1580) is launched as
 *   iter_begin (iIter++, Boltzmann factors, initial slices)
 *   for s in 0 .. maxlen-2: one pass per grid axis over every active chain
 *   iter_end   (Q, densities, fused update, finalize, p shift)
 * on the context's own stream; with use_graph the sequence is captured once
 * and replayed. Every instance of a context shares the grid, the MASK setting
 * and which species are present; contour counts (NS), box lengths, chi, G1 and
 * noise amplitudes may differ. Instances with the same diffusion factors share
 * one set of operator tables.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "scft_internal.h"

static thread_local char g_err[512] = "";

static void set_err(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

extern "C" const char *scft_last_error(void) { return g_err; }

extern "C" int scft_device_memory(int device, size_t *free_bytes, size_t *total_bytes)
{
    if (!free_bytes || !total_bytes) return SCFT_ERR_PARAM;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
        cudaGetLastError();
        return SCFT_ERR_NODEV;
    }
    int cur = 0;
    cudaGetDevice(&cur);
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaMemGetInfo(free_bytes, total_bytes);
    cudaSetDevice(cur);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return SCFT_ERR_CUDA;
    }
    return SCFT_OK;
}

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) {                                                                   \
            set_err("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);   \
            return e_ == cudaErrorMemoryAllocation ? SCFT_ERR_OOM : SCFT_ERR_CUDA;                 \
        }                                                                                          \
    } while (0)

struct Axis {
    AxisGeom g;
    int tile;
    int ntiles;
    int h, even;
    int dirichlet_dense; /* 1: dense operator (Dirichlet or a length with other prime factors) */
    int dirichlet;       /* 1: the MASK 1 z axis */
    int src;             /* grid axis 0, 1, 2 */
};

/* Propagator chains of one instance in the reference's order of species:
 * homopolymers (one chain each), diblocks (forward and complementary), brushes
 * (forward from the mask, complementary from ones). */
struct ChainSpec {
    int len, f0, f1, seg_end, init, init_arg;
};

struct scft_ctx {
    scft_options opt;
    int B = 0;
    int psize = 8;
    int sms = 152;
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<scft_surface> surf;
    std::vector<scft_derived> der;
    long m = 0, sm = 0;
    int nx = 0, ny = 0, nz = 0;
    int nchains = 0, nblocks = 0, maxlen = 0;
    unsigned field_use = 0;
    std::vector<ChainDesc> chains_h;   /* [B * nchains] */
    std::vector<BlockDesc> blocks_h;   /* [B * nblocks] */
    std::vector<SpeciesDesc> species_h; /* [B * 17] */
    std::vector<Axis> axes;
    /* operator tables: one InstOps per distinct (alphax, alphay, alphaz) */
    std::vector<InstOps> ops_h;
    std::vector<int> ops_of; /* [B]: index into ops_h */
    std::vector<double> ops_alpha; /* [3 * sets]: alphax, alphay, alphaz of each set */
    InstOps *ops = nullptr;  /* device, room for SCFT_OPS_CAP sets */
    std::vector<int> cap;    /* [B * nchains]: contour slices allocated per chain */
    std::vector<ChainSpec> cs0; /* instance 0's chains: the composition every instance shares */
    /* fused contour loops: 2D (scft_step2d.cu), 64^3 clusters (scft_step3d.cu) */
    int fused2d = 0;
    int wide2d = 0; /* fused 2D loop with two threads per line (batches of at most one chain per SM) */
    int fused3d = 0;
    int *order = nullptr; /* chain indices, longest first */
    /* device noise replay (SCFT_NOISE_DRAND48) */
    unsigned long long *rng_in = nullptr;
    int *rng_counts = nullptr;
    long *rng_prefix = nullptr, *rng_total = nullptr;
    long rng_chunks = 0;
    /* device memory */
    double *w = nullptr, *phi = nullptr, *raw = nullptr, *mask = nullptr, *partial = nullptr, *noise = nullptr;
    void *bz = nullptr;
    InstParams *params = nullptr;
    InstState *state = nullptr;
    ChainDesc *chains = nullptr;
    BlockDesc *blocks = nullptr;
    SpeciesDesc *species = nullptr;
    scft_iter_out *hist = nullptr;
    scft_iter_out *last = nullptr;      /* [B] latest record per instance */
    scft_iter_out *hist_host = nullptr; /* pinned */
    int hist_cap = 0;
    int pending = 0; /* iterations enqueued and not yet collected */
    cudaEvent_t chunk_done = nullptr; /* recorded after the records copy of the enqueued chunk */
    int nparts = 0;
    size_t device_bytes = 0;
    std::vector<void *> allocs;
    /* host mirrors */
    std::vector<unsigned long> iter;
    std::vector<unsigned short> rng; /* 3 per instance */
    std::vector<int> fields_set;
    /* graph */
    cudaGraphExec_t graph_exec = nullptr;
    cudaGraph_t graph = nullptr;
    /* timing */
    int timing = 0;
    std::vector<cudaEvent_t> ev; /* 2 per iteration slot + 2 overall */
    scft_timing last_timing{};
    long launches_per_iter = 0, prop_launches_per_iter = 0;
};

/* operator sets a context can hold (scft_set_surface may add sets) */
#define SCFT_OPS_CAP 256

static int dalloc(scft_ctx *c, void **p, size_t bytes)
{
    *p = nullptr;
    if (bytes == 0) bytes = 256;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        set_err("cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
        *p = nullptr;
        return SCFT_ERR_OOM;
    }
    c->allocs.push_back(*p);
    c->device_bytes += bytes;
    cudaMemsetAsync(*p, 0, bytes, c->stream);
    return SCFT_OK;
}

extern "C" void scft_options_default(scft_options *o)
{
    memset(o, 0, sizeof(*o));
    o->precision = SCFT_PREC_FP64;
    o->device = 0;
    o->noise_mode = SCFT_NOISE_HOST;
    o->use_graph = 0;
    o->n_instances = 1;
    o->autotune = 1;
}

/* ------------------------------------------------------- shape helpers */
static const int DBK_FX[4] = {0, 3, 5, 7};

/* Radix decomposition for the Stockham FFT: 4s, then 2, then 3s. Returns 0
 * if n has another prime factor (the axis then uses the dense operator). */
static int radices(int n, int *rad, int *nrad)
{
    int k = 0;
    while (n % 4 == 0 && k < SCFT_MAX_RADIX_STAGES) {
        rad[k++] = 4;
        n /= 4;
    }
    while (n % 2 == 0 && k < SCFT_MAX_RADIX_STAGES) {
        rad[k++] = 2;
        n /= 2;
    }
    while (n % 3 == 0 && k < SCFT_MAX_RADIX_STAGES) {
        rad[k++] = 3;
        n /= 3;
    }
    *nrad = k;
    return n == 1;
}

/* k of spectral index t on a periodic axis of length n, as the reference
 * computes it for aExpArg: 2 pi (n/2 - |t - n/2|) / n (SCFT.c:993-995). */
static double kval(int t, int n) { return 2.0 * M_PI * (n / 2.0 - fabs(t - n / 2.0)) / n; }

/* Dense 1-D operator of one axis, n x n, row-major K[i*n + j]. */
static void dense_operator(int n, double alpha, int dirichlet, std::vector<long double> &K)
{
    K.assign((size_t)n * n, 0.0L);
    if (dirichlet) {
        /* odd extension of length N = 2(n+1): K = (2/L) sum_m E_m sin(pi m a/L) sin(pi m b/L) */
        const int L = n + 1, N = 2 * L;
        std::vector<long double> E(n + 1);
        for (int m = 1; m <= n; ++m) {
            const double kz = kval(m, N);
            E[m] = expl(-(long double)alpha * (long double)kz * (long double)kz);
        }
        const long double pi = 3.141592653589793238462643383279502884L;
        for (int a = 0; a < n; ++a)
            for (int b = a; b < n; ++b) {
                long double s = 0.0L;
                for (int m = 1; m <= n; ++m)
                    s += E[m] * sinl(pi * m * (a + 1) / L) * sinl(pi * m * (b + 1) / L);
                s *= 2.0L / L;
                K[(size_t)a * n + b] = s;
                K[(size_t)b * n + a] = s;
            }
    } else {
        /* circulant: K[i][j] = (1/n) sum_t E_t cos(2 pi t (i-j) / n) */
        const long double pi = 3.141592653589793238462643383279502884L;
        std::vector<long double> c(n);
        for (int d = 0; d < n; ++d) {
            long double s = 0.0L;
            for (int t = 0; t < n; ++t) {
                const double k = kval(t, n);
                s += expl(-(long double)alpha * k * k) * cosl(2.0L * pi * t * d / n);
            }
            c[d] = s / n;
        }
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) K[(size_t)i * n + j] = c[(i - j + n) % n];
    }
}

template <typename T>
static int upload(scft_ctx *c, void **dst, const std::vector<T> &v)
{
    int rc = dalloc(c, dst, sizeof(T) * v.size());
    if (rc) return rc;
    CK(cudaMemcpyAsync(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, c->stream));
    return SCFT_OK;
}

/* Convert a double vector to the context precision and upload: FP64 as is,
 * FP32 rounded to nearest, FP32x2 as the pair (hi, lo) nearest each value
 * (hi = fl32(v), lo = fl32(v - hi)). */
static int upload_p(scft_ctx *c, void **dst, const std::vector<double> &v)
{
    if (c->opt.precision == SCFT_PREC_FP64) return upload(c, dst, v);
    if (c->opt.precision == SCFT_PREC_FP32X2) {
        std::vector<float> f(2 * v.size());
        for (size_t i = 0; i < v.size(); ++i) {
            const float hi = (float)v[i];
            f[2 * i] = hi;
            f[2 * i + 1] = (float)(v[i] - (double)hi);
        }
        return upload(c, dst, f);
    }
    std::vector<float> f(v.begin(), v.end());
    return upload(c, dst, f);
}

/* Round an n x n operator block (row-major) to FP32 so that every column sum of
 * the FP32 values equals the FP64 column sum as closely as FP32 allows: each
 * entry is first rounded to nearest, then the residual of its column is handed
 * out in steps of one ulp, largest entries first, each entry moving by at most
 * one ulp. The mean mode of q passes through 1^T A only, so this keeps the FP32
 * step free of a systematic per-step gain that would otherwise add up over a
 * chain's contour steps (and bias ln Q). */
static std::vector<double> round_fp32_colsum(const std::vector<double> &A, int rows, int cols)
{
    std::vector<double> out(A.size());
    std::vector<int> order(rows);
    for (int k = 0; k < cols; ++k) {
        long double target = 0.0L, have = 0.0L;
        for (int i = 0; i < rows; ++i) {
            const float r = (float)A[(size_t)i * cols + k];
            out[(size_t)i * cols + k] = r;
            target += (long double)A[(size_t)i * cols + k];
            have += (long double)r;
        }
        for (int i = 0; i < rows; ++i) order[i] = i;
        std::sort(order.begin(), order.end(), [&](int x, int y) {
            return fabs(A[(size_t)x * cols + k]) > fabs(A[(size_t)y * cols + k]);
        });
        long double resid = target - have;
        for (int t = 0; t < rows && resid != 0.0L; ++t) {
            const int i = order[t];
            const float r = (float)out[(size_t)i * cols + k];
            if (r == 0.0f) continue;
            const float up = nextafterf(r, INFINITY), dn = nextafterf(r, -INFINITY);
            const long double ulp_up = (long double)up - r, ulp_dn = (long double)r - dn;
            if (resid >= ulp_up / 2) {
                out[(size_t)i * cols + k] = up;
                resid -= ulp_up;
            } else if (-resid >= ulp_dn / 2) {
                out[(size_t)i * cols + k] = dn;
                resid += ulp_dn;
            }
        }
    }
    return out;
}

static int pick_tile(long lines_per_chain, long inner_or_lines, int total_chains, int sms, int start)
{
    int tile = start;
    while (tile > 2 && (inner_or_lines % tile != 0 || (lines_per_chain / tile) * (long)total_chains < 2L * sms)) tile /= 2;
    while (tile > 1 && inner_or_lines % tile != 0) tile /= 2;
    return tile;
}

/* bf16 round to nearest (ties to even) through FP32, and back */
static uint16_t bf16_rn(long double v)
{
    const float f = (float)v;
    uint32_t u;
    memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}
static long double bf16_val(uint16_t b)
{
    const uint32_t u = (uint32_t)b << 16;
    float f;
    memcpy(&f, &u, 4);
    return (long double)f;
}

/* Table of the tensor-core z operator of the fused FP32 2D loop (see
 * scft_step2d.cu): y = Kb x + Kt x, with Kb a band |j - k| <= 3 (circular for a
 * periodic axis) in FP32 and Kt = K - Kb.
 *   Band: the R0 = 8 rows at either end keep their own FP32 entries of K;
 *   every interior row uses the same four constants c_d = K[h][h+d] (d = 0..3,
 *   c_-d = c_d, h = nz/2), the Toeplitz part of K. Everything else, including
 *   the interior rows' small Hankel parts near the diagonal and the FP32
 *   rounding residuals of the band, is in the tail.
 *   Tail: centrosymmetric halves Ae = (T[i][k] + T[i][nz-1-k]) / 2,
 *   Ao = (T[i][k] - T[i][nz-1-k]) / 2 of the top rows (i, k < h), each split
 *   into bf16 pieces hi = rn(A), lo = rn(A - hi). Column sums of the operator
 *   the kernel applies (FP32 band plus the pieces' sums) are made equal to
 *   those of K by moving Ae's diagonal: the mean mode passes through the
 *   column sums, so no systematic per-step gain builds up over a chain.
 * The bottom rows are the mirror images of the top rows (K is centrosymmetric).
 * Layout (bytes): float band[2 R0][8] (rows 0..R0-1, then nz-R0..nz-1; slot
 * d + 3 multiplies x[(j + d) mod nz], zero where a Dirichlet row has no such
 * neighbour), float interior[8] = {c0, c1, c2, c3, 0...}, then Ae.hi, Ae.lo,
 * Ao.hi, Ao.lo as K-major 8 x 16-byte core matrices (element (i, k) at byte
 * (i/8) 16h + (k/8) 128 + (i%8) 16 + (k%8) 2 of its piece). */
static std::vector<unsigned char> ztc_table(const std::vector<long double> &K, int nz, int periodic)
{
    const int h = nz / 2, R0 = 8;
    auto at = [&](int j, int k) { return K[(size_t)j * nz + k]; };
    float cT[4];
    for (int d = 0; d < 4; ++d) cT[d] = (float)((at(h, h + d) + at(h, h - d)) / 2.0L);
    /* FP32 band value of top row i (< h) at column k, 0 off the band */
    auto band = [&](int i, int k) -> float {
        int d = k - i;
        if (periodic) {
            if (d > nz / 2) d -= nz;
            if (d < -nz / 2) d += nz;
        }
        if (d < -3 || d > 3) return 0.0f;
        if (i < R0) return (float)at(i, k);
        return cT[d < 0 ? -d : d];
    };
    std::vector<long double> Ae((size_t)h * h), Ao((size_t)h * h);
    for (int i = 0; i < h; ++i)
        for (int k = 0; k < h; ++k) {
            const long double t1 = at(i, k) - (long double)band(i, k);
            const long double t2 = at(i, nz - 1 - k) - (long double)band(i, nz - 1 - k);
            Ae[(size_t)i * h + k] = (t1 + t2) / 2.0L;
            Ao[(size_t)i * h + k] = (t1 - t2) / 2.0L;
        }
    std::vector<uint16_t> e1((size_t)h * h), e2((size_t)h * h), o1((size_t)h * h), o2((size_t)h * h);
    auto split = [](long double v, uint16_t &p, uint16_t &q) {
        p = bf16_rn(v);
        q = bf16_rn(v - bf16_val(p));
    };
    for (size_t u = 0; u < (size_t)h * h; ++u) {
        split(Ae[u], e1[u], e2[u]);
        split(Ao[u], o1[u], o2[u]);
    }
    /* column sums (k < h; column nz-1-k is its mirror): K against FP32 band +
     * 2 sum_i (Ae.hi + Ae.lo)[i][k]. The difference first goes onto Ae[k][k];
     * what its bf16 pair cannot hold is then handed out one ulp of a lo piece
     * at a time, largest entries first (at most one ulp per piece and pass). */
    auto colsum_resid = [&](int k) {
        long double target = 0.0L, have = 0.0L;
        for (int i = 0; i < h; ++i) {
            target += at(i, k) + at(i, nz - 1 - k);
            have += (long double)band(i, k) + (long double)band(i, nz - 1 - k);
            const size_t u = (size_t)i * h + k;
            have += 2.0L * (bf16_val(e1[u]) + bf16_val(e2[u]));
        }
        return target - have;
    };
    auto bf16_step = [](uint16_t b, int up) -> uint16_t { /* next bf16 toward +inf (up) or -inf */
        const bool neg = (b & 0x8000u) != 0;
        return (uint16_t)((up != neg) ? b + 1 : b - 1);
    };
    std::vector<int> order(h);
    for (int k = 0; k < h; ++k) {
        for (int pass = 0; pass < 2; ++pass) {
            const size_t u = (size_t)k * h + k;
            Ae[u] += colsum_resid(k) / 2.0L;
            split(Ae[u], e1[u], e2[u]);
        }
        for (int i = 0; i < h; ++i) order[i] = i;
        std::sort(order.begin(), order.end(), [&](int x, int y) {
            return fabsl(Ae[(size_t)x * h + k]) > fabsl(Ae[(size_t)y * h + k]);
        });
        long double resid = colsum_resid(k);
        for (int pass = 0; pass < 8 && resid != 0.0L; ++pass)
            for (int i : order) {
                uint16_t &q = e2[(size_t)i * h + k];
                const long double v = bf16_val(q);
                if (v == 0.0L || (q & 0x7f80u) == 0x7f80u) continue;
                const uint16_t up = bf16_step(q, 1), dn = bf16_step(q, 0);
                const long double du = bf16_val(up) - v, dd = v - bf16_val(dn);
                if (resid >= du) {
                    q = up;
                    resid -= 2.0L * du;
                } else if (-resid >= dd) {
                    q = dn;
                    resid += 2.0L * dd;
                }
            }
    }
    const size_t nb = (size_t)32 * (2 * R0 + 1), piece = (size_t)2 * h * h;
    std::vector<unsigned char> out(nb + 4 * piece, 0);
    float *bt = reinterpret_cast<float *>(out.data());
    for (int r = 0; r < R0; ++r)
        for (int d = -3; d <= 3; ++d) {
            int k = r + d;
            if (k < 0) {
                if (!periodic) continue;
                k += nz;
            }
            const float v = band(r, k);
            bt[(size_t)r * 8 + (d + 3)] = v;                 /* top row r */
            bt[(size_t)(2 * R0 - 1 - r) * 8 + (3 - d)] = v;  /* its mirror, row nz-1-r */
        }
    for (int d = 0; d < 4; ++d) bt[(size_t)2 * R0 * 8 + d] = cT[d];
    const std::vector<uint16_t> *pcs[4] = {&e1, &e2, &o1, &o2};
    for (int p = 0; p < 4; ++p)
        for (int i = 0; i < h; ++i)
            for (int k = 0; k < h; ++k) {
                const size_t off = nb + p * piece + (size_t)(i / 8) * 16 * h + (size_t)(k / 8) * 128 + (i % 8) * 16 + (k % 8) * 2;
                memcpy(out.data() + off, &(*pcs[p])[(size_t)i * h + k], 2);
            }
    return out;
}

/* Test hook, not part of the ABI: the z operator that the tensor-core form of
 * the fused 2D loop applies, decoded from its table the way the kernel reads
 * it (k_eff, nz x nz row-major), next to the exact operator (k_ref). */
extern "C" int scft_ztc_operator(int nz, double alpha, int dirichlet, double *k_eff, double *k_ref)
{
    if (nz < 32 || nz % 32 != 0 || !k_eff || !k_ref) return SCFT_ERR_PARAM;
    const int h = nz / 2, R0 = 8;
    std::vector<long double> K;
    dense_operator(nz, alpha, dirichlet, K);
    const std::vector<unsigned char> t = ztc_table(K, nz, !dirichlet);
    const float *bt = reinterpret_cast<const float *>(t.data());
    std::vector<long double> E((size_t)nz * nz, 0.0L);
    for (int j = 0; j < nz; ++j)
        for (int d = -3; d <= 3; ++d) {
            float c;
            if (j < R0)
                c = bt[(size_t)j * 8 + d + 3];
            else if (j >= nz - R0)
                c = bt[(size_t)(j - nz + 2 * R0) * 8 + d + 3];
            else
                c = bt[(size_t)2 * R0 * 8 + (d < 0 ? -d : d)];
            E[(size_t)j * nz + (j + d + nz) % nz] += (long double)c;
        }
    const size_t nb = (size_t)32 * (2 * R0 + 1), piece = (size_t)2 * h * h;
    auto pc = [&](int p, int i, int k) {
        uint16_t b;
        memcpy(&b, t.data() + nb + p * piece + (size_t)(i / 8) * 16 * h + (size_t)(k / 8) * 128 + (i % 8) * 16 + (k % 8) * 2, 2);
        return bf16_val(b);
    };
    for (int i = 0; i < h; ++i)
        for (int k = 0; k < h; ++k) {
            const long double ae = pc(0, i, k) + pc(1, i, k), ao = pc(2, i, k) + pc(3, i, k);
            E[(size_t)i * nz + k] += ae + ao;
            E[(size_t)i * nz + (nz - 1 - k)] += ae - ao;
            E[(size_t)(nz - 1 - i) * nz + k] += ae - ao;
            E[(size_t)(nz - 1 - i) * nz + (nz - 1 - k)] += ae + ao;
        }
    for (size_t u = 0; u < (size_t)nz * nz; ++u) {
        k_eff[u] = (double)E[u];
        k_ref[u] = (double)K[u];
    }
    return SCFT_OK;
}

/* z operator halves and x factor of one operator set for the fused 2D step. */
static int fused2d_tables(scft_ctx *c, const scft_derived &d, InstOps &o)
{
    const int nz = d.nz, h = nz / 2, nx = d.nx;
    std::vector<long double> K;
    dense_operator(nz, d.alphaz, c->surf[0].mask, K);
    if (scft_step2d_ztc(c->opt.precision, nx, nz)) {
        std::vector<double> ex(nx);
        for (int k = 0; k < nx; ++k) {
            const double kk = kval(k, nx);
            ex[k] = exp(-d.alphax * kk * kk) / nx;
        }
        void *kz_d = nullptr, *ex_d = nullptr;
        int rc = upload(c, &kz_d, ztc_table(K, nz, !c->surf[0].mask));
        if (!rc) rc = upload_p(c, &ex_d, ex);
        if (rc) return rc;
        o.kz = kz_d;
        o.ex = ex_d;
        return SCFT_OK;
    }
    std::vector<double> kz((size_t)2 * h * h);
    for (int i = 0; i < h; ++i)
        for (int j = 0; j < h; ++j) {
            const long double kij = K[(size_t)i * nz + j], kim = K[(size_t)i * nz + (nz - 1 - j)];
            kz[(size_t)i * h + j] = (double)((kij + kim) / 2.0L);
            kz[(size_t)h * h + (size_t)i * h + j] = (double)((kij - kim) / 2.0L);
        }
    if (c->psize == 4) {
        std::vector<double> Ah(kz.begin(), kz.begin() + (size_t)h * h), Bh(kz.begin() + (size_t)h * h, kz.end());
        Ah = round_fp32_colsum(Ah, h, h);
        Bh = round_fp32_colsum(Bh, h, h);
        std::copy(Ah.begin(), Ah.end(), kz.begin());
        std::copy(Bh.begin(), Bh.end(), kz.begin() + (size_t)h * h);
    }
    std::vector<double> ex(nx);
    for (int k = 0; k < nx; ++k) {
        const double kk = kval(k, nx);
        ex[k] = exp(-d.alphax * kk * kk) / nx;
    }
    void *kz_d = nullptr, *ex_d = nullptr;
    int rc = upload_p(c, &kz_d, kz);
    if (!rc) rc = upload_p(c, &ex_d, ex);
    if (rc) return rc;
    o.kz = kz_d;
    o.ex = ex_d;
    return SCFT_OK;
}

/* The fused 2D step: z operator rows (A then B, row-major) and the x factor
 * E(k)/NX per operator set, the four-step twiddles along x once. */
static int build_fused2d(scft_ctx *c)
{
    const scft_derived &d0 = c->der[0];
    if (c->opt.kernel_path != 0 || d0.ny != 1 || d0.nx < 2 || d0.nz < 2) return SCFT_OK;
    if (scft_step2d_smem(c->opt.precision, d0.nx, d0.nz) == 0) return SCFT_OK;
    const int nx = d0.nx, n1 = scft_step2d_n1(nx), n2 = nx / n1;
    std::vector<double> twx(2 * (size_t)nx);
    for (int q2 = 0; q2 < n2; ++q2)
        for (int k1 = 0; k1 < n1; ++k1) {
            const double ang = 2.0 * M_PI * (double)((q2 * k1) % nx) / nx;
            twx[2 * (q2 * n1 + k1)] = cos(ang);
            twx[2 * (q2 * n1 + k1) + 1] = -sin(ang);
        }
    void *twx_d = nullptr;
    int rc = upload_p(c, &twx_d, twx);
    if (rc) return rc;
    for (size_t u = 0; u < c->ops_h.size(); ++u) {
        int b = 0;
        while (c->ops_of[b] != (int)u) ++b;
        rc = fused2d_tables(c, c->der[b], c->ops_h[u]);
        if (rc) return rc;
        c->ops_h[u].twx = twx_d;
    }
    Step2DArgs a;
    memset(&a, 0, sizeof(a));
    CK(scft_launch_step2d(c->opt.precision, nx, d0.nz, a, 0, c->stream, 1, 0));
    c->fused2d = 1;
    /* a batch with at most one chain per SM runs one CTA per SM either way: twice
     * the threads per chain shortens each step, with bit-identical results */
    c->wide2d = scft_step2d_wide(c->opt.precision, nx, d0.nz) && (long)c->B * c->nchains <= c->sms;
    return SCFT_OK;
}
/* Operator tables of one grid axis (pass slot ai) for one operator set. */
static int axis_tables(scft_ctx *c, const Axis &A, double alpha, InstOps &o, int ai)
{
    const int n = A.g.n;
    if (!A.dirichlet_dense) {
        std::vector<double> spec(n), tw(2 * n);
        for (int t = 0; t < n; ++t) {
            const double k = kval(t, n);
            spec[t] = exp(-alpha * k * k) / n;
            tw[2 * t] = cos(2.0 * M_PI * t / n);
            tw[2 * t + 1] = -sin(2.0 * M_PI * t / n);
        }
        void *sp = nullptr, *twd = nullptr;
        int rc = upload_p(c, &sp, spec);
        if (!rc) rc = upload_p(c, &twd, tw);
        if (rc) return rc;
        o.spec[ai] = sp;
        o.tw[ai] = twd;
        return SCFT_OK;
    }
    std::vector<long double> K;
    dense_operator(n, alpha, A.dirichlet, K);
    if (A.even) {
        const int h = n / 2;
        std::vector<double> Ar((size_t)h * h), Br((size_t)h * h), At((size_t)h * h), Bt((size_t)h * h);
        for (int i = 0; i < h; ++i)
            for (int j = 0; j < h; ++j) {
                const long double kij = K[(size_t)i * n + j], kim = K[(size_t)i * n + (n - 1 - j)];
                Ar[(size_t)i * h + j] = (double)((kij + kim) / 2.0L);
                Br[(size_t)i * h + j] = (double)((kij - kim) / 2.0L);
            }
        if (c->psize == 4) {
            Ar = round_fp32_colsum(Ar, h, h);
            Br = round_fp32_colsum(Br, h, h);
        }
        for (int i = 0; i < h; ++i)
            for (int j = 0; j < h; ++j) {
                At[(size_t)j * h + i] = Ar[(size_t)i * h + j];
                Bt[(size_t)j * h + i] = Br[(size_t)i * h + j];
            }
        void *ka = nullptr, *kb = nullptr;
        int rc = upload_p(c, &ka, At);
        if (!rc) rc = upload_p(c, &kb, Bt);
        if (rc) return rc;
        o.kA[ai] = ka;
        o.kB[ai] = kb;
    } else {
        std::vector<double> Kt((size_t)n * n);
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) Kt[(size_t)j * n + i] = (double)K[(size_t)i * n + j];
        void *ka = nullptr;
        int rc = upload_p(c, &ka, Kt);
        if (rc) return rc;
        o.kA[ai] = ka;
        o.kB[ai] = ka;
    }
    return SCFT_OK;
}

/* Per-axis pass geometry (shared by every instance) and each operator set's
 * tables. Instances with equal (alphax, alphay, alphaz) share one set. */
/* The cluster-resident 3D contour loop uses the per-axis spectra of the FFT
 * passes (spec[x], spec[y], spec[z]); it needs an 8-CTA cluster with ~200 KB
 * of shared memory per CTA to be schedulable on the device. */
static int build_fused3d(scft_ctx *c)
{
    const scft_derived &d0 = c->der[0];
    if (c->opt.kernel_path != 0 || c->surf[0].mask || c->fused2d) return SCFT_OK;
    if (scft_step3d_smem(c->opt.precision, d0.nx, d0.ny, d0.nz) == 0 || c->axes.size() != 3) return SCFT_OK;
    for (const Axis &A : c->axes)
        if (A.dirichlet_dense) return SCFT_OK;
    Step2DArgs a;
    memset(&a, 0, sizeof(a));
    const cudaError_t e = scft_launch_step3d(a, 0, c->stream, 1);
    if (e != cudaSuccess) {
        /* the cluster cannot be resident on this device (or the query is not
         * available): the per-axis passes run, which scft_get_timing reports */
        cudaGetLastError();
        return SCFT_OK;
    }
    c->fused3d = 1;
    return SCFT_OK;
}

static int build_axes(scft_ctx *c)
{
    const scft_derived &d = c->der[0];
    const int dims[3] = {d.nx, d.ny, d.nz};
    const int total_chains = c->B * c->nchains;
    c->ops_of.assign(c->B, 0);
    c->ops_h.clear();
    std::vector<int> rep; /* first instance of each operator set */
    for (int b = 0; b < c->B; ++b) {
        const scft_derived &db = c->der[b];
        int u = 0;
        for (; u < (int)rep.size(); ++u) {
            const scft_derived &dr = c->der[rep[u]];
            if (dr.alphax == db.alphax && dr.alphay == db.alphay && dr.alphaz == db.alphaz) break;
        }
        if (u == (int)rep.size()) {
            rep.push_back(b);
            c->ops_alpha.insert(c->ops_alpha.end(), {db.alphax, db.alphay, db.alphaz});
            InstOps o;
            memset(&o, 0, sizeof(o));
            c->ops_h.push_back(o);
        }
        c->ops_of[b] = u;
    }
    int optin_limit = 0;
    CK(cudaDeviceGetAttribute(&optin_limit, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    for (int ax = 0; ax < 3; ++ax) {
        const int n = dims[ax];
        if (n <= 1) continue;
        Axis A;
        memset(&A, 0, sizeof(A));
        A.src = ax;
        A.g.n = n;
        A.g.ls = ax == 0 ? d.ny * d.nz : (ax == 1 ? d.nz : 1);
        A.g.inner = ax == 2 ? 1 : A.g.ls;
        A.g.outer = ax == 0 ? 1 : (ax == 1 ? d.nx : d.nx * d.ny);
        A.dirichlet = (ax == 2 && c->surf[0].mask);
        const int fft_ok = !A.dirichlet && radices(n, A.g.rad, &A.g.nrad);
        if (fft_ok) {
            /* x / d == umulhi(x, ceil(2^32 / d)) for x * d < 2^32 (lines and
             * butterflies of one pass stay far below that) */
            auto magic = [](unsigned dv) -> unsigned {
                return dv <= 1 ? 0u : (unsigned)((0xFFFFFFFFull + dv) / dv);
            };
            int ns = 1;
            for (int st = 0; st < A.g.nrad; ++st) {
                A.g.mag_nr[st] = magic((unsigned)(n / A.g.rad[st]));
                A.g.mag_ns[st] = magic((unsigned)ns);
                ns *= A.g.rad[st];
            }
        }
        A.g.dirichlet = fft_ok ? 0 : 1;
        A.dirichlet_dense = !fft_ok;
        const long lines = c->m / n;
        const long divisor = ax == 2 ? lines : A.g.inner;
        if (fft_ok) {
            A.tile = pick_tile(lines, divisor, total_chains, c->sms, c->psize == 8 ? 16 : 32);
        } else {
            A.tile = pick_tile(lines, divisor, total_chains, c->sms, c->psize == 8 ? 8 : 16);
            A.even = (n % 2 == 0);
            A.h = A.even ? n / 2 : n;
        }
        const size_t smem = scft_pass_smem_bytes(A.g, A.tile, A.h, c->psize);
        if (smem > (size_t)optin_limit) {
            set_err("axis %d of length %d needs %zu bytes of shared memory", ax, n, smem);
            return SCFT_ERR_PARAM;
        }
        A.ntiles = (int)(lines / A.tile);
        const int ai = (int)c->axes.size();
        for (size_t u = 0; u < rep.size(); ++u) {
            const scft_derived &dr = c->der[rep[u]];
            const double alpha = ax == 0 ? dr.alphax : (ax == 1 ? dr.alphay : dr.alphaz);
            int rc = axis_tables(c, A, alpha, c->ops_h[u], ai);
            if (rc) return rc;
        }
        c->axes.push_back(A);
    }
    /* the limit is a cap, not a reservation: set the device maximum once */
    CK(scft_pass_configure(optin_limit));
    return SCFT_OK;
}

/* ------------------------------------------------------------ autotuner */
/* Tiles (lines per CTA) of the per-axis passes, timed on the context's own
 * chains: every candidate that divides the axis' line layout and fits shared
 * memory runs a few contour-step passes, and the fastest is kept. Only even
 * tiles are candidates for the FFT passes, so the pairing of real lines into
 * complex ones (2q, 2q+1) and with it every rounding is the same for every
 * candidate: tuning never changes results. The radix order is not tuned for
 * the same reason (it would change the rounding). Choices are cached per
 * precision, axis geometry and number of chains. */
static std::mutex g_tune_mu;
static std::map<std::string, int> g_tune_cache;

static int autotune_axes(scft_ctx *c)
{
    if (c->axes.empty()) return SCFT_OK;
    int optin = 0;
    CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    const int npass = (int)c->axes.size();
    const int total = c->B * c->nchains;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    int rc = SCFT_OK;
    for (int ai = 0; ai < npass && rc == SCFT_OK; ++ai) {
        Axis &A = c->axes[ai];
        const long lines = c->m / A.g.n;
        const long divisor = A.src == 2 ? lines : A.g.inner;
        char key[160];
        snprintf(key, sizeof(key), "%d|%d,%d,%d,%d,%d|%d|%d", c->opt.precision, A.g.n, A.g.ls, A.g.inner, A.g.outer,
                 A.g.dirichlet, total, ai == 0 ? 1 : (ai == npass - 1 ? 2 : 0));
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            auto it = g_tune_cache.find(key);
            if (it != g_tune_cache.end()) {
                A.tile = it->second;
                A.ntiles = (int)(lines / A.tile);
                continue;
            }
        }
        /* every divisor up to 64 (even ones for the FFT passes), not only powers of
         * two: with few chains (a single solve) a tile that gives about one CTA per
         * SM avoids a second, mostly empty wave */
        std::vector<int> cand;
        for (int t = A.g.dirichlet ? 1 : 2; t <= 64; t += A.g.dirichlet ? 1 : 2)
            if (divisor % t == 0 && lines / t >= 1 && scft_pass_smem_bytes(A.g, t, A.h, c->psize) <= (size_t)optin)
                cand.push_back(t);
        if (cand.size() > 1) {
            float best_ms = 1e30f;
            int best = A.tile;
            for (int t : cand) {
                PassArgs pa;
                memset(&pa, 0, sizeof(pa));
                pa.chains = c->chains;
                pa.nchains = total;
                pa.s = 0;
                pa.first = ai == 0;
                pa.last = ai == npass - 1;
                pa.tile = t;
                pa.sstride = c->sm;
                pa.axis = ai;
                pa.h = A.h;
                pa.even = A.even;
                const int nt = (int)(lines / t);
                cudaError_t e = scft_launch_pass(c->opt.precision, A.g, pa, nt, c->stream); /* warm-up */
                if (e == cudaSuccess) e = cudaEventRecord(e0, c->stream);
                for (int r = 0; r < 3 && e == cudaSuccess; ++r) e = scft_launch_pass(c->opt.precision, A.g, pa, nt, c->stream);
                if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
                if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                float ms = 0.f;
                if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
                if (e != cudaSuccess) {
                    set_err("autotune: %s", cudaGetErrorString(e));
                    rc = SCFT_ERR_CUDA;
                    break;
                }
                if (ms < best_ms) {
                    best_ms = ms;
                    best = t;
                }
            }
            A.tile = best;
            A.ntiles = (int)(lines / A.tile);
        }
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = A.tile;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

/* The fused 2D contour loop's launch form: one or two threads per line (every
 * value computed by the same arithmetic either way, so results are
 * bit-identical). Both are timed on the context's own chains (one persistent
 * launch of a whole iteration's contour steps, after a warm-up launch) and the
 * faster is kept, cached per (shape, precision, chains, contour length). The
 * launches run on whatever the chains' buffers hold at creation: the timing
 * does not depend on the values, and every buffer is rewritten before use. */
static int autotune_fused2d(scft_ctx *c)
{
    if (!c->fused2d || !scft_step2d_wide(c->opt.precision, c->nx, c->nz)) return SCFT_OK;
    const int total = c->B * c->nchains;
    char key[160];
    snprintf(key, sizeof(key), "fused2d|%d|%d,%d|%d|%d", c->psize, c->nx, c->nz, total, c->maxlen);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            c->wide2d = it->second;
            return SCFT_OK;
        }
    }
    Step2DArgs a;
    memset(&a, 0, sizeof(a));
    a.chains = c->chains;
    a.order = c->order;
    a.state = nullptr; /* every chain runs */
    a.s = 0;
    a.s_end = c->maxlen - 1;
    a.sstride = c->sm;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float best_ms = 1e30f;
    int best = c->wide2d;
    cudaError_t e = cudaSuccess;
    for (int wide = 0; wide <= 1 && e == cudaSuccess; ++wide) {
        e = scft_launch_step2d(c->opt.precision, c->nx, c->nz, a, total, c->stream, 0, wide); /* warm-up */
        if (e == cudaSuccess) e = cudaEventRecord(e0, c->stream);
        for (int r = 0; r < 2 && e == cudaSuccess; ++r)
            e = scft_launch_step2d(c->opt.precision, c->nx, c->nz, a, total, c->stream, 0, wide);
        if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && ms < best_ms) {
            best_ms = ms;
            best = wide;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) {
        set_err("autotune: %s", cudaGetErrorString(e));
        return SCFT_ERR_CUDA;
    }
    scft_step2d_take_fault(); /* a tensor-core wait that gave up on the timing runs is not an iteration's */
    c->wide2d = best;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = best;
    return SCFT_OK;
}

/* Instances of one context share the grid, the MASK setting and the active
 * field set (the noise layout); the species composition is compared after the
 * chains are built. */
static int same_shape(const scft_surface &a, const scft_derived &da, const scft_surface &b, const scft_derived &db)
{
    if (da.nx != db.nx || da.ny != db.ny || da.nz != db.nz || a.mask != b.mask) return 0;
    if (da.n_active != db.n_active || memcmp(da.active, db.active, sizeof(da.active))) return 0;
    return 1;
}

/* Chains, density blocks and species table of one instance (see ChainSpec). */
static void build_instance(const scft_surface &s, const scft_derived &d, std::vector<ChainSpec> &cs,
                           std::vector<BlockDesc> &blocks, SpeciesDesc *species)
{
    cs.clear();
    blocks.clear();
    memset(species, 0, sizeof(SpeciesDesc) * SCFT_NSPECIES);
    for (int h = 0; h < 10; ++h) {
        if (d.ns_homo[h] <= 0) continue;
        const int ci = (int)cs.size();
        cs.push_back({d.ns_homo[h], h, h, d.ns_homo[h], SCFT_INIT_ONES, 0});
        blocks.push_back({ci, ci, 0, d.ns_homo[h] - 1, d.ns_homo[h], 4 + h, h, 1});
        species[4 + h] = {1, ci, d.ns_homo[h], 0};
    }
    for (int k = 0; k < 4; ++k) {
        if (!(s.vol_dbk[k] > 0.0)) continue;
        const int fx = DBK_FX[k], fy = fx + 1, ns = d.ns_dbk[k], nx_ = d.ns_dbk_x[k], ny_ = d.ns_dbk_y[k];
        const int cf = (int)cs.size();
        cs.push_back({ns, fx, fy, nx_ - 1, (k == 0 && s.enable_seed == 1) ? SCFT_INIT_SEED : SCFT_INIT_ONES, 0});
        const int cb = (int)cs.size();
        cs.push_back({ns, fy, fx, ny_, SCFT_INIT_ONES, 0});
        blocks.push_back({cf, cb, 0, nx_ - 1, ns, k, fx, 0});
        blocks.push_back({cf, cb, nx_ - 1, ns - 1, ns, k, fy, 0});
        /* Q from the complementary chain for dbk1/2, the forward chain for dbk3/4 (SCFT.c:1271, :1314, :1357, :1399) */
        species[k] = {1, k < 2 ? cb : cf, ns, 0};
    }
    for (int k = 0; k < 3; ++k) {
        if (d.ns_s[k] <= 0) continue;
        const int ns = d.ns_s[k];
        const int cf = (int)cs.size();
        cs.push_back({ns, 10 + k, 10 + k, ns, SCFT_INIT_MASK, k});
        const int cb = (int)cs.size();
        cs.push_back({ns, 10 + k, 10 + k, ns, SCFT_INIT_ONES, 0});
        blocks.push_back({cf, cb, 0, ns - 1, ns, 14 + k, 10 + k, 0});
        species[14 + k] = {1, cf, ns, 0};
    }
}

/* Same chains and blocks up to contour counts: equal fields, species and parts. */
static int same_composition(const std::vector<ChainSpec> &ca, const std::vector<BlockDesc> &ba,
                            const std::vector<ChainSpec> &cb, const std::vector<BlockDesc> &bb)
{
    if (ca.size() != cb.size() || ba.size() != bb.size()) return 0;
    for (size_t k = 0; k < ca.size(); ++k)
        if (ca[k].f0 != cb[k].f0 || ca[k].f1 != cb[k].f1) return 0;
    for (size_t k = 0; k < ba.size(); ++k)
        if (ba[k].species != bb[k].species || ba[k].field != bb[k].field || ba[k].part != bb[k].part ||
            ba[k].chain_f != bb[k].chain_f || ba[k].chain_b != bb[k].chain_b)
            return 0;
    return 1;
}

static void fill_params(const scft_surface &s, const scft_derived &d, const BlockDesc *blocks, int nblocks,
                        const SpeciesDesc *species, InstParams &ip)
{
    memset(&ip, 0, sizeof(ip));
    memcpy(ip.chi, d.chi_eff, sizeof(ip.chi));
    memcpy(ip.phi_avg, d.phi_avg, sizeof(ip.phi_avg));
    const double coat = d.coating_vol;
    for (int k = 0; k < nblocks; ++k) {
        const BlockDesc &bd = blocks[k];
        double frac;
        if (bd.species < 4)
            frac = s.vol_dbk[bd.species] * (1.0 - coat);
        else if (bd.species < 14)
            frac = s.vol_homo[bd.species - 4] * (1.0 - coat);
        else
            frac = s.vol_s[bd.species - 14];
        ip.frac[k] = frac > 0.0 ? frac : 1.0; /* funVolFrac scales only for frac > 0 */
    }
    for (int sp = 0; sp < SCFT_NSPECIES; ++sp) {
        if (!species[sp].present) continue;
        if (sp < 4)
            ip.lnq_coef[sp] = (s.vol_dbk[sp] / d.alpha_dbk[sp] * (1.0 - coat));
        else if (sp < 14)
            ip.lnq_coef[sp] = (s.vol_homo[sp - 4] / d.alpha_homo[sp - 4] * (1.0 - coat));
        else
            ip.lnq_coef[sp] = s.vol_s[sp - 14] / d.alpha_s[sp - 14];
    }
    ip.g1 = s.g1;
    ip.g2 = s.g1 / 6.0;
    ip.dt_noise = s.dt_noise;
    ip.ds = d.ds;
    ip.relaxation = s.relaxation;
    memcpy(ip.active, d.active, sizeof(ip.active));
    ip.n_active = d.n_active;
    ip.enable_seed = s.enable_seed;
    ip.seed_steps = s.seed_steps;
    ip.seed_area_delta = s.seed_area_delta;
    ip.mask = s.mask;
}

extern "C" int scft_ctx_destroy(scft_ctx *c)
{
    if (!c) return SCFT_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    if (c->graph) cudaGraphDestroy(c->graph);
    for (cudaEvent_t e : c->ev) cudaEventDestroy(e);
    if (c->chunk_done) cudaEventDestroy(c->chunk_done);
    for (void *p : c->allocs) cudaFree(p);
    if (c->hist_host) cudaFreeHost(c->hist_host);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return SCFT_OK;
}

extern "C" int scft_ctx_create(const scft_surface *surfaces, const scft_options *opt_in, scft_ctx **out)
{
    if (!surfaces || !out) return SCFT_ERR_PARAM;
    *out = nullptr;
    scft_options opt;
    if (opt_in)
        opt = *opt_in;
    else
        scft_options_default(&opt);
    if (opt.n_instances < 1) opt.n_instances = 1;
    if (opt.precision != SCFT_PREC_FP64 && opt.precision != SCFT_PREC_FP32 && opt.precision != SCFT_PREC_FP32X2)
        return SCFT_ERR_PARAM;
    if (opt.noise_mode != SCFT_NOISE_HOST && opt.noise_mode != SCFT_NOISE_DRAND48) {
        set_err("unknown noise_mode %d", opt.noise_mode);
        return SCFT_ERR_PARAM;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        set_err("no CUDA device");
        return SCFT_ERR_NODEV;
    }
    if (opt.device < 0 || opt.device >= ndev) return SCFT_ERR_PARAM;

    scft_ctx *c = new scft_ctx();
    c->opt = opt;
    c->B = opt.n_instances;
    c->psize = opt.precision == SCFT_PREC_FP32 ? 4 : 8; /* FP64, or an FP32 pair */
    c->device = opt.device;
    cudaSetDevice(opt.device);
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, opt.device);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_err("cudaStreamCreate failed");
        delete c;
        return SCFT_ERR_CUDA;
    }
    c->surf.assign(surfaces, surfaces + c->B);
    c->der.resize(c->B);
    for (int b = 0; b < c->B; ++b) {
        int rc = scft_derive(&c->surf[b], &c->der[b]);
        if (rc != SCFT_OK) {
            set_err("instance %d: parameter derivation failed (%d)", b, rc);
            scft_ctx_destroy(c);
            return rc;
        }
        if (b > 0 && !same_shape(c->surf[0], c->der[0], c->surf[b], c->der[b])) {
            set_err("instance %d differs from instance 0 in grid, MASK or active fields", b);
            scft_ctx_destroy(c);
            return SCFT_ERR_PARAM;
        }
    }
    const scft_derived &d = c->der[0];
    const scft_surface &s = c->surf[0];
    c->nx = d.nx;
    c->ny = d.ny;
    c->nz = d.nz;
    c->m = d.m;
    c->sm = (d.m + 63) / 64 * 64;

    /* chains, blocks, species per instance (same composition, own contour counts) */
    std::vector<std::vector<ChainSpec>> cs(c->B);
    std::vector<BlockDesc> blk;
    c->species_h.assign((size_t)c->B * SCFT_NSPECIES, SpeciesDesc{});
    for (int b = 0; b < c->B; ++b) {
        build_instance(c->surf[b], c->der[b], cs[b], blk, &c->species_h[(size_t)b * SCFT_NSPECIES]);
        if (b == 0) {
            c->blocks_h = blk;
            c->nblocks = (int)blk.size();
            continue;
        }
        const std::vector<BlockDesc> b0(c->blocks_h.begin(), c->blocks_h.begin() + c->nblocks);
        int same = same_composition(cs[0], b0, cs[b], blk);
        for (int sp = 0; sp < SCFT_NSPECIES && same; ++sp) {
            const SpeciesDesc &x = c->species_h[sp], &y = c->species_h[(size_t)b * SCFT_NSPECIES + sp];
            same = x.present == y.present && x.q_chain == y.q_chain;
        }
        if (!same) {
            set_err("instance %d differs from instance 0 in which species are present", b);
            scft_ctx_destroy(c);
            return SCFT_ERR_PARAM;
        }
        c->blocks_h.insert(c->blocks_h.end(), blk.begin(), blk.end());
    }
    if (cs[0].empty()) {
        set_err("no species with a positive volume fraction");
        scft_ctx_destroy(c);
        return SCFT_ERR_PARAM;
    }
    c->nchains = (int)cs[0].size();
    c->maxlen = 0;
    c->field_use = 0;
    for (int b = 0; b < c->B; ++b)
        for (const ChainSpec &x : cs[b]) {
            if (x.len > c->maxlen) c->maxlen = x.len;
            c->field_use |= 1u << x.f0;
            c->field_use |= 1u << x.f1;
        }

    int rc = SCFT_OK;
    const long sm = c->sm;
    const int B = c->B;
    void *p = nullptr;
#define ALLOC(ptr, bytes)                                    \
    do {                                                     \
        rc = dalloc(c, &p, (bytes));                         \
        if (rc) {                                            \
            scft_ctx_destroy(c);                             \
            return rc;                                       \
        }                                                    \
        ptr = (decltype(ptr))p;                              \
    } while (0)
    ALLOC(c->w, sizeof(double) * B * 14 * sm);
    ALLOC(c->phi, sizeof(double) * B * 14 * sm);
    ALLOC(c->raw, sizeof(double) * B * c->nblocks * sm);
    ALLOC(c->mask, sizeof(double) * B * 3 * sm);
    ALLOC(c->bz, (size_t)c->psize * B * SCFT_NFIELDS * sm);
    c->nparts = scft_post_nparts(c->m, c->sms);
    ALLOC(c->partial, sizeof(double) * B * SCFT_NSPECIES * c->nparts);
    ALLOC(c->noise, sizeof(double) * B * d.n_active * sm);
    c->hist_cap = SCFT_HIST_CAP;
    ALLOC(c->hist, sizeof(scft_iter_out) * c->hist_cap * B);
    ALLOC(c->last, sizeof(scft_iter_out) * B);
    if (cudaMallocHost((void **)&c->hist_host, sizeof(scft_iter_out) * c->hist_cap * B) != cudaSuccess) {
        set_err("cudaMallocHost failed");
        scft_ctx_destroy(c);
        return SCFT_ERR_OOM;
    }
#undef ALLOC
    if ((rc = build_axes(c)) || (rc = build_fused2d(c)) || (rc = build_fused3d(c))) {
        scft_ctx_destroy(c);
        return rc;
    }
    if ((int)c->ops_h.size() > SCFT_OPS_CAP) {
        set_err("more than %d distinct operator sets in one context", SCFT_OPS_CAP);
        scft_ctx_destroy(c);
        return SCFT_ERR_PARAM;
    }
    rc = dalloc(c, (void **)&p, sizeof(InstOps) * SCFT_OPS_CAP);
    if (rc) {
        scft_ctx_destroy(c);
        return rc;
    }
    c->ops = (InstOps *)p;
    if (cudaMemcpyAsync(c->ops, c->ops_h.data(), sizeof(InstOps) * c->ops_h.size(), cudaMemcpyHostToDevice,
                        c->stream) != cudaSuccess) {
        set_err("operator upload failed");
        scft_ctx_destroy(c);
        return SCFT_ERR_CUDA;
    }
    c->cs0 = cs[0];
#define ALLOC(ptr, bytes)                                    \
    do {                                                     \
        rc = dalloc(c, &p, (bytes));                         \
        if (rc) {                                            \
            scft_ctx_destroy(c);                             \
            return rc;                                       \
        }                                                    \
        ptr = (decltype(ptr))p;                              \
    } while (0)
    c->chains_h.resize((size_t)B * c->nchains);
    for (int b = 0; b < B; ++b)
        for (int k = 0; k < c->nchains; ++k) {
            const ChainSpec &x = cs[b][k];
            ChainDesc &cd = c->chains_h[(size_t)b * c->nchains + k];
            memset(&cd, 0, sizeof(cd));
            void *q, *t;
            ALLOC(q, (size_t)c->psize * x.len * sm);
            ALLOC(t, (size_t)c->psize * sm);
            cd.q = q;
            cd.tmp = t;
            cd.b0 = (char *)c->bz + (size_t)c->psize * ((size_t)b * SCFT_NFIELDS + x.f0) * sm;
            cd.b1 = (char *)c->bz + (size_t)c->psize * ((size_t)b * SCFT_NFIELDS + x.f1) * sm;
            cd.seg_end = x.seg_end;
            cd.len = x.len;
            cd.init = x.init;
            cd.init_arg = x.init_arg;
            cd.instance = b;
            cd.ops = c->ops + c->ops_of[b];
            c->cap.push_back(x.len);
        }
    std::vector<InstParams> ip(B);
    for (int b = 0; b < B; ++b)
        fill_params(c->surf[b], c->der[b], &c->blocks_h[(size_t)b * c->nblocks], c->nblocks,
                    &c->species_h[(size_t)b * SCFT_NSPECIES], ip[b]);
    if ((rc = upload(c, (void **)&c->params, ip)) || (rc = upload(c, (void **)&c->chains, c->chains_h)) ||
        (rc = upload(c, (void **)&c->blocks, c->blocks_h)) || (rc = upload(c, (void **)&c->species, c->species_h))) {
        scft_ctx_destroy(c);
        return rc;
    }
    ALLOC(c->state, sizeof(InstState) * B);
    if (opt.noise_mode == SCFT_NOISE_DRAND48) {
        c->rng_chunks = scft_noise_chunks(c->m, d.n_active);
        ALLOC(c->rng_in, sizeof(unsigned long long) * B);
        ALLOC(c->rng_counts, sizeof(int) * B * c->rng_chunks);
        ALLOC(c->rng_prefix, sizeof(long) * B * c->rng_chunks);
        ALLOC(c->rng_total, sizeof(long) * B);
        if (scft_noise_setup() != cudaSuccess) {
            set_err("noise set-up failed");
            scft_ctx_destroy(c);
            return SCFT_ERR_CUDA;
        }
    }
#undef ALLOC
    if (opt.autotune && !c->fused2d && !c->fused3d && (rc = autotune_axes(c))) {
        scft_ctx_destroy(c);
        return rc;
    }
    {
        /* longest chains first, so the persistent launch ends with short ones */
        std::vector<int> ord((size_t)B * c->nchains);
        for (size_t k = 0; k < ord.size(); ++k) ord[k] = (int)k;
        std::stable_sort(ord.begin(), ord.end(),
                         [&](int x, int y) { return c->chains_h[x].len > c->chains_h[y].len; });
        if ((rc = upload(c, (void **)&c->order, ord))) {
            scft_ctx_destroy(c);
            return rc;
        }
    }
    if (opt.autotune && c->fused2d && (rc = autotune_fused2d(c))) {
        scft_ctx_destroy(c);
        return rc;
    }
    c->iter.assign(B, 0);
    c->rng.assign(3 * B, 0);
    c->fields_set.assign(B, 0);
    c->prop_launches_per_iter = (c->fused2d || c->fused3d) ? 1L : (long)(c->maxlen - 1) * (long)c->axes.size();
    c->launches_per_iter = c->prop_launches_per_iter + 2 + 6 + (opt.noise_mode == SCFT_NOISE_DRAND48 ? 5 : 0);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
        set_err("context set-up failed: %s", cudaGetErrorString(cudaGetLastError()));
        scft_ctx_destroy(c);
        return SCFT_ERR_CUDA;
    }
    *out = c;
    return SCFT_OK;
}

extern "C" int scft_ctx_derived(const scft_ctx *c, int b, scft_derived *d)
{
    if (!c || !d || b < 0 || b >= c->B) return SCFT_ERR_PARAM;
    *d = c->der[b];
    return SCFT_OK;
}

extern "C" size_t scft_ctx_device_bytes(const scft_ctx *c) { return c ? c->device_bytes : 0; }

extern "C" int scft_set_fields(scft_ctx *c, int b, const double *w14)
{
    if (!c || !w14 || b < 0 || b >= c->B) return SCFT_ERR_PARAM;
    cudaSetDevice(c->device);
    for (int f = 0; f < 14; ++f)
        CK(cudaMemcpyAsync(c->w + ((size_t)b * 14 + f) * c->sm, w14 + (size_t)f * c->m, sizeof(double) * c->m,
                           cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->fields_set[b] = 1;
    return SCFT_OK;
}

extern "C" int scft_set_masks(scft_ctx *c, int b, const double *mask3)
{
    if (!c || !mask3 || b < 0 || b >= c->B) return SCFT_ERR_PARAM;
    cudaSetDevice(c->device);
    for (int f = 0; f < 3; ++f)
        CK(cudaMemcpyAsync(c->mask + ((size_t)b * 3 + f) * c->sm, mask3 + (size_t)f * c->m, sizeof(double) * c->m,
                           cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SCFT_OK;
}

extern "C" int scft_set_iteration(scft_ctx *c, int b, unsigned long it)
{
    if (!c || b < 0 || b >= c->B) return SCFT_ERR_PARAM;
    cudaSetDevice(c->device);
    c->iter[b] = it;
    static const int zero = 0;
    CK(cudaMemcpyAsync(&c->state[b].iter, &c->iter[b], sizeof(unsigned long), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(&c->state[b].done, &zero, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    /* a re-armed instance starts without the error status of its last run */
    CK(cudaMemcpyAsync(&c->state[b].status, &zero, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SCFT_OK;
}

extern "C" int scft_freeze(scft_ctx *c, int b)
{
    if (!c || b < 0 || b >= c->B) return SCFT_ERR_PARAM;
    if (c->pending) return SCFT_ERR_STATE;
    cudaSetDevice(c->device);
    static const int one = 1;
    CK(cudaMemcpyAsync(&c->state[b].done, &one, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SCFT_OK;
}

/* Operator tables of a new operator set (per-axis passes and, where the
 * context uses it, the fused 2D step). */
static int build_opset(scft_ctx *c, const scft_derived &d, InstOps &o)
{
    memset(&o, 0, sizeof(o));
    for (size_t ai = 0; ai < c->axes.size(); ++ai) {
        const Axis &A = c->axes[ai];
        const double alpha = A.src == 0 ? d.alphax : (A.src == 1 ? d.alphay : d.alphaz);
        int rc = axis_tables(c, A, alpha, o, (int)ai);
        if (rc) return rc;
    }
    if (c->fused2d) {
        int rc = fused2d_tables(c, d, o);
        if (rc) return rc;
        o.twx = c->ops_h[0].twx;
    }
    return SCFT_OK;
}

extern "C" int scft_set_surface(scft_ctx *c, int b, const scft_surface *s)
{
    if (!c || !s || b < 0 || b >= c->B) return SCFT_ERR_PARAM;
    if (c->pending) {
        set_err("scft_set_surface while iterations are in flight");
        return SCFT_ERR_STATE;
    }
    cudaSetDevice(c->device);
    scft_derived d;
    int rc = scft_derive(s, &d);
    if (rc != SCFT_OK) {
        set_err("parameter derivation failed (%d)", rc);
        return rc;
    }
    if (!same_shape(c->surf[0], c->der[0], *s, d)) {
        set_err("the surface differs from the context in grid, MASK or active fields");
        return SCFT_ERR_PARAM;
    }
    std::vector<ChainSpec> cs;
    std::vector<BlockDesc> blk;
    SpeciesDesc sp[SCFT_NSPECIES];
    build_instance(*s, d, cs, blk, sp);
    const std::vector<BlockDesc> b0(c->blocks_h.begin(), c->blocks_h.begin() + c->nblocks);
    int same = same_composition(c->cs0, b0, cs, blk);
    for (int k = 0; k < SCFT_NSPECIES && same; ++k)
        same = c->species_h[k].present == sp[k].present && c->species_h[k].q_chain == sp[k].q_chain;
    if (!same) {
        set_err("the surface differs from the context in which species are present");
        return SCFT_ERR_PARAM;
    }
    for (int k = 0; k < c->nchains; ++k)
        if (cs[k].len > c->cap[(size_t)b * c->nchains + k]) {
            set_err("chain %d needs %d contour slices; slot %d holds %d", k, cs[k].len, b,
                    c->cap[(size_t)b * c->nchains + k]);
            return SCFT_ERR_PARAM;
        }
    /* operator set: reuse one with the same diffusion factors, else add one */
    int u = 0;
    for (; u < (int)c->ops_h.size(); ++u) {
        const double *al = &c->ops_alpha[3 * (size_t)u];
        if (al[0] == d.alphax && al[1] == d.alphay && al[2] == d.alphaz) break;
    }
    if (u == (int)c->ops_h.size()) {
        if (u >= SCFT_OPS_CAP) {
            set_err("operator-set capacity (%d) of the context is used up", SCFT_OPS_CAP);
            return SCFT_ERR_PARAM;
        }
        InstOps o;
        rc = build_opset(c, d, o);
        if (rc) return rc;
        c->ops_h.push_back(o);
        c->ops_alpha.insert(c->ops_alpha.end(), {d.alphax, d.alphay, d.alphaz});
        CK(cudaMemcpyAsync(c->ops + u, &o, sizeof(InstOps), cudaMemcpyHostToDevice, c->stream));
    }
    c->ops_of[b] = u;
    for (int k = 0; k < c->nchains; ++k) {
        ChainDesc &cd = c->chains_h[(size_t)b * c->nchains + k];
        cd.seg_end = cs[k].seg_end;
        cd.len = cs[k].len;
        cd.init = cs[k].init;
        cd.init_arg = cs[k].init_arg;
        cd.ops = c->ops + u;
    }
    std::copy(blk.begin(), blk.end(), c->blocks_h.begin() + (size_t)b * c->nblocks);
    std::copy(sp, sp + SCFT_NSPECIES, c->species_h.begin() + (size_t)b * SCFT_NSPECIES);
    c->surf[b] = *s;
    c->der[b] = d;
    InstParams ip;
    fill_params(*s, d, blk.data(), c->nblocks, sp, ip);
    std::vector<int> ord((size_t)c->B * c->nchains);
    for (size_t k = 0; k < ord.size(); ++k) ord[k] = (int)k;
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return c->chains_h[x].len > c->chains_h[y].len; });
    CK(cudaMemcpyAsync(c->params + b, &ip, sizeof(ip), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->chains + (size_t)b * c->nchains, &c->chains_h[(size_t)b * c->nchains],
                       sizeof(ChainDesc) * c->nchains, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->blocks + (size_t)b * c->nblocks, blk.data(), sizeof(BlockDesc) * c->nblocks,
                       cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->species + (size_t)b * SCFT_NSPECIES, sp, sizeof(sp), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->order, ord.data(), sizeof(int) * ord.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SCFT_OK;
}

extern "C" int scft_set_stop(scft_ctx *c, int b, double rms_tol)
{
    if (!c || b < 0 || b >= c->B || !(rms_tol >= 0.0)) return SCFT_ERR_PARAM;
    cudaSetDevice(c->device);
    CK(cudaMemcpyAsync(&c->state[b].stop_rms, &rms_tol, sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SCFT_OK;
}

extern "C" int scft_set_rng(scft_ctx *c, int b, const unsigned short seed[3])
{
    if (!c || !seed || b < 0 || b >= c->B) return SCFT_ERR_PARAM;
    memcpy(&c->rng[3 * b], seed, 3 * sizeof(unsigned short));
    if (c->opt.noise_mode == SCFT_NOISE_DRAND48) {
        cudaSetDevice(c->device);
        const unsigned long long x = ((unsigned long long)seed[2] << 32) | ((unsigned long long)seed[1] << 16) | seed[0];
        CK(cudaMemcpyAsync(&c->state[b].rng, &x, sizeof(x), cudaMemcpyHostToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    return SCFT_OK;
}

extern "C" int scft_get_rng(const scft_ctx *c, int b, unsigned short seed[3])
{
    if (!c || !seed || b < 0 || b >= c->B) return SCFT_ERR_PARAM;
    if (c->opt.noise_mode == SCFT_NOISE_DRAND48) {
        cudaSetDevice(c->device);
        unsigned long long x = 0;
        CK(cudaMemcpyAsync(&x, &c->state[b].rng, sizeof(x), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        seed[0] = (unsigned short)(x & 0xFFFF);
        seed[1] = (unsigned short)((x >> 16) & 0xFFFF);
        seed[2] = (unsigned short)((x >> 32) & 0xFFFF);
        return SCFT_OK;
    }
    memcpy(seed, &c->rng[3 * b], 3 * sizeof(unsigned short));
    return SCFT_OK;
}

static PostArgs post_args(scft_ctx *c, const double *noise_dev)
{
    PostArgs a;
    memset(&a, 0, sizeof(a));
    a.params = c->params;
    a.state = c->state;
    a.chains = c->chains;
    a.blocks = c->blocks;
    a.species = c->species;
    a.nchains = c->nchains;
    a.nblocks = c->nblocks;
    a.n_active = c->der[0].n_active;
    a.B = c->B;
    a.nx = c->nx;
    a.ny = c->ny;
    a.nz = c->nz;
    a.m = c->m;
    a.sm = c->sm;
    a.w = c->w;
    a.phi = c->phi;
    a.raw = c->raw;
    a.mask = c->mask;
    a.bz = c->bz;
    a.field_use = c->field_use;
    a.partial = c->partial;
    a.nparts = c->nparts;
    a.noise = noise_dev;
    a.hist = c->hist;
    a.last = c->last;
    a.hist_cap = c->hist_cap;
    for (int f = 0; f < SCFT_NFIELDS; ++f) a.part0[f] = a.part1[f] = -1;
    for (int k = 0; k < c->nblocks; ++k) {
        const BlockDesc &bd = c->blocks_h[k];
        if (bd.part == 0)
            a.part0[bd.field] = k;
        else
            a.part1[bd.field] = k;
    }
    return a;
}

/* All contour steps of every chain: one launch per axis per step. */
static int launch_steps(scft_ctx *c, const ChainDesc *chains, int nchains_total, int maxlen)
{
    if (c->fused2d || c->fused3d) {
        /* one persistent launch: every chain runs its whole contour loop */
        Step2DArgs a;
        a.chains = chains;
        a.order = (chains == c->chains) ? c->order : nullptr;
        a.state = (chains == c->chains) ? c->state : nullptr;
        a.s = 0;
        a.s_end = maxlen - 1;
        a.sstride = c->sm;
        if (c->fused3d)
            CK(scft_launch_step3d(a, nchains_total, c->stream, 0));
        else
            CK(scft_launch_step2d(c->opt.precision, c->nx, c->nz, a, nchains_total, c->stream, 0, c->wide2d));
        return SCFT_OK;
    }
    const int npass = (int)c->axes.size();
    for (int s = 0; s < maxlen - 1; ++s) {
        for (int pi = 0; pi < npass; ++pi) {
            const Axis &A = c->axes[pi];
            PassArgs pa;
            memset(&pa, 0, sizeof(pa));
            pa.chains = chains;
            pa.state = (chains == c->chains) ? c->state : nullptr;
            pa.nchains = nchains_total;
            pa.s = s;
            pa.first = pi == 0;
            pa.last = pi == npass - 1;
            pa.tile = A.tile;
            pa.sstride = c->sm;
            pa.axis = pi;
            pa.h = A.h;
            pa.even = A.even;
            CK(scft_launch_pass(c->opt.precision, A.g, pa, A.ntiles, c->stream));
        }
    }
    return SCFT_OK;
}

static int launch_iteration(scft_ctx *c, const double *noise_dev, int slot)
{
    PostArgs a = post_args(c, noise_dev);
    CK(scft_post_iter_begin(a, c->opt.precision, c->sms, c->stream));
    if (c->opt.noise_mode == SCFT_NOISE_DRAND48) {
        NoiseArgs na;
        na.state = c->state;
        na.params = c->params;
        na.state_in = c->rng_in;
        na.counts = c->rng_counts;
        na.prefix = c->rng_prefix;
        na.total = c->rng_total;
        na.noise = c->noise;
        na.nchunks = c->rng_chunks;
        na.m = c->m;
        na.sm = c->sm;
        na.nx = c->nx;
        na.ny = c->ny;
        na.nz = c->nz;
        na.B = c->B;
        CK(scft_noise_launch(na, c->stream));
    }
    if (c->timing) CK(cudaEventRecord(c->ev[2 + 2 * slot], c->stream));
    int rc = launch_steps(c, c->chains, c->B * c->nchains, c->maxlen);
    if (rc) return rc;
    if (c->timing) CK(cudaEventRecord(c->ev[3 + 2 * slot], c->stream));
    CK(scft_post_iter_end(a, c->opt.precision, c->sms, c->stream));
    return SCFT_OK;
}

/* Enqueue chunk <= hist_cap iterations on the context's stream, with host
 * noise for them ([chunk][B][n_active][M]) or NULL, and the copy of their
 * records to pinned memory. Nothing waits. */
static int enqueue_chunk(scft_ctx *c, int chunk, const double *noise)
{
    if (c->timing && c->ev.empty()) {
        c->ev.resize(2 + 2 * c->hist_cap);
        for (cudaEvent_t &e : c->ev) CK(cudaEventCreate(&e));
    }
    PostArgs a = post_args(c, nullptr);
    CK(scft_post_mark_start(a, c->stream));
    if (c->timing) CK(cudaEventRecord(c->ev[0], c->stream));
    for (int k = 0; k < chunk; ++k) {
        const double *nd = nullptr;
        if (noise) {
            const size_t m = (size_t)c->m, na = c->der[0].n_active;
            for (int b = 0; b < c->B; ++b)
                for (size_t f = 0; f < na; ++f)
                    CK(cudaMemcpyAsync(c->noise + ((size_t)b * na + f) * c->sm,
                                       noise + ((size_t)k * c->B * na + (size_t)b * na + f) * m, sizeof(double) * m,
                                       cudaMemcpyHostToDevice, c->stream));
            nd = c->noise;
        }
        if (c->opt.use_graph && !c->timing) {
            if (!c->graph_exec) {
                /* the graph always reads noise from c->noise; with no noise the
                 * buffer holds zeros and MF*DT_NOISE == 0 skips it */
                CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
                int rc = launch_iteration(c, c->noise, k);
                cudaGraph_t g = nullptr;
                cudaError_t e = cudaStreamEndCapture(c->stream, &g);
                if (rc) return rc;
                CK(e);
                c->graph = g;
                CK(cudaGraphInstantiate(&c->graph_exec, g, 0));
            }
            CK(cudaGraphLaunch(c->graph_exec, c->stream));
        } else {
            int rc = launch_iteration(c, c->opt.noise_mode == SCFT_NOISE_DRAND48 ? c->noise : nd, k);
            if (rc) return rc;
        }
    }
    if (c->timing) CK(cudaEventRecord(c->ev[1], c->stream));
    CK(cudaMemcpyAsync(c->hist_host, c->hist, sizeof(scft_iter_out) * chunk * c->B, cudaMemcpyDeviceToHost,
                       c->stream));
    if (!c->chunk_done) CK(cudaEventCreateWithFlags(&c->chunk_done, cudaEventDisableTiming));
    CK(cudaEventRecord(c->chunk_done, c->stream));
    c->pending = chunk;
    return SCFT_OK;
}

/* Wait for the enqueued chunk; records to out ([chunk][B], may be NULL). */
static int collect_chunk(scft_ctx *c, scft_iter_out *out)
{
    const int chunk = c->pending;
    c->pending = 0;
    CK(cudaStreamSynchronize(c->stream));
    if (c->timing) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
        c->last_timing.total_ms += ms;
        for (int k = 0; k < chunk; ++k) {
            float pm = 0.f;
            cudaEventElapsedTime(&pm, c->ev[2 + 2 * k], c->ev[3 + 2 * k]);
            c->last_timing.prop_ms += pm;
        }
    }
    c->last_timing.prop_launches += (long)chunk * c->prop_launches_per_iter;
    c->last_timing.kernel_launches += (long)chunk * c->launches_per_iter;
    int status = SCFT_OK;
    for (int k = 0; k < chunk; ++k)
        for (int b = 0; b < c->B; ++b) {
            const scft_iter_out &r = c->hist_host[(size_t)k * c->B + b];
            if (out) out[(size_t)k * c->B + b] = r;
            if (r.status != SCFT_OK) status = r.status;
        }
    if (chunk > 0)
        for (int b = 0; b < c->B; ++b) c->iter[b] = c->hist_host[(size_t)(chunk - 1) * c->B + b].iter;
    if (status != SCFT_OK) {
        if (c->fused2d && scft_step2d_take_fault())
            set_err("non-finite Q, free energy or RMS (a tensor-core wait of the contour loop gave up)");
        else
            set_err("non-finite Q, free energy or RMS");
        return status;
    }
    return SCFT_OK;
}

static int check_iterate(scft_ctx *c, int n, const double *noise)
{
    if (c->pending) {
        set_err("iterations enqueued by scft_iterate_async have not been collected");
        return SCFT_ERR_STATE;
    }
    for (int b = 0; b < c->B; ++b)
        if (!c->fields_set[b]) {
            set_err("instance %d: scft_set_fields was not called", b);
            return SCFT_ERR_STATE;
        }
    if (noise && c->opt.noise_mode == SCFT_NOISE_DRAND48) {
        set_err("this context draws its noise on the device; pass NULL");
        return SCFT_ERR_PARAM;
    }
    if (!noise && c->opt.noise_mode == SCFT_NOISE_HOST) {
        /* without noise arrays every iteration must have MF*DT_NOISE == 0 */
        for (int b = 0; b < c->B; ++b)
            for (int k = 1; k <= n; ++k) {
                const unsigned long it = c->iter[b] + k;
                const double mf = it > (unsigned long)c->surf[b].relaxation ? 0.0 : 1.0;
                if (mf * c->surf[b].dt_noise != 0.0) {
                    set_err("iteration %lu of instance %d adds noise but no noise arrays were passed", it, b);
                    return SCFT_ERR_PARAM;
                }
            }
    }
    return SCFT_OK;
}

extern "C" int scft_iterate(scft_ctx *c, int n, const double *noise, scft_iter_out *out)
{
    if (!c || n < 0) return SCFT_ERR_PARAM;
    cudaSetDevice(c->device);
    int rc = check_iterate(c, n, noise);
    if (rc) return rc;
    c->last_timing = scft_timing{};
    const size_t per_iter = (size_t)c->B * c->der[0].n_active * (size_t)c->m;
    int done = 0;
    while (done < n) {
        const int chunk = (n - done) < c->hist_cap ? (n - done) : c->hist_cap;
        rc = enqueue_chunk(c, chunk, noise ? noise + (size_t)done * per_iter : nullptr);
        if (rc) {
            cudaStreamSynchronize(c->stream);
            c->pending = 0;
            return rc;
        }
        rc = collect_chunk(c, out ? out + (size_t)done * c->B : nullptr);
        if (rc) return rc;
        done += chunk;
    }
    return SCFT_OK;
}

extern "C" int scft_iterate_async(scft_ctx *c, int n)
{
    if (!c || n < 1 || n > SCFT_HIST_CAP) return SCFT_ERR_PARAM;
    cudaSetDevice(c->device);
    int rc = check_iterate(c, n, nullptr);
    if (rc) return rc;
    c->last_timing = scft_timing{};
    rc = enqueue_chunk(c, n, nullptr);
    if (rc) {
        cudaStreamSynchronize(c->stream);
        c->pending = 0;
    }
    return rc;
}

extern "C" int scft_iterate_ready(scft_ctx *c)
{
    if (!c) return SCFT_ERR_PARAM;
    if (!c->pending) return 1;
    cudaSetDevice(c->device);
    const cudaError_t e = cudaEventQuery(c->chunk_done);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) return 0;
    set_err("scft_iterate_ready: %s", cudaGetErrorString(e));
    return SCFT_ERR_CUDA;
}

extern "C" int scft_iterate_wait(scft_ctx *c, scft_iter_out *out)
{
    if (!c) return SCFT_ERR_PARAM;
    cudaSetDevice(c->device);
    return collect_chunk(c, out);
}

extern "C" int scft_get_fields(scft_ctx *c, int b, double *w14)
{
    if (!c || b < 0 || b >= c->B) return SCFT_ERR_PARAM;
    if (!w14) return SCFT_OK;
    cudaSetDevice(c->device);
    for (int f = 0; f < 14; ++f)
        CK(cudaMemcpyAsync(w14 + (size_t)f * c->m, c->w + ((size_t)b * 14 + f) * c->sm, sizeof(double) * c->m,
                           cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SCFT_OK;
}

extern "C" int scft_get_densities(scft_ctx *c, int b, double *phi13, double *phi_tot)
{
    if (!c || b < 0 || b >= c->B) return SCFT_ERR_PARAM;
    cudaSetDevice(c->device);
    if (phi13)
        for (int f = 0; f < 13; ++f)
            CK(cudaMemcpyAsync(phi13 + (size_t)f * c->m, c->phi + ((size_t)b * 14 + f) * c->sm, sizeof(double) * c->m,
                               cudaMemcpyDeviceToHost, c->stream));
    if (phi_tot)
        CK(cudaMemcpyAsync(phi_tot, c->phi + ((size_t)b * 14 + 13) * c->sm, sizeof(double) * c->m,
                           cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SCFT_OK;
}

/* rows of m doubles between a dense host block and the device's sm-strided
 * arrays: one plain copy when the two layouts coincide */
static cudaError_t copy_rows(scft_ctx *c, void *dst, size_t dpitch, const void *src, size_t spitch, size_t rows,
                             cudaMemcpyKind kind)
{
    const size_t width = sizeof(double) * c->m;
    if (dpitch == width && spitch == width) return cudaMemcpyAsync(dst, src, width * rows, kind, c->stream);
    return cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, rows, kind, c->stream);
}

extern "C" int scft_set_fields_all_async(scft_ctx *c, const double *w14_all)
{
    if (!c || !w14_all) return SCFT_ERR_PARAM;
    cudaSetDevice(c->device);
    CK(copy_rows(c, c->w, sizeof(double) * c->sm, w14_all, sizeof(double) * c->m, (size_t)c->B * 14,
                 cudaMemcpyHostToDevice));
    for (int b = 0; b < c->B; ++b) c->fields_set[b] = 1;
    return SCFT_OK;
}

extern "C" int scft_get_fields_all_async(scft_ctx *c, double *w14_all)
{
    if (!c || !w14_all) return SCFT_ERR_PARAM;
    cudaSetDevice(c->device);
    CK(copy_rows(c, w14_all, sizeof(double) * c->m, c->w, sizeof(double) * c->sm, (size_t)c->B * 14,
                 cudaMemcpyDeviceToHost));
    return SCFT_OK;
}

extern "C" int scft_get_densities_all_async(scft_ctx *c, double *phi14_all)
{
    if (!c || !phi14_all) return SCFT_ERR_PARAM;
    cudaSetDevice(c->device);
    CK(copy_rows(c, phi14_all, sizeof(double) * c->m, c->phi, sizeof(double) * c->sm, (size_t)c->B * 14,
                 cudaMemcpyDeviceToHost));
    return SCFT_OK;
}

extern "C" int scft_sync(scft_ctx *c)
{
    if (!c) return SCFT_ERR_PARAM;
    cudaSetDevice(c->device);
    CK(cudaStreamSynchronize(c->stream));
    return SCFT_OK;
}

extern "C" int scft_set_fields_all(scft_ctx *c, const double *w14_all)
{
    int rc = scft_set_fields_all_async(c, w14_all);
    return rc ? rc : scft_sync(c);
}

extern "C" int scft_get_fields_all(scft_ctx *c, double *w14_all)
{
    int rc = scft_get_fields_all_async(c, w14_all);
    return rc ? rc : scft_sync(c);
}

extern "C" int scft_get_densities_all(scft_ctx *c, double *phi14_all)
{
    int rc = scft_get_densities_all_async(c, phi14_all);
    return rc ? rc : scft_sync(c);
}

extern "C" int scft_propagate(scft_ctx *c, const double *q0, const double *w, int steps, double *q_out)
{
    if (!c || !q0 || !w || !q_out || steps < 0) return SCFT_ERR_PARAM;
    cudaSetDevice(c->device);
    const size_t sm = c->sm, m = c->m;
    double *wd = nullptr, *qd = nullptr;
    void *q = nullptr, *tmp = nullptr, *bzd = nullptr;
    ChainDesc *cdd = nullptr;
    int rc = SCFT_OK;
    cudaError_t e = cudaSuccess;
    e = cudaMalloc(&wd, sizeof(double) * sm);
    if (e == cudaSuccess) e = cudaMalloc(&qd, sizeof(double) * sm * (steps + 1));
    if (e == cudaSuccess) e = cudaMalloc(&q, (size_t)c->psize * sm * (steps + 1));
    if (e == cudaSuccess) e = cudaMalloc(&tmp, (size_t)c->psize * sm);
    if (e == cudaSuccess) e = cudaMalloc(&bzd, (size_t)c->psize * sm);
    if (e == cudaSuccess) e = cudaMalloc(&cdd, sizeof(ChainDesc));
    if (e != cudaSuccess) {
        set_err("scft_propagate: allocation failed: %s", cudaGetErrorString(e));
        rc = SCFT_ERR_OOM;
    }
    if (rc == SCFT_OK) {
        ChainDesc cd;
        memset(&cd, 0, sizeof(cd));
        cd.q = q;
        cd.tmp = tmp;
        cd.b0 = bzd;
        cd.b1 = bzd;
        cd.seg_end = steps + 1;
        cd.len = steps + 1;
        cd.ops = c->ops + c->ops_of[0];
        e = cudaMemcpyAsync(cdd, &cd, sizeof(cd), cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(wd, w, sizeof(double) * m, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(qd, q0, sizeof(double) * m, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = scft_boltz_one(c->opt.precision, wd, bzd, c->der[0].ds, (long)m, c->stream);
        if (e == cudaSuccess) e = scft_convert(c->opt.precision, qd, q, (long)m, 1, c->stream);
        if (e != cudaSuccess) {
            set_err("scft_propagate: %s", cudaGetErrorString(e));
            rc = SCFT_ERR_CUDA;
        }
    }
    if (rc == SCFT_OK) rc = launch_steps(c, cdd, 1, steps + 1);
    if (rc == SCFT_OK) {
        e = scft_convert(c->opt.precision, (const double *)q, qd, (long)(sm * (steps + 1)), 0, c->stream);
        for (int s = 0; s <= steps && e == cudaSuccess; ++s)
            e = cudaMemcpyAsync(q_out + (size_t)s * m, qd + (size_t)s * sm, sizeof(double) * m, cudaMemcpyDeviceToHost,
                                c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) {
            set_err("scft_propagate: %s", cudaGetErrorString(e));
            rc = SCFT_ERR_CUDA;
        }
    }
    cudaStreamSynchronize(c->stream);
    cudaFree(wd);
    cudaFree(qd);
    cudaFree(q);
    cudaFree(tmp);
    cudaFree(bzd);
    cudaFree(cdd);
    return rc;
}

extern "C" int scft_density(scft_ctx *c, const double *qf, const double *qb, int len, int start, int stop, double q,
                            double *phi)
{
    if (!c || !qf || !qb || !phi || len < 2 || start < 0 || stop <= start || stop > len - 1 || !(q != 0.0))
        return SCFT_ERR_PARAM;
    cudaSetDevice(c->device);
    const size_t sm = c->sm, m = c->m, ps = (size_t)c->psize;
    double *stage = nullptr, *raw = nullptr;
    void *qfd = nullptr, *qbd = nullptr;
    ChainDesc *cdd = nullptr;
    BlockDesc *bdd = nullptr;
    InstState *std_ = nullptr;
    int rc = SCFT_OK;
    cudaError_t e = cudaMalloc(&stage, sizeof(double) * sm * len);
    if (e == cudaSuccess) e = cudaMalloc(&raw, sizeof(double) * sm);
    if (e == cudaSuccess) e = cudaMalloc(&qfd, ps * sm * len);
    if (e == cudaSuccess) e = cudaMalloc(&qbd, ps * sm * len);
    if (e == cudaSuccess) e = cudaMalloc(&cdd, 2 * sizeof(ChainDesc));
    if (e == cudaSuccess) e = cudaMalloc(&bdd, sizeof(BlockDesc));
    if (e == cudaSuccess) e = cudaMalloc(&std_, sizeof(InstState));
    if (e != cudaSuccess) {
        set_err("scft_density: allocation failed: %s", cudaGetErrorString(e));
        rc = SCFT_ERR_OOM;
    }
    if (rc == SCFT_OK) {
        ChainDesc cd[2];
        memset(cd, 0, sizeof(cd));
        cd[0].q = qfd;
        cd[1].q = qbd;
        cd[0].len = cd[1].len = len;
        BlockDesc bd = {0, 1, start, stop, len, 0, 0, 0};
        InstState st;
        memset(&st, 0, sizeof(st));
        e = cudaMemcpyAsync(cdd, cd, sizeof(cd), cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(bdd, &bd, sizeof(bd), cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(std_, &st, sizeof(st), cudaMemcpyHostToDevice, c->stream);
        const double *src[2] = {qf, qb};
        void *dst[2] = {qfd, qbd};
        for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
            e = cudaMemcpy2DAsync(stage, sizeof(double) * sm, src[k], sizeof(double) * m, sizeof(double) * m, len,
                                  cudaMemcpyHostToDevice, c->stream);
            if (e == cudaSuccess) e = scft_convert(c->opt.precision, stage, dst[k], (long)(sm * len), 1, c->stream);
        }
        if (e == cudaSuccess) {
            PostArgs a;
            memset(&a, 0, sizeof(a));
            a.state = std_;
            a.chains = cdd;
            a.blocks = bdd;
            a.nchains = 2;
            a.nblocks = 1;
            a.B = 1;
            a.m = c->m;
            a.sm = c->sm;
            a.raw = raw;
            e = scft_density_launch(a, c->opt.precision, c->sms, c->stream);
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(phi, raw, sizeof(double) * m, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) {
            set_err("scft_density: %s", cudaGetErrorString(e));
            rc = SCFT_ERR_CUDA;
        }
    }
    if (rc == SCFT_OK) {
        /* (sum / 3) * (DS_EFF / Q), SCFT.c:2298-2299 */
        const double f = (1.0 / (len - 1)) / q;
        for (size_t i = 0; i < m; ++i) phi[i] = (phi[i] / 3.0) * f;
    }
    cudaStreamSynchronize(c->stream);
    cudaFree(stage);
    cudaFree(raw);
    cudaFree(qfd);
    cudaFree(qbd);
    cudaFree(cdd);
    cudaFree(bdd);
    cudaFree(std_);
    return rc;
}

extern "C" int scft_enable_timing(scft_ctx *c, int on)
{
    if (!c) return SCFT_ERR_PARAM;
    c->timing = on ? 1 : 0;
    return SCFT_OK;
}

extern "C" int scft_get_timing(const scft_ctx *c, scft_timing *t)
{
    if (!c || !t) return SCFT_ERR_PARAM;
    *t = c->last_timing;
    t->fused_chain = c->fused2d ? 1 : (c->fused3d ? 2 : 0);
    t->threads_per_line = c->fused2d && c->wide2d ? 2 : 1;
    return SCFT_OK;
}

/* ------------------------------------------------- internal hooks */
/* Used by scft_noalloc.cu: context facts and the contour-step launcher on a
 * caller-provided chain descriptor. */
int scft_ctx_info(const scft_ctx *c, int *device, int *prec, long *m, long *sm, double *ds, cudaStream_t *st,
                  const InstOps **ops0)
{
    if (!c) return SCFT_ERR_PARAM;
    *ops0 = c->ops + c->ops_of[0];
    *device = c->device;
    *prec = c->opt.precision;
    *m = c->m;
    *sm = c->sm;
    *ds = c->der[0].ds;
    *st = c->stream;
    return SCFT_OK;
}

int scft_ctx_run_chain(scft_ctx *c, const ChainDesc *dev_desc, int len) { return launch_steps(c, dev_desc, 1, len); }

void scft_set_error(const char *msg) { set_err("%s", msg); }
