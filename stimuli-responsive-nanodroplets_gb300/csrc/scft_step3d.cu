/*
 * scft_step3d.cu — the whole contour loop of one chain on a 64^3 periodic grid
 * (MASK 0) in one thread-block cluster, FP32:
 *   q_{s+1} = b . Kz Ky Kx (b . q_s),   b = exp(-DS w / 2)
 * (funPDESolver / funPDESolver_periodic, SCFT.c:2310-2412, :2474-2525).
 *
 * The 1 MB slice of a chain lives in the shared memory of an 8-CTA cluster for
 * the chain's whole contour loop: CTA r owns the x planes 8r .. 8r+7 (row pitch
 * 65 floats, plane pitch 64*65+4, so the column and row walks below are free of
 * bank conflicts). Per contour step only q_{s+1} goes to HBM (for the
 * densities) and b is read once; the factor is separable and real and even
 * per axis, so each axis is applied as a real circulant with two real lines
 * packed into one complex line:
 *   z, y (local): one thread per packed line (rows p, p+32 / columns p, p+32 of
 *     one plane), a 64-point FFT in registers (8 x 8 two-factor), E(k)/64, the
 *     inverse FFT, back to shared memory;
 *   x (across the cluster): x = 8c + l with c the owning CTA and l its local
 *     plane; CTA r handles the rows y in [8r, 8r+8) of every plane in two
 *     chunks of four rows: 8-point DFTs over c read straight from the owners'
 *     shared memory (DSMEM), the twiddle W_64^(l k1), a transpose through a
 *     local buffer, 8-point DFTs over l, E(k)/64, the inverse, the transpose
 *     back and the inverse 8-point DFTs over c written back to the owners.
 * Two cluster barriers per step bracket the x phase; everything else is
 * CTA-local. All control flow is uniform over the cluster (one chain per
 * cluster), and a last cluster barrier keeps every CTA's shared memory alive
 * until no other CTA can address it.
 */
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "scft_internal.h"

namespace cg = cooperative_groups;

namespace {

constexpr int N3 = 64;            /* points per axis */
constexpr int CL = 8;             /* CTAs per cluster */
constexpr int PL = N3 / CL;       /* x planes per CTA */
constexpr int RP = N3 + 1;        /* row pitch (floats) */
constexpr int PP = N3 * RP + 4;   /* plane pitch (floats) */
constexpr int NT = 256;           /* threads per CTA: 8 warps x 32 lanes */
constexpr int YC = 4;             /* rows per x-phase chunk */
constexpr int RSTRIDE = 65;       /* complex slots per (row, lane) in the transpose buffer */

struct C2 {
    float x, y;
};

__device__ __forceinline__ C2 c_add(C2 a, C2 b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ C2 c_sub(C2 a, C2 b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ C2 c_mul(C2 a, C2 b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
/* a * conj(b) */
__device__ __forceinline__ C2 c_mulc(C2 a, C2 b) { return {a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y}; }
template <bool INV>
__device__ __forceinline__ C2 c_si(C2 a) /* sign*i*a, sign = -1 forward */
{
    return INV ? C2{-a.y, a.x} : C2{a.y, -a.x};
}

/* cos and sin of 2 pi k / 64 */
__constant__ float c_cos64[64] = {
    1.000000000e+00f, 9.951847267e-01f, 9.807852804e-01f, 9.569403357e-01f, 9.238795325e-01f, 8.819212643e-01f,
    8.314696123e-01f, 7.730104534e-01f, 7.071067812e-01f, 6.343932842e-01f, 5.555702330e-01f, 4.713967368e-01f,
    3.826834324e-01f, 2.902846773e-01f, 1.950903220e-01f, 9.801714033e-02f, 6.123233996e-17f, -9.801714033e-02f,
    -1.950903220e-01f, -2.902846773e-01f, -3.826834324e-01f, -4.713967368e-01f, -5.555702330e-01f,
    -6.343932842e-01f, -7.071067812e-01f, -7.730104534e-01f, -8.314696123e-01f, -8.819212643e-01f,
    -9.238795325e-01f, -9.569403357e-01f, -9.807852804e-01f, -9.951847267e-01f, -1.000000000e+00f,
    -9.951847267e-01f, -9.807852804e-01f, -9.569403357e-01f, -9.238795325e-01f, -8.819212643e-01f,
    -8.314696123e-01f, -7.730104534e-01f, -7.071067812e-01f, -6.343932842e-01f, -5.555702330e-01f,
    -4.713967368e-01f, -3.826834324e-01f, -2.902846773e-01f, -1.950903220e-01f, -9.801714033e-02f,
    -1.836970199e-16f, 9.801714033e-02f, 1.950903220e-01f, 2.902846773e-01f, 3.826834324e-01f, 4.713967368e-01f,
    5.555702330e-01f, 6.343932842e-01f, 7.071067812e-01f, 7.730104534e-01f, 8.314696123e-01f, 8.819212643e-01f,
    9.238795325e-01f, 9.569403357e-01f, 9.807852804e-01f, 9.951847267e-01f};
__constant__ float c_sin64[64] = {
    0.000000000e+00f, 9.801714033e-02f, 1.950903220e-01f, 2.902846773e-01f, 3.826834324e-01f, 4.713967368e-01f,
    5.555702330e-01f, 6.343932842e-01f, 7.071067812e-01f, 7.730104534e-01f, 8.314696123e-01f, 8.819212643e-01f,
    9.238795325e-01f, 9.569403357e-01f, 9.807852804e-01f, 9.951847267e-01f, 1.000000000e+00f, 9.951847267e-01f,
    9.807852804e-01f, 9.569403357e-01f, 9.238795325e-01f, 8.819212643e-01f, 8.314696123e-01f, 7.730104534e-01f,
    7.071067812e-01f, 6.343932842e-01f, 5.555702330e-01f, 4.713967368e-01f, 3.826834324e-01f, 2.902846773e-01f,
    1.950903220e-01f, 9.801714033e-02f, 1.224646799e-16f, -9.801714033e-02f, -1.950903220e-01f,
    -2.902846773e-01f, -3.826834324e-01f, -4.713967368e-01f, -5.555702330e-01f, -6.343932842e-01f,
    -7.071067812e-01f, -7.730104534e-01f, -8.314696123e-01f, -8.819212643e-01f, -9.238795325e-01f,
    -9.569403357e-01f, -9.807852804e-01f, -9.951847267e-01f, -1.000000000e+00f, -9.951847267e-01f,
    -9.807852804e-01f, -9.569403357e-01f, -9.238795325e-01f, -8.819212643e-01f, -8.314696123e-01f,
    -7.730104534e-01f, -7.071067812e-01f, -6.343932842e-01f, -5.555702330e-01f, -4.713967368e-01f,
    -3.826834324e-01f, -2.902846773e-01f, -1.950903220e-01f, -9.801714033e-02f};

/* W_64^e = exp(sign 2 pi i e / 64), sign = -1 forward */
template <bool INV>
__device__ __forceinline__ C2 w64(int e)
{
    e &= 63;
    return {c_cos64[e], INV ? c_sin64[e] : -c_sin64[e]};
}

/* 4- and 8-point DFTs, natural order in and out */
template <bool INV>
__device__ __forceinline__ void dft4(C2 *v)
{
    const C2 b0 = c_add(v[0], v[2]), b1 = c_sub(v[0], v[2]);
    const C2 b2 = c_add(v[1], v[3]), b3 = c_si<INV>(c_sub(v[1], v[3]));
    v[0] = c_add(b0, b2);
    v[1] = c_add(b1, b3);
    v[2] = c_sub(b0, b2);
    v[3] = c_sub(b1, b3);
}

template <bool INV>
__device__ __forceinline__ void dft8(C2 *v)
{
    /* 8 = 4 x 2: 4-point DFTs over the even and odd inputs, twiddle W_8^k1, 2-point DFTs */
    C2 e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    dft4<INV>(e);
    dft4<INV>(o);
    const float h = 0.70710678118654752f;
    const C2 o1 = INV ? C2{h * (o[1].x - o[1].y), h * (o[1].x + o[1].y)} : C2{h * (o[1].x + o[1].y), h * (o[1].y - o[1].x)};
    const C2 o2 = c_si<INV>(o[2]);
    const C2 o3 = INV ? C2{-h * (o[3].x + o[3].y), h * (o[3].x - o[3].y)} : C2{h * (o[3].y - o[3].x), -h * (o[3].x + o[3].y)};
    v[0] = c_add(e[0], o[0]);
    v[4] = c_sub(e[0], o[0]);
    v[1] = c_add(e[1], o1);
    v[5] = c_sub(e[1], o1);
    v[2] = c_add(e[2], o2);
    v[6] = c_sub(e[2], o2);
    v[3] = c_add(e[3], o3);
    v[7] = c_sub(e[3], o3);
}

/* 64-point DFT, natural order in and out: 8-point DFTs over stride-8 inputs,
 * twiddles W_64^(b k1), 8-point DFTs; output k = k1 + 8 k2 */
template <bool INV>
__device__ __forceinline__ void fft64(C2 *v)
{
    C2 t[64];
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        C2 col[8];
#pragma unroll
        for (int a = 0; a < 8; ++a) col[a] = v[8 * a + b];
        dft8<INV>(col);
#pragma unroll
        for (int k1 = 0; k1 < 8; ++k1) t[b * 8 + k1] = (b * k1 == 0) ? col[k1] : c_mul(col[k1], w64<INV>(b * k1));
    }
#pragma unroll
    for (int k1 = 0; k1 < 8; ++k1) {
        C2 row[8];
#pragma unroll
        for (int b = 0; b < 8; ++b) row[b] = t[b * 8 + k1];
        dft8<INV>(row);
#pragma unroll
        for (int k2 = 0; k2 < 8; ++k2) v[k1 + 8 * k2] = row[k2];
    }
}

/* real circulant along one local axis for two packed lines: x0[i*st], x1[i*st] */
__device__ __forceinline__ void conv_line(float *x0, float *x1, int st, const float *E)
{
    C2 v[64];
#pragma unroll
    for (int i = 0; i < 64; ++i) v[i] = C2{x0[i * st], x1[i * st]};
    fft64<false>(v);
#pragma unroll
    for (int k = 0; k < 64; ++k) {
        const float f = E[k];
        v[k].x *= f;
        v[k].y *= f;
    }
    fft64<true>(v);
#pragma unroll
    for (int i = 0; i < 64; ++i) {
        x0[i * st] = v[i].x;
        x1[i * st] = v[i].y;
    }
}

} // namespace

constexpr size_t STEP3D_Q_BYTES = sizeof(float) * PL * PP;
constexpr size_t STEP3D_R_BYTES = sizeof(C2) * YC * 32 * RSTRIDE;
constexpr size_t STEP3D_E_BYTES = sizeof(float) * 3 * N3;
constexpr size_t STEP3D_SMEM = STEP3D_Q_BYTES + STEP3D_R_BYTES + STEP3D_E_BYTES;

__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(NT, 1) k_chain3d(Step2DArgs a)
{
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int slot = blockIdx.x / CL;
    const ChainDesc cd = a.chains[a.order ? a.order[slot] : slot];
    /* uniform over the cluster: every CTA reads the same descriptor and state */
    if (a.state && a.state[cd.instance].done) return;
    const int s_end = a.s_end < cd.len - 1 ? a.s_end : cd.len - 1;
    if (a.s >= s_end) return;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *Q = reinterpret_cast<float *>(smem_raw);
    C2 *R = reinterpret_cast<C2 *>(smem_raw + STEP3D_Q_BYTES);
    float *E = reinterpret_cast<float *>(smem_raw + STEP3D_Q_BYTES + STEP3D_R_BYTES); /* x, y, z factors */

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long own = (long)rank * PL * N3 * N3; /* first element of this CTA's planes in a slice */

    for (int e = tid; e < 3 * N3; e += NT) E[e] = reinterpret_cast<const float *>(cd.ops->spec[e / N3])[e % N3];

    /* Q = b_s . q_s */
    {
        const float4 *q4 = reinterpret_cast<const float4 *>(reinterpret_cast<const float *>(cd.q) +
                                                            (long)a.s * a.sstride + own);
        const float4 *b4 = reinterpret_cast<const float4 *>(
            reinterpret_cast<const float *>(a.s < cd.seg_end ? cd.b0 : cd.b1) + own);
#pragma unroll 4
        for (int e4 = tid; e4 < PL * N3 * N3 / 4; e4 += NT) {
            const float4 qv = q4[e4], bv = b4[e4];
            const int e = 4 * e4, xl = e >> 12, y = (e >> 6) & 63, z = e & 63;
            float *d = Q + xl * PP + y * RP + z;
            d[0] = qv.x * bv.x;
            d[1] = qv.y * bv.y;
            d[2] = qv.z * bv.z;
            d[3] = qv.w * bv.w;
        }
    }
    __syncthreads();

    for (int s = a.s; s < s_end; ++s) {
        /* z: plane `warp`, rows lane and lane+32 */
        {
            float *r0 = Q + warp * PP + lane * RP;
            conv_line(r0, r0 + 32 * RP, 1, E + 2 * N3);
        }
        __syncthreads();
        /* y: plane `warp`, columns lane and lane+32 */
        {
            float *c0 = Q + warp * PP + lane;
            conv_line(c0, c0 + 32, RP, E + N3);
        }
        cl.sync(); /* every CTA's y/z work is done before any x line is read */
        /* x across the cluster, rows y in [8 rank, 8 rank + 8), packed columns (lane, lane+32) */
        for (int chunk = 0; chunk < PL / YC; ++chunk) {
            const int y0 = PL * rank + YC * chunk;
            {
                const int l = warp; /* local plane of the inputs this thread combines */
#pragma unroll
                for (int j = 0; j < YC; ++j) {
                    const int off = l * PP + (y0 + j) * RP + lane;
                    C2 v[8];
#pragma unroll
                    for (int c = 0; c < CL; ++c) {
                        const float *rq = cl.map_shared_rank(Q, c);
                        v[c] = C2{rq[off], rq[off + 32]};
                    }
                    dft8<false>(v); /* over c -> k1 */
                    C2 *rr = R + (j * 32 + lane) * RSTRIDE;
#pragma unroll
                    for (int k1 = 0; k1 < 8; ++k1) rr[k1 * 8 + l] = (k1 == 0) ? v[0] : c_mul(v[k1], w64<false>(l * k1));
                }
            }
            __syncthreads();
            {
                const int k1 = warp;
#pragma unroll
                for (int j = 0; j < YC; ++j) {
                    C2 *rr = R + (j * 32 + lane) * RSTRIDE + k1 * 8;
                    C2 v[8];
#pragma unroll
                    for (int l = 0; l < 8; ++l) v[l] = rr[l];
                    dft8<false>(v); /* over l -> k2 */
#pragma unroll
                    for (int k2 = 0; k2 < 8; ++k2) {
                        const float f = E[k1 + 8 * k2];
                        v[k2].x *= f;
                        v[k2].y *= f;
                    }
                    dft8<true>(v); /* k2 -> l */
#pragma unroll
                    for (int l = 0; l < 8; ++l) rr[l] = (l == 0) ? v[0] : c_mulc(v[l], w64<false>(l * k1));
                }
            }
            __syncthreads();
            {
                const int l = warp;
#pragma unroll
                for (int j = 0; j < YC; ++j) {
                    const C2 *rr = R + (j * 32 + lane) * RSTRIDE;
                    C2 v[8];
#pragma unroll
                    for (int k1 = 0; k1 < 8; ++k1) v[k1] = rr[k1 * 8 + l];
                    dft8<true>(v); /* k1 -> c */
                    const int off = l * PP + (y0 + j) * RP + lane;
#pragma unroll
                    for (int c = 0; c < CL; ++c) {
                        float *rq = cl.map_shared_rank(Q, c);
                        rq[off] = v[c].x;
                        rq[off + 32] = v[c].y;
                    }
                }
            }
            __syncthreads(); /* the transpose buffer is reused by the next chunk */
        }
        cl.sync(); /* every x line is back in its owner's planes */
        /* q_{s+1} = b_s . y to HBM; the next step starts from b_{s+1} . q_{s+1} */
        {
            const float4 *b4 = reinterpret_cast<const float4 *>(
                reinterpret_cast<const float *>(s < cd.seg_end ? cd.b0 : cd.b1) + own);
            const bool more = s + 1 < s_end;
            const float *bn = reinterpret_cast<const float *>(s + 1 < cd.seg_end ? cd.b0 : cd.b1);
            const bool same = bn == reinterpret_cast<const float *>(s < cd.seg_end ? cd.b0 : cd.b1);
            const float4 *bn4 = reinterpret_cast<const float4 *>(bn + own);
            float4 *o4 = reinterpret_cast<float4 *>(reinterpret_cast<float *>(cd.q) + (long)(s + 1) * a.sstride + own);
#pragma unroll 4
            for (int e4 = tid; e4 < PL * N3 * N3 / 4; e4 += NT) {
                const float4 bv = b4[e4];
                const int e = 4 * e4, xl = e >> 12, y = (e >> 6) & 63, z = e & 63;
                float *d = Q + xl * PP + y * RP + z;
                const float4 o = {d[0] * bv.x, d[1] * bv.y, d[2] * bv.z, d[3] * bv.w};
                o4[e4] = o;
                if (more) {
                    const float4 nb = same ? bv : bn4[e4];
                    d[0] = o.x * nb.x;
                    d[1] = o.y * nb.y;
                    d[2] = o.z * nb.z;
                    d[3] = o.w * nb.w;
                }
            }
        }
        __syncthreads();
    }
    cl.sync(); /* no CTA leaves while another could still address its shared memory */
}

size_t scft_step3d_smem(int prec, int nx, int ny, int nz)
{
    if (prec != SCFT_PREC_FP32 || nx != N3 || ny != N3 || nz != N3) return 0;
    return STEP3D_SMEM;
}

/* configure = 1: raise the shared-memory limit and check that an 8-CTA cluster
 * with this footprint can be resident (returns cudaErrorNotSupported if not). */
cudaError_t scft_launch_step3d(const Step2DArgs &a, int nchains, cudaStream_t st, int configure)
{
    if (configure) {
        cudaError_t e = cudaFuncSetAttribute(k_chain3d, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)STEP3D_SMEM);
        if (e != cudaSuccess) return e;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(CL, 1, 1);
        cfg.blockDim = dim3(NT, 1, 1);
        cfg.dynamicSmemBytes = STEP3D_SMEM;
        cudaLaunchAttribute attr;
        attr.id = cudaLaunchAttributeClusterDimension;
        attr.val.clusterDim.x = CL;
        attr.val.clusterDim.y = 1;
        attr.val.clusterDim.z = 1;
        cfg.attrs = &attr;
        cfg.numAttrs = 1;
        int nclusters = 0;
        e = cudaOccupancyMaxActiveClusters(&nclusters, k_chain3d, &cfg);
        if (e != cudaSuccess) return e;
        return nclusters > 0 ? cudaSuccess : cudaErrorNotSupported;
    }
    if (nchains <= 0) return cudaSuccess;
    k_chain3d<<<dim3(nchains * CL), dim3(NT), STEP3D_SMEM, st>>>(a);
    return cudaGetLastError();
}
