/*
 * scft_step3d.cu — the whole contour loop of one chain on a 64^3 periodic grid
 * (MASK 0) in one thread-block cluster, FP32:
 *   q_{s+1} = b . Kz Ky Kx (b . q_s),   b = exp(-DS w / 2)
 * (funPDESolver / funPDESolver_periodic, SCFT.c:2310-2412, :2474-2525).
 *
 * The 1 MB slice of a chain lives in the shared memory of an 8-CTA cluster for
 * the chain's whole contour loop, as 8 planes of 64 rows of 64 z values per CTA
 * (row pitch 68 floats: every row starts on a 16-byte boundary, so rows move as
 * 128-bit words, and a quarter-warp walking 8 rows side by side in 128-bit
 * steps touches 8 different bank groups; column walks are conflict-free for
 * any pitch). Two distributions alternate:
 *   D1: CTA r holds x in [8r, 8r+8) as planes, y as rows;
 *   D2: CTA r holds y in [8r, 8r+8) as planes, x as rows.
 * The factor is separable, real and even per axis, so each axis is applied as
 * a real circulant with two real lines packed into one complex line, one
 * thread per packed line, a 64-point FFT in registers (8 x 8 two-factor),
 * E(k)/64 and the inverse FFT. z lines and row lines are local in both
 * distributions, so a step starting in D1 applies z and y, moves to D2 (one
 * all-to-all through distributed shared memory), applies x, and the next step
 * does z and x, moves back and applies y. Per step: one exchange (each CTA
 * pulls 7/8 of its new contents into registers as 128-bit words, a cluster
 * barrier, writes them to its own planes), two cluster barriers, and to HBM only q_{s+1} (for the
 * densities) with b read once. All control flow is uniform over the cluster
 * (one chain per cluster), and a last cluster barrier keeps every CTA's shared
 * memory alive until no other CTA can address it.
 */
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "scft_internal.h"

namespace cg = cooperative_groups;

namespace {

constexpr int N3 = 64;            /* points per axis */
constexpr int CL = 8;             /* CTAs per cluster */
constexpr int PL = N3 / CL;       /* x planes per CTA */
constexpr int RP = N3 + 4;        /* row pitch (floats), a multiple of 4 */
constexpr int PP = N3 * RP;       /* plane pitch (floats) */
constexpr int RP4 = RP / 4, PP4 = PP / 4; /* the same in float4 */
constexpr int NT = 256;           /* threads per CTA: 8 warps x 32 lanes */
constexpr int UB = 16;            /* float4 loads in flight per thread in the pointwise phases */

struct C2 {
    float x, y;
};

/* complex add and subtract as one packed f32x2 instruction each */
__device__ __forceinline__ C2 c_add(C2 a, C2 b)
{
    C2 r;
    asm("{\n\t.reg .b64 pa, pb, pr;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "add.rn.f32x2 pr, pa, pb;\n\tmov.b64 {%0, %1}, pr;\n\t}"
        : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ C2 c_sub(C2 a, C2 b)
{
    C2 r;
    asm("{\n\t.reg .b64 pa, pb, pr;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "sub.rn.f32x2 pr, pa, pb;\n\tmov.b64 {%0, %1}, pr;\n\t}"
        : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ C2 c_mul(C2 a, C2 b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
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

/* real circulant along one local axis for two packed lines: x0[i*ST], x1[i*ST]
 * (ST = 1: the lines are rows and move as 128-bit words). The inverse transform
 * is the forward one on the conjugate (conj(F(conj Y))), so one copy of the
 * 64-point FFT code, run as a loop of two passes, serves both directions. */
template <int ST>
__device__ __forceinline__ void conv_line(float *x0, float *x1, const float *E)
{
    C2 v[64];
    if constexpr (ST == 1) {
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const float4 a = reinterpret_cast<const float4 *>(x0)[i], b = reinterpret_cast<const float4 *>(x1)[i];
            v[4 * i] = C2{a.x, b.x};
            v[4 * i + 1] = C2{a.y, b.y};
            v[4 * i + 2] = C2{a.z, b.z};
            v[4 * i + 3] = C2{a.w, b.w};
        }
    } else {
#pragma unroll
        for (int i = 0; i < 64; ++i) v[i] = C2{x0[i * ST], x1[i * ST]};
    }
#pragma unroll 1
    for (int pass = 0; pass < 2; ++pass) {
        fft64<false>(v);
        if (pass == 0) {
#pragma unroll
            for (int k = 0; k < 64; ++k) {
                const float f = E[k];
                v[k] = C2{v[k].x * f, -(v[k].y * f)}; /* E(k)/64, then conjugate */
            }
        }
    }
    if constexpr (ST == 1) {
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            reinterpret_cast<float4 *>(x0)[i] = make_float4(v[4 * i].x, v[4 * i + 1].x, v[4 * i + 2].x, v[4 * i + 3].x);
            reinterpret_cast<float4 *>(x1)[i] =
                make_float4(-v[4 * i].y, -v[4 * i + 1].y, -v[4 * i + 2].y, -v[4 * i + 3].y);
        }
    } else {
#pragma unroll
        for (int i = 0; i < 64; ++i) {
            x0[i * ST] = v[i].x;
            x1[i * ST] = -v[i].y;
        }
    }
}

} // namespace

constexpr size_t STEP3D_Q_BYTES = sizeof(float) * PL * PP;
constexpr size_t STEP3D_E_BYTES = sizeof(float) * 3 * N3;
constexpr size_t STEP3D_SMEM = STEP3D_Q_BYTES + STEP3D_E_BYTES;

/* global index of element e (= plane*4096 + row*64 + z) of CTA `rank` in distribution d */
__device__ __forceinline__ long g_index(int e, int rank, int d)
{
    const int p = e >> 12, r = (e >> 6) & 63, z = e & 63;
    return d == 0 ? (long)(PL * rank + p) * (N3 * N3) + r * N3 + z
                  : (long)r * (N3 * N3) + (PL * rank + p) * N3 + z;
}

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
    float *E = reinterpret_cast<float *>(smem_raw + STEP3D_Q_BYTES); /* x, y, z factors */

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int e = tid; e < 3 * N3; e += NT) E[e] = reinterpret_cast<const float *>(cd.ops->spec[e / N3])[e % N3];

    /* Q = b_s . q_s in D1 */
    {
        const float *q = reinterpret_cast<const float *>(cd.q) + (long)a.s * a.sstride;
        const float *b = reinterpret_cast<const float *>(a.s < cd.seg_end ? cd.b0 : cd.b1);
        for (int base = tid; base < PL * N3 * N3 / 4; base += NT * UB) {
            float4 qv[UB], bv[UB];
#pragma unroll
            for (int u = 0; u < UB; ++u) {
                const long g = g_index(4 * (base + u * NT), rank, 0);
                qv[u] = __ldg(reinterpret_cast<const float4 *>(q + g));
                bv[u] = __ldg(reinterpret_cast<const float4 *>(b + g));
            }
#pragma unroll
            for (int u = 0; u < UB; ++u) {
                const int e = 4 * (base + u * NT);
                float4 *dq = reinterpret_cast<float4 *>(Q + (e >> 12) * PP + ((e >> 6) & 63) * RP + (e & 63));
                *dq = make_float4(qv[u].x * bv[u].x, qv[u].y * bv[u].y, qv[u].z * bv[u].z, qv[u].w * bv[u].w);
            }
        }
    }
    __syncthreads();

    int d = 0; /* current distribution */
    for (int s = a.s; s < s_end; ++s) {
        /* z lines: plane `warp`, rows lane and lane+32 */
        {
            float *r0 = Q + warp * PP + lane * RP;
            conv_line<1>(r0, r0 + 32 * RP, E + 2 * N3);
        }
        __syncthreads();
        /* row lines (y in D1, x in D2): plane `warp`, columns lane and lane+32 */
        {
            float *c0 = Q + warp * PP + lane;
            conv_line<RP>(c0, c0 + 32, E + (d == 0 ? N3 : 0));
        }
        cl.sync(); /* every CTA's planes are final for this half of the step */
        /* exchange: (CTA c, plane p, row 8 rank + j) -> (this CTA, plane j, row 8 c + p); warp w
         * pulls everything this CTA receives from CTA w: 64 rows of 16 128-bit words, two rows
         * per warp-wide load, 32 words per thread in registers */
        {
            const float4 *src = reinterpret_cast<const float4 *>(cl.map_shared_rank(Q, warp));
            float4 *dst = reinterpret_cast<float4 *>(Q);
            const int f = lane & 15, half = lane >> 4;
            float4 v[32];
#pragma unroll
            for (int it = 0; it < 32; ++it) {
                const int ri = 2 * it + half, p = ri >> 3, j = ri & 7;
                v[it] = src[p * PP4 + (PL * rank + j) * RP4 + f];
            }
            cl.sync(); /* every CTA has its inputs: planes may be overwritten */
#pragma unroll
            for (int it = 0; it < 32; ++it) {
                const int ri = 2 * it + half, p = ri >> 3, j = ri & 7;
                dst[j * PP4 + (PL * warp + p) * RP4 + f] = v[it];
            }
        }
        d ^= 1;
        __syncthreads();
        /* the remaining axis along the rows of the new distribution */
        {
            float *c0 = Q + warp * PP + lane;
            conv_line<RP>(c0, c0 + 32, E + (d == 0 ? N3 : 0));
        }
        __syncthreads();
        /* q_{s+1} = b_s . y to HBM; the next step starts from b_{s+1} . q_{s+1} */
        {
            const float *b = reinterpret_cast<const float *>(s < cd.seg_end ? cd.b0 : cd.b1);
            const float *bn = reinterpret_cast<const float *>(s + 1 < cd.seg_end ? cd.b0 : cd.b1);
            const bool more = s + 1 < s_end, same = bn == b;
            float *qn = reinterpret_cast<float *>(cd.q) + (long)(s + 1) * a.sstride;
            for (int base = tid; base < PL * N3 * N3 / 4; base += NT * UB) {
                float4 bv[UB], nv[UB];
#pragma unroll
                for (int u = 0; u < UB; ++u) {
                    const long g = g_index(4 * (base + u * NT), rank, d);
                    bv[u] = __ldg(reinterpret_cast<const float4 *>(b + g));
                    nv[u] = (more && !same) ? __ldg(reinterpret_cast<const float4 *>(bn + g)) : bv[u];
                }
#pragma unroll
                for (int u = 0; u < UB; ++u) {
                    const int e = 4 * (base + u * NT);
                    const long g = g_index(e, rank, d);
                    float4 *dq = reinterpret_cast<float4 *>(Q + (e >> 12) * PP + ((e >> 6) & 63) * RP + (e & 63));
                    const float4 y = *dq;
                    const float4 o = {y.x * bv[u].x, y.y * bv[u].y, y.z * bv[u].z, y.w * bv[u].w};
                    *reinterpret_cast<float4 *>(qn + g) = o;
                    if (more) *dq = make_float4(o.x * nv[u].x, o.y * nv[u].y, o.z * nv[u].z, o.w * nv[u].w);
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
