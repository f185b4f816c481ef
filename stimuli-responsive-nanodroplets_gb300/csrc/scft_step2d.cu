/*
 * scft_step2d.cu — the whole contour loop of a chain in one persistent launch
 * for 2D (NY = 1) grids, FP32:
 *   q_{s+1} = b . Kz . Kx . (b . q_s),   b = exp(-DS w / 2)
 * (funPDESolver_periodic / funPDESolver_DirichletBC, SCFT.c:2474-2631).
 *
 * One CTA owns one NX x NZ slice of one chain of one instance, entirely in
 * shared memory for all of the chain's steps (row pitch NZ+2 keeps the
 * 64/128-bit row accesses of the z phase conflict-free), so a step reads b
 * once and writes q_{s+1} once; q_s never comes back from HBM. The store phase
 * of a step also runs the next step's first FFT phase (below) on the values it
 * has in registers. A CTA has one thread per line, or two (TM = 2) when the
 * batch has at most one chain per SM: every value is then computed by the
 * same arithmetic on another thread, so results do not depend on TM.
 *
 *  x axis (periodic): pairs of adjacent z columns form one complex column, as
 *  the factor is real and even in k. Each complex column of length N = NX =
 *  N1*N2 is transformed by a four-step FFT with register codelets: A) N2 DFTs
 *  of length N1 over stride-N2 rows and the twiddle W_N^(n2 k1); B) N1 DFTs of
 *  length N2 over contiguous row blocks, the factor E(k)/N, the inverse DFTs of
 *  length N2 and the conjugate twiddle, all in registers; C) the inverse DFTs
 *  of length N1. Every work item reads and writes the same set of rows, so a
 *  stage needs no barrier between its loads and stores.
 *  z axis: y = Kz x with Kz symmetric and centrosymmetric (the DST-I factor of
 *  the odd extension for MASK 1, the circulant factor for MASK 0) as two
 *  half-size products on x_k +- x_{NZ-1-k} (NZ^2/2 multiply-adds per row).
 *  FP32: a pair of threads shares two rows, each thread holding one half of
 *  the k range of both rows' sums and differences, so every 128-bit operator
 *  load feeds both rows; the halves' partial sums meet through a shuffle.
 *  Otherwise one row per thread with operator rows as broadcast loads.
 */
#include <cuda_runtime.h>

#include <type_traits>

#include "scft_internal.h"

/* Build switches of the fused chain kernel. */
#ifndef SCFT_F32X2
#define SCFT_F32X2 1 /* packed f32x2 FMA in the z phase */
#endif
#ifndef SCFT_BRES
#define SCFT_BRES 1 /* store-phase items whose Boltzmann factors stay in registers */
#endif
#ifndef SCFT_ZROWS
#define SCFT_ZROWS 2 /* output rows per pass of the packed z phase (2 or 4; measured equal) */
#endif

namespace {

template <typename P>
struct V2;
template <>
struct V2<float> {
    using T = float2;
};
template <>
struct V2<double> {
    using T = double2;
};

template <typename P>
struct V4;
template <>
struct V4<float> {
    using T = float4; /* 16-byte operator loads */
    static constexpr int W = 4;
};
template <>
struct V4<double> {
    using T = double2;
    static constexpr int W = 2;
    static_assert(W * sizeof(double) == sizeof(T), "one 16-byte load");
};

template <typename P>
struct Cx {
    P x, y;
};

constexpr size_t align16(size_t b) { return (b + 15) / 16 * 16; }

/* The z operator runs on the tensor cores (band on the FP32 pipe, tail by
 * tcgen05.mma) for FP32 shapes whose half size is a multiple of 16 (the MMA's
 * K step and N granule) and whose lines fill at most two 128-row tiles. */
template <typename P, int NX, int NZ>
struct ZTcOk {
    static constexpr bool value = sizeof(P) == 4 && (NZ / 2) % 16 == 0 && NX % 32 == 0 && NX <= 256;
};

/* TMEM columns of the tensor-core z tail: D = [Pe | Po] (H columns each,
 * FP32), then the A operand pieces U1, U2, V1, V2 (bf16 pairs, H/2 columns
 * each). */
template <int NZ>
struct ZTail {
    static constexpr int H = NZ / 2;
    static constexpr int PC = H / 2;
    static constexpr int COL_PE = 0, COL_PO = H, COL_A = 2 * H;
    static constexpr int USED = 2 * H + 4 * PC;
    static constexpr int TCOLS = USED <= 32 ? 32 : USED <= 64 ? 64 : USED <= 128 ? 128 : USED <= 256 ? 256 : 512;
    static constexpr int PIECE = 2 * H * H;      /* bytes of one H x H bf16 operator piece */
    static constexpr int SBO = 16 * H;           /* bytes between 8-row core-matrix groups */
    static constexpr int LBO = 128;              /* bytes between K-adjacent core matrices */
    static constexpr int R0 = 8;                 /* rows at either end with their own band coefficients */
    static constexpr int BAND_BYTES = 32 * (2 * R0 + 1); /* float[2 R0][8] + the interior constants float[8] */
};

/* byte offsets of the shared-memory regions: X, KA, KB, TW, EX; with the
 * tensor-core z tail KA..KB holds the four bf16 operator pieces (the same 8 H^2
 * bytes), followed by the band coefficients, the mbarrier and the TMEM slot */
template <typename P, int NX, int NZ>
struct Smem2D {
    static constexpr bool TC = ZTcOk<P, NX, NZ>::value;
    static constexpr size_t H = NZ / 2;
    static constexpr size_t X = 0;
    static constexpr size_t KA = align16(X + sizeof(P) * NX * (NZ + 2));
    static constexpr size_t KB = align16(KA + sizeof(P) * H * H);
    static constexpr size_t TW = align16(KB + sizeof(P) * H * H);
    static constexpr size_t EX = align16(TW + 2 * sizeof(P) * NX);
    static constexpr size_t BAND = align16(EX + sizeof(P) * NX);
    static constexpr size_t MBAR = TC ? align16(BAND + ZTail<NZ>::BAND_BYTES) : BAND;
    static constexpr size_t END = TC ? align16(MBAR + 16) : BAND;
    static_assert(!TC || 8 * H * H == KB - KA + sizeof(P) * H * H, "the bf16 pieces fill KA and KB");
};

template <typename P>
__device__ __forceinline__ Cx<P> cmul(Cx<P> a, Cx<P> b)
{
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
/* a * conj(b) */
template <typename P>
__device__ __forceinline__ Cx<P> cmulc(Cx<P> a, Cx<P> b)
{
    return {a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y};
}
template <typename P>
__device__ __forceinline__ Cx<P> cadd(Cx<P> a, Cx<P> b) { return {a.x + b.x, a.y + b.y}; }
template <typename P>
__device__ __forceinline__ Cx<P> csub(Cx<P> a, Cx<P> b) { return {a.x - b.x, a.y - b.y}; }
/* FP32: one packed f32x2 instruction per complex add or subtract */
template <>
__device__ __forceinline__ Cx<float> cadd(Cx<float> a, Cx<float> b)
{
    Cx<float> r;
    asm("{\n\t.reg .b64 pa, pb, pr;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "add.rn.f32x2 pr, pa, pb;\n\tmov.b64 {%0, %1}, pr;\n\t}"
        : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
template <>
__device__ __forceinline__ Cx<float> csub(Cx<float> a, Cx<float> b)
{
    Cx<float> r;
    asm("{\n\t.reg .b64 pa, pb, pr;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "sub.rn.f32x2 pr, pa, pb;\n\tmov.b64 {%0, %1}, pr;\n\t}"
        : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
template <typename P, bool INV>
__device__ __forceinline__ Cx<P> mul_si(Cx<P> a) /* sign*i*a, sign = -1 forward */
{
    return INV ? Cx<P>{-a.y, a.x} : Cx<P>{a.y, -a.x};
}

/* cos and sin of 2 pi k / N for N = 8, 12, 16 */
__constant__ double c_cos8[8] = {1.0, 0.70710678118654757274, 0.0, -0.70710678118654746172, -1.0,
                                 -0.70710678118654768376, 0.0, 0.70710678118654735069};
__constant__ double c_sin8[8] = {0.0, 0.70710678118654746172, 1.0, 0.70710678118654757274, 0.0,
                                 -0.70710678118654746172, -1.0, -0.70710678118654768376};
__constant__ double c_cos12[12] = {1.0, 0.86602540378443870761, 0.5, 0.0, -0.5, -0.86602540378443870761,
                                   -1.0, -0.86602540378443881863, -0.5, 0.0, 0.5, 0.86602540378443837454};
__constant__ double c_sin12[12] = {0.0, 0.5, 0.86602540378443859659, 1.0, 0.86602540378443870761, 0.5,
                                   0.0, -0.5, -0.86602540378443837454, -1.0, -0.86602540378443859659, -0.5};
__constant__ double c_cos16[16] = {1.0, 0.92387953251128673848, 0.70710678118654757274, 0.38268343236508983729,
                                   0.0, -0.38268343236508972627, -0.70710678118654746172, -0.92387953251128673848,
                                   -1.0, -0.92387953251128684951, -0.70710678118654768376, -0.38268343236509033689,
                                   0.0, 0.38268343236509000382, 0.70710678118654735069, 0.92387953251128651644};
__constant__ double c_sin16[16] = {0.0, 0.38268343236508978178, 0.70710678118654746172, 0.92387953251128673848,
                                   1.0, 0.92387953251128673848, 0.70710678118654757274, 0.38268343236508989280,
                                   0.0, -0.38268343236508967076, -0.70710678118654746172, -0.92387953251128651644,
                                   -1.0, -0.92387953251128662746, -0.70710678118654768376, -0.38268343236509039240};

/* the same tables in FP32 */
__constant__ float c_cos8f[8] = {1.000000000e+00f, 7.071067812e-01f, 6.123233996e-17f, -7.071067812e-01f, -1.000000000e+00f, -7.071067812e-01f, -1.836970199e-16f, 7.071067812e-01f};
__constant__ float c_sin8f[8] = {0.000000000e+00f, 7.071067812e-01f, 1.000000000e+00f, 7.071067812e-01f, 1.224646799e-16f, -7.071067812e-01f, -1.000000000e+00f, -7.071067812e-01f};
__constant__ float c_cos12f[12] = {1.000000000e+00f, 8.660254038e-01f, 5.000000000e-01f, 6.123233996e-17f, -5.000000000e-01f, -8.660254038e-01f, -1.000000000e+00f, -8.660254038e-01f, -5.000000000e-01f, -1.836970199e-16f, 5.000000000e-01f, 8.660254038e-01f};
__constant__ float c_sin12f[12] = {0.000000000e+00f, 5.000000000e-01f, 8.660254038e-01f, 1.000000000e+00f, 8.660254038e-01f, 5.000000000e-01f, 1.224646799e-16f, -5.000000000e-01f, -8.660254038e-01f, -1.000000000e+00f, -8.660254038e-01f, -5.000000000e-01f};
__constant__ float c_cos16f[16] = {1.000000000e+00f, 9.238795325e-01f, 7.071067812e-01f, 3.826834324e-01f, 6.123233996e-17f, -3.826834324e-01f, -7.071067812e-01f, -9.238795325e-01f, -1.000000000e+00f, -9.238795325e-01f, -7.071067812e-01f, -3.826834324e-01f, -1.836970199e-16f, 3.826834324e-01f, 7.071067812e-01f, 9.238795325e-01f};
__constant__ float c_sin16f[16] = {0.000000000e+00f, 3.826834324e-01f, 7.071067812e-01f, 9.238795325e-01f, 1.000000000e+00f, 9.238795325e-01f, 7.071067812e-01f, 3.826834324e-01f, 1.224646799e-16f, -3.826834324e-01f, -7.071067812e-01f, -9.238795325e-01f, -1.000000000e+00f, -9.238795325e-01f, -7.071067812e-01f, -3.826834324e-01f};

/* W_N^e = exp(sign 2 pi i e / N) for a compile-time e after unrolling */
template <typename P, int N, bool INV>
__device__ __forceinline__ Cx<P> wconst(int e)
{
    e %= N;
    if (sizeof(P) == 4) {
        const float c = N == 8 ? c_cos8f[e] : (N == 12 ? c_cos12f[e] : c_cos16f[e]);
        const float s = N == 8 ? c_sin8f[e] : (N == 12 ? c_sin12f[e] : c_sin16f[e]);
        return {(P)c, INV ? (P)s : (P)-s};
    }
    double c, s;
    if (N == 8) {
        c = c_cos8[e];
        s = c_sin8[e];
    } else if (N == 12) {
        c = c_cos12[e];
        s = c_sin12[e];
    } else {
        c = c_cos16[e];
        s = c_sin16[e];
    }
    return {(P)c, INV ? (P)s : (P)-s};
}

/* Packed FP32 pairs in one 64-bit register (the f32x2 arithmetic of sm_100+). */
__device__ __forceinline__ unsigned long long pack2(float lo, float hi)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ float lo2(unsigned long long r)
{
    float lo;
    asm("mov.b64 {%0, _}, %1;" : "=f"(lo) : "l"(r));
    return lo;
}
__device__ __forceinline__ float hi2(unsigned long long r)
{
    float hi;
    asm("mov.b64 {_, %0}, %1;" : "=f"(hi) : "l"(r));
    return hi;
}
/* c + a * b lane-wise, round to nearest */
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b, unsigned long long c)
{
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

/* In-register DFTs, natural order in and out. */
template <typename P, int N, bool INV>
struct Dft;

template <typename P, bool INV>
struct Dft<P, 2, INV> {
    static __device__ __forceinline__ void run(Cx<P> *v)
    {
        Cx<P> a = v[0];
        v[0] = cadd(a, v[1]);
        v[1] = csub(a, v[1]);
    }
};

template <typename P, bool INV>
struct Dft<P, 3, INV> {
    static __device__ __forceinline__ void run(Cx<P> *v)
    {
        const P h = (P)0.86602540378443864676;
        Cx<P> s = cadd(v[1], v[2]), d = csub(v[1], v[2]);
        Cx<P> c = {v[0].x - (P)0.5 * s.x, v[0].y - (P)0.5 * s.y};
        Cx<P> e = mul_si<P, INV>(d);
        v[0] = cadd(v[0], s);
        v[1] = {c.x + h * e.x, c.y + h * e.y};
        v[2] = {c.x - h * e.x, c.y - h * e.y};
    }
};

template <typename P, bool INV>
struct Dft<P, 4, INV> {
    static __device__ __forceinline__ void run(Cx<P> *v)
    {
        Cx<P> b0 = cadd(v[0], v[2]), b1 = csub(v[0], v[2]);
        Cx<P> b2 = cadd(v[1], v[3]), b3 = mul_si<P, INV>(csub(v[1], v[3]));
        v[0] = cadd(b0, b2);
        v[1] = cadd(b1, b3);
        v[2] = csub(b0, b2);
        v[3] = csub(b1, b3);
    }
};

/* N = A*B: A-point DFTs over stride-B inputs, twiddles W_N^(b k1), B-point DFTs. */
template <typename P, int A, int B, bool INV>
__device__ __forceinline__ void dft_two_factor(Cx<P> *v)
{
    constexpr int N = A * B;
    Cx<P> t[N];
#pragma unroll
    for (int b = 0; b < B; ++b) {
        Cx<P> col[A];
#pragma unroll
        for (int a = 0; a < A; ++a) col[a] = v[B * a + b];
        Dft<P, A, INV>::run(col);
#pragma unroll
        for (int k1 = 0; k1 < A; ++k1) t[b * A + k1] = (b * k1 == 0) ? col[k1] : cmul(col[k1], wconst<P, N, INV>(b * k1));
    }
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) {
        Cx<P> row[B];
#pragma unroll
        for (int b = 0; b < B; ++b) row[b] = t[b * A + k1];
        Dft<P, B, INV>::run(row);
#pragma unroll
        for (int k2 = 0; k2 < B; ++k2) v[k1 + A * k2] = row[k2];
    }
}

template <typename P, bool INV>
struct Dft<P, 8, INV> {
    static __device__ __forceinline__ void run(Cx<P> *v) { dft_two_factor<P, 4, 2, INV>(v); }
};
template <typename P, bool INV>
struct Dft<P, 12, INV> {
    static __device__ __forceinline__ void run(Cx<P> *v) { dft_two_factor<P, 4, 3, INV>(v); }
};
template <typename P, bool INV>
struct Dft<P, 16, INV> {
    static __device__ __forceinline__ void run(Cx<P> *v) { dft_two_factor<P, 4, 4, INV>(v); }
};

/* z operator, two lines per thread pair: thread (p, h) holds the k-half h of
 * the sums and differences of lines 2p and 2p+1, so every operator value it
 * loads feeds both lines; the two partial sums of an output meet through one
 * shuffle, and each thread finishes the outputs of its own half. With TM > 1
 * thread groups (TM * NX threads), group g computes the outputs jo in
 * [g KH/TM, (g+1) KH/TM) of every line pair with the same arithmetic, so the
 * results do not depend on TM. */
template <int NX, int NZ, int TM = 1>
__device__ __forceinline__ void z_split2(float *X, const float *KA, const float *KB, int t)
{
    constexpr int ZP = NZ + 2, H = NZ / 2, KH = H / 2, KQ = KH / 4;
    static_assert(KH % TM == 0, "output groups must split the half rows evenly");
    /* the lanes of this warp that exist in a block of NX * TM threads */
    constexpr int NT = NX * TM;
    const int lanes = NT - (t & ~31);
    const unsigned MASK = (NT % 32 == 0 || lanes >= 32) ? 0xffffffffu : ((1u << lanes) - 1u);
    const int tid = TM == 1 ? t : t % NX, g = TM == 1 ? 0 : t / NX;
    const int p = tid >> 1, h = tid & 1;
    float *r0 = X + (2 * p) * ZP;
    float *r1 = r0 + ZP;
    const int k0 = h * KH;
    unsigned long long u0[KH / 2], v0[KH / 2], u1[KH / 2], v1[KH / 2];
#pragma unroll
    for (int j = 0; j < KH / 2; ++j) {
        const int k = k0 + 2 * j;
        const float2 a0 = *reinterpret_cast<const float2 *>(r0 + k);
        const float2 a1 = *reinterpret_cast<const float2 *>(r1 + k);
        const float2 m0 = *reinterpret_cast<const float2 *>(r0 + NZ - 2 - k); /* x[NZ-2-k], x[NZ-1-k] */
        const float2 m1 = *reinterpret_cast<const float2 *>(r1 + NZ - 2 - k);
        u0[j] = pack2(a0.x + m0.y, a0.y + m0.x);
        v0[j] = pack2(a0.x - m0.y, a0.y - m0.x);
        u1[j] = pack2(a1.x + m1.y, a1.y + m1.x);
        v1[j] = pack2(a1.x - m1.y, a1.y - m1.x);
    }
    if constexpr (TM > 1) __syncthreads(); /* every group has its lines before any output lands */
    for (int jo = g * (KH / TM); jo < (g + 1) * (KH / TM); ++jo) {
        unsigned long long s00 = 0ull, s01 = 0ull, s10 = 0ull, s11 = 0ull; /* s[row][line] */
        unsigned long long d00 = 0ull, d01 = 0ull, d10 = 0ull, d11 = 0ull;
        const float4 *a0p = reinterpret_cast<const float4 *>(KA + jo * H + k0);
        const float4 *a1p = reinterpret_cast<const float4 *>(KA + (KH + jo) * H + k0);
        const float4 *b0p = reinterpret_cast<const float4 *>(KB + jo * H + k0);
        const float4 *b1p = reinterpret_cast<const float4 *>(KB + (KH + jo) * H + k0);
#pragma unroll
        for (int q = 0; q < KQ; ++q) {
            const float4 a0 = a0p[q], a1 = a1p[q], b0 = b0p[q], b1 = b1p[q];
            const unsigned long long a0l = pack2(a0.x, a0.y), a0h = pack2(a0.z, a0.w);
            const unsigned long long a1l = pack2(a1.x, a1.y), a1h = pack2(a1.z, a1.w);
            const unsigned long long b0l = pack2(b0.x, b0.y), b0h = pack2(b0.z, b0.w);
            const unsigned long long b1l = pack2(b1.x, b1.y), b1h = pack2(b1.z, b1.w);
            s00 = fma2(a0h, u0[2 * q + 1], fma2(a0l, u0[2 * q], s00));
            s01 = fma2(a0h, u1[2 * q + 1], fma2(a0l, u1[2 * q], s01));
            s10 = fma2(a1h, u0[2 * q + 1], fma2(a1l, u0[2 * q], s10));
            s11 = fma2(a1h, u1[2 * q + 1], fma2(a1l, u1[2 * q], s11));
            d00 = fma2(b0h, v0[2 * q + 1], fma2(b0l, v0[2 * q], d00));
            d01 = fma2(b0h, v1[2 * q + 1], fma2(b0l, v1[2 * q], d01));
            d10 = fma2(b1h, v0[2 * q + 1], fma2(b1l, v0[2 * q], d10));
            d11 = fma2(b1h, v1[2 * q + 1], fma2(b1l, v1[2 * q], d11));
        }
        /* keep the row of this half (jo for h = 0, KH + jo for h = 1), send the other */
        const float ks0 = h ? lo2(s10) + hi2(s10) : lo2(s00) + hi2(s00);
        const float ks1 = h ? lo2(s11) + hi2(s11) : lo2(s01) + hi2(s01);
        const float kd0 = h ? lo2(d10) + hi2(d10) : lo2(d00) + hi2(d00);
        const float kd1 = h ? lo2(d11) + hi2(d11) : lo2(d01) + hi2(d01);
        const float ts0 = h ? lo2(s00) + hi2(s00) : lo2(s10) + hi2(s10);
        const float ts1 = h ? lo2(s01) + hi2(s01) : lo2(s11) + hi2(s11);
        const float td0 = h ? lo2(d00) + hi2(d00) : lo2(d10) + hi2(d10);
        const float td1 = h ? lo2(d01) + hi2(d01) : lo2(d11) + hi2(d11);
        const float S0 = ks0 + __shfl_xor_sync(MASK, ts0, 1);
        const float S1 = ks1 + __shfl_xor_sync(MASK, ts1, 1);
        const float D0 = kd0 + __shfl_xor_sync(MASK, td0, 1);
        const float D1 = kd1 + __shfl_xor_sync(MASK, td1, 1);
        const int i = h ? KH + jo : jo;
        r0[i] = S0 + D0;
        r0[NZ - 1 - i] = S0 - D0;
        r1[i] = S1 + D1;
        r1[NZ - 1 - i] = S1 - D1;
    }
}

/* ------------------------------------------ z operator on the tensor cores
 * y = Kb x + Kt x. Kb is the band |j - k| <= 3 of the operator (circular for a
 * periodic axis), applied in FP32 with round-to-nearest FMAs; it carries all
 * but ~0.3 % of every row's weight. Kt = K - Kb, the tail, is applied as its
 * centrosymmetric halves (Pe = U Ae^T, Po = V Ao^T with u = x + Jx, v = x - Jx)
 * by tcgen05.mma on bf16 pairs: u = u1 + u2 and Ae = Ae1 + Ae2 (16 bits each),
 * three products per half (u2 Ae1 + u1 Ae2 + u1 Ae1), FP32 accumulation in
 * TMEM. The tensor cores' accumulation truncates, but only on the tail, so its
 * bias is ~3e-3 of an FP32 ulp of y per step; the split's own error is ~2^-17
 * of the tail, below FP32 rounding of y. Lines are the MMA's M rows: lines
 * 0..127 form tile 0 (TMEM lanes = line), lines 128..255 tile 1 (lanes =
 * line - 128), run one after the other through the same TMEM columns. */
__device__ __forceinline__ uint32_t bf16x2_rn(float hi, float lo)
{
    uint32_t d;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}
__device__ __forceinline__ float bf16_lo(uint32_t p) { return __uint_as_float(p << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t p) { return __uint_as_float(p & 0xffff0000u); }

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tm_st8(uint32_t ta, const uint32_t (&r)[8])
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(ta), "r"(r[0]),
                 "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7])
                 : "memory");
}
__device__ __forceinline__ void tm_ld16(uint32_t ta, uint32_t (&r)[16])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(ta)
                 : "memory");
}

/* shared-memory matrix descriptor: K-major, no swizzle, 8 x 16-byte core matrices */
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ void mma_bf16(uint32_t d, uint32_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d),
                 "r"(a), "l"(b), "r"(idesc), "r"(acc)
                 : "memory");
}

/* Bounded wait for the mbarrier phase of the given parity: false after ~0.1 s. */
__device__ __forceinline__ bool mbar_wait(uint32_t mb, uint32_t parity)
{
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred P1;\n\tmbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n\t"
                     "selp.b32 %0, 1, 0, P1;\n\t}"
                     : "=r"(done)
                     : "r"(mb), "r"(parity)
                     : "memory");
        if (done) return true;
        if (clock64() - t0 > (1LL << 28)) return false;
    }
}

/* u, v of one line split into bf16 pairs and stored to the A columns of its
 * TMEM lane (ta = lane address of column COL_A); the line is read from shared
 * memory 16 columns (and their mirror images) at a time. */
template <int NZ>
__device__ __forceinline__ void ztc_store_a(const float *row, uint32_t ta)
{
    using Z = ZTail<NZ>;
#pragma unroll
    for (int c = 0; c < Z::H / 16; ++c) {
        float lo[16], hi[16]; /* x[16c + i], x[NZ - 16 - 16c + i] */
#pragma unroll
        for (int i = 0; i < 16; i += 2) {
            const float2 a = *reinterpret_cast<const float2 *>(row + 16 * c + i);
            const float2 m = *reinterpret_cast<const float2 *>(row + NZ - 16 - 16 * c + i);
            lo[i] = a.x;
            lo[i + 1] = a.y;
            hi[i] = m.x;
            hi[i + 1] = m.y;
        }
        uint32_t u1[8], u2[8], v1[8], v2[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            /* k = 16c + 2j: x[k], x[k+1] and their mirrors x[NZ-1-k], x[NZ-2-k] */
            const float xa = lo[2 * j], xb = lo[2 * j + 1], ma = hi[15 - 2 * j], mb = hi[14 - 2 * j];
            const float ua = xa + ma, ub = xb + mb, va = xa - ma, vb = xb - mb;
            u1[j] = bf16x2_rn(ub, ua); /* even k in the low half */
            v1[j] = bf16x2_rn(vb, va);
            u2[j] = bf16x2_rn(ub - bf16_hi(u1[j]), ua - bf16_lo(u1[j]));
            v2[j] = bf16x2_rn(vb - bf16_hi(v1[j]), va - bf16_lo(v1[j]));
        }
        tm_st8(ta + 0 * Z::PC + 8 * c, u1);
        tm_st8(ta + 1 * Z::PC + 8 * c, u2);
        tm_st8(ta + 2 * Z::PC + 8 * c, v1);
        tm_st8(ta + 3 * Z::PC + 8 * c, v2);
    }
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

/* One thread issues the tail products of one half of one tile (HALF 0: Pe =
 * U Ae^T, HALF 1: Po = V Ao^T) and commits them to mb (two arrivals per tile). */
template <int NZ, int HALF>
__device__ __forceinline__ void ztc_issue(uint32_t tmem, uint32_t pieces, uint32_t mb)
{
    using Z = ZTail<NZ>;
    constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(Z::H >> 3) << 17) | (8u << 24);
    const uint32_t d = tmem + (HALF ? Z::COL_PO : Z::COL_PE);
    const uint32_t p1 = pieces + (HALF ? 2 : 0) * Z::PIECE, p2 = p1 + Z::PIECE;
#pragma unroll
    for (int c = 0; c < Z::H / 16; ++c) {
        const uint32_t a1 = tmem + Z::COL_A + (HALF ? 2 : 0) * Z::PC + 8 * c, a2 = a1 + Z::PC;
        const uint64_t k1 = smem_desc(p1 + 256u * c, Z::LBO, Z::SBO);
        const uint64_t k2 = smem_desc(p2 + 256u * c, Z::LBO, Z::SBO);
        mma_bf16(d, a2, k1, IDESC, c > 0 ? 1u : 0u);
        mma_bf16(d, a1, k2, IDESC, 1u);
        mma_bf16(d, a1, k1, IDESC, 1u);
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb) : "memory");
}

/* The two halves of a tile's tail, issued by lane 0 of warps w0 and w0 + 1
 * (idle warps where there are any; a CTA of one warp issues both). */
template <int NZ, int T>
__device__ __forceinline__ void ztc_issue_tile(int tid, int w0, uint32_t tmem, uint32_t pieces, uint32_t mb)
{
    if (tid == 32 * w0) ztc_issue<NZ, 0>(tmem, pieces, mb);
    if (tid == (T > 32 ? 32 * (w0 + 1) : 0)) ztc_issue<NZ, 1>(tmem, pieces, mb);
}

/* Band part of one line, written over the line in place. The R0 rows at
 * either end have their own coefficients (slot d + 3 of table row r multiplies
 * x[(j + d) mod NZ], zero where a Dirichlet row has no such neighbour); every
 * interior row applies the symmetric constants c0..c3:
 * y = c0 x_j + c1 (x_j-1 + x_j+1) + c2 (x_j-2 + x_j+2) + c3 (x_j-3 + x_j+3),
 * small terms first. A window x[j-3 .. j+5] moves along the line in registers,
 * so every value is read before its slot is written; the last two pairs wrap
 * to the saved head of the line. */
template <int NZ>
__device__ __forceinline__ void ztc_band(float *row, const float *bt)
{
    constexpr int R0 = ZTail<NZ>::R0;
    static_assert(NZ >= 2 * R0 + 8 && R0 % 2 == 0, "interior rows between the end rows");
    const float4 *b4 = reinterpret_cast<const float4 *>(bt);
    const float4 cc = b4[4 * R0]; /* c0, c1, c2, c3 */
    const float2 h01 = *reinterpret_cast<const float2 *>(row);
    const float2 h23 = *reinterpret_cast<const float2 *>(row + 2);
    const float2 t0 = *reinterpret_cast<const float2 *>(row + NZ - 4);
    const float2 t1 = *reinterpret_cast<const float2 *>(row + NZ - 2);
    const float head[4] = {h01.x, h01.y, h23.x, h23.y};
    float w[9]; /* w[i] = x[j - 3 + i] */
    w[0] = t0.y;
    w[1] = t1.x;
    w[2] = t1.y;
    w[3] = head[0];
    w[4] = head[1];
    w[5] = head[2];
    w[6] = head[3];
    auto shift = [&]() {
#pragma unroll
        for (int i = 0; i < 7; ++i) w[i] = w[i + 2];
    };
    /* rows j, j+1 with their own coefficients (table rows r, r+1) */
    auto pair_rows = [&](int j, int r) {
        float y[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const float4 ca = b4[2 * (r + e)], cb = b4[2 * (r + e) + 1];
            const float *x = w + e; /* x[d + 3] = x_{j+e+d} */
            float t = ca.x * x[0];
            t = fmaf(cb.z, x[6], t);
            t = fmaf(ca.y, x[1], t);
            t = fmaf(cb.y, x[5], t);
            t = fmaf(ca.z, x[2], t);
            t = fmaf(cb.x, x[4], t);
            y[e] = fmaf(ca.w, x[3], t);
        }
        *reinterpret_cast<float2 *>(row + j) = make_float2(y[0], y[1]);
    };
    auto pair_const = [&](int j) {
        float y[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const float *x = w + e;
            float t = cc.w * (x[0] + x[6]);
            t = fmaf(cc.z, x[1] + x[5], t);
            t = fmaf(cc.y, x[2] + x[4], t);
            y[e] = fmaf(cc.x, x[3], t);
        }
        *reinterpret_cast<float2 *>(row + j) = make_float2(y[0], y[1]);
    };
    auto next = [&](int j) { /* x[j+4], x[j+5] into the window */
        if (j + 4 < NZ) {
            const float2 n = *reinterpret_cast<const float2 *>(row + j + 4);
            w[7] = n.x;
            w[8] = n.y;
        } else {
            w[7] = head[j + 4 - NZ];
            w[8] = head[j + 5 - NZ];
        }
    };
#pragma unroll
    for (int j = 0; j < R0; j += 2) {
        next(j);
        pair_rows(j, j);
        shift();
    }
#pragma unroll 4
    for (int j = R0; j < NZ - R0; j += 2) {
        const float2 n = *reinterpret_cast<const float2 *>(row + j + 4);
        w[7] = n.x;
        w[8] = n.y;
        pair_const(j);
        shift();
    }
#pragma unroll
    for (int j = NZ - R0; j < NZ; j += 2) {
        next(j);
        pair_rows(j, j - NZ + 2 * R0);
        shift();
    }
}

/* Adds the tail (Pe + Po on top, Pe - Po mirrored below) to the band values of
 * the line (td = lane address of column 0). */
template <int NZ>
__device__ __forceinline__ void ztc_combine(float *row, uint32_t td)
{
    using Z = ZTail<NZ>;
#pragma unroll
    for (int c0 = 0; c0 < Z::H; c0 += 16) {
        uint32_t pe[16], po[16];
        tm_ld16(td + Z::COL_PE + c0, pe);
        tm_ld16(td + Z::COL_PO + c0, po);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const float e = __uint_as_float(pe[i]), o = __uint_as_float(po[i]);
            row[c0 + i] += e + o;
            row[NZ - 1 - c0 - i] += e - o;
        }
    }
}

} // namespace

/* Set when a tensor-core wait of the chain kernel gave up (the chain's slice
 * is then written as NaN, so the instance reports a non-finite status). */
__device__ int g_scft_tc_fault;

/* ------------------------------------------------------------------ kernel */
/* 16-byte asynchronous copy global -> shared (no register staging) */
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned dst = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(gmem));
}

/* One CTA runs contour steps s = a.s .. min(a.s_end, len-1)-1 of one chain:
 * the slice stays in shared memory from step to step (q_{s+1} is written to
 * HBM for the densities and kept for the next step), the operator tables are
 * loaded once. Chains are taken longest first through a.order. */
/* CTAs per SM the loop is compiled for (one thread per line): as many as the
 * shared memory and, with the tensor-core z tail, the TMEM columns allow, at
 * most 4; the register budget per thread follows from it. */
template <typename P, int NX, int NZ, int TM>
struct MinBlocks2D {
    static constexpr long S = (long)Smem2D<P, NX, NZ>::END + 1024;
    static constexpr long by_smem = 233472 / S;
    static constexpr long by_tmem = Smem2D<P, NX, NZ>::TC ? 512 / ZTail<NZ>::TCOLS : 8;
    static constexpr long v = by_smem < by_tmem ? by_smem : by_tmem;
    static constexpr int value = TM > 1 ? 1 : (v < 1 ? 1 : (v > 4 ? 4 : (int)v));
};

template <typename P, int NX, int NZ, int N1, int N2, int TM>
__global__ void __launch_bounds__(NX * TM, (MinBlocks2D<P, NX, NZ, TM>::value)) k_chain2d(Step2DArgs a)
{
    constexpr int T = NX * TM; /* threads: TM per line */
    static_assert(N1 * N2 == NX, "NX = N1 * N2");
    static_assert(NZ % 4 == 0, "NZ must be a multiple of 4");
    constexpr int ZP = NZ + 2;  /* row pitch (elements) */
    constexpr int ZP2 = ZP / 2; /* row pitch in complex pairs */
    constexpr int NZ2 = NZ / 2; /* complex columns */
    constexpr int H = NZ / 2;   /* half size of the z operator */
    using T2 = typename V2<P>::T;

    const ChainDesc cd = a.chains[a.order ? a.order[blockIdx.x] : blockIdx.x];
    if (a.state && a.state[cd.instance].done) return; /* uniform over the CTA */
    const int s_end = a.s_end < cd.len - 1 ? a.s_end : cd.len - 1;
    if (a.s >= s_end) return;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    using L = Smem2D<P, NX, NZ>;
    P *X = reinterpret_cast<P *>(smem_raw + L::X);       /* NX * ZP */
    P *KA = reinterpret_cast<P *>(smem_raw + L::KA);     /* H * H, row-major [i][k] */
    P *KB = reinterpret_cast<P *>(smem_raw + L::KB);     /* H * H */
    Cx<P> *TW = reinterpret_cast<Cx<P> *>(smem_raw + L::TW); /* N: W_N^(n2 k1) at n2*N1 + k1 */
    P *EX = reinterpret_cast<P *>(smem_raw + L::EX);     /* N: E(k)/N */
    Cx<P> *XC = reinterpret_cast<Cx<P> *>(X);

    const int tid = threadIdx.x;
    const P *qs = reinterpret_cast<const P *>(cd.q) + (long)a.s * a.sstride;
    /* phase A folded into the store phase: every thread owns whole work items */
    constexpr bool FUSE_A = sizeof(P) == 4 && (N2 * NZ2) % NX == 0;
    constexpr int ITEMS = (N2 * NZ2 + T - 1) / T;
    constexpr bool ITEMS_EVEN = (N2 * NZ2) % T == 0;

    constexpr bool ZTC = L::TC;
    /* operators and tables, once per chain (16-byte asynchronous copies) */
    {
        constexpr int VP = 16 / sizeof(P);
        const P *gA = reinterpret_cast<const P *>(cd.ops->kz);
        if constexpr (ZTC) {
            /* band coefficients (FP32), then the four bf16 pieces (8 H^2 bytes) */
            constexpr int NB = ZTail<NZ>::BAND_BYTES / 16, NP = 8 * H * H / 16;
            const unsigned char *g = reinterpret_cast<const unsigned char *>(gA);
            for (int e = tid; e < NB; e += T) cp_async16(smem_raw + L::BAND + 16 * e, g + 16 * e);
            for (int e = tid; e < NP; e += T) cp_async16(smem_raw + L::KA + 16 * e, g + 16 * NB + 16 * e);
        } else {
            for (int e = tid; e < H * H / VP; e += T) {
                cp_async16(KA + e * VP, gA + e * VP);
                cp_async16(KB + e * VP, gA + H * H + e * VP);
            }
        }
        const P *gT = reinterpret_cast<const P *>(cd.ops->twx);
        for (int e = tid; e < 2 * NX / VP; e += T) cp_async16(reinterpret_cast<P *>(TW) + e * VP, gT + e * VP);
        const P *gE = reinterpret_cast<const P *>(cd.ops->ex);
        for (int e = tid; e < NX / VP; e += T) cp_async16(EX + e * VP, gE + e * VP);
    }
    /* load q_s into the padded rows with asynchronous 2-element copies: every
     * copy of the slice is in flight at once and none holds a register */
    for (int e = tid; e < NX * NZ2; e += T) {
        const int x = e / NZ2, c = e - x * NZ2;
        const unsigned dst = (unsigned)__cvta_generic_to_shared(reinterpret_cast<T2 *>(X) + x * ZP2 + c);
        if (sizeof(T2) == 8)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(dst), "l"(reinterpret_cast<const T2 *>(qs) + e));
        else
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(reinterpret_cast<const T2 *>(qs) + e));
    }
    asm volatile("cp.async.commit_group;\n" ::);
    /* tensor-core z tail: the mbarrier, the TMEM base address and the fault
     * flag of this CTA live in shared memory (no registers across the loop) */
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem_raw + L::MBAR + 8);
    int *fault_flag = reinterpret_cast<int *>(smem_raw + L::MBAR + 12);
    if constexpr (ZTC) {
        const uint32_t mbar = (uint32_t)__cvta_generic_to_shared(smem_raw + L::MBAR);
        if (tid == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 2;" ::"r"(mbar) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            *fault_flag = 0;
        }
        if (tid < 32) {
            asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                             (uint32_t)__cvta_generic_to_shared(tslot)),
                         "r"(ZTail<NZ>::TCOLS)
                         : "memory");
            asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        }
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    if constexpr (ZTC) {
        /* the operator pieces are read by the tensor cores (async proxy) */
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();
    }
    __syncthreads();
    if constexpr (ZTC) tc_fence_after();

    /* the first step's input b . q_s; later steps get theirs from the store phase */
    {
        const P *b_first = reinterpret_cast<const P *>(a.s < cd.seg_end ? cd.b0 : cd.b1);
#pragma unroll 4
        for (int e = tid; e < NX * NZ2; e += T) {
            const int x = e / NZ2, c = e - x * NZ2;
            const T2 b2 = reinterpret_cast<const T2 *>(b_first)[e];
            T2 &v = reinterpret_cast<T2 *>(X)[x * ZP2 + c];
            v.x *= b2.x;
            v.y *= b2.y;
        }
    }
    __syncthreads();

    /* the Boltzmann factor of a chain segment is the same slice at every step:
     * each thread keeps its values for its first RES store-phase items in
     * registers from step to step (reloaded at the diblock junction) */
    constexpr int RES = FUSE_A ? (ITEMS < SCFT_BRES ? ITEMS : SCFT_BRES) : 0;
    T2 bres[RES > 0 ? RES * N1 : 1];
    const void *bres_src = nullptr;

    for (int s = a.s; s < s_end; ++s) {
    const P *bz = reinterpret_cast<const P *>(s < cd.seg_end ? cd.b0 : cd.b1);
    const P *bnext = reinterpret_cast<const P *>(s + 1 < cd.seg_end ? cd.b0 : cd.b1);
    P *qn = reinterpret_cast<P *>(cd.q) + (long)(s + 1) * a.sstride;
    /* A: DFT_N1 over rows N2*n1 + n2 of b . q_s, twiddle, back to rows N2*k1 + n2
     * (after the first step this runs inside the previous step's store phase) */
    if (!FUSE_A || s == a.s) {
    for (int w = tid; w < N2 * NZ2; w += T) {
        const int n2 = w / NZ2, c = w - n2 * NZ2;
        Cx<P> v[N1];
#pragma unroll
        for (int n1 = 0; n1 < N1; ++n1) v[n1] = XC[(N2 * n1 + n2) * ZP2 + c];
        Dft<P, N1, false>::run(v);
#pragma unroll
        for (int k1 = 1; k1 < N1; ++k1) v[k1] = cmul(v[k1], TW[n2 * N1 + k1]);
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) XC[(N2 * k1 + n2) * ZP2 + c] = v[k1];
    }
    __syncthreads();
    }
    /* B: DFT_N2 over rows N2*k1 .. N2*k1+N2-1, E(k)/N, inverse, conjugate twiddle */
    for (int w = tid; w < N1 * NZ2; w += T) {
        const int k1 = w / NZ2, c = w - k1 * NZ2;
        Cx<P> u[N2];
#pragma unroll
        for (int n2 = 0; n2 < N2; ++n2) u[n2] = XC[(N2 * k1 + n2) * ZP2 + c];
        Dft<P, N2, false>::run(u);
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) {
            if (k2 == 0 && k1 == 0) {
                /* mean mode, E(0) = 1: a correctly rounded division by N keeps the
                 * per-step gain of the mean unbiased (a rounded 1/N would not) */
                u[0].x = u[0].x / (P)NX;
                u[0].y = u[0].y / (P)NX;
                continue;
            }
            const P f = EX[k1 + N1 * k2];
            u[k2].x *= f;
            u[k2].y *= f;
        }
        Dft<P, N2, true>::run(u);
#pragma unroll
        for (int n2 = 1; n2 < N2; ++n2) u[n2] = cmulc(u[n2], TW[n2 * N1 + k1]);
#pragma unroll
        for (int n2 = 0; n2 < N2; ++n2) XC[(N2 * k1 + n2) * ZP2 + c] = u[n2];
    }
    __syncthreads();
    /* C: inverse DFT_N1 back to natural rows */
    for (int w = tid; w < N2 * NZ2; w += T) {
        const int n2 = w / NZ2, c = w - n2 * NZ2;
        Cx<P> v[N1];
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) v[k1] = XC[(N2 * k1 + n2) * ZP2 + c];
        Dft<P, N1, true>::run(v);
#pragma unroll
        for (int n1 = 0; n1 < N1; ++n1) XC[(N2 * n1 + n2) * ZP2 + c] = v[n1];
    }
    __syncthreads();

    /* z: one row per thread, y = A (x + Jx) -> s, B (x - Jx) -> d */
    static_assert(TM == 1 || (sizeof(P) == 4 && SCFT_F32X2 && (NZ / 2) % 8 == 0),
                  "two threads per line need the split z phase");
    if constexpr (ZTC) {
        /* band on the FP32 pipe, tail on the tensor cores; lines are the
         * threads tid < NX (with TM = 2 the second group waits at the barriers) */
        constexpr int NTILE = (NX + 127) / 128;
        const bool line_thr = tid < NX;
        const int tile = tid >> 7;
        const uint32_t lane = (uint32_t)(tid & 96) << 16; /* 32 * (warp % 4): this warp's TMEM lanes */
        const uint32_t pieces = (uint32_t)__cvta_generic_to_shared(smem_raw + L::KA);
        const uint32_t mbar = (uint32_t)__cvta_generic_to_shared(smem_raw + L::MBAR);
        const uint32_t tmem = *tslot;
        uint32_t ncommit = (uint32_t)(s - a.s) * NTILE; /* tail commits before this step */
        float *row = reinterpret_cast<float *>(X) + (line_thr ? tid : 0) * ZP;
        const float *bt = reinterpret_cast<const float *>(smem_raw + L::BAND);
        if (line_thr && tile == 0) ztc_store_a<NZ>(row, tmem + lane + ZTail<NZ>::COL_A);
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        /* tile 0's products: from the tile-1 warps, idle until they finish */
        ztc_issue_tile<NZ, T>(tid, NTILE > 1 ? 4 : 0, tmem, pieces, mbar);
        if (line_thr) {
            /* tile 0: band while the tail runs, then the tail; tile 1: its
             * operand once tile 0's products have read theirs */
            if (tile == 0) ztc_band<NZ>(row, bt);
            /* warp-uniform: the TMEM accesses below are warp-collective */
            const bool ok = __all_sync(0xffffffffu, mbar_wait(mbar, ncommit & 1));
            tc_fence_after();
            if (!ok) *fault_flag = 1;
            if (tile == 0) {
                if (ok) ztc_combine<NZ>(row, tmem + lane);
            } else if (ok) {
                ztc_store_a<NZ>(row, tmem + lane + ZTail<NZ>::COL_A);
            }
        }
        ++ncommit;
        if constexpr (NTILE > 1) {
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
            ztc_issue_tile<NZ, T>(tid, 0, tmem, pieces, mbar);
            if (line_thr && tile == 1) {
                ztc_band<NZ>(row, bt);
                const bool ok = __all_sync(0xffffffffu, mbar_wait(mbar, ncommit & 1));
                tc_fence_after();
                if (ok)
                    ztc_combine<NZ>(row, tmem + lane);
                else
                    *fault_flag = 1;
            }
            ++ncommit;
        }
        tc_fence_before();
    } else if constexpr (sizeof(P) == 4 && SCFT_F32X2 && (NZ / 2) % 8 == 0) {
        z_split2<NX, NZ, TM>(reinterpret_cast<float *>(X), reinterpret_cast<const float *>(KA),
                         reinterpret_cast<const float *>(KB), tid);
    } else {
        P *row = X + tid * ZP;
        P u[H], v[H];
#pragma unroll
        for (int j = 0; j < NZ2; ++j) {
            const T2 t = reinterpret_cast<const T2 *>(row)[j];
            /* positions 2j and 2j+1 */
            if (2 * j < H) {
                u[2 * j] = t.x;
                v[2 * j] = t.x;
            } else {
                u[NZ - 1 - 2 * j] += t.x;
                v[NZ - 1 - 2 * j] -= t.x;
            }
            if (2 * j + 1 < H) {
                u[2 * j + 1] = t.y;
                v[2 * j + 1] = t.y;
            } else {
                u[NZ - 2 - 2 * j] += t.y;
                v[NZ - 2 - 2 * j] -= t.y;
            }
        }
        using T4 = typename V4<P>::T;
        constexpr int W = V4<P>::W;
        static_assert(H % W == 0, "operator rows must split into 16-byte loads");
        if constexpr (sizeof(P) == 4 && SCFT_F32X2) {
            /* packed FP32 pairs: each f32x2 FMA adds an (even k, odd k) pair of one
             * output row, so one 128-bit operator load feeds two packed FMAs */
            unsigned long long u2[H / 2], v2[H / 2];
#pragma unroll
            for (int j = 0; j < H / 2; ++j) {
                u2[j] = pack2(u[2 * j], u[2 * j + 1]);
                v2[j] = pack2(v[2 * j], v[2 * j + 1]);
            }
            constexpr int R = (SCFT_ZROWS == 4 && H % 4 == 0) ? 4 : 2;
            for (int i = 0; i < H; i += R) {
                unsigned long long sacc[R], dacc[R];
#pragma unroll
                for (int r = 0; r < R; ++r) sacc[r] = dacc[r] = 0ull;
#pragma unroll
                for (int k = 0; k < H; k += 4) {
                    float4 av[R], bv[R];
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        av[r] = reinterpret_cast<const float4 *>(KA + (i + r) * H)[k / 4];
                        bv[r] = reinterpret_cast<const float4 *>(KB + (i + r) * H)[k / 4];
                    }
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        sacc[r] = fma2(pack2(av[r].x, av[r].y), u2[k / 2], sacc[r]);
                        sacc[r] = fma2(pack2(av[r].z, av[r].w), u2[k / 2 + 1], sacc[r]);
                        dacc[r] = fma2(pack2(bv[r].x, bv[r].y), v2[k / 2], dacc[r]);
                        dacc[r] = fma2(pack2(bv[r].z, bv[r].w), v2[k / 2 + 1], dacc[r]);
                    }
                }
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const float sr = lo2(sacc[r]) + hi2(sacc[r]), dr = lo2(dacc[r]) + hi2(dacc[r]);
                    row[i + r] = sr + dr;
                    row[NZ - 1 - i - r] = sr - dr;
                }
            }
        } else
        /* two output rows per pass: four independent accumulation chains */
        for (int i = 0; i < H; i += 2) {
            P s0 = 0, d0 = 0, s1 = 0, d1 = 0;
            const T4 *ar0 = reinterpret_cast<const T4 *>(KA + i * H);
            const T4 *br0 = reinterpret_cast<const T4 *>(KB + i * H);
            const T4 *ar1 = reinterpret_cast<const T4 *>(KA + (i + 1) * H);
            const T4 *br1 = reinterpret_cast<const T4 *>(KB + (i + 1) * H);
#pragma unroll
            for (int k = 0; k < H; k += W) {
                const T4 a0 = ar0[k / W], b0 = br0[k / W], a1 = ar1[k / W], b1 = br1[k / W];
                const P *pa0 = reinterpret_cast<const P *>(&a0);
                const P *pb0 = reinterpret_cast<const P *>(&b0);
                const P *pa1 = reinterpret_cast<const P *>(&a1);
                const P *pb1 = reinterpret_cast<const P *>(&b1);
#pragma unroll
                for (int r = 0; r < W; ++r) {
                    s0 += pa0[r] * u[k + r];
                    d0 += pb0[r] * v[k + r];
                    s1 += pa1[r] * u[k + r];
                    d1 += pb1[r] * v[k + r];
                }
            }
            row[i] = s0 + d0;
            row[NZ - 1 - i] = s0 - d0;
            row[i + 1] = s1 + d1;
            row[NZ - 2 - i] = s1 - d1;
        }
    }
    __syncthreads();
    /* a tensor-core wait that gave up: this step's slice goes out as NaN (the
     * instance then reports a non-finite status) and the chain stops */
    bool stop_chain = false;
    if constexpr (ZTC) {
        tc_fence_after();
        stop_chain = *fault_flag != 0;
        if (stop_chain) {
            if (tid == 0) atomicExch(&g_scft_tc_fault, 1);
            for (int e = tid; e < NX * ZP; e += T) X[e] = __int_as_float(0x7fc00000);
            __syncthreads();
        }
    }
    /* q_{s+1} = b . y to HBM for the densities; the next step's input
     * b_next . q_{s+1} stays in shared memory (b_next differs from b only at the
     * diblock junction), so b is read once per step. Each thread issues all of
     * its b loads before using any: L2 latency is paid once per step. Unless
     * this is the last step, each thread walks the columns of its phase-A work
     * items, so the next step's phase A runs on the values in registers. */
    if (FUSE_A && s + 1 < s_end) {
        const T2 *b2p = reinterpret_cast<const T2 *>(bz);
        const T2 *n2p = reinterpret_cast<const T2 *>(bnext);
        /* the next step's factor differs only at the diblock junction: a
         * separate body for that step keeps its extra loads out of every other */
        auto load = [&](int it, T2 *dst) {
            const int w = tid + it * T, n2 = w / NZ2, c = w - n2 * NZ2;
            if (ITEMS_EVEN || w < N2 * NZ2) {
#pragma unroll
                for (int n1 = 0; n1 < N1; ++n1) dst[n1] = b2p[(N2 * n1 + n2) * NZ2 + c];
            }
        };
        if (bres_src != bz) {
#pragma unroll
            for (int it = 0; it < RES; ++it) load(it, bres + it * N1);
            bres_src = bz;
        }
        auto store_items = [&](auto next_differs) {
            constexpr bool NB = decltype(next_differs)::value;
            /* items past the resident ones: loads one item ahead of their use */
            T2 cur[N1], nxt[N1];
            if (RES < ITEMS) load(RES, cur);
#pragma unroll
            for (int it = 0; it < ITEMS; ++it) {
                if (it >= RES && it + 1 < ITEMS) load(it + 1, nxt);
                const int w = tid + it * T, n2 = w / NZ2, c = w - n2 * NZ2;
                if (!ITEMS_EVEN && w >= N2 * NZ2) break;
                Cx<P> v[N1];
#pragma unroll
                for (int n1 = 0; n1 < N1; ++n1) {
                    const int e = (N2 * n1 + n2) * NZ2 + c;
                    const T2 y = reinterpret_cast<const T2 *>(X)[(N2 * n1 + n2) * ZP2 + c];
                    const T2 bv = it < RES ? bres[it * N1 + n1] : cur[n1];
                    T2 o;
                    o.x = y.x * bv.x;
                    o.y = y.y * bv.y;
                    reinterpret_cast<T2 *>(qn)[e] = o;
                    const T2 nb = NB ? n2p[e] : bv;
                    v[n1].x = o.x * nb.x;
                    v[n1].y = o.y * nb.y;
                }
                Dft<P, N1, false>::run(v);
#pragma unroll
                for (int k1 = 1; k1 < N1; ++k1) v[k1] = cmul(v[k1], TW[n2 * N1 + k1]);
#pragma unroll
                for (int k1 = 0; k1 < N1; ++k1) XC[(N2 * k1 + n2) * ZP2 + c] = v[k1];
                if (it >= RES) {
#pragma unroll
                    for (int n1 = 0; n1 < N1; ++n1) cur[n1] = nxt[n1];
                }
            }
        };
        if (bnext == bz)
            store_items(std::false_type{});
        else
            store_items(std::true_type{});
    } else {
        static_assert(NZ2 % TM == 0, "pairs must split evenly over the threads");
        constexpr int PER = NZ2 / TM; /* pairs per thread */
        constexpr int BATCH = PER;
        const T2 *b2p = reinterpret_cast<const T2 *>(bz);
        const T2 *n2p = reinterpret_cast<const T2 *>(bnext);
        const bool same_b = (bnext == bz);
        for (int j0 = 0; j0 < PER; j0 += BATCH) {
            T2 bb[BATCH];
#pragma unroll
            for (int j = 0; j < BATCH; ++j) bb[j] = b2p[tid + (j0 + j) * T];
#pragma unroll
            for (int j = 0; j < BATCH; ++j) {
                const int e = tid + (j0 + j) * T;
                const int x = e / NZ2, c = e - x * NZ2;
                T2 &slot = reinterpret_cast<T2 *>(X)[x * ZP2 + c];
                T2 o = slot;
                o.x *= bb[j].x;
                o.y *= bb[j].y;
                reinterpret_cast<T2 *>(qn)[e] = o;
                const T2 nb = same_b ? bb[j] : n2p[e];
                o.x *= nb.x;
                o.y *= nb.y;
                slot = o;
            }
        }
    }
    __syncthreads();
    if (stop_chain) break;
    } /* contour steps */
    if constexpr (ZTC) {
        /* every TMEM access of this CTA has completed (waited loads, and the
         * barrier above); the allocating warp frees the columns */
        tc_fence_before();
        __syncthreads();
        if (tid < 32) {
            tc_fence_after();
            asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(*tslot), "r"(ZTail<NZ>::TCOLS)
                         : "memory");
        }
    }
}

/* ---------------------------------------------------------------- dispatch */
template <typename P, int NX, int NZ, int N1, int N2>
static size_t smem_bytes_t()
{
    return Smem2D<P, NX, NZ>::END;
}

/* Dynamic shared memory of a launch. With the tensor-core z tail every CTA
 * holds TCOLS of the SM's 512 TMEM columns for its whole chain, so the request
 * is raised until no more CTAs fit on an SM than the columns serve: a CTA never
 * waits in tcgen05.alloc for another chain to end. */
template <typename P, int NX, int NZ, int N1, int N2>
static size_t smem_launch_t()
{
    static size_t cached = 0;
    if (cached) return cached;
    size_t s = Smem2D<P, NX, NZ>::END;
    if constexpr (Smem2D<P, NX, NZ>::TC) {
        const int maxc = 512 / ZTail<NZ>::TCOLS;
        int dev = 0, per_sm = 0, resv = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess) {
            cudaGetLastError();
            per_sm = 233472;
            resv = 1024;
        }
        /* (maxc + 1) CTAs of s + resv bytes each must not fit */
        const long need = (long)per_sm / (maxc + 1) - resv + 16;
        if (need > (long)s) s = (size_t)(need + 15) / 16 * 16;
    }
    cached = s;
    return s;
}

/* Two threads per line where the z phase is the split one (NZ/2 a multiple of 8). */
template <int NX, int NZ>
struct WideOk {
    static constexpr bool value = (NZ / 2) % 8 == 0 && SCFT_F32X2;
};

template <typename P, int NX, int NZ, int N1, int N2>
static cudaError_t launch_t(const Step2DArgs &a, int nblocks, cudaStream_t st, int configure, int wide)
{
    const size_t smem = smem_launch_t<P, NX, NZ, N1, N2>();
    if (configure) {
        cudaError_t e = cudaFuncSetAttribute(k_chain2d<P, NX, NZ, N1, N2, 1>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if constexpr (WideOk<NX, NZ>::value)
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(k_chain2d<P, NX, NZ, N1, N2, 2>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        return e;
    }
    if constexpr (WideOk<NX, NZ>::value) {
        if (wide) {
            k_chain2d<P, NX, NZ, N1, N2, 2><<<nblocks, 2 * NX, smem, st>>>(a);
            return cudaGetLastError();
        }
    }
    k_chain2d<P, NX, NZ, N1, N2, 1><<<nblocks, NX, smem, st>>>(a);
    return cudaGetLastError();
}

#define SCFT_STEP2D_SHAPES(X)                                                                                          \
    X(192, 96, 16, 12)                                                                                                 \
    X(192, 128, 16, 12)                                                                                                \
    X(128, 96, 16, 8)                                                                                                  \
    X(96, 64, 8, 12)                                                                                                   \
    X(64, 64, 8, 8)                                                                                                    \
    X(64, 32, 8, 8)                                                                                                    \
    X(32, 32, 8, 4)                                                                                                    \
    X(32, 24, 8, 4)                                                                                                    \
    X(32, 16, 8, 4)                                                                                                    \
    X(24, 16, 8, 3)                                                                                                    \
    X(16, 16, 4, 4)

/* Returns the shared-memory bytes of the fused step for (nx, nz) in this
 * precision, or 0 if the shape has no fused kernel. Only the FP32 form has
 * one: an FP64 or double-float row pair does not fit in registers, and those
 * forms are bound by arithmetic, so they keep the per-axis passes. */
size_t scft_step2d_smem(int prec, int nx, int nz)
{
#define X(NX_, NZ_, A_, B_)                                                                                           \
    if (nx == NX_ && nz == NZ_) return prec != SCFT_PREC_FP32 ? 0 : smem_bytes_t<float, NX_, NZ_, A_, B_>();
    SCFT_STEP2D_SHAPES(X)
#undef X
    return 0;
}

/* 1 if the fused FP32 loop of (nx, nz) applies the z operator as an FP32 band
 * plus a tensor-core tail (its operator table is then the band coefficients
 * and the bf16 pieces, not the FP32 halves). */
int scft_step2d_ztc(int prec, int nx, int nz)
{
    if (prec != SCFT_PREC_FP32) return 0;
#define X(NX_, NZ_, A_, B_) \
    if (nx == NX_ && nz == NZ_) return ZTcOk<float, NX_, NZ_>::value ? 1 : 0;
    SCFT_STEP2D_SHAPES(X)
#undef X
    return 0;
}

/* 1 if the shape has the two-threads-per-line kernel (bit-identical results,
 * for batches of at most one chain per SM). */
int scft_step2d_wide(int prec, int nx, int nz)
{
    if (prec != SCFT_PREC_FP32) return 0;
#define X(NX_, NZ_, A_, B_) \
    if (nx == NX_ && nz == NZ_) return WideOk<NX_, NZ_>::value ? 1 : 0;
    SCFT_STEP2D_SHAPES(X)
#undef X
    return 0;
}

/* configure = 1 raises the kernels' shared-memory limit (call once, outside
 * any stream capture); configure = 0 launches, with two threads per line if
 * wide is set and the shape has that kernel. */
cudaError_t scft_launch_step2d(int prec, int nx, int nz, const Step2DArgs &a, int nblocks, cudaStream_t st,
                               int configure, int wide)
{
#define X(NX_, NZ_, A_, B_)                                                                                           \
    if (nx == NX_ && nz == NZ_)                                                                                        \
        return prec != SCFT_PREC_FP32 ? cudaErrorInvalidValue                                                         \
                                      : launch_t<float, NX_, NZ_, A_, B_>(a, nblocks, st, configure, wide);
    SCFT_STEP2D_SHAPES(X)
#undef X
    return cudaErrorInvalidValue;
}

int scft_step2d_take_fault(void)
{
    int v = 0;
    const int zero = 0;
    if (cudaMemcpyFromSymbol(&v, g_scft_tc_fault, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (v) cudaMemcpyToSymbol(g_scft_tc_fault, &zero, sizeof(int));
    return v;
}

/* N1 of the four-step factorisation NX = N1 * N2 used for shape nx. */
int scft_step2d_n1(int nx)
{
#define X(NX_, NZ_, A_, B_) \
    if (nx == NX_) return A_;
    SCFT_STEP2D_SHAPES(X)
#undef X
    return 0;
}
