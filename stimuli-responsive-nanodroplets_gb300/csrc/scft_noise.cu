/*
 * scft_noise.cu — the reference's noise draws replayed on the device.
 *
 * funUpdate (SCFT.c:2044-2117) draws one Gaussian per active field per grid
 * point with funGaussDev (SCFT.c:1769-1782): Marsaglia's polar method on the
 * POSIX 48-bit generator drand48 (x <- a x + c mod 2^48), points in the loop
 * order k, j, i and fields in order A..S3, every iteration (also when the noise
 * is multiplied by MF = 0, SCFT.c:2103). The stream is sequential, but the
 * generator is affine, so any position is reachable by composing jump maps
 * x -> A x + C; the only data dependence is the polar rejection. Three passes
 * per instance and iteration:
 *   count  each thread walks a chunk of CH attempts (two draws each) from its
 *          jumped start state and counts the accepted ones;
 *   scan   exclusive prefix sum of the counts gives every accepted attempt its
 *          global draw index g;
 *   emit   draw g < G = n_active * M lands at (active field g % n_active, point
 *          g / n_active in the loop order); the chunk holding draw G-1 stores
 *          the state after it, the reference's state after the iteration.
 * The accept test uses separately rounded products and sum, as the reference's
 * double expression x1*x1 + x2*x2 evaluates without contraction; the integer
 * state is exact. The Gaussian itself goes through the device log and sqrt
 * (within an ulp of the host libm).
 */
#include <cuda_runtime.h>

#include "scft_internal.h"

#define RNG_THREADS 256
#define RNG_CH 32 /* attempts per thread chunk */

static const unsigned long long LCG_A = 0x5DEECE66DULL, LCG_C = 0xBULL, M48 = (1ULL << 48) - 1;

struct Affine {
    unsigned long long a, c; /* x -> a x + c (mod 2^48) */
};

/* jump[k] advances the state by 2*RNG_CH*2^k draws */
__constant__ Affine c_jump[48];

__device__ __forceinline__ unsigned long long lcg_next(unsigned long long x) { return (LCG_A * x + LCG_C) & M48; }

__device__ __forceinline__ unsigned long long jump_to_chunk(unsigned long long x, unsigned long long chunk)
{
    for (int k = 0; chunk; ++k, chunk >>= 1)
        if (chunk & 1ULL) x = (c_jump[k].a * x + c_jump[k].c) & M48;
    return x;
}

/* x1 = 2 u1 - 1 and w = x1*x1 + x2*x2 from the two draws' states, rounded as
 * the reference's double expressions are (each product and the sum separately) */
__device__ __forceinline__ void polar_values(unsigned long long s1, unsigned long long s2, double &x1, double &w)
{
    const double u1 = (double)s1 * 0x1.0p-48;
    const double u2 = (double)s2 * 0x1.0p-48;
    x1 = __dsub_rn(__dmul_rn(2.0, u1), 1.0);
    const double x2 = __dsub_rn(__dmul_rn(2.0, u2), 1.0);
    w = __dadd_rn(__dmul_rn(x1, x1), __dmul_rn(x2, x2));
}

/* One polar attempt from state x: advances x by two draws and returns the
 * reference's accept decision w < 1. The decision is taken in FP32 (x1, x2
 * are exact multiples of 2^-47; their FP32 roundings put w within 4e-7 of
 * its exact value) unless w is within 4e-6 of 1, where the reference's FP64
 * arithmetic decides. s1, s2: the two draws' states. */
__device__ __forceinline__ bool polar_attempt(unsigned long long &x, unsigned long long &s1, unsigned long long &s2)
{
    s1 = lcg_next(x);
    s2 = lcg_next(s1);
    x = s2;
    const float f1 = (float)((long long)s1 - (1LL << 47)) * 0x1.0p-47f;
    const float f2 = (float)((long long)s2 - (1LL << 47)) * 0x1.0p-47f;
    const float wf = f1 * f1 + f2 * f2;
    if (wf < 1.0f - 4e-6f) return true;
    if (wf > 1.0f + 4e-6f) return false;
    double x1, w;
    polar_values(s1, s2, x1, w);
    return w < 1.0;
}

__global__ void k_rng_count(NoiseArgs n)
{
    const int b = blockIdx.y;
    const long chunk = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (chunk >= n.nchunks || n.state[b].done) return;
    unsigned long long x = jump_to_chunk(n.state_in[b], (unsigned long long)chunk);
    int cnt = 0;
    unsigned long long s1, s2;
#pragma unroll 4
    for (int t = 0; t < RNG_CH; ++t) cnt += polar_attempt(x, s1, s2) ? 1 : 0;
    n.counts[(long)b * n.nchunks + chunk] = cnt;
}

/* exclusive scan of one instance's chunk counts (one CTA per instance) */
__global__ void k_rng_scan(NoiseArgs n)
{
    __shared__ long warp_tot[32];
    __shared__ long carry;
    const int b = blockIdx.x;
    if (n.state[b].done) return; /* uniform over the CTA */
    const int *cnt = n.counts + (long)b * n.nchunks;
    long *pre = n.prefix + (long)b * n.nchunks;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (long base = 0; base < n.nchunks; base += blockDim.x) {
        const long i = base + threadIdx.x;
        long v = i < n.nchunks ? cnt[i] : 0;
        long incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) warp_tot[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            long wt = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
            long wincl = wt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const long t = __shfl_up_sync(0xffffffffu, wincl, o);
                if (lane >= o) wincl += t;
            }
            if (lane < (int)(blockDim.x >> 5)) warp_tot[lane] = wincl - wt; /* exclusive warp offsets */
        }
        __syncthreads();
        const long excl = carry + warp_tot[wid] + (incl - v);
        if (i < n.nchunks) pre[i] = excl;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) n.total[b] = carry;
}

__global__ void k_rng_emit(NoiseArgs n)
{
    const int b = blockIdx.y;
    const long chunk = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (chunk >= n.nchunks || n.state[b].done) return;
    const InstParams &ip = n.params[b];
    const unsigned long iter = n.state[b].iter;
    const double mf = iter > (unsigned long)ip.relaxation ? 0.0 : 1.0;
    const bool write = (ip.dt_noise * mf != 0.0);
    const long G = (long)ip.n_active * n.m;
    long g = n.prefix[(long)b * n.nchunks + chunk];
    if (g >= G) return;
    /* with MF*DT_NOISE == 0 the draws are not used: only the chunk holding draw
     * G-1 replays its attempts, to leave the state where the reference's is */
    if (!write && g + n.counts[(long)b * n.nchunks + chunk] < G) return;
    unsigned long long x = jump_to_chunk(n.state_in[b], (unsigned long long)chunk);
    unsigned long long s1, s2;
    const int na = ip.n_active;
    for (int t = 0; t < RNG_CH && g < G; ++t) {
        if (!polar_attempt(x, s1, s2)) continue;
        if (write) {
            double x1, w;
            polar_values(s1, s2, x1, w);
            const double v = x1 * sqrt((-2.0 * log(w)) / w);
            const long p = g / na;
            const int a = (int)(g - p * na);
            const long plane = (long)n.ny * n.nx;
            const long k = p / plane, rem = p - k * plane;
            const long j = rem / n.nx, i = rem - j * n.nx;
            const long idx = k + (long)n.nz * (j + (long)n.ny * i);
            n.noise[((long)b * na + a) * n.sm + idx] = v;
        }
        if (g == G - 1) n.state[b].rng = x;
        ++g;
    }
}

__global__ void k_rng_snapshot(NoiseArgs n)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < n.B) n.state_in[b] = n.state[b].rng;
}

__global__ void k_rng_check(NoiseArgs n)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < n.B && !n.state[b].done) {
        const long G = (long)n.params[b].n_active * n.m;
        if (n.total[b] < G) n.state[b].status = SCFT_ERR_STATE; /* not enough attempts: never expected */
    }
}

/* ------------------------------------------------------------ host side */
static Affine compose(Affine f, Affine g) /* g after f */
{
    Affine h;
    h.a = (g.a * f.a) & M48;
    h.c = (g.a * f.c + g.c) & M48;
    return h;
}

long scft_noise_chunks(long m, int n_active)
{
    const long G = (long)n_active * m;
    const long attempts = (G * 27) / 20 + 1024; /* 1.35 G: acceptance is pi/4 = 0.785 */
    return (attempts + RNG_CH - 1) / RNG_CH;
}

cudaError_t scft_noise_setup(void)
{
    Affine step = {LCG_A, LCG_C}, id = {1, 0};
    Affine chunk = id;
    for (int t = 0; t < 2 * RNG_CH; ++t) chunk = compose(chunk, step);
    Affine tab[48];
    tab[0] = chunk;
    for (int k = 1; k < 48; ++k) tab[k] = compose(tab[k - 1], tab[k - 1]);
    return cudaMemcpyToSymbol(c_jump, tab, sizeof(tab));
}

cudaError_t scft_noise_launch(const NoiseArgs &n, cudaStream_t st)
{
    k_rng_snapshot<<<(n.B + 127) / 128, 128, 0, st>>>(n);
    dim3 g((unsigned)((n.nchunks + RNG_THREADS - 1) / RNG_THREADS), n.B);
    k_rng_count<<<g, RNG_THREADS, 0, st>>>(n);
    k_rng_scan<<<n.B, 1024, 0, st>>>(n);
    k_rng_emit<<<g, RNG_THREADS, 0, st>>>(n);
    k_rng_check<<<(n.B + 127) / 128, 128, 0, st>>>(n);
    return cudaGetLastError();
}
