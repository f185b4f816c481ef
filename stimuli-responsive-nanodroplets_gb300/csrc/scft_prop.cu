/*
 * scft_prop.cu — the contour step of the modified diffusion equation,
 *   q_{s+1} = b . exp(ds Laplacian) . (b . q_s),   b = exp(-DS w / 2),
 * the operator funPDESolver_periodic (SCFT.c:2474-2525) and
 * funPDESolver_DirichletBC (SCFT.c:2527-2631) apply with two 3D FFTs.
 *
 * GB300 form. The diffusion factor exp(-ax kx^2 - ay ky^2 - az kz^2) is a
 * product of one factor per axis, so the step is applied one axis at a time:
 *   - periodic axis of length n: real lines are packed two per complex line
 *     (the factor is real and even in k, so real and imaginary parts never
 *     mix), transformed with a shared-memory Stockham FFT (radix 4/2/3),
 *     scaled by E(k)/n and transformed back;
 *   - Dirichlet z axis (MASK 1): the reference's odd extension of length
 *     2(NZ+1) makes the z factor a DST-I; its matrix K = (2/L) S diag(E) S is
 *     symmetric and centrosymmetric, so y = K x is applied as two half-size
 *     dense products on x_i +- x_{n-1-i} (n^2/2 multiply-adds per line), which
 *     also covers lengths with large prime factors (NZ+1 = 97, 43*3).
 * Each pass is one launch over (line tile, chain) for every chain of every
 * instance that is active at contour step s; the first pass multiplies by b
 * on load, the last multiplies by b on store and writes slice s+1.
 *
 * The kernels are written once over the value type P: double (plain form),
 * float (per-axis passes of the FP32 form) and dfloat (the FP32x2 form: slices,
 * Boltzmann factors and operator tables stored as FP32 pairs, every operation
 * in double-float arithmetic; FP64 only converts the line length for the mean
 * mode's division).
 */
#include <cuda_runtime.h>

#include <type_traits>

#include "scft_dfloat.cuh"
#include "scft_internal.h"

template <typename P>
struct Cx {
    P x, y;
};

template <typename P>
__device__ __forceinline__ Cx<P> cmul(Cx<P> a, Cx<P> b)
{
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
/* double-float complex product: each part is one two-product difference with a
 * single renormalisation */
__device__ __forceinline__ Cx<dfloat> cmul(Cx<dfloat> a, Cx<dfloat> b)
{
    return {dfo::mul_sub(a.x, b.x, a.y, b.y), dfo::mul_add(a.x, b.y, a.y, b.x)};
}
template <typename P>
__device__ __forceinline__ Cx<P> cadd(Cx<P> a, Cx<P> b) { return {a.x + b.x, a.y + b.y}; }
template <typename P>
__device__ __forceinline__ Cx<P> csub(Cx<P> a, Cx<P> b) { return {a.x - b.x, a.y - b.y}; }

/* multiply by sign*i: forward (sign=-1) gives (y, -x), inverse gives (-y, x) */
template <typename P, bool INV>
__device__ __forceinline__ Cx<P> mul_si(Cx<P> a)
{
    return INV ? Cx<P>{-a.y, a.x} : Cx<P>{a.y, -a.x};
}

template <typename P, bool INV>
__device__ __forceinline__ void dft2(Cx<P> *v)
{
    Cx<P> a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}

template <typename P, bool INV>
__device__ __forceinline__ void dft4(Cx<P> *v)
{
    Cx<P> b0 = cadd(v[0], v[2]), b1 = csub(v[0], v[2]);
    Cx<P> b2 = cadd(v[1], v[3]), b3 = mul_si<P, INV>(csub(v[1], v[3]));
    v[0] = cadd(b0, b2);
    v[1] = cadd(b1, b3);
    v[2] = csub(b0, b2);
    v[3] = csub(b1, b3);
}

template <typename P, bool INV>
__device__ __forceinline__ void dft3(Cx<P> *v)
{
    const P h = (P)0.86602540378443864676; /* sqrt(3)/2 */
    Cx<P> s = cadd(v[1], v[2]);
    Cx<P> d = csub(v[1], v[2]);
    Cx<P> c = {v[0].x - (P)0.5 * s.x, v[0].y - (P)0.5 * s.y};
    Cx<P> e = mul_si<P, INV>(d); /* sign*i*d */
    v[0] = cadd(v[0], s);
    v[1] = {c.x + h * e.x, c.y + h * e.y};
    v[2] = {c.x - h * e.x, c.y - h * e.y};
}

/* floor(x / d) for x * d < 2^32, given mag = ceil(2^32 / d) (0 for d = 1) */
__device__ __forceinline__ int div_mag(int x, unsigned mag) { return mag ? (int)__umulhi((unsigned)x, mag) : x; }

/* One Stockham autosort stage (Govindaraju et al., SC'08 formulation) over nl
 * complex lines of length n with line pitch ldl. tw[t] = exp(-2 pi i t / n).
 * The double-float stages divide by multiply-high with the host-computed
 * reciprocals and index the twiddles without a reduction modulo n
 * (r * k * tws < n); the FP32 and FP64 stages keep integer division, as
 * measured fastest for them. */
template <typename P, bool INV, int R>
__device__ __forceinline__ void stockham_stage(const Cx<P> *__restrict__ a, Cx<P> *__restrict__ b, int n, int ldl,
                                               int nl, int Ns, unsigned mag_nr, unsigned mag_ns,
                                               const Cx<P> *__restrict__ tw)
{
    const int nr = n / R;
    const int tws = n / (Ns * R);
    constexpr bool DF = std::is_same<P, dfloat>::value;
    for (int w = threadIdx.x; w < nl * nr; w += blockDim.x) {
        const int line = DF ? div_mag(w, mag_nr) : w / nr;
        const int j = w - line * nr;
        const Cx<P> *in = a + line * ldl;
        Cx<P> *out = b + line * ldl;
        const int jq = DF ? div_mag(j, mag_ns) : j / Ns;
        const int k = j - jq * Ns;
        Cx<P> v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            v[r] = in[j + r * nr];
            if (r > 0 && k > 0) {
                Cx<P> t = tw[DF ? r * k * tws : (r * k * tws) % n];
                if (INV) t.y = -t.y;
                v[r] = cmul(v[r], t);
            }
        }
        if (R == 2) dft2<P, INV>(v);
        if (R == 3) dft3<P, INV>(v);
        if (R == 4) dft4<P, INV>(v);
        const int base = jq * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) out[base + r * Ns] = v[r];
    }
}

/* Full transform; returns the buffer holding the result. */
template <typename P, bool INV>
__device__ Cx<P> *stockham(Cx<P> *a, Cx<P> *b, int n, int ldl, int nl, const AxisGeom &g, const Cx<P> *tw)
{
    int Ns = 1;
    for (int st = 0; st < g.nrad; ++st) {
        const int R = g.rad[st];
        const unsigned mnr = g.mag_nr[st], mns = g.mag_ns[st];
        if (R == 4)
            stockham_stage<P, INV, 4>(a, b, n, ldl, nl, Ns, mnr, mns, tw);
        else if (R == 2)
            stockham_stage<P, INV, 2>(a, b, n, ldl, nl, Ns, mnr, mns, tw);
        else
            stockham_stage<P, INV, 3>(a, b, n, ldl, nl, Ns, mnr, mns, tw);
        __syncthreads();
        Cx<P> *t = a;
        a = b;
        b = t;
        Ns *= R;
    }
    return a;
}



/* Dot-product accumulator of the dense z pass: a plain multiply-add chain in
 * FP32 and FP64 (the expression the plain form has always used), the
 * compensated double-float accumulator for dfloat. */
template <typename P>
struct DotOf {
    P s;
    __device__ __forceinline__ void zero() { s = (P)0; }
    __device__ __forceinline__ void add(P a, P b) { s += a * b; }
    __device__ __forceinline__ P value() const { return s; }
};
template <>
struct DotOf<dfloat> {
    DotDF d;
    __device__ __forceinline__ void zero() { d.zero(); }
    __device__ __forceinline__ void add(dfloat a, dfloat b) { d.add(a, b); }
    __device__ __forceinline__ dfloat value() const { return d.value(); }
};

template <typename P>
__device__ __forceinline__ long elem_offset(const AxisGeom &g, long L, int t)
{
    const long o = L / g.inner;
    const long c = L - o * g.inner;
    return o * (long)g.n * g.ls + c + (long)g.ls * t;
}

template <typename P>
__global__ void __launch_bounds__(256) k_pass_fft(AxisGeom g, PassArgs a)
{
    const ChainDesc cd = a.chains[blockIdx.y];
    if (a.state && a.state[cd.instance].done) return; /* uniform over the CTA */
    if (a.s >= cd.len - 1) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = g.n;
    const int nl = (a.tile + 1) / 2;
    const int ldl = n + 1;
    Cx<P> *buf0 = reinterpret_cast<Cx<P> *>(smem_raw);
    Cx<P> *buf1 = buf0 + nl * ldl;
    Cx<P> *tw = buf1 + nl * ldl;
    P *spec = reinterpret_cast<P *>(tw + n);

    const P *src = a.first ? reinterpret_cast<const P *>(cd.q) + (long)a.s * a.sstride
                           : reinterpret_cast<const P *>(cd.tmp);
    P *dst = a.last ? reinterpret_cast<P *>(cd.q) + (long)(a.s + 1) * a.sstride : reinterpret_cast<P *>(cd.tmp);
    const P *bz = reinterpret_cast<const P *>(a.s < cd.seg_end ? cd.b0 : cd.b1);

    const Cx<P> *gtw = reinterpret_cast<const Cx<P> *>(cd.ops->tw[a.axis]);
    const P *gspec = reinterpret_cast<const P *>(cd.ops->spec[a.axis]);
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        tw[t] = gtw[t];
        spec[t] = gspec[t];
    }
    const int total = a.tile * n;
    const bool contiguous = (g.ls == 1);
    const long L0 = (long)blockIdx.x * a.tile;
    for (int e = threadIdx.x; e < nl * 2 * n; e += blockDim.x) {
        /* zero the imaginary half of a trailing unpaired line */
        const int l = e / n, t = e - l * n;
        if (l >= a.tile) reinterpret_cast<P *>(&buf0[(l / 2) * ldl + t])[l & 1] = (P)0;
    }
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        int l, t;
        if (contiguous) {
            l = e / n;
            t = e - l * n;
        } else {
            t = e / a.tile;
            l = e - t * a.tile;
        }
        const long off = elem_offset<P>(g, L0 + l, t);
        P v = src[off];
        if (a.first) v *= bz[off];
        reinterpret_cast<P *>(&buf0[(l >> 1) * ldl + t])[l & 1] = v;
    }
    __syncthreads();
    Cx<P> *r = stockham<P, false>(buf0, buf1, n, ldl, nl, g, tw);
    for (int e = threadIdx.x; e < nl * n; e += blockDim.x) {
        const int l = e / n, t = e - l * n;
        Cx<P> v = r[l * ldl + t];
        if (t == 0) {
            /* mean mode, E(0) = 1: divide by n (correctly rounded) rather than
             * multiply by a rounded 1/n, so its per-step gain is unbiased */
            r[l * ldl] = {v.x / (P)n, v.y / (P)n};
            continue;
        }
        const P f = spec[t];
        r[l * ldl + t] = {v.x * f, v.y * f};
    }
    __syncthreads();
    Cx<P> *other = (r == buf0) ? buf1 : buf0;
    r = stockham<P, true>(r, other, n, ldl, nl, g, tw);
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        int l, t;
        if (contiguous) {
            l = e / n;
            t = e - l * n;
        } else {
            t = e / a.tile;
            l = e - t * a.tile;
        }
        const long off = elem_offset<P>(g, L0 + l, t);
        P v = reinterpret_cast<const P *>(&r[(l >> 1) * ldl + t])[l & 1];
        if (a.last) v *= bz[off];
        dst[off] = v;
    }
}

template <typename P>
__global__ void __launch_bounds__(256) k_pass_dense(AxisGeom g, PassArgs a)
{
    const ChainDesc cd = a.chains[blockIdx.y];
    if (a.state && a.state[cd.instance].done) return; /* uniform over the CTA */
    if (a.s >= cd.len - 1) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = g.n, h = a.h;
    /* double-float: u and v rows have an odd pitch (h + 1 values), so the two
     * lines a warp can span broadcast from different banks (the space is
     * reserved for every type; FP32 and FP64 keep the dense pitch h) */
    const int hp = std::is_same<P, dfloat>::value ? h + 1 : h;
    P *x = reinterpret_cast<P *>(smem_raw);   /* tile * n */
    P *u = x + a.tile * n;                    /* tile * hp */
    P *v = u + a.tile * hp;                   /* tile * hp */
    P *kA = v + a.tile * hp;                  /* h * h */
    P *kB = kA + h * h;                       /* h * h (even n) */

    const P *src = a.first ? reinterpret_cast<const P *>(cd.q) + (long)a.s * a.sstride
                           : reinterpret_cast<const P *>(cd.tmp);
    P *dst = a.last ? reinterpret_cast<P *>(cd.q) + (long)(a.s + 1) * a.sstride : reinterpret_cast<P *>(cd.tmp);
    const P *bz = reinterpret_cast<const P *>(a.s < cd.seg_end ? cd.b0 : cd.b1);
    const P *gA = reinterpret_cast<const P *>(cd.ops->kA[a.axis]);
    const P *gB = reinterpret_cast<const P *>(cd.ops->kB[a.axis]);
    for (int e = threadIdx.x; e < h * h; e += blockDim.x) {
        kA[e] = gA[e];
        if (a.even) kB[e] = gB[e];
    }
    const int total = a.tile * n;
    const bool contiguous = (g.ls == 1);
    const long L0 = (long)blockIdx.x * a.tile;
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        int l, t;
        if (contiguous) {
            l = e / n;
            t = e - l * n;
        } else {
            t = e / a.tile;
            l = e - t * a.tile;
        }
        const long off = elem_offset<P>(g, L0 + l, t);
        P val = src[off];
        if (a.first) val *= bz[off];
        x[l * n + t] = val;
    }
    __syncthreads();
    if (a.even) {
        for (int e = threadIdx.x; e < a.tile * h; e += blockDim.x) {
            const int l = e / h, i = e - l * h;
            const P p0 = x[l * n + i], p1 = x[l * n + n - 1 - i];
            u[l * hp + i] = p0 + p1;
            v[l * hp + i] = p0 - p1;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < a.tile * h; e += blockDim.x) {
            const int l = e / h, i = e - l * h;
            const P *ul = u + l * hp;
            const P *vl = v + l * hp;
            DotOf<P> sacc, dacc;
            sacc.zero();
            dacc.zero();
            for (int j = 0; j < h; ++j) {
                sacc.add(kA[j * h + i], ul[j]);
                dacc.add(kB[j * h + i], vl[j]);
            }
            const long o0 = elem_offset<P>(g, L0 + l, i);
            const long o1 = elem_offset<P>(g, L0 + l, n - 1 - i);
            const P sv = sacc.value(), dv = dacc.value();
            P y0 = sv + dv, y1 = sv - dv;
            if (a.last) {
                y0 *= bz[o0];
                y1 *= bz[o1];
            }
            dst[o0] = y0;
            dst[o1] = y1;
        }
    } else {
        for (int e = threadIdx.x; e < a.tile * n; e += blockDim.x) {
            const int l = e / n, i = e - l * n;
            const P *xl = x + l * n;
            DotOf<P> dot;
            dot.zero();
            for (int j = 0; j < n; ++j) dot.add(kA[j * n + i], xl[j]);
            P acc = dot.value();
            const long o0 = elem_offset<P>(g, L0 + l, i);
            if (a.last) acc *= bz[o0];
            dst[o0] = acc;
        }
    }
}

/* ------------------------------------------------------------- launchers */
size_t scft_pass_smem_bytes(const AxisGeom &g, int tile, int h, int psize)
{
    if (g.dirichlet) {
        const int n = g.n;
        return (size_t)psize * ((size_t)tile * n + 2 * (size_t)tile * (h + 1) + 2 * (size_t)h * h);
    }
    const int nl = (tile + 1) / 2;
    return (size_t)psize * (2 * 2 * (size_t)nl * (g.n + 1) + 2 * (size_t)g.n + g.n);
}

template <typename P>
static cudaError_t launch_pass_t(const AxisGeom &g, const PassArgs &a, int ntiles, cudaStream_t st)
{
    const size_t smem = scft_pass_smem_bytes(g, a.tile, a.h, (int)sizeof(P));
    const dim3 grid(ntiles, a.nchains);
    if (g.dirichlet)
        k_pass_dense<P><<<grid, 256, smem, st>>>(g, a);
    else
        k_pass_fft<P><<<grid, 256, smem, st>>>(g, a);
    return cudaGetLastError();
}

cudaError_t scft_launch_pass(int prec, const AxisGeom &g, const PassArgs &a, int ntiles, cudaStream_t st)
{
    if (prec == SCFT_PREC_FP64) return launch_pass_t<double>(g, a, ntiles, st);
    if (prec == SCFT_PREC_FP32X2) return launch_pass_t<dfloat>(g, a, ntiles, st);
    return launch_pass_t<float>(g, a, ntiles, st);
}

/* Raise the dynamic shared-memory limit of the pass kernels once, outside any
 * stream capture. */
cudaError_t scft_pass_configure(int smem_bytes)
{
    cudaError_t e = cudaSuccess;
    const cudaFuncAttribute A = cudaFuncAttributeMaxDynamicSharedMemorySize;
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_pass_fft<double>, A, smem_bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_pass_fft<float>, A, smem_bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_pass_dense<double>, A, smem_bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_pass_dense<float>, A, smem_bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_pass_fft<dfloat>, A, smem_bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_pass_dense<dfloat>, A, smem_bytes);
    return e;
}
