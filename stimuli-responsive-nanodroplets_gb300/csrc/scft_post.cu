/*
 * scft_post.cu — everything in one SCFT iteration except the contour steps:
 * Boltzmann factors and initial slices, Q reductions, contour-integrated
 * densities, and the fused free-energy / field-update pass with its
 * reductions. All reductions are FP64 and run in a fixed order, so a result
 * does not depend on which other instances share the launch.
 */
#include <cuda_runtime.h>
#include <math.h>

#include <type_traits>

#include "scft_dfloat.cuh"
#include "scft_internal.h"

#define POST_THREADS 256



__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

/* Fixed-order block reduction of NV values; thread 0 gets the sums. */
template <int NV>
__device__ void block_sum(double (&v)[NV], double *sh)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) sh[k * 32 + wid] = v[k];
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double t = lane < nw ? sh[k * 32 + lane] : 0.0;
            v[k] = warp_sum(t);
        }
    }
    __syncthreads();
}

/* ---------------------------------------------------------- iteration begin */
__global__ void k_iter_begin(PostArgs a)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < a.B) {
        a.state[b].tick += 1;
        if (a.state[b].done == 2) a.state[b].done = 1; /* converged in the previous iteration */
        if (!a.state[b].done) {
            a.state[b].iter += 1; /* iIter++ (SCFT.c:1090) */
            a.state[b].status = SCFT_OK;
        }
    }
}

__global__ void k_iter_start_mark(PostArgs a)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < a.B) a.state[b].tick = 0;
}

/* Boltzmann factor exp(DS * (-w/2)) (SCFT.c:2344) in the propagator precision:
 * the FP64 exponential for the plain form. For the FP32 form the argument is
 * formed in FP64 and the factor taken as 1 + expm1f(arg): with |arg| of a few
 * hundredths the error of expm1f is a small fraction of an ulp of the factor,
 * so the result is the round-to-nearest of the exact factor except next to a
 * rounding boundary — no systematic bias that would add up over a chain's
 * contour steps — without the FP64 pipe GB300 runs at 1/58 of the FP32 rate. */
template <typename P>
__device__ __forceinline__ P boltz(double ds, double w)
{
    const double arg = ds * (-w / 2.0);
    if constexpr (sizeof(P) == 4)
        return 1.0f + expm1f((float)arg);
    else
        return P(exp(arg)); /* FP64, or the FP32 pair nearest the FP64 value */
}

/* b for the fields chains use, and the initial slice of every chain: 1, the
 * grafting mask (SCFT.c:2441) or the single-point seed while iIter <=
 * SEED_STEPS (SCFT.c:2346-2367). */
template <typename P>
__global__ void k_boltz_init(PostArgs a)
{
    const int b = blockIdx.y;
    if (a.state[b].done) return;
    const InstParams &ip = a.params[b];
    const unsigned long iter = a.state[b].iter;
    const bool seed_on = ip.enable_seed && iter <= (unsigned long)ip.seed_steps;
    P *bz = reinterpret_cast<P *>(a.bz) + (long)b * SCFT_NFIELDS * a.sm;
    const double *w = a.w + (long)b * 14 * a.sm;
    for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < a.m; idx += (long)gridDim.x * blockDim.x) {
        for (int f = 0; f < SCFT_NFIELDS; ++f)
            if (a.field_use >> f & 1u) bz[f * a.sm + idx] = boltz<P>(ip.ds, w[f * a.sm + idx]);
        const int k = (int)(idx % a.nz);
        const int j = (int)((idx / a.nz) % a.ny);
        const int i = (int)(idx / ((long)a.nz * a.ny));
        for (int c = 0; c < a.nchains; ++c) {
            const ChainDesc &cd = a.chains[b * a.nchains + c];
            P v = (P)1;
            if (cd.init == SCFT_INIT_MASK) {
                v = (P)a.mask[((long)b * 3 + cd.init_arg) * a.sm + idx];
            } else if (cd.init == SCFT_INIT_SEED && seed_on) {
                const int D = ip.seed_area_delta;
                const bool in = i > (a.nx / 2 - D) && i < (a.nx / 2 + D) && j > (a.ny / 2 - D) && j < (a.ny / 2 + D) &&
                                k > (a.nz / 4 - D) && k < (a.nz / 4 + D);
                v = in ? (P)1 : (P)0;
            }
            reinterpret_cast<P *>(cd.q)[idx] = v;
        }
    }
}

/* ------------------------------------------------------------------ Q */
/* Partial sums of q(r, NS_EFF-1) per species (funChemPotential, SCFT.c:1837-1859). */
template <typename P>
__global__ void __launch_bounds__(POST_THREADS) k_q_partial(PostArgs a)
{
    __shared__ double sh[32];
    const int sp = blockIdx.y, b = blockIdx.z;
    const SpeciesDesc sd = a.species[b * SCFT_NSPECIES + sp];
    if (!sd.present || a.state[b].done) return;
    const ChainDesc &cd = a.chains[b * a.nchains + sd.q_chain];
    const P *q = reinterpret_cast<const P *>(cd.q) + (long)(sd.len - 1) * a.sm;
    double v[1] = {0.0};
    for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < a.m; idx += (long)gridDim.x * blockDim.x)
        v[0] += (double)q[idx];
    block_sum<1>(v, sh);
    if (threadIdx.x == 0) a.partial[((long)b * SCFT_NSPECIES + sp) * gridDim.x + blockIdx.x] = v[0];
}

__global__ void k_q_final(PostArgs a, int nparts)
{
    const int sp = blockIdx.x, b = blockIdx.y;
    if (threadIdx.x != 0 || a.state[b].done) return;
    const SpeciesDesc sd = a.species[b * SCFT_NSPECIES + sp];
    double q = 0.0;
    if (sd.present) {
        const double *p = a.partial + ((long)b * SCFT_NSPECIES + sp) * nparts;
        double s = 0.0;
        for (int k = 0; k < nparts; ++k) s += p[k];
        q = s / (double)a.m; /* qrsum / dVol, SCFT.c:1861 */
    }
    a.state[b].q[sp] = q;
}

/* ------------------------------------------------------------- density */
/* Unnormalised Simpson sum of q(s) q+(NS_EFF-1-s) over [start, stop] with the
 * reference's index sets (funDensity, SCFT.c:2281-2297): weight 1 at both
 * ends, 4 at odd offsets up to stop-1, 2 at even offsets up to stop-2. For an
 * odd number of intervals the point stop-1 therefore gets no weight, as in
 * the reference. Each thread owns V consecutive points (one 16-byte load per
 * slice) and the contour loops are unrolled so that several slices are in
 * flight per thread; products and sums are FP64. */
/* Contour accumulators. FP64 form: plain FP64. FP32 form: double-float
 * (hi + lo) sums of exact products (fma gives the rounding error of x*y, Knuth's
 * TwoSum the error of each addition), which keeps about 48 significant bits,
 * at FP32 rate; the FP64 pipe of GB300 runs at 1/58 of the FP32 rate and
 * otherwise bounds this kernel. */
struct AccD {
    double s;
    __device__ __forceinline__ void zero() { s = 0.0; }
    __device__ __forceinline__ void add(double x, double y) { s += x * y; }
    __device__ __forceinline__ double value() const { return s; }
};
struct AccF {
    float hi, lo;
    __device__ __forceinline__ void zero() { hi = lo = 0.0f; }
    __device__ __forceinline__ void add(float x, float y)
    {
        const float p = x * y;
        const float e = fmaf(x, y, -p);
        const float t = hi + p;
        const float bb = t - hi;
        const float err = (hi - (t - bb)) + (p - bb);
        hi = t;
        lo += err + e;
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

/* FP32x2 form: products of double-float slices, compensated double-float sums */
struct AccDF {
    DotDF d;
    __device__ __forceinline__ void zero() { d.zero(); }
    __device__ __forceinline__ void add(dfloat x, dfloat y) { d.add(x, y); }
    __device__ __forceinline__ double value() const { return (double)d.hi + (double)d.lo; }
};

template <typename P>
struct AccOf;
template <>
struct AccOf<double> {
    using T = AccD;
};
template <>
struct AccOf<float> {
    using T = AccF;
};
template <>
struct AccOf<dfloat> {
    using T = AccDF;
};

template <typename P, int V>
__device__ __forceinline__ void load_p(const P *p, P (&o)[V])
{
    if constexpr (std::is_same<P, dfloat>::value) {
        const float4 t = *reinterpret_cast<const float4 *>(p); /* two double-float values */
        o[0] = P(t.x, t.y);
        o[1] = P(t.z, t.w);
    } else if (V == 4) {
        const float4 t = *reinterpret_cast<const float4 *>(p);
        reinterpret_cast<float *>(o)[0] = t.x;
        reinterpret_cast<float *>(o)[1] = t.y;
        reinterpret_cast<float *>(o)[2] = t.z;
        reinterpret_cast<float *>(o)[3] = t.w;
    } else {
        const double2 t = *reinterpret_cast<const double2 *>(p);
        reinterpret_cast<double *>(o)[0] = t.x;
        reinterpret_cast<double *>(o)[1] = t.y;
    }
}

template <typename P>
__global__ void __launch_bounds__(POST_THREADS) k_density(PostArgs a)
{
    constexpr int V = sizeof(P) == 4 ? 4 : 2;
    using Acc = typename AccOf<P>::T;
    const int blk = blockIdx.y, b = blockIdx.z;
    if (a.state[b].done) return;
    const BlockDesc bd = a.blocks[b * a.nblocks + blk];
    const P *qf = reinterpret_cast<const P *>(a.chains[b * a.nchains + bd.chain_f].q);
    const P *qb = reinterpret_cast<const P *>(a.chains[b * a.nchains + bd.chain_b].q);
    double *out = a.raw + ((long)b * a.nblocks + blk) * a.sm;
    const int top = bd.len - 1;
    const bool sym = bd.chain_f == bd.chain_b && bd.start == 0 && bd.stop == top && (top % 2) == 0;
    const long nvec = a.m / V;
    for (long iv = blockIdx.x * (long)blockDim.x + threadIdx.x; iv < (a.m + V - 1) / V;
         iv += (long)gridDim.x * blockDim.x) {
        const long idx = iv * V;
        if (iv < nvec && sym) {
            /* one chain with an even number of intervals: term s equals term top-s
             * and both have the same weight, so each slice is read once and the
             * pair sums count twice (the middle term once) */
            const int mid = top / 2;
            Acc e2[V], h4[V], h2[V], mm[V];
            P x[V], y[V];
#pragma unroll
            for (int v = 0; v < V; ++v) {
                e2[v].zero();
                h4[v].zero();
                h2[v].zero();
                mm[v].zero();
            }
            load_p<P, V>(qf + idx, x);
            load_p<P, V>(qf + (long)top * a.sm + idx, y);
#pragma unroll
            for (int v = 0; v < V; ++v) e2[v].add(x[v], y[v]);
#pragma unroll 4
            for (int s = 1; s < mid; s += 2) {
                load_p<P, V>(qf + (long)s * a.sm + idx, x);
                load_p<P, V>(qf + (long)(top - s) * a.sm + idx, y);
#pragma unroll
                for (int v = 0; v < V; ++v) h4[v].add(x[v], y[v]);
            }
#pragma unroll 4
            for (int s = 2; s < mid; s += 2) {
                load_p<P, V>(qf + (long)s * a.sm + idx, x);
                load_p<P, V>(qf + (long)(top - s) * a.sm + idx, y);
#pragma unroll
                for (int v = 0; v < V; ++v) h2[v].add(x[v], y[v]);
            }
            if (mid > 0) {
                load_p<P, V>(qf + (long)mid * a.sm + idx, x);
#pragma unroll
                for (int v = 0; v < V; ++v) mm[v].add(x[v], x[v]);
            }
            const double w_mid = mid == 0 ? 0.0 : ((mid & 1) ? 4.0 : 2.0);
#pragma unroll
            for (int v = 0; v < V; ++v)
                out[idx + v] = 2.0 * e2[v].value() + 8.0 * h4[v].value() + 4.0 * h2[v].value() + w_mid * mm[v].value();
        } else if (iv < nvec) {
            Acc ends[V], a4[V], a2[V];
            P x[V], y[V];
#pragma unroll
            for (int v = 0; v < V; ++v) {
                ends[v].zero();
                a4[v].zero();
                a2[v].zero();
            }
            load_p<P, V>(qf + (long)bd.start * a.sm + idx, x);
            load_p<P, V>(qb + (long)(top - bd.start) * a.sm + idx, y);
#pragma unroll
            for (int v = 0; v < V; ++v) ends[v].add(x[v], y[v]);
            load_p<P, V>(qf + (long)bd.stop * a.sm + idx, x);
            load_p<P, V>(qb + (long)(top - bd.stop) * a.sm + idx, y);
#pragma unroll
            for (int v = 0; v < V; ++v) ends[v].add(x[v], y[v]);
#pragma unroll 4
            for (int s = bd.start + 1; s <= bd.stop - 1; s += 2) {
                load_p<P, V>(qf + (long)s * a.sm + idx, x);
                load_p<P, V>(qb + (long)(top - s) * a.sm + idx, y);
#pragma unroll
                for (int v = 0; v < V; ++v) a4[v].add(x[v], y[v]);
            }
#pragma unroll 4
            for (int s = bd.start + 2; s <= bd.stop - 2; s += 2) {
                load_p<P, V>(qf + (long)s * a.sm + idx, x);
                load_p<P, V>(qb + (long)(top - s) * a.sm + idx, y);
#pragma unroll
                for (int v = 0; v < V; ++v) a2[v].add(x[v], y[v]);
            }
#pragma unroll
            for (int v = 0; v < V; ++v) out[idx + v] = ends[v].value() + 4.0 * a4[v].value() + 2.0 * a2[v].value();
        } else {
            for (long i = idx; i < a.m; ++i) {
                Acc ends, a4, a2;
                ends.zero();
                a4.zero();
                a2.zero();
                ends.add(qf[(long)bd.start * a.sm + i], qb[(long)(top - bd.start) * a.sm + i]);
                ends.add(qf[(long)bd.stop * a.sm + i], qb[(long)(top - bd.stop) * a.sm + i]);
                for (int s = bd.start + 1; s <= bd.stop - 1; s += 2)
                    a4.add(qf[(long)s * a.sm + i], qb[(long)(top - s) * a.sm + i]);
                for (int s = bd.start + 2; s <= bd.stop - 2; s += 2)
                    a2.add(qf[(long)s * a.sm + i], qb[(long)(top - s) * a.sm + i]);
                out[i] = ends.value() + 4.0 * a4.value() + 2.0 * a2.value();
            }
        }
    }
}

/* -------------------------------------------------------- fused update */
/* Per grid point: block densities (funDensity normalisation SCFT.c:2299 and
 * funVolFrac SCFT.c:1458-1482), totals (funAddArray SCFT.c:1486-1512), the free
 * energy integrand on pre-update fields (funFreeEnergy SCFT.c:1874-1917), the
 * field update (funUpdate SCFT.c:2044-2117) and the RMS term (SCFT.c:1566-1578).
 *
 * Everything runs over the compacted list of active fields: a field that is not
 * active has no density (its terms in H and in the totals are exact zeros in
 * the reference) and is not updated. The list, the chi sub-table and the block
 * factors sit in shared memory; per-point values stay in registers because all
 * register-array indices are loop counters of fully unrolled loops.
 * Block partials of H, p and (phi_tot-1)^2 go to a.partial. The pass is bound
 * by the FP64 pipe's latency, so it is built for three CTAs per SM with up to
 * four active fields and two otherwise (a few registers spill; measured faster
 * than one or two CTAs without spills). */
template <int NA>
__global__ void __launch_bounds__(POST_THREADS, (NA <= 4 ? 3 : 2)) k_update(PostArgs a)
{
    __shared__ double sh[3 * 32];
    __shared__ double coef[SCFT_MAX_BLOCKS];
    __shared__ double chiA[SCFT_NFIELDS][SCFT_NFIELDS];
    __shared__ double pavgA[SCFT_NFIELDS];
    __shared__ double cA[SCFT_NFIELDS], eA[SCFT_NFIELDS]; /* row sums of chi, of chi . phi_avg */
    __shared__ double s_ctot;                             /* sum over pairs of chi */
    __shared__ int actf[SCFT_NFIELDS], p0[SCFT_NFIELDS], p1[SCFT_NFIELDS];
    __shared__ int s_na;
    const int b = blockIdx.y;
    if (a.state[b].done) return;
    const InstParams &ip = a.params[b];
    const InstState &st = a.state[b];
    const double mf = (st.iter > (unsigned long)ip.relaxation) ? 0.0 : 1.0; /* SCFT.c:1515-1522 */
    if (threadIdx.x < a.nblocks) {
        const BlockDesc bd = a.blocks[b * a.nblocks + threadIdx.x];
        const double ds_eff = 1.0 / (bd.len - 1);
        /* frac * ((raw / 3) * (DS_EFF / Q)) as one factor: the FP64 divisions
         * would otherwise dominate this kernel's FP64 pipe time */
        coef[threadIdx.x] = ip.frac[threadIdx.x] * ((ds_eff / st.q[bd.species]) / 3.0);
    }
    if (threadIdx.x == 0) {
        int n = 0;
        for (int f = 0; f < SCFT_NFIELDS; ++f)
            if (ip.active[f]) {
                actf[n] = f;
                p0[n] = a.part0[f];
                p1[n] = a.part1[f];
                pavgA[n] = ip.phi_avg[f];
                ++n;
            }
        s_na = n;
    }
    __syncthreads();
    /* every instance of a context has NA active fields (checked at creation) */
    constexpr int na = NA;
    for (int e = threadIdx.x; e < na * na; e += blockDim.x) {
        const int i = e / na, j = e - i * na;
        chiA[i][j] = ip.chi[actf[i]][actf[j]];
    }
    __syncthreads();
    if (threadIdx.x < na) {
        const int i = threadIdx.x;
        double c = 0.0, e = 0.0;
        for (int j = 0; j < na; ++j)
            if (j != i) {
                c += chiA[i][j];
                e += chiA[i][j] * pavgA[j];
            }
        cA[i] = c;
        eA[i] = e;
    }
    if (threadIdx.x == 0) {
        double c = 0.0;
        for (int i = 0; i < na; ++i)
            for (int j = i + 1; j < na; ++j) c += chiA[i][j];
        s_ctot = c;
    }
    __syncthreads();
    const double g1 = ip.g1, g2 = ip.g2, g12 = g1 - g2, dt = ip.dt_noise;
    const double inv_na = 1.0 / na;
    const int mask = ip.mask;
    double *w = a.w + (long)b * 14 * a.sm;
    double *phi = a.phi + (long)b * 14 * a.sm;
    const double *raw = a.raw + (long)b * a.nblocks * a.sm;
    const double *noise = a.noise ? a.noise + (long)b * ip.n_active * a.sm : nullptr;
    const bool add_noise = noise && (dt * mf != 0.0);
    double acc[3] = {0.0, 0.0, 0.0};
    for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < a.m; idx += (long)gridDim.x * blockDim.x) {
        double ph[NA], wv[NA], dw[NA];
        double tot = 0.0, sphi = 0.0, wphi = 0.0, hint = 0.0;
        const double pv = w[13 * a.sm + idx];
        bool first_tot = true;
#pragma unroll
        for (int i = 0; i < NA; ++i) {
            const int f = actf[i], b0 = p0[i], b1 = p1[i];
            /* (raw / 3) * (DS_EFF / Q), then * VOL factor, as funDensity and funVolFrac */
            double v = 0.0;
            if (b0 >= 0) v = raw[(long)b0 * a.sm + idx] * coef[b0];
            if (b1 >= 0) {
                const double u = raw[(long)b1 * a.sm + idx] * coef[b1];
                v = (b0 >= 0) ? v + u : u;
            }
            ph[i] = v;
            wv[i] = w[(long)f * a.sm + idx];
            /* phi_tot adds the free-polymer totals A..J and, with MASK, S1..S3 */
            if (f < 10 || mask) {
                tot = first_tot ? v : tot + v;
                first_tot = false;
            }
        }
        /* r = phi - phi_avg over the active fields; t_i = sum_{j != i} chi_ij r_j serves the
         * field force dw_i = -w_i + p + t_i (SCFT.c:2060-2075), the pair energy
         * sum_{i<j} chi_ij phi_i phi_j = 1/2 sum_i phi_i (t_i + e_i) with e_i = sum_{j != i}
         * chi_ij phi_avg_j (SCFT.c:1886-1895), and the correction sum_{f<g} chi_fg sum_{h != f,g}
         * r_h = R C - sum_f r_f c_f with C = sum_{f<g} chi_fg, c_f = sum_{g != f} chi_fg
         * (SCFT.c:2076-2091); G = G1 on the diagonal and G1/6 elsewhere, so the mixing sum is
         * G2 sum_j dw_j + (G1 - G2) dw_i (SCFT.c:2093-2101). Same sums as the reference,
         * grouped to O(n_active^2) per point. */
        double r[NA];
        double rsum = 0.0;
#pragma unroll
        for (int i = 0; i < NA; ++i) {
            wphi += wv[i] * ph[i];
            sphi += ph[i];
            phi[(long)actf[i] * a.sm + idx] = ph[i];
            r[i] = ph[i] - pavgA[i];
            rsum += r[i];
        }
        phi[13 * a.sm + idx] = tot;
        double hpair = 0.0, dsum = 0.0, rc = 0.0;
#pragma unroll
        for (int i = 0; i < NA; ++i) {
            double t = 0.0;
#pragma unroll
            for (int j = 0; j < NA; ++j) {
                if (j != i) t += chiA[i][j] * r[j];
            }
            hpair += ph[i] * (t + eA[i]);
            dw[i] = -wv[i] + pv + t;
            dsum += dw[i];
            rc += r[i] * cA[i];
        }
        hint = 0.5 * hpair - wphi - pv * (1.0 - sphi);
        const double corr = na > 1 ? rsum * s_ctot - rc : 0.0;
        double psum = 0.0;
#pragma unroll
        for (int i = 0; i < NA; ++i) {
            double wn = wv[i] + (g2 * dsum + g12 * dw[i]);
            if (add_noise) wn += dt * mf * noise[(long)i * a.sm + idx];
            w[(long)actf[i] * a.sm + idx] = wn;
            psum += wn;
        }
        const double pn = (psum + corr) * inv_na;
        w[13 * a.sm + idx] = pn;
        acc[0] += hint;
        acc[1] += pn;
        acc[2] += (tot - 1.0) * (tot - 1.0);
    }
    block_sum<3>(acc, sh);
    if (threadIdx.x == 0) {
        double *pp = a.partial + ((long)b * gridDim.x + blockIdx.x) * 3;
        pp[0] = acc[0];
        pp[1] = acc[1];
        pp[2] = acc[2];
    }
}

/* Reduce the update partials of one instance, finish H (ln Q terms,
 * SCFT.c:1528-1555), mu (SCFT.c:1862-1869), RMS and <p>; write the record. */
__global__ void k_finalize(PostArgs a, int nparts)
{
    const int b = blockIdx.x;
    __shared__ double sh[3 * 32];
    InstState &st = a.state[b];
    const long slot = (long)st.tick - 1;
    if (st.done) {
        /* frozen: repeat the converging iteration's record */
        if (threadIdx.x == 0 && slot >= 0 && slot < a.hist_cap) a.hist[slot * a.B + b] = a.last[b];
        return;
    }
    double v[3] = {0.0, 0.0, 0.0};
    /* fixed assignment of partials to threads keeps the order deterministic */
    for (int k = threadIdx.x; k < nparts; k += blockDim.x) {
        const double *pp = a.partial + ((long)b * nparts + k) * 3;
        v[0] += pp[0];
        v[1] += pp[1];
        v[2] += pp[2];
    }
    block_sum<3>(v, sh);
    if (threadIdx.x != 0) return;
    const InstParams &ip = a.params[b];
    const double dvol = (double)a.m;
    double H = v[0] / dvol;
    double frac = 0.0;
    int bad = 0;
    scft_iter_out rec;
    for (int sp = 0; sp < SCFT_NSPECIES; ++sp) {
        const double q = st.q[sp];
        rec.q[sp] = q;
        rec.mu[sp] = 0.0;
        if (!a.species[b * SCFT_NSPECIES + sp].present) continue;
        const double qm = q * q;
        rec.mu[sp] = (qm == 0.0) ? 0.0 : -log(qm) / 2.0;
        frac += ip.lnq_coef[sp] * log(q);
        if (!isfinite(q)) bad = 1;
    }
    H -= frac;
    const double pavg = v[1] / dvol;
    const double rms = sqrt(v[2] / dvol);
    if (!isfinite(H) || !isfinite(rms) || !isfinite(pavg)) bad = 1;
    st.p_avg = pavg;
    if (bad) st.status = SCFT_ERR_NONFINITE; /* keeps an error set earlier in the iteration */
    rec.iter = st.iter;
    rec.free_energy = H;
    rec.rms = rms;
    rec.mf = (st.iter > (unsigned long)ip.relaxation) ? 0.0 : 1.0;
    rec.status = st.status;
    rec.converged = 0;
    if (st.stop_rms > 0.0 && st.status == SCFT_OK && rms < st.stop_rms) {
        st.done = 2; /* frozen from the next iteration on; this one still ends with the p shift */
        rec.converged = 1;
    }
    /* with a stop criterion (batch and serving forms) a non-finite instance is
     * frozen too: its records repeat the failing iteration and it costs nothing
     * until its slot is re-armed; without one (the fixed-ITER drop-in) it keeps
     * iterating as the reference does */
    if (st.stop_rms > 0.0 && st.status != SCFT_OK) st.done = 2;
    a.last[b] = rec;
    if (slot >= 0 && slot < a.hist_cap) a.hist[slot * a.B + b] = rec;
}

/* p -= <p> (SCFT.c:2119-2123). */
__global__ void k_p_shift(PostArgs a)
{
    const int b = blockIdx.y;
    if (a.state[b].done == 1) return;
    const double pavg = a.state[b].p_avg;
    double *p = a.w + ((long)b * 14 + 13) * a.sm;
    for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < a.m; idx += (long)gridDim.x * blockDim.x)
        p[idx] -= pavg;
}

/* ------------------------------------------------------------ launchers */
static int grid_for(long m, int sms)
{
    long g = (m + POST_THREADS - 1) / POST_THREADS;
    long cap = (long)sms * 4;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

cudaError_t scft_post_iter_begin(const PostArgs &a, int prec, int sms, cudaStream_t st)
{
    k_iter_begin<<<(a.B + 127) / 128, 128, 0, st>>>(a);
    dim3 g(grid_for(a.m, sms), a.B);
    if (prec == SCFT_PREC_FP64)
        k_boltz_init<double><<<g, POST_THREADS, 0, st>>>(a);
    else if (prec == SCFT_PREC_FP32X2)
        k_boltz_init<dfloat><<<g, POST_THREADS, 0, st>>>(a);
    else
        k_boltz_init<float><<<g, POST_THREADS, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t scft_post_mark_start(const PostArgs &a, cudaStream_t st)
{
    k_iter_start_mark<<<(a.B + 127) / 128, 128, 0, st>>>(a);
    return cudaGetLastError();
}

int scft_post_nparts(long m, int sms) { return grid_for(m, sms); }

cudaError_t scft_density_launch(const PostArgs &a, int prec, int sms, cudaStream_t st)
{
    const int vw = prec == SCFT_PREC_FP32 ? 4 : 2;
    dim3 gd(grid_for((a.m + vw - 1) / vw, sms), a.nblocks, a.B);
    if (prec == SCFT_PREC_FP64)
        k_density<double><<<gd, POST_THREADS, 0, st>>>(a);
    else if (prec == SCFT_PREC_FP32X2)
        k_density<dfloat><<<gd, POST_THREADS, 0, st>>>(a);
    else
        k_density<float><<<gd, POST_THREADS, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t scft_post_iter_end(const PostArgs &a, int prec, int sms, cudaStream_t st)
{
    const int gp = grid_for(a.m, sms);
    dim3 gq(gp, SCFT_NSPECIES, a.B);
    if (prec == SCFT_PREC_FP64)
        k_q_partial<double><<<gq, POST_THREADS, 0, st>>>(a);
    else if (prec == SCFT_PREC_FP32X2)
        k_q_partial<dfloat><<<gq, POST_THREADS, 0, st>>>(a);
    else
        k_q_partial<float><<<gq, POST_THREADS, 0, st>>>(a);
    k_q_final<<<dim3(SCFT_NSPECIES, a.B), 32, 0, st>>>(a, gp);
    const int vw = prec == SCFT_PREC_FP32 ? 4 : 2;
    dim3 gd(grid_for((a.m + vw - 1) / vw, sms), a.nblocks, a.B);
    if (prec == SCFT_PREC_FP64)
        k_density<double><<<gd, POST_THREADS, 0, st>>>(a);
    else if (prec == SCFT_PREC_FP32X2)
        k_density<dfloat><<<gd, POST_THREADS, 0, st>>>(a);
    else
        k_density<float><<<gd, POST_THREADS, 0, st>>>(a);
    {
        const dim3 gu(gp, a.B);
        switch (a.n_active) {
        case 1: k_update<1><<<gu, POST_THREADS, 0, st>>>(a); break;
        case 2: k_update<2><<<gu, POST_THREADS, 0, st>>>(a); break;
        case 3: k_update<3><<<gu, POST_THREADS, 0, st>>>(a); break;
        case 4: k_update<4><<<gu, POST_THREADS, 0, st>>>(a); break;
        case 5: k_update<5><<<gu, POST_THREADS, 0, st>>>(a); break;
        case 6: k_update<6><<<gu, POST_THREADS, 0, st>>>(a); break;
        case 7: k_update<7><<<gu, POST_THREADS, 0, st>>>(a); break;
        case 8: k_update<8><<<gu, POST_THREADS, 0, st>>>(a); break;
        case 9: k_update<9><<<gu, POST_THREADS, 0, st>>>(a); break;
        case 10: k_update<10><<<gu, POST_THREADS, 0, st>>>(a); break;
        case 11: k_update<11><<<gu, POST_THREADS, 0, st>>>(a); break;
        case 12: k_update<12><<<gu, POST_THREADS, 0, st>>>(a); break;
        case 13: k_update<13><<<gu, POST_THREADS, 0, st>>>(a); break;
        default: return cudaErrorInvalidValue;
        }
    }
    k_finalize<<<a.B, POST_THREADS, 0, st>>>(a, gp);
    k_p_shift<<<dim3(gp, a.B), POST_THREADS, 0, st>>>(a);
    return cudaGetLastError();
}

/* ----------------------------------------------------- unit-entry helpers */
template <typename P>
__global__ void k_d2p(const double *s, P *d, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) d[i] = (P)s[i];
}
template <typename P>
__global__ void k_p2d(const P *s, double *d, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) d[i] = (double)s[i];
}
template <typename P>
__global__ void k_boltz1(const double *w, P *bz, double ds, long m)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < m; i += (long)gridDim.x * blockDim.x)
        bz[i] = boltz<P>(ds, w[i]);
}

/* to_p = 1: double -> P (src double, dst P); to_p = 0: P -> double (src is P). */
cudaError_t scft_convert(int prec, const double *src, void *dst, long n, int to_p, cudaStream_t st)
{
    const int g = (int)((n + 255) / 256 > 4096 ? 4096 : (n + 255) / 256);
    if (prec == SCFT_PREC_FP64) {
        if (to_p)
            k_d2p<double><<<g, 256, 0, st>>>(src, (double *)dst, n);
        else
            k_p2d<double><<<g, 256, 0, st>>>((const double *)src, (double *)dst, n);
    } else if (prec == SCFT_PREC_FP32X2) {
        if (to_p)
            k_d2p<dfloat><<<g, 256, 0, st>>>(src, (dfloat *)dst, n);
        else
            k_p2d<dfloat><<<g, 256, 0, st>>>((const dfloat *)(const void *)src, (double *)dst, n);
    } else {
        if (to_p)
            k_d2p<float><<<g, 256, 0, st>>>(src, (float *)dst, n);
        else
            k_p2d<float><<<g, 256, 0, st>>>((const float *)(const void *)src, (double *)dst, n);
    }
    return cudaGetLastError();
}

cudaError_t scft_boltz_one(int prec, const double *w, void *bz, double ds, long m, cudaStream_t st)
{
    const int g = (int)((m + 255) / 256 > 4096 ? 4096 : (m + 255) / 256);
    if (prec == SCFT_PREC_FP64)
        k_boltz1<double><<<g, 256, 0, st>>>(w, (double *)bz, ds, m);
    else if (prec == SCFT_PREC_FP32X2)
        k_boltz1<dfloat><<<g, 256, 0, st>>>(w, (dfloat *)bz, ds, m);
    else
        k_boltz1<float><<<g, 256, 0, st>>>(w, (float *)bz, ds, m);
    return cudaGetLastError();
}
