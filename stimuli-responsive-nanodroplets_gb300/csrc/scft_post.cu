/*
 * scft_post.cu — everything in one SCFT iteration except the contour steps:
 * Boltzmann factors and initial slices, Q reductions, contour-integrated
 * densities, and the fused free-energy / field-update pass with its
 * reductions. All reductions are FP64 and run in a fixed order, so a result
 * does not depend on which other instances share the launch.
 */
#include <cuda_runtime.h>
#include <math.h>

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
        a.state[b].iter += 1; /* iIter++ (SCFT.c:1090) */
        a.state[b].status = SCFT_OK;
    }
}

__global__ void k_iter_start_mark(PostArgs a)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < a.B) a.state[b].iter0 = a.state[b].iter;
}

/* b = exp(DS * (-w/2)) for the fields chains use (SCFT.c:2344), and the initial
 * slice of every chain: 1, the grafting mask (SCFT.c:2441) or the single-point
 * seed while iIter <= SEED_STEPS (SCFT.c:2346-2367). */
template <typename P>
__global__ void k_boltz_init(PostArgs a)
{
    const int b = blockIdx.y;
    const InstParams &ip = a.params[b];
    const unsigned long iter = a.state[b].iter;
    const bool seed_on = ip.enable_seed && iter <= (unsigned long)ip.seed_steps;
    P *bz = reinterpret_cast<P *>(a.bz) + (long)b * SCFT_NFIELDS * a.sm;
    const double *w = a.w + (long)b * 14 * a.sm;
    for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < a.m; idx += (long)gridDim.x * blockDim.x) {
        for (int f = 0; f < SCFT_NFIELDS; ++f)
            if (a.field_use >> f & 1u) bz[f * a.sm + idx] = (P)exp(ip.ds * (-w[f * a.sm + idx] / 2.0));
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
    const SpeciesDesc sd = a.species[sp];
    if (!sd.present) return;
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
    if (threadIdx.x != 0) return;
    const SpeciesDesc sd = a.species[sp];
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
 * the reference. */
template <typename P>
__global__ void __launch_bounds__(POST_THREADS) k_density(PostArgs a)
{
    const int blk = blockIdx.y, b = blockIdx.z;
    const BlockDesc bd = a.blocks[blk];
    const ChainDesc &cf = a.chains[b * a.nchains + bd.chain_f];
    const ChainDesc &cb = a.chains[b * a.nchains + bd.chain_b];
    const P *qf = reinterpret_cast<const P *>(cf.q);
    const P *qb = reinterpret_cast<const P *>(cb.q);
    double *out = a.raw + ((long)b * a.nblocks + blk) * a.sm;
    const int top = bd.len - 1;
    for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < a.m; idx += (long)gridDim.x * blockDim.x) {
        double acc = (double)qf[(long)bd.start * a.sm + idx] * (double)qb[(long)(top - bd.start) * a.sm + idx] +
                     (double)qf[(long)bd.stop * a.sm + idx] * (double)qb[(long)(top - bd.stop) * a.sm + idx];
        double a4 = 0.0, a2 = 0.0;
        for (int s = bd.start + 1; s <= bd.stop - 1; s += 2)
            a4 += (double)qf[(long)s * a.sm + idx] * (double)qb[(long)(top - s) * a.sm + idx];
        for (int s = bd.start + 2; s <= bd.stop - 2; s += 2)
            a2 += (double)qf[(long)s * a.sm + idx] * (double)qb[(long)(top - s) * a.sm + idx];
        out[idx] = acc + 4.0 * a4 + 2.0 * a2;
    }
}

/* -------------------------------------------------------- fused update */
/* Per grid point: block densities (funDensity normalisation SCFT.c:2299 and
 * funVolFrac SCFT.c:1458-1482), totals (funAddArray SCFT.c:1486-1512), the free
 * energy integrand on pre-update fields (funFreeEnergy SCFT.c:1874-1917), the
 * field update (funUpdate SCFT.c:2044-2117) and the RMS term (SCFT.c:1566-1578).
 * Block partials of H, p and (phi_tot-1)^2 go to a.partial. */
__global__ void __launch_bounds__(POST_THREADS) k_update(PostArgs a)
{
    __shared__ double sh[3 * 32];
    __shared__ double coef[SCFT_MAX_BLOCKS];
    const int b = blockIdx.y;
    const InstParams &ip = a.params[b];
    const InstState &st = a.state[b];
    const double mf = (st.iter > (unsigned long)ip.relaxation) ? 0.0 : 1.0; /* SCFT.c:1515-1522 */
    if (threadIdx.x < a.nblocks) {
        const BlockDesc bd = a.blocks[threadIdx.x];
        const double ds_eff = 1.0 / (bd.len - 1);
        coef[threadIdx.x] = ds_eff / st.q[bd.species];
    }
    __syncthreads();
    double *w = a.w + (long)b * 14 * a.sm;
    double *phi = a.phi + (long)b * 14 * a.sm;
    const double *raw = a.raw + (long)b * a.nblocks * a.sm;
    const double *noise = a.noise ? a.noise + (long)b * ip.n_active * a.sm : nullptr;
    const bool add_noise = noise && (ip.dt_noise * mf != 0.0);
    double acc[3] = {0.0, 0.0, 0.0};
    for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < a.m; idx += (long)gridDim.x * blockDim.x) {
        double part[SCFT_NFIELDS][2];
        int has[SCFT_NFIELDS][2];
#pragma unroll
        for (int f = 0; f < SCFT_NFIELDS; ++f) has[f][0] = has[f][1] = 0;
        for (int k = 0; k < a.nblocks; ++k) {
            const BlockDesc bd = a.blocks[k];
            const double v = ip.frac[k] * ((raw[(long)k * a.sm + idx] / 3.0) * coef[k]);
            part[bd.field][bd.part] = v;
            has[bd.field][bd.part] = 1;
        }
        double ph[SCFT_NFIELDS];
#pragma unroll
        for (int f = 0; f < SCFT_NFIELDS; ++f) {
            if (has[f][0] && has[f][1])
                ph[f] = part[f][0] + part[f][1];
            else if (has[f][0])
                ph[f] = part[f][0];
            else if (has[f][1])
                ph[f] = part[f][1];
            else
                ph[f] = 0.0;
        }
        double tot = ph[0] + ph[1];
#pragma unroll
        for (int f = 2; f < 10; ++f) tot = tot + ph[f];
        if (ip.mask) tot = tot + ph[10] + ph[11] + ph[12];

        double wv[SCFT_NFIELDS];
#pragma unroll
        for (int f = 0; f < SCFT_NFIELDS; ++f) wv[f] = w[f * a.sm + idx];
        const double pv = w[13 * a.sm + idx];

        /* free-energy integrand on the pre-update fields */
        double hint = 0.0, sphi = 0.0, wphi = 0.0;
#pragma unroll
        for (int f = 0; f < SCFT_NFIELDS; ++f) {
#pragma unroll
            for (int g = f + 1; g < SCFT_NFIELDS; ++g) hint += ip.chi[f][g] * ph[f] * ph[g];
            wphi += wv[f] * ph[f];
            sphi += ph[f];
        }
        hint = hint - wphi - pv * (1.0 - sphi);

        /* field update */
        double rmr[SCFT_NFIELDS], dw[SCFT_NFIELDS];
        double rsum = 0.0;
#pragma unroll
        for (int f = 0; f < SCFT_NFIELDS; ++f) {
            rmr[f] = ip.active[f] ? ph[f] - ip.phi_avg[f] : 0.0;
            rsum += rmr[f];
        }
#pragma unroll
        for (int f = 0; f < SCFT_NFIELDS; ++f) {
            double d = -wv[f] + pv;
#pragma unroll
            for (int g = 0; g < SCFT_NFIELDS; ++g)
                if (g != f && ip.active[g]) d += ip.chi[f][g] * rmr[g];
            dw[f] = d;
        }
        /* correction: sum over active pairs f<g of chi_fg * sum_{h != f,g} rmr_h
         * (SCFT.c:2076-2091), written as chi_fg * (R - rmr_f - rmr_g) */
        double corr = 0.0;
        if (ip.n_active > 1) {
#pragma unroll
            for (int f = 0; f < SCFT_NFIELDS; ++f) {
                if (!ip.active[f]) continue;
#pragma unroll
                for (int g = f + 1; g < SCFT_NFIELDS; ++g)
                    if (ip.active[g]) corr += ip.chi[f][g] * (rsum - rmr[f] - rmr[g]);
            }
        }
        double psum = 0.0;
        int an = 0;
#pragma unroll
        for (int f = 0; f < SCFT_NFIELDS; ++f) {
            if (!ip.active[f]) continue;
            double wn = wv[f];
#pragma unroll
            for (int g = 0; g < SCFT_NFIELDS; ++g)
                if (ip.active[g]) wn += (g == f ? ip.g1 : ip.g2) * dw[g];
            if (add_noise) wn += ip.dt_noise * mf * noise[(long)an * a.sm + idx];
            ++an;
            w[f * a.sm + idx] = wn;
            psum += wn;
        }
        const double pn = (psum + corr) / ip.n_active;
        w[13 * a.sm + idx] = pn;
#pragma unroll
        for (int f = 0; f < SCFT_NFIELDS; ++f) phi[f * a.sm + idx] = ph[f];
        phi[13 * a.sm + idx] = tot;
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
    InstState &st = a.state[b];
    const double dvol = (double)a.m;
    double H = v[0] / dvol;
    double frac = 0.0;
    int bad = 0;
    scft_iter_out rec;
    for (int sp = 0; sp < SCFT_NSPECIES; ++sp) {
        const double q = st.q[sp];
        rec.q[sp] = q;
        rec.mu[sp] = 0.0;
        if (!a.species[sp].present) continue;
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
    st.status = bad ? SCFT_ERR_NONFINITE : SCFT_OK;
    rec.iter = st.iter;
    rec.free_energy = H;
    rec.rms = rms;
    rec.mf = (st.iter > (unsigned long)ip.relaxation) ? 0.0 : 1.0;
    rec.status = st.status;
    rec.pad = 0;
    const long slot = (long)(st.iter - st.iter0 - 1);
    if (slot >= 0 && slot < a.hist_cap) a.hist[slot * a.B + b] = rec;
}

/* p -= <p> (SCFT.c:2119-2123). */
__global__ void k_p_shift(PostArgs a)
{
    const int b = blockIdx.y;
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

cudaError_t scft_post_iter_end(const PostArgs &a, int prec, int sms, cudaStream_t st)
{
    const int gp = grid_for(a.m, sms);
    dim3 gq(gp, SCFT_NSPECIES, a.B);
    if (prec == SCFT_PREC_FP64)
        k_q_partial<double><<<gq, POST_THREADS, 0, st>>>(a);
    else
        k_q_partial<float><<<gq, POST_THREADS, 0, st>>>(a);
    k_q_final<<<dim3(SCFT_NSPECIES, a.B), 32, 0, st>>>(a, gp);
    dim3 gd(gp, a.nblocks, a.B);
    if (prec == SCFT_PREC_FP64)
        k_density<double><<<gd, POST_THREADS, 0, st>>>(a);
    else
        k_density<float><<<gd, POST_THREADS, 0, st>>>(a);
    k_update<<<dim3(gp, a.B), POST_THREADS, 0, st>>>(a);
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
        bz[i] = (P)exp(ds * (-w[i] / 2.0));
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
    else
        k_boltz1<float><<<g, 256, 0, st>>>(w, (float *)bz, ds, m);
    return cudaGetLastError();
}
