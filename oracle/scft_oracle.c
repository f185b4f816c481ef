/*
 * scft_oracle.c — CPU restatement of the reference solver's hot path.
 *
 * TEST INFRASTRUCTURE. This is the checker for the GPU library and the CPU
 * baseline that bench.py times; the product never links or calls it. It
 * restates SCFT.c with runtime parameters instead of parameters.h macros and
 * keeps the reference's algorithm and data layout: AoS propagators
 * q[s + NS_EFF*idx], complex 3D FFTs through the FFTW3 API (here the project
 * shim in fftw_shim/), the odd extension of length 2(NZ+1) for Dirichlet z,
 * the same Simpson index sets, the same update loops and the same draw order
 * of the drand48 noise. Each function cites the SCFT.c lines it follows.
 *
 * Parity is pinned against the reference itself: tests/golden holds outputs
 * of SCFT.c built from its own source (oracle/build.py) on seeded inputs,
 * and the oracle must reproduce them.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3.h"

#define NF 13
#define NSPEC 17

/* Same memory layout as the library's scft_surface (a test checks sizeof). */
typedef struct orc_surface {
    double lx, ly, lz;
    long iter, d_wrt, relaxation, d_wrt_energies;
    double dt_noise;
    int mask, enable_seed, seed_steps, seed_area_delta, ns, pad0;
    double dr_target, g1;
    double chi_n[NF][NF];
    double f_dbk[4], len_dbk[4], vol_dbk[4];
    double vol_homo[10], len_homo[10];
    double vol_s[3], len_s[3];
} orc_surface;

typedef struct {
    int present;
    int len;                 /* NS_EFF */
    int nsx, nsy;            /* diblock block split */
    int fx, fy;              /* field of each block (fy unused for one-block species) */
    double vol;              /* VOL of the species */
    double alpha;            /* ALPHA (contour length) */
    double *q, *qmod, *qmult;
    double *phix, *phiy;
    double Q, mu;
} orc_species;

typedef struct orc {
    orc_surface S;
    int NX, NY, NZ, N;       /* N = 2(NZ+1) with MASK */
    long M;
    double DS, ALPHAX, ALPHAY, ALPHAZ;
    double phi_avg[NF];
    double chi[NF][NF];      /* chi_EFF table (getCHI_N_EFF, SCFT.c:1928-1951) */
    double coating;
    int active[NF], nactive;
    orc_species sp[NSPEC];
    double *w[NF], *p;
    double *phi_tot_f[NF];   /* aPhi_A_Tot .. aPhi_J_Tot, aPhi_S1..S3 */
    double *phi_total;
    double *mask[3];
    double *exparg;
    fftw_complex *indata, *outdata, *expfield, *ext_in, *ext_out;
    fftw_plan fwd, bwd;
    unsigned long iter;
    unsigned short rng[3];
    double H, rms;
    float MF;
    int NS_EFF;
} orc;

/* ----------------------------------------------------------- set-up */
static int npoints(double L, double dr) { return L == 1.0 ? 1 : (int)((L / dr) + 0.5); } /* SCFT.c:103-105 */

static void setup_species(orc *o)
{
    const orc_surface *S = &o->S;
    const int NS = S->ns;
    const double DS = o->DS;
    memset(o->sp, 0, sizeof(o->sp));
    for (int d = 0; d < 4; ++d) { /* SCFT.c:121-172 */
        orc_species *x = &o->sp[d];
        if (!(S->vol_dbk[d] > 0.0)) continue;
        int n = (int)floor(S->len_dbk[d] * NS);
        if (n % 2 == 0) n -= 1;
        int a = (int)floor(S->f_dbk[d] * n) + 1;
        if (a % 2 == 0) a -= 1;
        x->present = 1;
        x->len = n;
        x->nsx = a;
        x->nsy = n - a;
        x->fx = d == 0 ? 0 : 2 * d + 1;
        x->fy = x->fx + 1;
        x->vol = S->vol_dbk[d];
        x->alpha = (double)((n - 1) * DS);
    }
    for (int h = 0; h < 10; ++h) { /* SCFT.c:174-272 */
        orc_species *x = &o->sp[4 + h];
        if (!(S->vol_homo[h] > 0.0)) continue;
        int n = (int)floor(S->len_homo[h] * NS);
        if (n % 2 == 0 || n > NS) n -= 1;
        x->present = 1;
        x->len = n;
        x->fx = h;
        x->vol = S->vol_homo[h];
        x->alpha = (double)((n - 1) * DS);
    }
    if (S->mask)
        for (int k = 0; k < 3; ++k) { /* SCFT.c:274-288 */
            orc_species *x = &o->sp[14 + k];
            if (!(S->vol_s[k] > 0.0)) continue;
            int n = (int)floor(S->len_s[k] * NS);
            if (n % 2 == 0) n -= 1;
            x->present = 1;
            x->len = n;
            x->fx = 10 + k;
            x->vol = S->vol_s[k];
            x->alpha = (double)((n - 1) * DS);
        }
}

static void setup_chi(orc *o)
{
    const orc_surface *S = &o->S;
    const double eps = 0.000001;
    const double *V = S->vol_dbk, *F = S->f_dbk, *H = S->vol_homo;
    /* SCFT.c:290-300 */
    double pa[NF] = {H[0] + F[0] * V[0], H[1] + (1.0 - F[0]) * V[0], H[2], H[3] + F[1] * V[1],
                     H[4] + (1.0 - F[1]) * V[1], H[5] + F[2] * V[2], H[6] + (1.0 - F[2]) * V[2],
                     H[7] + F[3] * V[3], H[8] + (1.0 - F[3]) * V[3], H[9], 0.0, 0.0, 0.0};
    for (int f = 0; f < NF; ++f)
        for (int g = 0; g < NF; ++g) o->chi[f][g] = f == g ? 0.0 : S->chi_n[f][g];
    int off[NF] = {0};
    for (int f = 0; f < 10; ++f) off[f] = fabs(pa[f]) <= eps; /* SCFT.c:302-351 */
    for (int k = 0; k < 3; ++k) {                             /* SCFT.c:352-396 */
        if (S->mask && !(fabs(S->vol_s[k]) <= eps))
            pa[10 + k] = S->vol_s[k];
        else
            off[10 + k] = 1;
    }
    for (int f = 0; f < NF; ++f)
        if (off[f])
            for (int g = 0; g < NF; ++g) o->chi[f][g] = o->chi[g][f] = 0.0;
    o->coating = 0.0;
    if (S->mask) { /* SCFT.c:718-733 */
        o->coating = S->vol_s[0] + S->vol_s[1] + S->vol_s[2];
        for (int f = 0; f < 10; ++f) pa[f] = pa[f] * (1.0 - o->coating);
    }
    memcpy(o->phi_avg, pa, sizeof(pa));
    /* funUpdate's active set, SCFT.c:2002-2042 */
    for (int f = 0; f < 10; ++f) o->active[f] = S->vol_homo[f] > 0.0;
    for (int k = 0; k < 3; ++k) o->active[10 + k] = S->vol_s[k] > 0.0;
    for (int d = 0; d < 4; ++d)
        if (S->vol_dbk[d] > 0.0) o->active[o->sp[d].fx] = o->active[o->sp[d].fy] = 1;
    o->nactive = 0;
    for (int f = 0; f < NF; ++f) o->nactive += o->active[f];
}

static void setup_exparg(orc *o)
{
    /* SCFT.c:983-1023: one table over the FFT box (NZ or N in z). */
    const int NZB = o->S.mask ? o->N : o->NZ;
    for (int k = 0; k < NZB; ++k)
        for (int j = 0; j < o->NY; ++j)
            for (int i = 0; i < o->NX; ++i) {
                const size_t idx = k + (size_t)NZB * (j + (size_t)o->NY * i);
                const double kx = 2.0 * M_PI * (o->NX / 2.0 - fabs(i - o->NX / 2.0)) / o->NX;
                const double ky = 2.0 * M_PI * (o->NY / 2.0 - fabs(j - o->NY / 2.0)) / o->NY;
                const double kz = 2.0 * M_PI * (NZB / 2.0 - fabs(k - NZB / 2.0)) / NZB;
                o->exparg[idx] = exp(-o->ALPHAX * pow(kx, 2) - o->ALPHAY * pow(ky, 2) - o->ALPHAZ * pow(kz, 2));
            }
}

orc *orc_create(const orc_surface *S)
{
    orc *o = calloc(1, sizeof(orc));
    o->S = *S;
    o->NX = npoints(S->lx, S->dr_target);
    o->NY = npoints(S->ly, S->dr_target);
    o->NZ = npoints(S->lz, S->dr_target);
    o->M = (long)o->NX * o->NY * o->NZ;
    o->N = S->mask ? 2 * (o->NZ + 1) : o->NZ;
    o->DS = 1.0 / (S->ns - 1);
    const double DX = S->lx / o->NX, DY = S->ly / o->NY, DZ = S->lz / o->NZ; /* parameters.h:173-179 */
    o->ALPHAX = o->DS / (DX * DX);
    o->ALPHAY = o->DS / (DY * DY);
    o->ALPHAZ = o->DS / (DZ * DZ);
    setup_species(o);
    setup_chi(o);
    const long M = o->M;
    for (int f = 0; f < NF; ++f) {
        o->w[f] = calloc(M, sizeof(double));
        o->phi_tot_f[f] = calloc(M, sizeof(double));
    }
    o->p = calloc(M, sizeof(double));
    o->phi_total = calloc(M, sizeof(double));
    for (int k = 0; k < 3; ++k) o->mask[k] = calloc(M, sizeof(double));
    for (int s = 0; s < NSPEC; ++s) {
        orc_species *x = &o->sp[s];
        if (!x->present) continue;
        x->q = calloc((size_t)M * x->len, sizeof(double));
        x->qmod = calloc((size_t)M * x->len, sizeof(double));
        x->qmult = calloc((size_t)M * x->len, sizeof(double));
        x->phix = calloc(M, sizeof(double));
        x->phiy = calloc(M, sizeof(double));
        for (long idx = 0; idx < M; ++idx) { /* q[0] = 1, SCFT.c:882-981 */
            x->q[x->len * idx] = 1.0;
            x->qmod[x->len * idx] = 1.0;
        }
    }
    const long MB = (long)o->NX * o->NY * o->N;
    o->indata = fftw_malloc(sizeof(fftw_complex) * M);
    o->outdata = fftw_malloc(sizeof(fftw_complex) * MB);
    o->expfield = fftw_malloc(sizeof(fftw_complex) * M);
    o->ext_in = fftw_malloc(sizeof(fftw_complex) * MB);
    o->ext_out = fftw_malloc(sizeof(fftw_complex) * MB);
    o->exparg = calloc(MB, sizeof(double));
    o->fwd = fftw_plan_dft_3d(o->NX, o->NY, o->N, o->ext_in, o->ext_out, FFTW_FORWARD, FFTW_MEASURE);
    o->bwd = fftw_plan_dft_3d(o->NX, o->NY, o->N, o->ext_in, o->ext_out, FFTW_BACKWARD, FFTW_MEASURE);
    setup_exparg(o);
    return o;
}

void orc_destroy(orc *o)
{
    if (!o) return;
    for (int f = 0; f < NF; ++f) {
        free(o->w[f]);
        free(o->phi_tot_f[f]);
    }
    free(o->p);
    free(o->phi_total);
    for (int k = 0; k < 3; ++k) free(o->mask[k]);
    for (int s = 0; s < NSPEC; ++s) {
        free(o->sp[s].q);
        free(o->sp[s].qmod);
        free(o->sp[s].qmult);
        free(o->sp[s].phix);
        free(o->sp[s].phiy);
    }
    fftw_free(o->indata);
    fftw_free(o->outdata);
    fftw_free(o->expfield);
    fftw_free(o->ext_in);
    fftw_free(o->ext_out);
    free(o->exparg);
    fftw_destroy_plan(o->fwd);
    fftw_destroy_plan(o->bwd);
    free(o);
}

/* ----------------------------------------------------- state access */
long orc_m(const orc *o) { return o->M; }
void orc_grid(const orc *o, int *g) { g[0] = o->NX; g[1] = o->NY; g[2] = o->NZ; }
int orc_nactive(const orc *o) { return o->nactive; }

void orc_set_fields(orc *o, const double *w14)
{
    for (int f = 0; f < NF; ++f) memcpy(o->w[f], w14 + f * o->M, sizeof(double) * o->M);
    memcpy(o->p, w14 + 13 * o->M, sizeof(double) * o->M);
}
void orc_get_fields(const orc *o, double *w14)
{
    for (int f = 0; f < NF; ++f) memcpy(w14 + f * o->M, o->w[f], sizeof(double) * o->M);
    memcpy(w14 + 13 * o->M, o->p, sizeof(double) * o->M);
}
void orc_set_masks(orc *o, const double *m3)
{
    for (int k = 0; k < 3; ++k) memcpy(o->mask[k], m3 + k * o->M, sizeof(double) * o->M);
}
void orc_set_iter(orc *o, unsigned long it) { o->iter = it; }
void orc_set_rng(orc *o, const unsigned short s[3]) { memcpy(o->rng, s, sizeof(o->rng)); }
void orc_get_rng(const orc *o, unsigned short s[3]) { memcpy(s, o->rng, sizeof(o->rng)); }
void orc_get_densities(const orc *o, double *phi13, double *tot)
{
    for (int f = 0; f < NF; ++f) memcpy(phi13 + f * o->M, o->phi_tot_f[f], sizeof(double) * o->M);
    if (tot) memcpy(tot, o->phi_total, sizeof(double) * o->M);
}
/* derived scalars for cross-checks: [DS, ALPHAX, ALPHAY, ALPHAZ, coating, phi_avg[13], chi[169]] */
void orc_derived(const orc *o, int *ints, double *dbls)
{
    /* ints: NX NY NZ N nactive active[13] then per species (len nsx nsy) */
    int k = 0;
    ints[k++] = o->NX;
    ints[k++] = o->NY;
    ints[k++] = o->NZ;
    ints[k++] = o->N;
    ints[k++] = o->nactive;
    for (int f = 0; f < NF; ++f) ints[k++] = o->active[f];
    for (int s = 0; s < NSPEC; ++s) {
        ints[k++] = o->sp[s].len;
        ints[k++] = o->sp[s].nsx;
        ints[k++] = o->sp[s].nsy;
    }
    k = 0;
    dbls[k++] = o->DS;
    dbls[k++] = o->ALPHAX;
    dbls[k++] = o->ALPHAY;
    dbls[k++] = o->ALPHAZ;
    dbls[k++] = o->coating;
    for (int f = 0; f < NF; ++f) dbls[k++] = o->phi_avg[f];
    for (int f = 0; f < NF; ++f)
        for (int g = 0; g < NF; ++g) dbls[k++] = o->chi[f][g];
    for (int s = 0; s < NSPEC; ++s) dbls[k++] = o->sp[s].alpha;
}

/* ----------------------------------------------------- propagation */
/* funPDESolver_periodic, SCFT.c:2474-2525 */
static void step_periodic(orc *o)
{
    const long M = o->M;
    for (long idx = 0; idx < M; ++idx) o->indata[idx] = o->indata[idx] * o->expfield[idx];
    fftw_execute_dft(o->fwd, o->indata, o->outdata);
    for (long idx = 0; idx < M; ++idx) o->indata[idx] = o->outdata[idx] * o->exparg[idx];
    fftw_execute_dft(o->bwd, o->indata, o->outdata);
    for (long idx = 0; idx < M; ++idx) o->indata[idx] = o->outdata[idx] * o->expfield[idx];
}

/* funPDESolver_DirichletBC, SCFT.c:2527-2631: odd extension of length N. */
static void step_dirichlet(orc *o)
{
    const int NX = o->NX, NY = o->NY, NZ = o->NZ, N = o->N;
    for (int i = 0; i < NX; ++i)
        for (int j = 0; j < NY; ++j) {
            fftw_complex *e = o->ext_in + (size_t)N * (j + (size_t)NY * i);
            const size_t base = (size_t)NZ * (j + (size_t)NY * i);
            e[0] = 0.0;
            for (int k = 0; k < NZ; ++k) e[k + 1] = o->indata[base + k] * o->expfield[base + k];
            e[NZ + 1] = 0.0;
            for (int k = NZ + 2; k < N; ++k) e[k] = -o->indata[base + (N - 1 - k)] * o->expfield[base + (N - 1 - k)];
        }
    const long MB = (long)NX * NY * N;
    fftw_execute_dft(o->fwd, o->ext_in, o->ext_out);
    for (long idx = 0; idx < MB; ++idx) o->ext_in[idx] = o->ext_out[idx] * o->exparg[idx];
    fftw_execute_dft(o->bwd, o->ext_in, o->ext_out);
    for (int i = 0; i < NX; ++i)
        for (int j = 0; j < NY; ++j) {
            const fftw_complex *e = o->ext_out + (size_t)N * (j + (size_t)NY * i);
            const size_t base = (size_t)NZ * (j + (size_t)NY * i);
            for (int k = 0; k < NZ; ++k) o->indata[base + k] = e[k + 1] * o->expfield[base + k];
        }
}

/* The contour loop of funPDESolver (SCFT.c:2310-2412) and funPDESolverBrush
 * (SCFT.c:2414-2472). init: 0 use q[start]; 1 dbk1 seed rule; 2 mask. */
static void pde(orc *o, int start, int stop, double *qr, const double *w, int init, const double *mask)
{
    const int NX = o->NX, NY = o->NY, NZ = o->NZ, NS = o->NS_EFF;
    const int dirichlet = o->S.mask || init == 2;
    const double dvol = dirichlet ? (double)(NX * NY * o->N) : (double)(NX * NY * NZ);
    const int D = o->S.seed_area_delta;
    for (int k = 0; k < NZ; ++k)
        for (int j = 0; j < NY; ++j)
            for (int i = 0; i < NX; ++i) {
                const size_t idx = k + (size_t)NZ * (j + (size_t)NY * i);
                o->expfield[idx] = cexp(o->DS * (-w[idx] / 2.0) * (1 + 0 * I));
                if (init == 2) {
                    qr[start + NS * idx] = mask[idx];
                } else if (init == 1 && o->iter <= (unsigned long)o->S.seed_steps) {
                    const int in = i > (NX / 2 - D) && i < (NX / 2 + D) && j > (NY / 2 - D) && j < (NY / 2 + D) &&
                                   k > (NZ / 4 - D) && k < (NZ / 4 + D);
                    qr[start + NS * idx] = in ? 1.0 : 0.0;
                } else if (init == 1) {
                    qr[start + NS * idx] = 1.0;
                }
                o->indata[idx] = qr[start + NS * idx] + 0 * I;
            }
    for (int s = start; s < stop; ++s) {
        if (dirichlet)
            step_dirichlet(o);
        else
            step_periodic(o);
        for (long idx = 0; idx < o->M; ++idx) {
            o->indata[idx] = o->indata[idx] / dvol;
            qr[(s + 1) + NS * idx] = creal(o->indata[idx]);
        }
    }
}

/* Unit entry: steps of one block from q0 in w, seedless (funPDESolver). */
void orc_propagate(orc *o, const double *q0, const double *w, int steps, double *qout /* [steps+1][M] */)
{
    const long M = o->M;
    double *qr = calloc((size_t)M * (steps + 1), sizeof(double));
    o->NS_EFF = steps + 1;
    for (long idx = 0; idx < M; ++idx) qr[(steps + 1) * idx] = q0[idx];
    pde(o, 0, steps, qr, w, 0, NULL);
    for (int s = 0; s <= steps; ++s)
        for (long idx = 0; idx < M; ++idx) qout[s * M + idx] = qr[s + (steps + 1) * idx];
    free(qr);
}

/* funChemPotential, SCFT.c:1837-1872 */
static void chem(orc *o, orc_species *x, const double *qr)
{
    const int NS = o->NS_EFF;
    double sum = 0.0;
    for (int k = 0; k < o->NZ; ++k)
        for (int j = 0; j < o->NY; ++j)
            for (int i = 0; i < o->NX; ++i) sum = sum + qr[(NS - 1) + NS * (k + (size_t)o->NZ * (j + (size_t)o->NY * i))];
    const double dvol = o->NX * o->NY * o->NZ;
    sum = sum / dvol;
    const double qm = pow(sum, 2);
    x->Q = sum;
    x->mu = qm == 0 ? 0.0 : -log(qm) / 2.0;
}

/* funMultiplyQs, SCFT.c:2243-2268 */
static void multiply(orc *o, const double *a, const double *b, double *out)
{
    const int NS = o->NS_EFF;
    for (long idx = 0; idx < o->M; ++idx)
        for (int s = 0; s < NS; ++s) out[s + NS * idx] = a[s + NS * idx] * b[(NS - 1 - s) + NS * idx];
}

/* funDensity, SCFT.c:2270-2308 */
static void density(orc *o, int start, int stop, double *phir, const double *qc, double Q)
{
    const int NS = o->NS_EFF;
    const double ds_eff = 1.0 / (NS - 1);
    for (long idx = 0; idx < o->M; ++idx) {
        double phi = qc[start + NS * idx] + qc[stop + NS * idx];
        for (int s = start + 1; s <= stop - 1; s += 2) phi = phi + 4.0 * qc[s + NS * idx];
        for (int s = start + 2; s <= stop - 2; s += 2) phi = phi + 2.0 * qc[s + NS * idx];
        phi = phi / 3.0;
        phir[idx] = phi * (ds_eff / Q);
    }
}

/* funMultiplyQs then funDensity for one block of a chain of len slices given
 * contour-major ([len][M]) as the unit entry points take them (SCFT.c:2243-2308) */
void orc_density(orc *o, const double *qf, const double *qb, int len, int start, int stop, double Q, double *phi)
{
    const long M = o->M;
    double *a = malloc(sizeof(double) * M * len), *b = malloc(sizeof(double) * M * len);
    double *qc = malloc(sizeof(double) * M * len);
    for (int s = 0; s < len; ++s)
        for (long idx = 0; idx < M; ++idx) {
            a[s + (long)len * idx] = qf[(long)s * M + idx];
            b[s + (long)len * idx] = qb[(long)s * M + idx];
        }
    o->NS_EFF = len;
    multiply(o, a, b, qc);
    density(o, start, stop, phi, qc, Q);
    free(a);
    free(b);
    free(qc);
}

static double polar_gauss(unsigned short st[3]) /* funGaussDev, SCFT.c:1769-1782 */
{
    double x1, x2, w;
    do {
        x1 = 2.0 * erand48(st) - 1.0;
        x2 = 2.0 * erand48(st) - 1.0;
        w = x1 * x1 + x2 * x2;
    } while (w >= 1.0);
    w = sqrt((-2.0 * log(w)) / w);
    return x1 * w;
}

/* funFreeEnergy, SCFT.c:1874-1917 (pair order f<g is the reference's term order) */
static double free_energy(orc *o)
{
    double H = 0.0;
    double *phi[NF];
    for (int f = 0; f < NF; ++f) phi[f] = o->phi_tot_f[f];
    for (int k = 0; k < o->NZ; ++k)
        for (int j = 0; j < o->NY; ++j)
            for (int i = 0; i < o->NX; ++i) {
                const size_t idx = k + (size_t)o->NZ * (j + (size_t)o->NY * i);
                double h = 0.0;
                int first = 1;
                for (int f = 0; f < NF; ++f)
                    for (int g = f + 1; g < NF; ++g) {
                        const double t = o->chi[f][g] * phi[f][idx] * phi[g][idx];
                        h = first ? t : h + t;
                        first = 0;
                    }
                for (int f = 0; f < NF; ++f) h = h - o->w[f][idx] * phi[f][idx];
                double r = 1;
                for (int f = 0; f < NF; ++f) r = r - phi[f][idx];
                h = h - o->p[idx] * r;
                H = H + h;
            }
    return H / (double)(o->NX * o->NY * o->NZ);
}

/* funUpdate, SCFT.c:1993-2124 */
static void update(orc *o, double dt)
{
    const double G1 = o->S.g1, G2 = o->S.g1 / 6.0;
    double pavg = 0.0;
    double wi[NF], rmr[NF], dw[NF];
    for (int k = 0; k < o->NZ; ++k)
        for (int j = 0; j < o->NY; ++j)
            for (int i = 0; i < o->NX; ++i) {
                const size_t idx = k + (size_t)o->NZ * (j + (size_t)o->NY * i);
                for (int f = 0; f < NF; ++f)
                    if (o->active[f]) {
                        wi[f] = o->w[f][idx];
                        rmr[f] = o->phi_tot_f[f][idx] - o->phi_avg[f];
                    }
                for (int f = 0; f < NF; ++f) {
                    if (!o->active[f]) continue;
                    dw[f] = -wi[f] + o->p[idx];
                    for (int g = 0; g < NF; ++g)
                        if (o->active[g] && f != g) dw[f] += o->chi[f][g] * rmr[g];
                }
                double corr = 0.0;
                if (o->nactive > 1)
                    for (int f = 0; f < NF; ++f) {
                        if (!o->active[f]) continue;
                        for (int g = f + 1; g < NF; ++g) {
                            if (!o->active[g]) continue;
                            for (int h = 0; h < NF; ++h)
                                if (o->active[h] && h != f && h != g) corr += o->chi[f][g] * rmr[h];
                        }
                    }
                double psum = 0.0;
                for (int f = 0; f < NF; ++f) {
                    if (!o->active[f]) continue;
                    o->w[f][idx] = wi[f];
                    for (int g = 0; g < NF; ++g)
                        if (o->active[g]) o->w[f][idx] += (f == g ? G1 : G2) * dw[g];
                    o->w[f][idx] += dt * o->MF * polar_gauss(o->rng);
                    psum += o->w[f][idx];
                }
                o->p[idx] = (psum + corr) / o->nactive;
                pavg += o->p[idx];
            }
    pavg /= (double)(o->NX * o->NY * o->NZ);
    for (long idx = 0; idx < o->M; ++idx) o->p[idx] -= pavg;
}

static void add_arrays(orc *o, const double *a, const double *b, double *sum) /* funAddArray, SCFT.c:1805-1835 */
{
    if (!a && !b) return;
    for (long idx = 0; idx < o->M; ++idx) {
        if (!a)
            sum[idx] = b[idx];
        else if (!b)
            sum[idx] = a[idx];
        else
            sum[idx] = (1 * a[idx]) + (1 * b[idx]);
    }
}

static void vol_frac(orc *o, double frac, double *arr) /* funVolFrac, SCFT.c:1784-1803 */
{
    if (!(frac > 0.0) || !arr) return;
    for (long idx = 0; idx < o->M; ++idx) arr[idx] = frac * arr[idx];
}

/* One iteration, SCFT.c:1090-1580. rec: iter, H, rms, MF, mu[17], Q[17]. */
static void iterate_once(orc *o, double *rec)
{
    o->iter++;
    for (int h = 0; h < 10; ++h) { /* SCFT.c:1092-1240 */
        orc_species *x = &o->sp[4 + h];
        if (!x->present) continue;
        o->NS_EFF = x->len;
        pde(o, 0, x->len - 1, x->q, o->w[h], 0, NULL);
        chem(o, x, x->q);
        multiply(o, x->q, x->q, x->qmult);
        density(o, 0, x->len - 1, x->phix, x->qmult, x->Q);
    }
    for (int d = 0; d < 4; ++d) { /* SCFT.c:1242-1410 */
        orc_species *x = &o->sp[d];
        if (!x->present) continue;
        o->NS_EFF = x->len;
        pde(o, 0, x->nsx - 1, x->q, o->w[x->fx], (d == 0 && o->S.enable_seed == 1) ? 1 : 0, NULL);
        pde(o, x->nsx - 1, x->len - 1, x->q, o->w[x->fy], 0, NULL);
        pde(o, 0, x->nsy, x->qmod, o->w[x->fy], 0, NULL);
        pde(o, x->nsy, x->len - 1, x->qmod, o->w[x->fx], 0, NULL);
        chem(o, x, d < 2 ? x->qmod : x->q);
        multiply(o, x->q, x->qmod, x->qmult);
        density(o, 0, x->nsx - 1, x->phix, x->qmult, x->Q);
        density(o, x->nsx - 1, x->len - 1, x->phiy, x->qmult, x->Q);
    }
    for (int k = 0; k < 3; ++k) { /* SCFT.c:1412-1456 */
        orc_species *x = &o->sp[14 + k];
        if (!x->present) continue;
        o->NS_EFF = x->len;
        pde(o, 0, x->len - 1, x->q, o->w[10 + k], 2, o->mask[k]);
        pde(o, 0, x->len - 1, x->qmod, o->w[10 + k], 0, NULL);
        chem(o, x, x->q);
        multiply(o, x->q, x->qmod, x->qmult);
        density(o, 0, x->len - 1, x->phix, x->qmult, x->Q);
    }
    const double coat = o->coating;
    for (int d = 0; d < 4; ++d)
        if (o->sp[d].present) {
            vol_frac(o, o->S.vol_dbk[d] * (1.0 - coat), o->sp[d].phix);
            vol_frac(o, o->S.vol_dbk[d] * (1.0 - coat), o->sp[d].phiy);
        }
    for (int h = 0; h < 10; ++h)
        if (o->sp[4 + h].present) vol_frac(o, o->S.vol_homo[h] * (1.0 - coat), o->sp[4 + h].phix);
    if (o->S.mask)
        for (int k = 0; k < 3; ++k)
            if (o->sp[14 + k].present) vol_frac(o, o->S.vol_s[k], o->sp[14 + k].phix);
    /* totals, SCFT.c:1486-1512 */
    const double *dbk_part[10] = {0};
    for (int d = 0; d < 4; ++d)
        if (o->sp[d].present) {
            dbk_part[o->sp[d].fx] = o->sp[d].phix;
            dbk_part[o->sp[d].fy] = o->sp[d].phiy;
        }
    for (int f = 0; f < 10; ++f)
        add_arrays(o, dbk_part[f], o->sp[4 + f].present ? o->sp[4 + f].phix : NULL, o->phi_tot_f[f]);
    for (int k = 0; k < 3; ++k)
        if (o->sp[14 + k].present) memcpy(o->phi_tot_f[10 + k], o->sp[14 + k].phix, sizeof(double) * o->M);
    add_arrays(o, o->phi_tot_f[0], o->phi_tot_f[1], o->phi_total);
    for (int f = 2; f < 10; ++f) add_arrays(o, o->phi_total, o->phi_tot_f[f], o->phi_total);
    if (o->S.mask)
        for (int k = 0; k < 3; ++k) add_arrays(o, o->phi_total, o->phi_tot_f[10 + k], o->phi_total);
    o->MF = o->iter > (unsigned long)o->S.relaxation ? 0.0f : 1.0f; /* SCFT.c:1515-1522 */
    double H = free_energy(o);
    double frac = 0.0; /* SCFT.c:1528-1553 */
    for (int d = 0; d < 4; ++d)
        if (o->S.vol_dbk[d] > 0.0) frac += (o->S.vol_dbk[d] / o->sp[d].alpha * (1.0 - coat)) * log(o->sp[d].Q);
    for (int h = 0; h < 10; ++h)
        if (o->S.vol_homo[h] > 0.0) frac += (o->S.vol_homo[h] / o->sp[4 + h].alpha * (1.0 - coat)) * log(o->sp[4 + h].Q);
    if (o->S.mask)
        for (int k = 0; k < 3; ++k)
            if (o->S.vol_s[k] > 0.0) frac += o->S.vol_s[k] / o->sp[14 + k].alpha * log(o->sp[14 + k].Q);
    H -= frac;
    update(o, o->S.dt_noise);
    double r = 0.0; /* SCFT.c:1564-1580 */
    for (int k = 0; k < o->NZ; ++k)
        for (int j = 0; j < o->NY; ++j)
            for (int i = 0; i < o->NX; ++i) r = r + pow((o->phi_total[k + (size_t)o->NZ * (j + (size_t)o->NY * i)] - 1.0), 2);
    o->rms = pow((r / (o->NX * o->NY * o->NZ)), 0.5);
    o->H = H;
    if (rec) {
        rec[0] = (double)o->iter;
        rec[1] = H;
        rec[2] = o->rms;
        rec[3] = o->MF;
        for (int s = 0; s < NSPEC; ++s) {
            rec[4 + s] = o->sp[s].present ? o->sp[s].mu : 0.0;
            rec[4 + NSPEC + s] = o->sp[s].present ? o->sp[s].Q : 0.0;
        }
    }
}

/* Run n iterations; rec (if not NULL) receives 4 + 2*17 doubles per iteration. */
int orc_iterate(orc *o, int n, double *rec)
{
    for (int k = 0; k < n; ++k) iterate_once(o, rec ? rec + (size_t)k * (4 + 2 * NSPEC) : NULL);
    return 0;
}

size_t orc_surface_size(void) { return sizeof(orc_surface); }
