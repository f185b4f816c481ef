/*
 * scft_derive.c — the quantities SCFT.c's main() derives from parameters.h
 * before its loop, computed from a runtime scft_surface.
 *
 * Expression order follows the reference so the derived doubles are the same
 * bits: DS = 1/(NS-1) (parameters.h:20), ALPHA = (NS_x - 1) * DS
 * (SCFT.c:131, :151, ...), ALPHAX = DS/(DX*DX) with DX = LX/NX
 * (parameters.h:173-179).
 */
#include <math.h>
#include <string.h>

#include "scft_gpu.h"

static int grid_points(double len, double dr)
{
    /* SCFT.c:103-105: a length of exactly 1.0 collapses to one point. */
    if (len == 1.0) return 1;
    return (int)((len / dr) + 0.5);
}

/* Diblock contour counts, SCFT.c:121-172: total forced odd, the X block
 * (floor(f*NS_DBK)+1) forced odd, Y takes the rest. */
static void diblock_counts(double len, double f, int ns, int *tot, int *x, int *y)
{
    int n = (int)floor(len * ns);
    if (n % 2 == 0) n = n - 1;
    int nx = (int)floor(f * n) + 1;
    if (nx % 2 == 0) nx = nx - 1;
    *tot = n;
    *x = nx;
    *y = n - nx;
}

int scft_derive(const scft_surface *s, scft_derived *d)
{
    if (!s || !d) return SCFT_ERR_PARAM;
    memset(d, 0, sizeof(*d));
    const double eps = 0.000001;

    /* Volume check, SCFT.c:84-101 (brush volumes are not part of the sum). */
    double vc = s->vol_dbk[0] + s->vol_dbk[1] + s->vol_dbk[2] + s->vol_dbk[3];
    for (int h = 0; h < 10; ++h) vc = vc + s->vol_homo[h];
    d->volume_sum = vc;
    d->volume_ok = fabs(1.0 - vc) < eps;

    if (s->ns < 3 || s->dr_target <= 0.0) return SCFT_ERR_PARAM;

    d->nx = grid_points(s->lx, s->dr_target);
    d->ny = grid_points(s->ly, s->dr_target);
    d->nz = grid_points(s->lz, s->dr_target);
    if (d->nx < 1 || d->ny < 1 || d->nz < 1) return SCFT_ERR_PARAM;
    d->m = (long)d->nx * d->ny * d->nz;
    d->n_ext = s->mask ? 2 * (d->nz + 1) : d->nz;

    const double DS = 1.0 / (s->ns - 1);
    d->ds = DS;
    d->dx = s->lx / d->nx;
    d->dy = s->ly / d->ny;
    d->dz = s->lz / d->nz;
    d->alphax = DS / (d->dx * d->dx);
    d->alphay = DS / (d->dy * d->dy);
    d->alphaz = DS / (d->dz * d->dz);

    for (int b = 0; b < 4; ++b) {
        if (s->vol_dbk[b] > 0.0) {
            diblock_counts(s->len_dbk[b], s->f_dbk[b], s->ns, &d->ns_dbk[b], &d->ns_dbk_x[b], &d->ns_dbk_y[b]);
            d->alpha_dbk[b] = (double)((d->ns_dbk[b] - 1) * DS);
        }
    }
    /* Homopolymers, SCFT.c:174-272: decremented when even or longer than NS,
     * so LEN > 1 can leave an even count. */
    for (int h = 0; h < 10; ++h) {
        if (s->vol_homo[h] > 0.0) {
            int n = (int)floor(s->len_homo[h] * s->ns);
            if (n % 2 == 0 || n > s->ns) n = n - 1;
            d->ns_homo[h] = n;
            d->alpha_homo[h] = (double)((n - 1) * DS);
        }
    }
    /* Brushes exist only with MASK (SCFT.c:274-288). */
    if (s->mask) {
        for (int k = 0; k < 3; ++k) {
            if (s->vol_s[k] > 0.0) {
                int n = (int)floor(s->len_s[k] * s->ns);
                if (n % 2 == 0) n = n - 1;
                d->ns_s[k] = n;
                d->alpha_s[k] = (double)((n - 1) * DS);
            }
        }
    }

    /* Average densities, SCFT.c:290-300. */
    const double *V = s->vol_dbk, *F = s->f_dbk, *H = s->vol_homo;
    d->phi_avg[0] = H[0] + F[0] * V[0];
    d->phi_avg[1] = H[1] + (1.0 - F[0]) * V[0];
    d->phi_avg[2] = H[2];
    d->phi_avg[3] = H[3] + F[1] * V[1];
    d->phi_avg[4] = H[4] + (1.0 - F[1]) * V[1];
    d->phi_avg[5] = H[5] + F[2] * V[2];
    d->phi_avg[6] = H[6] + (1.0 - F[2]) * V[2];
    d->phi_avg[7] = H[7] + F[3] * V[3];
    d->phi_avg[8] = H[8] + (1.0 - F[3]) * V[3];
    d->phi_avg[9] = H[9];

    /* chi_EFF: the symmetric table with every pair of an absent species zeroed
     * (SCFT.c:107-119, :302-396). */
    for (int f = 0; f < SCFT_NFIELDS; ++f)
        for (int g = 0; g < SCFT_NFIELDS; ++g) d->chi_eff[f][g] = (f == g) ? 0.0 : s->chi_n[f][g];
    int zero[SCFT_NFIELDS] = {0};
    for (int f = 0; f < 10; ++f)
        if (fabs(d->phi_avg[f]) <= eps) zero[f] = 1;
    if (s->mask) {
        for (int k = 0; k < 3; ++k) {
            if (fabs(s->vol_s[k]) <= eps)
                zero[10 + k] = 1;
            else
                d->phi_avg[10 + k] = s->vol_s[k];
        }
    } else {
        for (int k = 0; k < 3; ++k) {
            d->phi_avg[10 + k] = 0.0;
            zero[10 + k] = 1;
        }
    }
    for (int f = 0; f < SCFT_NFIELDS; ++f) {
        if (!zero[f]) continue;
        for (int g = 0; g < SCFT_NFIELDS; ++g) {
            d->chi_eff[f][g] = 0.0;
            d->chi_eff[g][f] = 0.0;
        }
    }

    /* Coating rescale of the free-polymer averages, SCFT.c:718-733. */
    if (s->mask) {
        d->coating_vol = s->vol_s[0] + s->vol_s[1] + s->vol_s[2];
        for (int f = 0; f < 10; ++f) d->phi_avg[f] = d->phi_avg[f] * (1.0 - d->coating_vol);
    }

    /* Active set of funUpdate, SCFT.c:2002-2042: a homopolymer or brush volume
     * above zero, or the diblock owning the field. Brush volumes count even
     * with MASK 0. */
    for (int h = 0; h < 10; ++h) d->active[h] = s->vol_homo[h] > 0.0;
    for (int k = 0; k < 3; ++k) d->active[10 + k] = s->vol_s[k] > 0.0;
    for (int b = 0; b < 4; ++b)
        if (s->vol_dbk[b] > 0.0) {
            const int fx = (b == 0) ? 0 : 2 * b + 1; /* dbk1: A/B, dbk2: D/E, dbk3: F/G, dbk4: H/I */
            d->active[fx] = 1;
            d->active[fx + 1] = 1;
        }
    d->n_active = 0;
    for (int f = 0; f < SCFT_NFIELDS; ++f) d->n_active += d->active[f];

    return d->volume_ok ? SCFT_OK : SCFT_ERR_VOLUME;
}
