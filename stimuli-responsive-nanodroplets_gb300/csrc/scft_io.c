/*
 * scft_io.c — the reference's text inputs and outputs, byte for byte, plus the
 * host replay of its noise draws.
 *
 * File formats are an interface that must match SCFT.c exactly, so each
 * writer produces the same characters as the fprintf it replaces (cited per
 * function). Rows of grid files run k outer, j, i inner while the array index
 * is idx = k + NZ*(j + NY*i) (SCFT.c:1612-1620).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "scft_gpu.h"

/* ---------------------------------------------------------- file names */
void scft_file_names_default(scft_file_names *n)
{
    if (!n) return;
    memset(n, 0, sizeof(*n));
    strcpy(n->counter, "counter.dat");
    strcpy(n->density, "densities_dbk_");
    strcpy(n->deviations, "deviations.dat");
    strcpy(n->energy, "energies.dat");
    strcpy(n->restart_fields, "restart_fields.dat");
    strcpy(n->restart_random, "restart_random.dat");
    strcpy(n->run_params, "run.txt");
    strcpy(n->w_mask, "wMask.dat");
    strcpy(n->free_energy, "free_energy.dat");
}

static scft_file_names g_names;
static int g_names_set;

static const scft_file_names *names(void)
{
    if (!g_names_set) {
        scft_file_names_default(&g_names);
        g_names_set = 1;
    }
    return &g_names;
}

int scft_set_file_names(const scft_file_names *n)
{
    if (!n) {
        scft_file_names_default(&g_names);
        g_names_set = 1;
        return SCFT_OK;
    }
    const char *all[9] = {n->counter, n->density, n->deviations, n->energy, n->restart_fields,
                          n->restart_random, n->run_params, n->w_mask, n->free_energy};
    for (int i = 0; i < 9; ++i)
        if (!all[i][0] || memchr(all[i], 0, SCFT_NAME_MAX) == NULL) return SCFT_ERR_PARAM;
    g_names = *n;
    g_names_set = 1;
    return SCFT_OK;
}

static FILE *open_in(const char *dir, const char *name, const char *mode)
{
    char path[4096];
    if (dir && dir[0])
        snprintf(path, sizeof(path), "%s/%s", dir, name);
    else
        snprintf(path, sizeof(path), "%s", name);
    return fopen(path, mode);
}

/* ------------------------------------------------------------- readers */
int scft_read_counter(const char *dir, unsigned long *iter)
{
    FILE *f = open_in(dir, names()->counter, "r");
    if (!f) return SCFT_ERR_IO;
    int ok = fscanf(f, "%lu", iter) == 1;
    fclose(f);
    return ok ? SCFT_OK : SCFT_ERR_IO;
}

int scft_read_restart_fields(const char *dir, const scft_derived *d, double *w14)
{
    FILE *f = open_in(dir, names()->restart_fields, "r");
    if (!f) return SCFT_ERR_IO;
    const long M = d->m;
    int bad = 0;
    for (int k = 0; k < d->nz; ++k)
        for (int j = 0; j < d->ny; ++j)
            for (int i = 0; i < d->nx; ++i) {
                const long idx = k + (long)d->nz * (j + (long)d->ny * i);
                for (int c = 0; c < 14; ++c)
                    if (fscanf(f, "%lf", &w14[c * M + idx]) != 1) bad = 1;
            }
    fclose(f);
    return bad ? SCFT_ERR_IO : SCFT_OK;
}

int scft_read_restart_random(const char *dir, unsigned short seed[3])
{
    FILE *f = open_in(dir, names()->restart_random, "r");
    if (!f) return SCFT_ERR_IO;
    int ok = fscanf(f, "%hu %hu %hu", &seed[0], &seed[1], &seed[2]) == 3;
    fclose(f);
    return ok ? SCFT_OK : SCFT_ERR_IO;
}

int scft_read_mask(const char *dir, const scft_derived *d, double *mask3)
{
    FILE *f = open_in(dir, names()->w_mask, "r");
    if (!f) return SCFT_ERR_IO;
    const long M = d->m;
    int bad = 0;
    for (int k = 0; k < d->nz; ++k)
        for (int j = 0; j < d->ny; ++j)
            for (int i = 0; i < d->nx; ++i) {
                const long idx = k + (long)d->nz * (j + (long)d->ny * i);
                if (fscanf(f, "%lf %lf %lf", &mask3[idx], &mask3[M + idx], &mask3[2 * M + idx]) != 3) bad = 1;
            }
    fclose(f);
    return bad ? SCFT_ERR_IO : SCFT_OK;
}

/* ------------------------------------------------------------- writers */
int scft_write_volume_error(const char *dir, double volume_sum)
{
    FILE *f = open_in(dir, "DENSITY_CHECK_FAIL.error", "w"); /* SCFT.c:92-96 */
    if (!f) return SCFT_ERR_IO;
    fprintf(f, "%lf", volume_sum);
    fclose(f);
    return SCFT_OK;
}

static const char *const FNAME[SCFT_NFIELDS] = {"A", "B", "C", "D", "E", "F", "G", "H", "I", "J", "S1", "S2", "S3"};

int scft_write_run_params(const char *dir, const scft_surface *s, const scft_derived *d, unsigned long iter)
{
    /* run.txt, appended at launch (SCFT.c:1025-1085). */
    FILE *f = open_in(dir, names()->run_params, "a");
    if (!f) return SCFT_ERR_IO;
    const double (*X)[SCFT_NFIELDS] = (const double (*)[SCFT_NFIELDS])d->chi_eff;
    fprintf(f, "-----------------------------------------\n\n");
    fprintf(f, "These are the run parameter values: \n\n");
    fprintf(f, "Iteration  = %ld \n", (long)iter);
    fprintf(f, "NX, NY, NZ  = %d, %d, %d \n", d->nx, d->ny, d->nz);
    fprintf(f, "NS  = %d \n\n", s->ns);
    for (int b = 0; b < 4; ++b)
        fprintf(f, "DBK_%d:: NS_DBK_%d, NS_DBK_%d_X, NS_DBK_%d_Y, LEN_DBK_%d, F_INPUT_DBK_%d, VOL_DBK_%d  = %d, %d, %d, %f, %f, %f \n",
                b + 1, b + 1, b + 1, b + 1, b + 1, b + 1, b + 1, d->ns_dbk[b], d->ns_dbk_x[b], d->ns_dbk_y[b], s->len_dbk[b],
                s->f_dbk[b], s->vol_dbk[b]);
    for (int h = 0; h < 10; ++h)
        fprintf(f, "HOMOPOLYMER %s:: NS_HOMO_%s, HOMOPOLYMER_LEN_%s, VOL_HOMOPOLYMER_%s  = %d, %f, %f \n%s", FNAME[h], FNAME[h],
                FNAME[h], FNAME[h], d->ns_homo[h], s->len_homo[h], s->vol_homo[h], h == 9 ? "\n" : "");
    const double g2 = s->g1 / 6.0;
    fprintf(f, "G1 = %f", s->g1);
    for (int g = 2; g <= 13; ++g) fprintf(f, ", G%d = %f", g, g2);
    fprintf(f, " \n\n");
    for (int k = 0; k < SCFT_NFIELDS; ++k)
        fprintf(f, "%sphi_%s_avg = %lf", k ? ", " : "", FNAME[k], d->phi_avg[k]);
    fprintf(f, " \n\n");
    for (int a = 0; a < 9; ++a) {
        fprintf(f, "Chi*N %ss", FNAME[a]);
        for (int b = a + 1; b < 10; ++b) fprintf(f, "%s %s%s = %f", b == a + 1 ? "," : ",", FNAME[a], FNAME[b], X[a][b]);
        fprintf(f, " \n%s", a == 8 ? "\n" : "");
    }
    fprintf(f, "Substrate settings: \n");
    fprintf(f, "MASK = %d, vol S[1+2+3]: %f \n", s->mask, d->coating_vol);
    for (int k = 0; k < 3; ++k)
        fprintf(f, "S%d: NS_S%d, LEN_S%d, VOL_S%d  = %d, %f, %f \n%s", k + 1, k + 1, k + 1, k + 1, d->ns_s[k], s->len_s[k],
                s->vol_s[k], k == 2 ? "\n" : "");
    fprintf(f, "CHI_N_S1_S2_EFF = %f, CHI_N_S1_S3_EFF = %f, CHI_N_S2_S3_EFF = %f \n", X[10][11], X[10][12], X[11][12]);
    for (int a = 0; a < 10; ++a)
        fprintf(f, "CHI_N_S1_%s_EFF = %f, CHI_N_S2_%s_EFF = %f, CHI_N_S3_%s_EFF = %f \n%s", FNAME[a], X[10][a], FNAME[a],
                X[11][a], FNAME[a], X[12][a], a == 9 ? "\n" : "");
    fprintf(f, "DS  = %f \n", d->ds);
    fprintf(f, "LX, LY, LZ  = %f, %f, %f \n", s->lx, s->ly, s->lz);
    fprintf(f, "DX, DY, DZ  = %f, %f, %f \n\n", d->dx, d->dy, d->dz);
    fprintf(f, "-----------------------------------------\n\n");
    fclose(f);
    return SCFT_OK;
}

int scft_write_energies(const char *dir, const scft_derived *d, const scft_iter_out *o)
{
    /* SCFT.c:1585-1598: one line each in energies.dat, free_energy.dat and
     * deviations.dat (the last also echoes chi_AB, chi_AC, chi_BC EFF). */
    FILE *f = open_in(dir, names()->energy, "a");
    if (!f) return SCFT_ERR_IO;
    fprintf(f, "%lu", o->iter);
    for (int sp = 0; sp < SCFT_NSPECIES; ++sp) fprintf(f, " %lf", o->mu[sp]);
    fprintf(f, "\n");
    fclose(f);
    f = open_in(dir, names()->free_energy, "a");
    if (!f) return SCFT_ERR_IO;
    fprintf(f, "%lu  %lf  %f \n", o->iter, o->free_energy, (double)(float)o->mf);
    fclose(f);
    f = open_in(dir, names()->deviations, "a");
    if (!f) return SCFT_ERR_IO;
    fprintf(f, "%lu  %lf %lf %lf %lf \n", o->iter, o->rms, d->chi_eff[0][1], d->chi_eff[0][2], d->chi_eff[1][2]);
    fclose(f);
    return SCFT_OK;
}

int scft_write_snapshot(const char *dir, const scft_derived *d, unsigned long iter, const double *phi13,
                        const double *w14, const unsigned short seed[3])
{
    const long M = d->m;
    char name[SCFT_NAME_MAX + 32];
    /* densities_dbk_<100000000 + iIter>.dat (SCFT.c:1603-1610). */
    snprintf(name, sizeof(name), "%s%d.dat", names()->density, (int)(100000000 + iter));
    FILE *f = open_in(dir, name, "w");
    if (!f) return SCFT_ERR_IO;
    for (int k = 0; k < d->nz; ++k)
        for (int j = 0; j < d->ny; ++j)
            for (int i = 0; i < d->nx; ++i) {
                const long idx = k + (long)d->nz * (j + (long)d->ny * i);
                fprintf(f, "%5d %5d %5d", i, j, k);
                for (int c = 0; c < SCFT_NFIELDS; ++c) fprintf(f, " %10.6lf", phi13[c * M + idx]);
                for (int c = 0; c < 14; ++c) fprintf(f, " %12.6lf", w14[c * M + idx]);
                fprintf(f, " \n");
            }
    fclose(f);

    f = open_in(dir, names()->counter, "w"); /* SCFT.c:1631-1634 */
    if (!f) return SCFT_ERR_IO;
    fprintf(f, "%lu", iter);
    fclose(f);

    f = open_in(dir, names()->restart_fields, "w"); /* SCFT.c:1636-1650 */
    if (!f) return SCFT_ERR_IO;
    for (int k = 0; k < d->nz; ++k)
        for (int j = 0; j < d->ny; ++j)
            for (int i = 0; i < d->nx; ++i) {
                const long idx = k + (long)d->nz * (j + (long)d->ny * i);
                for (int c = 0; c < 14; ++c) fprintf(f, c ? " %lf" : "%lf", w14[c * M + idx]);
                fprintf(f, " \n");
            }
    fclose(f);

    if (seed) {
        f = open_in(dir, names()->restart_random, "w"); /* SCFT.c:1652-1663 */
        if (!f) return SCFT_ERR_IO;
        fprintf(f, "%hu %hu %hu", seed[0], seed[1], seed[2]);
        fclose(f);
    }
    return SCFT_OK;
}

/* --------------------------------------------------------------- noise */
/* The POSIX 48-bit generator drand48 uses after seed48: x <- (a*x + c) mod 2^48
 * with a = 0x5DEECE66D, c = 0xB, returning x / 2^48. Written out here so the
 * state is explicit and independent of libc's hidden global. */
static double lcg48_next(unsigned short st[3])
{
    unsigned long long x = ((unsigned long long)st[2] << 32) | ((unsigned long long)st[1] << 16) | st[0];
    x = (0x5DEECE66DULL * x + 0xBULL) & 0xFFFFFFFFFFFFULL;
    st[0] = (unsigned short)(x & 0xFFFF);
    st[1] = (unsigned short)((x >> 16) & 0xFFFF);
    st[2] = (unsigned short)((x >> 32) & 0xFFFF);
    return ldexp((double)x, -48);
}

/* Marsaglia's polar method, as funGaussDev (SCFT.c:1769-1782) applies it. */
static double polar_gauss(unsigned short st[3])
{
    double x1, x2, w;
    do {
        x1 = 2.0 * lcg48_next(st) - 1.0;
        x2 = 2.0 * lcg48_next(st) - 1.0;
        w = x1 * x1 + x2 * x2;
    } while (w >= 1.0);
    w = sqrt((-2.0 * log(w)) / w);
    return x1 * w;
}

int scft_noise_fill(unsigned short state[3], const scft_derived *d, double *out)
{
    if (!state || !d) return SCFT_ERR_PARAM;
    const long M = d->m;
    for (int k = 0; k < d->nz; ++k)
        for (int j = 0; j < d->ny; ++j)
            for (int i = 0; i < d->nx; ++i) {
                const long idx = k + (long)d->nz * (j + (long)d->ny * i);
                int a = 0;
                for (int f = 0; f < SCFT_NFIELDS; ++f) {
                    if (!d->active[f]) continue;
                    const double g = polar_gauss(state);
                    if (out) out[a * M + idx] = g;
                    ++a;
                }
            }
    return SCFT_OK;
}
