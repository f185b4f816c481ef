/*
 * scft_main.c — drop-in replacement for SCFT.c's main() (SCFT.c:82-1764).
 *
 * Compile against the run's parameters.h exactly as SCFT.c is:
 *     gcc -O2 -I<dir with parameters.h> -I<repo>/include scft_main.c \
 *         -L<pkg> -lscft_gb300 -Wl,-rpath,<pkg> -lm -o scft_gb300
 * (stimuli-responsive-nanodroplets_gb300/build.py:build_host does this). Run it
 * in the run directory: it reads counter.dat, restart_fields.dat,
 * restart_random.dat and wMask.dat, and writes run.txt, energies.dat,
 * free_energy.dat, deviations.dat, densities_dbk_*.dat, counter.dat,
 * restart_fields.dat and restart_random.dat with the reference's formats and
 * cadence. The hot path runs on the GPU through the C ABI of scft_gpu.h.
 *
 * The FP64 plain form is the default; SCFT_GB300_PRECISION=fp32 selects the
 * FP32-propagator form. The drand48 noise stream is replayed on the device;
 * SCFT_GB300_NOISE=host draws it on the host instead (same numbers). The
 * file-name macros of parameters.h (COUNTER, DENSITY, DEVIATIONS, ENERGY,
 * RESTART_FIELDS, RESTART_RANDOM, RUN_PARAMS, W_MASK, FREE_ENERGY;
 * parameters.h:181-190) name the files as they do for SCFT.c; a header without
 * them gets the reference's names.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "parameters.h"
#include "scft_gpu.h"

#ifndef COUNTER
#define COUNTER "counter.dat"
#endif
#ifndef DENSITY
#define DENSITY "densities_dbk_"
#endif
#ifndef DEVIATIONS
#define DEVIATIONS "deviations.dat"
#endif
#ifndef ENERGY
#define ENERGY "energies.dat"
#endif
#ifndef RESTART_FIELDS
#define RESTART_FIELDS "restart_fields.dat"
#endif
#ifndef RESTART_RANDOM
#define RESTART_RANDOM "restart_random.dat"
#endif
#ifndef RUN_PARAMS
#define RUN_PARAMS "run.txt"
#endif
#ifndef W_MASK
#define W_MASK "wMask.dat"
#endif
#ifndef FREE_ENERGY
#define FREE_ENERGY "free_energy.dat"
#endif

/* the run's file names as SCFT.c compiles them in (parameters.h:181-190) */
static void set_names(void)
{
    scft_file_names n;
    memset(&n, 0, sizeof(n));
    snprintf(n.counter, sizeof(n.counter), "%s", COUNTER);
    snprintf(n.density, sizeof(n.density), "%s", DENSITY);
    snprintf(n.deviations, sizeof(n.deviations), "%s", DEVIATIONS);
    snprintf(n.energy, sizeof(n.energy), "%s", ENERGY);
    snprintf(n.restart_fields, sizeof(n.restart_fields), "%s", RESTART_FIELDS);
    snprintf(n.restart_random, sizeof(n.restart_random), "%s", RESTART_RANDOM);
    snprintf(n.run_params, sizeof(n.run_params), "%s", RUN_PARAMS);
    snprintf(n.w_mask, sizeof(n.w_mask), "%s", W_MASK);
    snprintf(n.free_energy, sizeof(n.free_energy), "%s", FREE_ENERGY);
    if (scft_set_file_names(&n) != SCFT_OK) {
        fprintf(stderr, "invalid file names in parameters.h\n");
        exit(EXIT_FAILURE);
    }
}

#define CHI(f, g, v)                  \
    do {                              \
        s->chi_n[f][g] = (double)(v); \
        s->chi_n[g][f] = (double)(v); \
    } while (0)

/* parameters.h macros -> scft_surface (field order A..J = 0..9, S1..S3 = 10..12) */
static void surface_from_macros(scft_surface *s)
{
    memset(s, 0, sizeof(*s));
    s->lx = LX;
    s->ly = LY;
    s->lz = LZ;
    s->iter = ITER;
    s->d_wrt = D_WRT;
    s->relaxation = RELAXATION;
    s->d_wrt_energies = D_WRT_ENERGIES;
    s->dt_noise = DT_NOISE;
    s->mask = MASK;
    s->enable_seed = ENABLE_SEED;
    s->seed_steps = SEED_STEPS;
    s->seed_area_delta = SEED_AREA_DELTA;
    s->ns = NS;
    s->dr_target = DR_TARGET;
    s->g1 = G1;
    CHI(0, 1, CHI_N_AB); CHI(0, 2, CHI_N_AC); CHI(0, 3, CHI_N_AD); CHI(0, 4, CHI_N_AE); CHI(0, 5, CHI_N_AF);
    CHI(0, 6, CHI_N_AG); CHI(0, 7, CHI_N_AH); CHI(0, 8, CHI_N_AI); CHI(0, 9, CHI_N_AJ);
    CHI(1, 2, CHI_N_BC); CHI(1, 3, CHI_N_BD); CHI(1, 4, CHI_N_BE); CHI(1, 5, CHI_N_BF); CHI(1, 6, CHI_N_BG);
    CHI(1, 7, CHI_N_BH); CHI(1, 8, CHI_N_BI); CHI(1, 9, CHI_N_BJ);
    CHI(2, 3, CHI_N_CD); CHI(2, 4, CHI_N_CE); CHI(2, 5, CHI_N_CF); CHI(2, 6, CHI_N_CG); CHI(2, 7, CHI_N_CH);
    CHI(2, 8, CHI_N_CI); CHI(2, 9, CHI_N_CJ);
    CHI(3, 4, CHI_N_DE); CHI(3, 5, CHI_N_DF); CHI(3, 6, CHI_N_DG); CHI(3, 7, CHI_N_DH); CHI(3, 8, CHI_N_DI);
    CHI(3, 9, CHI_N_DJ);
    CHI(4, 5, CHI_N_EF); CHI(4, 6, CHI_N_EG); CHI(4, 7, CHI_N_EH); CHI(4, 8, CHI_N_EI); CHI(4, 9, CHI_N_EJ);
    CHI(5, 6, CHI_N_FG); CHI(5, 7, CHI_N_FH); CHI(5, 8, CHI_N_FI); CHI(5, 9, CHI_N_FJ);
    CHI(6, 7, CHI_N_GH); CHI(6, 8, CHI_N_GI); CHI(6, 9, CHI_N_GJ);
    CHI(7, 8, CHI_N_HI); CHI(7, 9, CHI_N_HJ);
    CHI(8, 9, CHI_N_IJ);
    CHI(10, 11, CHI_N_S1_S2); CHI(10, 12, CHI_N_S1_S3); CHI(11, 12, CHI_N_S2_S3);
    CHI(10, 0, CHI_N_S1_A); CHI(10, 1, CHI_N_S1_B); CHI(10, 2, CHI_N_S1_C); CHI(10, 3, CHI_N_S1_D);
    CHI(10, 4, CHI_N_S1_E); CHI(10, 5, CHI_N_S1_F); CHI(10, 6, CHI_N_S1_G); CHI(10, 7, CHI_N_S1_H);
    CHI(10, 8, CHI_N_S1_I); CHI(10, 9, CHI_N_S1_J);
    CHI(11, 0, CHI_N_S2_A); CHI(11, 1, CHI_N_S2_B); CHI(11, 2, CHI_N_S2_C); CHI(11, 3, CHI_N_S2_D);
    CHI(11, 4, CHI_N_S2_E); CHI(11, 5, CHI_N_S2_F); CHI(11, 6, CHI_N_S2_G); CHI(11, 7, CHI_N_S2_H);
    CHI(11, 8, CHI_N_S2_I); CHI(11, 9, CHI_N_S2_J);
    CHI(12, 0, CHI_N_S3_A); CHI(12, 1, CHI_N_S3_B); CHI(12, 2, CHI_N_S3_C); CHI(12, 3, CHI_N_S3_D);
    CHI(12, 4, CHI_N_S3_E); CHI(12, 5, CHI_N_S3_F); CHI(12, 6, CHI_N_S3_G); CHI(12, 7, CHI_N_S3_H);
    CHI(12, 8, CHI_N_S3_I); CHI(12, 9, CHI_N_S3_J);
    const double f[4] = {F_INPUT_DBK_1, F_INPUT_DBK_2, F_INPUT_DBK_3, F_INPUT_DBK_4};
    const double ld[4] = {LEN_DBK_1, LEN_DBK_2, LEN_DBK_3, LEN_DBK_4};
    const double vd[4] = {VOL_DBK_1, VOL_DBK_2, VOL_DBK_3, VOL_DBK_4};
    const double vh[10] = {VOL_HOMOPOLYMER_A, VOL_HOMOPOLYMER_B, VOL_HOMOPOLYMER_C, VOL_HOMOPOLYMER_D,
                           VOL_HOMOPOLYMER_E, VOL_HOMOPOLYMER_F, VOL_HOMOPOLYMER_G, VOL_HOMOPOLYMER_H,
                           VOL_HOMOPOLYMER_I, VOL_HOMOPOLYMER_J};
    const double lh[10] = {LEN_HOMO_A, LEN_HOMO_B, LEN_HOMO_C, LEN_HOMO_D, LEN_HOMO_E,
                           LEN_HOMO_F, LEN_HOMO_G, LEN_HOMO_H, LEN_HOMO_I, LEN_HOMO_J};
    const double vs[3] = {VOL_S1, VOL_S2, VOL_S3};
    const double ls[3] = {LEN_S1, LEN_S2, LEN_S3};
    memcpy(s->f_dbk, f, sizeof(f));
    memcpy(s->len_dbk, ld, sizeof(ld));
    memcpy(s->vol_dbk, vd, sizeof(vd));
    memcpy(s->vol_homo, vh, sizeof(vh));
    memcpy(s->len_homo, lh, sizeof(lh));
    memcpy(s->vol_s, vs, sizeof(vs));
    memcpy(s->len_s, ls, sizeof(ls));
}

static void die(const char *what)
{
    perror(what);
    exit(EXIT_FAILURE);
}

static void check(int rc, const char *what)
{
    if (rc != SCFT_OK) {
        fprintf(stderr, "%s failed (%d): %s\n", what, rc, scft_last_error());
        exit(EXIT_FAILURE);
    }
}

int main(void)
{
    set_names();
    scft_surface S;
    surface_from_macros(&S);
    scft_derived d;
    const int drc = scft_derive(&S, &d);
    if (drc == SCFT_ERR_VOLUME) { /* SCFT.c:92-101 */
        scft_write_volume_error(NULL, d.volume_sum);
        printf("                      <=============================\n");
        printf("Volumes do not sum up to 1.0, check the input parameters\n");
        printf("!!!!!!!!!!!!!!!!!!!!!!!!!!!\n");
        return 0;
    }
    check(drc, "scft_derive");
    const long M = d.m;
    unsigned long iter = 0;
    if (scft_read_counter(NULL, &iter) != SCFT_OK) die("Error opening counter file");
    double *mask3 = calloc((size_t)3 * M, sizeof(double));
    double *w14 = calloc((size_t)14 * M, sizeof(double));
    double *phi13 = calloc((size_t)13 * M, sizeof(double));
    double *noise = malloc(sizeof(double) * (size_t)(d.n_active > 0 ? d.n_active : 1) * M);
    if (!mask3 || !w14 || !phi13 || !noise) die("Error allocating host buffers");
    if (S.mask && scft_read_mask(NULL, &d, mask3) != SCFT_OK) die("Error opening the w field mask file");
    unsigned short seed[3];
    if (iter == 0) { /* fresh start: zero fields, clock-seeded drand48 (SCFT.c:785-797) */
        struct timespec ts;
        clock_gettime(CLOCK_REALTIME, &ts);
        const long t = ts.tv_nsec;
        seed[0] = (unsigned short)t;
        seed[1] = (unsigned short)(t + 1);
        seed[2] = (unsigned short)(t + 2);
        printf("iSeed new = %hu, %hu, %hu\n\n", seed[0], seed[1], seed[2]);
    } else {
        if (scft_read_restart_fields(NULL, &d, w14) != SCFT_OK) die("Error opening restart fields file");
        if (scft_read_restart_random(NULL, seed) != SCFT_OK) die("Error opening restart random file");
    }
    check(scft_write_run_params(NULL, &S, &d, iter), "scft_write_run_params");

    scft_options opt;
    scft_options_default(&opt);
    const char *prec = getenv("SCFT_GB300_PRECISION");
    if (prec && strcmp(prec, "fp32") == 0) opt.precision = SCFT_PREC_FP32;
    if (prec && strcmp(prec, "fp32x2") == 0) opt.precision = SCFT_PREC_FP32X2;
    const char *nm = getenv("SCFT_GB300_NOISE");
    const int host_noise = nm && strcmp(nm, "host") == 0;
    opt.noise_mode = host_noise ? SCFT_NOISE_HOST : SCFT_NOISE_DRAND48;
    scft_ctx *ctx = NULL;
    check(scft_ctx_create(&S, &opt, &ctx), "scft_ctx_create");
    check(scft_set_fields(ctx, 0, w14), "scft_set_fields");
    if (S.mask) check(scft_set_masks(ctx, 0, mask3), "scft_set_masks");
    check(scft_set_iteration(ctx, 0, iter), "scft_set_iteration");
    if (!host_noise) check(scft_set_rng(ctx, 0, seed), "scft_set_rng");

    /* restart_random.dat carries the state saved at the previous snapshot, as
     * the reference's seed48 sequence leaves it (SCFT.c:1653-1662) */
    unsigned short saved[3] = {seed[0], seed[1], seed[2]};
    enum { CHUNK = 256 };
    scft_iter_out *recs = malloc(sizeof(scft_iter_out) * CHUNK);
    scft_iter_out *done_recs = malloc(sizeof(scft_iter_out) * CHUNK);
    if (!recs || !done_recs) die("Error allocating host buffers");
    /* Output of a finished chunk (its energies lines and, at a snapshot, the
     * snapshot files) is written while the next chunk runs on the GPU; the
     * files and their order are those of the synchronous loop. */
    int done_n = 0, done_snap = 0;
    unsigned long done_first = 0, done_iter = 0;
    unsigned short done_saved[3] = {0, 0, 0};
    while (iter <= (unsigned long)S.iter || done_n > 0 || done_snap) {
        int n = 0;
        if (iter <= (unsigned long)S.iter) { /* SCFT.c:1088: iterations iter+1 .. ITER+1 */
            /* run up to the next snapshot (or CHUNK iterations) in one call */
            unsigned long last = iter + 1;
            while (last < (unsigned long)S.iter + 1 && last - iter < CHUNK &&
                   !(fmod((double)last, (double)S.d_wrt) == 0 || last == 1))
                ++last;
            n = (int)(last - iter);
            if (host_noise) {
                n = 1;
                const unsigned long it = iter + 1;
                const double mf = it > (unsigned long)S.relaxation ? 0.0 : 1.0;
                const int need = mf * S.dt_noise != 0.0;
                /* the reference draws its noise every iteration, used or not */
                scft_noise_fill(seed, &d, need ? noise : NULL);
                check(scft_iterate(ctx, 1, need ? noise : NULL, recs), "scft_iterate");
            } else {
                check(scft_iterate_async(ctx, n), "scft_iterate_async");
            }
        }
        /* the previous chunk's output, overlapping the GPU work just enqueued */
        for (int k = 0; k < done_n; ++k) {
            const unsigned long it = done_first + (unsigned long)k;
            if (fmod((double)it, (double)S.d_wrt_energies) == 0)
                check(scft_write_energies(NULL, &d, &done_recs[k]), "energies");
        }
        done_n = 0;
        if (done_snap) {
            check(scft_write_snapshot(NULL, &d, done_iter, phi13, w14, done_saved), "snapshot");
            done_snap = 0;
        }
        if (n == 0) break;
        if (!host_noise) check(scft_iterate_wait(ctx, recs), "scft_iterate_wait");
        memcpy(done_recs, recs, sizeof(scft_iter_out) * (size_t)n);
        done_n = n;
        done_first = iter + 1;
        iter += (unsigned long)n;
        if (fmod((double)iter, (double)S.d_wrt) == 0 || iter == 1) {
            if (!host_noise) check(scft_get_rng(ctx, 0, seed), "scft_get_rng");
            check(scft_get_fields(ctx, 0, w14), "scft_get_fields");
            check(scft_get_densities(ctx, 0, phi13, NULL), "scft_get_densities");
            memcpy(done_saved, saved, sizeof(saved));
            memcpy(saved, seed, sizeof(saved));
            done_iter = iter;
            done_snap = 1;
        }
    }
    free(done_recs);
    free(recs);
    scft_ctx_destroy(ctx);
    free(mask3);
    free(w14);
    free(phi13);
    free(noise);
    return 0;
}
