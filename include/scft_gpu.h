/*
 * scft_gpu.h — C ABI of the GB300 (sm_103a) SCFT hot path.
 *
 * The reference (SCFT.c) has no library interface: its run surface is the
 * compile-time parameters.h plus text input/output files, and its hot path is a
 * set of process-global functions (SCFT.c:13-32). This header is the boundary a
 * drop-in replacement exports instead: plain C types, caller-owned host buffers,
 * library-owned device memory, int status codes, no CUDA or torch types.
 *
 * Layout conventions (identical to the reference):
 *   grid index  idx = k + NZ*(j + NY*i)   (z fastest, x slowest; SCFT.c:773, :806)
 *   field order A B C D E F G H I J S1 S2 S3 (SCFT.c:1930-1945), p last where a
 *   14-column block is used (restart_fields.dat columns, SCFT.c:1645-1646).
 *   A "w14" buffer is 14 consecutive arrays of M = NX*NY*NZ doubles (field-major).
 *   Species order for the 17 per-species scalars (mu, Q) is the energies.dat
 *   order: dbk1..dbk4, homo A..J, S1..S3 (SCFT.c:1587-1590).
 */
#ifndef SCFT_GPU_H
#define SCFT_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define SCFT_OK 0
#define SCFT_ERR_PARAM (-1)     /* invalid argument or parameter set */
#define SCFT_ERR_CUDA (-2)      /* CUDA runtime error (message via scft_last_error) */
#define SCFT_ERR_OOM (-3)       /* device allocation failed */
#define SCFT_ERR_NONFINITE (-4) /* NaN/Inf in Q, free energy or RMS */
#define SCFT_ERR_VOLUME (-5)    /* volume fractions do not sum to 1 (SCFT.c:84-101) */
#define SCFT_ERR_STATE (-6)     /* call out of order (e.g. iterate before set_fields) */
#define SCFT_ERR_IO (-7)        /* file could not be opened or parsed */
#define SCFT_ERR_NODEV (-8)     /* no CUDA device */

#define SCFT_NFIELDS 13
#define SCFT_NSPECIES 17

/* --------------------------------------------------------- run surface */
/* Every macro of parameters.h (parameters.h:1-190) as a runtime value.
 * chi_n is the symmetric chi*N table in field order; the diagonal is ignored.
 * Replaces: the compile-time macro surface read by SCFT.c:10. */
typedef struct scft_surface {
    double lx, ly, lz;          /* LX LY LZ */
    long iter;                  /* ITER */
    long d_wrt;                 /* D_WRT */
    long relaxation;            /* RELAXATION */
    long d_wrt_energies;        /* D_WRT_ENERGIES */
    double dt_noise;            /* DT_NOISE */
    int mask;                   /* MASK */
    int enable_seed;            /* ENABLE_SEED */
    int seed_steps;             /* SEED_STEPS */
    int seed_area_delta;        /* SEED_AREA_DELTA */
    int ns;                     /* NS */
    int pad0;
    double dr_target;           /* DR_TARGET */
    double g1;                  /* G1 (G2..G13 = G1/6, parameters.h:160-171) */
    double chi_n[SCFT_NFIELDS][SCFT_NFIELDS];
    double f_dbk[4], len_dbk[4], vol_dbk[4];
    double vol_homo[10], len_homo[10];
    double vol_s[3], len_s[3];
} scft_surface;

/* Quantities main() derives from the surface before the loop.
 * Replaces: SCFT.c:84-119 (volume check, grid, chi_EFF), :121-288 (contour
 * counts, ALPHA), :290-396 (phi averages, chi zeroing), :718-733 (coating). */
typedef struct scft_derived {
    int nx, ny, nz;
    int n_ext;                  /* z length of the FFT box: 2(NZ+1) if MASK else NZ (SCFT.c:680) */
    long m;                     /* NX*NY*NZ */
    double ds;                  /* DS = 1/(NS-1) */
    double dx, dy, dz;          /* DX DY DZ (parameters.h:173-175) */
    double alphax, alphay, alphaz; /* ALPHA* = DS/D*^2 (parameters.h:177-179) */
    int ns_dbk[4], ns_dbk_x[4], ns_dbk_y[4];
    int ns_homo[10];
    int ns_s[3];
    double alpha_dbk[4], alpha_homo[10], alpha_s[3];
    double phi_avg[SCFT_NFIELDS];
    double chi_eff[SCFT_NFIELDS][SCFT_NFIELDS];
    double coating_vol;
    int active[SCFT_NFIELDS];   /* fields updated by funUpdate (SCFT.c:2002-2042) */
    int n_active;
    double volume_sum;          /* the sum SCFT.c:86-88 checks */
    int volume_ok;
} scft_derived;

/* Fill *d from *s exactly as SCFT.c's main() does. Returns SCFT_ERR_VOLUME (with
 * *d filled) when the volume fractions miss 1 by >= 1e-6 (SCFT.c:92-101). */
int scft_derive(const scft_surface *s, scft_derived *d);

/* ------------------------------------------------------------ context */
typedef struct scft_ctx scft_ctx;

#define SCFT_PREC_FP64 0 /* plain form: every kernel in FP64 (the drop-in) */
#define SCFT_PREC_FP32 1 /* precision form: propagators FP32, reductions FP64 */
#define SCFT_PREC_FP32X2 2 /* propagators in double-float arithmetic (pairs of FP32, ~48-bit
                              significand, FP32 exponent range) on double-float slices,
                              reductions FP64: the finishing form below the FP32 form's floor */

#define SCFT_NOISE_HOST 0    /* caller passes noise arrays to scft_iterate */
#define SCFT_NOISE_DRAND48 1 /* device replays the drand48 stream (funGaussDev) */

typedef struct scft_options {
    int precision;   /* SCFT_PREC_* */
    int device;      /* CUDA device ordinal */
    int noise_mode;  /* SCFT_NOISE_* */
    int use_graph;   /* capture one iteration as a CUDA graph and replay it */
    int n_instances; /* instances in this context (batching form); 1 for a single solve */
    int kernel_path; /* 0: fused single-launch contour step where the shape has one, else per-axis
                        passes; 1: per-axis passes only */
    int autotune;    /* 1 (default): time the launch forms on the context's own chains at
                        creation and keep the fastest (cached per shape and batch size): per-axis
                        pass tiles, the fused 2D loop's one or two threads per line; 0: heuristics.
                        Every candidate gives bit-identical results. The timing is taken with the
                        context alone on the GPU: contexts whose iterations are kept in flight side
                        by side (pipelined parts of one batch, serving pools) run better on the
                        heuristic forms. */
    int reserved;
} scft_options;

void scft_options_default(scft_options *o);

/* Create a context for n_instances solves that share the grid, MASK and the
 * set of species present (surfaces[b] may differ in NS, LEN_*, F_INPUT_*, box
 * lengths, chi, G1, DT_NOISE, ...). Allocates all device memory up front
 * (fields, propagators, densities). Instances whose diffusion factors agree
 * share one set of operator tables.
 * Replaces: allocation and plan setup SCFT.c:433-701 and aExpArg SCFT.c:983-1023. */
int scft_ctx_create(const scft_surface *surfaces, const scft_options *opt, scft_ctx **out);
int scft_ctx_destroy(scft_ctx *ctx);
int scft_ctx_derived(const scft_ctx *ctx, int instance, scft_derived *d);
size_t scft_ctx_device_bytes(const scft_ctx *ctx);

/* Upload the 14 restart columns (w_A..w_J, w_S1..w_S3, p) of one instance.
 * Replaces: restart_fields.dat read SCFT.c:844-865 / zero start :799-842. */
int scft_set_fields(scft_ctx *ctx, int instance, const double *w14);
/* Upload the three grafting masks (S1, S2, S3; 3*M doubles).
 * Replaces: wMask.dat read SCFT.c:756-781. */
int scft_set_masks(scft_ctx *ctx, int instance, const double *mask3);
/* Set the iteration counter (the value read from counter.dat, SCFT.c:704-716).
 * Also re-arms an instance that a stop criterion froze. */
int scft_set_iteration(scft_ctx *ctx, int instance, unsigned long iter);
/* Convergence-driven stopping (no counterpart in the reference, which always
 * runs ITER iterations; SCFT.c:1088): once an iteration ends with
 * RMS(phi_tot - 1) < rms_tol the instance is frozen. Later iterations of the
 * context skip all of its work (contour steps, densities, update, noise draws),
 * and its records repeat the converging iteration with converged = 1. With a
 * stop criterion an instance whose Q, free energy or RMS turns non-finite is
 * frozen the same way (its records repeat status SCFT_ERR_NONFINITE) until
 * scft_set_iteration re-arms it, which also clears the status.
 * rms_tol = 0 (the default) keeps the fixed-ITER semantics. */
int scft_set_stop(scft_ctx *ctx, int instance, double rms_tol);
/* Freeze an instance now (an idle slot): later iterations skip it until
 * scft_set_iteration re-arms it. */
int scft_freeze(scft_ctx *ctx, int instance);
/* Give slot `instance` a new surface (continuous batching: a finished solve's
 * slot takes the next request). The surface must match the context's grid,
 * MASK, active fields and species composition, and every chain must fit the
 * contour slices allocated for the slot at creation (create the context with
 * the largest NS the slot will serve). New diffusion factors add an operator
 * set. Follow with scft_set_fields / scft_set_iteration. */
int scft_set_surface(scft_ctx *ctx, int instance, const scft_surface *s);
/* Set the 48-bit drand48 state (restart_random.dat, SCFT.c:867-878). */
int scft_set_rng(scft_ctx *ctx, int instance, const unsigned short seed[3]);
int scft_get_rng(const scft_ctx *ctx, int instance, unsigned short seed[3]);

/* Per-iteration scalars (what energies.dat, free_energy.dat, deviations.dat hold). */
typedef struct scft_iter_out {
    unsigned long iter;          /* iIter of this iteration */
    double free_energy;          /* H_fe after the ln Q terms (SCFT.c:1525-1555) */
    double rms;                  /* RMSDev (SCFT.c:1564-1580) */
    double mf;                   /* MF (SCFT.c:1515-1522) */
    double mu[SCFT_NSPECIES];    /* chemPot_* = -ln(Q^2)/2 (SCFT.c:1837-1872) */
    double q[SCFT_NSPECIES];     /* Qsum_* */
    int status;                  /* SCFT_OK or SCFT_ERR_NONFINITE */
    int converged;               /* 1: the stop criterion of scft_set_stop has been met */
} scft_iter_out;

/* Run n SCFT iterations on every instance (one pass of SCFT.c:1088-1580 each).
 * noise: NULL, or host noise for SCFT_NOISE_HOST: n * n_instances * n_active * M
 * doubles ordered [iteration][instance][active field][idx], the funGaussDev draws
 * the reference makes inside funUpdate (SCFT.c:2103). NULL with SCFT_NOISE_HOST
 * is allowed only while MF*DT_NOISE == 0.
 * out: NULL or n * n_instances records, [iteration][instance].
 * Replaces: the loop body SCFT.c:1090-1580. */
int scft_iterate(scft_ctx *ctx, int n, const double *noise, scft_iter_out *out);

/* scft_iterate in two halves, so that the host can keep several contexts (on
 * their own streams) busy at once: _async enqueues n <= SCFT_HIST_CAP
 * iterations without waiting (no host noise: SCFT_NOISE_DRAND48 or
 * MF*DT_NOISE == 0 throughout); _wait blocks until they finish and copies the
 * n * n_instances records to out (may be NULL). When an instance's records
 * carry SCFT_ERR_NONFINITE, _wait (like scft_iterate) still fills out with
 * every instance's records and then returns SCFT_ERR_NONFINITE: the caller
 * tells the failed instances from the others by their records' status. */
#define SCFT_HIST_CAP 256
int scft_iterate_async(scft_ctx *ctx, int n);
int scft_iterate_wait(scft_ctx *ctx, scft_iter_out *out);
/* 1 when the enqueued iterations have finished (or none are enqueued), 0 while
 * they run, a negative status on a device error. Never blocks. */
int scft_iterate_ready(scft_ctx *ctx);

/* Batching form over uneven grid sizes (no counterpart in the reference, which
 * runs one instance per process). A batch groups n surfaces by grid, MASK,
 * active fields and species composition into one context per group (own
 * stream, persistent chain kernel over the group's chains, optional CUDA graph
 * from opt->use_graph) and runs the groups side by side. Instance i is
 * addressed by its index in surfaces[]; scft_batch_locate gives its context
 * and slot for the per-context calls. */
typedef struct scft_batch scft_batch;
typedef struct scft_batch_result {
    unsigned long iterations; /* iterations run by the last scft_batch_run */
    unsigned long iter;       /* iIter after it */
    double free_energy;       /* of the last iteration run */
    double rms;
    int converged;            /* the stop criterion (scft_batch_set_stop) was met */
    int status;
} scft_batch_result;
int scft_batch_create(const scft_surface *surfaces, int n, const scft_options *opt, scft_batch **out);
int scft_batch_destroy(scft_batch *b);
int scft_batch_groups(const scft_batch *b);
int scft_batch_locate(const scft_batch *b, int instance, int *group, int *slot);
scft_ctx *scft_batch_context(scft_batch *b, int group);
int scft_batch_set_fields(scft_batch *b, int instance, const double *w14);
int scft_batch_set_masks(scft_batch *b, int instance, const double *mask3);
int scft_batch_set_iteration(scft_batch *b, int instance, unsigned long iter);
int scft_batch_set_rng(scft_batch *b, int instance, const unsigned short seed[3]);
int scft_batch_set_stop(scft_batch *b, int instance, double rms_tol);
/* Stop an instance now (scft_freeze on its context); scft_batch_set_iteration re-arms it.
 * scft_batch_run does not enqueue a group whose instances are all stopped. */
int scft_batch_freeze(scft_batch *b, int instance);
int scft_batch_get_fields(scft_batch *b, int instance, double *w14);
int scft_batch_get_densities(scft_batch *b, int instance, double *phi13, double *phi_tot);
/* Iterate every instance until it converges or has run max_iter iterations in
 * this call, chunk (<= SCFT_HIST_CAP) iterations per group per round. res: NULL
 * or n results. */
int scft_batch_run(scft_batch *b, int max_iter, int chunk, scft_batch_result *res);

/* Download fields (w14 layout), the 13 total densities (13*M, field order) and
 * phi_tot (M). Any pointer may be NULL. */
int scft_get_fields(scft_ctx *ctx, int instance, double *w14);
int scft_get_densities(scft_ctx *ctx, int instance, double *phi13, double *phi_tot);

/* The same transfers for every instance at once (one strided copy each):
 * w14_all is n_instances consecutive w14 blocks; phi14_all is n_instances
 * blocks of the 13 total densities followed by phi_tot. Pinned host buffers
 * make these run at the host link's bandwidth. */
int scft_set_fields_all(scft_ctx *ctx, const double *w14_all);
int scft_get_fields_all(scft_ctx *ctx, double *w14_all);
int scft_get_densities_all(scft_ctx *ctx, double *phi14_all);
/* The same transfers enqueued on the context's stream without waiting, in
 * order with scft_iterate_async; the host buffers must stay valid (and, to
 * overlap with other contexts' work, be pinned) until scft_sync or
 * scft_iterate_wait returns. */
int scft_set_fields_all_async(scft_ctx *ctx, const double *w14_all);
int scft_get_fields_all_async(scft_ctx *ctx, double *w14_all);
int scft_get_densities_all_async(scft_ctx *ctx, double *phi14_all);
int scft_sync(scft_ctx *ctx);

/* Unit entry point: contour steps of one block, as funPDESolver does
 * (SCFT.c:2310-2412) in this context's geometry and precision. q0 is the
 * initial slice (M doubles), w the field (M doubles); q_out receives
 * steps+1 slices (contour-major, slice 0 = q0). */
int scft_propagate(scft_ctx *ctx, const double *q0, const double *w, int steps, double *q_out);

/* Unit entry point: funMultiplyQs + funDensity (SCFT.c:2243-2308) on host
 * propagators qf, qb (len slices of M doubles, contour-major as scft_propagate
 * returns them): phi = (sum_s w_s qf[s] qb[len-1-s] / 3) * (DS_EFF / q), the
 * reference's Simpson weights over s in [start, stop], DS_EFF = 1/(len-1). The
 * propagators are held in the context's precision and summed as the iteration
 * does (FP64, or double-float for FP32 propagators). */
int scft_density(scft_ctx *ctx, const double *qf, const double *qb, int len, int start, int stop, double q,
                 double *phi);

/* scft_propagate for callers that must not allocate device memory at run time
 * (hosts whose memory pools already own the device, code that cannot accept the
 * device synchronisation cudaMalloc/cudaFree may cause or an allocation failure
 * mid-run). Same arguments and result; the working buffers live in one fixed
 * device array of scft_static_scratch_bytes() bytes per GPU, held until exit.
 * The first call on a device looks up that array's address and keeps it, so
 * the device must not be reset after that call. Every call synchronises its
 * stream and copies to pageable host memory: it cannot be called inside a
 * stream capture. Calls share the array: overlapping calls on one GPU race and
 * must be serialised by the caller (each call returns only after its own GPU
 * work has finished, on errors too). Sizes that do not fit return
 * SCFT_ERR_PARAM with a message in scft_last_error(). It has no counterpart in
 * the reference. */
int scft_propagate_static(scft_ctx *ctx, const double *q0, const double *w, int steps, double *q_out);
size_t scft_static_scratch_bytes(void);

/* Timing of the last scft_iterate call, measured with CUDA events on the
 * context's stream: total device time, time in propagator-step kernels and
 * the number of propagator-step launches. */
typedef struct scft_timing {
    double total_ms;
    double prop_ms;
    long prop_launches;
    long kernel_launches;
    int fused_chain;   /* contour steps run in one persistent launch: 1 the fused 2D chain kernel,
                          2 the 64^3 cluster kernel; 0 per-axis passes */
    int threads_per_line; /* fused 2D kernel: 2 when a batch of at most one chain per SM gives each
                             line two threads (bit-identical results), else 1 */
} scft_timing;
int scft_enable_timing(scft_ctx *ctx, int on);
int scft_get_timing(const scft_ctx *ctx, scft_timing *t);

const char *scft_last_error(void);

/* Free and total device memory of a GPU (for admission by memory budget in
 * the serving form; no counterpart in the reference). SCFT_ERR_NODEV without
 * a usable device. */
int scft_device_memory(int device, size_t *free_bytes, size_t *total_bytes);

/* ---------------------------------------------------------- host side */
/* Fill noise for one iteration of one instance with the reference's draws:
 * one Marsaglia-polar Gaussian per active field per grid point, points in the
 * loop order k, j, i and fields in order A..S3 (funGaussDev SCFT.c:1769-1782
 * called from funUpdate SCFT.c:2103), advancing the 48-bit state exactly as
 * drand48 does after seed48. out: n_active * M doubles, [active field][idx].
 * out may be NULL to only advance the state (the reference draws even when MF=0). */
int scft_noise_fill(unsigned short state[3], const scft_derived *d, double *out);

/* File names of the text I/O: the file-name macros of parameters.h
 * (parameters.h:181-190, opened by SCFT.c at :704, :756, :847, :869, :1026,
 * :1585-1661). density is the prefix of the snapshot names (density +
 * 100000000+iter + ".dat"). Names are relative to dir (or the cwd). */
#define SCFT_NAME_MAX 256
typedef struct scft_file_names {
    char counter[SCFT_NAME_MAX];        /* COUNTER        "counter.dat" */
    char density[SCFT_NAME_MAX];        /* DENSITY        "densities_dbk_" */
    char deviations[SCFT_NAME_MAX];     /* DEVIATIONS     "deviations.dat" */
    char energy[SCFT_NAME_MAX];         /* ENERGY         "energies.dat" */
    char restart_fields[SCFT_NAME_MAX]; /* RESTART_FIELDS "restart_fields.dat" */
    char restart_random[SCFT_NAME_MAX]; /* RESTART_RANDOM "restart_random.dat" */
    char run_params[SCFT_NAME_MAX];     /* RUN_PARAMS     "run.txt" */
    char w_mask[SCFT_NAME_MAX];         /* W_MASK         "wMask.dat" */
    char free_energy[SCFT_NAME_MAX];    /* FREE_ENERGY    "free_energy.dat" */
} scft_file_names;
/* Fills n with the reference's default names. */
void scft_file_names_default(scft_file_names *n);
/* Sets the names every reader and writer below uses from now on, in this
 * process (NULL restores the defaults). Empty or unterminated names return
 * SCFT_ERR_PARAM. Not thread-safe against concurrent I/O calls: set the names
 * once, before the run, as SCFT.c compiles them in. */
int scft_set_file_names(const scft_file_names *n);

/* Text I/O with the reference's exact formats. dir may be NULL for the cwd. */
int scft_read_counter(const char *dir, unsigned long *iter);             /* SCFT.c:704-716 */
int scft_read_restart_fields(const char *dir, const scft_derived *d, double *w14); /* :844-865 */
int scft_read_restart_random(const char *dir, unsigned short seed[3]);   /* :867-878 */
int scft_read_mask(const char *dir, const scft_derived *d, double *mask3); /* :756-781 */
int scft_write_volume_error(const char *dir, double volume_sum);        /* :92-101 */
int scft_write_run_params(const char *dir, const scft_surface *s, const scft_derived *d,
                          unsigned long iter);                          /* :1025-1085 */
/* energies.dat, free_energy.dat, deviations.dat lines (SCFT.c:1583-1599). */
int scft_write_energies(const char *dir, const scft_derived *d, const scft_iter_out *o);
/* densities_dbk_<100000000+iter>.dat, counter.dat, restart_fields.dat,
 * restart_random.dat (SCFT.c:1601-1663). */
int scft_write_snapshot(const char *dir, const scft_derived *d, unsigned long iter,
                        const double *phi13, const double *w14, const unsigned short seed[3]);

#ifdef __cplusplus
}
#endif
#endif /* SCFT_GPU_H */
