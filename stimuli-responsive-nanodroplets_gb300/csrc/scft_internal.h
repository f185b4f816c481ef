/*
 * scft_internal.h — device-side layout of one SCFT context (not part of the ABI).
 *
 * HBM layout per context (B instances that share grid and contour counts):
 *   fields   w[b][14][SM]      FP64: 13 chemical potentials + pressure p
 *   boltz    bz[b][13][SM]     P: exp(-DS*w/2) per field (SCFT.c:2344)
 *   masks    mk[b][3][SM]      FP64: brush grafting masks (wMask.dat)
 *   q        per chain c: q_c[s][SM] P, s = 0..len-1 (contour-major SoA; the
 *            reference is AoS q[s + NS*idx], SCFT.c:2398)
 *   tmp      per chain c: one slice, the intermediate of a multi-pass step
 *   raw      raw[b][block][SM] FP64: unnormalised Simpson sums per density block
 *   phi      phi[b][14][SM] FP64: 13 total densities + phi_tot
 * SM is M rounded up to a multiple of 64 elements so every slice starts on a
 * 512-byte boundary.
 */
#pragma once

#include <cuda_runtime.h>

#include "scft_gpu.h"

#define SCFT_MAX_CHAINS 26  /* 10 homo + 4*2 dbk + 3*2 brush */
#define SCFT_MAX_BLOCKS 21  /* 10 homo + 4*2 dbk + 3 brush */
#define SCFT_MAX_RADIX_STAGES 12
#define SCFT_INIT_ONES 0
#define SCFT_INIT_MASK 1
#define SCFT_INIT_SEED 2

/* Diffusion operators of one instance (they depend on DS and the grid
 * spacing, so instances with different NS or box lengths have their own):
 * tables of the fused 2D chain kernel and, per grid axis in the context's axis
 * order, those of the per-axis passes. Instances with equal operators share. */
struct InstOps {
    const void *kz, *twx, *ex;
    const void *spec[3], *tw[3], *kA[3], *kB[3];
};

/* One propagator chain of one instance: q[0] from init, then len-1 contour
 * steps; steps s < seg_end use field f0, later steps field f1 (the diblock
 * junction). */
struct ChainDesc {
    void *q;        /* len slices */
    void *tmp;      /* one slice */
    const void *b0; /* Boltzmann factor slice of f0 */
    const void *b1; /* ... of f1 */
    int seg_end;
    int len;
    int init;       /* SCFT_INIT_* */
    int init_arg;   /* mask index for SCFT_INIT_MASK */
    int instance;
    int pad;
    const InstOps *ops; /* the instance's operators (device) */
};

/* One funDensity call (SCFT.c:2270-2308) of one species block. */
struct BlockDesc {
    int chain_f;   /* forward propagator chain (index within the instance) */
    int chain_b;   /* complementary chain (== chain_f for homopolymers) */
    int start, stop;
    int len;       /* NS_EFF of the species */
    int species;   /* 0..16: which Q normalises it */
    int field;     /* 0..12: which total it adds to */
    int part;      /* 0: first operand of funAddArray (diblock/brush), 1: second (homo) */
};

/* Species whose Q comes from chain q_chain at slice len-1 (SCFT.c:1837-1872). */
struct SpeciesDesc {
    int present;
    int q_chain;
    int len;
    int pad;
};

/* Per-instance scalars read by the fused update kernel. */
struct InstParams {
    double chi[SCFT_NFIELDS][SCFT_NFIELDS];
    double phi_avg[SCFT_NFIELDS];
    double frac[SCFT_MAX_BLOCKS];        /* funVolFrac factor per block */
    double lnq_coef[SCFT_NSPECIES];      /* H_fe_fraction coefficient per species */
    double g1, g2, dt_noise, ds;
    long relaxation;
    int active[SCFT_NFIELDS];
    int n_active;
    int enable_seed, seed_steps, seed_area_delta;
    int mask;
    int pad;
};

/* Per-instance device state that changes every iteration. */
struct InstState {
    unsigned long iter;   /* iIter, incremented at the start of each iteration */
    unsigned long tick;   /* iterations launched in the current scft_iterate call (history slot + 1) */
    unsigned long long rng; /* 48-bit drand48 state (device noise replay) */
    double q[SCFT_NSPECIES];
    double p_avg;
    double stop_rms;      /* 0: run every iteration; else freeze once RMS < stop_rms */
    int status;
    int done;             /* 1: frozen, every kernel skips the instance; 2: met the stop criterion in
                             this iteration (the p shift still runs; the next iteration begins frozen) */
};

/* Geometry of one axis pass of the propagator step. */
struct AxisGeom {
    int n;         /* line length */
    int ls;        /* element stride along the line */
    int inner;     /* lines per outer group sharing a base (x, y axes) */
    int outer;     /* number of outer groups */
    int dirichlet; /* 1: dense Dirichlet operator, 0: periodic FFT */
    int nrad;
    int rad[SCFT_MAX_RADIX_STAGES];
    /* per stage: ceil(2^32 / d) for d = n / rad (the butterflies of a line) and
     * d = the product of the earlier radices (0 when d = 1), so the Stockham
     * stages divide by a multiply-high instead of an integer division */
    unsigned mag_nr[SCFT_MAX_RADIX_STAGES];
    unsigned mag_ns[SCFT_MAX_RADIX_STAGES];
};

/* Arguments of one axis pass of the propagator step (scft_prop.cu). */
struct PassArgs {
    const ChainDesc *chains;
    const InstState *state; /* [B]: chains of frozen instances are skipped (NULL: no check) */
    int nchains;
    int s;          /* contour step: reads slice s, writes slice s+1 */
    int first;      /* multiply by b on load, read q[s] */
    int last;       /* multiply by b on store, write q[s+1] */
    int tile;       /* lines per CTA */
    long sstride;   /* slice stride (elements) */
    int axis;       /* operator slot in InstOps: spec/tw (periodic FFT) or kA/kB (dense) */
    int h;          /* half size (n even) or n (odd: kA holds the full matrix) */
    int even;
};

size_t scft_pass_smem_bytes(const AxisGeom &g, int tile, int h, int psize);
cudaError_t scft_pass_configure(int smem_bytes);
cudaError_t scft_launch_pass(int prec, const AxisGeom &g, const PassArgs &a, int ntiles, cudaStream_t st);

/* Arguments shared by the non-propagator kernels (scft_post.cu). */
struct PostArgs {
    const InstParams *params;   /* [B] */
    InstState *state;           /* [B] */
    const ChainDesc *chains;    /* [B * nchains] */
    const BlockDesc *blocks;    /* [B][nblocks] */
    const SpeciesDesc *species; /* [B][17] */
    int nchains, nblocks;
    int n_active;               /* active fields, the same for every instance */
    int B;
    int nx, ny, nz;
    long m, sm;                 /* points, slice stride */
    double *w;                  /* [B][14][sm] */
    double *phi;                /* [B][14][sm]: 13 totals + phi_tot */
    double *raw;                /* [B][nblocks][sm] */
    const double *mask;         /* [B][3][sm] */
    void *bz;                   /* [B][13][sm] P */
    unsigned field_use;         /* bit f: some chain propagates with field f */
    double *partial;            /* [B][nparts][...] */
    int nparts;
    const double *noise;        /* [B][n_active][sm] or NULL */
    scft_iter_out *hist;        /* [cap][B] */
    scft_iter_out *last;        /* [B]: the latest record (repeated while frozen) */
    int hist_cap;
    /* which density blocks make up each field's total (funAddArray operands,
     * SCFT.c:1486-1495): first operand (diblock or brush block), second
     * operand (homopolymer block), -1 if absent. Same for every instance. */
    int part0[SCFT_NFIELDS];
    int part1[SCFT_NFIELDS];
};

cudaError_t scft_post_iter_begin(const PostArgs &a, int prec, int sms, cudaStream_t st);
cudaError_t scft_post_mark_start(const PostArgs &a, cudaStream_t st);
cudaError_t scft_post_iter_end(const PostArgs &a, int prec, int sms, cudaStream_t st);
/* k_density alone (the unit entry point scft_density) */
cudaError_t scft_density_launch(const PostArgs &a, int prec, int sms, cudaStream_t st);
int scft_post_nparts(long m, int sms);
cudaError_t scft_convert(int prec, const double *src, void *dst, long n, int to_p, cudaStream_t st);
cudaError_t scft_boltz_one(int prec, const double *w, void *bz, double ds, long m, cudaStream_t st);

/* Arguments of the fused 2D contour step (scft_step2d.cu). */
struct Step2DArgs {
    const ChainDesc *chains;
    const int *order;  /* chain indices, longest first (or NULL) */
    const InstState *state; /* [B]: chains of frozen instances return at once (NULL: no check) */
    int s;             /* first contour step: reads slice s */
    int s_end;         /* runs steps s .. min(s_end, len-1)-1 */
    long sstride;      /* slice stride (elements) */
    /* per chain through ChainDesc::ops: kz P[2*H*H] (A[i][k] then B[i][k],
     * H = NZ/2) or, where scft_step2d_ztc is 1, float band[NZ][8] followed by
     * the bf16 pieces Ae1, Ae2, Ao1, Ao2 of the tail (H x H each, K-major
     * core-matrix layout); twx Cx<P>[NX] (exp(-2 pi i n2 k1 / NX) at
     * n2*N1 + k1), ex P[NX] (E_x(k)/NX) */
};

size_t scft_step2d_smem(int prec, int nx, int nz);
/* 64^3 periodic FP32 grids: one 8-CTA cluster per chain (scft_step3d.cu) */
size_t scft_step3d_smem(int prec, int nx, int ny, int nz);
cudaError_t scft_launch_step3d(const Step2DArgs &a, int nchains, cudaStream_t st, int configure);
int scft_step2d_n1(int nx);
cudaError_t scft_launch_step2d(int prec, int nx, int nz, const Step2DArgs &a, int nblocks, cudaStream_t st,
                               int configure, int wide);
/* 1 if (nx, nz) has the two-threads-per-line form of the fused 2D loop */
int scft_step2d_wide(int prec, int nx, int nz);
/* 1 if the fused 2D loop of (nx, nz) runs the z tail on the tensor cores */
int scft_step2d_ztc(int prec, int nx, int nz);
/* 1 if a tensor-core wait of the 2D loop gave up since the last call (clears it) */
int scft_step2d_take_fault(void);

/* Internal hooks of scft_ctx.cu for the allocation-free propagator entry point. */
int scft_ctx_info(const scft_ctx *c, int *device, int *prec, long *m, long *sm, double *ds, cudaStream_t *st,
                  const InstOps **ops0);
int scft_ctx_run_chain(scft_ctx *c, const ChainDesc *dev_desc, int len);
void scft_set_error(const char *msg);

/* Device replay of the drand48 noise stream (scft_noise.cu). */
struct NoiseArgs {
    InstState *state;
    const InstParams *params;
    unsigned long long *state_in; /* [B] state at the start of the iteration */
    int *counts;                  /* [B][nchunks] */
    long *prefix;                 /* [B][nchunks] */
    long *total;                  /* [B] */
    double *noise;                /* [B][n_active][sm] */
    long nchunks;
    long m, sm;
    int nx, ny, nz;
    int B;
};

long scft_noise_chunks(long m, int n_active);
cudaError_t scft_noise_setup(void);
cudaError_t scft_noise_launch(const NoiseArgs &n, cudaStream_t st);
