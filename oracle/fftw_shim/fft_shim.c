/*
 * fft_shim.c — O(n log n) complex FFT behind the FFTW3 API subset declared in
 * fftw3.h. TEST INFRASTRUCTURE ONLY (builds the reference solver and the CPU
 * oracle in an image without FFTW3); the GPU product never links it.
 *
 * 1D engine: recursive decimation-in-time mixed-radix Cooley-Tukey. A length
 * n = p0*p1*...*pk is split into p0 interleaved sub-sequences of length n/p0,
 * each transformed recursively; a radix-p0 butterfly with twiddles
 * w^(k*u) = exp(sign*2*pi*i*k*u/n) combines them. Radix 4, 2, 3 and 5 have
 * hand-written butterflies, other primes up to 13 use a direct p-point DFT.
 * Lengths with a larger prime factor use Bluestein's identity
 *   jk = (j^2 + k^2 - (k-j)^2) / 2,
 * which turns the DFT into a linear convolution with the chirp exp(sign*pi*i*j^2/n),
 * evaluated by a power-of-two FFT of length >= 2n-1.
 *
 * 3D transforms apply the 1D engine along each axis (row-major, last index
 * contiguous), as FFTW's fftw_plan_dft_3d specifies.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3.h"

typedef double _Complex cpx;

#define OFFT_MAX_SMALL_PRIME 13

typedef struct offt_plan1d {
    int n;
    int sign;
    int nfac;
    int fac[64]; /* (radix, remaining length) pairs */
    cpx *tw;     /* tw[k] = exp(sign*2*pi*i*k/n), k < n */
    cpx *gen;    /* scratch for the generic radix butterfly */
    /* Bluestein */
    int blue;
    int m;
    cpx *chirp; /* chirp[j] = exp(sign*pi*i*(j^2 mod 2n)/n), j < n */
    cpx *kern;  /* forward FFT (length m) of conj(chirp) wrapped, divided by m */
    struct offt_plan1d *fm, *im;
    cpx *buf;
} offt_plan1d;

struct offt_plan3d {
    int n[3];
    int sign;
    offt_plan1d *axis[3];
    cpx *line_in, *line_out;
};

static cpx cis(double angle) { return cos(angle) + sin(angle) * I; }

static int is_smooth(int n)
{
    for (int p = 2; p <= OFFT_MAX_SMALL_PRIME; ++p)
        while (n % p == 0) n /= p;
    return n == 1;
}

static offt_plan1d *plan1d_create(int n, int sign);

static void plan1d_destroy(offt_plan1d *p)
{
    if (!p) return;
    free(p->tw);
    free(p->gen);
    free(p->chirp);
    free(p->kern);
    free(p->buf);
    plan1d_destroy(p->fm);
    plan1d_destroy(p->im);
    free(p);
}

static void transform(const offt_plan1d *p, cpx *out, const cpx *in, size_t istride);

static offt_plan1d *plan1d_create(int n, int sign)
{
    offt_plan1d *p = calloc(1, sizeof(*p));
    p->n = n;
    p->sign = sign;
    if (n > 1 && !is_smooth(n)) {
        /* Bluestein: a length-m power-of-two convolution with m >= 2n-1. */
        p->blue = 1;
        int m = 1;
        while (m < 2 * n - 1) m <<= 1;
        p->m = m;
        p->chirp = malloc(sizeof(cpx) * n);
        for (long long j = 0; j < n; ++j) {
            long long r = (j * j) % (2LL * n);
            p->chirp[j] = cis(sign * M_PI * (double)r / (double)n);
        }
        p->fm = plan1d_create(m, FFTW_FORWARD);
        p->im = plan1d_create(m, FFTW_BACKWARD);
        cpx *h = calloc(m, sizeof(cpx));
        h[0] = conj(p->chirp[0]);
        for (int d = 1; d < n; ++d) {
            h[d] = conj(p->chirp[d]);
            h[m - d] = conj(p->chirp[d]);
        }
        p->kern = malloc(sizeof(cpx) * m);
        transform(p->fm, p->kern, h, 1);
        for (int k = 0; k < m; ++k) p->kern[k] /= (double)m;
        free(h);
        p->buf = malloc(sizeof(cpx) * 2 * m);
        return p;
    }
    /* Factor: radix 4 first, then 2, 3, 5, then the remaining small primes. */
    int rem = n, nf = 0;
    const int order[] = {4, 2, 3, 5, 7, 11, 13};
    for (size_t t = 0; t < sizeof(order) / sizeof(order[0]) && rem > 1; ++t) {
        int r = order[t];
        while (rem % r == 0) {
            rem /= r;
            p->fac[2 * nf] = r;
            p->fac[2 * nf + 1] = rem;
            ++nf;
        }
    }
    if (n == 1) {
        p->fac[0] = 1;
        p->fac[1] = 1;
        nf = 1;
    }
    p->nfac = nf;
    p->tw = malloc(sizeof(cpx) * (n > 0 ? n : 1));
    for (int k = 0; k < n; ++k) p->tw[k] = cis(sign * 2.0 * M_PI * (double)k / (double)n);
    p->gen = malloc(sizeof(cpx) * (OFFT_MAX_SMALL_PRIME + 1));
    return p;
}

static void bfly2(const offt_plan1d *p, cpx *out, size_t fs, int m)
{
    for (int u = 0; u < m; ++u) {
        cpx t = out[u + m] * p->tw[u * fs];
        out[u + m] = out[u] - t;
        out[u] += t;
    }
}

static void bfly4(const offt_plan1d *p, cpx *out, size_t fs, int m)
{
    const cpx wq = (p->sign < 0) ? -I : I; /* exp(sign*i*pi/2) */
    for (int u = 0; u < m; ++u) {
        cpx a0 = out[u];
        cpx a1 = out[u + m] * p->tw[u * fs];
        cpx a2 = out[u + 2 * m] * p->tw[2 * u * fs];
        cpx a3 = out[u + 3 * m] * p->tw[3 * u * fs];
        cpx b0 = a0 + a2, b1 = a0 - a2, b2 = a1 + a3, b3 = (a1 - a3) * wq;
        out[u] = b0 + b2;
        out[u + m] = b1 + b3;
        out[u + 2 * m] = b0 - b2;
        out[u + 3 * m] = b1 - b3;
    }
}

static void bfly3(const offt_plan1d *p, cpx *out, size_t fs, int m)
{
    const double h = p->sign * (sqrt(3.0) / 2.0);
    for (int u = 0; u < m; ++u) {
        cpx a0 = out[u];
        cpx a1 = out[u + m] * p->tw[u * fs];
        cpx a2 = out[u + 2 * m] * p->tw[2 * u * fs];
        cpx s = a1 + a2, d = (a1 - a2) * (h * I);
        cpx c = a0 - 0.5 * s;
        out[u] = a0 + s;
        out[u + m] = c + d;
        out[u + 2 * m] = c - d;
    }
}

static void bfly_generic(const offt_plan1d *p, cpx *out, size_t fs, int m, int radix)
{
    cpx *a = p->gen;
    const int n = p->n;
    for (int u = 0; u < m; ++u) {
        for (int k = 0; k < radix; ++k) a[k] = out[u + k * m] * p->tw[(size_t)k * u * fs];
        for (int s = 0; s < radix; ++s) {
            cpx acc = a[0];
            for (int k = 1; k < radix; ++k) acc += a[k] * p->tw[((size_t)k * s * m * fs) % n];
            out[u + s * m] = acc;
        }
    }
}

static void dit(const offt_plan1d *p, cpx *out, const cpx *in, size_t fs, size_t istride, const int *fac)
{
    const int radix = fac[0], m = fac[1];
    if (m == 1) {
        for (int k = 0; k < radix; ++k) out[k] = in[(size_t)k * fs * istride];
    } else {
        for (int k = 0; k < radix; ++k)
            dit(p, out + (size_t)k * m, in + (size_t)k * fs * istride, fs * radix, istride, fac + 2);
    }
    switch (radix) {
    case 1: break;
    case 2: bfly2(p, out, fs, m); break;
    case 3: bfly3(p, out, fs, m); break;
    case 4: bfly4(p, out, fs, m); break;
    default: bfly_generic(p, out, fs, m, radix); break;
    }
}

/* out[k] = sum_j in[j*istride] * exp(sign*2*pi*i*j*k/n); out must not alias in. */
static void transform(const offt_plan1d *p, cpx *out, const cpx *in, size_t istride)
{
    if (!p->blue) {
        dit(p, out, in, 1, istride, p->fac);
        return;
    }
    const int n = p->n, m = p->m;
    cpx *a = p->buf, *A = p->buf + m;
    for (int j = 0; j < n; ++j) a[j] = in[(size_t)j * istride] * p->chirp[j];
    for (int j = n; j < m; ++j) a[j] = 0;
    transform(p->fm, A, a, 1);
    for (int k = 0; k < m; ++k) A[k] *= p->kern[k];
    transform(p->im, a, A, 1);
    for (int k = 0; k < n; ++k) out[k] = a[k] * p->chirp[k];
}

fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in, fftw_complex *out, int sign,
                           unsigned flags)
{
    (void)in;
    (void)out;
    (void)flags;
    if (n0 <= 0 || n1 <= 0 || n2 <= 0) return NULL;
    struct offt_plan3d *p = calloc(1, sizeof(*p));
    p->n[0] = n0;
    p->n[1] = n1;
    p->n[2] = n2;
    p->sign = sign;
    int nmax = 1;
    for (int a = 0; a < 3; ++a) {
        p->axis[a] = plan1d_create(p->n[a], sign);
        if (p->n[a] > nmax) nmax = p->n[a];
    }
    p->line_in = malloc(sizeof(cpx) * nmax);
    p->line_out = malloc(sizeof(cpx) * nmax);
    return p;
}

void fftw_execute_dft(const fftw_plan p, fftw_complex *in, fftw_complex *out)
{
    const size_t n0 = p->n[0], n1 = p->n[1], n2 = p->n[2];
    const size_t total = n0 * n1 * n2;
    if (out != in) memcpy(out, in, sizeof(cpx) * total);
    cpx *li = p->line_in, *lo = p->line_out;
    /* axis 2: contiguous lines */
    if (n2 > 1)
        for (size_t r = 0; r < n0 * n1; ++r) {
            cpx *line = out + r * n2;
            transform(p->axis[2], lo, line, 1);
            memcpy(line, lo, sizeof(cpx) * n2);
        }
    /* axis 1: stride n2 inside each n1*n2 slab */
    if (n1 > 1)
        for (size_t a = 0; a < n0; ++a)
            for (size_t c = 0; c < n2; ++c) {
                cpx *base = out + a * n1 * n2 + c;
                transform(p->axis[1], lo, base, n2);
                for (size_t b = 0; b < n1; ++b) base[b * n2] = lo[b];
            }
    /* axis 0: stride n1*n2 */
    if (n0 > 1)
        for (size_t c = 0; c < n1 * n2; ++c) {
            cpx *base = out + c;
            transform(p->axis[0], lo, base, n1 * n2);
            for (size_t a = 0; a < n0; ++a) base[a * n1 * n2] = lo[a];
        }
    (void)li;
}

void fftw_destroy_plan(fftw_plan p)
{
    if (!p) return;
    for (int a = 0; a < 3; ++a) plan1d_destroy(p->axis[a]);
    free(p->line_in);
    free(p->line_out);
    free(p);
}

void *fftw_malloc(size_t n)
{
    void *ptr = NULL;
    if (posix_memalign(&ptr, 64, n ? n : 1) != 0) return NULL;
    return ptr;
}

void fftw_free(void *p) { free(p); }
