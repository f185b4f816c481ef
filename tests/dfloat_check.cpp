// Host check of the double-float arithmetic in csrc/scft_dfloat.cuh against
// long double: random operands over several decades, each operation's error
// measured against its exact value and compared with a double-word bound
// (a few 2^-48 of the operands' magnitudes). Prints the worst ratio of error
// to bound per operation; exit status 1 if any bound is exceeded.
// Built by tests/test_dfloat_host.py with g++ (IEEE single precision, no
// FMA contraction: -ffp-contract=off) against the CUDA runtime headers.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "scft_dfloat.cuh"

typedef long double LD;

static LD val(dfloat x) { return (LD)x.hi + (LD)x.lo; }

static unsigned long long rng_state = 0x9E3779B97F4A7C15ull;
static double urand()
{
    rng_state ^= rng_state << 13;
    rng_state ^= rng_state >> 7;
    rng_state ^= rng_state << 17;
    return (double)(rng_state >> 11) * (1.0 / 9007199254740992.0);
}
/* a double of random sign, magnitude 10^[-3, 3) */
static double rnd() { return (urand() < 0.5 ? -1.0 : 1.0) * pow(10.0, 6.0 * urand() - 3.0); }

static const LD U = 3.552713678800501e-15L; /* 2^-48 */

struct Worst {
    const char *name;
    double ratio;
    void see(LD err, LD bound)
    {
        const double r = (double)(fabsl(err) / bound);
        if (r > ratio) ratio = r;
    }
};

int main()
{
    Worst wadd{"add", 0}, wmul{"mul", 0}, wms{"mul_sub", 0}, wdiv{"div", 0}, wdot{"dot48", 0}, wnorm{"normalised", 0};
    const int N = 200000;
    for (int t = 0; t < N; ++t) {
        const dfloat x(rnd()), y(rnd()), u(rnd()), v(rnd());
        const LD X = val(x), Y = val(y), Uu = val(u), V = val(v);
        const dfloat s = x + y;
        wadd.see(val(s) - (X + Y), 4 * U * (fabsl(X) + fabsl(Y)));
        const dfloat p = x * y;
        wmul.see(val(p) - X * Y, 5 * U * fabsl(X * Y));
        const dfloat m = dfo::mul_sub(x, y, u, v);
        wms.see(val(m) - (X * Y - Uu * V), 6 * U * (fabsl(X * Y) + fabsl(Uu * V)));
        const dfloat q = x / y;
        wdiv.see(val(q) - X / Y, 8 * U * fabsl(X / Y));
        /* results are normalised pairs: |lo| <= ulp(hi) / 2 */
        for (dfloat r : {s, p, m, q})
            if (r.hi != 0.0f) wnorm.see(r.lo, 0.5L * ldexpl(1.0L, ilogbf(r.hi) - 23));
    }
    for (int t = 0; t < N / 100; ++t) {
        DotDF d;
        d.zero();
        LD exact = 0, mag = 0;
        for (int j = 0; j < 48; ++j) {
            const dfloat a(rnd()), b(rnd());
            d.add(a, b);
            exact += val(a) * val(b);
            mag += fabsl(val(a) * val(b));
        }
        wdot.see(val(d.value()) - exact, 48 * 2 * U * mag);
    }
    int bad = 0;
    /* integers convert exactly (the FFT pass divides the mean mode by the line length) */
    for (long long i : {0LL, 1LL, -1LL, 192LL, 16777217LL, -16777219LL, 2147483647LL, -2147483647LL - 1}) {
        const dfloat d((int)i);
        if (val(d) != (LD)i) {
            printf("int %lld converts to %.21Lg\n", i, val(d));
            bad = 1;
        }
    }
    for (const Worst *w : {&wadd, &wmul, &wms, &wdiv, &wdot, &wnorm}) {
        printf("%-10s worst error / bound = %.3f\n", w->name, w->ratio);
        if (!(w->ratio <= 1.0)) bad = 1;
    }
    return bad;
}
