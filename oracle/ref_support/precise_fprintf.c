/*
 * precise_fprintf.c — TEST INFRASTRUCTURE for building the reference solver.
 * oracle/build_ref.py appends "#define fprintf oracle_fprintf" to a generated
 * parameters.h (SCFT.c includes it after <stdio.h>), so every fprintf in
 * SCFT.c lands here. Each floating conversion (%f, %lf, %10.6lf, ...) is
 * rewritten to %.17g, which round-trips doubles exactly; every other
 * conversion and all literal text are kept. This gives full-precision golden
 * outputs without touching the reference source.
 */
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

int oracle_fprintf(FILE *f, const char *fmt, ...)
{
    char out[8192];
    size_t o = 0;
    const char *p = fmt;
    while (*p && o < sizeof(out) - 16) {
        if (*p != '%') {
            out[o++] = *p++;
            continue;
        }
        const char *spec = p++;
        if (*p == '%') {
            out[o++] = '%';
            out[o++] = '%';
            ++p;
            continue;
        }
        while (*p && strchr("-+ #0123456789.", *p)) ++p;
        while (*p && strchr("hlLqjzt", *p)) ++p;
        const char conv = *p ? *p++ : 0;
        if (conv == 'f' || conv == 'F' || conv == 'e' || conv == 'g') {
            memcpy(out + o, "%.17g", 5);
            o += 5;
        } else {
            memcpy(out + o, spec, (size_t)(p - spec));
            o += (size_t)(p - spec);
        }
    }
    out[o] = 0;
    va_list ap;
    va_start(ap, fmt);
    int r = vfprintf(f, out, ap);
    va_end(ap);
    return r;
}
