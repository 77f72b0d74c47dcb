/* The integer-pipe FP32 <-> FP64 conversions of fpconv.cuh against the C
 * casts (IEEE round to nearest even), on random bit patterns, random values
 * over a wide exponent range, values next to rounding ties, and normal
 * doubles; and the truncating estimate against its error bound.  Built and
 * run by tests/test_fpconv.py; exit status 0 when everything matches. */
#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include <float.h>
#include "fpconv.cuh"
static uint64_t s = 88172645463325252ull;
static uint64_t xr(void) { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; }
int main(void) {
    long bad = 0, n = 0;
    for (long i = 0; i < 4000000; i++) {
        uint64_t u = xr();
        double d;
        int mode = i % 4;
        if (mode == 0) { memcpy(&d, &u, 8); }
        else if (mode == 1) { d = ldexp((double)(u >> 11) / 9007199254740992.0, (int)(xr() % 300) - 150) * ((u & 1) ? -1 : 1); }
        else if (mode == 2) { float f = (float)((double)(u>>11) / 9007199254740992.0 * 100.0 - 50.0); double t = f; uint64_t tu; memcpy(&tu,&t,8); tu ^= ((u >> 40) & 1) << 28; tu += (xr() % 3) - 1; memcpy(&d,&tu,8); }
        else { d = ldexp(1.0 + (double)(xr() >> 12) / 4503599627370496.0, (int)(xr() % 280) - 140); }
        float a = d2f_rn(d), b = (float)d;
        uint32_t ua = fpc_f2u(a), ub = fpc_f2u(b);
        if (ua != ub && !(isnan(a) && isnan(b))) { if (bad < 5) printf("d2f %a: %a vs %a\n", d, a, b); bad++; }
        float f = fpc_u2f((uint32_t)xr());
        double x = f2d_exact(f), y = (double)f;
        if (fpc_d2u(x) != fpc_d2u(y) && !(isnan(x) && isnan(y))) { if (bad < 5) printf("f2d %a\n", f); bad++; }
        float e = d2f_est(d);
        if (isfinite(d) && fabs(d) > 1e-37 && fabs(d) < 1e37 && fabs((double)e - d) > fabs(d) * 1.2e-7) { if (bad < 5) printf("est %a %a\n", d, e); bad++; }
        if (isnan(d) != isnan(e) || (fabs(d) > 3.5e38 && !isnan(d) && !isinf(e)) || (fabs(d) < 1e-39 && e != 0.0f)) { if (bad < 5) printf("est range %a %a\n", d, e); bad++; }
        n++;
    }
    printf("%ld cases, %ld mismatches\n", n, bad);
    return bad != 0;
}
