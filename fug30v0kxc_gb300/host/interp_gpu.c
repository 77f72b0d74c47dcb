/*
 * interp_gpu.c -- the reference's interpolate program (interpolate/main.F90)
 * as a C host on the GB300 library: reads restart.nc, expands the eight
 * fields R, T, U, V, W, Bx, By, Bz from (nx, ny, nz) to (2 nx, 2 ny, nz) with
 * the spectral expand of interpolate/fft.F90:834-927 (vec_expand), prints
 * the diagnostics of interpolate/main.F90:290-370 and writes output.nc in
 * the 64-bit-offset NetCDF format with double fields
 * (interpolate/main.F90:384-395).
 *
 *   interp_gpu [--in restart.nc] [--out output.nc]
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "vec.h"

#define CHECK(call)                                                                     \
    do {                                                                                \
        int st_ = (call);                                                               \
        if (st_ != VEC_OK) {                                                            \
            fprintf(stderr, "ERROR: %s returned %d (%s)\n", #call, st_, vec_last_error()); \
            return 1;                                                                   \
        }                                                                               \
    } while (0)

static void minmax(const double *a, size_t n, double *mn, double *mx)
{
    *mn = a[0];
    *mx = a[0];
    for (size_t i = 1; i < n; i++) {
        if (a[i] < *mn) *mn = a[i];
        if (a[i] > *mx) *mx = a[i];
    }
}

int main(int argc, char **argv)
{
    const char *in = "restart.nc", *out = "output.nc";
    for (int i = 1; i < argc; i++) {
        if (!strcmp(argv[i], "--in") && i + 1 < argc) in = argv[++i];
        else if (!strcmp(argv[i], "--out") && i + 1 < argc) out = argv[++i];
        else { fprintf(stderr, "unknown option %s\n", argv[i]); return 2; }
    }
    /* sizes and parameters, then the fields (interpolate/netcdf.F90 ReadNetCDF) */
    vec_snapshot s;
    memset(&s, 0, sizeof(s));
    CHECK(vec_nc_read(in, &s));
    const size_t n = (size_t)s.nx * s.ny * s.nz, n2 = 4 * n;
    double *f[8], *g[8];
    for (int i = 0; i < 8; i++) {
        f[i] = (double *)malloc(sizeof(double) * n);
        g[i] = (double *)malloc(sizeof(double) * n2);
        if (!f[i] || !g[i]) { fprintf(stderr, "out of host memory\n"); return 1; }
        s.fields[i] = f[i];
    }
    CHECK(vec_nc_read(in, &s));
    printf(" -------------------------------\n");
    printf(" nx %d ny %d nz %d\n", s.nx, s.ny, s.nz);
    printf(" -------------------------------\n");

    vec_params p;
    CHECK(vec_params_default(&p));
    p.gamma = s.gamma; p.sigma = s.sigma; p.theta = s.theta; p.ck = s.ck; p.cm = s.cm; p.f = s.f;
    p.tayl = s.tayl; p.psi = s.psi; p.zeta = s.zeta; p.xmax = s.xmax; p.ymax = s.ymax;
    p.nx = s.nx; p.ny = s.ny; p.nz = s.nz;
    p.precision = VEC_PREC_FP64;
    vec_params p2 = p;
    p2.nx = 2 * s.nx;
    p2.ny = 2 * s.ny;
    vec_ctx *c = NULL, *c2 = NULL;
    CHECK(vec_create(&p, &c));
    CHECK(vec_create(&p2, &c2));
    static const int ids[8] = { VEC_F_R, VEC_F_T, VEC_F_U, VEC_F_V, VEC_F_W, VEC_F_BX, VEC_F_BY, VEC_F_BZ };
    for (int i = 0; i < 8; i++) CHECK(vec_set_field(c, ids[i], f[i]));
    double dt;
    CHECK(vec_calcdt(c, &dt));
    printf(" Initial Timestep, dt = %.10e\n\n", dt);
    for (int i = 0; i < 8; i++) CHECK(vec_expand(c, c2, f[i], g[i]));
    printf(" TTIME %.10e\n", s.time);
    vec_diag_out d;
    int st = vec_diag(c, &d);   /* GlobalAverages of the input state */
    if (st != VEC_OK && st != VEC_ERR_DIVB) CHECK(st);
    printf(" ubar= %.8e vbar= %.8e\n", d.ubar, d.vbar);
    /* sminmax of the expanded fields and of |u|^2/T, |B|^2/rho, |u|^2 */
    double mn[8], mx[8];
    for (int i = 0; i < 8; i++) minmax(g[i], n2, &mn[i], &mx[i]);
    double mach[2] = { 1e300, -1e300 }, alf[2] = { 1e300, -1e300 }, rms[2] = { 1e300, -1e300 };
    for (size_t q = 0; q < n2; q++) {
        const double uu = g[2][q] * g[2][q] + g[3][q] * g[3][q] + g[4][q] * g[4][q];
        const double bb = g[5][q] * g[5][q] + g[6][q] * g[6][q] + g[7][q] * g[7][q];
        const double a = uu / g[1][q], b = bb / g[0][q];
        if (a < mach[0]) mach[0] = a;
        if (a > mach[1]) mach[1] = a;
        if (b < alf[0]) alf[0] = b;
        if (b > alf[1]) alf[1] = b;
        if (uu < rms[0]) rms[0] = uu;
        if (uu > rms[1]) rms[1] = uu;
    }
    printf(" alfvenmin= %.8e alfvenmax= %.8e\n", sqrt(s.f * alf[0]), sqrt(s.f * alf[1]));
    printf(" machmin= %.8e machmax= %.8e\n", sqrt(mach[0] / s.gamma), sqrt(mach[1] / s.gamma));
    printf(" rmsmin= %.8e rmsmax= %.8e\n", sqrt(rms[0]), sqrt(rms[1]));
    printf(" rmin= %.8e rmax= %.8e\n tmin= %.8e tmax= %.8e\n", mn[0], mx[0], mn[1], mx[1]);
    printf(" umin= %.8e umax= %.8e\n vmin= %.8e vmax= %.8e\n", mn[2], mx[2], mn[3], mx[3]);
    printf(" wmin= %.8e wmax= %.8e\n", mn[4], mx[4]);
    printf(" bxmin= %.8e bxmax= %.8e\n bymin= %.8e bymax= %.8e\n", mn[5], mx[5], mn[6], mx[6]);
    printf(" bzmin= %.8e bzmax= %.8e\n", mn[7], mx[7]);
    /* output.nc: double fields, 64-bit offsets */
    vec_snapshot o = s;
    o.nx = 2 * s.nx;
    o.ny = 2 * s.ny;
    for (int i = 0; i < 8; i++) o.fields[i] = g[i];
    CHECK(vec_nc_write_fmt(out, &o, 8, 2));
    vec_destroy(c);
    vec_destroy(c2);
    for (int i = 0; i < 8; i++) { free(f[i]); free(g[i]); }
    return 0;
}
