/*
 * p3d_gpu.c -- the reference's main program (src/main.F90) as a C host that
 * drives the GB300 library through include/vec.h.
 *
 * Reads INPUT (src/initial.F90:94-201), starts from the static polytrope
 * (nframe 0) or restart.nc (nframe 1: parameters from the file; nframe 2:
 * parameters from INPUT), runs ntotal iterations of the time loop on the
 * GPU, prints the ndu06 diagnostics of src/main.F90:552-647 (every value
 * with 17 significant digits, as Fortran list-directed output prints a
 * double) and writes the T16_NNN.nc snapshots of src/main.F90:689-740.
 *
 * Options not in INPUT (the reference hard-codes them, src/main.F90:108-116):
 *   --constflux --radbc --perfect --kinematic --dynamo --no-dealias
 *   --eta-contrast C   eta(z) = zeta ck (1 + (C-1) z)      (default 1)
 *   --noise A          static-state noise amplitude        (default 0.1)
 *   --split            FP32-bulk / FP64-state form
 *   --input PATH       INPUT file (default ./INPUT)
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "vec.h"

static double now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

#define CHECK(call)                                                                  \
    do {                                                                             \
        int st_ = (call);                                                            \
        if (st_ != VEC_OK) {                                                         \
            fprintf(stderr, "ERROR: %s returned %d (%s)\n", #call, st_, vec_last_error()); \
            return st_ == VEC_ERR_DIVB ? 12 : 1;                                     \
        }                                                                            \
    } while (0)

int main(int argc, char **argv)
{
    const char *input = "INPUT";
    vec_params p;
    double eta = 1.0, noise = 0.1;
    int constflux = 0, radbc = 0, perfect = 0, kinematic = 0, dynamo = 0, dalias = 1, split = 0;
    for (int i = 1; i < argc; i++) {
        if (!strcmp(argv[i], "--constflux")) constflux = 1;
        else if (!strcmp(argv[i], "--radbc")) radbc = 1;
        else if (!strcmp(argv[i], "--perfect")) perfect = 1;
        else if (!strcmp(argv[i], "--kinematic")) kinematic = 1;
        else if (!strcmp(argv[i], "--dynamo")) dynamo = 1;
        else if (!strcmp(argv[i], "--no-dealias")) dalias = 0;
        else if (!strcmp(argv[i], "--split")) split = 1;
        else if (!strcmp(argv[i], "--eta-contrast") && i + 1 < argc) eta = atof(argv[++i]);
        else if (!strcmp(argv[i], "--noise") && i + 1 < argc) noise = atof(argv[++i]);
        else if (!strcmp(argv[i], "--input") && i + 1 < argc) input = argv[++i];
        else { fprintf(stderr, "unknown option %s\n", argv[i]); return 2; }
    }
    CHECK(vec_params_read_input(input, &p));
    if (p.nframe == 1) {
        /* parameters from restart.nc (src/netcdf.F90:591-713) */
        vec_snapshot s;
        memset(&s, 0, sizeof(s));
        CHECK(vec_nc_read("restart.nc", &s));
        p.gamma = s.gamma; p.sigma = s.sigma; p.theta = s.theta; p.ck = s.ck; p.cm = s.cm; p.f = s.f;
        p.tayl = s.tayl; p.psi = s.psi; p.zeta = s.zeta; p.xmax = s.xmax; p.ymax = s.ymax;
        p.nx = s.nx; p.ny = s.ny; p.nz = s.nz;
    }
    p.constflux = constflux; p.radbc = radbc; p.perfect = perfect; p.kinematic = kinematic;
    p.dynamo = dynamo; p.dalias = dalias; p.eta_contrast = eta; p.noise_amp = noise;
    p.precision = split ? VEC_PREC_SPLIT : VEC_PREC_FP64;

    printf(" ---------------------------------------------------\n");
    printf(" Simulations of compressible 3-D magnetoconvection  \n");
    printf(" ---------------------------------------------------\n");
    printf(" GB300 library, %s form\n", split ? "FP32-bulk / FP64-state" : "FP64");
    printf("    nx = %d  ny = %d  nz = %d\n", p.nx, p.ny, p.nz);
    printf("  GAMMA = %g SIGMA = %g THETA = %g CK = %.10g CM = %g F = %.10g\n", p.gamma, p.sigma, p.theta,
           p.ck, p.cm, p.f);
    printf("  ZETA = %g XMAX = %g YMAX = %g SF = %g NFRAME = %d ETA CONTRAST = %g\n", p.zeta, p.xmax, p.ymax,
           p.sf, p.nframe, p.eta_contrast);

    vec_ctx *ctx = NULL;
    CHECK(vec_create(&p, &ctx));
    if (p.nframe == 0) CHECK(vec_static(ctx));
    else CHECK(vec_read_restart(ctx, "restart.nc"));
    double dt;
    CHECK(vec_calcdt(ctx, &dt));
    printf(" Initial Timestep, dt = %.10e\n", dt);
    if (p.f != 0.0 || p.kinematic) CHECK(vec_mag_init(ctx));

    double t0 = now(), tsteps = 0.0;
    for (int nit = 1; nit <= p.ntotal; nit++) {
        double a = now();
        int st = vec_step(ctx, 1);
        if (st == VEC_ERR_DIVB) {
            vec_diag_out d;
            vec_last_diag(ctx, &d);
            printf(" ERROR: DIV B is not zero\n DIV B = %g\n", d.divbmax > -d.divbmin ? d.divbmax : -d.divbmin);
            vec_destroy(ctx);
            return 12;
        }
        CHECK(st);
        if (p.ndu06 > 0 && nit % p.ndu06 == 0) {
            vec_scalars s;
            vec_diag_out d;
            CHECK(vec_get_scalars(ctx, &s));
            CHECK(vec_last_diag(ctx, &d));
            printf("\n NIT= %d TTIME %.16e\n", nit, s.ttime);
            printf(" ubar= %.16e vbar= %.16e\n", d.ubar, d.vbar);
            printf(" divbmin= %.16e divbmax= %.16e\n", d.divbmin, d.divbmax);
            printf(" alfvenmin= %.16e alfvenmax= %.16e\n", d.alfvenmin, d.alfvenmax);
            printf(" machmin= %.16e machmax= %.16e\n", d.machmin, d.machmax);
            printf(" rmsmin= %.16e rmsmax= %.16e\n", d.rmsmin, d.rmsmax);
            printf(" rmin= %.16e rmax= %.16e\n tmin= %.16e tmax= %.16e\n", d.rmin, d.rmax, d.tmin, d.tmax);
            printf(" umin= %.16e umax= %.16e\n vmin= %.16e vmax= %.16e\n", d.umin, d.umax, d.vmin, d.vmax);
            printf(" wmin= %.16e wmax= %.16e\n", d.wmin, d.wmax);
            printf(" bxmin= %.16e bxmax= %.16e\n bymin= %.16e bymax= %.16e\n", d.bxmin, d.bxmax, d.bymin, d.bymax);
            printf(" bzmin= %.16e bzmax= %.16e\n\n", d.bzmin, d.bzmax);
            printf(" magenergy= %.16e\n kinenergy= %.16e\n Nusselt= %.16e\n", d.menergy, d.kenergy, d.nusselt);
            if (nit % 10 == 0) printf(" New value of dt %.16e\n", s.dt);
        }
        if (p.ndu16 > 0 && nit % p.ndu16 == 0) {
            /* src/main.F90:695-740: float by default, double at the end and
             * every ndurestart dumps */
            int iprec = 4;
            if (nit >= p.ntotal) iprec = 8;
            if (p.ndurestart > 0 && nit % (p.ndurestart * p.ndu16) == 0) iprec = 8;
            vec_scalars s;
            CHECK(vec_get_scalars(ctx, &s));
            int k = (s.iter / p.ndu16) % 1000;
            char name[32];
            snprintf(name, sizeof name, "T16_%c%c%c.nc", '0' + k / 100, '0' + (k % 100) / 10, '0' + k % 10);
            CHECK(vec_write_snapshot(ctx, name, iprec, "Created by p3d_gpu (GB300)"));
        }
        tsteps += now() - a;
    }
    CHECK(vec_sync(ctx));
    double total = now() - t0;
    printf(" %d steps, %.3f s, %.4e grid-point-steps/s\n", p.ntotal, total,
           (double)p.nx * p.ny * p.nz * p.ntotal / total);
    (void)tsteps;
    vec_destroy(ctx);
    return 0;
}
