/*
 * p3d_oracle.h -- CPU restatement of the VarElecCond (p3d) serial time-step
 * path.  TEST INFRASTRUCTURE ONLY: this is the parity checker for the CUDA
 * library and the timed CPU baseline; no product code links it.
 *
 * Every routine follows the serial branch (nproc=1, izstart=1,
 * nlayer=nz) of the reference file:line cited beside it.  Arrays are
 * double[nx*ny*nz], x fastest (the Fortran (nx,ny,nz) layout).
 */
#ifndef P3D_ORACLE_H
#define P3D_ORACLE_H

#include "../include/vec.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_ctx or_ctx;

or_ctx *or_create(const vec_params *p, int *status);
void or_destroy(or_ctx *c);
int or_nthreads(int n);                  /* set OpenMP threads (<=0: query) */

/* raw FFTW-2 style transforms of one line (unnormalised, halfcomplex) */
int or_r2hc(int n, const double *in, double *out);
int or_hc2r(int n, const double *in, double *out);

/* state access (field ids of vec.h) */
int or_field(or_ctx *c, int field, double *dst, const double *src);
int or_mean(or_ctx *c, int mean, double *dst, const double *src);
int or_scalars(or_ctx *c, vec_scalars *dst, const vec_scalars *src);
double or_bzbar(or_ctx *c, const double *set);

/* set-up */
int or_static(or_ctx *c);
int or_mag_init(or_ctx *c);
int or_calcdt(or_ctx *c, double *dt);

/* operators (caller arrays) */
int or_d1bydx(or_ctx *c, const double *fin, double *fout);
int or_d1bydy(or_ctx *c, const double *fin, double *fout);
int or_d2bydx(or_ctx *c, const double *fin, double *f1, double *f2);
int or_d2bydy(or_ctx *c, const double *fin, double *f1, double *f2);
int or_dealias(or_ctx *c, double *z);
int or_forwardfft(or_ctx *c, const double *fin, double *fout);
int or_inversefft(or_ctx *c, const double *fin, double *fout);
int or_d1bydz(or_ctx *c, const double *fin, double *fout, int dflag);
int or_d1upbydz(or_ctx *c, const double *fin, double *fout, int dflag);
int or_d2bydz(or_ctx *c, const double *fin, double *fout, int dflag);
int or_d1bydz1d(or_ctx *c, const double *fin, double *fout, int dflag);
int or_d2bydz1d(or_ctx *c, const double *fin, double *fout, int dflag);

/* physics on the context state */
int or_hydro_deriv(or_ctx *c);
int or_mag_deriv(or_ctx *c);
int or_bandj(or_ctx *c);
int or_magdealias(or_ctx *c);
int or_boundary(or_ctx *c);
int or_mag_boundary(or_ctx *c);
int or_ab3_update(or_ctx *c);
int or_diag(or_ctx *c, vec_diag_out *out);
int or_step(or_ctx *c, int nsteps);
int or_last_diag(or_ctx *c, vec_diag_out *out);

#ifdef __cplusplus
}
#endif
#endif
