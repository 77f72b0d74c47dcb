/*
 * p3d_oracle.c -- CPU restatement of the VarElecCond (p3d) serial path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA
 * library (tests/, __graft_entry__.smoke) and the timed CPU baseline of
 * bench.py.  It is never linked into, called by, or a fallback of the
 * product library.
 *
 * It restates, in the same order of arithmetic where that is practical,
 * the serial branches (nproc=1, izstart=1, izfinish=nz, nlayer=nz) of:
 *   src/fft.F90, src/dbydz.F90, src/hydro_deriv.f90, src/magnetic.f90,
 *   src/main.F90 (time loop), src/utils.F90, src/initial.F90 (static),
 *   src/ranset.f90, src/constants.f90, src/trans_params.f90.
 * Paths are relative to the reference's VarElecCond/ directory.
 *
 * FFTW 2.x (2.1.5, named in Makefile:33) is not available; its rfftw
 * real<->halfcomplex transforms are restated from FFTW's documented
 * definition: forward X_k = sum_j x_j exp(-2 pi i jk/n), backward
 * x_j = sum_k X_k exp(+2 pi i jk/n), both unnormalised; halfcomplex order
 * r0, r1, ..., r_{n/2}, i_{(n+1)/2-1}, ..., i1.  The restatement uses a
 * mixed-radix decimation-in-time complex FFT on two real lines at once.
 *
 * The eta(z) induction extension (eta_contrast != 1) has no reference
 * counterpart; with eta_contrast == 1 every expression reduces to the
 * reference one, operation for operation.
 */
#include "p3d_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double re, im; } cpx;

#define MAXN 4096
#define MAXF 32

typedef struct {
    int n, nf, fac[MAXF];
    double *cs, *sn;          /* cos/sin(2 pi e / n), e = 0..n-1 */
} fftplan;

struct or_ctx {
    vec_params p;
    int nx, ny, nz;
    size_t np, n;             /* plane size, total size */
    /* src/constants.f90:21-49 */
    double dx, dy, dz, dd, xn, xzn, taylt, cpsi, spsi, cor;
    double gck, sck, zck, scko3, sckg, fzckg, thmplus1, fo2, g1, gm1, nusstmp;
    double dtvisc0x, dtvisc0z, dtdiff0x, dtdiff0z;
    double ho12, sc1;          /* src/dbydz.F90:355-362 */
    /* src/fft.F90:60-80 */
    double *akx1, *akx2, *aky1, *aky2;
    int icutoffx, icutoffy;
    fftplan px, py;
    /* src/trans_params.f90 and the eta(z) extension */
    double *kappa, *dkappa, *eta, *deta;
    /* src/arrays.f90:14-74 */
    double *r, *t, *u, *v, *w, *bx, *by, *bz, *jsq, *pol, *tor;
    double *rdot[3], *tdot[3], *udot[3], *vdot[3], *wdot[3], *poldot[3], *tordot[3];
    double *wk1, *wk2, *wk3, *wk4, *ex, *ey, *ez;
    double *bxbar, *bybar, *bxbardot[3], *bybardot[3], *wk1_1d, *wk2_1d, *tmp1d;
    double bzbar;
    /* src/main.F90:84-103 + control.f90 */
    double dt, dt1, dt2, ttime;
    int iter, nit, first, second;
    vec_diag_out last;
};

/* ===================================================================== */
/* twiddles: exact at multiples of n/4                                    */
/* ===================================================================== */
static void sincos2pi(long e, long n, double *c, double *s)
{
    e %= n;
    if (e < 0) e += n;
    long q = (4 * e) / n;            /* quadrant */
    long r = 4 * e - q * n;          /* remainder, angle = (pi/2) r/n */
    double cf, sf;
    if (2 * r <= n) {
        double a = (M_PI / 2.0) * ((double)r / (double)n);
        cf = cos(a); sf = sin(a);
    } else {
        double a = (M_PI / 2.0) * ((double)(n - r) / (double)n);
        cf = sin(a); sf = cos(a);
    }
    switch (q) {
    case 0: *c = cf;  *s = sf;  break;
    case 1: *c = -sf; *s = cf;  break;
    case 2: *c = -cf; *s = -sf; break;
    default: *c = sf; *s = -cf; break;
    }
}

static int plan_init(fftplan *pl, int n)
{
    pl->n = n;
    pl->nf = 0;
    int m = n;
    while (m % 4 == 0) { pl->fac[pl->nf++] = 4; m /= 4; }
    while (m % 2 == 0) { pl->fac[pl->nf++] = 2; m /= 2; }
    for (int p = 3; m > 1; p += 2)
        while (m % p == 0) { pl->fac[pl->nf++] = p; m /= p; }
    for (int i = 0; i < pl->nf; i++)
        if (pl->fac[i] > 64) return -32;   /* radix buffer limit */
    pl->cs = (double *)malloc(sizeof(double) * n);
    pl->sn = (double *)malloc(sizeof(double) * n);
    if (!pl->cs || !pl->sn) return -5;
    for (int e = 0; e < n; e++) sincos2pi(e, n, &pl->cs[e], &pl->sn[e]);
    return 0;
}

static void plan_free(fftplan *pl) { free(pl->cs); free(pl->sn); }

/* out[0..n) = DFT_sign of x[0], x[s], ..., x[(n-1)s]; tw = N/n */
static void fft_rec(const fftplan *pl, int n, int f, const cpx *x, int s,
                    cpx *out, int sign, int tw)
{
    if (n == 1) { out[0] = x[0]; return; }
    const int N = pl->n;
    int p = pl->fac[f], m = n / p;
    for (int q = 0; q < p; q++)
        fft_rec(pl, m, f + 1, x + (size_t)q * s, s * p, out + (size_t)q * m, sign, tw * p);
    double sg = (double)sign;
    for (int k = 0; k < m; k++) {
        cpx t[64];
        t[0] = out[k];
        for (int q = 1; q < p; q++) {
            long e = ((long)q * k * tw) % N;
            double c = pl->cs[e], sn = sg * pl->sn[e];
            cpx y = out[(size_t)q * m + k];
            t[q].re = y.re * c - y.im * sn;
            t[q].im = y.re * sn + y.im * c;
        }
        if (p == 2) {
            out[k].re = t[0].re + t[1].re;      out[k].im = t[0].im + t[1].im;
            out[k + m].re = t[0].re - t[1].re;  out[k + m].im = t[0].im - t[1].im;
        } else if (p == 4) {
            /* W4^1 = sign*i */
            cpx a0 = { t[0].re + t[2].re, t[0].im + t[2].im };
            cpx a1 = { t[0].re - t[2].re, t[0].im - t[2].im };
            cpx b0 = { t[1].re + t[3].re, t[1].im + t[3].im };
            cpx b1 = { t[1].re - t[3].re, t[1].im - t[3].im };
            /* i*sign*b1 */
            cpx ib1 = { -sg * b1.im, sg * b1.re };
            out[k].re = a0.re + b0.re;          out[k].im = a0.im + b0.im;
            out[k + m].re = a1.re + ib1.re;     out[k + m].im = a1.im + ib1.im;
            out[k + 2 * m].re = a0.re - b0.re;  out[k + 2 * m].im = a0.im - b0.im;
            out[k + 3 * m].re = a1.re - ib1.re; out[k + 3 * m].im = a1.im - ib1.im;
        } else {
            for (int so = 0; so < p; so++) {
                double ar = 0.0, ai = 0.0;
                for (int q = 0; q < p; q++) {
                    long e = (((long)q * so) % p) * (N / p);
                    double c = pl->cs[e], sn = sg * pl->sn[e];
                    ar += t[q].re * c - t[q].im * sn;
                    ai += t[q].re * sn + t[q].im * c;
                }
                out[k + (size_t)m * so].re = ar;
                out[k + (size_t)m * so].im = ai;
            }
        }
    }
}

/* forward real transform of two lines a,b (b may be NULL) -> halfcomplex */
static void r2hc_pair(const fftplan *pl, const double *a, const double *b,
                      double *ha, double *hb, cpx *z, cpx *Z)
{
    const int n = pl->n;
    for (int j = 0; j < n; j++) { z[j].re = a[j]; z[j].im = b ? b[j] : 0.0; }
    fft_rec(pl, n, 0, z, 1, Z, -1, 1);
    ha[0] = Z[0].re;
    if (hb) hb[0] = Z[0].im;
    for (int k = 1; k <= n / 2; k++) {
        cpx zk = Z[k], wk = Z[(n - k) % n];
        double are = 0.5 * (zk.re + wk.re), aim = 0.5 * (zk.im - wk.im);
        double bre = 0.5 * (zk.im + wk.im), bim = 0.5 * (wk.re - zk.re);
        ha[k] = are;
        if (hb) hb[k] = bre;
        if (k < n - k) {
            ha[n - k] = aim;
            if (hb) hb[n - k] = bim;
        }
    }
}

/* backward real transform (unnormalised) of two halfcomplex lines */
static void hc2r_pair(const fftplan *pl, const double *ha, const double *hb,
                      double *a, double *b, cpx *z, cpx *Z)
{
    const int n = pl->n;
    for (int k = 0; k < n; k++) {
        double ar, ai, br = 0.0, bi = 0.0;
        int kk = k <= n / 2 ? k : n - k;
        double sgn = k <= n / 2 ? 1.0 : -1.0;
        ar = ha[kk];
        ai = (kk == 0 || 2 * kk == n) ? 0.0 : sgn * ha[n - kk];
        if (hb) {
            br = hb[kk];
            bi = (kk == 0 || 2 * kk == n) ? 0.0 : sgn * hb[n - kk];
        }
        Z[k].re = ar - bi;
        Z[k].im = ai + br;
    }
    fft_rec(pl, n, 0, Z, 1, z, +1, 1);
    for (int j = 0; j < n; j++) {
        a[j] = z[j].re;
        if (b) b[j] = z[j].im;
    }
}

int or_r2hc(int n, const double *in, double *out)
{
    if (n < 1 || n > MAXN) return -31;
    fftplan pl;
    if (plan_init(&pl, n)) return -5;
    cpx *z = malloc(sizeof(cpx) * n), *Z = malloc(sizeof(cpx) * n);
    r2hc_pair(&pl, in, NULL, out, NULL, z, Z);
    free(z); free(Z); plan_free(&pl);
    return 0;
}

int or_hc2r(int n, const double *in, double *out)
{
    if (n < 1 || n > MAXN) return -31;
    fftplan pl;
    if (plan_init(&pl, n)) return -5;
    cpx *z = malloc(sizeof(cpx) * n), *Z = malloc(sizeof(cpx) * n);
    hc2r_pair(&pl, in, NULL, out, NULL, z, Z);
    free(z); free(Z); plan_free(&pl);
    return 0;
}

int or_nthreads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* ===================================================================== */
/* line transforms over a whole (nx,ny,nz) array                          */
/* dir 0: x lines (contiguous), dir 1: y lines (stride nx)                 */
/* ===================================================================== */
typedef enum { SP_NONE, SP_D1, SP_D2, SP_DEALIAS } spop;

/* spectral operation on one halfcomplex line h (length n) */
static void apply_spec(spop op, int n, double *h, const double *k1,
                       const double *k2, int icut)
{
    switch (op) {
    case SP_NONE: break;
    case SP_D1:   /* src/fft.F90:292-302 */
        h[0] = 0.0;
        h[n / 2] = 0.0;
        for (int i = 1; i <= n / 2 - 1; i++) {
            double fac = h[i];
            h[i] = -h[n - i] * k1[i];
            h[n - i] = fac * k1[n - i];
        }
        break;
    case SP_D2:   /* second-derivative half of src/fft.F90:442-454 */
        h[0] = 0.0;
        for (int i = 1; i <= n / 2 - 1; i++) {
            h[i] = h[i] * k2[i];
            h[n - i] = h[n - i] * k2[n - i];
        }
        h[n / 2] = h[n / 2] * k2[n / 2];
        break;
    case SP_DEALIAS:  /* src/fft.F90:618-626 */
        for (int i = 1; i <= icut; i++) {
            h[n / 2 + i] = 0.0;
            h[n / 2 - i] = 0.0;
        }
        h[n / 2] = 0.0;
        break;
    }
}

/*
 * For every line along dir: out1 = inv(op1(fwd(in)))/n and, if out2,
 * out2 = inv(op2(fwd(in)))/n.  With fwd_only, out1 = fwd(in) (no
 * normalisation); with inv_only, out1 = inv(in)/n.
 */
static void line_pass(or_ctx *c, int dir, const double *in, double *out1, spop op1,
                      double *out2, spop op2, int fwd_only, int inv_only)
{
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    const int n = dir == 0 ? nx : ny;
    const int nl = dir == 0 ? ny : nx;   /* lines per plane */
    const fftplan *pl = dir == 0 ? &c->px : &c->py;
    const double *k1 = dir == 0 ? c->akx1 : c->aky1;
    const double *k2 = dir == 0 ? c->akx2 : c->aky2;
    const int icut = dir == 0 ? c->icutoffx : c->icutoffy;
    const double dn = (double)n;
    const size_t stride = dir == 0 ? 1 : (size_t)nx;
    const size_t lstep = dir == 0 ? (size_t)nx : 1;

#pragma omp parallel
    {
        cpx *z = malloc(sizeof(cpx) * n), *Z = malloc(sizeof(cpx) * n);
        double *a = malloc(sizeof(double) * n * 6);
        double *b = a + n, *ha = a + 2 * n, *hb = a + 3 * n, *ga = a + 4 * n, *gb = a + 5 * n;
#pragma omp for collapse(2) schedule(static)
        for (int k = 0; k < nz; k++) {
            for (int l0 = 0; l0 < nl; l0 += 2) {
                int two = (l0 + 1 < nl);
                size_t base0 = (size_t)k * c->np + (size_t)l0 * lstep;
                size_t base1 = base0 + lstep;
                for (int q = 0; q < n; q++) {
                    a[q] = in[base0 + q * stride];
                    if (two) b[q] = in[base1 + q * stride];
                }
                if (fwd_only) {
                    r2hc_pair(pl, a, two ? b : NULL, ha, hb, z, Z);
                    for (int q = 0; q < n; q++) {
                        out1[base0 + q * stride] = ha[q];
                        if (two) out1[base1 + q * stride] = hb[q];
                    }
                    continue;
                }
                if (inv_only) {
                    hc2r_pair(pl, a, two ? b : NULL, ha, hb, z, Z);
                    for (int q = 0; q < n; q++) {
                        out1[base0 + q * stride] = ha[q] / dn;
                        if (two) out1[base1 + q * stride] = hb[q] / dn;
                    }
                    continue;
                }
                r2hc_pair(pl, a, two ? b : NULL, ha, hb, z, Z);
                if (out2) {
                    memcpy(ga, ha, sizeof(double) * n);
                    memcpy(gb, hb, sizeof(double) * n);
                    apply_spec(op2, n, ga, k1, k2, icut);
                    if (two) apply_spec(op2, n, gb, k1, k2, icut);
                }
                apply_spec(op1, n, ha, k1, k2, icut);
                if (two) apply_spec(op1, n, hb, k1, k2, icut);
                hc2r_pair(pl, ha, two ? hb : NULL, a, b, z, Z);
                for (int q = 0; q < n; q++) {
                    out1[base0 + q * stride] = a[q] / dn;
                    if (two) out1[base1 + q * stride] = b[q] / dn;
                }
                if (out2) {
                    hc2r_pair(pl, ga, two ? gb : NULL, a, b, z, Z);
                    for (int q = 0; q < n; q++) {
                        out2[base0 + q * stride] = a[q] / dn;
                        if (two) out2[base1 + q * stride] = b[q] / dn;
                    }
                }
            }
        }
        free(z); free(Z); free(a);
    }
}

/* src/fft.F90:255-324 */
int or_d1bydx(or_ctx *c, const double *fin, double *fout)
{ line_pass(c, 0, fin, fout, SP_D1, NULL, SP_NONE, 0, 0); return 0; }
/* src/fft.F90:329-398 */
int or_d1bydy(or_ctx *c, const double *fin, double *fout)
{ line_pass(c, 1, fin, fout, SP_D1, NULL, SP_NONE, 0, 0); return 0; }
/* src/fft.F90:403-489 */
int or_d2bydx(or_ctx *c, const double *fin, double *f1, double *f2)
{ line_pass(c, 0, fin, f1, SP_D1, f2, SP_D2, 0, 0); return 0; }
/* src/fft.F90:495-581 */
int or_d2bydy(or_ctx *c, const double *fin, double *f1, double *f2)
{ line_pass(c, 1, fin, f1, SP_D1, f2, SP_D2, 0, 0); return 0; }
/* src/fft.F90:586-682: x then y */
int or_dealias(or_ctx *c, double *z)
{
    line_pass(c, 0, z, z, SP_DEALIAS, NULL, SP_NONE, 0, 0);
    line_pass(c, 1, z, z, SP_DEALIAS, NULL, SP_NONE, 0, 0);
    return 0;
}
/* src/fft.F90:687-735: x (out of place) then y (in place) */
int or_forwardfft(or_ctx *c, const double *fin, double *fout)
{
    line_pass(c, 0, fin, fout, SP_NONE, NULL, SP_NONE, 1, 0);
    line_pass(c, 1, fout, fout, SP_NONE, NULL, SP_NONE, 1, 0);
    return 0;
}
/* src/fft.F90:740-799: x inverse /nx then y inverse /ny */
int or_inversefft(or_ctx *c, const double *fin, double *fout)
{
    line_pass(c, 0, fin, fout, SP_NONE, NULL, SP_NONE, 0, 1);
    line_pass(c, 1, fout, fout, SP_NONE, NULL, SP_NONE, 0, 1);
    return 0;
}

/* ===================================================================== */
/* z finite differences, src/dbydz.F90 (Appendix of stencils)             */
/* ===================================================================== */
#define AT(f, k) ((f) + (size_t)(k) * np)   /* plane k (0-based) */

static int d1_flag_ok(int f) { return f == 0 || f == 1 || f == 2 || f == 5; }

/* topdz :927, row k=1; flags 0/2 -> 0, 1 -> 14,36,-18,4; 5 -> -22,36,-18,4 */
static inline double topdz(double h, int fl, double f1, double f2, double f3, double f4)
{
    if (fl == 1) return h * (14.0 * f1 + 36.0 * f2 - 18.0 * f3 + 4.0 * f4);
    if (fl == 5) return h * (-22.0 * f1 + 36.0 * f2 - 18.0 * f3 + 4.0 * f4);
    return 0.0;
}
/* topdz_low :1053 (all flags) */
static inline double topdz_low(double h, double f1, double f2, double f3, double f4)
{ return h * (-4.0 * f1 - 6.0 * f2 + 12.0 * f3 - 2.0 * f4); }
/* interior :371 */
static inline double interior(double h, double fm2, double fm1, double fp1, double fp2)
{ return h * (fm2 - 8.0 * fm1 + 8.0 * fp1 - fp2); }
/* lastdz_up :776 (all flags) */
static inline double lastdz_up(double h, double f0, double fm1, double fm2, double fm3)
{ return h * (4.0 * f0 + 6.0 * fm1 - 12.0 * fm2 + 2.0 * fm3); }
/* lastdz :626 */
static inline double lastdz(double h, int fl, double f0, double fm1, double fm2, double fm3)
{
    if (fl == 1) return h * (-14.0 * f0 - 36.0 * fm1 + 18.0 * fm2 - 4.0 * fm3);
    if (fl == 5) return h * (22.0 * f0 - 36.0 * fm1 + 18.0 * fm2 - 4.0 * fm3);
    return 0.0;
}
/* dupinterior :485 */
static inline double dupinterior(double h, double wv, double fm3, double fm2, double fm1,
                                 double f0, double fp1, double fp2, double fp3)
{
    if (wv >= 0.0)
        return h * (-fm3 + 6.0 * fm2 - 18.0 * fm1 + 10.0 * f0 + 3.0 * fp1);
    return h * (fp3 - 6.0 * fp2 + 18.0 * fp1 - 10.0 * f0 - 3.0 * fm1);
}
/* dup_up :532 */
static inline double dup_up(double h, double wv, double fm2, double fm1, double f0,
                            double fp1, double fp2, double fp3)
{
    if (wv >= 0.0)
        return h * (2.0 * fm2 - 12.0 * fm1 + 6.0 * f0 + 4.0 * fp1);
    return h * (fp3 - 6.0 * fp2 + 18.0 * fp1 - 10.0 * f0 - 3.0 * fm1);
}
/* dup_low :579 */
static inline double dup_low(double h, double wv, double fm3, double fm2, double fm1,
                             double f0, double fp1, double fp2)
{
    if (wv >= 0.0)
        return h * (-fm3 + 6.0 * fm2 - 18.0 * fm1 + 10.0 * f0 + 3.0 * fp1);
    return h * (-2.0 * fp2 + 12.0 * fp1 - 6.0 * f0 - 4.0 * fm1);
}
/* d2topdz :1368 (flags 0, 3) */
static inline double d2topdz(double s, int fl, double f0, double f1, double f2, double f3,
                             double f4, double f5)
{
    if (fl == 3)
        return s * (45.0 * f0 - 154.0 * f1 + 214.0 * f2 - 156.0 * f3 + 61.0 * f4 - 10.0 * f5);
    return 0.0;
}
/* d2topdz_low :1462 / d2lastdz_up :1271 (all flags) */
static inline double d2edge_low(double s, double f0, double f1, double f2, double f3,
                                double f4, double f5)
{ return s * (10.0 * f0 - 15.0 * f1 - 4.0 * f2 + 14.0 * f3 - 6.0 * f4 + f5); }
/* d2interior :428 */
static inline double d2interior(double s, double fm2, double fm1, double f0, double fp1,
                                double fp2)
{ return s * (-fm2 + 16.0 * fm1 - 30.0 * f0 + 16.0 * fp1 - fp2); }

/* d1bydz serial branch, src/dbydz.F90:1685-1751 */
static int d1z_core(int nz, size_t np, double h, const double *fin, double *fout, int fl)
{
    if (!d1_flag_ok(fl)) return VEC_ERR_FLAG;
    if (nz < 6) return VEC_ERR_NZ;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; k++) {
        for (size_t q = 0; q < np; q++) {
#define F(kk) fin[(size_t)(kk) * np + q]
            double o;
            if (k == 0) o = topdz(h, fl, F(0), F(1), F(2), F(3));
            else if (k == 1) o = topdz_low(h, F(0), F(1), F(2), F(3));
            else if (k == nz - 2) o = lastdz_up(h, F(nz - 1), F(nz - 2), F(nz - 3), F(nz - 4));
            else if (k == nz - 1) o = lastdz(h, fl, F(nz - 1), F(nz - 2), F(nz - 3), F(nz - 4));
            else o = interior(h, F(k - 2), F(k - 1), F(k + 1), F(k + 2));
            fout[(size_t)k * np + q] = o;
#undef F
        }
    }
    return 0;
}

/* d1upbydz serial branch, src/dbydz.F90:2353-2424 (+ bottom rows) */
static int d1up_core(int nz, size_t np, double h, const double *fin, double *fout, int fl,
                     const double *w)
{
    if (!d1_flag_ok(fl)) return VEC_ERR_FLAG;
    if (nz < 6) return VEC_ERR_NZ;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; k++) {
        for (size_t q = 0; q < np; q++) {
#define F(kk) fin[(size_t)(kk) * np + q]
            double wv = w[(size_t)k * np + q];
            double o;
            if (k == 0) o = topdz(h, fl, F(0), F(1), F(2), F(3));
            else if (k == 1) o = topdz_low(h, F(0), F(1), F(2), F(3));
            else if (k == 2) o = dup_up(h, wv, F(0), F(1), F(2), F(3), F(4), F(5));
            else if (k == nz - 3)
                o = dup_low(h, wv, F(nz - 6), F(nz - 5), F(nz - 4), F(nz - 3), F(nz - 2), F(nz - 1));
            else if (k == nz - 2) o = lastdz_up(h, F(nz - 1), F(nz - 2), F(nz - 3), F(nz - 4));
            else if (k == nz - 1) o = lastdz(h, fl, F(nz - 1), F(nz - 2), F(nz - 3), F(nz - 4));
            else o = dupinterior(h, wv, F(k - 3), F(k - 2), F(k - 1), F(k), F(k + 1), F(k + 2), F(k + 3));
            fout[(size_t)k * np + q] = o;
#undef F
        }
    }
    return 0;
}

/* d2bydz serial branch, src/dbydz.F90:3007-3083 */
static int d2z_core(int nz, size_t np, double s, const double *fin, double *fout, int fl)
{
    if (fl != 0 && fl != 3) return VEC_ERR_FLAG;
    if (nz < 6) return VEC_ERR_NZ;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; k++) {
        for (size_t q = 0; q < np; q++) {
#define F(kk) fin[(size_t)(kk) * np + q]
            double o;
            if (k == 0) o = d2topdz(s, fl, F(0), F(1), F(2), F(3), F(4), F(5));
            else if (k == 1) o = d2edge_low(s, F(0), F(1), F(2), F(3), F(4), F(5));
            else if (k == nz - 2)
                o = d2edge_low(s, F(nz - 1), F(nz - 2), F(nz - 3), F(nz - 4), F(nz - 5), F(nz - 6));
            else if (k == nz - 1)
                o = d2topdz(s, fl, F(nz - 1), F(nz - 2), F(nz - 3), F(nz - 4), F(nz - 5), F(nz - 6));
            else o = d2interior(s, F(k - 2), F(k - 1), F(k), F(k + 1), F(k + 2));
            fout[(size_t)k * np + q] = o;
#undef F
        }
    }
    return 0;
}

int or_d1bydz(or_ctx *c, const double *fin, double *fout, int dflag)
{ return d1z_core(c->nz, c->np, c->ho12, fin, fout, dflag); }
int or_d1upbydz(or_ctx *c, const double *fin, double *fout, int dflag)
{ return d1up_core(c->nz, c->np, c->ho12, fin, fout, dflag, c->w); }
int or_d2bydz(or_ctx *c, const double *fin, double *fout, int dflag)
{ return d2z_core(c->nz, c->np, c->sc1, fin, fout, dflag); }
/* d1bydz1D :1922 and d2bydz1D :3306 use the same stencils on nz values */
int or_d1bydz1d(or_ctx *c, const double *fin, double *fout, int dflag)
{ return d1z_core(c->nz, 1, c->ho12, fin, fout, dflag); }
int or_d2bydz1d(or_ctx *c, const double *fin, double *fout, int dflag)
{ return d2z_core(c->nz, 1, c->sc1, fin, fout, dflag); }

/* ===================================================================== */
/* context                                                                */
/* ===================================================================== */
static double *dalloc(size_t n)
{
    double *p = (double *)calloc(n ? n : 1, sizeof(double));
    return p;
}

/* src/constants.f90:56-109 and src/dbydz.F90:355-362 */
static void set_constants(or_ctx *c)
{
    const vec_params *p = &c->p;
    c->dx = p->xmax / (double)c->nx;
    c->dy = p->ymax / (double)c->ny;
    c->dz = 1.0 / (double)(c->nz - 1);
    c->dd = c->dx < c->dy ? c->dx : c->dy;
    c->xn = 1.0 / (double)(c->nx * c->ny);
    c->xzn = c->dx * c->dy * c->dz;
    c->taylt = p->tayl / pow(1.0 + p->theta / 2.0, 2.0 * p->cm);
    c->cpsi = cos(p->psi);
    c->spsi = sin(p->psi);
    c->cor = p->ck * p->sigma * sqrt(c->taylt);
    c->gck = p->gamma * p->ck;
    c->sck = p->sigma * p->ck;
    c->zck = p->zeta * p->ck;
    c->scko3 = c->sck / 3.0;
    c->sckg = p->sigma * p->ck * (p->gamma - 1.0);
    c->fzckg = p->f * p->zeta * p->ck * (p->gamma - 1.0);
    c->thmplus1 = p->theta * (p->cm + 1.0);
    c->fo2 = p->f / 2.0;
    c->g1 = sqrt(p->gamma);
    c->gm1 = p->gamma - 1.0;
    c->nusstmp = p->theta * (p->cm + 1.0) * (1.0 - (1.0 / p->gamma));
    c->dtvisc0x = 0.1 * 0.75 * c->dd * c->dd / p->sigma / p->ck;
    c->dtvisc0z = 0.2 * c->dz * c->dz / p->sigma / p->ck * (1.0 + p->theta / 7.0);
    c->dtdiff0x = 0.1 * c->dd * c->dd / p->gamma / p->ck;
    c->dtdiff0z = 0.2 * c->dz * c->dz / p->gamma / p->ck * (1.0 + p->theta / 7.0);
    c->ho12 = (double)(c->nz - 1) / 12.0;
    c->sc1 = (double)((c->nz - 1) * (c->nz - 1)) / 12.0;
}

/* src/fft.F90:171-221 */
static void init_wavenumbers(or_ctx *c)
{
    const int nx = c->nx, ny = c->ny;
    c->icutoffx = (nx / 2) / 3;
    c->icutoffy = (ny / 2) / 3;
    double cx = 8.0 * atan(1.0) / c->p.xmax;
    double cy = 8.0 * atan(1.0) / c->p.ymax;
    for (int i = 1; i <= nx / 2 - 1; i++) {
        c->akx1[i] = (double)i * cx;
        c->akx1[nx - i] = (double)i * cx;
        c->akx2[i] = -(double)i * (double)i * cx * cx;
        c->akx2[nx - i] = -(double)i * (double)i * cx * cx;
    }
    c->akx2[nx / 2] = -(double)(nx / 2) * (double)(nx / 2) * cx * cx;
    for (int i = 1; i <= ny / 2 - 1; i++) {
        c->aky1[i] = (double)i * cy;
        c->aky1[ny - i] = (double)i * cy;
        c->aky2[i] = -(double)i * (double)i * cy * cy;
        c->aky2[ny - i] = -(double)i * (double)i * cy * cy;
    }
    c->aky2[ny / 2] = -(double)(ny / 2) * (double)(ny / 2) * cy * cy;
}

/* src/trans_params.f90:15-69 plus eta(z) = zck (1 + (contrast-1) z) */
static void ini_trans_params(or_ctx *c)
{
    const double constA = 10.0;
    for (int k = 0; k < c->nz; k++) {
        double z = (double)k * c->dz;
        if (c->p.kappa_uniform) {
            c->kappa[k] = 1.0;
            c->dkappa[k] = 0.0;
        } else {
            double constB = constA * (z - 5.0e-1);
            c->kappa[k] = 5.0e-1 * (tanh(constB) + 1);
            c->dkappa[k] = 5.0e-1 * constA * pow(cosh(constB), -2.0);
        }
        double ec = c->p.eta_contrast;
        c->eta[k] = c->zck * (1.0 + (ec - 1.0) * z);
        c->deta[k] = c->zck * (ec - 1.0);
    }
}

or_ctx *or_create(const vec_params *p, int *status)
{
    int st = 0;
    if (p->nx < 4 || p->nx % 2) st = VEC_ERR_NX;
    else if (p->ny < 4 || p->ny % 2) st = VEC_ERR_NY;
    else if (p->nz < 6) st = VEC_ERR_NZ;
    else if (p->nx > MAXN || p->ny > MAXN) st = VEC_ERR_SIZE;
    if (st) { if (status) *status = st; return NULL; }
    or_ctx *c = (or_ctx *)calloc(1, sizeof(or_ctx));
    c->p = *p;
    c->nx = p->nx; c->ny = p->ny; c->nz = p->nz;
    c->np = (size_t)c->nx * c->ny;
    c->n = c->np * c->nz;
    set_constants(c);
    c->akx1 = dalloc(c->nx); c->akx2 = dalloc(c->nx);
    c->aky1 = dalloc(c->ny); c->aky2 = dalloc(c->ny);
    init_wavenumbers(c);
    if (plan_init(&c->px, c->nx) || plan_init(&c->py, c->ny)) st = VEC_ERR_ALLOC;
    c->kappa = dalloc(c->nz); c->dkappa = dalloc(c->nz);
    c->eta = dalloc(c->nz); c->deta = dalloc(c->nz);
    ini_trans_params(c);
    double **f3[] = { &c->r, &c->t, &c->u, &c->v, &c->w, &c->bx, &c->by, &c->bz, &c->jsq,
                      &c->pol, &c->tor, &c->wk1, &c->wk2, &c->wk3, &c->wk4, &c->ex,
                      &c->ey, &c->ez };
    for (size_t i = 0; i < sizeof(f3) / sizeof(f3[0]); i++)
        if (!(*f3[i] = dalloc(c->n))) st = VEC_ERR_ALLOC;
    for (int s = 0; s < 3; s++) {
        c->rdot[s] = dalloc(c->n); c->tdot[s] = dalloc(c->n); c->udot[s] = dalloc(c->n);
        c->vdot[s] = dalloc(c->n); c->wdot[s] = dalloc(c->n);
        c->poldot[s] = dalloc(c->n); c->tordot[s] = dalloc(c->n);
        if (!c->rdot[s] || !c->tdot[s] || !c->udot[s] || !c->vdot[s] || !c->wdot[s] ||
            !c->poldot[s] || !c->tordot[s]) st = VEC_ERR_ALLOC;
        c->bxbardot[s] = dalloc(c->nz); c->bybardot[s] = dalloc(c->nz);
    }
    c->bxbar = dalloc(c->nz); c->bybar = dalloc(c->nz);
    c->wk1_1d = dalloc(c->nz); c->wk2_1d = dalloc(c->nz); c->tmp1d = dalloc(2 * (size_t)c->nz);
    c->first = 1; c->second = 0;
    if (st) { or_destroy(c); if (status) *status = st; return NULL; }
    if (status) *status = 0;
    return c;
}

void or_destroy(or_ctx *c)
{
    if (!c) return;
    double *all[] = { c->akx1, c->akx2, c->aky1, c->aky2, c->kappa, c->dkappa, c->eta,
                      c->deta, c->r, c->t, c->u, c->v, c->w, c->bx, c->by, c->bz, c->jsq,
                      c->pol, c->tor, c->wk1, c->wk2, c->wk3, c->wk4, c->ex, c->ey, c->ez,
                      c->bxbar, c->bybar, c->wk1_1d, c->wk2_1d, c->tmp1d };
    for (size_t i = 0; i < sizeof(all) / sizeof(all[0]); i++) free(all[i]);
    for (int s = 0; s < 3; s++) {
        free(c->rdot[s]); free(c->tdot[s]); free(c->udot[s]); free(c->vdot[s]);
        free(c->wdot[s]); free(c->poldot[s]); free(c->tordot[s]);
        free(c->bxbardot[s]); free(c->bybardot[s]);
    }
    if (c->px.cs) plan_free(&c->px);
    if (c->py.cs) plan_free(&c->py);
    free(c);
}

static double *field_ptr(or_ctx *c, int f)
{
    switch (f) {
    case VEC_F_R: return c->r;   case VEC_F_T: return c->t;   case VEC_F_U: return c->u;
    case VEC_F_V: return c->v;   case VEC_F_W: return c->w;   case VEC_F_BX: return c->bx;
    case VEC_F_BY: return c->by; case VEC_F_BZ: return c->bz; case VEC_F_JSQ: return c->jsq;
    case VEC_F_POL: return c->pol; case VEC_F_TOR: return c->tor;
    default: break;
    }
    if (f >= VEC_F_RDOT && f < VEC_F_COUNT) {
        int b = (f - VEC_F_RDOT) / 3, s = (f - VEC_F_RDOT) % 3;
        double **tab[] = { c->rdot, c->tdot, c->udot, c->vdot, c->wdot, c->poldot, c->tordot };
        return tab[b][s];
    }
    return NULL;
}

int or_field(or_ctx *c, int field, double *dst, const double *src)
{
    double *f = field_ptr(c, field);
    if (!f) return VEC_ERR_ARG;
    if (src) memcpy(f, src, sizeof(double) * c->n);
    if (dst) memcpy(dst, f, sizeof(double) * c->n);
    return 0;
}

int or_mean(or_ctx *c, int mean, double *dst, const double *src)
{
    double *m = NULL;
    switch (mean) {
    case VEC_M_BXBAR: m = c->bxbar; break;
    case VEC_M_BYBAR: m = c->bybar; break;
    case VEC_M_KAPPA: m = c->kappa; break;
    case VEC_M_DKAPPA: m = c->dkappa; break;
    case VEC_M_ETA: m = c->eta; break;
    case VEC_M_DETA: m = c->deta; break;
    default:
        if (mean >= VEC_M_BXBARDOT && mean < VEC_M_BXBARDOT + 3) m = c->bxbardot[mean - VEC_M_BXBARDOT];
        else if (mean >= VEC_M_BYBARDOT && mean < VEC_M_BYBARDOT + 3) m = c->bybardot[mean - VEC_M_BYBARDOT];
    }
    if (!m) return VEC_ERR_ARG;
    if (src) memcpy(m, src, sizeof(double) * c->nz);
    if (dst) memcpy(dst, m, sizeof(double) * c->nz);
    return 0;
}

int or_scalars(or_ctx *c, vec_scalars *dst, const vec_scalars *src)
{
    if (src) {
        c->dt = src->dt; c->dt1 = src->dt1; c->dt2 = src->dt2; c->ttime = src->ttime;
        c->iter = src->iter; c->nit = src->nit; c->first = src->first; c->second = src->second;
    }
    if (dst) {
        dst->dt = c->dt; dst->dt1 = c->dt1; dst->dt2 = c->dt2; dst->ttime = c->ttime;
        dst->iter = c->iter; dst->nit = c->nit; dst->first = c->first; dst->second = c->second;
    }
    return 0;
}

double or_bzbar(or_ctx *c, const double *set)
{
    if (set) c->bzbar = *set;
    return c->bzbar;
}

/* ===================================================================== */
/* initial state: src/initial.F90:25-86, src/ranset.f90:1-29              */
/* ===================================================================== */
static double ran0(int *idum)
{
    const int IA = 16807, IM = 2147483647, IQ = 127773, IR = 2836, MASK = 123459876;
    const double AM = 1.0 / IM;
    *idum ^= MASK;
    int k = *idum / IQ;
    *idum = IA * (*idum - k * IQ) - IR * k;
    if (*idum < 0) *idum += IM;
    double r = AM * *idum;
    *idum ^= MASK;
    return r;
}

static void ranset(int id, double *a, size_t n, double amp, int base)
{
    int iseed = base + 64 * id;
    for (size_t i = 0; i < n; i++) a[i] = 2.0 * (ran0(&iseed) - 0.5) * amp;
}

int or_static(or_ctx *c)
{
    const double amp = c->p.noise_amp;
    for (int k = 0; k < c->nz; k++) {
        double z = (double)k * c->dz;
        double t0 = 1.0 + z * c->p.theta;
        double r0 = pow(t0, c->p.cm);
        const size_t np = c->np;
        double *tk = AT(c->t, k);
        ranset(k + 1, tk, np, amp, c->p.seed_base);
        for (size_t q = 0; q < np; q++) {
            AT(c->u, k)[q] = 0.0; AT(c->v, k)[q] = 0.0; AT(c->w, k)[q] = 0.0;
            AT(c->r, k)[q] = r0;
            tk[q] = tk[q] + t0;
            if (c->p.perfect) { AT(c->bx, k)[q] = 1.0; AT(c->by, k)[q] = 0.0; AT(c->bz, k)[q] = 0.0; }
            else { AT(c->bx, k)[q] = 0.0; AT(c->by, k)[q] = 0.0; AT(c->bz, k)[q] = 1.0; }
        }
    }
    ini_trans_params(c);
    return 0;
}
#undef AT

/* ===================================================================== */
/* spectral helpers on 2-D halfcomplex planes                              */
/* ===================================================================== */
/* out = d/dx of in (x halfcomplex index shuffle), src/magnetic.f90:141-150 */
static void spec_dx(or_ctx *c, const double *in, double *out)
{
    const int nx = c->nx, ny = c->ny;
#pragma omp parallel for
    for (int k = 0; k < c->nz; k++)
        for (int j = 0; j < ny; j++) {
            const double *a = in + (size_t)k * c->np + (size_t)j * nx;
            double *o = out + (size_t)k * c->np + (size_t)j * nx;
            o[0] = 0.0;
            o[nx / 2] = 0.0;
            for (int i = 1; i <= nx / 2 - 1; i++) {
                double re = a[i], im = a[nx - i];
                o[i] = -im * c->akx1[i];
                o[nx - i] = re * c->akx1[nx - i];
            }
        }
}

/* out = d/dy of in, src/magnetic.f90:155-164 */
static void spec_dy(or_ctx *c, const double *in, double *out)
{
    const int nx = c->nx, ny = c->ny;
#pragma omp parallel for
    for (int k = 0; k < c->nz; k++) {
        const double *a = in + (size_t)k * c->np;
        double *o = out + (size_t)k * c->np;
        for (int i = 0; i < nx; i++) {
            o[i] = 0.0;
            o[(size_t)(ny / 2) * nx + i] = 0.0;
        }
        for (int j = 1; j <= ny / 2 - 1; j++)
            for (int i = 0; i < nx; i++) {
                double re = a[(size_t)j * nx + i], im = a[(size_t)(ny - j) * nx + i];
                o[(size_t)j * nx + i] = -im * c->aky1[j];
                o[(size_t)(ny - j) * nx + i] = re * c->aky1[ny - j];
            }
    }
}

/* a /= (akx2+aky2) with the (1,1) mode set to 0, src/magnetic.f90:429-446 */
static void spec_inv_lap(or_ctx *c, double *a)
{
    const int nx = c->nx, ny = c->ny;
#pragma omp parallel for
    for (int k = 0; k < c->nz; k++) {
        double *p = a + (size_t)k * c->np;
        p[0] = 0.0;
        for (int i = 1; i < nx; i++) p[i] = p[i] / c->akx2[i];
        for (int j = 1; j < ny; j++) p[(size_t)j * nx] = p[(size_t)j * nx] / c->aky2[j];
        for (int j = 1; j < ny; j++)
            for (int i = 1; i < nx; i++)
                p[(size_t)j * nx + i] = p[(size_t)j * nx + i] / (c->akx2[i] + c->aky2[j]);
    }
}

/* zero the truncated modes of a 2-D spectral field, src/magnetic.f90:666-717 */
static void spec_truncate(or_ctx *c, double *a)
{
    const int nx = c->nx, ny = c->ny;
#pragma omp parallel for
    for (int k = 0; k < c->nz; k++) {
        double *p = a + (size_t)k * c->np;
        for (int j = 0; j < ny; j++) {
            for (int i = 1; i <= c->icutoffx; i++) {
                p[(size_t)j * nx + nx / 2 + i] = 0.0;
                p[(size_t)j * nx + nx / 2 - i] = 0.0;
            }
            p[(size_t)j * nx + nx / 2] = 0.0;
        }
        for (int i = 0; i < nx; i++) {
            p[(size_t)(ny / 2) * nx + i] = 0.0;
            for (int j = 1; j <= c->icutoffy; j++) {
                p[(size_t)(ny / 2 + j) * nx + i] = 0.0;
                p[(size_t)(ny / 2 - j) * nx + i] = 0.0;
            }
        }
    }
}

static void zero(or_ctx *c, double *a) { memset(a, 0, sizeof(double) * c->n); }

/* ===================================================================== */
/* hydro_deriv: src/hydro_deriv.f90:5-505                                  */
/* ===================================================================== */
int or_hydro_deriv(or_ctx *c)
{
    const size_t np = c->np;
    const int nz = c->nz;
    double *r = c->r, *t = c->t, *u = c->u, *v = c->v, *w = c->w;
    double *bx = c->bx, *by = c->by, *bz = c->bz, *jsq = c->jsq;
    double *wk1 = c->wk1, *wk2 = c->wk2, *wk3 = c->wk3, *wk4 = c->wk4;
    double *ex = c->ex, *ey = c->ey, *ez = c->ez;
    double *rdot = c->rdot[2], *tdot = c->tdot[2], *udot = c->udot[2], *vdot = c->vdot[2],
           *wdot = c->wdot[2];
    const double gck = c->gck, fzckg = c->fzckg, gm1 = c->gm1, sckg = c->sckg, fo2 = c->fo2,
                 scko3 = c->scko3, f = c->p.f, thmplus1 = c->thmplus1, cor = c->cor,
                 cpsi = c->cpsi, spsi = c->spsi, sck = c->sck, zck = c->zck;
    const double third = 1.0 / 3.0;
    int st;

    or_d1bydx(c, r, wk1);                                   /* :33 */
    or_d1bydy(c, r, wk2);                                   /* :34 */
#pragma omp parallel for
    for (size_t q = 0; q < c->n; q++) {                     /* :45-53 */
        rdot[q] = -u[q] * wk1[q] - v[q] * wk2[q];
        ex[q] = -t[q] * wk1[q];
        ey[q] = -t[q] * wk2[q];
    }
    or_d2bydx(c, t, udot, wk1);                             /* :64 */
    or_d2bydy(c, t, vdot, wk2);                             /* :65 */
    if ((st = or_d1upbydz(c, t, wdot, 5))) return st;       /* :66 */
    or_d1bydz(c, t, wk4, 5);                                /* :67 */
    or_d2bydz(c, t, wk3, 0);                                /* :68 */
    /* :74 ini_trans_params (kappa is time-independent; computed at create) */
#pragma omp parallel for
    for (int k = 0; k < nz; k++) {                          /* :82-110 */
        double ohm = c->p.eta_contrast == 1.0 ? 1.0 : c->eta[k] / zck;
        for (size_t i = 0; i < np; i++) {
            size_t q = (size_t)k * np + i;
            double u0 = u[q], v0 = v[q], w0 = w[q];
            tdot[q] = -r[q] * (u0 * udot[q] + v0 * vdot[q] + w0 * wdot[q])
                      + gck * c->kappa[k] * (wk1[q] + wk2[q] + wk3[q])
                      + gck * c->dkappa[k] * wdot[q]
                      + fzckg * ohm * jsq[q];
            udot[q] = ex[q] - r[q] * udot[q];
            vdot[q] = ey[q] - r[q] * vdot[q];
            wdot[q] = -r[q] * wk4[q];
            ex[q] = 0.0;
            ey[q] = 0.0;
        }
    }
    or_d1bydx(c, u, wk1);                                   /* :122 */
    or_d1bydy(c, v, wk2);                                   /* :123 */
    or_d1upbydz(c, w, wk3, 1);                              /* :124 */
    or_d1bydz(c, w, wk4, 1);                                /* :125 */
#pragma omp parallel for
    for (size_t q = 0; q < c->n; q++) {                     /* :139-168 */
        double z1 = wk1[q], z2 = wk2[q], z3 = wk3[q], z4 = wk4[q];
        double tt = t[q], rr = r[q];
        double divu = z1 + z2 + z4;
        rdot[q] = rdot[q] - rr * divu;
        tdot[q] = tdot[q] - gm1 * tt * divu * rr
                  + 2 * sckg * (z1 * z1 + z2 * z2 + z4 * z4 - third * divu * divu);
        double temp1 = fo2 * bx[q] * bx[q];
        double temp2 = fo2 * by[q] * by[q];
        double temp3 = fo2 * bz[q] * bz[q];
        divu = scko3 * divu;
        double u0 = u[q], v0 = v[q], w0 = w[q];
        udot[q] = udot[q] - rr * u0 * z1;
        vdot[q] = vdot[q] - rr * v0 * z2;
        wdot[q] = wdot[q] - rr * w0 * z3;
        wk1[q] = divu + temp1 - temp2 - temp3;
        wk2[q] = divu + temp2 - temp1 - temp3;
        wk3[q] = scko3 * z1 + scko3 * z2 + temp3 - temp1 - temp2;
        wk4[q] = 4.0 * scko3 * z4;
    }
    or_d1bydx(c, wk1, ex);                                  /* :181 */
    or_d1bydy(c, wk2, ey);                                  /* :182 */
    or_d1bydz(c, wk3, ez, 2);                               /* :183 */
    or_d1bydz(c, wk4, wk3, 5);                              /* :184 */
    or_d1bydx(c, v, wk2);                                   /* :190 */
    or_d1bydy(c, u, wk1);                                   /* :191 */
#pragma omp parallel for
    for (size_t q = 0; q < c->n; q++) {                     /* :201-219 */
        udot[q] = udot[q] + ex[q];
        vdot[q] = vdot[q] + ey[q];
        wdot[q] = wdot[q] + ez[q] + wk3[q];
        ex[q] = 0.0; ey[q] = 0.0; ez[q] = 0.0;
        double rr = r[q], w1 = wk1[q], w2 = wk2[q];
        udot[q] = udot[q] - rr * v[q] * w1;
        vdot[q] = vdot[q] - rr * u[q] * w2;
        wk3[q] = f * by[q] * bx[q];
        tdot[q] = tdot[q] + sckg * (w1 + w2) * (w1 + w2);
    }
    or_d1bydx(c, wk3, wk2);                                 /* :230 */
    or_d1bydy(c, wk3, wk1);                                 /* :231 */
    or_d1bydx(c, w, wk3);                                   /* :232 */
    or_d1upbydz(c, u, wk4, 2);                              /* :233 */
#pragma omp parallel for
    for (size_t q = 0; q < c->n; q++) {                     /* :245-261 */
        udot[q] = udot[q] + wk1[q];
        vdot[q] = vdot[q] + wk2[q];
        double rr = r[q], w3 = wk3[q], w4 = wk4[q];
        udot[q] = udot[q] - rr * w[q] * w4;
        wdot[q] = wdot[q] - rr * u[q] * w3;
        double temp1 = f * bz[q] * bx[q];
        wk1[q] = temp1;
        wk2[q] = temp1;
        tdot[q] = tdot[q] + sckg * (w3 + w4) * (w3 + w4);
    }
    or_d1bydz(c, wk1, wk3, 5);                              /* :272 */
    or_d1bydx(c, wk2, wk4);                                 /* :273 */
    or_d1bydy(c, w, wk1);                                   /* :274 */
    or_d1upbydz(c, v, wk2, 2);                              /* :275 */
#pragma omp parallel for
    for (size_t q = 0; q < c->n; q++) {                     /* :287-309 */
        double rr = r[q];
        udot[q] = udot[q] + wk3[q];
        wdot[q] = wdot[q] + wk4[q] + thmplus1 * rr;
        double w1 = wk1[q], w2 = wk2[q];
        vdot[q] = vdot[q] - rr * w[q] * w2;
        wdot[q] = wdot[q] - rr * v[q] * w1;
        double temp1 = f * bz[q] * by[q];
        wk3[q] = temp1;
        wk4[q] = temp1;
        tdot[q] = tdot[q] + sckg * (w1 + w2) * (w1 + w2);
        udot[q] = udot[q] - rr * cor * (w[q] * cpsi + v[q] * spsi);
        vdot[q] = vdot[q] - rr * cor * (-u[q] * spsi);
        wdot[q] = wdot[q] - rr * cor * (-u[q] * cpsi);
    }
    or_d1bydy(c, wk3, wk1);                                 /* :320 */
    or_d1bydz(c, wk4, wk2, 5);                              /* :321 */
#pragma omp parallel for
    for (size_t q = 0; q < c->n; q++) {                     /* :331-338 */
        vdot[q] = vdot[q] + wk2[q];
        wdot[q] = wdot[q] + wk1[q];
    }
    or_d2bydz(c, u, wk1, 3);                                /* :349 */
    or_d2bydz(c, v, wk2, 3);                                /* :350 */
#pragma omp parallel for
    for (size_t q = 0; q < c->n; q++) {                     /* :360-367 */
        udot[q] = udot[q] + sck * wk1[q];
        vdot[q] = vdot[q] + sck * wk2[q];
    }
    or_d2bydx(c, u, ex, wk1);                               /* :378 */
    or_d2bydx(c, v, ey, wk2);                               /* :379 */
    or_d2bydx(c, w, ez, wk3);                               /* :380 */
#pragma omp parallel for
    for (size_t q = 0; q < c->n; q++) {                     /* :390-398 */
        udot[q] = udot[q] + sck * wk1[q];
        vdot[q] = vdot[q] + sck * wk2[q];
        wdot[q] = wdot[q] + sck * wk3[q];
    }
    or_d2bydy(c, u, ex, wk1);                               /* :409 */
    or_d2bydy(c, v, ey, wk2);                               /* :410 */
    or_d2bydy(c, w, ez, wk3);                               /* :411 */
#pragma omp parallel for
    for (size_t q = 0; q < c->n; q++) {                     /* :421-432 */
        udot[q] = udot[q] + sck * wk1[q];
        vdot[q] = vdot[q] + sck * wk2[q];
        wdot[q] = wdot[q] + sck * wk3[q];
        ex[q] = 0.0; ey[q] = 0.0; ez[q] = 0.0;
    }
    or_d1upbydz(c, r, wk1, 0);                              /* :443 */
    or_d1bydz(c, r, wk2, 0);                                /* :444 */
    for (size_t i = 0; i < np; i++) {                       /* :455-470 */
        wk1[i] = wdot[i] / t[i];
        wk2[i] = wdot[i] / t[i];
        size_t q = (size_t)(nz - 1) * np + i;
        wk1[q] = wdot[q] / t[q];
        wk2[q] = wdot[q] / t[q];
    }
#pragma omp parallel for
    for (size_t q = 0; q < c->n; q++) {                     /* :475-482 */
        rdot[q] = rdot[q] - w[q] * wk1[q];
        wdot[q] = wdot[q] - t[q] * wk2[q];
    }
#pragma omp parallel for
    for (size_t q = 0; q < c->n; q++) {                     /* :487-497 */
        double rr = 1.0 / (r[q]);
        tdot[q] = tdot[q] * rr;
        udot[q] = udot[q] * rr;
        vdot[q] = vdot[q] * rr;
        wdot[q] = wdot[q] * rr;
    }
    return 0;
}

/* ===================================================================== */
/* mag_deriv: src/magnetic.f90:285-487 (+ eta(z) extension)                */
/* ===================================================================== */
int or_mag_deriv(or_ctx *c)
{
    const size_t np = c->np;
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    double *u = c->u, *v = c->v, *w = c->w, *bx = c->bx, *by = c->by, *bz = c->bz;
    double *wk1 = c->wk1, *wk2 = c->wk2, *wk3 = c->wk3, *wk4 = c->wk4;
    double *ex = c->ex, *ey = c->ey, *ez = c->ez;
    const double zck = c->zck, xn = c->xn;
    const int var_eta = c->p.eta_contrast != 1.0;

#pragma omp parallel for
    for (size_t q = 0; q < c->n; q++) {                     /* :308-316 */
        wk1[q] = v[q] * bz[q] - w[q] * by[q];
        wk2[q] = w[q] * bx[q] - u[q] * bz[q];
        wk3[q] = u[q] * by[q] - v[q] * bx[q];
    }
    or_forwardfft(c, wk1, ex);                              /* :321-323 */
    or_forwardfft(c, wk2, ey);
    or_forwardfft(c, wk3, ez);
    for (int k = 0; k < nz; k++) {                          /* :328-331 */
        c->wk1_1d[k] = xn * ex[(size_t)k * np];
        c->wk2_1d[k] = xn * ey[(size_t)k * np];
    }
    double *bxd = c->bxbardot[2], *byd = c->bybardot[2];
    or_d1bydz1d(c, c->wk2_1d, bxd, 5);                      /* :337 */
    or_d1bydz1d(c, c->wk1_1d, byd, 5);                      /* :338 */
    or_d2bydz1d(c, c->bxbar, c->wk1_1d, 3);                 /* :343 */
    or_d2bydz1d(c, c->bybar, c->wk2_1d, 3);                 /* :344 */
    if (!var_eta) {
        for (int k = 0; k < nz; k++) {                      /* :349-352 */
            bxd[k] = zck * c->wk1_1d[k] - bxd[k];
            byd[k] = zck * c->wk2_1d[k] + byd[k];
        }
    } else {
        /* extension: d(bxbar)/dt gains eta' d(bxbar)/dz, same for bybar */
        double *gx = c->tmp1d, *gy = c->tmp1d + nz;
        or_d1bydz1d(c, c->bxbar, gx, 5);
        or_d1bydz1d(c, c->bybar, gy, 5);
        for (int k = 0; k < nz; k++) {
            bxd[k] = c->eta[k] * c->wk1_1d[k] - bxd[k] + c->deta[k] * gx[k];
            byd[k] = c->eta[k] * c->wk2_1d[k] + byd[k] + c->deta[k] * gy[k];
        }
    }
    /* :362-407: wk1 = dEx/dx + dEy/dy, wk2 = dEx/dy - dEy/dx (spectral) */
    spec_dx(c, ex, wk1);
    spec_dx(c, ey, wk2);
    spec_dy(c, ex, wk3);
    spec_dy(c, ey, wk4);
#pragma omp parallel for
    for (size_t q = 0; q < c->n; q++) {
        wk2[q] = wk3[q] - wk2[q];
        wk1[q] = wk1[q] + wk4[q];
    }
    or_d1bydz(c, wk1, wk3, 5);                              /* :419 */
    spec_inv_lap(c, wk2);                                   /* :429-446 */
    spec_inv_lap(c, wk3);
    or_d2bydz(c, c->pol, wk1, 3);                           /* :457 */
    or_d2bydz(c, c->tor, wk4, 3);                           /* :458 */
    double *poldot = c->poldot[2], *tordot = c->tordot[2], *pol = c->pol, *tor = c->tor;
    if (!var_eta) {
#pragma omp parallel for
        for (int k = 0; k < nz; k++)                        /* :470-479 */
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++) {
                    size_t q = (size_t)k * np + (size_t)j * nx + i;
                    poldot[q] = zck * pol[q] * (c->akx2[i] + c->aky2[j]) + zck * wk1[q] + wk2[q];
                    tordot[q] = zck * tor[q] * (c->akx2[i] + c->aky2[j]) + zck * wk4[q] - wk3[q] + ez[q];
                }
    } else {
        /* extension: eta(z) replaces zck; tordot gains eta' d(tor)/dz */
        or_d1bydz(c, tor, ex, 5);
#pragma omp parallel for
        for (int k = 0; k < nz; k++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++) {
                    size_t q = (size_t)k * np + (size_t)j * nx + i;
                    double e = c->eta[k];
                    poldot[q] = e * pol[q] * (c->akx2[i] + c->aky2[j]) + e * wk1[q] + wk2[q];
                    tordot[q] = e * tor[q] * (c->akx2[i] + c->aky2[j]) + e * wk4[q] - wk3[q] + ez[q]
                                + c->deta[k] * ex[q];
                }
    }
    return 0;
}

/* ===================================================================== */
/* bandj: src/magnetic.f90:492-664                                        */
/* ===================================================================== */
int or_bandj(or_ctx *c)
{
    const size_t np = c->np;
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    double *wk1 = c->wk1, *wk2 = c->wk2, *wk3 = c->wk3, *wk4 = c->wk4;
    double *ex = c->ex, *ey = c->ey, *ez = c->ez, *pol = c->pol, *tor = c->tor;
    or_d1bydz(c, pol, wk1, 5);                              /* :519 */
    spec_dx(c, wk1, ex);                                    /* :525-538 */
    spec_dx(c, tor, wk3);
    spec_dy(c, wk1, ey);                                    /* :544-557 */
    spec_dy(c, tor, wk2);
#pragma omp parallel for
    for (int k = 0; k < nz; k++)                            /* :562-570 */
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                size_t q = (size_t)k * np + (size_t)j * nx + i;
                ex[q] = ex[q] + wk2[q];
                ey[q] = ey[q] - wk3[q];
                ez[q] = -1.0 * pol[q] * (c->akx2[i] + c->aky2[j]);
            }
    or_inversefft(c, ex, c->bx);                            /* :575-577 */
    or_inversefft(c, ey, c->by);
    or_inversefft(c, ez, c->bz);
#pragma omp parallel for
    for (int k = 0; k < nz; k++)                            /* :584-593 */
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                size_t q = (size_t)k * np + (size_t)j * nx + i;
                c->bx[q] = c->bx[q] + c->bxbar[k];
                c->by[q] = c->by[q] + c->bybar[k];
                c->bz[q] = c->bz[q] + c->bzbar;
                wk3[q] = -1.0 * tor[q] * (c->akx2[i] + c->aky2[j]);
            }
    spec_dy(c, ez, wk1);                                    /* :600-617 */
    spec_dx(c, ez, wk2);
    or_inversefft(c, wk1, ex);                              /* :623-625 */
    or_inversefft(c, wk2, ey);
    or_inversefft(c, wk3, ez);
    or_d1bydz(c, c->by, wk1, 5);                            /* :630 */
    or_d1bydz(c, c->bx, wk2, 5);                            /* :631 */
#pragma omp parallel for
    for (size_t q = 0; q < c->n; q++)                       /* :636-645 */
        c->jsq[q] = ez[q] * ez[q] + ((ex[q] - wk1[q]) * (ex[q] - wk1[q]))
                    + ((wk2[q] - ey[q]) * (wk2[q] - ey[q]));
    zero(c, ex); zero(c, ey); zero(c, ez);                  /* :650-656 */
    zero(c, wk1); zero(c, wk2); zero(c, wk3); zero(c, wk4);
    return 0;
}

int or_magdealias(or_ctx *c)
{
    spec_truncate(c, c->pol);
    spec_truncate(c, c->tor);
    return 0;
}

/* ===================================================================== */
/* mag_init: src/magnetic.f90:5-279                                        */
/* ===================================================================== */
int or_mag_init(or_ctx *c)
{
    const size_t np = c->np;
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    double *wk1 = c->wk1, *wk2 = c->wk2, *wk3 = c->wk3, *wk4 = c->wk4;
    double *ex = c->ex, *ey = c->ey, *ez = c->ez, *pol = c->pol, *tor = c->tor;
    if (c->p.dynamo) {                                      /* :29-57 */
        const double seedfield = 0.003;
        const double twopionx = 8.0 * atan(1.0) / (nx * 1.0);
        const double twopiony = 8.0 * atan(1.0) / (ny * 1.0);
        for (int k = 0; k < nz; k++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++) {
                    size_t q = (size_t)k * np + (size_t)j * nx + i;
                    if (c->p.perfect) {
                        c->bx[q] = seedfield * cos(twopiony * (j + 1));
                        c->by[q] = seedfield * cos(twopionx * (i + 1));
                        c->bz[q] = 0.0;
                    } else {
                        c->bx[q] = 0.0;
                        c->by[q] = 0.0;
                        c->bz[q] = seedfield * cos(twopionx * (i + 1)) * cos(twopiony * (j + 1));
                    }
                }
    }
    or_forwardfft(c, c->bx, ex);                            /* :63-65 */
    or_forwardfft(c, c->by, ey);
    or_forwardfft(c, c->bz, ez);
    spec_truncate(c, ex);                                   /* :70-103 */
    spec_truncate(c, ey);
    spec_truncate(c, ez);
    for (int k = 0; k < nz; k++) {                          /* :111-117 */
        c->bxbar[k] = ex[(size_t)k * np];
        c->bybar[k] = ey[(size_t)k * np];
    }
    for (int k = 0; k < nz; k++) { c->bxbar[k] *= c->xn; c->bybar[k] *= c->xn; }
    c->bzbar = ez[0] * c->xn;
    /* :123-136 pol = -ez/(akx2+aky2), DC = 0 */
    memcpy(pol, ez, sizeof(double) * c->n);
    spec_inv_lap(c, pol);
    for (size_t q = 0; q < c->n; q++) pol[q] = -1.0 * pol[q];
    /* careful: the reference forms -1*ez/kk; (-ez)/kk == -(ez/kk) exactly */
    spec_dx(c, ey, wk3);                                    /* :141-150 */
    spec_dy(c, ex, wk4);                                    /* :155-164 */
    for (size_t q = 0; q < c->n; q++) wk3[q] = wk3[q] - wk4[q];   /* :169-175 */
    memcpy(tor, wk3, sizeof(double) * c->n);                /* :181-194 */
    spec_inv_lap(c, tor);
    for (size_t q = 0; q < c->n; q++) tor[q] = -1.0 * tor[q];
#pragma omp parallel for
    for (int k = 0; k < nz; k++)                            /* :199-205 */
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                size_t q = (size_t)k * np + (size_t)j * nx + i;
                wk3[q] = -1.0 * tor[q] * (c->akx2[i] + c->aky2[j]);
            }
    spec_dy(c, ez, wk1);                                    /* :210-219 */
    spec_dx(c, ez, wk2);                                    /* :224-233 */
    or_inversefft(c, wk1, ex);                              /* :239-241 */
    or_inversefft(c, wk2, ey);
    or_inversefft(c, wk3, ez);
    or_d1bydz(c, c->by, wk1, 5);                            /* :246-247 */
    or_d1bydz(c, c->bx, wk2, 5);
    for (size_t q = 0; q < c->n; q++)                       /* :252-261 */
        c->jsq[q] = ez[q] * ez[q] + ((ex[q] - wk1[q]) * (ex[q] - wk1[q]))
                    + ((wk2[q] - ey[q]) * (wk2[q] - ey[q]));
    or_mag_boundary(c);                                     /* :266 */
    zero(c, ex); zero(c, ey); zero(c, ez);
    zero(c, wk1); zero(c, wk2); zero(c, wk3); zero(c, wk4);
    return 0;
}

/* ===================================================================== */
/* boundary conditions                                                     */
/* ===================================================================== */
/* src/dbydz.F90:3686-4197, serial parts :3807-3831, :3878-3902, :4036-4187 */
int or_boundary(or_ctx *c)
{
    const size_t np = c->np;
    const int nz = c->nz;
    const double elf = 1.0 / 11.0, theta = c->p.theta, dz = c->dz;
    double *u = c->u, *v = c->v, *w = c->w, *t = c->t;
#define P(f, k) ((f) + (size_t)(k) * np)
    for (size_t q = 0; q < np; q++) {
        P(w, 0)[q] = 0.0;
        P(u, 0)[q] = elf * (18.0 * P(u, 1)[q] - 9.0 * P(u, 2)[q] + 2.0 * P(u, 3)[q]);
        P(v, 0)[q] = elf * (18.0 * P(v, 1)[q] - 9.0 * P(v, 2)[q] + 2.0 * P(v, 3)[q]);
    }
    for (size_t q = 0; q < np; q++) {
        P(w, nz - 1)[q] = 0.0;
        P(u, nz - 1)[q] = elf * (18.0 * P(u, nz - 2)[q] - 9.0 * P(u, nz - 3)[q] + 2.0 * P(u, nz - 4)[q]);
        P(v, nz - 1)[q] = elf * (18.0 * P(v, nz - 2)[q] - 9.0 * P(v, nz - 3)[q] + 2.0 * P(v, nz - 4)[q]);
    }
    if (c->p.radbc) {
        for (size_t q = 0; q < np; q++) {
            double t1old = P(t, 0)[q], ft1 = 0.0, dft1 = 1.0;
            for (int it = 0; it < 10; it++) {
                ft1 = 6.0 * theta * dz * t1old * t1old * t1old * t1old + 11.0 * t1old
                      - 18.0 * P(t, 1)[q] + 9.0 * P(t, 2)[q] - 2.0 * P(t, 3)[q];
                dft1 = 24.0 * theta * dz * t1old * t1old * t1old + 11.0;
                t1old = t1old - (ft1 / dft1);
            }
            P(t, 0)[q] = t1old;
        }
    } else {
        for (size_t q = 0; q < np; q++) P(t, 0)[q] = 1.0;
    }
    if (c->p.constflux) {
        for (size_t q = 0; q < np; q++)
            P(t, nz - 1)[q] = elf * (18.0 * P(t, nz - 2)[q] - 9.0 * P(t, nz - 3)[q]
                                     + 2.0 * P(t, nz - 4)[q] + 6.0 * theta * dz);
    } else {
        for (size_t q = 0; q < np; q++) P(t, nz - 1)[q] = 1.0 + theta;
    }
    return 0;
}

/* src/dbydz.F90:4205-4791: perfect :4407-4560, vertical field :4663-4780 */
int or_mag_boundary(or_ctx *c)
{
    const size_t np = c->np;
    const int nz = c->nz;
    const double elf = 1.0 / 11.0;
    double *pol = c->pol, *tor = c->tor, *bxb = c->bxbar, *byb = c->bybar;
    if (c->p.perfect) {
        for (size_t q = 0; q < np; q++) P(pol, 0)[q] = 0.0;
        bxb[0] = elf * (18.0 * bxb[1] - 9.0 * bxb[2] + 2.0 * bxb[3]);
        byb[0] = elf * (18.0 * byb[1] - 9.0 * byb[2] + 2.0 * byb[3]);
        for (size_t q = 0; q < np; q++)
            P(tor, 0)[q] = elf * (18.0 * P(tor, 1)[q] - 9.0 * P(tor, 2)[q] + 2.0 * P(tor, 3)[q]);
        for (size_t q = 0; q < np; q++) P(pol, nz - 1)[q] = 0.0;
        bxb[nz - 1] = elf * (18.0 * bxb[nz - 2] - 9.0 * bxb[nz - 3] + 2.0 * bxb[nz - 4]);
        byb[nz - 1] = elf * (18.0 * byb[nz - 2] - 9.0 * byb[nz - 3] + 2.0 * byb[nz - 4]);
        for (size_t q = 0; q < np; q++)
            P(tor, nz - 1)[q] = elf * (18.0 * P(tor, nz - 2)[q] - 9.0 * P(tor, nz - 3)[q]
                                       + 2.0 * P(tor, nz - 4)[q]);
    } else {
        bxb[0] = 0.0; byb[0] = 0.0;
        for (size_t q = 0; q < np; q++) P(tor, 0)[q] = 0.0;
        for (size_t q = 0; q < np; q++)
            P(pol, 0)[q] = elf * (18.0 * P(pol, 1)[q] - 9.0 * P(pol, 2)[q] + 2.0 * P(pol, 3)[q]);
        bxb[nz - 1] = 0.0; byb[nz - 1] = 0.0;
        for (size_t q = 0; q < np; q++) P(tor, nz - 1)[q] = 0.0;
        for (size_t q = 0; q < np; q++)
            P(pol, nz - 1)[q] = elf * (18.0 * P(pol, nz - 2)[q] - 9.0 * P(pol, nz - 3)[q]
                                       + 2.0 * P(pol, nz - 4)[q]);
    }
    return 0;
}

/* ===================================================================== */
/* calcdt: src/utils.F90:144-244 (+ magnetic-diffusion limit for eta(z))   */
/* ===================================================================== */
int or_calcdt(or_ctx *c, double *dtout)
{
    double denmn = c->r[0], velmxx = -1.0e-50, velmxz = -1.0e-50;
    const double g1 = c->g1, f = c->p.f;
    for (size_t q = 0; q < c->n; q++) {
        double u0 = c->u[q], v0 = c->v[q], w0 = c->w[q], r0 = c->r[q], t0 = c->t[q];
        double bz0 = c->bz[q], bx0 = c->bx[q], by0 = c->by[q];
        double bsq0 = bx0 * bx0 + by0 * by0 + bz0 * bz0;
        double xx = sqrt(u0 * u0 + v0 * v0) + g1 * sqrt(t0) + sqrt((bsq0 * f) / r0);
        double xz = sqrt(w0 * w0) + g1 * sqrt(t0) + sqrt((bsq0 * f) / r0);
        denmn = fmin(denmn, r0);
        velmxx = fmax(velmxx, xx);
        velmxz = fmax(velmxz, xz);
    }
    double dtcflx = 0.16 * c->dd / velmxx;
    double dtcflz = 0.3 * c->dz / velmxz;
    double m = dtcflx;
    double lim[] = { dtcflz, c->dtvisc0x * denmn, c->dtvisc0z * denmn, c->dtdiff0x * denmn,
                     c->dtdiff0z * denmn };
    for (int i = 0; i < 5; i++) m = fmin(m, lim[i]);
    if (c->p.eta_contrast != 1.0) {
        /* extension: explicit magnetic diffusion limits for eta(z) */
        double emax = 0.0;
        for (int k = 0; k < c->nz; k++) emax = fmax(emax, c->eta[k]);
        m = fmin(m, 0.1 * c->dd * c->dd / emax);
        m = fmin(m, 0.2 * c->dz * c->dz / emax);
    }
    double dt = c->p.sf * m;
    c->dt = dt;
    if (dtout) *dtout = dt;
    return 0;
}

/* ===================================================================== */
/* AB3 update: src/main.F90:381-489 + magdealias (:503-509 handled by step) */
/* ===================================================================== */
int or_ab3_update(or_ctx *c)
{
    double dt = c->dt, c0, c1, c2;
    if (c->first) {
        c->first = 0; c->second = 1;
        c->dt1 = 0.0; c->dt2 = 0.0;
        c0 = dt; c1 = 0.0; c2 = 0.0;
    } else if (c->second) {
        c->first = 0; c->second = 0;
        c->dt2 = 0.0;
        c0 = dt * (1.0 + 0.5 * (dt / c->dt1));
        c1 = -0.5 * dt * (dt / c->dt1);
        c2 = 0.0;
    } else {
        double dt1 = c->dt1, dt2 = c->dt2;
        c0 = dt + (((dt * dt) / (dt1 * dt2)) * ((dt / 3.0) + 0.5 * (dt1 + dt2)));
        c1 = ((dt * dt) / (dt1 * (dt1 - dt2))) * ((dt / 3.0) + 0.5 * dt2);
        c2 = -((dt * dt) / (dt2 * (dt1 - dt2))) * ((dt / 3.0) + 0.5 * dt1);
    }
    const size_t np = c->np;
#pragma omp parallel for
    for (int k = 0; k < c->nz; k++) {
        for (size_t i = 0; i < np; i++) {
            size_t q = (size_t)k * np + i;
            double *x[7] = { c->u, c->v, c->w, c->r, c->t, c->pol, c->tor };
            double **d[7] = { c->udot, c->vdot, c->wdot, c->rdot, c->tdot, c->poldot, c->tordot };
            for (int f = 0; f < 7; f++)
                x[f][q] = x[f][q] + c0 * d[f][2][q] + c1 * d[f][1][q] + c2 * d[f][0][q];
            if (c->r[q] < 0.05) {
                c->r[q] = 0.05;
                c->rdot[0][q] = 0.0; c->rdot[1][q] = 0.0; c->rdot[2][q] = 0.0;
            }
            for (int f = 0; f < 7; f++) {
                d[f][0][q] = d[f][1][q];
                d[f][1][q] = d[f][2][q];
            }
        }
        c->bxbar[k] = c->bxbar[k] + c0 * c->bxbardot[2][k] + c1 * c->bxbardot[1][k] + c2 * c->bxbardot[0][k];
        c->bybar[k] = c->bybar[k] + c0 * c->bybardot[2][k] + c1 * c->bybardot[1][k] + c2 * c->bybardot[0][k];
        c->bxbardot[0][k] = c->bxbardot[1][k]; c->bxbardot[1][k] = c->bxbardot[2][k];
        c->bybardot[0][k] = c->bybardot[1][k]; c->bybardot[1][k] = c->bybardot[2][k];
    }
    c->dt2 = dt + c->dt1;                                   /* :488-489 */
    c->dt1 = dt;
    return 0;
}

/* ===================================================================== */
/* diagnostics: src/utils.F90:22-371, src/dbydz.F90:4796-4925,             */
/* src/main.F90:552-647                                                   */
/* ===================================================================== */
static void sminmax(or_ctx *c, const double *z, double *zmin, double *zmax)
{
    double mn = z[0], mx = z[0];
    for (size_t q = 0; q < c->n; q++) { mn = fmin(mn, z[q]); mx = fmax(mx, z[q]); }
    *zmin = mn; *zmax = mx;
}

int or_diag(or_ctx *c, vec_diag_out *o)
{
    const size_t np = c->np;
    const int nz = c->nz;
    vec_diag_out d;
    memset(&d, 0, sizeof(d));
    /* GlobalAverages, src/utils.F90:22-139 */
    double urbar = 0.0, vrbar = 0.0, rbar = 0.0, me = 0.0, ke = 0.0;
    for (int k = 0; k < nz; k++) {
        double urav = 0.0, vrav = 0.0, rav = 0.0, keav = 0.0, bsqav = 0.0;
        for (size_t i = 0; i < np; i++) {
            size_t q = (size_t)k * np + i;
            double uu = c->u[q], vv = c->v[q], rr = c->r[q], ww = c->w[q];
            rav = rav + rr;
            urav = urav + rr * uu;
            vrav = vrav + rr * vv;
            keav = keav + 0.5 * rr * (uu * uu + vv * vv + ww * ww);
            bsqav = bsqav + c->bx[q] * c->bx[q] + c->by[q] * c->by[q] + c->bz[q] * c->bz[q];
        }
        if (k == 0 || k == nz - 1) {
            urbar += 0.5 * urav; vrbar += 0.5 * vrav; rbar += 0.5 * rav;
            me += 0.25 * bsqav; ke += 0.5 * keav;
        } else {
            urbar += urav; vrbar += vrav; rbar += rav; me += 0.5 * bsqav; ke += keav;
        }
    }
    d.ubar = urbar / rbar;
    d.vbar = vrbar / rbar;
    me = me * c->xzn;
    ke = ke * c->xzn;
    for (size_t q = 0; q < c->n; q++) { c->u[q] -= d.ubar; c->v[q] -= d.vbar; }
    d.kenergy = ke;
    d.menergy = c->p.kinematic ? me : c->p.f * me;          /* main.F90:567-571 */
    /* nusselt, src/dbydz.F90:4877-4921 */
    double tzbar = 0.0;
    for (size_t i = 0; i < np; i++) {
        const double *t = c->t;
        tzbar = tzbar + ((1.0 / (6.0 * c->dz)) *
                         (11.0 * t[(size_t)(nz - 1) * np + i] - 18.0 * t[(size_t)(nz - 2) * np + i]
                          + 9.0 * t[(size_t)(nz - 3) * np + i] - 2.0 * t[(size_t)(nz - 4) * np + i]));
    }
    tzbar = tzbar * c->xn;
    d.nusselt = (tzbar - c->nusstmp) / (c->p.theta - c->nusstmp);
    /* checkdivb, src/utils.F90:249-318 */
    or_d1bydx(c, c->bx, c->wk1);
    or_d1bydy(c, c->by, c->wk2);
    or_d1bydz(c, c->bz, c->wk3, 5);
    double dmax = -1.0e30, dmin = 1.0;
    for (int k = 0; k < nz; k++) {
        double tlmax = -1.0e30, tlmin = 1.0e30;
        for (size_t i = 0; i < np; i++) {
            size_t q = (size_t)k * np + i;
            double t1 = c->wk1[q] + c->wk2[q] + c->wk3[q];
            tlmax = fmax(tlmax, t1);
            tlmin = fmin(tlmin, t1);
        }
        dmax = fmax(dmax, tlmax);
        dmin = fmin(dmin, tlmin);
    }
    d.divbmax = dmax;
    d.divbmin = dmin;
    /* sminmax + derived, src/main.F90:593-621 */
    sminmax(c, c->r, &d.rmin, &d.rmax);
    sminmax(c, c->t, &d.tmin, &d.tmax);
    sminmax(c, c->u, &d.umin, &d.umax);
    sminmax(c, c->v, &d.vmin, &d.vmax);
    sminmax(c, c->w, &d.wmin, &d.wmax);
    sminmax(c, c->bx, &d.bxmin, &d.bxmax);
    sminmax(c, c->by, &d.bymin, &d.bymax);
    sminmax(c, c->bz, &d.bzmin, &d.bzmax);
    for (size_t q = 0; q < c->n; q++) {
        double uu = c->u[q], vv = c->v[q], ww = c->w[q];
        c->wk1[q] = (uu * uu + vv * vv + ww * ww) / c->t[q];
        c->wk2[q] = (c->bx[q] * c->bx[q] + c->by[q] * c->by[q] + c->bz[q] * c->bz[q]) / c->r[q];
        c->wk3[q] = (uu * uu + vv * vv + ww * ww);
    }
    sminmax(c, c->wk1, &d.machmin, &d.machmax);
    sminmax(c, c->wk2, &d.alfvenmin, &d.alfvenmax);
    sminmax(c, c->wk3, &d.rmsmin, &d.rmsmax);
    double fa = c->p.kinematic ? 1.0 : c->p.f;
    d.alfvenmin = sqrt(fa * d.alfvenmin);
    d.alfvenmax = sqrt(fa * d.alfvenmax);
    d.machmin = sqrt(d.machmin / c->p.gamma);
    d.machmax = sqrt(d.machmax / c->p.gamma);
    d.rmsmin = sqrt(d.rmsmin);
    d.rmsmax = sqrt(d.rmsmax);
    zero(c, c->wk1); zero(c, c->wk2); zero(c, c->wk3);
    c->last = d;
    if (o) *o = d;
    double divbtest = fmax(fabs(dmax), fabs(dmin));
    if (divbtest > 0.01) return VEC_ERR_DIVB;               /* main.F90:583-590 */
    return 0;
}

int or_last_diag(or_ctx *c, vec_diag_out *out) { *out = c->last; return 0; }

/* ===================================================================== */
/* the time loop body, src/main.F90:340-747 (no printing / snapshots)      */
/* ===================================================================== */
int or_step(or_ctx *c, int nsteps)
{
    const int mag = (c->p.f != 0.0) || c->p.kinematic;
    int st;
    for (int s = 0; s < nsteps; s++) {
        c->nit = c->nit + 1;
        c->iter = c->iter + 1;
        c->ttime = c->ttime + c->dt;
        if ((st = or_hydro_deriv(c))) return st;
        if (mag) {
            or_mag_deriv(c);
        } else {
            memset(c->poldot[2], 0, sizeof(double) * c->n);
            memset(c->tordot[2], 0, sizeof(double) * c->n);
            memset(c->bxbardot[2], 0, sizeof(double) * c->nz);
            memset(c->bybardot[2], 0, sizeof(double) * c->nz);
        }
        or_ab3_update(c);
        if (c->p.dalias) {
            if (c->nit % 10 == 0) {
                or_dealias(c, c->r); or_dealias(c, c->t); or_dealias(c, c->u);
                or_dealias(c, c->v); or_dealias(c, c->w);
            }
            if (mag) or_magdealias(c);
        }
        if (mag) or_bandj(c);
        or_boundary(c);
        if (mag) or_mag_boundary(c);
        if (c->p.diag_cadence && c->p.ndu06 > 0 && c->nit % c->p.ndu06 == 0) {
            if ((st = or_diag(c, NULL))) return st;
        }
        if (c->nit % 10 == 0) or_calcdt(c, NULL);
    }
    return 0;
}
