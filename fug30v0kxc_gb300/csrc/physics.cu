// physics.cu -- the FP64 (plain drop-in) right-hand sides, update, boundary
// conditions and reductions of the VarElecCond time step, for sm_103a.
//
// hydro_deriv (src/hydro_deriv.f90:5-505) is regrouped by data dependence
// into four passes instead of the reference's 37 operator calls and 11
// pointwise loops:
//   1. one x-line launch and one y-line launch produce the 18 horizontal
//      derivatives of r,t,u,v,w (one forward FFT per field and direction,
//      d1 and d2 from it);
//   2. a pointwise kernel evaluates every z derivative of the state on the
//      fly, completes the energy equation and accumulates the momentum and
//      continuity terms that need no second-level derivative, and forms the
//      second-level inputs (viscous grad-div, Maxwell stresses);
//   3. x- and y-line launches differentiate those inputs straight into the
//      momentum accumulators (accumulate epilogue);
//   4. a pointwise kernel adds their z derivatives, applies the boundary
//      override of d(rho)/dz (:455-470) and divides by rho (:487-497).
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "common.cuh"
#include "engine.h"
#include "fpconv.cuh"
#include "zstencil.cuh"
#include "magkern.cuh"

#define TPB 256
static inline unsigned nblk(size_t n, int tpb = TPB)
{
    size_t b = (n + tpb - 1) / tpb;
    return (unsigned)(b > 0x7fffffff ? 0x7fffffff : b);
}

#define KLAUNCHB(E, name, bytes, kern, grid, block, ...)         \
    do {                                                         \
        (E)->prof_begin(name, (double)(bytes));                  \
        CUDA_TRY(launch_k(*(E), kern, dim3(grid), dim3(block), 0, __VA_ARGS__)); \
        (E)->prof_end();                                         \
        CUDA_TRY(cudaGetLastError());                            \
    } while (0)
#define KLAUNCH(E, name, kern, grid, block, ...) KLAUNCHB(E, name, 0, kern, grid, block, __VA_ARGS__)
// algorithmic bytes of a pointwise kernel touching nf full fields of esz bytes
#define FB(E, nf, esz) ((double)(nf) * (double)(E)->n * (double)(esz))

// ============================================================================
// z-derivative operators (per-operator entry points)
// ============================================================================
template <typename R>
__global__ void k_d1z(const R *in, R *out, int fl, size_t np, int nz, R h)
{
    PDL_WAIT();
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= np * nz) return;
    int k = (int)(idx / np);
    size_t q = idx - (size_t)k * np;
    out[idx] = zd1(in + q, np, k, nz, fl, h);
}
template <typename R>
__global__ void k_d1upz(const R *in, const R *w, R *out, int fl, size_t np, int nz, R h)
{
    PDL_WAIT();
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= np * nz) return;
    int k = (int)(idx / np);
    size_t q = idx - (size_t)k * np;
    out[idx] = zd1up(in + q, np, k, nz, fl, h, w[idx]);
}
template <typename R>
__global__ void k_d2z(const R *in, R *out, int fl, size_t np, int nz, R s)
{
    PDL_WAIT();
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= np * nz) return;
    int k = (int)(idx / np);
    size_t q = idx - (size_t)k * np;
    out[idx] = zd2(in + q, np, k, nz, fl, s);
}

int op_d1z(Engine *E, const double *in, double *out, int flag, int np, int nz)
{
    if (!(flag == 0 || flag == 1 || flag == 2 || flag == 5)) return VEC_ERR_FLAG;
    KLAUNCHB(E, "d1bydz_f64", 2.0 * np * nz * 8, k_d1z<double>, nblk((size_t)np * nz), TPB, in, out, flag, (size_t)np, nz, E->k.ho12);
    return VEC_OK;
}
int op_d1upz(Engine *E, const double *in, double *out, int flag)
{
    if (!(flag == 0 || flag == 1 || flag == 2 || flag == 5)) return VEC_ERR_FLAG;
    KLAUNCH(E, "d1upbydz_f64", k_d1upz<double>, nblk(E->n), TPB, in, E->w, out, flag, E->np, E->nz, E->k.ho12);
    return VEC_OK;
}
int op_d2z(Engine *E, const double *in, double *out, int flag, int np, int nz)
{
    if (!(flag == 0 || flag == 3)) return VEC_ERR_FLAG;
    KLAUNCH(E, "d2bydz_f64", k_d2z<double>, nblk((size_t)np * nz), TPB, in, out, flag, (size_t)np, nz, E->k.sc1);
    return VEC_OK;
}

// ============================================================================
// hydro_deriv
// ============================================================================
struct HydroArgs {
    const double *r, *t, *u, *v, *w, *bx, *by, *bz, *jsq;
    const double *rx, *tx, *txx, *ux, *uxx, *vx, *vxx, *wx, *wxx;
    const double *ry, *ty, *tyy, *uy, *uyy, *vy, *vyy, *wy, *wyy;
    const double *kappa, *dkappa, *eta;
    const HistTable *ht;    // tdot = newest slot of t
    double *racc, *uacc, *vacc, *wacc;
    double *p1, *p2, *q, *g, *hh, *p3, *p4;
    double gck, fzckg, gm1, sckg, fo2, scko3, f, thmplus1, cor, cpsi, spsi, sck, zck, ho12, sc1;
    int var_eta;
    size_t np;
    int nz;
};

// pass 2: src/hydro_deriv.f90:45-53, 82-110, 139-168, 201-219, 245-261,
// 287-309, 360-367, 390-398, 421-432 (every term without a second-level
// derivative); the energy equation is complete here.
// (three CTAs per SM, 80 registers: 2.68 ms at 256^2 x 129 against 2.74 at
// the compiler's own 96 registers and two CTAs, 2.84 at 120 registers)
__global__ void __launch_bounds__(256, 3) k_hydro_pass2(HydroArgs a)
{
    PDL_WAIT();
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= a.np * a.nz) return;
    const int nz = a.nz;
    const size_t np = a.np;
    const int k = (int)(idx / np);
    const size_t q = idx - (size_t)k * np;
    const double h = a.ho12, s = a.sc1;

    const double rr = a.r[idx], tt = a.t[idx], u0 = a.u[idx], v0 = a.v[idx], w0 = a.w[idx];
    const double bx = a.bx[idx], by = a.by[idx], bz = a.bz[idx];
    const double rx = a.rx[idx], ry = a.ry[idx];
    const double tx = a.tx[idx], txx = a.txx[idx], ty = a.ty[idx], tyy = a.tyy[idx];
    const double ux = a.ux[idx], uxx = a.uxx[idx], uy = a.uy[idx], uyy = a.uyy[idx];
    const double vx = a.vx[idx], vxx = a.vxx[idx], vy = a.vy[idx], vyy = a.vyy[idx];
    const double wx = a.wx[idx], wxx = a.wxx[idx], wy = a.wy[idx], wyy = a.wyy[idx];

    // z derivatives (flags: src/hydro_deriv.f90:66-68, 124-125, 233, 275, 349-350)
    const double tzu = zd1up(a.t + q, np, k, nz, 5, h, w0);
    const double tz = zd1(a.t + q, np, k, nz, 5, h);
    const double tzz = zd2(a.t + q, np, k, nz, 0, s);
    const double wzu = zd1up(a.w + q, np, k, nz, 1, h, w0);
    const double wz = zd1(a.w + q, np, k, nz, 1, h);
    const double uzu = zd1up(a.u + q, np, k, nz, 2, h, w0);
    const double vzu = zd1up(a.v + q, np, k, nz, 2, h, w0);
    const double uzz = zd2(a.u + q, np, k, nz, 3, s);
    const double vzz = zd2(a.v + q, np, k, nz, 3, s);

    const double third = 1.0 / 3.0;
    const double ohm = a.var_eta ? a.eta[k] / a.zck : 1.0;
    const double divu = ux + vy + wz;

    // continuity: :48, :149 (the w d(rho)/dz term is added in pass 4)
    a.racc[idx] = -u0 * rx - v0 * ry - rr * divu;

    // energy (rho * dT/dt): :88-102, :150-151, :216, :258, :300, then / rho
    double td = -rr * (u0 * tx + v0 * ty + w0 * tzu)
                + a.gck * a.kappa[k] * (txx + tyy + tzz)
                + a.gck * a.dkappa[k] * tzu
                + a.fzckg * ohm * a.jsq[idx];
    td = td - a.gm1 * tt * divu * rr + 2 * a.sckg * (ux * ux + vy * vy + wz * wz - third * divu * divu);
    td = td + a.sckg * (uy + vx) * (uy + vx);
    td = td + a.sckg * (wx + uzu) * (wx + uzu);
    td = td + a.sckg * (wy + vzu) * (wy + vzu);
    ((double *)a.ht->p[1][2])[idx] = td * (1.0 / rr);

    // momentum: :103-105, :159-161, :213-214, :253-254, :292-306, :363-364, :393-395, :424-426
    double ud = -tt * rx - rr * tx;
    ud = ud - rr * u0 * ux - rr * v0 * uy - rr * w0 * uzu;
    ud = ud - rr * a.cor * (w0 * a.cpsi + v0 * a.spsi);
    ud = ud + a.sck * uzz + a.sck * uxx + a.sck * uyy;
    double vd = -tt * ry - rr * ty;
    vd = vd - rr * v0 * vy - rr * u0 * vx - rr * w0 * vzu;
    vd = vd - rr * a.cor * (-u0 * a.spsi);
    vd = vd + a.sck * vzz + a.sck * vxx + a.sck * vyy;
    double wd = -rr * tz;
    wd = wd - rr * w0 * wzu + a.thmplus1 * rr - rr * u0 * wx - rr * v0 * wy;
    wd = wd - rr * a.cor * (-u0 * a.cpsi);
    wd = wd + a.sck * wxx + a.sck * wyy;
    a.uacc[idx] = ud;
    a.vacc[idx] = vd;
    a.wacc[idx] = wd;

    // second-level inputs: :152-165, :215, :255-257, :297-299
    const double temp1 = a.fo2 * bx * bx, temp2 = a.fo2 * by * by, temp3 = a.fo2 * bz * bz;
    const double dv = a.scko3 * divu;
    a.p1[idx] = dv + temp1 - temp2 - temp3;
    a.p2[idx] = dv + temp2 - temp1 - temp3;
    a.p3[idx] = a.scko3 * ux + a.scko3 * vy + temp3 - temp1 - temp2;
    a.p4[idx] = 4.0 * a.scko3 * wz;
    a.q[idx] = a.f * by * bx;
    a.g[idx] = a.f * bz * bx;
    a.hh[idx] = a.f * bz * by;
}

struct Hydro4Args {
    const double *r, *t, *w, *p3, *p4, *g, *hh, *racc, *uacc, *vacc, *wacc;
    const HistTable *ht;    // rdot, udot, vdot, wdot = newest slots
    double ho12;
    size_t np;
    int nz;
};

// pass 4: :183-184, :272, :321 (z derivatives of second-level inputs),
// :443-497 (d(rho)/dz with the boundary override, division by rho)
__global__ void k_hydro_pass4(Hydro4Args a)
{
    PDL_WAIT();
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= a.np * a.nz) return;
    const int nz = a.nz;
    const size_t np = a.np;
    const int k = (int)(idx / np);
    const size_t q = idx - (size_t)k * np;
    const double h = a.ho12;
    const double w0 = a.w[idx], tt = a.t[idx], rr = a.r[idx];
    double wd = a.wacc[idx] + zd1(a.p3 + q, np, k, nz, 2, h) + zd1(a.p4 + q, np, k, nz, 5, h);
    double ud = a.uacc[idx] + zd1(a.g + q, np, k, nz, 5, h);
    double vd = a.vacc[idx] + zd1(a.hh + q, np, k, nz, 5, h);
    double rzu, rz;
    if (k == 0 || k == nz - 1) {
        rzu = wd / tt;
        rz = wd / tt;
    } else {
        rzu = zd1up(a.r + q, np, k, nz, 0, h, w0);
        rz = zd1(a.r + q, np, k, nz, 0, h);
    }
    ((double *)a.ht->p[0][2])[idx] = a.racc[idx] - w0 * rzu;
    wd = wd - tt * rz;
    const double ri = 1.0 / rr;
    ((double *)a.ht->p[2][2])[idx] = ud * ri;
    ((double *)a.ht->p[3][2])[idx] = vd * ri;
    ((double *)a.ht->p[4][2])[idx] = wd * ri;
}

int phys_hydro64(Engine *E)
{
    double *W[W_COUNT];
    for (int i = 0; i < W_COUNT; i++) W[i] = E->W<double>(i);
    int st;
    // pass 1: horizontal derivatives (:33-34, :64-65, :122-123, :190-191,
    // :232, :274, :378-380, :409-411)
    LineJob<double> jx[5] = {
        ljob<double>(E->r, W[W_RX], OP_D1),
        ljob<double>(E->t, W[W_TX], OP_D1, W[W_TXX], OP_D2),
        ljob<double>(E->u, W[W_UX], OP_D1, W[W_UXX], OP_D2),
        ljob<double>(E->v, W[W_VX], OP_D1, W[W_VXX], OP_D2),
        ljob<double>(E->w, W[W_WX], OP_D1, W[W_WXX], OP_D2),
    };
    if ((st = launch_lines<double>(E, 0, jx, 5))) return st;
    LineJob<double> jy[5] = {
        ljob<double>(E->r, W[W_RY], OP_D1),
        ljob<double>(E->t, W[W_TY], OP_D1, W[W_TYY], OP_D2),
        ljob<double>(E->u, W[W_UY], OP_D1, W[W_UYY], OP_D2),
        ljob<double>(E->v, W[W_VY], OP_D1, W[W_VYY], OP_D2),
        ljob<double>(E->w, W[W_WY], OP_D1, W[W_WYY], OP_D2),
    };
    if ((st = launch_lines<double>(E, 1, jy, 5))) return st;

    HydroArgs a;
    a.r = E->r; a.t = E->t; a.u = E->u; a.v = E->v; a.w = E->w;
    a.bx = E->bx; a.by = E->by; a.bz = E->bz; a.jsq = E->jsq;
    a.rx = W[W_RX]; a.tx = W[W_TX]; a.txx = W[W_TXX]; a.ux = W[W_UX]; a.uxx = W[W_UXX];
    a.vx = W[W_VX]; a.vxx = W[W_VXX]; a.wx = W[W_WX]; a.wxx = W[W_WXX];
    a.ry = W[W_RY]; a.ty = W[W_TY]; a.tyy = W[W_TYY]; a.uy = W[W_UY]; a.uyy = W[W_UYY];
    a.vy = W[W_VY]; a.vyy = W[W_VYY]; a.wy = W[W_WY]; a.wyy = W[W_WYY];
    a.kappa = E->kappa; a.dkappa = E->dkappa; a.eta = E->eta;
    a.racc = W[W_RACC]; a.ht = E->ht;
    a.uacc = W[W_UACC]; a.vacc = W[W_VACC]; a.wacc = W[W_WACC];
    a.p1 = W[W_P1]; a.p2 = W[W_P2]; a.q = W[W_Q]; a.g = W[W_G]; a.hh = W[W_H];
    a.p3 = W[W_P3]; a.p4 = W[W_P4];
    const Consts &c = E->k;
    a.gck = c.gck; a.fzckg = c.fzckg; a.gm1 = c.gm1; a.sckg = c.sckg; a.fo2 = c.fo2;
    a.scko3 = c.scko3; a.f = c.f; a.thmplus1 = c.thmplus1; a.cor = c.cor; a.cpsi = c.cpsi;
    a.spsi = c.spsi; a.sck = c.sck; a.zck = c.zck; a.ho12 = c.ho12; a.sc1 = c.sc1;
    a.var_eta = c.var_eta; a.np = E->np; a.nz = E->nz;
    KLAUNCHB(E, "hydro_pass2_f64", FB(E, 39, 8), k_hydro_pass2, nblk(E->n), TPB, a);

    // pass 3: d/dx, d/dy of the second-level inputs into the accumulators
    // (:181-182, :230-231, :273, :320)
    LineJob<double> kx[3] = {
        ljob<double>(W[W_P1], W[W_UACC], OP_D1, nullptr, OP_NONE, 1),
        ljob<double>(W[W_Q], W[W_VACC], OP_D1, nullptr, OP_NONE, 1),
        ljob<double>(W[W_G], W[W_WACC], OP_D1, nullptr, OP_NONE, 1),
    };
    if ((st = launch_lines<double>(E, 0, kx, 3))) return st;
    LineJob<double> ky[3] = {
        ljob<double>(W[W_P2], W[W_VACC], OP_D1, nullptr, OP_NONE, 1),
        ljob<double>(W[W_Q], W[W_UACC], OP_D1, nullptr, OP_NONE, 1),
        ljob<double>(W[W_H], W[W_WACC], OP_D1, nullptr, OP_NONE, 1),
    };
    if ((st = launch_lines<double>(E, 1, ky, 3))) return st;

    Hydro4Args b;
    b.r = E->r; b.t = E->t; b.w = E->w; b.p3 = W[W_P3]; b.p4 = W[W_P4]; b.g = W[W_G]; b.hh = W[W_H];
    b.racc = W[W_RACC]; b.uacc = W[W_UACC]; b.vacc = W[W_VACC]; b.wacc = W[W_WACC];
    b.ht = E->ht;
    b.ho12 = c.ho12; b.np = E->np; b.nz = E->nz;
    KLAUNCHB(E, "hydro_pass4_f64", FB(E, 15, 8), k_hydro_pass4, nblk(E->n), TPB, b);
    return VEC_OK;
}

// ============================================================================
// mag_deriv: src/magnetic.f90:285-487 (+ eta(z) extension)
// ============================================================================
int phys_mag64(Engine *E)
{
    double *W[W_COUNT];
    for (int i = 0; i < W_COUNT; i++) W[i] = E->W<double>(i);
    int st;
    KLAUNCHB(E, "emf_f64", FB(E, 9, 8), k_emf<double>, nblk(E->n), TPB, E->u, E->v, E->w, E->bx, E->by, E->bz, W[W_M1], W[W_M2], W[W_M3], E->n, 0.0);
    // forwardfft x3 (:321-323): x pass then y pass in place
    LineJob<double> fx[3] = { ljob<double>(W[W_M1], W[W_EX], OP_FWD), ljob<double>(W[W_M2], W[W_EY], OP_FWD),
                              ljob<double>(W[W_M3], W[W_EZ], OP_FWD) };
    if ((st = launch_lines<double>(E, 0, fx, 3))) return st;
    LineJob<double> fy[3] = { ljob<double>(W[W_EX], W[W_EX], OP_FWD), ljob<double>(W[W_EY], W[W_EY], OP_FWD),
                              ljob<double>(W[W_EZ], W[W_EZ], OP_FWD) };
    if ((st = launch_lines<double>(E, 1, fy, 3))) return st;
    const Consts &c = E->k;
    MeanArgs<double> ma;
    ma.ex = W[W_EX]; ma.ey = W[W_EY]; ma.bxbar = E->bxbar; ma.bybar = E->bybar; ma.eta = E->eta; ma.deta = E->deta;
    ma.ht = E->ht; ma.scratch = E->w1d; ma.np = E->np; ma.nz = E->nz;
    ma.xn = c.xn; ma.zck = c.zck; ma.ho12 = c.ho12; ma.sc1 = c.sc1; ma.var_eta = c.var_eta;
    ma.ds = nullptr; ma.bxm = nullptr; ma.bym = nullptr;
    KLAUNCH(E, "mean_rhs", k_mean_rhs<double>, 1, 256, ma);
    KLAUNCHB(E, "mag_div_f64", FB(E, 3, 8), k_mag_div<double>, plane_grid(*E), TPB, W[W_EX], W[W_EY], W[W_M4],
             E->nx, E->ny, E->hd);
    MagArgs<double> a;
    a.ex = W[W_EX]; a.ey = W[W_EY]; a.ez = W[W_EZ]; a.w1 = W[W_M4]; a.pol = E->pol; a.tor = E->tor;
    a.eta = E->eta; a.deta = E->deta; a.h = E->hd;
    a.ht = E->ht;
    a.zck = c.zck; a.ho12 = c.ho12; a.sc1 = c.sc1; a.var_eta = c.var_eta;
    a.nx = E->nx; a.ny = E->ny; a.nz = E->nz;
    KLAUNCHB(E, "mag_final_f64", FB(E, 8, 8), k_mag_final<double>, plane_grid(*E), TPB, a);
    return VEC_OK;
}

int phys_zero_mag_rhs_m(Engine *const *Es, int nE)
{
    Engine *E = Es[0];
    size_t cnt = E->n > (size_t)E->nz ? E->n : (size_t)E->nz;
    auto mk = [](Engine *e) { return ZeroMagArgs{ e->ht, e->n, e->nz }; };
    if (E->split)
        return launch_members<ZeroMagArgs>(Es, nE, "zero_mag_rhs", 0.0, dim3(nblk(cnt)), dim3(TPB), 0,
                                           k_zero_mag_rhs<float, 1>, k_zero_mag_rhs<float, BATCH_MAX>, mk);
    return launch_members<ZeroMagArgs>(Es, nE, "zero_mag_rhs", 0.0, dim3(nblk(cnt)), dim3(TPB), 0,
                                       k_zero_mag_rhs<double, 1>, k_zero_mag_rhs<double, BATCH_MAX>, mk);
}
int phys_zero_mag_rhs(Engine *E) { return phys_zero_mag_rhs_m(&E, 1); }

// ============================================================================
// bandj: src/magnetic.f90:492-664
// ============================================================================
int phys_bandj64(Engine *E)
{
    double *W[W_COUNT];
    for (int i = 0; i < W_COUNT; i++) W[i] = E->W<double>(i);
    int st;
    if ((st = op_d1z(E, E->pol, W[W_M1], 5, (int)E->np, E->nz))) return st;   // :519
    BandjArgs<double> a;
    a.dzs = W[W_M1]; a.pol = E->pol; a.tor = E->tor; a.h = E->hd;
    a.bxh = W[W_EX]; a.byh = W[W_EY]; a.bzh = W[W_EZ]; a.dybz = W[W_M2]; a.dxbz = W[W_M3]; a.jzh = W[W_M4];
    a.nx = E->nx; a.ny = E->ny; a.nz = E->nz;
    KLAUNCHB(E, "bandj_spec_f64", FB(E, 9, 8), k_bandj_spec<double>, plane_grid(*E), TPB, a);
    // six inverse 2-D transforms (:575-577, :623-625): x pass in place, then y
    LineJob<double> ix[6] = { ljob<double>(W[W_EX], W[W_EX], OP_INV), ljob<double>(W[W_EY], W[W_EY], OP_INV),
                              ljob<double>(W[W_EZ], W[W_EZ], OP_INV), ljob<double>(W[W_M2], W[W_M2], OP_INV),
                              ljob<double>(W[W_M3], W[W_M3], OP_INV), ljob<double>(W[W_M4], W[W_M4], OP_INV) };
    if ((st = launch_lines<double>(E, 0, ix, 6))) return st;
    LineJob<double> iy[6] = { ljob<double>(W[W_EX], E->bx, OP_INV), ljob<double>(W[W_EY], E->by, OP_INV),
                              ljob<double>(W[W_EZ], E->bz, OP_INV), ljob<double>(W[W_M2], W[W_M2], OP_INV),
                              ljob<double>(W[W_M3], W[W_M3], OP_INV), ljob<double>(W[W_M4], W[W_M4], OP_INV) };
    iy[0].addk = E->bxbar;       // :587-589
    iy[1].addk = E->bybar;
    iy[2].addc = E->bzbar;
    if ((st = launch_lines<double>(E, 1, iy, 6))) return st;
    KLAUNCHB(E, "jsq_f64", FB(E, 6, 8), k_jsq<double>, plane_grid(*E), TPB, W[W_M4], W[W_M2], W[W_M3], E->bx,
             E->by, E->jsq, E->np, E->nz, E->k.ho12);
    return VEC_OK;
}

// ============================================================================
// magdealias (src/magnetic.f90:666-717) and spectral truncation
// ============================================================================
int phys_magdealias(Engine *E)
{
    KLAUNCH(E, "magdealias_f64", k_truncate<double>, plane_grid(*E), TPB, E->pol, E->tor, E->nx, E->ny, E->nz,
            E->k.icutoffx, E->k.icutoffy);
    return VEC_OK;
}

// ============================================================================
// boundary conditions: src/dbydz.F90:3686-4197 and :4205-4791
// ============================================================================
// In the split form (m != nullptr) the FP32 mirrors of the two boundary
// planes are written here too: m = {u32, v32, w32, t32}, t0 = T0(z).
__device__ __forceinline__ void boundary_column(double *u, double *v, double *w, double *t, size_t np, int nz,
                                                double theta, double dz, int radbc, int constflux,
                                                const BoundaryMirrors &mb, size_t q)
{
    const double elf = 1.0 / 11.0;
#define P(f, kk) f[(size_t)(kk) * np + q]
    P(w, 0) = 0.0;
    P(u, 0) = elf * (18.0 * P(u, 1) - 9.0 * P(u, 2) + 2.0 * P(u, 3));
    P(v, 0) = elf * (18.0 * P(v, 1) - 9.0 * P(v, 2) + 2.0 * P(v, 3));
    P(w, nz - 1) = 0.0;
    P(u, nz - 1) = elf * (18.0 * P(u, nz - 2) - 9.0 * P(u, nz - 3) + 2.0 * P(u, nz - 4));
    P(v, nz - 1) = elf * (18.0 * P(v, nz - 2) - 9.0 * P(v, nz - 3) + 2.0 * P(v, nz - 4));
    if (radbc) {   // :4036-4055, Newton iterations on the radiative condition
        double t1old = P(t, 0);
        for (int it = 0; it < 10; it++) {
            double ft1 = 6.0 * theta * dz * t1old * t1old * t1old * t1old + 11.0 * t1old - 18.0 * P(t, 1)
                         + 9.0 * P(t, 2) - 2.0 * P(t, 3);
            double dft1 = 24.0 * theta * dz * t1old * t1old * t1old + 11.0;
            t1old = t1old - (ft1 / dft1);
        }
        P(t, 0) = t1old;
    } else {
        P(t, 0) = 1.0;
    }
    if (constflux)
        P(t, nz - 1) = elf * (18.0 * P(t, nz - 2) - 9.0 * P(t, nz - 3) + 2.0 * P(t, nz - 4) + 6.0 * theta * dz);
    else
        P(t, nz - 1) = 1.0 + theta;
    if (mb.u32) {
        const int ks[2] = { 0, nz - 1 };
        for (int e = 0; e < 2; e++) {
            const int kk = ks[e];
            mb.u32[(size_t)kk * np + q] = d2f_rn(P(u, kk));
            mb.v32[(size_t)kk * np + q] = d2f_rn(P(v, kk));
            mb.w32[(size_t)kk * np + q] = d2f_rn(P(w, kk));
            mb.t32[(size_t)kk * np + q] = d2f_rn(P(t, kk) - mb.t0[kk]);
        }
    }
#undef P
}

// arguments of k_boundary / k_boundaries
struct BndArgs {
    double *u, *v, *w, *t, *pol, *tor, *bxb, *byb;
    size_t np;
    int nz;
    double theta, dz;
    int radbc, constflux, perfect;
    BoundaryMirrors mb;
};

static BndArgs bnd_args(Engine *E)
{
    BndArgs a;
    BoundaryMirrors mb = {};
    if (E->split) {
        mb.u32 = E->u32; mb.v32 = E->v32; mb.w32 = E->w32; mb.t32 = E->t32; mb.t0 = split_bg_t0(E);
        mb.pol32 = E->pol32; mb.tor32 = E->tor32;
    }
    a.u = E->u; a.v = E->v; a.w = E->w; a.t = E->t; a.pol = E->pol; a.tor = E->tor; a.bxb = E->bxbar; a.byb = E->bybar;
    a.np = E->np; a.nz = E->nz; a.theta = E->p.theta; a.dz = E->k.dz;
    a.radbc = E->p.radbc; a.constflux = E->p.constflux; a.perfect = E->p.perfect; a.mb = mb;
    return a;
}

template <int NB>
__global__ void k_boundary(const __grid_constant__ Batch<BndArgs, NB> bt)
{
    PDL_WAIT();
    const BndArgs &a = BATCH_MEMBER(bt, NB);
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < a.np) boundary_column(a.u, a.v, a.w, a.t, a.np, a.nz, a.theta, a.dz, a.radbc, a.constflux, a.mb, q);
}

int phys_boundary_m(Engine *const *Es, int nE)
{
    return launch_members<BndArgs>(Es, nE, "boundary_f64", 0.0, dim3(nblk(Es[0]->np)), dim3(TPB), 0, k_boundary<1>,
                                   k_boundary<BATCH_MAX>, bnd_args);
}
int phys_boundary(Engine *E) { return phys_boundary_m(&E, 1); }

__device__ __forceinline__ void mag_boundary_column(double *pol, double *tor, double *bxb, double *byb, size_t np,
                                                    int nz, int perfect, const BoundaryMirrors &mb, size_t q)
{
    const double elf = 1.0 / 11.0;
    if (q == 0) {
        if (perfect) {
            bxb[0] = elf * (18.0 * bxb[1] - 9.0 * bxb[2] + 2.0 * bxb[3]);
            byb[0] = elf * (18.0 * byb[1] - 9.0 * byb[2] + 2.0 * byb[3]);
            bxb[nz - 1] = elf * (18.0 * bxb[nz - 2] - 9.0 * bxb[nz - 3] + 2.0 * bxb[nz - 4]);
            byb[nz - 1] = elf * (18.0 * byb[nz - 2] - 9.0 * byb[nz - 3] + 2.0 * byb[nz - 4]);
        } else {
            bxb[0] = 0.0; byb[0] = 0.0; bxb[nz - 1] = 0.0; byb[nz - 1] = 0.0;
        }
    }
    if (q >= np) return;
#define P(f, kk) f[(size_t)(kk) * np + q]
    if (perfect) {   // :4407-4560
        P(pol, 0) = 0.0;
        P(tor, 0) = elf * (18.0 * P(tor, 1) - 9.0 * P(tor, 2) + 2.0 * P(tor, 3));
        P(pol, nz - 1) = 0.0;
        P(tor, nz - 1) = elf * (18.0 * P(tor, nz - 2) - 9.0 * P(tor, nz - 3) + 2.0 * P(tor, nz - 4));
    } else {         // :4663-4780
        P(tor, 0) = 0.0;
        P(pol, 0) = elf * (18.0 * P(pol, 1) - 9.0 * P(pol, 2) + 2.0 * P(pol, 3));
        P(tor, nz - 1) = 0.0;
        P(pol, nz - 1) = elf * (18.0 * P(pol, nz - 2) - 9.0 * P(pol, nz - 3) + 2.0 * P(pol, nz - 4));
    }
    if (mb.pol32) {
        mb.pol32[q] = d2f_rn(P(pol, 0));
        mb.tor32[q] = d2f_rn(P(tor, 0));
        mb.pol32[(size_t)(nz - 1) * np + q] = d2f_rn(P(pol, nz - 1));
        mb.tor32[(size_t)(nz - 1) * np + q] = d2f_rn(P(tor, nz - 1));
    }
#undef P
}

__global__ void k_mag_boundary(double *pol, double *tor, double *bxb, double *byb, size_t np, int nz, int perfect,
                               BoundaryMirrors mb)
{
    PDL_WAIT();
    mag_boundary_column(pol, tor, bxb, byb, np, nz, perfect, mb, (size_t)blockIdx.x * blockDim.x + threadIdx.x);
}

// boundary and mag_boundary of one step in one launch (disjoint fields)
template <int NB>
__global__ void k_boundaries(const __grid_constant__ Batch<BndArgs, NB> bt)
{
    PDL_WAIT();
    const BndArgs &a = BATCH_MEMBER(bt, NB);
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < a.np) boundary_column(a.u, a.v, a.w, a.t, a.np, a.nz, a.theta, a.dz, a.radbc, a.constflux, a.mb, q);
    mag_boundary_column(a.pol, a.tor, a.bxb, a.byb, a.np, a.nz, a.perfect, a.mb, q);
}

int phys_boundaries_m(Engine *const *Es, int nE)
{
    return launch_members<BndArgs>(Es, nE, "boundaries", 0.0, dim3(nblk(Es[0]->np)), dim3(TPB), 0, k_boundaries<1>,
                                   k_boundaries<BATCH_MAX>, bnd_args);
}
int phys_boundaries(Engine *E) { return phys_boundaries_m(&E, 1); }

int phys_mag_boundary(Engine *E)
{
    BoundaryMirrors mb = {};
    if (E->split) { mb.pol32 = E->pol32; mb.tor32 = E->tor32; }
    KLAUNCH(E, "mag_boundary_f64", k_mag_boundary, nblk(E->np), TPB, E->pol, E->tor, E->bxbar, E->bybar,
            E->np, E->nz, E->p.perfect, mb);
    return VEC_OK;
}

// ============================================================================
// AB3: src/main.F90:381-489
// ============================================================================
// coefficients (:381-403), dt1/dt2 (:488-489), ttime (:345) and the 1-D mean
// update (:469-476) on one CTA
struct CoefArgs {
    DevScalars *ds;
    double *bxbar, *bybar;
    const HistTable *ht;
    int nz, do_means;
};
template <int NB>
__global__ void k_ab3_coef(const __grid_constant__ Batch<CoefArgs, NB> bt)
{
    PDL_WAIT();
    const CoefArgs &a = BATCH_MEMBER(bt, NB);
    ab3_coef_block(a.ds, a.bxbar, a.bybar, a.ht, a.nz, a.do_means);
}

struct Ab3Args {
    double *x[7];
    int hmap[7];                 // history table row of each state field
    const HistTable *ht;
    const DevScalars *ds;
    int nx, ny, nz, cx, cy, magdealias;
};

// :413-462 with the history shift done by pointer rotation on the host and
// magdealias (:503-509) applied to the new pol/tor
__global__ void k_ab3_update(Ab3Args a)
{
    PDL_WAIT();
    const size_t np = (size_t)a.nx * a.ny;
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= np * a.nz) return;
    const double c0 = a.ds->c0, c1 = a.ds->c1, c2 = a.ds->c2;
#define H(f, s) ((const double *)a.ht->p[a.hmap[f]][s])
#pragma unroll
    for (int f = 0; f < 5; f++)
        a.x[f][idx] = a.x[f][idx] + c0 * H(f, 2)[idx] + c1 * H(f, 1)[idx] + c2 * H(f, 0)[idx];
    // order of the reference: u,v,w,r,t then pol,tor; density floor after all
    if (a.x[3][idx] < 0.05) {
        a.x[3][idx] = 0.05;
        ((double *)a.ht->p[0][1])[idx] = 0.0;   // become slots 1 and 2 after the shift
        ((double *)a.ht->p[0][2])[idx] = 0.0;
    }
    bool trunc = false;
    if (a.magdealias) {
        size_t q = idx % np;
        int j = (int)(q / a.nx), i = (int)(q - (size_t)j * a.nx);
        trunc = truncated(i, j, a.nx, a.ny, a.cx, a.cy);
    }
#pragma unroll
    for (int f = 5; f < 7; f++) {
        double xn = a.x[f][idx] + c0 * H(f, 2)[idx] + c1 * H(f, 1)[idx] + c2 * H(f, 0)[idx];
        a.x[f][idx] = trunc ? 0.0 : xn;
    }
#undef H
}

int phys_rotate_hist_m(Engine *const *Es, int nE)
{
    return launch_members<HistTable *>(Es, nE, "rotate_hist", 0.0, dim3(1), dim3(32), 0, k_rotate_hist<1>,
                                       k_rotate_hist<BATCH_MAX>, [](Engine *e) { return e->ht; });
}
int phys_rotate_hist(Engine *E) { return phys_rotate_hist_m(&E, 1); }

int hist_table_host(Engine *E, HistTable *h)
{
    CUDA_TRY(cudaMemcpyAsync(h, E->ht, sizeof(HistTable), cudaMemcpyDeviceToHost, E->stream));
    CUDA_TRY(cudaStreamSynchronize(E->stream));
    return VEC_OK;
}

int phys_ab3_coef_m(Engine *const *Es, int nE)
{
    return launch_members<CoefArgs>(Es, nE, "ab3_coef", 0.0, dim3(1), dim3(256), 0, k_ab3_coef<1>,
                                    k_ab3_coef<BATCH_MAX>,
                                    [](Engine *e) { return CoefArgs{ e->ds, e->bxbar, e->bybar, e->ht, e->nz, 1 }; });
}
int phys_ab3_coef(Engine *E) { return phys_ab3_coef_m(&E, 1); }

int phys_ab3(Engine *E, int magdealias)
{
    int st = phys_ab3_coef(E);
    if (st) return st;
    Ab3Args a;
    // order of the reference's loop body: u, v, w, r, t, pol, tor
    double *xs[7] = { E->u, E->v, E->w, E->r, E->t, E->pol, E->tor };
    const int hmap[7] = { 2, 3, 4, 0, 1, 5, 6 };
    for (int f = 0; f < 7; f++) {
        a.x[f] = xs[f];
        a.hmap[f] = hmap[f];
    }
    a.ht = E->ht;
    a.ds = E->ds;
    a.nx = E->nx; a.ny = E->ny; a.nz = E->nz; a.cx = E->k.icutoffx; a.cy = E->k.icutoffy;
    a.magdealias = magdealias;
    KLAUNCHB(E, "ab3_update_f64", FB(E, 35, 8), k_ab3_update, nblk(E->n), TPB, a);
    return phys_rotate_hist(E);
}

// dealias(r,t,u,v,w): src/main.F90:495-502 -> src/fft.F90:586-682
int phys_dealias_state(Engine *E)
{
    double *f[5] = { E->r, E->t, E->u, E->v, E->w };
    LineJob<double> j[5];
    int st;
    for (int i = 0; i < 5; i++) j[i] = ljob<double>(f[i], f[i], OP_DEALIAS);
    if ((st = launch_lines<double>(E, 0, j, 5))) return st;
    if ((st = launch_lines<double>(E, 1, j, 5))) return st;
    return VEC_OK;
}

// ============================================================================
// calcdt: src/utils.F90:144-244
// ============================================================================
// order-preserving map of a double onto an unsigned 64-bit key (all
// non-NaN values, negatives included), so that atomicMax/atomicMin on the
// keys give the max/min of the doubles
__device__ __forceinline__ unsigned long long okey(double x)
{
    unsigned long long u = (unsigned long long)__double_as_longlong(x);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double okey_dec(unsigned long long e)
{
    unsigned long long u = (e >> 63) ? (e & 0x7fffffffffffffffull) : ~e;
    return __longlong_as_double((long long)u);
}

// The maxima of src/utils.F90:190-214 need the FP64 expression only at the
// points that can hold them, and GB300's FP64 square roots are slow.  So:
//
// pass 1 (k_calcdt_est): per chunk of CDT_CHUNK points, FP32 estimates of
//   xx = |u_h| + g1 sqrt(T) + sqrt(f B^2 / rho) and xz (|w| in place of |u_h|)
//   and the minimum density, their chunk extrema, and the global extrema;
// pass 2 (k_calcdt_exact): the few chunks whose estimate lies within
//   CDT_MARGIN of the global one evaluate the FP64 expression at every point
//   whose estimate does, and reduce those exact values.
//
// The estimates carry a relative error of a few FP32 ulps (all terms are
// non-negative), far below CDT_MARGIN, so the point holding the exact
// maximum (minimum) always passes both filters.  Estimates only choose
// points; the results are the same FP64 extrema as a full FP64 pass.
#define CDT_CHUNK 8192
#define CDT_MARGIN 1.0e-3f

// order-preserving keys of floats (as okey for doubles)
__device__ __forceinline__ unsigned okey32(float x)
{
    unsigned u = __float_as_uint(x);
    return (u >> 31) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float okey32_dec(unsigned e)
{
    unsigned u = (e >> 31) ? (e & 0x7fffffffu) : ~e;
    return __uint_as_float(u);
}

// initial values of the three global estimate keys
__device__ __forceinline__ void cdt_reset_keys(unsigned *gkey)
{
    gkey[0] = 0u;              // below every float's key
    gkey[1] = 0u;
    gkey[2] = 0xffffffffu;     // above every float's key
    gkey[3] = 0u;              // no non-finite value seen
}
__global__ void k_cdt_init(unsigned *gkey) {
    PDL_WAIT(); cdt_reset_keys(gkey); }
int cdt_init(float *cdt)
{
    k_cdt_init<<<1, 1>>>(reinterpret_cast<unsigned *>(cdt));
    CUDA_TRY(cudaGetLastError());
    return VEC_OK;
}

struct CdtArgs {
    const double *u, *v, *w, *r, *t, *bx, *by, *bz;
    size_t n;
    double g1, f;
    float *chunk;           // [3][nchunks]: xx max, xz max, rho min estimates
    unsigned *gkey;         // [3]: keys of the global estimates
    int nchunks;
    DevScalars *ds;
};

struct CdtEst { float xx, xz, r; };

__device__ __forceinline__ CdtEst cdt_estimate(const CdtArgs &a, size_t i)
{
    // (conversions by truncation on the integer pipe: relative error < 2^-23)
    const float u0 = d2f_est(a.u[i]), v0 = d2f_est(a.v[i]), w0 = d2f_est(a.w[i]), r0 = d2f_est(a.r[i]);
    const float t0 = d2f_est(a.t[i]), bx0 = d2f_est(a.bx[i]), by0 = d2f_est(a.by[i]), bz0 = d2f_est(a.bz[i]);
    const float bsq = bx0 * bx0 + by0 * by0 + bz0 * bz0;
    const float c = (float)a.g1 * sqrtf(t0) + sqrtf((bsq * (float)a.f) / r0);
    CdtEst e;
    e.xx = sqrtf(u0 * u0 + v0 * v0) + c;
    e.xz = fabsf(w0) + c;
    e.r = r0;
    return e;
}

__device__ __forceinline__ void block_reduce3(float &mx, float &mz, float &mn, float *sh)
{
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        mz = fmaxf(mz, __shfl_xor_sync(0xffffffffu, mz, o));
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    }
    const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0) { sh[wid] = mx; sh[32 + wid] = mz; sh[64 + wid] = mn; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < nw; q++) { mx = fmaxf(mx, sh[q]); mz = fmaxf(mz, sh[32 + q]); mn = fminf(mn, sh[64 + q]); }
    }
}

template <int NB>
__global__ void __launch_bounds__(256) k_calcdt_est(const __grid_constant__ Batch<CdtArgs, NB> bt)
{
    PDL_WAIT();
    const CdtArgs &a = BATCH_MEMBER(bt, NB);
    if ((int)blockIdx.x >= a.nchunks) return;
    __shared__ float sh[96];
    const size_t i0 = (size_t)blockIdx.x * CDT_CHUNK;
    const size_t i1 = i0 + CDT_CHUNK < a.n ? i0 + CDT_CHUNK : a.n;
    float mx = -INFINITY, mz = -INFINITY, mn = INFINITY;
    // A NaN or infinity in u, v, w, T, B makes the speed estimates non-finite,
    // and one in rho its own estimate (a negative T or rho gives a NaN square
    // root, as in the FP64 expression); fmaxf / fminf would skip NaNs, so they
    // are counted separately.
    int bad = 0;
    for (size_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const CdtEst e = cdt_estimate(a, i);
        mx = fmaxf(mx, e.xx);
        mz = fmaxf(mz, e.xz);
        mn = fminf(mn, e.r);
        bad |= !(isfinite(e.xx) && isfinite(e.xz) && isfinite(e.r));
    }
    bad = __syncthreads_or(bad);
    block_reduce3(mx, mz, mn, sh);
    if (threadIdx.x == 0) {
        if (bad) atomicOr(&a.gkey[3], 1u);
        a.chunk[blockIdx.x] = mx;
        a.chunk[a.nchunks + blockIdx.x] = mz;
        a.chunk[2 * a.nchunks + blockIdx.x] = mn;
        atomicMax(&a.gkey[0], okey32(mx));
        atomicMax(&a.gkey[1], okey32(mz));
        atomicMin(&a.gkey[2], okey32(mn));
    }
}

template <int NB>
__global__ void __launch_bounds__(256) k_calcdt_exact(const __grid_constant__ Batch<CdtArgs, NB> bt)
{
    PDL_WAIT();
    const CdtArgs &a = BATCH_MEMBER(bt, NB);
    if ((int)blockIdx.x >= a.nchunks) return;
    const float gx = okey32_dec(a.gkey[0]), gz = okey32_dec(a.gkey[1]), gr = okey32_dec(a.gkey[2]);
    // thresholds a relative margin below (above) the estimates; scaling
    // keeps infinite estimates infinite
    const float tx = gx * (gx >= 0.0f ? 1.0f - CDT_MARGIN : 1.0f + CDT_MARGIN);
    const float tz = gz * (gz >= 0.0f ? 1.0f - CDT_MARGIN : 1.0f + CDT_MARGIN);
    const float tr = gr * (gr >= 0.0f ? 1.0f + CDT_MARGIN : 1.0f - CDT_MARGIN);
    const int c = blockIdx.x;
    const bool fx = a.chunk[c] >= tx, fz = a.chunk[a.nchunks + c] >= tz, fr = a.chunk[2 * a.nchunks + c] <= tr;
    if (!(fx || fz || fr)) return;
    const size_t i0 = (size_t)c * CDT_CHUNK;
    const size_t i1 = i0 + CDT_CHUNK < a.n ? i0 + CDT_CHUNK : a.n;
    double mxx = -1.0e-50, mxz = -1.0e-50, mn = 1.0e300;
    for (size_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const CdtEst e = cdt_estimate(a, i);
        const bool px = fx && e.xx >= tx, pz = fz && e.xz >= tz;
        if (px || pz) {
            // src/utils.F90:190-205, in FP64
            const double u0 = a.u[i], v0 = a.v[i], w0 = a.w[i], r0 = a.r[i], t0 = a.t[i];
            const double bz0 = a.bz[i], bx0 = a.bx[i], by0 = a.by[i];
            const double bsq0 = bx0 * bx0 + by0 * by0 + bz0 * bz0;
            const double cc = a.g1 * sqrt(t0);
            const double cb = sqrt((bsq0 * a.f) / r0);
            if (px) mxx = fmax(mxx, sqrt(u0 * u0 + v0 * v0) + cc + cb);
            if (pz) mxz = fmax(mxz, sqrt(w0 * w0) + cc + cb);
        }
        if (fr && e.r <= tr) mn = fmin(mn, a.r[i]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mxx = fmax(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
        mxz = fmax(mxz, __shfl_xor_sync(0xffffffffu, mxz, o));
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&a.ds->velmxx, okey(mxx));
        atomicMax(&a.ds->velmxz, okey(mxz));
        atomicMin(&a.ds->denmn, okey(mn));
    }
}

struct CdtFinArgs {
    DevScalars *ds;
    unsigned *gkey;
    double dd, dz, dtvisc0x, dtvisc0z, dtdiff0x, dtdiff0z, sf;
    int var_eta;
    double eta_max;
};
template <int NB>
__global__ void k_calcdt_fin(const __grid_constant__ Batch<CdtFinArgs, NB> bt)
{
    PDL_WAIT();
    const CdtFinArgs &A = BATCH_MEMBER(bt, NB);
    DevScalars *ds = A.ds;
    unsigned *gkey = A.gkey;
    const double dd = A.dd, dz = A.dz, dtvisc0x = A.dtvisc0x, dtvisc0z = A.dtvisc0z, dtdiff0x = A.dtdiff0x;
    const double dtdiff0z = A.dtdiff0z, sf = A.sf, eta_max = A.eta_max;
    const int var_eta = A.var_eta;
    double velmxx = okey_dec(ds->velmxx);
    double velmxz = okey_dec(ds->velmxz);
    double denmn = okey_dec(ds->denmn);
    double m = 0.16 * dd / velmxx;
    m = fmin(m, 0.3 * dz / velmxz);
    m = fmin(m, dtvisc0x * denmn);
    m = fmin(m, dtvisc0z * denmn);
    m = fmin(m, dtdiff0x * denmn);
    m = fmin(m, dtdiff0z * denmn);
    if (var_eta) {   // extension: explicit magnetic diffusion limits for eta(z)
        m = fmin(m, 0.1 * dd * dd / eta_max);
        m = fmin(m, 0.2 * dz * dz / eta_max);
    }
    ds->dt = sf * m;
    ds->nonfinite = gkey[3] != 0u;
    ds->res[60] = velmxx; ds->res[61] = velmxz; ds->res[62] = denmn;
    ds->velmxx = OKEY_NEG_HUGE; ds->velmxz = OKEY_NEG_HUGE; ds->denmn = OKEY_POS_HUGE;
    cdt_reset_keys(gkey);
}

int cdt_chunks(size_t n) { return (int)((n + CDT_CHUNK - 1) / CDT_CHUNK); }

static CdtArgs cdt_args(Engine *E)
{
    CdtArgs a;
    a.u = E->u; a.v = E->v; a.w = E->w; a.r = E->r; a.t = E->t; a.bx = E->bx; a.by = E->by; a.bz = E->bz;
    a.n = E->n; a.g1 = E->k.g1; a.f = E->k.f;
    a.nchunks = cdt_chunks(E->n);
    a.gkey = reinterpret_cast<unsigned *>(E->cdt);
    a.chunk = E->cdt + 4;
    a.ds = E->ds;
    return a;
}

int phys_calcdt_m(Engine *const *Es, int nE)
{
    Engine *E = Es[0];
    const unsigned nch = (unsigned)cdt_chunks(E->n);
    int st;
    if ((st = launch_members<CdtArgs>(Es, nE, "calcdt_est_f64", FB(E, 8, 8), dim3(nch), dim3(256), 0,
                                      k_calcdt_est<1>, k_calcdt_est<BATCH_MAX>, cdt_args)))
        return st;
    if ((st = launch_members<CdtArgs>(Es, nE, "calcdt_exact", 0.0, dim3(nch), dim3(256), 0, k_calcdt_exact<1>,
                                      k_calcdt_exact<BATCH_MAX>, cdt_args)))
        return st;
    return launch_members<CdtFinArgs>(Es, nE, "calcdt_fin", 0.0, dim3(1), dim3(1), 0, k_calcdt_fin<1>,
                                      k_calcdt_fin<BATCH_MAX>, [](Engine *e) {
                                          const Consts &c = e->k;
                                          return CdtFinArgs{ e->ds, reinterpret_cast<unsigned *>(e->cdt), c.dd, c.dz,
                                                             c.dtvisc0x, c.dtvisc0z, c.dtdiff0x, c.dtdiff0z, c.sf,
                                                             c.var_eta, c.eta_max };
                                      });
}
int phys_calcdt(Engine *E) { return phys_calcdt_m(&E, 1); }

// ============================================================================
// diagnostics: GlobalAverages (src/utils.F90:22-139), nusselt
// (src/dbydz.F90:4877-4921), checkdivb (src/utils.F90:249-318), sminmax
// ============================================================================
// per-plane sums: rav, urav, vrav, keav, bsqav (one CTA per plane, fixed order)
__global__ void k_plane_sums(const double *r, const double *u, const double *v, const double *w,
                             const double *bx, const double *by, const double *bz, size_t np, double *out)
{
    PDL_WAIT();
    const int k = blockIdx.x;
    const size_t base = (size_t)k * np;
    double s[5] = { 0, 0, 0, 0, 0 };
    for (size_t i = threadIdx.x; i < np; i += blockDim.x) {
        size_t q = base + i;
        double uu = u[q], vv = v[q], rr = r[q], ww = w[q];
        s[0] += rr;
        s[1] += rr * uu;
        s[2] += rr * vv;
        s[3] += 0.5 * rr * (uu * uu + vv * vv + ww * ww);
        s[4] += bx[q] * bx[q] + by[q] * by[q] + bz[q] * bz[q];
    }
    __shared__ double sh[5][256];
    for (int m = 0; m < 5; m++) sh[m][threadIdx.x] = s[m];
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int m = 0; m < 5; m++) sh[m][threadIdx.x] += sh[m][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x < 5) out[(size_t)k * 8 + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void k_sub_mean(double *u, double *v, size_t n, const DevScalars *ds)
{
    PDL_WAIT();
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    u[i] = u[i] - ds->res[0];
    v[i] = v[i] - ds->res[1];
}

__global__ void k_globalavg_fin(const double *ps, int nz, double xzn, DevScalars *ds)
{
    PDL_WAIT();
    double urbar = 0, vrbar = 0, rbar = 0, me = 0, ke = 0;
    for (int k = 0; k < nz; k++) {
        const double *p = ps + (size_t)k * 8;
        if (k == 0 || k == nz - 1) {
            urbar += 0.5 * p[1]; vrbar += 0.5 * p[2]; rbar += 0.5 * p[0];
            me += 0.25 * p[4]; ke += 0.5 * p[3];
        } else {
            urbar += p[1]; vrbar += p[2]; rbar += p[0]; me += 0.5 * p[4]; ke += p[3];
        }
    }
    ds->res[0] = urbar / rbar;
    ds->res[1] = vrbar / rbar;
    ds->res[2] = ke * xzn;
    ds->res[3] = me * xzn;
}

// block partial min/max of 11 quantities + divB, and the Nusselt plane sum
#define NMM 12
__global__ void k_minmax(const double *r, const double *t, const double *u, const double *v, const double *w,
                         const double *bx, const double *by, const double *bz, const double *dxbx,
                         const double *dyby, size_t np, int nz, double ho12, double *out)
{
    PDL_WAIT();
    double mn[NMM], mx[NMM];
    for (int m = 0; m < NMM; m++) { mn[m] = 1.0e300; mx[m] = -1.0e300; }
    const size_t n = np * nz;
    int bad = 0;    // a NaN or infinity among the state values or div B (fmin / fmax skip NaNs)
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        int k = (int)(i / np);
        size_t q = i - (size_t)k * np;
        double vals[NMM];
        double uu = u[i], vv = v[i], ww = w[i];
        vals[0] = r[i]; vals[1] = t[i]; vals[2] = uu; vals[3] = vv; vals[4] = ww;
        vals[5] = bx[i]; vals[6] = by[i]; vals[7] = bz[i];
        vals[8] = (uu * uu + vv * vv + ww * ww) / t[i];
        vals[9] = (bx[i] * bx[i] + by[i] * by[i] + bz[i] * bz[i]) / r[i];
        vals[10] = (uu * uu + vv * vv + ww * ww);
        vals[11] = dxbx[i] + dyby[i] + zd1(bz + q, np, k, nz, 5, ho12);
        for (int m = 0; m < NMM; m++) { mn[m] = fmin(mn[m], vals[m]); mx[m] = fmax(mx[m], vals[m]); }
        bool fin = isfinite(vals[11]);
#pragma unroll
        for (int m = 0; m < 8; m++) fin = fin && isfinite(vals[m]);
        bad |= !fin;
    }
    bad = __syncthreads_or(bad);
    for (int m = 0; m < NMM; m++)
        for (int o = 16; o > 0; o >>= 1) {
            mn[m] = fmin(mn[m], __shfl_xor_sync(0xffffffffu, mn[m], o));
            mx[m] = fmax(mx[m], __shfl_xor_sync(0xffffffffu, mx[m], o));
        }
    __shared__ double sh[2 * NMM][8];
    int wid = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int m = 0; m < NMM; m++) { sh[m][wid] = mn[m]; sh[NMM + m][wid] = mx[m]; }
    __syncthreads();
    if (threadIdx.x < NMM) {
        int m = threadIdx.x;
        double a = 1.0e300, b = -1.0e300;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) { a = fmin(a, sh[m][q]); b = fmax(b, sh[NMM + m][q]); }
        out[(size_t)blockIdx.x * 2 * NMM + m] = a;
        out[(size_t)blockIdx.x * 2 * NMM + NMM + m] = b;
    }
    // one flag per CTA after the min/max block
    if (threadIdx.x == 0) out[(size_t)gridDim.x * 2 * NMM + blockIdx.x] = bad ? 1.0 : 0.0;
}

__global__ void k_nusselt_sum(const double *t, size_t np, int nz, double dz, double *out)
{
    PDL_WAIT();
    double s = 0.0;
    for (size_t i = threadIdx.x; i < np; i += blockDim.x)
        s += ((1.0 / (6.0 * dz)) * (11.0 * t[(size_t)(nz - 1) * np + i] - 18.0 * t[(size_t)(nz - 2) * np + i]
                                     + 9.0 * t[(size_t)(nz - 3) * np + i] - 2.0 * t[(size_t)(nz - 4) * np + i]));
    __shared__ double sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = sh[0];
}

int phys_diag(Engine *E, vec_diag_out *out)
{
    const Consts &c = E->k;
    double *ps = E->red;                       // nz*8 plane sums
    KLAUNCH(E, "plane_sums", k_plane_sums, E->nz, 256, E->r, E->u, E->v, E->w, E->bx, E->by, E->bz, E->np, ps);
    KLAUNCH(E, "globalavg_fin", k_globalavg_fin, 1, 1, ps, E->nz, c.xzn, E->ds);
    KLAUNCH(E, "sub_mean", k_sub_mean, nblk(E->n), TPB, E->u, E->v, E->n, E->ds);
    double *nus = E->red + (size_t)E->nz * 8;
    KLAUNCH(E, "nusselt_sum", k_nusselt_sum, 1, 256, E->t, E->np, E->nz, c.dz, nus);
    // checkdivb: d1bydx(bx), d1bydy(by) (src/utils.F90:263-265)
    int st;
    LineJob<double> jx = ljob<double>(E->bx, E->s64[0], OP_D1);
    LineJob<double> jy = ljob<double>(E->by, E->s64[1], OP_D1);
    if ((st = launch_lines<double>(E, 0, &jx, 1))) return st;
    if ((st = launch_lines<double>(E, 1, &jy, 1))) return st;
    double *mm = nus + 8;
    int blocks = E->red_blocks;
    KLAUNCH(E, "minmax", k_minmax, blocks, 256, E->r, E->t, E->u, E->v, E->w, E->bx, E->by, E->bz, E->s64[0],
            E->s64[1], E->np, E->nz, c.ho12, mm);
    CUDA_TRY(cudaMemcpyAsync(E->hs, E->ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, E->stream));
    std::vector<double> h((size_t)blocks * (2 * NMM + 1) + 8);
    CUDA_TRY(cudaMemcpyAsync(h.data(), nus, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, E->stream));
    CUDA_TRY(cudaStreamSynchronize(E->stream));
    vec_diag_out d;
    memset(&d, 0, sizeof(d));
    d.ubar = E->hs->res[0];
    d.vbar = E->hs->res[1];
    d.kenergy = E->hs->res[2];
    d.menergy = E->p.kinematic ? E->hs->res[3] : E->p.f * E->hs->res[3];
    double tzbar = h[0] * c.xn;
    d.nusselt = (tzbar - c.nusstmp) / (c.theta - c.nusstmp);
    double mn[NMM], mx[NMM];
    for (int m = 0; m < NMM; m++) { mn[m] = 1.0e300; mx[m] = -1.0e300; }
    for (int b = 0; b < blocks; b++)
        for (int m = 0; m < NMM; m++) {
            mn[m] = fmin(mn[m], h[8 + (size_t)b * 2 * NMM + m]);
            mx[m] = fmax(mx[m], h[8 + (size_t)b * 2 * NMM + NMM + m]);
        }
    d.rmin = mn[0]; d.rmax = mx[0]; d.tmin = mn[1]; d.tmax = mx[1]; d.umin = mn[2]; d.umax = mx[2];
    d.vmin = mn[3]; d.vmax = mx[3]; d.wmin = mn[4]; d.wmax = mx[4]; d.bxmin = mn[5]; d.bxmax = mx[5];
    d.bymin = mn[6]; d.bymax = mx[6]; d.bzmin = mn[7]; d.bzmax = mx[7];
    double fa = E->p.kinematic ? 1.0 : E->p.f;
    d.machmin = sqrt(mn[8] / E->p.gamma); d.machmax = sqrt(mx[8] / E->p.gamma);
    d.alfvenmin = sqrt(fa * mn[9]); d.alfvenmax = sqrt(fa * mx[9]);
    d.rmsmin = sqrt(mn[10]); d.rmsmax = sqrt(mx[10]);
    // checkdivb starts its minimum at 1.0 (src/utils.F90:275-276)
    d.divbmax = fmax(-1.0e30, mx[11]);
    d.divbmin = fmin(1.0, mn[11]);
    if (out) *out = d;
    E->last_diag = d;
    E->have_diag = 1;
    for (int b = 0; b < blocks; b++)
        if (h[8 + (size_t)blocks * 2 * NMM + b] != 0.0) {
            vec_set_error("non-finite value in the state or in div B (diagnostics)");
            return VEC_ERR_NAN;
        }
    double divbtest = fmax(fabs(d.divbmax), fabs(d.divbmin));
    if (divbtest > 0.01) return VEC_ERR_DIVB;
    return VEC_OK;
}

// ============================================================================
// initial state: src/initial.F90:25-86 with RANSET (src/ranset.f90:1-29)
// ============================================================================
// RAN0 keeps s = idum XOR MASK as a pure Park-Miller sequence
// s_{m+1} = 16807 s_m mod (2^31-1) and returns AM*s_{m+1}, so the n-th draw
// of a layer is AM * 16807^(n+1) s_0 mod (2^31-1): each point jumps ahead on
// its own.
__device__ __forceinline__ unsigned long long mulmod31(unsigned long long a, unsigned long long b)
{
    return (a * b) % 2147483647ull;
}

__global__ void k_static(double *r, double *t, double *u, double *v, double *w, double *bx, double *by,
                         double *bz, const double *t0k, const double *r0k, size_t np, int nz, double amp,
                         int seed_base, int perfect)
{
    PDL_WAIT();
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= np * nz) return;
    const int k = (int)(idx / np);
    const size_t q = idx - (size_t)k * np;
    const unsigned MASK = 123459876u;
    unsigned s0 = (unsigned)(seed_base + 64 * (k + 1)) ^ MASK;
    // 16807^(q+1) mod M
    unsigned long long e = (unsigned long long)q + 1ull, base = 16807ull, pw = 1ull;
    while (e) {
        if (e & 1ull) pw = mulmod31(pw, base);
        base = mulmod31(base, base);
        e >>= 1;
    }
    unsigned long long s = mulmod31(pw, (unsigned long long)s0);
    const double AM = 1.0 / 2147483647.0;
    double ran = __dmul_rn(AM, (double)s);
    double noise = __dmul_rn(__dmul_rn(2.0, __dsub_rn(ran, 0.5)), amp);
    u[idx] = 0.0; v[idx] = 0.0; w[idx] = 0.0;
    r[idx] = r0k[k];
    t[idx] = __dadd_rn(noise, t0k[k]);
    if (perfect) { bx[idx] = 1.0; by[idx] = 0.0; bz[idx] = 0.0; }
    else { bx[idx] = 0.0; by[idx] = 0.0; bz[idx] = 1.0; }
}

int phys_static(Engine *E)
{
    std::vector<double> t0(E->nz), r0(E->nz);
    for (int k = 0; k < E->nz; k++) {
        double z = (double)k * E->k.dz;
        t0[k] = 1.0 + z * E->p.theta;
        r0[k] = pow(t0[k], E->p.cm);
    }
    double *d = E->w1d;   // 8 nz scratch
    CUDA_TRY(cudaMemcpyAsync(d, t0.data(), sizeof(double) * E->nz, cudaMemcpyHostToDevice, E->stream));
    CUDA_TRY(cudaMemcpyAsync(d + E->nz, r0.data(), sizeof(double) * E->nz, cudaMemcpyHostToDevice, E->stream));
    KLAUNCH(E, "static_ic", k_static, nblk(E->n), TPB, E->r, E->t, E->u, E->v, E->w, E->bx, E->by, E->bz, d,
            d + E->nz, E->np, E->nz, E->p.noise_amp, E->p.seed_base, E->p.perfect);
    CUDA_TRY(cudaStreamSynchronize(E->stream));
    return VEC_OK;
}

// ============================================================================
// mag_init: src/magnetic.f90:5-279
// ============================================================================
__global__ void k_dynamo_seed(double *bx, double *by, double *bz, int nx, int ny, size_t n, int perfect)
{
    PDL_WAIT();
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n) return;
    size_t np = (size_t)nx * ny;
    size_t q = idx % np;
    int j = (int)(q / nx), i = (int)(q - (size_t)j * nx);
    const double seedfield = 0.003;
    const double tpx = 8.0 * atan(1.0) / (nx * 1.0), tpy = 8.0 * atan(1.0) / (ny * 1.0);
    if (perfect) {
        bx[idx] = seedfield * cos(tpy * (j + 1));
        by[idx] = seedfield * cos(tpx * (i + 1));
        bz[idx] = 0.0;
    } else {
        bx[idx] = 0.0;
        by[idx] = 0.0;
        bz[idx] = seedfield * cos(tpx * (i + 1)) * cos(tpy * (j + 1));
    }
}

struct MagInitArgs {
    const double *ex, *ey, *ez, *akx1, *aky1, *akx2, *aky2;
    double *pol, *tor, *w1, *w2, *w3;
    int nx, ny, nz;
};

// :123-233: pol, tor from the truncated spectra; Jz, dBz/dy, dBz/dx spectra
__global__ void k_mag_init_spec(MagInitArgs a)
{
    PDL_WAIT();
    const size_t np = (size_t)a.nx * a.ny;
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= np * a.nz) return;
    const int k = (int)(idx / np);
    const size_t q = idx - (size_t)k * np;
    const int j = (int)(q / a.nx), i = (int)(q - (size_t)j * a.nx);
    const double *pey = a.ey + (size_t)k * np, *pex = a.ex + (size_t)k * np, *pez = a.ez + (size_t)k * np;
    const double kk = a.akx2[i] + a.aky2[j];
    double pol, tor;
    if (i == 0 && j == 0) { pol = 0.0; tor = 0.0; }
    else {
        pol = -1.0 * a.ez[idx] / kk;
        double jz = sdx(pey, i, j, a.nx, a.akx1) - sdy(pex, i, j, a.nx, a.ny, a.aky1);
        tor = -1.0 * jz / kk;
    }
    a.pol[idx] = pol;
    a.tor[idx] = tor;
    a.w3[idx] = -1.0 * tor * kk;
    a.w1[idx] = sdy(pez, i, j, a.nx, a.ny, a.aky1);
    a.w2[idx] = sdx(pez, i, j, a.nx, a.akx1);
}

__global__ void k_mag_init_means(const double *ex, const double *ey, const double *ez, double *bxbar,
                                 double *bybar, double *bzbar_out, size_t np, int nz, double xn)
{
    PDL_WAIT();
    for (int k = threadIdx.x; k < nz; k += blockDim.x) {
        bxbar[k] = ex[(size_t)k * np] * xn;
        bybar[k] = ey[(size_t)k * np] * xn;
    }
    if (threadIdx.x == 0) bzbar_out[0] = ez[0] * xn;
}

int phys_mag_init(Engine *E)
{
    // six FP64 work arrays (valid in both forms, see Engine::W64)
    double *W[W_COUNT];
    for (int i = 0; i < W_COUNT; i++) W[i] = nullptr;
    W[W_EX] = E->W64(0); W[W_EY] = E->W64(1); W[W_EZ] = E->W64(2);
    W[W_M1] = E->W64(3); W[W_M2] = E->W64(4); W[W_M3] = E->W64(5);
    int st;
    if (E->p.dynamo)
        KLAUNCH(E, "dynamo_seed", k_dynamo_seed, nblk(E->n), TPB, E->bx, E->by, E->bz, E->nx, E->ny, E->n, E->p.perfect);
    LineJob<double> fx[3] = { ljob<double>(E->bx, W[W_EX], OP_FWD), ljob<double>(E->by, W[W_EY], OP_FWD),
                              ljob<double>(E->bz, W[W_EZ], OP_FWD) };
    if ((st = launch_lines<double>(E, 0, fx, 3))) return st;
    LineJob<double> fy[3] = { ljob<double>(W[W_EX], W[W_EX], OP_FWD), ljob<double>(W[W_EY], W[W_EY], OP_FWD),
                              ljob<double>(W[W_EZ], W[W_EZ], OP_FWD) };
    if ((st = launch_lines<double>(E, 1, fy, 3))) return st;
    for (int f = 0; f < 3; f++)     // :70-103
        KLAUNCH(E, "truncate_f64", k_truncate<double>, plane_grid(*E), TPB, W[W_EX + f], (double *)nullptr, E->nx, E->ny,
                E->nz, E->k.icutoffx, E->k.icutoffy);
    KLAUNCH(E, "mag_init_means", k_mag_init_means, 1, 256, W[W_EX], W[W_EY], W[W_EZ], E->bxbar, E->bybar,
            E->w1d + 7 * E->nz, E->np, E->nz, E->k.xn);
    double bzb = 0.0;
    CUDA_TRY(cudaMemcpyAsync(&bzb, E->w1d + 7 * E->nz, sizeof(double), cudaMemcpyDeviceToHost, E->stream));
    CUDA_TRY(cudaStreamSynchronize(E->stream));
    E->bzbar = bzb;
    MagInitArgs a;
    a.ex = W[W_EX]; a.ey = W[W_EY]; a.ez = W[W_EZ]; a.akx1 = E->akx1; a.aky1 = E->aky1; a.akx2 = E->akx2;
    a.aky2 = E->aky2; a.pol = E->pol; a.tor = E->tor; a.w1 = W[W_M1]; a.w2 = W[W_M2]; a.w3 = W[W_M3];
    a.nx = E->nx; a.ny = E->ny; a.nz = E->nz;
    KLAUNCH(E, "mag_init_spec", k_mag_init_spec, nblk(E->n), TPB, a);
    LineJob<double> ix[3] = { ljob<double>(W[W_M1], W[W_M1], OP_INV), ljob<double>(W[W_M2], W[W_M2], OP_INV),
                              ljob<double>(W[W_M3], W[W_M3], OP_INV) };
    if ((st = launch_lines<double>(E, 0, ix, 3))) return st;
    if ((st = launch_lines<double>(E, 1, ix, 3))) return st;
    // jsq (:246-261): ex = inv(dBz/dy), ey = inv(dBz/dx), ez = inv(Jz)
    KLAUNCH(E, "jsq_f64", k_jsq<double>, plane_grid(*E), TPB, W[W_M3], W[W_M1], W[W_M2], E->bx, E->by,
            E->jsq, E->np, E->nz, E->k.ho12);
    return phys_mag_boundary(E);
}
