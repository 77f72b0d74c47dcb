// split.cu -- the FP32-bulk / FP64-background form of the time step.
//
// FP64 is kept for: the state and its AB3 accumulation (r,t,u,v,w,pol,tor),
// the horizontally uniform polytropic background rho0(z) = T0(z)^m,
// T0(z) = 1 + theta z, the residual of the discrete pressure-gradient-minus-
// gravity balance of that background, the mean fields and the diagnostics.
// Everything else -- the FFTs, z stencils, nonlinear products and the RHS
// histories -- runs in FP32 on perturbation mirrors of the state:
//     r32 = r - rho0(z),  t32 = t - T0(z),  bz32 = bz - bzbar,
// so that no FP32 operation ever has to resolve the O(1e-3) dynamics on top
// of the O(10) background.
//
// The split is exact in exact arithmetic: every z stencil is linear, so
// D(rho0 + r') = D(rho0) + D(r'), and the background parts D(rho0), D(T0)
// are applied once on the host in FP64 with the same stencils and flags the
// reference uses (src/hydro_deriv.f90:66-68, 184, 443-444).  In the
// vertical momentum equation the large terms
//     -rho dT/dz + theta(m+1) rho - T d(rho)/dz
// become  [-rho0 T0' + theta(m+1) rho0 - T0 rho0'](z)   (FP64, 1-D)
//       + [-rho0 T'z - r' T0' - r' T'z + theta(m+1) r' - T0 r'z - T' rho0' - T' r'z]
// and the magnetic pressure uses bz^2 - bzbar^2 = bz'(2 bzbar + bz'), whose
// horizontal and vertical derivatives equal those of bz^2 (the difference is
// a constant; the spectral derivative drops the mean and every z stencil
// annihilates constants).
#include <math.h>
#include <string.h>

#include <vector>

#include "common.cuh"
#include "engine.h"
#include "fpconv.cuh"
#include "magkern.cuh"
#include "tma.cuh"
#include "zstencil.cuh"

#define TPB 256
static inline unsigned nblk(size_t n) { return (unsigned)((n + TPB - 1) / TPB); }

#define KLAUNCHB(E, name, bytes, kern, grid, block, ...)         \
    do {                                                         \
        (E)->prof_begin(name, (double)(bytes));                  \
        CUDA_TRY(launch_k(*(E), kern, dim3(grid), dim3(block), 0, __VA_ARGS__)); \
        (E)->prof_end();                                         \
        CUDA_TRY(cudaGetLastError());                            \
    } while (0)
#define FB(E, nf, esz) ((double)(nf) * (double)(E)->n * (double)(esz))

// 1-D FP64 background profiles and their discrete derivatives
enum Bg {
    BG_RHO0, BG_T0, BG_T0Z5, BG_T0ZU_P, BG_T0ZU_M, BG_T0ZZ0, BG_RHO0Z0, BG_RHO0ZU_P, BG_RHO0ZU_M,
    BG_A, BG_B, BG_COUNT
};

// The same profiles (and kappa, eta) rounded once to FP32, per plane: the
// FP32 kernels read these instead of converting FP64 values at every point
// (identical values; GB300's FP64 and conversion rates are low)
enum Pc {
    PC_RHO0, PC_T0, PC_T0Z5, PC_T0ZU_P, PC_T0ZU_M, PC_T0ZZ0, PC_RHO0Z0, PC_RHO0ZU_P, PC_RHO0ZU_M,
    PC_AB,       // A + B, summed in FP64
    PC_KAPPA, PC_DKAPPA,
    PC_OHM,      // eta / (zeta ck), divided in FP64
    PC_ETA, PC_DETA,
    PC_COUNT
};

__global__ void k_make_pcf(const double *bg, const double *kappa, const double *dkappa, const double *eta,
                           const double *deta, double zck, int nz, float *pc)
{
    PDL_WAIT();
    for (int k = threadIdx.x; k < nz; k += blockDim.x) {
        const int from[9] = { BG_RHO0, BG_T0, BG_T0Z5, BG_T0ZU_P, BG_T0ZU_M, BG_T0ZZ0, BG_RHO0Z0, BG_RHO0ZU_P,
                              BG_RHO0ZU_M };
        for (int q = 0; q < 9; q++) pc[q * nz + k] = (float)bg[from[q] * nz + k];
        pc[PC_AB * nz + k] = (float)(bg[BG_A * nz + k] + bg[BG_B * nz + k]);
        pc[PC_KAPPA * nz + k] = (float)kappa[k];
        pc[PC_DKAPPA * nz + k] = (float)dkappa[k];
        pc[PC_OHM * nz + k] = (float)(eta[k] / zck);
        pc[PC_ETA * nz + k] = (float)eta[k];
        pc[PC_DETA * nz + k] = (float)deta[k];
    }
}

const double *split_bg_t0(const Engine *E) { return E->hres + (size_t)BG_T0 * E->nz; }

// (re)builds the FP32 plane coefficients from the FP64 profiles
int split_refresh_coefs(Engine *E)
{
    k_make_pcf<<<1, 256, 0, E->stream>>>(E->hres, E->kappa, E->dkappa, E->eta, E->deta, E->k.zck, E->nz, E->pcf);
    CUDA_TRY(cudaGetLastError());
    return VEC_OK;
}

static int falloc(float **p, size_t n)
{
    if (cudaMalloc((void **)p, sizeof(float) * (n ? n : 1)) != cudaSuccess) {
        cudaGetLastError();
        vec_set_error("cudaMalloc of %zu floats failed", n);
        return VEC_ERR_ALLOC;
    }
    return cudaMemset(*p, 0, sizeof(float) * n) == cudaSuccess ? VEC_OK : VEC_ERR_CUDA;
}

int split_setup(Engine *E)
{
    const size_t n = E->n;
    const int nz = E->nz;
    float **m[] = { &E->r32, &E->t32, &E->u32, &E->v32, &E->w32, &E->bx32, &E->by32, &E->bz32, &E->jsq32,
                    &E->pol32, &E->tor32 };
    for (auto pp : m) {
        int st = falloc(pp, n);
        if (st) return st;
    }
    std::vector<double> bg((size_t)BG_COUNT * nz, 0.0);
    double *rho0 = &bg[(size_t)BG_RHO0 * nz], *t0 = &bg[(size_t)BG_T0 * nz];
    for (int k = 0; k < nz; k++) {
        double z = (double)k * E->k.dz;
        t0[k] = 1.0 + z * E->p.theta;
        rho0[k] = pow(t0[k], E->p.cm);
    }
    const double h = E->k.ho12, s = E->k.sc1;
    for (int k = 0; k < nz; k++) {
        bg[(size_t)BG_T0Z5 * nz + k] = zd1(t0, 1, k, nz, 5, h);
        bg[(size_t)BG_T0ZU_P * nz + k] = zd1up(t0, 1, k, nz, 5, h, 1.0);
        bg[(size_t)BG_T0ZU_M * nz + k] = zd1up(t0, 1, k, nz, 5, h, -1.0);
        bg[(size_t)BG_T0ZZ0 * nz + k] = zd2(t0, 1, k, nz, 0, s);
        bg[(size_t)BG_RHO0Z0 * nz + k] = zd1(rho0, 1, k, nz, 0, h);
        bg[(size_t)BG_RHO0ZU_P * nz + k] = zd1up(rho0, 1, k, nz, 0, h, 1.0);
        bg[(size_t)BG_RHO0ZU_M * nz + k] = zd1up(rho0, 1, k, nz, 0, h, -1.0);
    }
    for (int k = 0; k < nz; k++) {
        // -rho0 dT0/dz + theta(m+1) rho0  (the rho*tz and gravity terms)
        bg[(size_t)BG_A * nz + k] = -rho0[k] * bg[(size_t)BG_T0Z5 * nz + k] + E->k.thmplus1 * rho0[k];
        // -T0 d(rho0)/dz  (the t*rz term, interior rows)
        bg[(size_t)BG_B * nz + k] = -t0[k] * bg[(size_t)BG_RHO0Z0 * nz + k];
    }
    if (cudaMalloc((void **)&E->hres, sizeof(double) * bg.size()) != cudaSuccess) {
        cudaGetLastError();
        return VEC_ERR_ALLOC;
    }
    CUDA_TRY(cudaMemcpy(E->hres, bg.data(), sizeof(double) * bg.size(), cudaMemcpyHostToDevice));
    {
        int st = falloc(&E->pcf, (size_t)PC_COUNT * nz);
        if (st) return st;
        if ((st = split_refresh_coefs(E))) return st;
        CUDA_TRY(cudaStreamSynchronize(E->stream));
    }
    E->b32_auth = 0;
    return VEC_OK;
}

// ---- mirrors ---------------------------------------------------------------
struct MirrorArgs {
    const double *r, *t, *u, *v, *w, *pol, *tor, *bx, *by, *bz, *jsq, *bg;
    float *r32, *t32, *u32, *v32, *w32, *pol32, *tor32, *bx32, *by32, *bz32, *jsq32;
    double bzbar;
    size_t np;
    int nz, k0, k1, mask;   // planes [k0,k1); mask: MIR_* bits
};

// mirror masks: whole groups, or single fields
enum {
    MIR_STATE = 1,          // r, t, u, v, w, pol, tor
    MIR_UV = 2, MIR_B = 4,  // u and v; bx, by, bz, jsq
    MIR_POLTOR = 8,
    MIR_R = 16, MIR_T = 32, MIR_W = 64, MIR_U = 128, MIR_V = 256, MIR_POL = 512, MIR_TOR = 1024,
};

// FP32 mirrors of the FP64 fields, grid (np/256, k1-k0); conversions on the
// integer pipe (the same bits as the casts)
__global__ void k_mirror(MirrorArgs a)
{
    PDL_WAIT();
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.np) return;
    const int k = a.k0 + blockIdx.y;
    const size_t idx = (size_t)k * a.np + q;
    const int m = a.mask;
    if (m & (MIR_STATE | MIR_R)) a.r32[idx] = d2f_rn(a.r[idx] - a.bg[BG_RHO0 * a.nz + k]);
    if (m & (MIR_STATE | MIR_T)) a.t32[idx] = d2f_rn(a.t[idx] - a.bg[BG_T0 * a.nz + k]);
    if (m & (MIR_STATE | MIR_W)) a.w32[idx] = d2f_rn(a.w[idx]);
    if (m & (MIR_STATE | MIR_UV | MIR_U)) a.u32[idx] = d2f_rn(a.u[idx]);
    if (m & (MIR_STATE | MIR_UV | MIR_V)) a.v32[idx] = d2f_rn(a.v[idx]);
    if (m & (MIR_STATE | MIR_POLTOR | MIR_POL)) a.pol32[idx] = d2f_rn(a.pol[idx]);
    if (m & (MIR_STATE | MIR_POLTOR | MIR_TOR)) a.tor32[idx] = d2f_rn(a.tor[idx]);
    if (m & MIR_B) {
        a.bx32[idx] = d2f_rn(a.bx[idx]);
        a.by32[idx] = d2f_rn(a.by[idx]);
        a.bz32[idx] = d2f_rn(a.bz[idx] - a.bzbar);
        a.jsq32[idx] = d2f_rn(a.jsq[idx]);
    }
}

static int mirror(Engine *E, int mask, int k0, int k1)
{
    MirrorArgs a;
    a.r = E->r; a.t = E->t; a.u = E->u; a.v = E->v; a.w = E->w; a.pol = E->pol; a.tor = E->tor;
    a.bx = E->bx; a.by = E->by; a.bz = E->bz; a.jsq = E->jsq; a.bg = E->hres;
    a.r32 = E->r32; a.t32 = E->t32; a.u32 = E->u32; a.v32 = E->v32; a.w32 = E->w32;
    a.pol32 = E->pol32; a.tor32 = E->tor32; a.bx32 = E->bx32; a.by32 = E->by32; a.bz32 = E->bz32;
    a.jsq32 = E->jsq32; a.bzbar = E->bzbar; a.np = E->np; a.nz = E->nz; a.k0 = k0; a.k1 = k1; a.mask = mask;
    KLAUNCHB(E, "mirror", 0, k_mirror, dim3((unsigned)nblk(E->np), (unsigned)(k1 - k0)), TPB, a);
    return VEC_OK;
}

struct B64Args {
    const float *bx32, *by32, *bz32, *jsq32;
    double *bx, *by, *bz, *jsq;
    double bzbar;
    size_t n;
};
template <int NB>
__global__ void k_b64(const __grid_constant__ Batch<B64Args, NB> bt)
{
    PDL_WAIT();
    const B64Args &A = BATCH_MEMBER(bt, NB);
    const float *bx32 = A.bx32, *by32 = A.by32, *bz32 = A.bz32, *jsq32 = A.jsq32;
    double *bx = A.bx, *by = A.by, *bz = A.bz, *jsq = A.jsq;
    const double bzbar = A.bzbar;
    const size_t n = A.n;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // (conversions on the integer pipe, the same bits as the casts)
    bx[i] = f2d_exact(bx32[i]);
    by[i] = f2d_exact(by32[i]);
    bz[i] = bzbar + f2d_exact(bz32[i]);
    jsq[i] = f2d_exact(jsq32[i]);
}

// FP64 B and jsq from the FP32 ones when the FP32 copy is the newer one
// (every member of the batch, which all have it newer)
int split_sync_b64_m(Engine *const *Es, int nE)
{
    int st = launch_members<B64Args>(Es, nE, "b_to_f64", FB(Es[0], 4, 12), dim3(nblk(Es[0]->n)), dim3(TPB), 0,
                                     k_b64<1>, k_b64<BATCH_MAX>, [](Engine *e) {
                                         return B64Args{ e->bx32, e->by32, e->bz32, e->jsq32, e->bx, e->by, e->bz,
                                                         e->jsq, e->bzbar, e->n };
                                     });
    if (st) return st;
    for (int i = 0; i < nE; i++) Es[i]->b32_auth = 0;
    return VEC_OK;
}
int split_sync_b64(Engine *E)
{
    if (!E->b32_auth) return VEC_OK;
    return split_sync_b64_m(&E, 1);
}

// all FP32 mirrors from the FP64 state (after the state was set from outside)
int split_refresh(Engine *E)
{
    int st = split_sync_b64(E);
    if (st) return st;
    return mirror(E, MIR_STATE | MIR_B, 0, E->nz);
}

// the mirror of one state field (VEC_F_*) after that field was set
int split_refresh_field(Engine *E, int field)
{
    int m = 0;
    switch (field) {
    case VEC_F_R: m = MIR_R; break;
    case VEC_F_T: m = MIR_T; break;
    case VEC_F_U: m = MIR_U; break;
    case VEC_F_V: m = MIR_V; break;
    case VEC_F_W: m = MIR_W; break;
    case VEC_F_POL: m = MIR_POL; break;
    case VEC_F_TOR: m = MIR_TOR; break;
    default: m = MIR_B; break;   // bx, by, bz, jsq
    }
    return mirror(E, m, 0, E->nz);
}

int split_refresh_planes(Engine *E, int mask)
{
    int st = mirror(E, mask, 0, 1);
    if (st) return st;
    return mirror(E, mask, E->nz - 1, E->nz);
}

int split_refresh_uv(Engine *E) { return mirror(E, MIR_UV, 0, E->nz); }

// ---- hydro_deriv ------------------------------------------------------------
// a context with a magnetic field (its induction equation is stepped)
static inline int split_mag_on(const Engine &E) { return E.p.f != 0.0 || E.p.kinematic; }

struct SplitHydroArgs {
    const float *r, *t, *u, *v, *w, *bx, *by, *bz, *jsq;
    const float *rx, *tx, *txx, *ux, *uxx, *vx, *vxx, *wx, *wxx;
    const float *ry, *ty, *tyy, *uy, *uyy, *vy, *vyy, *wy, *wyy;
    const float *pc;        // per-plane FP32 coefficients [PC_COUNT][nz]
    const HistTable *ht;    // tdot = newest slot of t
    float *racc, *uacc, *vacc, *wacc;
    float *p1, *p2, *q, *g, *hh, *p3, *p4;
    float *e1, *e2, *e3;    // E = u x B (the emf of mag_deriv) when not null
    float gck, fzckg, gm1, sckg, fo2, scko3, f, thmplus1, cor, cpsi, spsi, sck, ho12, sc1, bzbar;
    int var_eta;
    int mag;                // 0: no magnetic field (Q = 0): B, J^2 and the Lorentz
                            // fluxes q, g, h are zero, neither read nor written
    size_t np;
    int nz;
    int kc;                 // z-pencil kernel: planes per chunk
    int *err;               // z-pencil kernel: the bounded waits' error flag
};

// the FP32 counterpart of k_hydro_pass2 (src/hydro_deriv.f90 terms without
// a second-level derivative) on perturbation mirrors, for one point; the z
// derivatives of t', u, v, w come from the caller (register windows in the
// interior, direct row formulas near the walls)
template <typename T> struct ZDer { T tzu, tzp, tzz, wzu, wz, uzu, vzu, uzz, vzz; };

// loads and stores of one point (float) or four consecutive points (V4)
template <typename T> __device__ __forceinline__ T ldv(const float *p, size_t i);
template <> __device__ __forceinline__ float ldv<float>(const float *p, size_t i) { return p[i]; }
template <> __device__ __forceinline__ V4 ldv<V4>(const float *p, size_t i) { return reinterpret_cast<const V4 *>(p)[i]; }
template <> __device__ __forceinline__ V2 ldv<V2>(const float *p, size_t i) { return reinterpret_cast<const V2 *>(p)[i]; }
__device__ __forceinline__ void stv(float *p, size_t i, V2 v) { reinterpret_cast<V2 *>(p)[i] = v; }
__device__ __forceinline__ void stv(float *p, size_t i, float v) { p[i] = v; }
__device__ __forceinline__ void stv(float *p, size_t i, V4 v) { reinterpret_cast<V4 *>(p)[i] = v; }
__device__ __forceinline__ float upsel(float w, float p, float m) { return w >= 0.0f ? p : m; }
__host__ __device__ __forceinline__ V4 operator/(V4 a, V4 b) { return V4(a.x / b.x, a.y / b.y, a.z / b.z, a.w / b.w); }

// the point inputs of pass 2 besides t', u, v, w (which the z stencils read)
enum P2Field {
    P2_R, P2_BX, P2_BY, P2_BZ, P2_JSQ, P2_RX, P2_RY, P2_TX, P2_TXX, P2_TY, P2_TYY, P2_UX, P2_UXX, P2_UY, P2_UYY,
    P2_VX, P2_VXX, P2_VY, P2_VYY, P2_WX, P2_WXX, P2_WY, P2_WYY, P2_COUNT
};
__device__ __forceinline__ const float *p2_src(const SplitHydroArgs &a, int f)
{
    switch (f) {
    case P2_R: return a.r; case P2_BX: return a.bx; case P2_BY: return a.by; case P2_BZ: return a.bz;
    case P2_JSQ: return a.jsq; case P2_RX: return a.rx; case P2_RY: return a.ry; case P2_TX: return a.tx;
    case P2_TXX: return a.txx; case P2_TY: return a.ty; case P2_TYY: return a.tyy; case P2_UX: return a.ux;
    case P2_UXX: return a.uxx; case P2_UY: return a.uy; case P2_UYY: return a.uyy; case P2_VX: return a.vx;
    case P2_VXX: return a.vxx; case P2_VY: return a.vy; case P2_VYY: return a.vyy; case P2_WX: return a.wx;
    case P2_WXX: return a.wxx; case P2_WY: return a.wy; default: return a.wyy;
    }
}
// the point inputs read from global memory
template <typename T> struct P2Global {
    const SplitHydroArgs &a;
    size_t idx;
    __device__ __forceinline__ T operator()(int f) const { return ldv<T>(p2_src(a, f), idx); }
};

// one point (T = float, idx a point index) or four (T = V4, idx a 4-vector
// index) of the terms without second-level derivatives
// (tp, u0, v0, w0: t', u, v, w at the point)
// (L(f): point input f of P2Field)
template <typename T, typename L>
__device__ __forceinline__ void split_pass2_point(const SplitHydroArgs &a, size_t idx, int k, const ZDer<T> &z,
                                                  const T tp, const T u0, const T v0, const T w0, const L &ld)
{
    const int nz = a.nz;
    const float *pc = a.pc;
    const T rho0 = T(pc[PC_RHO0 * nz + k]), t0 = T(pc[PC_T0 * nz + k]);
    const T rp = ld(P2_R);
    const T rr = rho0 + rp, tt = t0 + tp;
    // (without a magnetic field the B mirrors hold zeros: the same values)
    const bool mg = a.mag != 0;
    const T bx = mg ? ld(P2_BX) : T(0.0f), by = mg ? ld(P2_BY) : T(0.0f), bzp = mg ? ld(P2_BZ) : T(0.0f);
    const T bz = T(a.bzbar) + bzp;
    const T rx = ld(P2_RX), ry = ld(P2_RY);
    const T tx = ld(P2_TX), txx = ld(P2_TXX), ty = ld(P2_TY), tyy = ld(P2_TYY);
    const T ux = ld(P2_UX), uxx = ld(P2_UXX), uy = ld(P2_UY), uyy = ld(P2_UYY);
    const T vx = ld(P2_VX), vxx = ld(P2_VXX), vy = ld(P2_VY), vyy = ld(P2_VYY);
    const T wx = ld(P2_WX), wxx = ld(P2_WXX), wy = ld(P2_WY), wyy = ld(P2_WYY);

    const T tzu = z.tzu + upsel(w0, T(pc[PC_T0ZU_P * nz + k]), T(pc[PC_T0ZU_M * nz + k]));
    const T tzp = z.tzp;
    const T tzz = z.tzz + T(pc[PC_T0ZZ0 * nz + k]);
    const T wzu = z.wzu, wz = z.wz, uzu = z.uzu, vzu = z.vzu, uzz = z.uzz, vzz = z.vzz;

    const T third = T(1.0f / 3.0f);
    const T ohm = T(a.var_eta ? pc[PC_OHM * nz + k] : 1.0f);
    const T divu = ux + vy + wz;

    stv(a.racc, idx, -u0 * rx - v0 * ry - rr * divu);

    T td = -rr * (u0 * tx + v0 * ty + w0 * tzu)
           + T(a.gck) * T(pc[PC_KAPPA * nz + k]) * (txx + tyy + tzz)
           + T(a.gck) * T(pc[PC_DKAPPA * nz + k]) * tzu
           + T(a.fzckg) * ohm * (mg ? ld(P2_JSQ) : T(0.0f));
    td = td - T(a.gm1) * tt * divu * rr + T(2.0f) * T(a.sckg) * (ux * ux + vy * vy + wz * wz - third * divu * divu);
    td = td + T(a.sckg) * (uy + vx) * (uy + vx);
    td = td + T(a.sckg) * (wx + uzu) * (wx + uzu);
    td = td + T(a.sckg) * (wy + vzu) * (wy + vzu);
    stv((float *)a.ht->p[1][2], idx, td / rr);

    T ud = -tt * rx - rr * tx;
    ud = ud - rr * u0 * ux - rr * v0 * uy - rr * w0 * uzu;
    ud = ud - rr * T(a.cor) * (w0 * T(a.cpsi) + v0 * T(a.spsi));
    ud = ud + T(a.sck) * (uzz + uxx + uyy);
    T vd = -tt * ry - rr * ty;
    vd = vd - rr * v0 * vy - rr * u0 * vx - rr * w0 * vzu;
    vd = vd - rr * T(a.cor) * (-u0 * T(a.spsi));
    vd = vd + T(a.sck) * (vzz + vxx + vyy);
    // -rho dT/dz + theta(m+1) rho minus its FP64 background part
    const T t0z = T(pc[PC_T0Z5 * nz + k]);
    T wd = -rho0 * tzp - rp * t0z - rp * tzp + T(a.thmplus1) * rp;
    wd = wd - rr * w0 * wzu - rr * u0 * wx - rr * v0 * wy;
    wd = wd - rr * T(a.cor) * (-u0 * T(a.cpsi));
    wd = wd + T(a.sck) * (wxx + wyy);
    stv(a.uacc, idx, ud);
    stv(a.vacc, idx, vd);
    stv(a.wacc, idx, wd);

    const T b2z = bzp * (T(2.0f) * T(a.bzbar) + bzp);          // bz^2 - bzbar^2
    const T temp1 = T(a.fo2) * bx * bx, temp2 = T(a.fo2) * by * by, temp3 = T(a.fo2) * b2z;
    const T dv = T(a.scko3) * divu;
    stv(a.p1, idx, dv + temp1 - temp2 - temp3);
    stv(a.p2, idx, dv + temp2 - temp1 - temp3);
    stv(a.p3, idx, T(a.scko3) * ux + T(a.scko3) * vy + temp3 - temp1 - temp2);
    stv(a.p4, idx, T(4.0f) * T(a.scko3) * wz);
    if (mg) {
        stv(a.q, idx, T(a.f) * by * bx);
        stv(a.g, idx, T(a.f) * bz * bx);
        stv(a.hh, idx, T(a.f) * bz * by);
        // E = u x B from the same values (src/magnetic.f90 mag_deriv's emf)
        if (a.e1) {
            stv(a.e1, idx, v0 * bz - w0 * by);
            stv(a.e2, idx, w0 * bx - u0 * bz);
            stv(a.e3, idx, u0 * by - v0 * bx);
        }
    }
}
template <typename T>
__device__ __forceinline__ void split_pass2_point(const SplitHydroArgs &a, size_t idx, int k, const ZDer<T> &z)
{
    split_pass2_point<T>(a, idx, k, z, ldv<T>(a.t, idx), ldv<T>(a.u, idx), ldv<T>(a.v, idx), ldv<T>(a.w, idx),
                         P2Global<T>{ a, idx });
}

// two consecutive x points per thread, one plane per CTA row (grid
// (np/2/256, nz)); the z neighbours come through L1/L2.  (Three CTAs per
// SM at 80 registers: 4.9 TB/s, against 4.7 for four points per thread,
// whose ~175 live registers spill at two CTAs per SM.)
__global__ void __launch_bounds__(256, 3) k_split_pass2_v2(SplitHydroArgs a)
{
    PDL_WAIT();
    const size_t np2 = a.np / 2;
    const size_t q2 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q2 >= np2) return;
    const int nz = a.nz;
    const int k = blockIdx.y;
    const V2 h(a.ho12), s(a.sc1);
    const V2 *t2 = reinterpret_cast<const V2 *>(a.t) + q2, *u2 = reinterpret_cast<const V2 *>(a.u) + q2;
    const V2 *v2 = reinterpret_cast<const V2 *>(a.v) + q2, *w2 = reinterpret_cast<const V2 *>(a.w) + q2;
    const V2 w0 = w2[(size_t)k * np2];
    ZDer<V2> z;
    z.tzu = zd1up(t2, np2, k, nz, 5, h, w0); z.tzp = zd1(t2, np2, k, nz, 5, h); z.tzz = zd2(t2, np2, k, nz, 0, s);
    z.wzu = zd1up(w2, np2, k, nz, 1, h, w0); z.wz = zd1(w2, np2, k, nz, 1, h);
    z.uzu = zd1up(u2, np2, k, nz, 2, h, w0); z.vzu = zd1up(v2, np2, k, nz, 2, h, w0);
    z.uzz = zd2(u2, np2, k, nz, 3, s); z.vzz = zd2(v2, np2, k, nz, 3, s);
    split_pass2_point<V2>(a, (size_t)k * np2 + q2, k, z);
}

// Pass 2 with TMA-staged z-pencils.  A CTA owns ZT_TILE consecutive points
// of the plane (two per thread) and a chunk of planes [k0, k1) and marches
// down in z.  The planes of t', u, v, w that the z stencils read sit in a
// ring of ZT_SLOTS shared-memory slots (a slot = the tile of the four fields
// on one plane), filled by bulk copies (cp.async.bulk + mbarrier) one plane
// ahead of the row being computed.  Row k reads planes k-3..k+3 (0..5 and
// nz-6..nz-1 next to the walls), so every plane comes from DRAM/L2 once per
// chunk instead of once per stencil tap.  The other inputs of the point are
// read directly.  Same arithmetic as k_split_pass2_v2, value for value.
#define ZT_TILE 512
#define ZT_SLOTS 8
// one field of a ring whose slots hold NF fields' tiles
template <int NF> struct ZRingF {
    const V2 *base;     // slot 0 of one field, this thread's point pair
    __device__ __forceinline__ V2 operator()(int kk) const
    {
        return base[(size_t)(kk & (ZT_SLOTS - 1)) * (NF * ZT_TILE / 2)];
    }
};
using ZRing2 = ZRingF<4>;
// the z window of plane k's stencils (d1, d1up, d2 with their wall rows)
__device__ __forceinline__ int zt_lo(int k, int nz) { return max(0, k >= nz - 2 ? min(k - 3, nz - 6) : k - 3); }
__device__ __forceinline__ int zt_hi(int k, int nz) { return min(nz - 1, k <= 1 ? max(k + 3, 5) : k + 3); }

template <int NB>
__global__ void __launch_bounds__(ZT_TILE / 2, 3) k_split_pass2_zt(const __grid_constant__ Batch<SplitHydroArgs, NB> bt)
{
    PDL_WAIT();
    const SplitHydroArgs &a = BATCH_MEMBER(bt, NB);
    const int kc = a.kc;
    int *err = a.err;
    extern __shared__ __align__(128) float zring[];   // [slot][t', u, v, w][ZT_TILE]
    __shared__ __align__(8) uint64_t full[ZT_SLOTS];
    const int nz = a.nz;
    const size_t np = a.np;
    const size_t p0 = (size_t)blockIdx.x * ZT_TILE;
    const int k0 = blockIdx.y * kc, k1 = min(nz, k0 + kc);
    const int tid = threadIdx.x;
    auto lo_of = [&](int k) { return zt_lo(k, nz); };
    auto hi_of = [&](int k) { return zt_hi(k, nz); };
    const int kbase = lo_of(k0), kcap = hi_of(k1 - 1);
    auto parity = [&](int kk) { return (unsigned)(((kk - kbase) >> 3) & 1); };
    auto issue = [&](int kk) {   // one thread: plane kk of the four fields into slot kk mod 8
        uint64_t *b = &full[kk & (ZT_SLOTS - 1)];
        float *dst = zring + (size_t)(kk & (ZT_SLOTS - 1)) * 4 * ZT_TILE;
        const size_t off = (size_t)kk * np + p0;
        mbar_expect_tx(b, 4 * ZT_TILE * (unsigned)sizeof(float));
        tma_load(dst, a.t + off, ZT_TILE * sizeof(float), b);
        tma_load(dst + ZT_TILE, a.u + off, ZT_TILE * sizeof(float), b);
        tma_load(dst + 2 * ZT_TILE, a.v + off, ZT_TILE * sizeof(float), b);
        tma_load(dst + 3 * ZT_TILE, a.w + off, ZT_TILE * sizeof(float), b);
    };
    if (tid == 0) {
        for (int s = 0; s < ZT_SLOTS; s++) mbar_init(&full[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    int khi = min(kcap, hi_of(k0) + 1);   // highest plane issued (one plane of lookahead)
    if (tid == 0)
        for (int kk = kbase; kk <= khi; kk++) issue(kk);
    int kw = kbase - 1;                   // highest plane this thread has waited for
    bool ok = true;
    // after a failed wait: wait (bounded) for every copy still in flight
    auto drain = [&]() {
        for (int kk = max(kw + 1, khi - ZT_SLOTS + 1); kk <= khi; kk++)
            mbar_wait(&full[kk & (ZT_SLOTS - 1)], parity(kk));
    };
    const ZRing2 Rt{ reinterpret_cast<const V2 *>(zring) + tid };
    const ZRing2 Ru{ reinterpret_cast<const V2 *>(zring + ZT_TILE) + tid };
    const ZRing2 Rv{ reinterpret_cast<const V2 *>(zring + 2 * ZT_TILE) + tid };
    const ZRing2 Rw{ reinterpret_cast<const V2 *>(zring + 3 * ZT_TILE) + tid };
    const V2 h(a.ho12), sc(a.sc1);
    const size_t np2 = np / 2, q2 = p0 / 2 + tid;
    for (int k = k0; k < k1; k++) {
        if (k > k0) {
            // every thread is done with row k - 1: the slot of plane k - 4 is free
            if (!__syncthreads_and(ok)) {
                if (tid == 0) {
                    // report, then let the copies in flight land before the CTA exits
                    atomicExch(err, 1);
                    drain();
                }
                return;
            }
            const int want = min(kcap, hi_of(k) + 1);
            if (tid == 0 && want > khi) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                for (int kk = khi + 1; kk <= want; kk++) issue(kk);
            }
            khi = max(khi, want);
        }
        for (int kk = kw + 1; kk <= hi_of(k) && ok; kk++) ok = mbar_wait(&full[kk & (ZT_SLOTS - 1)], parity(kk));
        kw = max(kw, hi_of(k));
        if (!ok) continue;
        const V2 w0 = Rw(k);
        ZDer<V2> z;
        z.tzu = zd1upa(Rt, k, nz, 5, h, w0); z.tzp = zd1a(Rt, k, nz, 5, h); z.tzz = zd2a(Rt, k, nz, 0, sc);
        z.wzu = zd1upa(Rw, k, nz, 1, h, w0); z.wz = zd1a(Rw, k, nz, 1, h);
        z.uzu = zd1upa(Ru, k, nz, 2, h, w0); z.vzu = zd1upa(Rv, k, nz, 2, h, w0);
        z.uzz = zd2a(Ru, k, nz, 3, sc); z.vzz = zd2a(Rv, k, nz, 3, sc);
        split_pass2_point<V2>(a, (size_t)k * np2 + q2, k, z, Rt(k), Ru(k), Rv(k), w0,
                              P2Global<V2>{ a, (size_t)k * np2 + q2 });
    }
    if (!__syncthreads_and(ok) && tid == 0) {
        atomicExch(err, 1);
        drain();
    }
}

// z-marching: one thread per (i,j) column and chunk of kc planes, with
// 7-plane register windows of t', u, v, w
__global__ void __launch_bounds__(256) k_split_pass2(SplitHydroArgs a, int kc)
{
    PDL_WAIT();
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t np = a.np;
    if (q >= np) return;
    const int nz = a.nz;
    const int k0 = blockIdx.y * kc, k1 = min(nz, k0 + kc);
    const float h = a.ho12, s = a.sc1;
    float T[7], U[7], V[7], W[7];
#pragma unroll
    for (int d = 0; d < 7; d++) {
        const int kk = k0 - 3 + d;
        const bool ok = kk >= 0 && kk < nz;
        const size_t o = (size_t)kk * np + q;
        T[d] = ok ? a.t[o] : 0.0f;
        U[d] = ok ? a.u[o] : 0.0f;
        V[d] = ok ? a.v[o] : 0.0f;
        W[d] = ok ? a.w[o] : 0.0f;
    }
    for (int k = k0; k < k1; k++) {
        const size_t idx = (size_t)k * np + q;
        const float w0 = W[3];
        ZDer<float> z;
        if (k >= 3 && k <= nz - 4) {
            z.tzu = wd1up(T, h, w0); z.tzp = wd1(T, h); z.tzz = wd2(T, s);
            z.wzu = wd1up(W, h, w0); z.wz = wd1(W, h);
            z.uzu = wd1up(U, h, w0); z.vzu = wd1up(V, h, w0);
            z.uzz = wd2(U, s); z.vzz = wd2(V, s);
        } else {
            z.tzu = zd1up(a.t + q, np, k, nz, 5, h, w0); z.tzp = zd1(a.t + q, np, k, nz, 5, h);
            z.tzz = zd2(a.t + q, np, k, nz, 0, s);
            z.wzu = zd1up(a.w + q, np, k, nz, 1, h, w0); z.wz = zd1(a.w + q, np, k, nz, 1, h);
            z.uzu = zd1up(a.u + q, np, k, nz, 2, h, w0); z.vzu = zd1up(a.v + q, np, k, nz, 2, h, w0);
            z.uzz = zd2(a.u + q, np, k, nz, 3, s); z.vzz = zd2(a.v + q, np, k, nz, 3, s);
        }
        split_pass2_point<float>(a, idx, k, z);
#pragma unroll
        for (int d = 0; d < 6; d++) { T[d] = T[d + 1]; U[d] = U[d + 1]; V[d] = V[d + 1]; W[d] = W[d + 1]; }
        const int kn = k + 4;
        const bool ok = kn < nz;
        const size_t o = (size_t)kn * np + q;
        T[6] = ok ? a.t[o] : 0.0f;
        U[6] = ok ? a.u[o] : 0.0f;
        V[6] = ok ? a.v[o] : 0.0f;
        W[6] = ok ? a.w[o] : 0.0f;
    }
}

struct SplitHydro4Args {
    const float *r, *t, *w, *p3, *p4, *g, *hh, *racc, *uacc, *vacc, *wacc;
    // horizontal derivatives of the second-level fluxes: d(p1)/dx, d(q)/dy into
    // u; d(q)/dx, d(p2)/dy into v; d(g)/dx, d(h)/dy into w
    const float *dxu, *dyu, *dxv, *dyv, *dxw, *dyw;
    const double *bg;
    const float *pc;
    const HistTable *ht;    // rdot, udot, vdot, wdot = newest slots
    float ho12;
    int mag;                // 0: g, h and the derivatives of q, g, h are zero (not read)
    size_t np;
    int nz;
    int kc;                 // z-pencil kernel: planes per chunk
    int *err;               // z-pencil kernel: the bounded waits' error flag
};

// one thread per point, grid (np/256, nz): k = blockIdx.y
__global__ void k_split_pass4(SplitHydro4Args a)
{
    PDL_WAIT();
    const size_t np = a.np;
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const int nz = a.nz;
    const int k = blockIdx.y;
    const size_t idx = (size_t)k * np + q;
    const float h = a.ho12;
    const double *bg = a.bg;
    const float *pc = a.pc;
    const float rho0 = pc[PC_RHO0 * nz + k], t0 = pc[PC_T0 * nz + k];
    const float rp = a.r[idx], tp = a.t[idx], w0 = a.w[idx];
    const float rr = rho0 + rp, tt = t0 + tp;
    // (sums in the order of the reference's accumulation: x, then y, then z)
    // (without a magnetic field q, g and h are zero: their terms are left out)
    const bool mg = a.mag != 0;
    const float wacc = mg ? (a.wacc[idx] + a.dxw[idx]) + a.dyw[idx] : a.wacc[idx];
    const float uacc = mg ? (a.uacc[idx] + a.dxu[idx]) + a.dyu[idx] : a.uacc[idx] + a.dxu[idx];
    const float vacc = mg ? (a.vacc[idx] + a.dxv[idx]) + a.dyv[idx] : a.vacc[idx] + a.dyv[idx];
    float wd = wacc + zd1(a.p3 + q, np, k, nz, 2, h) + zd1(a.p4 + q, np, k, nz, 5, h);
    const float ud = mg ? uacc + zd1(a.g + q, np, k, nz, 5, h) : uacc;
    const float vd = mg ? vacc + zd1(a.hh + q, np, k, nz, 5, h) : vacc;
    float rdot, wfin;
    if (k == 0 || k == nz - 1) {
        // src/hydro_deriv.f90:455-470: d(rho)/dz chosen so that dw/dt = 0
        const double wdn = (double)wd + bg[BG_A * nz + k];
        const double rz = wdn / (double)tt;
        rdot = a.racc[idx] - w0 * (float)rz;
        wfin = (float)(wdn - (double)tt * rz);
    } else {
        const bool wpos = w0 >= 0.0f;
        const float rzu = zd1up(a.r + q, np, k, nz, 0, h, w0) + pc[(wpos ? PC_RHO0ZU_P : PC_RHO0ZU_M) * nz + k];
        const float rzp = zd1(a.r + q, np, k, nz, 0, h);
        rdot = a.racc[idx] - w0 * rzu;
        wfin = wd + pc[PC_AB * nz + k] - t0 * rzp - tp * pc[PC_RHO0Z0 * nz + k] - tp * rzp;
    }
    const float ri = 1.0f / rr;
    ((float *)a.ht->p[0][2])[idx] = rdot;
    ((float *)a.ht->p[2][2])[idx] = ud * ri;
    ((float *)a.ht->p[3][2])[idx] = vd * ri;
    ((float *)a.ht->p[4][2])[idx] = wfin * ri;
}

// per-component access of the vector point types
template <typename T> struct VecN;
template <> struct VecN<V4> {
    static constexpr int n = 4;
    static __device__ __forceinline__ void get(const V4 &v, float *o) { o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w; }
    static __device__ __forceinline__ V4 make(const float *o) { return V4(o[0], o[1], o[2], o[3]); }
    static __device__ __forceinline__ V4 recip(const V4 &v) { return V4(1.0f / v.x, 1.0f / v.y, 1.0f / v.z, 1.0f / v.w); }
};

// the same for VecN<T>::n consecutive x points per thread (nx % 4 == 0):
// 16-byte loads and stores, grid (np/n/256, nz)
template <typename T, int NB>
__device__ __forceinline__ void split_pass4_vec(const Batch<SplitHydro4Args, NB> &bt)
{
    constexpr int NV = VecN<T>::n;
    const SplitHydro4Args &a = BATCH_MEMBER(bt, NB);
    const size_t npv = a.np / NV;
    const size_t qv = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (qv >= npv) return;
    const int nz = a.nz;
    const int k = blockIdx.y;
    const size_t iv = (size_t)k * npv + qv;
    const T h(a.ho12);
    const double *bg = a.bg;
    const float *pc = a.pc;
    auto ld = [](const float *p, size_t i) { return reinterpret_cast<const T *>(p)[i]; };
    const T *p3 = reinterpret_cast<const T *>(a.p3) + qv, *p4 = reinterpret_cast<const T *>(a.p4) + qv;
    const T *g = reinterpret_cast<const T *>(a.g) + qv, *hh = reinterpret_cast<const T *>(a.hh) + qv;
    const T *rrv = reinterpret_cast<const T *>(a.r) + qv;
    const float rho0 = pc[PC_RHO0 * nz + k], t0 = pc[PC_T0 * nz + k];
    const T rp = ld(a.r, iv), tp = ld(a.t, iv), w0 = ld(a.w, iv);
    const T rr = T(rho0) + rp, tt = T(t0) + tp;
    // (without a magnetic field q, g and h are zero: their terms are left out)
    const bool mg = a.mag != 0;
    const T wacc = mg ? (ld(a.wacc, iv) + ld(a.dxw, iv)) + ld(a.dyw, iv) : ld(a.wacc, iv);
    const T uacc = mg ? (ld(a.uacc, iv) + ld(a.dxu, iv)) + ld(a.dyu, iv) : ld(a.uacc, iv) + ld(a.dxu, iv);
    const T vacc = mg ? (ld(a.vacc, iv) + ld(a.dxv, iv)) + ld(a.dyv, iv) : ld(a.vacc, iv) + ld(a.dyv, iv);
    T wd = wacc + zd1(p3, npv, k, nz, 2, h) + zd1(p4, npv, k, nz, 5, h);
    const T ud = mg ? uacc + zd1(g, npv, k, nz, 5, h) : uacc;
    const T vd = mg ? vacc + zd1(hh, npv, k, nz, 5, h) : vacc;
    const T racc = ld(a.racc, iv);
    T rdot, wfin;
    if (k == 0 || k == nz - 1) {
        // src/hydro_deriv.f90:455-470: d(rho)/dz chosen so that dw/dt = 0
        const double A = bg[BG_A * nz + k];
        float rd[NV], wf[NV], wdv[NV], ttv[NV], w0v[NV], rav[NV];
        VecN<T>::get(wd, wdv); VecN<T>::get(tt, ttv); VecN<T>::get(w0, w0v); VecN<T>::get(racc, rav);
#pragma unroll
        for (int c = 0; c < NV; c++) {
            const double wdn = (double)wdv[c] + A;
            const double rz = wdn / (double)ttv[c];
            rd[c] = rav[c] - w0v[c] * (float)rz;
            wf[c] = (float)(wdn - (double)ttv[c] * rz);
        }
        rdot = VecN<T>::make(rd);
        wfin = VecN<T>::make(wf);
    } else {
        const T up(pc[PC_RHO0ZU_P * nz + k]), um(pc[PC_RHO0ZU_M * nz + k]);
        const T rzu = zd1up(rrv, npv, k, nz, 0, h, w0) + upsel(w0, up, um);
        const T rzp = zd1(rrv, npv, k, nz, 0, h);
        rdot = racc - w0 * rzu;
        wfin = wd + T(pc[PC_AB * nz + k]) - T(t0) * rzp - tp * T(pc[PC_RHO0Z0 * nz + k]) - tp * rzp;
    }
    const T ri = VecN<T>::recip(rr);
    reinterpret_cast<T *>(a.ht->p[0][2])[iv] = rdot;
    reinterpret_cast<T *>(a.ht->p[2][2])[iv] = ud * ri;
    reinterpret_cast<T *>(a.ht->p[3][2])[iv] = vd * ri;
    reinterpret_cast<T *>(a.ht->p[4][2])[iv] = wfin * ri;
}

// four points per thread, four CTAs per SM (64 registers with a few spilled
// values; 5.3 TB/s against 4.2 at the compiler's own 94 registers, and 5.0
// against 4.3 for two points per thread at 56 registers without spills)
template <int NB>
__global__ void __launch_bounds__(256, 4) k_split_pass4_v4(const __grid_constant__ Batch<SplitHydro4Args, NB> bt)
{
    PDL_WAIT();
    split_pass4_vec<V4, NB>(bt);
}

// Pass 4 with TMA-staged z-pencils: the planes of the fields its z stencils
// read -- p3, p4, r' and (with a magnetic field) g, h -- in an eight-slot
// shared-memory ring filled by bulk copies one plane ahead, as in
// k_split_pass2_zt; a CTA owns ZT_TILE consecutive points of a chunk of
// about kc planes, two points per thread; the other inputs are read
// directly.  Same arithmetic as k_split_pass4_v4, value for value.
#define Z4_FIELDS 5
template <int NB>
__global__ void __launch_bounds__(ZT_TILE / 2, 2) k_split_pass4_zt(const __grid_constant__ Batch<SplitHydro4Args, NB> bt)
{
    PDL_WAIT();
    const SplitHydro4Args &a = BATCH_MEMBER(bt, NB);
    const int kc = a.kc;
    int *err = a.err;
    extern __shared__ __align__(128) float zring[];   // [slot][p3, p4, r', g, h][ZT_TILE]
    __shared__ __align__(8) uint64_t full[ZT_SLOTS];
    const int nz = a.nz;
    const size_t np = a.np;
    const size_t p0 = (size_t)blockIdx.x * ZT_TILE;
    const int k0 = blockIdx.y * kc, k1 = min(nz, k0 + kc);
    const int tid = threadIdx.x;
    const bool mg = a.mag != 0;
    const int nf = mg ? 5 : 3;   // (g and h are zero without a magnetic field)
    const int kbase = zt_lo(k0, nz), kcap = zt_hi(k1 - 1, nz);
    auto parity = [&](int kk) { return (unsigned)(((kk - kbase) >> 3) & 1); };
    auto issue = [&](int kk) {   // one thread: plane kk of the ring's fields into slot kk mod 8
        uint64_t *b = &full[kk & (ZT_SLOTS - 1)];
        float *dst = zring + (size_t)(kk & (ZT_SLOTS - 1)) * Z4_FIELDS * ZT_TILE;
        const size_t off = (size_t)kk * np + p0;
        mbar_expect_tx(b, (unsigned)nf * ZT_TILE * (unsigned)sizeof(float));
        tma_load(dst, a.p3 + off, ZT_TILE * sizeof(float), b);
        tma_load(dst + ZT_TILE, a.p4 + off, ZT_TILE * sizeof(float), b);
        tma_load(dst + 2 * ZT_TILE, a.r + off, ZT_TILE * sizeof(float), b);
        if (mg) {
            tma_load(dst + 3 * ZT_TILE, a.g + off, ZT_TILE * sizeof(float), b);
            tma_load(dst + 4 * ZT_TILE, a.hh + off, ZT_TILE * sizeof(float), b);
        }
    };
    if (tid == 0) {
        for (int s = 0; s < ZT_SLOTS; s++) mbar_init(&full[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    int khi = min(kcap, zt_hi(k0, nz) + 1);   // highest plane issued (one plane of lookahead)
    if (tid == 0)
        for (int kk = kbase; kk <= khi; kk++) issue(kk);
    int kw = kbase - 1;                       // highest plane this thread has waited for
    bool ok = true;
    // after a failed wait: wait (bounded) for every copy still in flight
    auto drain = [&]() {
        for (int kk = max(kw + 1, khi - ZT_SLOTS + 1); kk <= khi; kk++)
            mbar_wait(&full[kk & (ZT_SLOTS - 1)], parity(kk));
    };
    const V2 *zr = reinterpret_cast<const V2 *>(zring) + tid;
    const ZRingF<Z4_FIELDS> Rp3{ zr }, Rp4{ zr + ZT_TILE / 2 }, Rr{ zr + ZT_TILE }, Rg{ zr + 3 * ZT_TILE / 2 },
        Rh{ zr + 2 * ZT_TILE };
    const V2 h(a.ho12);
    const double *bg = a.bg;
    const float *pc = a.pc;
    const size_t np2 = np / 2, q2 = p0 / 2 + tid;
    for (int k = k0; k < k1; k++) {
        if (k > k0) {
            // every thread is done with row k - 1: the slot of plane k - 4 is free
            if (!__syncthreads_and(ok)) {
                if (tid == 0) {
                    // report, then let the copies in flight land before the CTA exits
                    atomicExch(err, 1);
                    drain();
                }
                return;
            }
            const int want = min(kcap, zt_hi(k, nz) + 1);
            if (tid == 0 && want > khi) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                for (int kk = khi + 1; kk <= want; kk++) issue(kk);
            }
            khi = max(khi, want);
        }
        for (int kk = kw + 1; kk <= zt_hi(k, nz) && ok; kk++) ok = mbar_wait(&full[kk & (ZT_SLOTS - 1)], parity(kk));
        kw = max(kw, zt_hi(k, nz));
        if (!ok) continue;
        const size_t i2 = (size_t)k * np2 + q2;
        const float rho0 = pc[PC_RHO0 * nz + k], t0 = pc[PC_T0 * nz + k];
        const V2 rp = Rr(k), tp = ldv<V2>(a.t, i2), w0 = ldv<V2>(a.w, i2);
        const V2 rr = V2(rho0) + rp, tt = V2(t0) + tp;
        const V2 wacc = mg ? (ldv<V2>(a.wacc, i2) + ldv<V2>(a.dxw, i2)) + ldv<V2>(a.dyw, i2) : ldv<V2>(a.wacc, i2);
        const V2 uacc = mg ? (ldv<V2>(a.uacc, i2) + ldv<V2>(a.dxu, i2)) + ldv<V2>(a.dyu, i2)
                           : ldv<V2>(a.uacc, i2) + ldv<V2>(a.dxu, i2);
        const V2 vacc = mg ? (ldv<V2>(a.vacc, i2) + ldv<V2>(a.dxv, i2)) + ldv<V2>(a.dyv, i2)
                           : ldv<V2>(a.vacc, i2) + ldv<V2>(a.dyv, i2);
        V2 wd = wacc + zd1a(Rp3, k, nz, 2, h) + zd1a(Rp4, k, nz, 5, h);
        const V2 ud = mg ? uacc + zd1a(Rg, k, nz, 5, h) : uacc;
        const V2 vd = mg ? vacc + zd1a(Rh, k, nz, 5, h) : vacc;
        const V2 racc = ldv<V2>(a.racc, i2);
        V2 rdot, wfin;
        if (k == 0 || k == nz - 1) {
            // src/hydro_deriv.f90:455-470: d(rho)/dz chosen so that dw/dt = 0
            const double A = bg[BG_A * nz + k];
            const float wdv[2] = { wd.x, wd.y }, ttv[2] = { tt.x, tt.y };
            const float w0v[2] = { w0.x, w0.y }, rav[2] = { racc.x, racc.y };
            float rd[2], wf[2];
#pragma unroll
            for (int c = 0; c < 2; c++) {
                const double wdn = (double)wdv[c] + A;
                const double rz = wdn / (double)ttv[c];
                rd[c] = rav[c] - w0v[c] * (float)rz;
                wf[c] = (float)(wdn - (double)ttv[c] * rz);
            }
            rdot = V2(rd[0], rd[1]);
            wfin = V2(wf[0], wf[1]);
        } else {
            const V2 up(pc[PC_RHO0ZU_P * nz + k]), um(pc[PC_RHO0ZU_M * nz + k]);
            const V2 rzu = zd1upa(Rr, k, nz, 0, h, w0) + upsel(w0, up, um);
            const V2 rzp = zd1a(Rr, k, nz, 0, h);
            rdot = racc - w0 * rzu;
            wfin = wd + V2(pc[PC_AB * nz + k]) - V2(t0) * rzp - tp * V2(pc[PC_RHO0Z0 * nz + k]) - tp * rzp;
        }
        const V2 ri(1.0f / rr.x, 1.0f / rr.y);
        stv((float *)a.ht->p[0][2], i2, rdot);
        stv((float *)a.ht->p[2][2], i2, ud * ri);
        stv((float *)a.ht->p[3][2], i2, vd * ri);
        stv((float *)a.ht->p[4][2], i2, wfin * ri);
    }
    if (!__syncthreads_and(ok) && tid == 0) {
        atomicExch(err, 1);
        drain();
    }
}

// the three forward transforms of E = u x B that mag_deriv starts with;
// with with_mag the x and y passes of the hydro derivatives carry them as
// extra jobs, so one launch per direction serves both
int split_emf_m(Engine *const *Es, int nE);
static void mag_fwd_jobs(Engine *E, LineJob<float> *fx, LineJob<float> *fy)
{
    float *W[W_COUNT];
    for (int i = 0; i < W_COUNT; i++) W[i] = E->W<float>(i);
    fx[0] = ljob<float>(W[W_M1], W[W_EX], OP_FWD);
    fx[1] = ljob<float>(W[W_M2], W[W_EY], OP_FWD);
    fx[2] = ljob<float>(W[W_M3], W[W_EZ], OP_FWD);
    fy[0] = ljob<float>(W[W_EX], W[W_EX], OP_FWD);
    fy[1] = ljob<float>(W[W_EY], W[W_EY], OP_FWD);
    fy[2] = ljob<float>(W[W_EZ], W[W_EZ], OP_FWD);
}

static SplitHydroArgs hydro_args(Engine *E)
{
    float *W[W_COUNT];
    for (int i = 0; i < W_COUNT; i++) W[i] = E->W<float>(i);
    const Consts &c = E->k;
    SplitHydroArgs a;
    a.r = E->r32; a.t = E->t32; a.u = E->u32; a.v = E->v32; a.w = E->w32;
    a.bx = E->bx32; a.by = E->by32; a.bz = E->bz32; a.jsq = E->jsq32;
    a.rx = W[W_RX]; a.tx = W[W_TX]; a.txx = W[W_TXX]; a.ux = W[W_UX]; a.uxx = W[W_UXX];
    a.vx = W[W_VX]; a.vxx = W[W_VXX]; a.wx = W[W_WX]; a.wxx = W[W_WXX];
    a.ry = W[W_RY]; a.ty = W[W_TY]; a.tyy = W[W_TYY]; a.uy = W[W_UY]; a.uyy = W[W_UYY];
    a.vy = W[W_VY]; a.vyy = W[W_VYY]; a.wy = W[W_WY]; a.wyy = W[W_WYY];
    a.pc = E->pcf;
    a.racc = W[W_RACC]; a.ht = E->ht;
    a.uacc = W[W_UACC]; a.vacc = W[W_VACC]; a.wacc = W[W_WACC];
    a.p1 = W[W_P1]; a.p2 = W[W_P2]; a.q = W[W_Q]; a.g = W[W_G]; a.hh = W[W_H]; a.p3 = W[W_P3]; a.p4 = W[W_P4];
    a.e1 = a.e2 = a.e3 = nullptr;
    a.gck = (float)c.gck; a.fzckg = (float)c.fzckg; a.gm1 = (float)c.gm1; a.sckg = (float)c.sckg;
    a.fo2 = (float)c.fo2; a.scko3 = (float)c.scko3; a.f = (float)c.f; a.thmplus1 = (float)c.thmplus1;
    a.cor = (float)c.cor; a.cpsi = (float)c.cpsi; a.spsi = (float)c.spsi; a.sck = (float)c.sck;
    a.ho12 = (float)c.ho12; a.sc1 = (float)c.sc1; a.bzbar = (float)E->bzbar;
    a.var_eta = c.var_eta; a.np = E->np; a.nz = E->nz;
    a.mag = split_mag_on(*E);
    // chunks of about kc_pass2 planes (tunable), balanced over nz
    const int kt = E->kc_pass2 > 0 ? E->kc_pass2 : 16;
    const int nch = (E->nz + kt - 1) / kt;
    a.kc = (E->nz + nch - 1) / nch;
    a.err = E->dev_err;
    return a;
}

// the second-level horizontal derivatives of pass 4 (the first-level
// derivative arrays, free once pass 2 has run)
#define DXU W_TXX
#define DXV W_UXX
#define DXW W_VXX
#define DYU W_TYY
#define DYV W_UYY
#define DYW W_VYY

static SplitHydro4Args hydro4_args(Engine *E)
{
    float *W[W_COUNT];
    for (int i = 0; i < W_COUNT; i++) W[i] = E->W<float>(i);
    SplitHydro4Args b;
    b.r = E->r32; b.t = E->t32; b.w = E->w32; b.p3 = W[W_P3]; b.p4 = W[W_P4]; b.g = W[W_G]; b.hh = W[W_H];
    b.racc = W[W_RACC]; b.uacc = W[W_UACC]; b.vacc = W[W_VACC]; b.wacc = W[W_WACC]; b.bg = E->hres; b.pc = E->pcf;
    b.dxu = W[DXU]; b.dyu = W[DYU]; b.dxv = W[DXV]; b.dyv = W[DYV]; b.dxw = W[DXW]; b.dyw = W[DYW];
    b.ht = E->ht;
    b.ho12 = (float)E->k.ho12; b.np = E->np; b.nz = E->nz;
    b.mag = split_mag_on(*E);
    b.kc = hydro_args(E).kc;
    b.err = E->dev_err;
    return b;
}

// True when the members' step can run as one launch per kernel: the
// four-point and z-pencil forms (a batch of one takes any form)
static bool batch_forms(Engine *const *Es, int nE)
{
    for (int i = 0; i < nE; i++) {
        const Engine *E = Es[i];
        if (!(E->nx % 4 == 0 && E->vec4 && E->zpencil && E->np % ZT_TILE == 0 && E->nz >= 6)) return nE == 1;
    }
    return true;
}

// hydro_deriv of the members (equally sized; one launch per kernel for all
// of them).  with_mag[i]: E = u x B of member i and its forward transforms
// ride in the line launches.
int split_hydro_m(Engine *const *Es, int nE, const bool *with_mag)
{
    Engine *E = Es[0];
    if (!batch_forms(Es, nE)) return VEC_ERR_ARG;
    int st;
    std::vector<LineJob<float>> jx, jy, kx, ky;
    for (int i = 0; i < nE; i++) {
        Engine *M = Es[i];
        float *W[W_COUNT];
        for (int q = 0; q < W_COUNT; q++) W[q] = M->W<float>(q);
        jx.push_back(ljob<float>(M->r32, W[W_RX], OP_D1));
        jx.push_back(ljob<float>(M->t32, W[W_TX], OP_D1, W[W_TXX], OP_D2));
        jx.push_back(ljob<float>(M->u32, W[W_UX], OP_D1, W[W_UXX], OP_D2));
        jx.push_back(ljob<float>(M->v32, W[W_VX], OP_D1, W[W_VXX], OP_D2));
        jx.push_back(ljob<float>(M->w32, W[W_WX], OP_D1, W[W_WXX], OP_D2));
        jy.push_back(ljob<float>(M->r32, W[W_RY], OP_D1));
        jy.push_back(ljob<float>(M->t32, W[W_TY], OP_D1, W[W_TYY], OP_D2));
        jy.push_back(ljob<float>(M->u32, W[W_UY], OP_D1, W[W_UYY], OP_D2));
        jy.push_back(ljob<float>(M->v32, W[W_VY], OP_D1, W[W_VYY], OP_D2));
        jy.push_back(ljob<float>(M->w32, W[W_WY], OP_D1, W[W_WYY], OP_D2));
        // the second-level fluxes' derivatives (after pass 2); the Lorentz
        // fluxes q, g, h only with a magnetic field
        kx.push_back(ljob<float>(W[W_P1], W[DXU], OP_D1));
        ky.push_back(ljob<float>(W[W_P2], W[DYV], OP_D1));
        if (split_mag_on(*M)) {
            kx.push_back(ljob<float>(W[W_Q], W[DXV], OP_D1));
            kx.push_back(ljob<float>(W[W_G], W[DXW], OP_D1));
            ky.push_back(ljob<float>(W[W_Q], W[DYU], OP_D1));
            ky.push_back(ljob<float>(W[W_H], W[DYW], OP_D1));
        }
        // with_mag: pass 2 writes E = u x B, and its forward transforms ride
        // in the second-level line launches
        if (with_mag[i]) {
            LineJob<float> fx[3], fy[3];
            mag_fwd_jobs(M, fx, fy);
            for (int q = 0; q < 3; q++) { kx.push_back(fx[q]); ky.push_back(fy[q]); }
        }
    }
    if ((st = launch_lines<float>(E, 0, jx.data(), (int)jx.size()))) return st;
    if ((st = launch_lines<float>(E, 1, jy.data(), (int)jy.size()))) return st;

    // pass 2 (with E = u x B for the members whose mag branch shares the
    // transforms: 3 fields more)
    int im = 0;
    auto p2args = [&im, with_mag](Engine *e) {
        SplitHydroArgs a = hydro_args(e);
        if (with_mag[im++]) {
            a.e1 = e->W<float>(W_M1);
            a.e2 = e->W<float>(W_M2);
            a.e3 = e->W<float>(W_M3);
        }
        return a;
    };
    const double p2b = FB(E, split_mag_on(*E) ? (with_mag[0] ? 42 : 39) : 32, 4);
    if (E->zpencil && E->np % ZT_TILE == 0 && E->nz >= 6) {
        static bool attr = false;
        const size_t smem = (size_t)ZT_SLOTS * 4 * ZT_TILE * sizeof(float);
        if (!attr) {
            CUDA_TRY(cudaFuncSetAttribute(k_split_pass2_zt<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            CUDA_TRY(cudaFuncSetAttribute(k_split_pass2_zt<BATCH_MAX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
            attr = true;
        }
        const int kc = hydro_args(E).kc;
        st = launch_members<SplitHydroArgs>(Es, nE, "hydro_pass2_f32", p2b,
                                            dim3((unsigned)(E->np / ZT_TILE), (unsigned)((E->nz + kc - 1) / kc)),
                                            dim3(ZT_TILE / 2), smem, k_split_pass2_zt<1>, k_split_pass2_zt<BATCH_MAX>,
                                            p2args);
        if (st) return st;
    } else if (E->nx % 4 == 0 && E->vec4) {
        if (nE != 1) return VEC_ERR_ARG;
        const SplitHydroArgs a = p2args(E);
        KLAUNCHB(E, "hydro_pass2_f32", p2b, k_split_pass2_v2, dim3((unsigned)nblk(E->np / 2), (unsigned)E->nz), TPB,
                 a);
    } else {
        if (nE != 1) return VEC_ERR_ARG;
        const SplitHydroArgs a = p2args(E);
        dim3 g2(nblk(E->np), (unsigned)((E->nz + a.kc - 1) / a.kc));
        KLAUNCHB(E, "hydro_pass2_f32", p2b, k_split_pass2, g2, TPB, a, a.kc);
    }

    // The second-level horizontal derivatives go to separate arrays and
    // pass 4 adds them: a line pass that accumulates into its output reads
    // each output element before writing it, and that dependent read made
    // those two launches the slowest line passes of the step.
    if ((st = launch_lines<float>(E, 0, kx.data(), (int)kx.size()))) return st;
    if ((st = launch_lines<float>(E, 1, ky.data(), (int)ky.size()))) return st;

    // (the z-pencil form pays where the per-plane form's z neighbours fall
    // out of L2: 4.8 against 3.9 TB/s at 1024^2 x 513; at 512^2 x 257 and
    // below its two CTAs per SM lose to four: 4.6 against 5.6 TB/s)
    const bool zt4 = E->zpencil4 == 1 || (E->zpencil4 < 0 && E->np >= (size_t)1024 * 1024);
    if (E->nx % 4 == 0 && E->vec4 && E->zpencil && zt4 && E->np % ZT_TILE == 0 && E->nz >= 6) {
        static bool attr4 = false;
        const size_t smem = (size_t)ZT_SLOTS * Z4_FIELDS * ZT_TILE * sizeof(float);
        if (!attr4) {
            CUDA_TRY(cudaFuncSetAttribute(k_split_pass4_zt<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            CUDA_TRY(cudaFuncSetAttribute(k_split_pass4_zt<BATCH_MAX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
            attr4 = true;
        }
        const int kc = hydro4_args(E).kc;
        if ((st = launch_members<SplitHydro4Args>(Es, nE, "hydro_pass4_f32", FB(E, split_mag_on(*E) ? 21 : 15, 4),
                                                  dim3((unsigned)(E->np / ZT_TILE), (unsigned)((E->nz + kc - 1) / kc)),
                                                  dim3(ZT_TILE / 2), smem, k_split_pass4_zt<1>,
                                                  k_split_pass4_zt<BATCH_MAX>, hydro4_args)))
            return st;
    } else if (E->nx % 4 == 0 && E->vec4) {
        if ((st = launch_members<SplitHydro4Args>(Es, nE, "hydro_pass4_f32", FB(E, split_mag_on(*E) ? 21 : 15, 4),
                                                  dim3((unsigned)nblk(E->np / 4), (unsigned)E->nz), dim3(TPB), 0,
                                                  k_split_pass4_v4<1>, k_split_pass4_v4<BATCH_MAX>, hydro4_args)))
            return st;
    } else {
        const SplitHydro4Args b = hydro4_args(E);
        KLAUNCHB(E, "hydro_pass4_f32", FB(E, split_mag_on(*E) ? 21 : 15, 4), k_split_pass4, plane_grid(*E), TPB, b);
    }
    return VEC_OK;
}
int split_hydro(Engine *E, bool with_mag) { return split_hydro_m(&E, 1, &with_mag); }

// ---- mag_deriv ---------------------------------------------------------------
// E = u x B (real space, FP32)
int split_emf_m(Engine *const *Es, int nE)
{
    Engine *E = Es[0];
    auto mk = [](Engine *e) {
        float *W1 = e->W<float>(W_M1), *W2 = e->W<float>(W_M2), *W3 = e->W<float>(W_M3);
        return Emf4Args{ e->u32, e->v32, e->w32, e->bx32, e->by32, e->bz32, W1, W2, W3, e->n / 4, (float)e->bzbar };
    };
    if (E->nx % 4 == 0 && E->vec4)
        return launch_members<Emf4Args>(Es, nE, "emf_f32", FB(E, 9, 4), dim3(nblk(E->n / 4)), dim3(TPB), 0,
                                        k_emf4<1>, k_emf4<BATCH_MAX>, mk);
    if (nE != 1) return VEC_ERR_ARG;
    KLAUNCHB(E, "emf_f32", FB(E, 9, 4), k_emf<float>, nblk(E->n), TPB, E->u32, E->v32, E->w32, E->bx32, E->by32,
             E->bz32, E->W<float>(W_M1), E->W<float>(W_M2), E->W<float>(W_M3), E->n, (float)E->bzbar);
    return VEC_OK;
}
int split_emf(Engine *E) { return split_emf_m(&E, 1); }

static MeanArgs<float> mean_args(Engine *E, bool ab3_coef)
{
    const Consts &c = E->k;
    const bool v4 = E->nx % 4 == 0 && E->vec4;
    MeanArgs<float> ma;
    ma.ex = E->W<float>(W_EX); ma.ey = E->W<float>(W_EY); ma.bxbar = E->bxbar; ma.bybar = E->bybar;
    ma.eta = E->eta; ma.deta = E->deta;
    ma.ht = E->ht; ma.scratch = E->w1d; ma.np = E->np; ma.nz = E->nz;
    ma.xn = c.xn; ma.zck = c.zck; ma.ho12 = c.ho12; ma.sc1 = c.sc1; ma.var_eta = c.var_eta;
    ma.ds = v4 && ab3_coef ? E->ds : nullptr; ma.bxm = E->bxbar; ma.bym = E->bybar;
    return ma;
}

static MagArgs<float> mag_args(Engine *E)
{
    const Consts &c = E->k;
    MagArgs<float> a;
    a.ex = E->W<float>(W_EX); a.ey = E->W<float>(W_EY); a.ez = E->W<float>(W_EZ); a.w1 = E->W<float>(W_M4);
    a.pol = E->pol32; a.tor = E->tor32;
    a.eta = E->pcf + PC_ETA * E->nz; a.deta = E->pcf + PC_DETA * E->nz; a.h = E->hf;
    a.ht = E->ht;
    a.zck = (float)c.zck; a.ho12 = (float)c.ho12; a.sc1 = (float)c.sc1; a.var_eta = c.var_eta;
    a.nx = E->nx; a.ny = E->ny; a.nz = E->nz;
    return a;
}

int split_mag_m(Engine *const *Es, int nE, bool ab3_coef, bool spectra_done)
{
    Engine *E = Es[0];
    int st;
    const bool v4 = E->nx % 4 == 0 && E->vec4;
    if (!v4 && nE != 1) return VEC_ERR_ARG;
    const dim3 g4((unsigned)nblk(E->np / 4), (unsigned)E->nz);
    if (!spectra_done) {
        if ((st = split_emf_m(Es, nE))) return st;
        std::vector<LineJob<float>> fx(3 * nE), fy(3 * nE);
        for (int i = 0; i < nE; i++) mag_fwd_jobs(Es[i], &fx[3 * i], &fy[3 * i]);
        if ((st = launch_lines<float>(E, 0, fx.data(), 3 * nE))) return st;
        if ((st = launch_lines<float>(E, 1, fy.data(), 3 * nE))) return st;
    }
    if (v4) {
        if ((st = launch_members<MagDiv4Args>(Es, nE, "mag_div_f32", FB(E, 3, 4), dim3(g4.x, g4.y + 1), dim3(TPB), 0,
                                              k_mag_div4<1>, k_mag_div4<BATCH_MAX>, [ab3_coef](Engine *e) {
                                                  return MagDiv4Args{ e->W<float>(W_EX), e->W<float>(W_EY),
                                                                      e->W<float>(W_M4), e->nx, e->ny, e->hf,
                                                                      mean_args(e, ab3_coef) };
                                              })))
            return st;
        return launch_members<MagArgs<float>>(Es, nE, "mag_final_f32", FB(E, 8, 4), g4, dim3(TPB), 0,
                                              k_mag_final4<1>, k_mag_final4<BATCH_MAX>, mag_args);
    }
    const MeanArgs<float> ma = mean_args(E, ab3_coef);
    KLAUNCHB(E, "mean_rhs", 0, k_mean_rhs<float>, 1, 256, ma);
    KLAUNCHB(E, "mag_div_f32", FB(E, 3, 4), k_mag_div<float>, plane_grid(*E), TPB, E->W<float>(W_EX),
             E->W<float>(W_EY), E->W<float>(W_M4), E->nx, E->ny, E->hf);
    const MagArgs<float> a = mag_args(E);
    KLAUNCHB(E, "mag_final_f32", FB(E, 8, 4), k_mag_final<float>, plane_grid(*E), TPB, a);
    if (ab3_coef) return phys_ab3_coef(E);
    return VEC_OK;
}
int split_mag(Engine *E, bool ab3_coef, bool spectra_done) { return split_mag_m(&E, 1, ab3_coef, spectra_done); }

// ---- bandj --------------------------------------------------------------------
// z-marching, grid (np/256, nz/kc)
__global__ void __launch_bounds__(256) k_d1z_f(const float *in, float *out, int fl, size_t np, int nz, float h,
                                               int kc)
{
    PDL_WAIT();
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const int k0 = blockIdx.y * kc, k1 = min(nz, k0 + kc);
    float v[7];
    zwin_init(v, in + q, np, k0, nz);
    for (int k = k0; k < k1; k++) {
        out[(size_t)k * np + q] = (k >= 3 && k <= nz - 4) ? wd1(v, h) : zd1(in + q, np, k, nz, fl, h);
        zwin_next(v, in + q, np, k, nz);
    }
}

// four consecutive x points per thread, grid (np/4/256, nz)
// with rot set, an extra first CTA row (blockIdx.y == 0) rotates the history
// table: the first kernel after the AB3 update, and none of its planes reads
// the table
struct D1z4Args {
    const float *in;
    float *out;
    int fl;
    size_t np;
    int nz;
    float h;
    HistTable *rot;
};
template <int NB>
__global__ void __launch_bounds__(256) k_d1z4(const __grid_constant__ Batch<D1z4Args, NB> bt)
{
    PDL_WAIT();
    const D1z4Args &A = BATCH_MEMBER(bt, NB);
    const float *in = A.in;
    float *out = A.out;
    const int fl = A.fl, nz = A.nz;
    const size_t np = A.np;
    const float h = A.h;
    HistTable *rot = A.rot;
    if (rot && blockIdx.y == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) rotate_hist_table(rot);
        return;
    }
    const size_t np4 = np / 4;
    const size_t q4 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q4 >= np4) return;
    const int k = (int)blockIdx.y - (rot ? 1 : 0);
    reinterpret_cast<V4 *>(out)[(size_t)k * np4 + q4] = zd1(reinterpret_cast<const V4 *>(in) + q4, np4, k, nz, fl, V4(h));
}

// bandj of the members (equally sized; one launch per kernel for all)
int split_bandj_m(Engine *const *Es, int nE, bool rotate_hist)
{
    Engine *E = Es[0];
    int st;
    const bool v4 = E->nx % 4 == 0 && E->vec4;
    if (!v4 && nE != 1) return VEC_ERR_ARG;
    const dim3 g4((unsigned)nblk(E->np / 4), (unsigned)E->nz);
    if (!v4 && rotate_hist && (st = phys_rotate_hist(E))) return st;
    if (v4) {
        if ((st = launch_members<D1z4Args>(Es, nE, "d1bydz_f32", FB(E, 2, 4), dim3(g4.x, g4.y + (rotate_hist ? 1 : 0)),
                                           dim3(TPB), 0, k_d1z4<1>, k_d1z4<BATCH_MAX>, [rotate_hist](Engine *e) {
                                               return D1z4Args{ e->pol32, e->W<float>(W_M1), 5, e->np, e->nz,
                                                                (float)e->k.ho12, rotate_hist ? e->ht : nullptr };
                                           })))
            return st;
    } else {
        KLAUNCHB(E, "d1bydz_f32", FB(E, 2, 4), k_d1z_f, zmarch_grid(E->np, E->nz), TPB, E->pol32, E->W<float>(W_M1),
                 5, E->np, E->nz, (float)E->k.ho12, ZCHUNK);
    }
    auto bj = [](Engine *e) {
        BandjArgs<float> a;
        a.dzs = e->W<float>(W_M1); a.pol = e->pol32; a.tor = e->tor32; a.h = e->hf;
        a.bxh = e->W<float>(W_EX); a.byh = e->W<float>(W_EY); a.bzh = e->W<float>(W_EZ);
        a.dybz = nullptr; a.dxbz = nullptr; a.jzh = e->W<float>(W_M4);   // d(bz)/dx, dy: below
        a.nx = e->nx; a.ny = e->ny; a.nz = e->nz;
        return a;
    };
    if (v4) {
        if ((st = launch_members<BandjArgs<float>>(Es, nE, "bandj_spec_f32", FB(E, 7, 4), g4, dim3(TPB), 0,
                                                   k_bandj_spec4<1>, k_bandj_spec4<BATCH_MAX>, bj)))
            return st;
    } else {
        const BandjArgs<float> a = bj(E);
        KLAUNCHB(E, "bandj_spec_f32", FB(E, 7, 4), k_bandj_spec<float>, plane_grid(*E), TPB, a);
    }
    std::vector<LineJob<float>> ix, iy;
    for (int i = 0; i < nE; i++) {
        Engine *M = Es[i];
        float *W[W_COUNT];
        for (int q = 0; q < W_COUNT; q++) W[q] = M->W<float>(q);
        // the x inverse of bz's spectrum also gives that of d(bz)/dx (into
        // M3); the y inverse of the former gives bz and d(bz)/dy (into M2)
        ix.push_back(ljob<float>(W[W_EX], W[W_EX], OP_INV));
        ix.push_back(ljob<float>(W[W_EY], W[W_EY], OP_INV));
        ix.push_back(ljob<float>(W[W_EZ], W[W_EZ], OP_INV, W[W_M3], OP_D1));
        ix.push_back(ljob<float>(W[W_M4], W[W_M4], OP_INV));
        // bz32 keeps bz - bzbar: no constant added
        LineJob<float> jbx = ljob<float>(W[W_EX], M->bx32, OP_INV), jby = ljob<float>(W[W_EY], M->by32, OP_INV);
        jbx.addk = M->bxbar;
        jby.addk = M->bybar;
        iy.push_back(jbx);
        iy.push_back(jby);
        iy.push_back(ljob<float>(W[W_EZ], M->bz32, OP_INV, W[W_M2], OP_D1));
        iy.push_back(ljob<float>(W[W_M3], W[W_M3], OP_INV));
        iy.push_back(ljob<float>(W[W_M4], W[W_M4], OP_INV));
    }
    if ((st = launch_lines<float>(E, 0, ix.data(), (int)ix.size()))) return st;
    if ((st = launch_lines<float>(E, 1, iy.data(), (int)iy.size()))) return st;
    if (v4) {
        if ((st = launch_members<Jsq4Args>(Es, nE, "jsq_f32", FB(E, 6, 4), g4, dim3(TPB), 0, k_jsq4<1>,
                                           k_jsq4<BATCH_MAX>, [](Engine *e) {
                                               return Jsq4Args{ e->W<float>(W_M4), e->W<float>(W_M2),
                                                                e->W<float>(W_M3), e->bx32, e->by32, e->jsq32, e->np,
                                                                e->nz, (float)e->k.ho12 };
                                           })))
            return st;
    } else {
        KLAUNCHB(E, "jsq_f32", FB(E, 6, 4), k_jsq<float>, plane_grid(*E), TPB, E->W<float>(W_M4), E->W<float>(W_M2),
                 E->W<float>(W_M3), E->bx32, E->by32, E->jsq32, E->np, E->nz, (float)E->k.ho12);
    }
    for (int i = 0; i < nE; i++) Es[i]->b32_auth = 1;
    return VEC_OK;
}
int split_bandj(Engine *E, bool rotate_hist) { return split_bandj_m(&E, 1, rotate_hist); }

// ---- AB3 update in FP64 with FP32 histories ------------------------------------------
struct SplitAb3Args {
    double *x[7];
    int hmap[7];           // history table row of each state field
    const HistTable *ht;
    float *m[7];           // mirrors, same order
    const double *bg;
    const DevScalars *ds;
    int nx, ny, nz, cx, cy, magdealias;
    int nf;                // 7, or 5 without a magnetic field: pol and tor
                           // (zero right-hand side) are left as they are
};

// src/main.F90:413-462 with FP64 accumulation; order u,v,w,r,t,pol,tor
__global__ void k_split_ab3(SplitAb3Args a)
{
    PDL_WAIT();
    const size_t np = (size_t)a.nx * a.ny;
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= np * a.nz) return;
    const int k = (int)(idx / np);
    const float c0 = (float)a.ds->c0, c1 = (float)a.ds->c1, c2 = (float)a.ds->c2;
#define H(f, s) ((const float *)a.ht->p[a.hmap[f]][s])
    double xs[7];
#pragma unroll
    for (int f = 0; f < 5; f++)
        xs[f] = a.x[f][idx] + (double)(c0 * H(f, 2)[idx] + c1 * H(f, 1)[idx] + c2 * H(f, 0)[idx]);
    if (xs[3] < 0.05) {
        xs[3] = 0.05;
        ((float *)a.ht->p[0][1])[idx] = 0.0f;
        ((float *)a.ht->p[0][2])[idx] = 0.0f;
    }
    bool trunc = false;
    if (a.magdealias) {
        size_t q = idx - (size_t)k * np;
        int j = (int)(q / a.nx), i = (int)(q - (size_t)j * a.nx);
        trunc = truncated(i, j, a.nx, a.ny, a.cx, a.cy);
    }
    const int nf = a.nf;
#pragma unroll
    for (int f = 5; f < 7; f++) {
        if (f >= nf) break;
        double v = a.x[f][idx] + (double)(c0 * H(f, 2)[idx] + c1 * H(f, 1)[idx] + c2 * H(f, 0)[idx]);
        xs[f] = trunc ? 0.0 : v;
    }
#undef H
#pragma unroll
    for (int f = 0; f < 7; f++)
        if (f < nf) a.x[f][idx] = xs[f];
    a.m[0][idx] = (float)xs[0];
    a.m[1][idx] = (float)xs[1];
    a.m[2][idx] = (float)xs[2];
    a.m[3][idx] = (float)(xs[3] - a.bg[BG_RHO0 * a.nz + k]);
    a.m[4][idx] = (float)(xs[4] - a.bg[BG_T0 * a.nz + k]);
    if (nf == 7) {
        a.m[5][idx] = (float)xs[5];
        a.m[6][idx] = (float)xs[6];
    }
}

// four consecutive points per thread (x fastest, nx % 4 == 0): 16-byte
// loads and stores of the FP32 histories/mirrors and of the FP64 state.
// ICVT: the float <-> double conversions on the integer pipe (fpconv.cuh),
// leaving the FP64 pipe only the additions; same bits as the casts.
// (no launch bound: the compiler's 78 registers at three CTAs per SM beat
// four CTAs at 64 registers, 6.0 against 5.8 TB/s)
template <bool ICVT, int NB>
__global__ void k_split_ab3_v4(const __grid_constant__ Batch<SplitAb3Args, NB> bt)
{
    PDL_WAIT();
    const SplitAb3Args &a = BATCH_MEMBER(bt, NB);
    const size_t np = (size_t)a.nx * a.ny;
    const size_t i4 = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) * 4;
    if (i4 >= np * a.nz) return;
    const int k = (int)(i4 / np);
    // the increment c0 h3 + c1 h2 + c2 h1 is formed in FP32 (the precision of
    // the histories); only the accumulation into the state is FP64
    const float c0 = (float)a.ds->c0, c1 = (float)a.ds->c1, c2 = (float)a.ds->c2;
    double xs[7][4];
    const int nf = a.nf;
#pragma unroll
    for (int f = 0; f < 7; f++) {
        if (f >= nf) break;
        const double2 s01 = *reinterpret_cast<const double2 *>(a.x[f] + i4);
        const double2 s23 = *reinterpret_cast<const double2 *>(a.x[f] + i4 + 2);
        const float *const *hp = (const float *const *)a.ht->p[a.hmap[f]];
        const float4 h2 = *reinterpret_cast<const float4 *>(hp[2] + i4);
        const float4 h1 = *reinterpret_cast<const float4 *>(hp[1] + i4);
        const float4 h0 = *reinterpret_cast<const float4 *>(hp[0] + i4);
        const float i0 = c0 * h2.x + c1 * h1.x + c2 * h0.x, i1 = c0 * h2.y + c1 * h1.y + c2 * h0.y;
        const float i2 = c0 * h2.z + c1 * h1.z + c2 * h0.z, i3 = c0 * h2.w + c1 * h1.w + c2 * h0.w;
        if (ICVT) {
            xs[f][0] = s01.x + f2d_exact(i0);
            xs[f][1] = s01.y + f2d_exact(i1);
            xs[f][2] = s23.x + f2d_exact(i2);
            xs[f][3] = s23.y + f2d_exact(i3);
        } else {
            xs[f][0] = s01.x + (double)i0;
            xs[f][1] = s01.y + (double)i1;
            xs[f][2] = s23.x + (double)i2;
            xs[f][3] = s23.y + (double)i3;
        }
    }
    // density floor (src/main.F90:438-443)
    const bool fl0 = xs[3][0] < 0.05, fl1 = xs[3][1] < 0.05, fl2 = xs[3][2] < 0.05, fl3 = xs[3][3] < 0.05;
    if (fl0 | fl1 | fl2 | fl3) {
        const bool fl[4] = { fl0, fl1, fl2, fl3 };
        float *r1 = (float *)a.ht->p[0][1], *r2 = (float *)a.ht->p[0][2];
#pragma unroll
        for (int q = 0; q < 4; q++)
            if (fl[q]) { xs[3][q] = 0.05; r1[i4 + q] = 0.0f; r2[i4 + q] = 0.0f; }
    }
    if (a.magdealias) {
        const size_t qq = i4 - (size_t)k * np;
        const int j = (int)(qq / a.nx), i = (int)(qq - (size_t)j * a.nx);
#pragma unroll
        for (int q = 0; q < 4; q++)
            if (truncated(i + q, j, a.nx, a.ny, a.cx, a.cy)) { xs[5][q] = 0.0; xs[6][q] = 0.0; }
    }
    const double rb = a.bg[BG_RHO0 * a.nz + k], tb = a.bg[BG_T0 * a.nz + k];
#pragma unroll
    for (int f = 0; f < 7; f++) {
        if (f >= nf) break;
        *reinterpret_cast<double2 *>(a.x[f] + i4) = make_double2(xs[f][0], xs[f][1]);
        *reinterpret_cast<double2 *>(a.x[f] + i4 + 2) = make_double2(xs[f][2], xs[f][3]);
        float4 m;
        if (f == 3 || f == 4) {
            const double b = f == 3 ? rb : tb;
            if (ICVT) m = make_float4(d2f_rn(xs[f][0] - b), d2f_rn(xs[f][1] - b), d2f_rn(xs[f][2] - b), d2f_rn(xs[f][3] - b));
            else m = make_float4((float)(xs[f][0] - b), (float)(xs[f][1] - b), (float)(xs[f][2] - b), (float)(xs[f][3] - b));
        } else {
            if (ICVT) m = make_float4(d2f_rn(xs[f][0]), d2f_rn(xs[f][1]), d2f_rn(xs[f][2]), d2f_rn(xs[f][3]));
            else m = make_float4((float)xs[f][0], (float)xs[f][1], (float)xs[f][2], (float)xs[f][3]);
        }
        *reinterpret_cast<float4 *>(a.m[f] + i4) = m;
    }
}

static SplitAb3Args ab3_args(Engine *E, int magdealias)
{
    SplitAb3Args a;
    double *xs[7] = { E->u, E->v, E->w, E->r, E->t, E->pol, E->tor };
    float *ms[7] = { E->u32, E->v32, E->w32, E->r32, E->t32, E->pol32, E->tor32 };
    const int hmap[7] = { 2, 3, 4, 0, 1, 5, 6 };
    for (int f = 0; f < 7; f++) {
        a.x[f] = xs[f];
        a.m[f] = ms[f];
        a.hmap[f] = hmap[f];
    }
    a.ht = E->ht;
    a.bg = E->hres;
    a.ds = E->ds;
    a.nx = E->nx; a.ny = E->ny; a.nz = E->nz; a.cx = E->k.icutoffx; a.cy = E->k.icutoffy;
    a.magdealias = magdealias;
    a.nf = split_mag_on(*E) ? 7 : 5;
    return a;
}

// AB3 update of the members (equally sized): magdealias[i] as in split_ab3;
// members not folded[i] get the coefficient step before and the history
// rotation after the update
int split_ab3_m(Engine *const *Es, int nE, const int *magdealias, const bool *folded)
{
    Engine *E = Es[0];
    int st;
    Engine *unf[BATCH_MAX];
    int nu = 0;
    int md[BATCH_MAX];
    for (int i = 0; i < nE; i++) {
        if (!folded[i]) unf[nu++] = Es[i];
        md[i] = magdealias[i];
    }
    if (nu && (st = phys_ab3_coef_m(unf, nu))) return st;
    // state 14 x 8 B, histories 21 x 4 B, mirrors 7 x 4 B (without a
    // magnetic field 10 x 8, 15 x 4 and 5 x 4 B)
    const double bytes = (double)E->n * (split_mag_on(*E) ? 14 * 8 + 21 * 4 + 7 * 4 : 10 * 8 + 15 * 4 + 5 * 4);
    if (E->nx % 4 == 0) {
        // (the members' magdealias flags, in member order)
        int i = 0;
        auto mk = [&i, md](Engine *e) { return ab3_args(e, md[i++]); };
        st = E->int_cvt ? launch_members<SplitAb3Args>(Es, nE, "ab3_update_split", bytes, dim3(nblk(E->n / 4)),
                                                       dim3(TPB), 0, k_split_ab3_v4<true, 1>,
                                                       k_split_ab3_v4<true, BATCH_MAX>, mk)
                        : launch_members<SplitAb3Args>(Es, nE, "ab3_update_split", bytes, dim3(nblk(E->n / 4)),
                                                       dim3(TPB), 0, k_split_ab3_v4<false, 1>,
                                                       k_split_ab3_v4<false, BATCH_MAX>, mk);
        if (st) return st;
    } else {
        if (nE != 1) return VEC_ERR_ARG;
        const SplitAb3Args a = ab3_args(E, md[0]);
        KLAUNCHB(E, "ab3_update_split", bytes, k_split_ab3, nblk(E->n), TPB, a);
    }
    return nu ? phys_rotate_hist_m(unf, nu) : VEC_OK;
}
int split_ab3(Engine *E, int magdealias, bool folded) { return split_ab3_m(&E, 1, &magdealias, &folded); }

// ---- dealias of r,t,u,v,w (every 10 steps) -----------------------------------------
// The background is horizontally uniform, so the 2/3 truncation only touches
// the perturbation: x64 -= x32 - D(x32), then the mirror is refreshed.
struct DealiasArgs {
    double *x[5];
    float *m[5];
    const float *d[5];
    const double *bg;
    size_t np;
    int nz;
};

// grid (np/256, nz); float <-> double conversions on the integer pipe (the
// same bits as the casts; the FP64 pipe keeps only the subtractions)
template <int NB>
__global__ void k_split_dealias_apply(const __grid_constant__ Batch<DealiasArgs, NB> bt)
{
    PDL_WAIT();
    const DealiasArgs &a = BATCH_MEMBER(bt, NB);
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.np) return;
    const int k = blockIdx.y;
    const size_t idx = (size_t)k * a.np + q;
#pragma unroll
    for (int f = 0; f < 5; f++) {
        double xn = a.x[f][idx] - (f2d_exact(a.m[f][idx]) - f2d_exact(a.d[f][idx]));
        a.x[f][idx] = xn;
        if (f < 2) a.m[f][idx] = d2f_rn(xn - a.bg[(f == 0 ? BG_RHO0 : BG_T0) * a.nz + k]);
        else a.m[f][idx] = d2f_rn(xn);
    }
}

static DealiasArgs dealias_args(Engine *E)
{
    DealiasArgs a;
    float *ms[5] = { E->r32, E->t32, E->u32, E->v32, E->w32 };
    double *xs[5] = { E->r, E->t, E->u, E->v, E->w };
    const int tmp[5] = { W_RX, W_TX, W_UX, W_VX, W_WX };
    for (int i = 0; i < 5; i++) { a.x[i] = xs[i]; a.m[i] = ms[i]; a.d[i] = E->W<float>(tmp[i]); }
    a.bg = E->hres; a.np = E->np; a.nz = E->nz;
    return a;
}

// dealias of r, t, u, v, w of the members (equally sized)
int split_dealias_m(Engine *const *Es, int nE)
{
    Engine *E = Es[0];
    std::vector<LineJob<float>> jx, jy;
    for (int m = 0; m < nE; m++) {
        const DealiasArgs a = dealias_args(Es[m]);
        for (int i = 0; i < 5; i++) {
            jx.push_back(ljob<float>(a.m[i], (float *)a.d[i], OP_DEALIAS));
            jy.push_back(ljob<float>(a.d[i], (float *)a.d[i], OP_DEALIAS));
        }
    }
    int st;
    if ((st = launch_lines<float>(E, 0, jx.data(), (int)jx.size())) ||
        (st = launch_lines<float>(E, 1, jy.data(), (int)jy.size())))
        return st;
    return launch_members<DealiasArgs>(Es, nE, "dealias_apply_split", FB(E, 5, 24), plane_grid(*E), dim3(TPB), 0,
                                       k_split_dealias_apply<1>, k_split_dealias_apply<BATCH_MAX>, dealias_args);
}
int split_dealias(Engine *E) { return split_dealias_m(&E, 1); }

// ---- calcdt on the FP64 state with the FP32 field ---------------------------------------
int split_calcdt(Engine *E)
{
    int st = split_sync_b64(E);
    if (st) return st;
    return phys_calcdt(E);
}

// calcdt of the members (equally sized)
int split_calcdt_m(Engine *const *Es, int nE)
{
    Engine *sync[BATCH_MAX];
    int ns = 0;
    for (int i = 0; i < nE; i++)
        if (Es[i]->b32_auth) sync[ns++] = Es[i];
    int st;
    if (ns && (st = split_sync_b64_m(sync, ns))) return st;
    return phys_calcdt_m(Es, nE);
}
