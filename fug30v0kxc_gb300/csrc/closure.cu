// closure.cu -- the learned closure coupled to the solver (no reference
// counterpart; the spectral upsampler follows interpolate/fft.F90:834-927).
//
// A closure pairs a fine context (the DNS) with coarse contexts of the same
// physics on a grid r times coarser in x and y and (nz_f - 1) = r (nz_c - 1)
// in z, so coarse planes sit on fine planes (vertex-aligned).
//
//  * box filter: weights (1, 2, ..., 2, 1) / 2r over 2r+1 fine points per
//    axis around the coarse point (periodic in x, y); the wall planes take
//    the wall values alone, so the filtered state keeps w = 0 and the wall
//    temperatures.
//  * training pair: input = filtered fine state (u, v, w, rho - rho0(z),
//    T - T0(z), Bx, By, Bz - mean Bz); target = filtered fine RHS minus the
//    coarse RHS evaluated at the filtered state, channels (du, dv, dw, drho,
//    dT, dBx, dBy, dBz)/dt.  dB/dt comes from the induction RHS (poldot,
//    tordot, mean-field RHS) through the linear part of bandj.
//  * inference: the network's correction is split into the hydro RHS
//    corrections and a magnetic correction projected on (pol, tor, means)
//    the way mag_init maps a real-space field (src/magnetic.f90:5-279); the
//    coarse step adds it to the newest RHS slots, so it is integrated by the
//    AB3 update like the rest of the RHS.
//  * the judged run: every J coarse steps the coarse state is upsampled to
//    the fine grid and the plain fine solver runs a short segment; when the
//    coarse run reaches the segment's end time, the Nusselt number and the
//    kinetic / magnetic energies are compared, and if any differs by more
//    than the tolerance the run continues on the fine solver.
#include <cuda_bf16.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "common.cuh"
#include "engine.h"
#include "closure_net.h"
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
        kern<<<(grid), (block), 0, (E)->stream>>>(__VA_ARGS__);  \
        (E)->prof_end();                                         \
        CUDA_TRY(cudaGetLastError());                            \
    } while (0)
#define KLAUNCH(E, name, kern, grid, block, ...) KLAUNCHB(E, name, 0, kern, grid, block, __VA_ARGS__)

typedef __nv_bfloat16 bf16;

extern "C" int vec_get_scalars(vec_ctx *c, vec_scalars *s);
extern "C" int vec_set_scalars(vec_ctx *c, const vec_scalars *s);
extern "C" int vec_step(vec_ctx *c, int nsteps);
extern "C" int vec_diag(vec_ctx *c, vec_diag_out *out);
extern "C" int vec_calcdt(vec_ctx *c, double *dt);
extern "C" int vec_create(const vec_params *p, vec_ctx **out);
extern "C" int vec_destroy(vec_ctx *c);
extern "C" int vec_net_create(int nx, int ny, int nz, int batch, unsigned long long seed, vec_net **out);
extern "C" int vec_net_destroy(vec_net *N);

static int mag_on(const Engine &E) { return E.p.f != 0.0 || E.p.kinematic; }

struct vec_closure {
    int r = 4;                       // coarsening factor
    int nxc, nyc, nzc;
    size_t npc;                      // coarse points per sample
    vec_net *net = nullptr;
    int batch = 8;
    int cap = 0, npairs = 0;
    float *in_ds = nullptr, *tg_ds = nullptr;   // [cap][npc][8] raw
    float *nrm = nullptr;            // device [32]: in mean, in std, out mean, out std
    float hnrm[32];
    float *filt_rhs = nullptr, *crhs = nullptr; // [npc][8] scratch
    double *stats = nullptr;         // [32] sums
    double *acc = nullptr;           // [2] evaluation sums
    double *rho0c = nullptr, *t0c = nullptr;    // coarse background profiles
    double *rho0f = nullptr, *t0f = nullptr;    // fine background profiles (allocated per fine nz)
    int nzf_bg = 0;
    vec_params pc;                   // coarse parameters
    float clip = 4.0f;               // |normalised output| limit at inference
    float gain = 1.0f;               // scale of the applied correction
    vec_ctx *cs = nullptr;           // scratch coarse context (filtered diagnostics of a fine state)
};

// ---- background profiles: T0 = 1 + theta z, rho0 = T0^m (src/initial.F90:49-58)
static int upload_bg(const vec_params &p, int nz, double **rho0, double **t0)
{
    std::vector<double> r(nz), t(nz);
    for (int k = 0; k < nz; k++) {
        const double z = (double)k / (double)(nz - 1);
        t[k] = 1.0 + p.theta * z;
        r[k] = pow(t[k], p.cm);
    }
    if (cudaMalloc(rho0, sizeof(double) * nz) != cudaSuccess || cudaMalloc(t0, sizeof(double) * nz) != cudaSuccess) {
        cudaGetLastError();
        return VEC_ERR_ALLOC;
    }
    CUDA_TRY(cudaMemcpy(*rho0, r.data(), sizeof(double) * nz, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(*t0, t.data(), sizeof(double) * nz, cudaMemcpyHostToDevice));
    return VEC_OK;
}

// ---- box filter -----------------------------------------------------------------------
struct FiltSrc {
    const void *f[8];
    int dbl[8];              // 1: double, 0: float
    const double *sub[8];    // per-plane background subtracted (or null)
    double off[8];           // constant subtracted
};

__device__ __forceinline__ double ldv(const void *p, int dbl, size_t i)
{
    return dbl ? ((const double *)p)[i] : (double)((const float *)p)[i];
}

// out[pc][c] (c = 0..7) from fine fields; r even
__global__ void k_box_filter(FiltSrc s, int nxf, int nyf, int nzf, int r, int nxc, int nyc, int nzc, float *out)
{
    const size_t npc = (size_t)nxc * nyc;
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= npc * nzc) return;
    const int kc = (int)(idx / npc);
    const size_t q = idx - (size_t)kc * npc;
    const int jc = (int)(q / nxc), ic = (int)(q - (size_t)jc * nxc);
    const int h = r / 2;
    const size_t npf = (size_t)nxf * nyf;
    const bool wall = kc == 0 || kc == nzc - 1;
    double acc[8];
#pragma unroll
    for (int c = 0; c < 8; c++) acc[c] = 0.0;
    for (int dk = wall ? 0 : -h; dk <= (wall ? 0 : h); dk++) {
        const int kf = r * kc + dk;
        const double wz = wall ? 1.0 : ((dk == -h || dk == h) ? 0.5 : 1.0) / r;
        for (int dj = -h; dj <= h; dj++) {
            const int jf = (r * jc + dj + nyf) % nyf;
            const double wy = ((dj == -h || dj == h) ? 0.5 : 1.0) / r;
            for (int di = -h; di <= h; di++) {
                const int jif = (r * ic + di + nxf) % nxf;
                const double wgt = wz * wy * ((di == -h || di == h) ? 0.5 : 1.0) / r;
                const size_t fi = (size_t)kf * npf + (size_t)jf * nxf + jif;
#pragma unroll
                for (int c = 0; c < 8; c++) {
                    double v = ldv(s.f[c], s.dbl[c], fi) - s.off[c];
                    if (s.sub[c]) v -= s.sub[c][kf];
                    acc[c] += wgt * v;
                }
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 8; c++) out[idx * 8 + c] = (float)acc[c];
}

// the same channels without filtering (coarse RHS)
__global__ void k_pack8(FiltSrc s, size_t n, float *out)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
#pragma unroll
    for (int c = 0; c < 8; c++) out[i * 8 + c] = (float)(ldv(s.f[c], s.dbl[c], i) - s.off[c]);
}

// state of a context from filtered channels
__global__ void k_set_state(const float *in, double *u, double *v, double *w, double *r, double *t, double *bx,
                            double *by, double *bz, const double *rho0, const double *t0, double bzbar, size_t np,
                            int nz)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np * nz) return;
    const int k = (int)(i / np);
    const float *a = in + i * 8;
    u[i] = a[0]; v[i] = a[1]; w[i] = a[2];
    r[i] = rho0[k] + a[3];
    t[i] = t0[k] + a[4];
    bx[i] = a[5]; by[i] = a[6]; bz[i] = bzbar + a[7];
}

__global__ void k_sub8(const float *a, const float *b, float *c, size_t n)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) c[i] = a[i] - b[i];
}

// ---- dB/dt from the induction RHS (the linear part of bandj, src/magnetic.f90:492-617)
template <typename R>
__global__ void k_d1z_t(const R *in, R *out, size_t np, int nz, R h)
{
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= np * nz) return;
    int k = (int)(idx / np);
    out[idx] = zd1(in + (idx - (size_t)k * np), np, k, nz, 5, h);
}

// bx, by, bz (real space, precision R) from spectral (pol, tor) and the
// means (bxm, bym); bz without a constant
template <typename R>
static int bandj_linear(Engine *E, const R *pol, const R *tor, const double *bxm, const double *bym, R *bx, R *by,
                        R *bz)
{
    R *W[W_COUNT];
    for (int i = 0; i < W_COUNT; i++) W[i] = E->W<R>(i);
    int st;
    KLAUNCH(E, "closure_d1z", k_d1z_t<R>, nblk(E->n), TPB, pol, W[W_M1], E->np, E->nz, (R)E->k.ho12);
    BandjArgs<R> a;
    a.dzs = W[W_M1]; a.pol = pol; a.tor = tor; a.h = htab<R>(*E);
    a.bxh = W[W_EX]; a.byh = W[W_EY]; a.bzh = W[W_EZ]; a.dybz = W[W_M2]; a.dxbz = W[W_M3]; a.jzh = W[W_M4];
    a.nx = E->nx; a.ny = E->ny; a.nz = E->nz;
    KLAUNCH(E, "closure_bandj_spec", k_bandj_spec<R>, plane_grid(*E), TPB, a);
    LineJob<R> ix[3] = { ljob<R>(W[W_EX], W[W_EX], OP_INV), ljob<R>(W[W_EY], W[W_EY], OP_INV),
                         ljob<R>(W[W_EZ], W[W_EZ], OP_INV) };
    if ((st = launch_lines<R>(E, 0, ix, 3))) return st;
    LineJob<R> iy[3] = { ljob<R>(W[W_EX], bx, OP_INV), ljob<R>(W[W_EY], by, OP_INV), ljob<R>(W[W_EZ], bz, OP_INV) };
    iy[0].addk = bxm;
    iy[1].addk = bym;
    return launch_lines<R>(E, 1, iy, 3);
}

// RHS of the current state into the newest history slots (hydro_deriv and
// mag_deriv, or the zeroed magnetic RHS when F = 0)
static int eval_rhs(Engine &E)
{
    int st;
    if ((st = E.split ? split_hydro(&E) : phys_hydro64(&E))) return st;
    if (mag_on(E)) return E.split ? split_mag(&E) : phys_mag64(&E);
    return phys_zero_mag_rhs(&E);
}

// FiltSrc of the eight RHS channels of a context after eval_rhs; the three
// dB/dt channels are computed into the context's FP64 scratch arrays s64[0..2]
// (each holds n values of either precision)
static int rhs_channels(Engine &E, FiltSrc *s)
{
    HistTable h;
    int st = hist_table_host(&E, &h);
    if (st) return st;
    void *bx = E.s64[0], *by = E.s64[1], *bz = E.s64[2];
    if (E.split) {
        if ((st = bandj_linear<float>(&E, (const float *)h.p[5][2], (const float *)h.p[6][2], h.bx[2], h.by[2],
                                      (float *)bx, (float *)by, (float *)bz)))
            return st;
    } else {
        if ((st = bandj_linear<double>(&E, (const double *)h.p[5][2], (const double *)h.p[6][2], h.bx[2], h.by[2],
                                       (double *)bx, (double *)by, (double *)bz)))
            return st;
    }
    // channels: du, dv, dw, drho, dT, dBx, dBy, dBz (history rows u=2, v=3, w=4, r=0, t=1)
    const void *f[8] = { h.p[2][2], h.p[3][2], h.p[4][2], h.p[0][2], h.p[1][2], bx, by, bz };
    for (int c = 0; c < 8; c++) {
        s->f[c] = f[c];
        s->dbl[c] = E.split ? 0 : 1;
        s->sub[c] = nullptr;
        s->off[c] = 0.0;
    }
    return VEC_OK;
}

// FP64 state channels (B made current first in the split form)
static int state_channels(Engine &E, const double *rho0, const double *t0, FiltSrc *s)
{
    int st;
    if (E.split && (st = split_sync_b64(&E))) return st;
    const void *f[8] = { E.u, E.v, E.w, E.r, E.t, E.bx, E.by, E.bz };
    for (int c = 0; c < 8; c++) {
        s->f[c] = f[c];
        s->dbl[c] = 1;
        s->sub[c] = nullptr;
        s->off[c] = 0.0;
    }
    s->sub[3] = rho0;
    s->sub[4] = t0;
    s->off[7] = E.bzbar;
    return VEC_OK;
}

static int check_pair(const vec_closure *cl, const Engine &F, const Engine &Cc)
{
    if (Cc.nx != cl->nxc || Cc.ny != cl->nyc || Cc.nz != cl->nzc || F.nx != cl->r * cl->nxc ||
        F.ny != cl->r * cl->nyc || F.nz - 1 != cl->r * (cl->nzc - 1)) {
        vec_set_error("closure: grids do not match (coarse %dx%dx%d, factor %d)", cl->nxc, cl->nyc, cl->nzc, cl->r);
        return VEC_ERR_ARG;
    }
    return VEC_OK;
}

static int fine_bg(vec_closure *cl, const Engine &F)
{
    if (cl->nzf_bg == F.nz) return VEC_OK;
    if (cl->rho0f) cudaFree(cl->rho0f);
    if (cl->t0f) cudaFree(cl->t0f);
    cl->rho0f = cl->t0f = nullptr;
    int st = upload_bg(F.p, F.nz, &cl->rho0f, &cl->t0f);
    if (!st) cl->nzf_bg = F.nz;
    return st;
}

// filtered fine state into out [npc][8] (on the coarse context's stream)
static int filter_state(vec_closure *cl, Engine &F, Engine &Cc, float *out)
{
    int st;
    if ((st = fine_bg(cl, F))) return st;
    FiltSrc s;
    if ((st = state_channels(F, cl->rho0f, cl->t0f, &s))) return st;
    KLAUNCH((&F), "box_filter", k_box_filter, nblk(cl->npc), TPB, s, F.nx, F.ny, F.nz, cl->r, Cc.nx, Cc.ny, Cc.nz,
            out);
    return VEC_OK;
}

// coarse context state from filtered channels, then pol/tor (mag_init), B
// and the boundary conditions as after a time step
static int set_coarse(vec_closure *cl, Engine &Cc, const float *in, double bzbar)
{
    int st;
    Cc.bzbar = bzbar;
    KLAUNCH((&Cc), "closure_set_state", k_set_state, nblk(Cc.n), TPB, in, Cc.u, Cc.v, Cc.w, Cc.r, Cc.t, Cc.bx, Cc.by,
            Cc.bz, cl->rho0c, cl->t0c, bzbar, Cc.np, Cc.nz);
    Cc.b32_auth = 0;
    if (mag_on(Cc) && (st = phys_mag_init(&Cc))) return st;
    if (Cc.split && (st = split_refresh(&Cc))) return st;
    if (mag_on(Cc) && (st = Cc.split ? split_bandj(&Cc) : phys_bandj64(&Cc))) return st;
    int s2 = phys_boundary(&Cc);
    if (s2) return s2;
    if (Cc.split && (st = split_refresh_planes(&Cc, 1 | 2))) return st;
    return VEC_OK;
}

// ---- normalisation and training batches ------------------------------------------------
__global__ void k_stats(const float *a, size_t n8, double *sums)
{
    double loc[16];
#pragma unroll
    for (int c = 0; c < 16; c++) loc[c] = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n8; i += (size_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const double v = a[i * 8 + c];
            loc[c] += v;
            loc[8 + c] += v * v;
        }
    }
    // warp reduction, then one atomic per warp and channel
#pragma unroll
    for (int c = 0; c < 16; c++) {
        double v = loc[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&sums[c], v);
    }
}

struct BatchIdx { int i[64]; };

// x0 [B][P][16]: normalised inputs, z coordinate in channel 8; tgt [B][P][8]
__global__ void k_gather(const float *in_ds, const float *tg_ds, BatchIdx bi, int B, size_t P, size_t np, int nz,
                         const float *nrm, bf16 *x0, float *tgt)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)B * P) return;
    const int b = (int)(i / P);
    const size_t p = i - (size_t)b * P;
    const size_t src = ((size_t)bi.i[b] * P + p) * 8;
    const int k = (int)(p / np);
    float v[16];
#pragma unroll
    for (int c = 0; c < 8; c++) v[c] = (in_ds[src + c] - nrm[c]) / nrm[8 + c];
    v[8] = nz > 1 ? -1.0f + 2.0f * (float)k / (float)(nz - 1) : 0.0f;
#pragma unroll
    for (int c = 9; c < 16; c++) v[c] = 0.0f;
#pragma unroll
    for (int c = 0; c < 16; c += 2)
        *reinterpret_cast<__nv_bfloat162 *>(x0 + i * 16 + c) = __floats2bfloat162_rn(v[c], v[c + 1]);
    if (tgt) {
#pragma unroll
        for (int c = 0; c < 8; c++) tgt[i * 8 + c] = (tg_ds[src + c] - nrm[16 + c]) / nrm[24 + c];
    }
}

// sums of (out - tgt)^2 and tgt^2
__global__ void k_eval_acc(const float *out, const float *tgt, size_t n, double *acc)
{
    double a = 0.0, b = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double d = (double)out[i] - tgt[i];
        a += d * d;
        b += (double)tgt[i] * tgt[i];
    }
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) { atomicAdd(&acc[0], a); atomicAdd(&acc[1], b); }
}

// ---- inference -----------------------------------------------------------------------------
// x0 [P][16] from a coarse context's state (B from the FP32 mirrors in the
// split form, whose bz32 is bz - bzbar)
__global__ void k_pack_state(const double *u, const double *v, const double *w, const double *r, const double *t,
                             const void *bx, const void *by, const void *bz, int bdbl, double bzoff,
                             const double *rho0, const double *t0, const float *nrm, size_t np, int nz, bf16 *x0)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np * nz) return;
    const int k = (int)(i / np);
    float a[16];
    a[0] = (float)u[i]; a[1] = (float)v[i]; a[2] = (float)w[i];
    a[3] = (float)(r[i] - rho0[k]);
    a[4] = (float)(t[i] - t0[k]);
    a[5] = (float)ldv(bx, bdbl, i);
    a[6] = (float)ldv(by, bdbl, i);
    a[7] = (float)(ldv(bz, bdbl, i) - bzoff);
#pragma unroll
    for (int c = 0; c < 8; c++) a[c] = (a[c] - nrm[c]) / nrm[8 + c];
    a[8] = nz > 1 ? -1.0f + 2.0f * (float)k / (float)(nz - 1) : 0.0f;
#pragma unroll
    for (int c = 9; c < 16; c++) a[c] = 0.0f;
#pragma unroll
    for (int c = 0; c < 16; c += 2)
        *reinterpret_cast<__nv_bfloat162 *>(x0 + i * 16 + c) = __floats2bfloat162_rn(a[c], a[c + 1]);
}

// denormalised network output -> hydro corrections (history rows r, t, u, v,
// w) and the real-space dB/dt correction (3 arrays)
// (the normalised output is limited to +-clip standard deviations of the
// training targets and the correction scaled by gain)
template <typename R>
__global__ void k_corr_split(const float *out, const float *nrm, size_t n, R *corr, R *bd, float clip, float gain)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float v[8];
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const float o = fminf(fmaxf(out[i * 8 + c], -clip), clip);
        v[c] = gain * (o * nrm[24 + c] + nrm[16 + c]);
    }
    corr[0 * n + i] = (R)v[3];   // rho
    corr[1 * n + i] = (R)v[4];   // T
    corr[2 * n + i] = (R)v[0];   // u
    corr[3 * n + i] = (R)v[1];   // v
    corr[4 * n + i] = (R)v[2];   // w
    bd[0 * n + i] = (R)v[5];
    bd[1 * n + i] = (R)v[6];
    bd[2 * n + i] = (R)v[7];
}

// (pol, tor) corrections from the truncated spectra of dB/dt, as mag_init
// maps B (src/magnetic.f90:123-150)
template <typename R>
__global__ void k_corr_poltor(const R *ex, const R *ey, const R *ez, R *pol, R *tor, int nx, int ny, int nz,
                              const double *akx1, const double *aky1, const double *akx2, const double *aky2)
{
    const size_t np = (size_t)nx * ny;
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= np * nz) return;
    const int k = (int)(idx / np);
    const size_t q = idx - (size_t)k * np;
    const int j = (int)(q / nx), i = (int)(q - (size_t)j * nx);
    const R *pey = ey + (size_t)k * np, *pex = ex + (size_t)k * np;
    const R kk = (R)(akx2[i] + aky2[j]);
    R p = (R)0, t = (R)0;
    if (!(i == 0 && j == 0)) {
        p = (R)-1 * ez[idx] / kk;
        const R jz = sdx(pey, i, j, nx, akx1) - sdy(pex, i, j, nx, ny, aky1);
        t = (R)-1 * jz / kk;
    }
    pol[idx] = p;
    tor[idx] = t;
}

template <typename R>
__global__ void k_corr_means(const R *ex, const R *ey, double *bxm, double *bym, size_t np, int nz, double xn)
{
    for (int k = threadIdx.x; k < nz; k += blockDim.x) {
        bxm[k] = (double)ex[(size_t)k * np] * xn;
        bym[k] = (double)ey[(size_t)k * np] * xn;
    }
}

// newest RHS slots += correction
template <typename R>
__global__ void k_add_corr(const HistTable *ht, const R *corr, const double *cbx, const double *cby, size_t n, int nz,
                           int mag)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
#pragma unroll
        for (int f = 0; f < 5; f++) ((R *)ht->p[f][2])[i] += corr[(size_t)f * n + i];
        if (mag) {
            ((R *)ht->p[5][2])[i] += corr[5 * n + i];
            ((R *)ht->p[6][2])[i] += corr[6 * n + i];
        }
    }
    if (mag && i < (size_t)nz) {
        ht->bx[2][i] += cbx[i];
        ht->by[2][i] += cby[i];
    }
}

// called inside the time step, after the RHS and before the AB3 update
int closure_apply_corr(Engine *E)
{
    if (!E->corr_on || !E->corr) return VEC_OK;
    const size_t cnt = E->n > (size_t)E->nz ? E->n : (size_t)E->nz;
    const int mag = mag_on(*E);
    if (E->split)
        KLAUNCH(E, "closure_add", k_add_corr<float>, nblk(cnt), TPB, E->ht, (const float *)E->corr, E->corr_bx,
                E->corr_by, E->n, E->nz, mag);
    else
        KLAUNCH(E, "closure_add", k_add_corr<double>, nblk(cnt), TPB, E->ht, (const double *)E->corr, E->corr_bx,
                E->corr_by, E->n, E->nz, mag);
    return VEC_OK;
}

template <typename R>
static int corr_from_out(Engine &E, const float *out, const float *nrm, float clip, float gain)
{
    R *corr = (R *)E.corr;
    R *bd = corr + 7 * E.n;
    KLAUNCH((&E), "closure_corr", k_corr_split<R>, nblk(E.n), TPB, out, nrm, E.n, corr, bd, clip, gain);
    if (!mag_on(E)) return VEC_OK;
    R *ex = bd, *ey = bd + E.n, *ez = bd + 2 * E.n;
    int st;
    LineJob<R> fx[3] = { ljob<R>(ex, ex, OP_FWD), ljob<R>(ey, ey, OP_FWD), ljob<R>(ez, ez, OP_FWD) };
    if ((st = launch_lines<R>(&E, 0, fx, 3))) return st;
    if ((st = launch_lines<R>(&E, 1, fx, 3))) return st;
    for (int f = 0; f < 3; f++)
        KLAUNCH((&E), "closure_truncate", k_truncate<R>, plane_grid(E), TPB, bd + (size_t)f * E.n, (R *)nullptr, E.nx,
                E.ny, E.nz, E.k.icutoffx, E.k.icutoffy);
    KLAUNCH((&E), "closure_corr_means", k_corr_means<R>, 1, 256, ex, ey, E.corr_bx, E.corr_by, E.np, E.nz, E.k.xn);
    KLAUNCH((&E), "closure_corr_poltor", k_corr_poltor<R>, nblk(E.n), TPB, ex, ey, ez, corr + 5 * E.n,
            corr + 6 * E.n, E.nx, E.ny, E.nz, E.akx1, E.aky1, E.akx2, E.aky2);
    return VEC_OK;
}

// ---- spectral upsampler (interpolate/fft.F90:834-927, any even factor, plus
// cubic interpolation between the vertex-aligned planes) ----------------------------------
// coarse halfcomplex x halfcomplex spectrum -> fine spectrum at fine plane
// r*kc: mode indices 0..n/2 (with the Nyquist real part) keep their index,
// the imaginary parts i > n/2 move to N - (n - i); scaled by sx*sy
__global__ void k_spec_scatter(const double *cs, double *fs, int nxc, int nyc, int nzc, int nxf, int nyf, int kstep,
                               double scale)
{
    const size_t npc = (size_t)nxc * nyc;
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= npc * nzc) return;
    const int kc = (int)(idx / npc);
    const size_t q = idx - (size_t)kc * npc;
    const int j = (int)(q / nxc), i = (int)(q - (size_t)j * nxc);
    const int I = i <= nxc / 2 ? i : nxf - (nxc - i);
    const int J = j <= nyc / 2 ? j : nyf - (nyc - j);
    fs[((size_t)kc * kstep) * nxf * nyf + (size_t)J * nxf + I] = cs[idx] * scale;
}

// planes between the vertex-aligned ones: cubic Lagrange through the four
// nearest coarse planes (one-sided next to the walls)
__global__ void k_zinterp(double *f, size_t np, int nzf, int r)
{
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= np * nzf) return;
    const int kf = (int)(idx / np);
    if (kf % r == 0) return;
    const size_t q = idx - (size_t)kf * np;
    const int nzc = (nzf - 1) / r + 1;
    const double s = (double)kf / r;
    int m0 = kf / r - 1;
    if (m0 < 0) m0 = 0;
    if (m0 > nzc - 4) m0 = nzc - 4;
    double v = 0.0;
    for (int a = 0; a < 4; a++) {
        double l = 1.0;
        for (int b = 0; b < 4; b++)
            if (b != a) l *= (s - (m0 + b)) / (double)(a - b);
        v += l * f[(size_t)(m0 + a) * r * np + q];
    }
    f[idx] = v;
}

__global__ void k_floor(double *r, size_t n, double lo)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && r[i] < lo) r[i] = lo;
}

// one FP64 field of C upsampled into the FP64 array dst of F (nz_f planes)
static int upsample_field(Engine &Cc, Engine &F, const double *src, double *dst, int r, int zinterp)
{
    double *cs = Cc.W64(0);
    double *fs = F.W64(0);
    int st;
    LineJob<double> fx = ljob<double>(src, cs, OP_FWD);
    if ((st = launch_lines<double>(&Cc, 0, &fx, 1))) return st;
    LineJob<double> fy = ljob<double>(cs, cs, OP_FWD);
    if ((st = launch_lines<double>(&Cc, 1, &fy, 1))) return st;
    // F waits for C's spectrum
    cudaEvent_t ev;
    CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CUDA_TRY(cudaEventRecord(ev, Cc.stream));
    CUDA_TRY(cudaStreamWaitEvent(F.stream, ev, 0));
    CUDA_TRY(cudaEventDestroy(ev));
    CUDA_TRY(cudaMemsetAsync(fs, 0, sizeof(double) * F.n, F.stream));
    const int kstep = zinterp ? r : 1;
    KLAUNCH((&F), "upsample_scatter", k_spec_scatter, nblk(Cc.n), TPB, cs, fs, Cc.nx, Cc.ny, Cc.nz, F.nx, F.ny, kstep,
            (double)(F.nx / Cc.nx) * (double)(F.ny / Cc.ny));
    LineJob<double> iy = ljob<double>(fs, fs, OP_INV);
    if ((st = launch_lines<double>(&F, 1, &iy, 1))) return st;
    LineJob<double> ixj = ljob<double>(fs, dst, OP_INV);
    if ((st = launch_lines<double>(&F, 0, &ixj, 1))) return st;
    if (zinterp) KLAUNCH((&F), "upsample_zinterp", k_zinterp, nblk(F.n), TPB, dst, F.np, F.nz, r);
    // C may reuse its scratch once F has read it
    CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CUDA_TRY(cudaEventRecord(ev, F.stream));
    CUDA_TRY(cudaStreamWaitEvent(Cc.stream, ev, 0));
    CUDA_TRY(cudaEventDestroy(ev));
    return VEC_OK;
}

// ---- C-ABI -------------------------------------------------------------------------------
extern "C" int vec_closure_destroy(vec_closure *cl)
{
    if (!cl) return VEC_OK;
    cudaDeviceSynchronize();
    if (cl->net) vec_net_destroy(cl->net);
    if (cl->cs) vec_destroy(cl->cs);
    void *ps[] = { cl->in_ds, cl->tg_ds, cl->nrm, cl->filt_rhs, cl->crhs, cl->stats, cl->acc, cl->rho0c, cl->t0c,
                   cl->rho0f, cl->t0f };
    for (void *p : ps) if (p) cudaFree(p);
    delete cl;
    return VEC_OK;
}

extern "C" int vec_closure_create(const vec_params *coarse, int factor, int capacity, int batch,
                                  unsigned long long seed, vec_closure **out)
{
    if (!coarse || !out || factor < 2 || factor % 2 || capacity < 0 || batch < 1 || batch > 64) return VEC_ERR_ARG;
    *out = nullptr;
    vec_closure *cl = new vec_closure();
    cl->r = factor;
    cl->nxc = coarse->nx; cl->nyc = coarse->ny; cl->nzc = coarse->nz;
    cl->npc = (size_t)coarse->nx * coarse->ny * coarse->nz;
    cl->batch = batch;
    cl->cap = capacity;
    cl->pc = *coarse;
    int st = vec_net_create(cl->nxc, cl->nyc, cl->nzc, batch, seed, &cl->net);
    if (st) { delete cl; return st; }
    auto al = [&](void **p, size_t bytes) {
        if (st) return;
        if (cudaMalloc(p, bytes ? bytes : 16) != cudaSuccess) {
            cudaGetLastError();
            vec_set_error("closure: cudaMalloc of %zu bytes failed", bytes);
            st = VEC_ERR_ALLOC;
        }
    };
    al((void **)&cl->in_ds, (size_t)capacity * cl->npc * 8 * 4);
    al((void **)&cl->tg_ds, (size_t)capacity * cl->npc * 8 * 4);
    al((void **)&cl->nrm, 32 * 4);
    al((void **)&cl->filt_rhs, cl->npc * 8 * 4);
    al((void **)&cl->crhs, cl->npc * 8 * 4);
    al((void **)&cl->stats, 32 * 8);
    al((void **)&cl->acc, 2 * 8);
    if (!st) st = upload_bg(*coarse, cl->nzc, &cl->rho0c, &cl->t0c);
    if (st) { vec_closure_destroy(cl); return st; }
    for (int c = 0; c < 8; c++) { cl->hnrm[c] = 0.0f; cl->hnrm[8 + c] = 1.0f; cl->hnrm[16 + c] = 0.0f; cl->hnrm[24 + c] = 1.0f; }
    if (cudaMemcpy(cl->nrm, cl->hnrm, sizeof(cl->hnrm), cudaMemcpyHostToDevice) != cudaSuccess) {
        vec_closure_destroy(cl);
        return VEC_ERR_CUDA;
    }
    *out = cl;
    return VEC_OK;
}

extern "C" vec_net *vec_closure_net(vec_closure *cl) { return cl ? cl->net : nullptr; }

extern "C" int vec_closure_set_output(vec_closure *cl, float clip, float gain)
{
    if (!cl || !(clip > 0.0f) || !(gain >= 0.0f)) return VEC_ERR_ARG;
    cl->clip = clip;
    cl->gain = gain;
    return VEC_OK;
}

// Nusselt number at the fixed-temperature top: the reference's formula
// (src/dbydz.F90:4877-4925) with the one-sided derivative mirrored to the
// top plane, (-11 T0 + 18 T1 - 9 T2 + 2 T3) / (6 dz); with a fixed-flux
// bottom the reference's own (bottom) Nusselt number is identically one
extern "C" int vec_top_nusselt(vec_ctx *c, double *nu)
{
    if (!c || !nu) return VEC_ERR_ARG;
    Engine &E = engine_of(c);
    std::vector<double> h(4 * E.np);
    CUDA_TRY(cudaMemcpyAsync(h.data(), E.t, sizeof(double) * 4 * E.np, cudaMemcpyDeviceToHost, E.stream));
    CUDA_TRY(cudaStreamSynchronize(E.stream));
    double s = 0.0;
    for (size_t q = 0; q < E.np; q++)
        s += (-11.0 * h[q] + 18.0 * h[E.np + q] - 9.0 * h[2 * E.np + q] + 2.0 * h[3 * E.np + q]) / (6.0 * E.k.dz);
    s /= (double)E.np;
    *nu = (s - E.k.nusstmp) / (E.k.theta - E.k.nusstmp);
    return VEC_OK;
}
extern "C" int vec_closure_npairs(vec_closure *cl) { return cl ? cl->npairs : 0; }

// synchronise s1 after s0
static int join(cudaStream_t s0, cudaStream_t s1)
{
    cudaEvent_t ev;
    CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CUDA_TRY(cudaEventRecord(ev, s0));
    CUDA_TRY(cudaStreamWaitEvent(s1, ev, 0));
    CUDA_TRY(cudaEventDestroy(ev));
    return VEC_OK;
}

extern "C" int vec_box_filter(vec_closure *cl, vec_ctx *fine, vec_ctx *coarse)
{
    if (!cl || !fine || !coarse) return VEC_ERR_ARG;
    Engine &F = engine_of(fine), &Cc = engine_of(coarse);
    int st;
    if ((st = check_pair(cl, F, Cc))) return st;
    if ((st = filter_state(cl, F, Cc, cl->crhs))) return st;
    if ((st = join(F.stream, Cc.stream))) return st;
    if ((st = set_coarse(cl, Cc, cl->crhs, F.bzbar))) return st;
    if ((st = join(Cc.stream, F.stream))) return st;
    CUDA_TRY(cudaStreamSynchronize(Cc.stream));
    return VEC_OK;
}

// one training pair from the fine context's current state; coarse is a
// scratch context (its state is overwritten)
extern "C" int vec_closure_add_pair(vec_closure *cl, vec_ctx *fine, vec_ctx *coarse)
{
    if (!cl || !fine || !coarse) return VEC_ERR_ARG;
    if (cl->npairs >= cl->cap) { vec_set_error("closure: dataset full (%d pairs)", cl->cap); return VEC_ERR_ARG; }
    Engine &F = engine_of(fine), &Cc = engine_of(coarse);
    int st;
    if ((st = check_pair(cl, F, Cc))) return st;
    float *in = cl->in_ds + (size_t)cl->npairs * cl->npc * 8;
    float *tg = cl->tg_ds + (size_t)cl->npairs * cl->npc * 8;
    // filtered fine state
    if ((st = filter_state(cl, F, Cc, in))) return st;
    // filtered fine RHS (dB/dt into F's FP64-sized scratch s64)
    if ((st = eval_rhs(F))) return st;
    FiltSrc s;
    if ((st = rhs_channels(F, &s))) return st;
    KLAUNCH((&F), "box_filter", k_box_filter, nblk(cl->npc), TPB, s, F.nx, F.ny, F.nz, cl->r, Cc.nx, Cc.ny, Cc.nz,
            cl->filt_rhs);
    if ((st = join(F.stream, Cc.stream))) return st;
    // coarse RHS at the filtered state
    if ((st = set_coarse(cl, Cc, in, F.bzbar))) return st;
    if ((st = eval_rhs(Cc))) return st;
    if ((st = rhs_channels(Cc, &s))) return st;
    KLAUNCH((&Cc), "closure_pack8", k_pack8, nblk(cl->npc), TPB, s, cl->npc, cl->crhs);
    KLAUNCH((&Cc), "closure_target", k_sub8, nblk(cl->npc * 8), TPB, cl->filt_rhs, cl->crhs, tg, cl->npc * 8);
    if ((st = join(Cc.stream, F.stream))) return st;
    CUDA_TRY(cudaStreamSynchronize(Cc.stream));
    cl->npairs += 1;
    return VEC_OK;
}

// host copies of pair i: in, tgt [npc][8] (either may be NULL)
extern "C" int vec_closure_get_pair(vec_closure *cl, int i, float *in, float *tgt)
{
    if (!cl || i < 0 || i >= cl->npairs) return VEC_ERR_ARG;
    const size_t b = cl->npc * 8 * 4;
    if (in) CUDA_TRY(cudaMemcpy(in, cl->in_ds + (size_t)i * cl->npc * 8, b, cudaMemcpyDeviceToHost));
    if (tgt) CUDA_TRY(cudaMemcpy(tgt, cl->tg_ds + (size_t)i * cl->npc * 8, b, cudaMemcpyDeviceToHost));
    return VEC_OK;
}

// per-channel mean and standard deviation of inputs and targets over pairs [0, n)
extern "C" int vec_closure_fit_norm(vec_closure *cl, int n)
{
    if (!cl || n <= 0 || n > cl->npairs) return VEC_ERR_ARG;
    cudaStream_t s = cl->net->stream;
    const size_t cnt = (size_t)n * cl->npc;
    double h[2][16];
    for (int w = 0; w < 2; w++) {
        CUDA_TRY(cudaMemsetAsync(cl->stats, 0, 16 * 8, s));
        k_stats<<<cl->net->num_sms * 4, 256, 0, s>>>(w == 0 ? cl->in_ds : cl->tg_ds, cnt, cl->stats);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaMemcpyAsync(h[w], cl->stats, 16 * 8, cudaMemcpyDeviceToHost, s));
    }
    CUDA_TRY(cudaStreamSynchronize(s));
    for (int w = 0; w < 2; w++)
        for (int c = 0; c < 8; c++) {
            const double m = h[w][c] / (double)cnt;
            double var = h[w][8 + c] / (double)cnt - m * m;
            double sd = var > 0.0 ? sqrt(var) : 0.0;
            if (!(sd > 1e-30)) sd = 1.0;
            cl->hnrm[16 * w + c] = (float)m;
            cl->hnrm[16 * w + 8 + c] = (float)sd;
        }
    CUDA_TRY(cudaMemcpy(cl->nrm, cl->hnrm, sizeof(cl->hnrm), cudaMemcpyHostToDevice));
    return VEC_OK;
}

extern "C" int vec_closure_get_norm(vec_closure *cl, float *out32)
{
    if (!cl || !out32) return VEC_ERR_ARG;
    memcpy(out32, cl->hnrm, sizeof(cl->hnrm));
    return VEC_OK;
}

extern "C" int vec_closure_set_norm(vec_closure *cl, const float *in32)
{
    if (!cl || !in32) return VEC_ERR_ARG;
    memcpy(cl->hnrm, in32, sizeof(cl->hnrm));
    CUDA_TRY(cudaMemcpy(cl->nrm, cl->hnrm, sizeof(cl->hnrm), cudaMemcpyHostToDevice));
    return VEC_OK;
}

static uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// iters Adam steps on batches drawn (seeded) from pairs [0, ntrain);
// losses (may be NULL) receives each iteration's loss
extern "C" int vec_closure_train(vec_closure *cl, int iters, float lr, int ntrain, unsigned long long seed,
                                 double *losses)
{
    if (!cl || iters < 0 || ntrain <= 0 || ntrain > cl->npairs) return VEC_ERR_ARG;
    vec_net *N = cl->net;
    const int B = cl->batch;
    int st;
    std::vector<double> lh(iters > 0 ? iters : 1, 0.0);
    for (int it = 0; it < iters; it++) {
        BatchIdx bi;
        for (int b = 0; b < B; b++) bi.i[b] = (int)(mix64(seed * 0x9e3779b97f4a7c15ULL + (uint64_t)it * 64 + b + 1) % (uint64_t)ntrain);
        k_gather<<<nblk((size_t)B * cl->npc), TPB, 0, N->stream>>>(cl->in_ds, cl->tg_ds, bi, B, cl->npc,
                                                                   (size_t)cl->nxc * cl->nyc, cl->nzc, cl->nrm, N->x0,
                                                                   N->tgt);
        CUDA_TRY(cudaGetLastError());
        if ((st = net_forward(N)) || (st = net_backward(N, N->tgt)) || (st = net_adam(N, lr))) return st;
        if (losses) CUDA_TRY(cudaMemcpyAsync(&lh[it], N->loss_d, 8, cudaMemcpyDeviceToHost, N->stream));
    }
    CUDA_TRY(cudaStreamSynchronize(N->stream));
    if (losses) memcpy(losses, lh.data(), sizeof(double) * iters);
    return VEC_OK;
}

// a-priori error on pairs [first, first + count): mse_net = mean (net -
// target)^2, mse_zero = mean target^2 (no closure), normalised units
extern "C" int vec_closure_eval(vec_closure *cl, int first, int count, double *mse_net, double *mse_zero)
{
    if (!cl || first < 0 || count <= 0 || first + count > cl->npairs) return VEC_ERR_ARG;
    vec_net *N = cl->net;
    const int B = cl->batch;
    int st;
    CUDA_TRY(cudaMemsetAsync(cl->acc, 0, 16, N->stream));
    const NetGeom g0 = N->g;
    for (int i0 = first; i0 < first + count; i0 += B) {
        const int nb = (first + count - i0) < B ? (first + count - i0) : B;
        BatchIdx bi;
        for (int b = 0; b < nb; b++) bi.i[b] = i0 + b;
        k_gather<<<nblk((size_t)nb * cl->npc), TPB, 0, N->stream>>>(cl->in_ds, cl->tg_ds, bi, nb, cl->npc,
                                                                    (size_t)cl->nxc * cl->nyc, cl->nzc, cl->nrm,
                                                                    N->x0, N->tgt);
        CUDA_TRY(cudaGetLastError());
        N->g.nb = nb;
        N->g.tiles = (long long)nb * g0.nz * (g0.nx * g0.ny / 128);
        st = net_forward(N);
        N->g = g0;
        if (st) return st;
        k_eval_acc<<<N->num_sms * 2, 256, 0, N->stream>>>(N->out, N->tgt, (size_t)nb * cl->npc * 8, cl->acc);
        CUDA_TRY(cudaGetLastError());
    }
    double h[2];
    CUDA_TRY(cudaMemcpyAsync(h, cl->acc, 16, cudaMemcpyDeviceToHost, N->stream));
    CUDA_TRY(cudaStreamSynchronize(N->stream));
    const double cnt = (double)count * cl->npc * 8;
    if (mse_net) *mse_net = h[0] / cnt;
    if (mse_zero) *mse_zero = h[1] / cnt;
    return VEC_OK;
}

// enable (on = 1) or disable the RHS correction of a coarse context
extern "C" int vec_closure_attach(vec_closure *cl, vec_ctx *coarse, int on)
{
    if (!cl || !coarse) return VEC_ERR_ARG;
    Engine &E = engine_of(coarse);
    if (E.nx != cl->nxc || E.ny != cl->nyc || E.nz != cl->nzc) return VEC_ERR_ARG;
    if (on && !E.corr) {
        const size_t esz = E.split ? 4 : 8;
        if (cudaMalloc(&E.corr, esz * E.n * 10) != cudaSuccess ||
            cudaMalloc((void **)&E.corr_bx, sizeof(double) * E.nz * 2) != cudaSuccess) {
            cudaGetLastError();
            return VEC_ERR_ALLOC;
        }
        E.corr_by = E.corr_bx + E.nz;
        CUDA_TRY(cudaMemsetAsync(E.corr, 0, esz * E.n * 10, E.stream));
        CUDA_TRY(cudaMemsetAsync(E.corr_bx, 0, sizeof(double) * E.nz * 2, E.stream));
    }
    E.corr_on = on ? 1 : 0;
    E.drop_graphs();
    return VEC_OK;
}

// the network's correction for the coarse context's current state
extern "C" int vec_closure_infer(vec_closure *cl, vec_ctx *coarse)
{
    if (!cl || !coarse) return VEC_ERR_ARG;
    Engine &E = engine_of(coarse);
    if (!E.corr) return VEC_ERR_ARG;
    vec_net *N = cl->net;
    int st;
    if ((st = join(E.stream, N->stream))) return st;
    const void *bx = E.split ? (const void *)E.bx32 : (const void *)E.bx;
    const void *by = E.split ? (const void *)E.by32 : (const void *)E.by;
    const void *bz = E.split ? (const void *)E.bz32 : (const void *)E.bz;
    const double bzoff = E.split ? 0.0 : E.bzbar;
    if (E.split && !E.b32_auth) {   // FP32 B older than the FP64 one
        bx = E.bx; by = E.by; bz = E.bz;
    }
    const int bdbl = (bx == (const void *)E.bx) ? 1 : 0;
    k_pack_state<<<nblk(E.n), TPB, 0, N->stream>>>(E.u, E.v, E.w, E.r, E.t, bx, by, bz, bdbl,
                                                   bdbl ? E.bzbar : bzoff, cl->rho0c, cl->t0c, cl->nrm, E.np, E.nz,
                                                   N->x0);
    CUDA_TRY(cudaGetLastError());
    const NetGeom g0 = N->g;
    N->g.nb = 1;
    N->g.tiles = (long long)g0.nz * (g0.nx * g0.ny / 128);
    st = net_forward(N);
    N->g = g0;
    if (st) return st;
    if ((st = join(N->stream, E.stream))) return st;
    st = E.split ? corr_from_out<float>(E, N->out, cl->nrm, cl->clip, cl->gain)
                 : corr_from_out<double>(E, N->out, cl->nrm, cl->clip, cl->gain);
    if (st) return st;
    return join(E.stream, N->stream);
}

// nsteps time steps of the coarse context with the correction recomputed
// before each step
extern "C" int vec_closure_step(vec_closure *cl, vec_ctx *coarse, int nsteps)
{
    if (!cl || !coarse || nsteps < 0) return VEC_ERR_ARG;
    for (int s = 0; s < nsteps; s++) {
        int st = vec_closure_infer(cl, coarse);
        if (st) return st;
        if ((st = vec_step(coarse, 1))) return st;
    }
    return VEC_OK;
}

// the reference's expand (interpolate/fft.F90:834-927): in (nx, ny, nz) ->
// out (r nx, r ny, nz) on host or device arrays, through the fine context
extern "C" int vec_expand(vec_ctx *coarse, vec_ctx *fine_same_nz, const double *in, double *out)
{
    if (!coarse || !fine_same_nz || !in || !out) return VEC_ERR_ARG;
    Engine &Cc = engine_of(coarse), &F = engine_of(fine_same_nz);
    if (F.nz != Cc.nz || F.nx % Cc.nx || F.ny % Cc.ny || F.nx / Cc.nx != F.ny / Cc.ny) return VEC_ERR_ARG;
    int st;
    double *din = Cc.s64[1], *dout = F.s64[1];
    CUDA_TRY(cudaMemcpyAsync(din, in, sizeof(double) * Cc.n, cudaMemcpyDefault, Cc.stream));
    if ((st = upsample_field(Cc, F, din, dout, F.nx / Cc.nx, 0))) return st;
    CUDA_TRY(cudaMemcpyAsync(out, dout, sizeof(double) * F.n, cudaMemcpyDefault, F.stream));
    CUDA_TRY(cudaStreamSynchronize(F.stream));
    CUDA_TRY(cudaStreamSynchronize(Cc.stream));
    return VEC_OK;
}

// fine context state from the coarse one: spectral upsampling of u, v, w,
// rho, T, Bx, By, Bz, cubic interpolation between the vertex-aligned
// planes, then pol/tor (mag_init), B and the boundary conditions; the fine
// run restarts its AB3 history (Euler first step) at the coarse time
extern "C" int vec_upsample(vec_ctx *coarse, vec_ctx *fine)
{
    if (!coarse || !fine) return VEC_ERR_ARG;
    Engine &Cc = engine_of(coarse), &F = engine_of(fine);
    const int r = F.nx / (Cc.nx ? Cc.nx : 1);
    if (r < 1 || F.nx != r * Cc.nx || F.ny != r * Cc.ny || F.nz - 1 != r * (Cc.nz - 1)) return VEC_ERR_ARG;
    int st;
    if (Cc.split && (st = split_sync_b64(&Cc))) return st;
    const double *src[8] = { Cc.u, Cc.v, Cc.w, Cc.r, Cc.t, Cc.bx, Cc.by, Cc.bz };
    double *dst[8] = { F.u, F.v, F.w, F.r, F.t, F.bx, F.by, F.bz };
    for (int f = 0; f < 8; f++)
        if ((st = upsample_field(Cc, F, src[f], dst[f], r, 1))) return st;
    // the density floor of the AB3 update (src/main.F90:438-442) on the
    // interpolated density, whose spectral interpolation can undershoot
    KLAUNCH((&F), "upsample_floor", k_floor, nblk(F.n), TPB, F.r, F.n, 0.05);
    F.bzbar = Cc.bzbar;
    F.b32_auth = 0;
    if (mag_on(F) && (st = phys_mag_init(&F))) return st;
    if (F.split && (st = split_refresh(&F))) return st;
    if (mag_on(F) && (st = F.split ? split_bandj(&F) : phys_bandj64(&F))) return st;
    if ((st = phys_boundary(&F))) return st;
    if (F.split && (st = split_refresh_planes(&F, 1 | 2))) return st;
    vec_scalars sc, sf;
    if ((st = vec_get_scalars(coarse, &sc)) || (st = vec_get_scalars(fine, &sf))) return st;
    sf.ttime = sc.ttime;
    sf.first = 1;
    sf.second = 0;
    if ((st = vec_set_scalars(fine, &sf))) return st;
    F.drop_graphs();
    double dt;
    return vec_calcdt(fine, &dt);
}

// The judged closure run: coarse steps with the correction until the time
// t_end; every `every` steps the current coarse state is upsampled into
// `fine` and the plain fine solver runs `nfine` steps; when the coarse run
// reaches that segment's end time its diagnostics are compared with the
// box-filtered fine ones, and if the Nusselt number (at the bottom, as the
// reference, and at the top), kinetic or magnetic energy differs by more than tol
// (relative), the coarse state fails the div B check, or the coarse run
// stops advancing, the run continues on the fine solver to t_end.  The fine
// context always holds the state the fall-back continues from: the
// upsampled start of the run, then the end of the last judged segment.
// With diag_every > 0, rows (time, Nu, kinetic energy, magnetic energy,
// top Nu) of the running solver (the fine one through the box filter) are
// appended to series every diag_every steps (at most cap rows).
extern "C" int vec_closure_run(vec_closure *cl, vec_ctx *coarse, vec_ctx *fine, double t_end, int every, int nfine,
                               double tol, int diag_every, double *series, int cap, vec_closure_report *rep)
{
    if (!cl || !coarse || !fine || every <= 0 || nfine <= 0 || !rep) return VEC_ERR_ARG;
    memset(rep, 0, sizeof(*rep));
    rep->fallback_step = -1;
    int st;
    // diagnostics of c (+ the top Nusselt number); the div B check of
    // src/main.F90:583-590 failing is reported through *divb, not as an
    // error.  The fine context is measured through the box filter (its state
    // filtered into a scratch coarse context), so that fine and coarse
    // diagnostics compare like with like.
    if (!cl->cs && (st = vec_create(&cl->pc, &cl->cs))) return st;
    auto diag = [&](vec_ctx *c, vec_diag_out *d, double *nutop, int *divb) -> int {
        int e;
        if (c == fine) {
            if ((e = vec_box_filter(cl, fine, cl->cs))) return e;
            c = cl->cs;
        }
        e = vec_diag(c, d);
        if (e == VEC_ERR_DIVB) { *divb = 1; e = VEC_OK; }
        if (e) return e;
        return vec_top_nusselt(c, nutop);
    };
    auto record = [&](vec_ctx *c, int *divb) -> int {
        if (diag_every <= 0 || !series || rep->nseries >= cap) return VEC_OK;
        vec_diag_out d;
        vec_scalars s;
        double nt = 0.0;
        int e = diag(c, &d, &nt, divb);
        if (e) return e;
        if ((e = vec_get_scalars(c, &s))) return e;
        double *row = series + 5 * (size_t)rep->nseries;
        row[0] = s.ttime; row[1] = d.nusselt; row[2] = d.kenergy; row[3] = d.menergy; row[4] = nt;
        rep->nseries += 1;
        return VEC_OK;
    };
    // a run makes progress while its time advances by finite steps not
    // below 1e-3 of its first, within 100 times the step count that first
    // step implies
    struct Progress {
        double t_prev, dt0, t0;
        long long n;
        bool ok(const vec_scalars &s, double t_end)
        {
            if (!(isfinite(s.ttime) && isfinite(s.dt) && s.dt > 0.0)) return false;
            if (n == 0) { dt0 = s.dt; t0 = s.ttime; t_prev = s.ttime; n = 1; return true; }
            const bool adv = s.ttime > t_prev && s.dt > 1e-3 * dt0;
            const bool cap = (double)n < 100.0 * (t_end - t0) / dt0 + 1000.0;
            t_prev = s.ttime;
            n += 1;
            return adv && cap;
        }
    };
    // the fine solver continues to t_end from the last state it holds
    auto fall_back = [&](long long at) -> int {
        rep->fallback_step = at;
        int e;
        if ((e = vec_closure_attach(cl, coarse, 0))) return e;
        vec_scalars sf;
        long long fs = 0;
        int ignore = 0;
        Progress pf = { 0.0, 0.0, 0.0, 0 };
        for (;;) {
            if ((e = vec_get_scalars(fine, &sf))) return e;
            if (sf.ttime >= t_end) break;
            if (!pf.ok(sf, t_end)) {
                vec_set_error("closure run: the fine solver stopped advancing (t = %g, dt = %g)", sf.ttime, sf.dt);
                return VEC_ERR_NAN;
            }
            if ((e = vec_step(fine, 1))) return e;
            rep->fine_steps += 1;
            fs += 1;
            if (diag_every > 0 && fs % diag_every == 0 && (e = record(fine, &ignore))) return e;
        }
        rep->end_time = sf.ttime;
        return VEC_OK;
    };
    if ((st = vec_closure_attach(cl, coarse, 1))) return st;
    if ((st = vec_upsample(coarse, fine))) return st;   // the fall-back start until the first judge
    vec_scalars sc;
    vec_diag_out dfine, dc, dfine0, dc0;
    double nutf = 0.0, nutc = 0.0, nutf0 = 0.0, nutc0 = 0.0;
    int pending = 0;
    double t_check = 0.0;
    long long step = 0;
    Progress pc = { 0.0, 0.0, 0.0, 0 };
    for (;;) {
        if ((st = vec_get_scalars(coarse, &sc))) return st;
        if (sc.ttime >= t_end) break;
        if (!pc.ok(sc, t_end)) {
            rep->blowup = 1;
            return fall_back(step);
        }
        if (pending && sc.ttime >= t_check) {
            int divb = 0;
            st = diag(coarse, &dc, &nutc, &divb);
            if (st == VEC_ERR_NAN) {   // the coarse state is no longer finite
                rep->blowup = 1;
                return fall_back(step);
            }
            if (st) return st;
            // drift over the segment: the change of each statistic in the
            // coarse run against its change in the fine run, relative to the
            // fine value.  (The filtered upsampled state differs from the
            // coarse one at the start -- the box filter damps resolved
            // modes -- and that offset is not drift.)
            auto drift = [](double c, double c0, double f, double f0) {
                return fabs((c - c0) - (f - f0)) / fmax(fabs(f), 1e-300);
            };
            const double e0 = fmax(drift(dc.nusselt, dc0.nusselt, dfine.nusselt, dfine0.nusselt),
                                   drift(nutc, nutc0, nutf, nutf0));
            const double e1 = drift(dc.kenergy, dc0.kenergy, dfine.kenergy, dfine0.kenergy);
            const double e2 = mag_on(engine_of(coarse)) ? drift(dc.menergy, dc0.menergy, dfine.menergy, dfine0.menergy)
                                                        : 0.0;
            rep->judges += 1;
            rep->last_err[0] = e0; rep->last_err[1] = e1; rep->last_err[2] = e2;
            rep->max_err[0] = fmax(rep->max_err[0], e0);
            rep->max_err[1] = fmax(rep->max_err[1], e1);
            rep->max_err[2] = fmax(rep->max_err[2], e2);
            pending = 0;
            if (divb) rep->divb_fail = 1;
            if (divb || e0 > tol || e1 > tol || e2 > tol) return fall_back(step);
        }
        if (!pending && step > 0 && step % every == 0) {
            if ((st = vec_upsample(coarse, fine))) return st;
            int ignore = 0;
            // both runs' statistics at the segment start
            if ((st = diag(fine, &dfine0, &nutf0, &ignore))) return st;
            st = diag(coarse, &dc0, &nutc0, &ignore);
            if (st == VEC_ERR_NAN) {
                rep->blowup = 1;
                return fall_back(step);
            }
            if (st) return st;
            if ((st = vec_step(fine, nfine))) return st;
            rep->fine_steps += nfine;
            vec_scalars sf;
            if ((st = vec_get_scalars(fine, &sf)) || (st = diag(fine, &dfine, &nutf, &ignore))) return st;
            t_check = sf.ttime;
            pending = 1;
        }
        st = vec_closure_step(cl, coarse, 1);
        if (st == VEC_ERR_NAN) {   // the time loop's non-finite check
            rep->blowup = 1;
            return fall_back(step + 1);
        }
        if (st) return st;
        step += 1;
        rep->coarse_steps += 1;
        int divb = 0;
        st = diag_every > 0 && step % diag_every == 0 ? record(coarse, &divb) : VEC_OK;
        if (st == VEC_ERR_NAN) {
            rep->blowup = 1;
            return fall_back(step);
        }
        if (st) return st;
        if (divb) {
            rep->divb_fail = 1;
            return fall_back(step);
        }
    }
    rep->end_time = sc.ttime;
    return vec_closure_attach(cl, coarse, 0);
}
