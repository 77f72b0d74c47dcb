// magkern.cuh -- induction and B/J kernels shared by the FP64 and the split
// forms (R = double or float).  src/magnetic.f90:285-717.
#pragma once
#include "zstencil.cuh"

// E = u x B (:308-316); bzoff is added to bz (the split form stores bz
// minus its constant mean bzbar)
template <typename R>
static __global__ void k_emf(const R *u, const R *v, const R *w, const R *bx, const R *by, const R *bz, R *e1,
                             R *e2, R *e3, size_t n, R bzoff)
{
    PDL_WAIT();
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const R bzv = bz[i] + bzoff;
    e1[i] = v[i] * bzv - w[i] * by[i];
    e2[i] = w[i] * bx[i] - u[i] * bzv;
    e3[i] = u[i] * by[i] - v[i] * bx[i];
}

// mean-field RHS (:328-352) on one CTA; ex, ey are the 2-D spectra of the EMF
template <typename R>
struct MeanArgs {
    const R *ex, *ey;
    const double *bxbar, *bybar, *eta, *deta;
    const HistTable *ht;
    double *scratch;
    size_t np;
    int nz;
    double xn, zck, ho12, sc1;
    int var_eta;
    // k_mag_div4 only: with ds set, the mean-field CTA goes on with the AB3
    // coefficient step and the mean update of ab3_coef_block on bxm, bym
    // (the bxbar, bybar above), which read the history it has just written
    DevScalars *ds;
    double *bxm, *bym;
};

template <typename R>
__device__ __forceinline__ void mean_rhs_block(const MeanArgs<R> &a)
{
    const int nz = a.nz;
    double *bxd = a.ht->bx[2], *byd = a.ht->by[2];
    double *e1 = a.scratch, *e2 = a.scratch + nz;
    for (int k = threadIdx.x; k < nz; k += blockDim.x) {
        e1[k] = a.xn * (double)a.ex[(size_t)k * a.np];
        e2[k] = a.xn * (double)a.ey[(size_t)k * a.np];
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nz; k += blockDim.x) {
        double dey = zd1(e2, 1, k, nz, 5, a.ho12);   // :337
        double dex = zd1(e1, 1, k, nz, 5, a.ho12);   // :338
        double d2x = zd2(a.bxbar, 1, k, nz, 3, a.sc1); // :343
        double d2y = zd2(a.bybar, 1, k, nz, 3, a.sc1); // :344
        if (!a.var_eta) {
            bxd[k] = a.zck * d2x - dey;              // :350
            byd[k] = a.zck * d2y + dex;              // :351
        } else {
            // extension: eta(z) d2b/dz2 + eta'(z) db/dz
            double gx = zd1(a.bxbar, 1, k, nz, 5, a.ho12), gy = zd1(a.bybar, 1, k, nz, 5, a.ho12);
            bxd[k] = a.eta[k] * d2x - dey + a.deta[k] * gx;
            byd[k] = a.eta[k] * d2y + dex + a.deta[k] * gy;
        }
    }
}

template <typename R>
static __global__ void k_mean_rhs(MeanArgs<R> a)
{
    PDL_WAIT();
    mean_rhs_block(a);
}

// The spectral kernels below run one CTA row per plane (grid (np/256, nz)):
// k = blockIdx.y, the in-plane index in 32 bits, and the wavenumber tables
// in the kernel's precision (HTab), so that no FP64 arithmetic or 64-bit
// division is spent per point.

// wk1 = dEx/dx + dEy/dy in spectral space (:362-407)
template <typename R>
static __global__ void k_mag_div(const R *ex, const R *ey, R *w1, int nx, int ny, HTab<R> h)
{
    PDL_WAIT();
    const unsigned np = (unsigned)nx * ny;
    const unsigned q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const size_t pb = (size_t)blockIdx.y * np;
    const int j = (int)(q / (unsigned)nx), i = (int)(q - (unsigned)j * nx);
    w1[pb + q] = sdx(ex + pb, i, j, nx, h.kx1) + sdy(ey + pb, i, j, nx, ny, h.ky1);
}

// the AB3 coefficients (src/main.F90:381-403), dt1/dt2 (:488-489), ttime
// (:345) and the 1-D mean update (:469-476), by one whole CTA
__device__ __forceinline__ void ab3_coef_block(DevScalars *ds, double *bxbar, double *bybar, const HistTable *ht,
                                               int nz, int do_means)
{
    const double *bxd0 = ht->bx[0], *bxd1 = ht->bx[1], *bxd2 = ht->bx[2];
    const double *byd0 = ht->by[0], *byd1 = ht->by[1], *byd2 = ht->by[2];
    __shared__ double cc[3];
    if (threadIdx.x == 0) {
        ab3_coefs(ds, cc);
        ab3_advance(ds, cc);
    }
    __syncthreads();
    if (!do_means) return;
    for (int k = threadIdx.x; k < nz; k += blockDim.x) {
        bxbar[k] = bxbar[k] + cc[0] * bxd2[k] + cc[1] * bxd1[k] + cc[2] * bxd0[k];
        bybar[k] = bybar[k] + cc[0] * byd2[k] + cc[1] * byd1[k] + cc[2] * byd0[k];
    }
}

template <typename R>
struct MagArgs {
    const R *ex, *ey, *ez, *w1, *pol, *tor;
    const R *eta, *deta;    // eta(z), eta'(z) in the kernel's precision
    HTab<R> h;
    const HistTable *ht;    // poldot / tordot = newest slots
    R zck, ho12, sc1;
    int var_eta, nx, ny, nz;
};

// :400-479 -- wk2 = dEx/dy - dEy/dx, wk3 = d/dz(wk1), inverse horizontal
// Laplacian, d2/dz2 of pol and tor, and the final poldot / tordot.  One
// thread per point (grid (np/256, nz)); the neighbouring planes of the z
// stencils come from L1/L2.
template <typename R>
static __global__ void k_mag_final(MagArgs<R> a)
{
    PDL_WAIT();
    const unsigned np = (unsigned)a.nx * a.ny;
    const unsigned q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const int k = blockIdx.y;
    const size_t pb = (size_t)k * np, idx = pb + q;
    const int j = (int)(q / (unsigned)a.nx), i = (int)(q - (unsigned)j * a.nx);
    R w2 = sdy(a.ex + pb, i, j, a.nx, a.ny, a.h.ky1) - sdx(a.ey + pb, i, j, a.nx, a.h.kx1);
    R w3 = zd1(a.w1 + q, (size_t)np, k, a.nz, 5, a.ho12);
    const R kk = a.h.kh2[q];
    if (q == 0) { w2 = (R)0; w3 = (R)0; }
    else { w2 = w2 / kk; w3 = w3 / kk; }
    const R d2p = zd2(a.pol + q, (size_t)np, k, a.nz, 3, a.sc1);
    const R d2t = zd2(a.tor + q, (size_t)np, k, a.nz, 3, a.sc1);
    R *poldot = (R *)a.ht->p[5][2], *tordot = (R *)a.ht->p[6][2];
    if (!a.var_eta) {
        const R zck = a.zck;
        poldot[idx] = zck * a.pol[idx] * kk + zck * d2p + w2;
        tordot[idx] = zck * a.tor[idx] * kk + zck * d2t - w3 + a.ez[idx];
    } else {
        // extension: eta(z) replaces zeta*ck, tordot gains eta'(z) d(tor)/dz
        const R e = a.eta[k];
        const R dt = zd1(a.tor + q, (size_t)np, k, a.nz, 5, a.ho12);
        poldot[idx] = e * a.pol[idx] * kk + e * d2p + w2;
        tordot[idx] = e * a.tor[idx] * kk + e * d2t - w3 + a.ez[idx] + a.deta[k] * dt;
    }
}

template <typename R>
struct BandjArgs {
    const R *dzs, *pol, *tor;
    HTab<R> h;
    R *bxh, *byh, *bzh, *dybz, *dxbz, *jzh;
    int nx, ny, nz;
};

// bandj in spectral space, src/magnetic.f90:525-570 and :584-617
template <typename R>
static __global__ void k_bandj_spec(BandjArgs<R> a)
{
    PDL_WAIT();
    const unsigned np = (unsigned)a.nx * a.ny;
    const unsigned q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const size_t pb = (size_t)blockIdx.y * np, idx = pb + q;
    const int j = (int)(q / (unsigned)a.nx), i = (int)(q - (unsigned)j * a.nx);
    const R *s = a.dzs + pb, *tp = a.tor + pb, *pp = a.pol + pb;
    a.bxh[idx] = sdx(s, i, j, a.nx, a.h.kx1) + sdy(tp, i, j, a.nx, a.ny, a.h.ky1);
    a.byh[idx] = sdy(s, i, j, a.nx, a.ny, a.h.ky1) - sdx(tp, i, j, a.nx, a.h.kx1);
    const R kk = a.h.kh2[q];
    a.bzh[idx] = (R)-1 * pp[q] * kk;
    a.jzh[idx] = (R)-1 * tp[q] * kk;
    // (dybz null: the line transforms take the derivatives of bz instead)
    if (!a.dybz) return;
    // d/dy and d/dx of ez = -pol*(akx2+aky2), evaluated at the mirrored index
    R dy = (R)0, dx = (R)0;
    if (!(j == 0 || 2 * j == a.ny)) {
        const unsigned m = (unsigned)(a.ny - j) * a.nx + i;
        R ezm = (R)-1 * pp[m] * a.h.kh2[m];
        dy = ezm * a.h.ky1[j];
        if (2 * j < a.ny) dy = -dy;
    }
    if (!(i == 0 || 2 * i == a.nx)) {
        const unsigned m = (unsigned)j * a.nx + (a.nx - i);
        R ezm = (R)-1 * pp[m] * a.h.kh2[m];
        dx = ezm * a.h.kx1[i];
        if (2 * i < a.nx) dx = -dx;
    }
    a.dybz[idx] = dy;
    a.dxbz[idx] = dx;
}

// :630-645: jsq from Jz, dBz/dy, dBz/dx and the z derivatives of Bx, By
// (grid (np/256, nz))
template <typename R>
static __global__ void k_jsq(const R *jz, const R *dybz, const R *dxbz, const R *bx, const R *by, R *jsq,
                             size_t np, int nz, R h)
{
    PDL_WAIT();
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const int k = blockIdx.y;
    const size_t idx = (size_t)k * np + q;
    R wk1 = zd1(by + q, np, k, nz, 5, h);
    R wk2 = zd1(bx + q, np, k, nz, 5, h);
    R ez = jz[idx], ex = dybz[idx], ey = dxbz[idx];
    jsq[idx] = ez * ez + ((ex - wk1) * (ex - wk1)) + ((wk2 - ey) * (wk2 - ey));
}

// planes per z-marching chunk and its grid
#define ZCHUNK 16
inline dim3 zmarch_grid(size_t np, int nz, int kc = ZCHUNK)
{
    return dim3((unsigned)((np + 255) / 256), (unsigned)((nz + kc - 1) / kc));
}

// ---- four consecutive x points per thread (FP32, nx % 4 == 0) -----------------
// Same arithmetic per component as the one-point kernels above, with 16-byte
// loads and stores; grid (np/4/256, nz).

__device__ __forceinline__ V4 ld4(const float *p, size_t i) { return reinterpret_cast<const V4 *>(p)[i]; }
__device__ __forceinline__ void st4(float *p, size_t i, V4 v) { reinterpret_cast<V4 *>(p)[i] = v; }

// sdx for points i0..i0+3 of row j: plane[j nx + (nx - i)] * akx1[i], negated
// for 2i < nx, zero at i = 0 and 2i = nx.  The mirrored points nx-i0-3 ..
// nx-i0 straddle two aligned 4-vectors.
__device__ __forceinline__ V4 sdx4(const float *plane, int i0, int j, int nx, const float *kx1)
{
    const float *row = plane + (size_t)j * nx;
    const V4 A = *reinterpret_cast<const V4 *>(row + nx - i0 - 4);
    const float b = i0 == 0 ? 0.0f : row[nx - i0];
    const V4 k = *reinterpret_cast<const V4 *>(kx1 + i0);
    const float m[4] = { b, A.w, A.z, A.y }, kk[4] = { k.x, k.y, k.z, k.w };
    float r[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const int i = i0 + c;
        float v = m[c] * kk[c];
        v = 2 * i < nx ? -v : v;
        r[c] = (i == 0 || 2 * i == nx) ? 0.0f : v;
    }
    return V4(r[0], r[1], r[2], r[3]);
}
// sdy for points i0..i0+3 of row j: plane[(ny - j) nx + i] * aky1[j]
__device__ __forceinline__ V4 sdy4(const float *plane, int i0, int j, int nx, int ny, const float *ky1)
{
    if (j == 0 || 2 * j == ny) return V4(0.0f);
    const V4 v = *reinterpret_cast<const V4 *>(plane + (size_t)(ny - j) * nx + i0) * V4(ky1[j]);
    return 2 * j < ny ? -v : v;
}

struct Emf4Args {
    const float *u, *v, *w, *bx, *by, *bz;
    float *e1, *e2, *e3;
    size_t n4;
    float bzoff;
};
template <int NB>
static __global__ void k_emf4(const __grid_constant__ Batch<Emf4Args, NB> bt)
{
    PDL_WAIT();
    const Emf4Args &A = BATCH_MEMBER(bt, NB);
    const float *u = A.u, *v = A.v, *w = A.w, *bx = A.bx, *by = A.by, *bz = A.bz;
    float *e1 = A.e1, *e2 = A.e2, *e3 = A.e3;
    const size_t n4 = A.n4;
    const float bzoff = A.bzoff;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n4) return;
    const V4 U = ld4(u, i), Vv = ld4(v, i), W = ld4(w, i), BX = ld4(bx, i), BY = ld4(by, i);
    const V4 BZ = ld4(bz, i) + V4(bzoff);
    st4(e1, i, Vv * BZ - W * BY);
    st4(e2, i, W * BX - U * BZ);
    st4(e3, i, U * BY - Vv * BX);
}

// (grid (np/4/256, nz + 1): the first CTA of the extra first row computes
// the mean-field RHS, which reads the same spectra -- one launch instead of
// two; the row is dispatched first, so that the CTA's serial FP64 work is
// not the grid's tail.  No plane of this kernel, and none of k_mag_final4
// that follows it, reads ds, bxbar, bybar or the bx/by histories.)
struct MagDiv4Args {
    const float *ex, *ey;
    float *w1;
    int nx, ny;
    HTab<float> h;
    MeanArgs<float> ma;
};
template <int NB>
static __global__ void k_mag_div4(const __grid_constant__ Batch<MagDiv4Args, NB> bt)
{
    PDL_WAIT();
    const MagDiv4Args &A = BATCH_MEMBER(bt, NB);
    const float *ex = A.ex, *ey = A.ey;
    float *w1 = A.w1;
    const int nx = A.nx, ny = A.ny;
    const HTab<float> &h = A.h;
    const MeanArgs<float> &ma = A.ma;
    if (blockIdx.y == 0) {
        if (blockIdx.x == 0) {
            mean_rhs_block(ma);
            if (ma.ds) {
                __syncthreads();   // the new history is written, bxbar and bybar are read
                ab3_coef_block(ma.ds, ma.bxm, ma.bym, ma.ht, ma.nz, 1);
            }
        }
        return;
    }
    const unsigned np4 = (unsigned)nx * ny / 4;
    const unsigned q4 = blockIdx.x * blockDim.x + threadIdx.x;
    if (q4 >= np4) return;
    const size_t pb = (size_t)(blockIdx.y - 1) * np4 * 4;
    const unsigned q = 4 * q4;
    const int j = (int)(q / (unsigned)nx), i0 = (int)(q - (unsigned)j * nx);
    st4(w1 + pb, q4, sdx4(ex + pb, i0, j, nx, h.kx1) + sdy4(ey + pb, i0, j, nx, ny, h.ky1));
}

// (four CTAs per SM: 3.4 TB/s against 2.1 at the compiler's own 90 registers
// and 3.0 at three CTAs per SM with 80 registers and no spills)
template <int NB>
static __global__ void __launch_bounds__(256, 4) k_mag_final4(const __grid_constant__ Batch<MagArgs<float>, NB> bt)
{
    PDL_WAIT();
    const MagArgs<float> &a = BATCH_MEMBER(bt, NB);
    const unsigned np = (unsigned)a.nx * a.ny, np4 = np / 4;
    const unsigned q4 = blockIdx.x * blockDim.x + threadIdx.x;
    if (q4 >= np4) return;
    const int k = blockIdx.y;
    const size_t pb = (size_t)k * np, i4 = (size_t)k * np4 + q4;
    const unsigned q = 4 * q4;
    const int j = (int)(q / (unsigned)a.nx), i0 = (int)(q - (unsigned)j * a.nx);
    const V4 w2a = sdy4(a.ex + pb, i0, j, a.nx, a.ny, a.h.ky1) - sdx4(a.ey + pb, i0, j, a.nx, a.h.kx1);
    const V4 *w1c = reinterpret_cast<const V4 *>(a.w1) + q4;
    const V4 *polc = reinterpret_cast<const V4 *>(a.pol) + q4, *torc = reinterpret_cast<const V4 *>(a.tor) + q4;
    const V4 w3a = zd1(w1c, (size_t)np4, k, a.nz, 5, V4(a.ho12));
    const V4 kk = ld4(a.h.kh2, q4);
    // the inverse horizontal Laplacian as a product with the reciprocal
    // table (rounded once from FP64; zero for the mean) instead of eight
    // divisions per four points
    const V4 ki = ld4(a.h.kh2inv, q4);
    const V4 w2 = w2a * ki, w3 = w3a * ki;
    const V4 d2p = zd2(polc, (size_t)np4, k, a.nz, 3, V4(a.sc1));
    const V4 d2t = zd2(torc, (size_t)np4, k, a.nz, 3, V4(a.sc1));
    float *poldot = (float *)a.ht->p[5][2], *tordot = (float *)a.ht->p[6][2];
    const V4 pc = polc[(size_t)k * np4], tc = torc[(size_t)k * np4], ez = ld4(a.ez, i4);
    if (!a.var_eta) {
        const V4 zck(a.zck);
        st4(poldot, i4, zck * pc * kk + zck * d2p + w2);
        st4(tordot, i4, zck * tc * kk + zck * d2t - w3 + ez);
    } else {
        const V4 e(a.eta[k]);
        const V4 dt = zd1(torc, (size_t)np4, k, a.nz, 5, V4(a.ho12));
        st4(poldot, i4, e * pc * kk + e * d2p + w2);
        st4(tordot, i4, e * tc * kk + e * d2t - w3 + ez + V4(a.deta[k]) * dt);
    }
}

template <int NB>
static __global__ void k_bandj_spec4(const __grid_constant__ Batch<BandjArgs<float>, NB> bt)
{
    PDL_WAIT();
    const BandjArgs<float> &a = BATCH_MEMBER(bt, NB);
    const unsigned np = (unsigned)a.nx * a.ny, np4 = np / 4;
    const unsigned q4 = blockIdx.x * blockDim.x + threadIdx.x;
    if (q4 >= np4) return;
    const size_t pb = (size_t)blockIdx.y * np, i4 = (size_t)blockIdx.y * np4 + q4;
    const unsigned q = 4 * q4;
    const int j = (int)(q / (unsigned)a.nx), i0 = (int)(q - (unsigned)j * a.nx);
    const float *s = a.dzs + pb, *tp = a.tor + pb, *pp = a.pol + pb;
    st4(a.bxh, i4, sdx4(s, i0, j, a.nx, a.h.kx1) + sdy4(tp, i0, j, a.nx, a.ny, a.h.ky1));
    st4(a.byh, i4, sdy4(s, i0, j, a.nx, a.ny, a.h.ky1) - sdx4(tp, i0, j, a.nx, a.h.kx1));
    const V4 kk = ld4(a.h.kh2, q4);
    st4(a.bzh, i4, V4(-1.0f) * ld4(pp, q4) * kk);
    st4(a.jzh, i4, V4(-1.0f) * ld4(tp, q4) * kk);
    // (dybz null: the line transforms take the derivatives of bz instead)
    if (!a.dybz) return;
    // d/dy of ez = -pol*(akx2+aky2) at the mirrored row
    V4 dy(0.0f);
    if (!(j == 0 || 2 * j == a.ny)) {
        const unsigned m = (unsigned)(a.ny - j) * a.nx + i0;
        const V4 ezm = V4(-1.0f) * *reinterpret_cast<const V4 *>(pp + m) * *reinterpret_cast<const V4 *>(a.h.kh2 + m);
        dy = ezm * V4(a.h.ky1[j]);
        if (2 * j < a.ny) dy = -dy;
    }
    // d/dx at the mirrored column nx - i (four reversed points, two aligned loads)
    const float *prow = pp + (size_t)j * a.nx, *krow = a.h.kh2 + (size_t)j * a.nx;
    const V4 PA = *reinterpret_cast<const V4 *>(prow + a.nx - i0 - 4), KA = *reinterpret_cast<const V4 *>(krow + a.nx - i0 - 4);
    const float pbv = i0 == 0 ? 0.0f : prow[a.nx - i0], kbv = i0 == 0 ? 0.0f : krow[a.nx - i0];
    const float pm[4] = { pbv, PA.w, PA.z, PA.y }, km[4] = { kbv, KA.w, KA.z, KA.y };
    const V4 k1 = ld4(a.h.kx1, (size_t)i0 / 4);
    const float k1v[4] = { k1.x, k1.y, k1.z, k1.w };
    float dx[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const int i = i0 + c;
        float v = 0.0f;
        if (!(i == 0 || 2 * i == a.nx)) {
            const float ezm = -1.0f * pm[c] * km[c];
            v = ezm * k1v[c];
            if (2 * i < a.nx) v = -v;
        }
        dx[c] = v;
    }
    st4(a.dybz, i4, dy);
    st4(a.dxbz, i4, V4(dx[0], dx[1], dx[2], dx[3]));
}

struct Jsq4Args {
    const float *jz, *dybz, *dxbz, *bx, *by;
    float *jsq;
    size_t np;
    int nz;
    float h;
};
template <int NB>
static __global__ void k_jsq4(const __grid_constant__ Batch<Jsq4Args, NB> bt)
{
    PDL_WAIT();
    const Jsq4Args &A = BATCH_MEMBER(bt, NB);
    const float *jz = A.jz, *dybz = A.dybz, *dxbz = A.dxbz, *bx = A.bx, *by = A.by;
    float *jsq = A.jsq;
    const size_t np = A.np;
    const int nz = A.nz;
    const float h = A.h;
    const size_t np4 = np / 4;
    const size_t q4 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q4 >= np4) return;
    const int k = blockIdx.y;
    const size_t i4 = (size_t)k * np4 + q4;
    const V4 wk1 = zd1(reinterpret_cast<const V4 *>(by) + q4, np4, k, nz, 5, V4(h));
    const V4 wk2 = zd1(reinterpret_cast<const V4 *>(bx) + q4, np4, k, nz, 5, V4(h));
    const V4 ez = ld4(jz, i4), ex = ld4(dybz, i4), ey = ld4(dxbz, i4);
    st4(jsq, i4, ez * ez + ((ex - wk1) * (ex - wk1)) + ((wk2 - ey) * (wk2 - ey)));
}

// spectral truncation of the 2/3 rule, src/magnetic.f90:666-717
__host__ __device__ __forceinline__ bool truncated(int i, int j, int nx, int ny, int cx, int cy)
{
    return (i >= nx / 2 - cx && i <= nx / 2 + cx) || (j >= ny / 2 - cy && j <= ny / 2 + cy);
}

// (grid (np/256, nz))
template <typename R>
static __global__ void k_truncate(R *a, R *b, int nx, int ny, int nz, int cx, int cy)
{
    PDL_WAIT();
    const unsigned np = (unsigned)nx * ny;
    const unsigned q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const size_t idx = (size_t)blockIdx.y * np + q;
    const int j = (int)(q / (unsigned)nx), i = (int)(q - (unsigned)j * nx);
    if (truncated(i, j, nx, ny, cx, cy)) {
        a[idx] = (R)0;
        if (b) b[idx] = (R)0;
    }
}

// zero the newest magnetic RHS slots (F = 0, src/main.F90:355-376)
struct ZeroMagArgs {
    const HistTable *ht;
    size_t n;
    int nz;
};
template <typename R, int NB>
static __global__ void k_zero_mag_rhs(const __grid_constant__ Batch<ZeroMagArgs, NB> bt)
{
    PDL_WAIT();
    const HistTable *ht = BATCH_MEMBER(bt, NB).ht;
    const size_t n = BATCH_MEMBER(bt, NB).n;
    const int nz = BATCH_MEMBER(bt, NB).nz;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) { ((R *)ht->p[5][2])[i] = (R)0; ((R *)ht->p[6][2])[i] = (R)0; }
    if (i < (size_t)nz) { ht->bx[2][i] = 0.0; ht->by[2][i] = 0.0; }
}

// the history shift of src/main.F90:448-461 and :473-476 as a rotation of
// the logical slots: 0 <- 1 <- 2 <- old 0 (reused for the next RHS)
__device__ __forceinline__ void rotate_hist_table(HistTable *ht)
{
    for (int f = 0; f < 7; f++) {
        void *o = ht->p[f][0];
        ht->p[f][0] = ht->p[f][1];
        ht->p[f][1] = ht->p[f][2];
        ht->p[f][2] = o;
    }
    double *x = ht->bx[0], *y = ht->by[0];
    ht->bx[0] = ht->bx[1]; ht->bx[1] = ht->bx[2]; ht->bx[2] = x;
    ht->by[0] = ht->by[1]; ht->by[1] = ht->by[2]; ht->by[2] = y;
}
template <int NB>
static __global__ void k_rotate_hist(const __grid_constant__ Batch<HistTable *, NB> bt)
{
    PDL_WAIT();
    if (threadIdx.x == 0) rotate_hist_table(BATCH_MEMBER(bt, NB));
}
