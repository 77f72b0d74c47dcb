// zstencil.cuh -- the 4th-order z finite differences of src/dbydz.F90,
// evaluated for one (i,j) column at plane k (0-based; k=0 is the top).
// f points at plane 0 of the column; planes are np elements apart.
// Row formulas (serial branches src/dbydz.F90:1685-1751, 2353-2424,
// 3007-3083):
//   d1:   k=0 topdz(flag) :927, k=1 topdz_low :1053, interior :371,
//         k=nz-2 lastdz_up :776, k=nz-1 lastdz(flag) :626
//   d1up: as d1 but k=2 dup_up :532, 3..nz-4 dupinterior :485,
//         k=nz-3 dup_low :579, sign test on w at the same point
//   d2:   k=0 d2topdz(flag) :1368, k=1 d2topdz_low :1462, d2interior :428,
//         k=nz-2 d2lastdz_up :1271, k=nz-1 d2lastdz(flag) :1180
#pragma once

// A column of planes: F(k) = f[k np].  The stencils below take any accessor
// F(k) -> value of plane k (a column in global memory, or a ring of planes
// in shared memory); the pointer forms wrap a column.
template <typename R> struct ZCol {
    const R *f;
    size_t np;
    __host__ __device__ __forceinline__ R operator()(int k) const { return f[(size_t)k * np]; }
};

template <typename R, typename A>
__host__ __device__ __forceinline__ R zd1a(const A &F, int k, int nz, int fl, R h)
{
    if (k == 0) {
        if (fl == 1) return h * ((R)14 * F(0) + (R)36 * F(1) - (R)18 * F(2) + (R)4 * F(3));
        if (fl == 5) return h * ((R)-22 * F(0) + (R)36 * F(1) - (R)18 * F(2) + (R)4 * F(3));
        return (R)0;
    }
    if (k == 1) return h * ((R)-4 * F(0) - (R)6 * F(1) + (R)12 * F(2) - (R)2 * F(3));
    if (k == nz - 2) return h * ((R)4 * F(nz - 1) + (R)6 * F(nz - 2) - (R)12 * F(nz - 3) + (R)2 * F(nz - 4));
    if (k == nz - 1) {
        if (fl == 1) return h * ((R)-14 * F(nz - 1) - (R)36 * F(nz - 2) + (R)18 * F(nz - 3) - (R)4 * F(nz - 4));
        if (fl == 5) return h * ((R)22 * F(nz - 1) - (R)36 * F(nz - 2) + (R)18 * F(nz - 3) - (R)4 * F(nz - 4));
        return (R)0;
    }
    return h * (F(k - 2) - (R)8 * F(k - 1) + (R)8 * F(k + 1) - F(k + 2));
}

template <typename R, typename A>
__host__ __device__ __forceinline__ R zd1upa(const A &F, int k, int nz, int fl, R h, R wv)
{
    if (k <= 1 || k >= nz - 2) return zd1a(F, k, nz, fl, h);
    if (k == 2) {
        if (wv >= (R)0) return h * ((R)2 * F(0) - (R)12 * F(1) + (R)6 * F(2) + (R)4 * F(3));
        return h * (F(5) - (R)6 * F(4) + (R)18 * F(3) - (R)10 * F(2) - (R)3 * F(1));
    }
    if (k == nz - 3) {
        if (wv >= (R)0)
            return h * (-F(nz - 6) + (R)6 * F(nz - 5) - (R)18 * F(nz - 4) + (R)10 * F(nz - 3) + (R)3 * F(nz - 2));
        return h * ((R)-2 * F(nz - 1) + (R)12 * F(nz - 2) - (R)6 * F(nz - 3) - (R)4 * F(nz - 4));
    }
    if (wv >= (R)0)
        return h * (-F(k - 3) + (R)6 * F(k - 2) - (R)18 * F(k - 1) + (R)10 * F(k) + (R)3 * F(k + 1));
    return h * (F(k + 3) - (R)6 * F(k + 2) + (R)18 * F(k + 1) - (R)10 * F(k) - (R)3 * F(k - 1));
}

template <typename R, typename A>
__host__ __device__ __forceinline__ R zd2a(const A &F, int k, int nz, int fl, R s)
{
    if (k == 0) {
        if (fl == 3)
            return s * ((R)45 * F(0) - (R)154 * F(1) + (R)214 * F(2) - (R)156 * F(3) + (R)61 * F(4) - (R)10 * F(5));
        return (R)0;
    }
    if (k == 1)
        return s * ((R)10 * F(0) - (R)15 * F(1) - (R)4 * F(2) + (R)14 * F(3) - (R)6 * F(4) + F(5));
    if (k == nz - 2)
        return s * ((R)10 * F(nz - 1) - (R)15 * F(nz - 2) - (R)4 * F(nz - 3) + (R)14 * F(nz - 4) - (R)6 * F(nz - 5) + F(nz - 6));
    if (k == nz - 1) {
        if (fl == 3)
            return s * ((R)45 * F(nz - 1) - (R)154 * F(nz - 2) + (R)214 * F(nz - 3) - (R)156 * F(nz - 4) + (R)61 * F(nz - 5) - (R)10 * F(nz - 6));
        return (R)0;
    }
    return s * (-F(k - 2) + (R)16 * F(k - 1) - (R)30 * F(k) + (R)16 * F(k + 1) - F(k + 2));
}

template <typename R>
__host__ __device__ __forceinline__ R zd1(const R *f, size_t np, int k, int nz, int fl, R h)
{ return zd1a(ZCol<R>{ f, np }, k, nz, fl, h); }
template <typename R>
__host__ __device__ __forceinline__ R zd1up(const R *f, size_t np, int k, int nz, int fl, R h, R wv)
{ return zd1upa(ZCol<R>{ f, np }, k, nz, fl, h, wv); }
template <typename R>
__host__ __device__ __forceinline__ R zd2(const R *f, size_t np, int k, int nz, int fl, R s)
{ return zd2a(ZCol<R>{ f, np }, k, nz, fl, s); }

// spectral d/dx of a 2-D halfcomplex plane at (i,j): index shuffle of
// src/fft.F90:292-302 (the reference's "+ik" on the x halfcomplex index).
// (K: the table's type; a table in the plane's precision needs no conversion)
template <typename R, typename K>
__device__ __forceinline__ R sdx(const R *plane, int i, int j, int nx, const K *akx1)
{
    if (i == 0 || 2 * i == nx) return (R)0;
    R v = plane[(unsigned)j * nx + (nx - i)] * (R)akx1[i];
    return 2 * i < nx ? -v : v;
}
template <typename R, typename K>
__device__ __forceinline__ R sdy(const R *plane, int i, int j, int nx, int ny, const K *aky1)
{
    if (j == 0 || 2 * j == ny) return (R)0;
    R v = plane[(unsigned)(ny - j) * nx + i] * (R)aky1[j];
    return 2 * j < ny ? -v : v;
}

// z-marching register windows: v[d] = f(k-3+d) for the current plane k of a
// column (f points at the column's plane 0), zero outside [0, nz)
template <typename R>
__device__ __forceinline__ void zwin_init(R *v, const R *f, size_t np, int k0, int nz)
{
#pragma unroll
    for (int d = 0; d < 7; d++) {
        const int kk = k0 - 3 + d;
        v[d] = (kk >= 0 && kk < nz) ? f[(size_t)kk * np] : (R)0;
    }
}
// advance the window from plane k to k + 1
template <typename R>
__device__ __forceinline__ void zwin_next(R *v, const R *f, size_t np, int k, int nz)
{
#pragma unroll
    for (int d = 0; d < 6; d++) v[d] = v[d + 1];
    v[6] = k + 4 < nz ? f[(size_t)(k + 4) * np] : (R)0;
}

// Four consecutive x points as one value: 16-byte loads and stores, and the
// templates above (zd1, zd2) evaluate the same formulas per component.
struct __align__(16) V4 {
    float x, y, z, w;
    __host__ __device__ __forceinline__ V4() {}
    __host__ __device__ __forceinline__ V4(float s) : x(s), y(s), z(s), w(s) {}
    __host__ __device__ __forceinline__ V4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
};
__host__ __device__ __forceinline__ V4 operator+(V4 a, V4 b) { return V4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__host__ __device__ __forceinline__ V4 operator-(V4 a, V4 b) { return V4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
__host__ __device__ __forceinline__ V4 operator*(V4 a, V4 b) { return V4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
__host__ __device__ __forceinline__ V4 operator-(V4 a) { return V4(-a.x, -a.y, -a.z, -a.w); }
// per component: w >= 0 ? p : m
__host__ __device__ __forceinline__ V4 upsel(V4 w, V4 p, V4 m)
{
    return V4(w.x >= 0.0f ? p.x : m.x, w.y >= 0.0f ? p.y : m.y, w.z >= 0.0f ? p.z : m.z, w.w >= 0.0f ? p.w : m.w);
}

// zd1up for four points: both one-sided stencils of each row, chosen per
// component by the sign of w (the same formulas and operation order as the
// scalar zd1up)
template <typename A>
__host__ __device__ __forceinline__ V4 zd1upa(const A &F, int k, int nz, int fl, V4 h, V4 wv)
{
    typedef V4 R;
    if (k <= 1 || k >= nz - 2) return zd1a(F, k, nz, fl, h);
    if (k == 2)
        return upsel(wv, h * ((R)2 * F(0) - (R)12 * F(1) + (R)6 * F(2) + (R)4 * F(3)),
                     h * (F(5) - (R)6 * F(4) + (R)18 * F(3) - (R)10 * F(2) - (R)3 * F(1)));
    if (k == nz - 3)
        return upsel(wv, h * (-F(nz - 6) + (R)6 * F(nz - 5) - (R)18 * F(nz - 4) + (R)10 * F(nz - 3) + (R)3 * F(nz - 2)),
                     h * ((R)-2 * F(nz - 1) + (R)12 * F(nz - 2) - (R)6 * F(nz - 3) - (R)4 * F(nz - 4)));
    return upsel(wv, h * (-F(k - 3) + (R)6 * F(k - 2) - (R)18 * F(k - 1) + (R)10 * F(k) + (R)3 * F(k + 1)),
                 h * (F(k + 3) - (R)6 * F(k + 2) + (R)18 * F(k + 1) - (R)10 * F(k) - (R)3 * F(k - 1)));
}
__host__ __device__ __forceinline__ V4 zd1up(const V4 *f, size_t np, int k, int nz, int fl, V4 h, V4 wv)
{ return zd1upa(ZCol<V4>{ f, np }, k, nz, fl, h, wv); }

// Two consecutive x points (8-byte loads), the same operators as V4
struct __align__(8) V2 {
    float x, y;
    __host__ __device__ __forceinline__ V2() {}
    __host__ __device__ __forceinline__ V2(float s) : x(s), y(s) {}
    __host__ __device__ __forceinline__ V2(float a, float b) : x(a), y(b) {}
};
__host__ __device__ __forceinline__ V2 operator+(V2 a, V2 b) { return V2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ V2 operator-(V2 a, V2 b) { return V2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ V2 operator*(V2 a, V2 b) { return V2(a.x * b.x, a.y * b.y); }
__host__ __device__ __forceinline__ V2 operator/(V2 a, V2 b) { return V2(a.x / b.x, a.y / b.y); }
__host__ __device__ __forceinline__ V2 operator-(V2 a) { return V2(-a.x, -a.y); }
__host__ __device__ __forceinline__ V2 upsel(V2 w, V2 p, V2 m)
{
    return V2(w.x >= 0.0f ? p.x : m.x, w.y >= 0.0f ? p.y : m.y);
}
template <typename A>
__host__ __device__ __forceinline__ V2 zd1upa(const A &F, int k, int nz, int fl, V2 h, V2 wv)
{
    typedef V2 R;
    if (k <= 1 || k >= nz - 2) return zd1a(F, k, nz, fl, h);
    if (k == 2)
        return upsel(wv, h * ((R)2 * F(0) - (R)12 * F(1) + (R)6 * F(2) + (R)4 * F(3)),
                     h * (F(5) - (R)6 * F(4) + (R)18 * F(3) - (R)10 * F(2) - (R)3 * F(1)));
    if (k == nz - 3)
        return upsel(wv, h * (-F(nz - 6) + (R)6 * F(nz - 5) - (R)18 * F(nz - 4) + (R)10 * F(nz - 3) + (R)3 * F(nz - 2)),
                     h * ((R)-2 * F(nz - 1) + (R)12 * F(nz - 2) - (R)6 * F(nz - 3) - (R)4 * F(nz - 4)));
    return upsel(wv, h * (-F(k - 3) + (R)6 * F(k - 2) - (R)18 * F(k - 1) + (R)10 * F(k) + (R)3 * F(k + 1)),
                 h * (F(k + 3) - (R)6 * F(k + 2) + (R)18 * F(k + 1) - (R)10 * F(k) - (R)3 * F(k - 1)));
}
__host__ __device__ __forceinline__ V2 zd1up(const V2 *f, size_t np, int k, int nz, int fl, V2 h, V2 wv)
{ return zd1upa(ZCol<V2>{ f, np }, k, nz, fl, h, wv); }

// Interior rows (3 <= k <= nz-4) from a register window v[d] = f(k-3+d):
// the same formulas and operation order as zd1 / zd1up / zd2.
template <typename R>
__host__ __device__ __forceinline__ R wd1(const R *v, R h)
{ return h * (v[1] - (R)8 * v[2] + (R)8 * v[4] - v[5]); }
template <typename R>
__host__ __device__ __forceinline__ R wd1up(const R *v, R h, R wv)
{
    if (wv >= (R)0) return h * (-v[0] + (R)6 * v[1] - (R)18 * v[2] + (R)10 * v[3] + (R)3 * v[4]);
    return h * (v[6] - (R)6 * v[5] + (R)18 * v[4] - (R)10 * v[3] - (R)3 * v[2]);
}
template <typename R>
__host__ __device__ __forceinline__ R wd2(const R *v, R s)
{ return s * (-v[1] + (R)16 * v[2] - (R)30 * v[3] + (R)16 * v[4] - v[5]); }
