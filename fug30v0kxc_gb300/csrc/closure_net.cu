// closure_net.cu -- the learned closure's network: four 3x3x3 convolutions
// (16 -> 32 -> 32 -> 32 -> 16 channels, GELU between them) with BF16 weights
// and activations and FP32 accumulation on the tensor cores (mma.sync
// m16n8k16), trained with Adam.  Every convolution pass -- forward, input
// gradient and weight gradient -- is an implicit GEMM over channel-last
// activations staged in shared memory.
//
// Layout: activations [sample][z][y][x][channel], channel fastest, BF16;
// periodic in x and y, zero padding in z (the walls).  Tap t = 9(dz+1) +
// 3(dy+1) + (dx+1) multiplies X[x+dx, y+dy, z+dz] (a correlation).  Forward
// weights are [27][cout][cin]; the input-gradient pass uses the same weights
// flipped in the tap and transposed, [27][cin][cout], so it runs through the
// forward kernel.
//
// A tile is 128 consecutive points of one z-plane (128/nx rows of nx points;
// nx in {16, 32, 64, 128}).  Its halo -- 3 planes x (rows + 2) x (nx + 2)
// points, wrapped in x and y, zero outside the walls -- is copied into
// shared memory with cp.async; rows are padded by 8 channels (16 bytes), so
// the ldmatrix row addresses of eight consecutive points fall in distinct
// bank groups.  CTAs are persistent over tiles and keep the weights of their
// layer in shared memory.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "common.cuh"
#include "closure_net.h"

namespace {

typedef __nv_bfloat16 bf16;
constexpr int TP = 128;       // points per tile
constexpr int NTAP = 27;

__device__ __forceinline__ unsigned su32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

// 16-byte asynchronous copy global -> shared, zero-filled when !valid
__device__ __forceinline__ void cp16(unsigned dst, const void *src, bool valid)
{
    const int sz = valid ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(sz) : "memory");
}
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__device__ __forceinline__ void ldsm4(unsigned a, uint32_t *r)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(a));
}
__device__ __forceinline__ void ldsm4t(unsigned a, uint32_t *r)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(a));
}
// D += A(16x16, row) * B(16x8, col), BF16 in, FP32 accumulate
__device__ __forceinline__ void mma16816(float *c, const uint32_t *a, uint32_t b0, uint32_t b1)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// GELU with the Gaussian CDF, and its derivative
__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float x)
{
    return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

struct TileAt {
    int b, z, y0;
    size_t plane0;    // global point index of (b, z, 0, 0)
    int q0;           // first point of the tile within the plane
};

// tile t of tp points (g.R = tp / nx rows)
__device__ __forceinline__ TileAt tile_at(const NetGeom &g, long long t, int tp = TP)
{
    const int tpp = g.nx * g.ny / tp;
    TileAt a;
    a.b = (int)(t / ((long long)g.nz * tpp));
    const int rem = (int)(t - (long long)a.b * g.nz * tpp);
    a.z = rem / tpp;
    const int tip = rem - a.z * tpp;
    a.y0 = tip * g.R;
    a.q0 = tip * tp;
    a.plane0 = ((size_t)a.b * g.nz + a.z) * (size_t)g.ny * g.nx;
    return a;
}

// halo [3][R+2][nx+2] points of C channels (row stride C + 8)
template <int C>
__device__ __forceinline__ void load_halo(bf16 *h, const bf16 *src, const NetGeom &g, const TileAt &a)
{
    constexpr int CS = C + 8, CH = C / 8;
    const int W = g.nx + 2, RR = g.R + 2;
    const int total = 3 * RR * W * CH;
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        const int c = e % CH;
        const int pt = e / CH;
        const int xi = pt % W;
        const int rr = (pt / W) % RR;
        const int dz = pt / (W * RR);
        const int zz = a.z + dz - 1;
        int yy = a.y0 + rr - 1;
        yy = yy < 0 ? yy + g.ny : (yy >= g.ny ? yy - g.ny : yy);
        int xx = xi - 1;
        xx = xx < 0 ? xx + g.nx : (xx >= g.nx ? xx - g.nx : xx);
        const bool ok = zz >= 0 && zz < g.nz;
        const size_t gp = ok ? ((((size_t)a.b * g.nz + zz) * g.ny + yy) * g.nx + xx) : 0;
        cp16(su32(h + (size_t)pt * CS + c * 8), src + gp * C + c * 8, ok);
    }
}

// ---- forward / input-gradient convolution -------------------------------------------
// EPI_ACT: pre = acc + bias -> o_pre (BF16), gelu(pre) -> o_act (BF16)
// EPI_OUT: acc + bias -> o_f32 (FP32, first cout_real channels)
// EPI_GATE: acc * gelu'(gate) -> o_act (BF16)      (input gradient)
enum { EPI_ACT = 0, EPI_OUT = 1, EPI_GATE = 2 };

// MT m-tiles (16 MT points) per warp: a CTA tile is 128 MT points, and g.R
// and g.tiles describe that tile.  KS warp groups of 8 split the 27 taps;
// groups above the first hand their partial sums over through shared memory
template <int CIN, int COUT, int EPI, int MT, int KS>
__global__ void __launch_bounds__(256 * KS, 1)
k_conv(const bf16 *__restrict__ x, const bf16 *__restrict__ wt, const float *__restrict__ bias, NetGeom g,
       bf16 *__restrict__ o_pre, bf16 *__restrict__ o_act, float *__restrict__ o_f32, int cout_real,
       const bf16 *__restrict__ gate)
{
    constexpr int CSI = CIN + 8;
    extern __shared__ __align__(128) unsigned char smem[];
    bf16 *ws = reinterpret_cast<bf16 *>(smem);               // [27][COUT][CSI]
    bf16 *hs = ws + (size_t)NTAP * COUT * CSI;               // halo
    const int tid = threadIdx.x, lane = tid & 31, w = (tid >> 5) & 7, gk = tid >> 8;
    const int tap0 = (NTAP * gk) / KS, tap1 = (NTAP * (gk + 1)) / KS;

    for (int e = tid; e < NTAP * COUT * (CIN / 8); e += blockDim.x) {
        const int row = e / (CIN / 8), c = e % (CIN / 8);
        cp16(su32(ws + (size_t)row * CSI + c * 8), wt + (size_t)row * CIN + c * 8, true);
    }
    const int W2 = g.nx + 2, RR = g.R + 2;
    int yl[MT], x0[MT];
#pragma unroll
    for (int m = 0; m < MT; m++) {
        yl[m] = (16 * (MT * w + m)) / g.nx;
        x0[m] = (16 * (MT * w + m)) % g.nx;
    }
    for (long long t = blockIdx.x; t < g.tiles; t += gridDim.x) {
        const TileAt a = tile_at(g, t, TP * MT);
        __syncthreads();                      // previous tile's reads of hs are done
        load_halo<CIN>(hs, x, g, a);
        cp_wait_all();
        __syncthreads();
        float acc[MT][COUT / 8][4];
#pragma unroll
        for (int m = 0; m < MT; m++)
#pragma unroll
            for (int j = 0; j < COUT / 8; j++) acc[m][j][0] = acc[m][j][1] = acc[m][j][2] = acc[m][j][3] = 0.0f;
        const int pa = (lane & 7) + ((lane >> 3) & 1) * 8, ca = (lane >> 4) * 8;    // A: point, channel
        const int nb_ = (lane & 7) + (lane >> 4) * 8, kb = ((lane >> 3) & 1) * 8;   // B: row n, column k
#pragma unroll 1
        for (int tap = tap0; tap < tap1; tap++) {
            const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
#pragma unroll
            for (int kk = 0; kk < CIN / 16; kk++) {
                uint32_t af[MT][4];
#pragma unroll
                for (int m = 0; m < MT; m++) {
                    const int hrow = (dz * RR + yl[m] + dy) * W2 + x0[m] + dx;
                    ldsm4(su32(hs + (size_t)(hrow + pa) * CSI + kk * 16 + ca), af[m]);
                }
#pragma unroll
                for (int np = 0; np < COUT / 16; np++) {
                    uint32_t bfr[4];
                    ldsm4(su32(ws + (size_t)(tap * COUT + np * 16 + nb_) * CSI + kk * 16 + kb), bfr);
#pragma unroll
                    for (int m = 0; m < MT; m++) {
                        mma16816(acc[m][2 * np], af[m], bfr[0], bfr[1]);
                        mma16816(acc[m][2 * np + 1], af[m], bfr[2], bfr[3]);
                    }
                }
            }
        }
        if (KS > 1) {
            // the other groups' partial sums through shared memory (the halo
            // is not read again before the next tile's barrier)
            float *red = reinterpret_cast<float *>(hs);
            __syncthreads();
            if (gk > 0) {
#pragma unroll
                for (int m = 0; m < MT; m++)
#pragma unroll
                    for (int j = 0; j < COUT / 8; j++)
#pragma unroll
                        for (int c = 0; c < 4; c++)
                            red[((((size_t)(gk - 1) * 8 + w) * MT + m) * (COUT / 8) + j) * 128 + c * 32 + lane] =
                                acc[m][j][c];
            }
            __syncthreads();
            if (gk > 0) continue;
            for (int q = 1; q < KS; q++)
#pragma unroll
                for (int m = 0; m < MT; m++)
#pragma unroll
                    for (int j = 0; j < COUT / 8; j++)
#pragma unroll
                        for (int c = 0; c < 4; c++)
                            acc[m][j][c] += red[((((size_t)(q - 1) * 8 + w) * MT + m) * (COUT / 8) + j) * 128 + c * 32 + lane];
        }
        // epilogue: c0,c1 at (row g, n 2t', 2t'+1), c2,c3 at row g+8
        const int gr = lane >> 2, tq = lane & 3;
#pragma unroll
        for (int m = 0; m < MT; m++)
#pragma unroll
            for (int j = 0; j < COUT / 8; j++) {
                const int n = 8 * j + 2 * tq;
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const size_t gp = a.plane0 + a.q0 + 16 * (MT * w + m) + gr + 8 * h;
                    float v0 = acc[m][j][2 * h], v1 = acc[m][j][2 * h + 1];
                    if (EPI == EPI_ACT) {
                        v0 += bias[n];
                        v1 += bias[n + 1];
                        *reinterpret_cast<__nv_bfloat162 *>(o_pre + gp * COUT + n) = __floats2bfloat162_rn(v0, v1);
                        *reinterpret_cast<__nv_bfloat162 *>(o_act + gp * COUT + n) =
                            __floats2bfloat162_rn(gelu_f(v0), gelu_f(v1));
                    } else if (EPI == EPI_OUT) {
                        if (n < cout_real) o_f32[gp * cout_real + n] = v0 + bias[n];
                        if (n + 1 < cout_real) o_f32[gp * cout_real + n + 1] = v1 + bias[n + 1];
                    } else {
                        const __nv_bfloat162 gg = *reinterpret_cast<const __nv_bfloat162 *>(gate + gp * COUT + n);
                        v0 *= gelu_d(__bfloat162float(gg.x));
                        v1 *= gelu_d(__bfloat162float(gg.y));
                        *reinterpret_cast<__nv_bfloat162 *>(o_act + gp * COUT + n) = __floats2bfloat162_rn(v0, v1);
                    }
                }
            }
    }
}

// ---- forward / input gradient on the 5th-generation tensor cores ---------------------
// For nx = 128 a tile is one row of 128 points: one M = 128 tcgen05.mma per
// tap and 16-channel K step, accumulating in 32 TMEM columns.  Operands sit
// in shared memory in the canonical K-major, non-swizzled layout (core
// matrices of 8 rows x 16 bytes): the halo as [halo row][8-channel block]
// [130 points][8 channels], so each tap's A operand is the same descriptor
// shifted by (row, dx); the weights as [tap][8-channel block][n][8].  One
// thread issues the 27 x CIN/16 MMAs of a tile, spread over four independent
// accumulator chains that the epilogue sums, and commits them to an
// mbarrier.  Two sets of accumulators (2 x 4 x 32 TMEM columns) and two halo
// buffers form a pipeline between a producer warp (halo copies, MMA issue)
// and eight epilogue warps (tcgen05.ld, the epilogue of k_conv): while tile
// i is read back, the halo and MMAs of tile i + 1 proceed.

// shared-memory matrix descriptor: start, leading (K-direction) and stride
// (M/N-direction) byte offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t umma_sdesc(unsigned saddr, unsigned lbo, unsigned sbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) |
           ((uint64_t)((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int m, int n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(unsigned tmem_d, uint64_t a, uint64_t b, uint32_t idesc, int accum)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
                 ::"r"(tmem_d), "l"(a), "l"(b), "r"(idesc), "r"(accum)
                 : "memory");
}

// bounded wait on an mbarrier phase; false when the limit ran out.  After a
// few polls the waiting thread sleeps between polls, so waiting warps leave
// the issue slots to the warp that issues the copies and MMAs.
__device__ __forceinline__ bool tc_mbar_wait(uint64_t *bar, unsigned parity)
{
    const unsigned a = su32(bar);
    for (long it = 0; it < (1L << 24); it++) {
        unsigned ok;
        asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                     : "=r"(ok)
                     : "r"(a), "r"(parity)
                     : "memory");
        if (ok) return true;
        if (it > 4) __nanosleep(64);
    }
    return false;
}

template <int NC>
__device__ __forceinline__ void tmem_ld(unsigned taddr, float *v);
template <>
__device__ __forceinline__ void tmem_ld<16>(unsigned taddr, float *v)
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                 "[%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

template <>
__device__ __forceinline__ void tmem_ld<8>(unsigned taddr, float *v)
{
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}

// halo row: 144 slots per (row, 8-channel block): x = -1 at slot 7, x = 0..127
// at slots 8..135 (a 128-byte aligned TMA box), x = 128 at slot 136
constexpr int TC_RL = 144;
constexpr int TC_X0 = 8;
constexpr int TC_ROWS = 9;         // 3 planes x 3 rows
constexpr int TC_TMEM_COLS = 256;  // two tiles x (3 x COUT <= 96) columns

// halo of row-tile a into h: [TC_ROWS][C/8][TC_RL][8].  One thread issues a
// TMA box (8 channels x 128 points, 2 KB) per row and channel block within
// the walls, counted on the mbarrier tb; all threads copy the two wrapped
// edge points per row and block with cp.async and zero the rows outside the
// walls.
__device__ __forceinline__ void tma_load_5d(unsigned dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            int c4, unsigned bar)
{
    asm volatile("cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
                 "%5, %6}], [%7];" ::"r"(dst),
                 "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
                 : "memory");
}

// (run by a group of nt threads; tl is the thread's index in the group)
template <int C>
__device__ __forceinline__ void load_halo_tc(bf16 *h, const CUtensorMap *tm, const bf16 *src, const NetGeom &g,
                                             const TileAt &a, uint64_t *tb, int tl, int nt)
{
    constexpr int C8 = C / 8;
    if (tl == 0) {
        int nr = 0;
        for (int row = 0; row < TC_ROWS; row++) {
            const int zz = a.z + row / 3 - 1;
            nr += (zz >= 0 && zz < g.nz) ? 1 : 0;
        }
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(tb)),
                     "r"((unsigned)(nr * C8 * 128 * 16))
                     : "memory");
        for (int row = 0; row < TC_ROWS; row++) {
            const int zz = a.z + row / 3 - 1;
            if (zz < 0 || zz >= g.nz) continue;
            int yy = a.y0 + row % 3 - 1;
            yy = yy < 0 ? yy + g.ny : (yy >= g.ny ? yy - g.ny : yy);
            for (int c = 0; c < C8; c++)
                tma_load_5d(su32(h + (((size_t)row * C8 + c) * TC_RL + TC_X0) * 8), tm, 0, c, 0, yy, a.b * g.nz + zz,
                            su32(tb));
        }
    }
    for (int e = tl; e < TC_ROWS * C8 * 2; e += nt) {
        const int row = e / (C8 * 2), c = (e / 2) % C8, side = e & 1;
        const int zz = a.z + row / 3 - 1;
        int yy = a.y0 + row % 3 - 1;
        yy = yy < 0 ? yy + g.ny : (yy >= g.ny ? yy - g.ny : yy);
        const int xx = side ? 0 : g.nx - 1;
        const bool ok = zz >= 0 && zz < g.nz;
        const size_t gp = ok ? ((((size_t)a.b * g.nz + zz) * g.ny + yy) * g.nx + xx) : 0;
        cp16(su32(h + (((size_t)row * C8 + c) * TC_RL + (side ? TC_X0 + 128 : TC_X0 - 1)) * 8), src + gp * C + c * 8, ok);
    }
    // rows outside the walls: only the first and last planes have any
    for (int dzr = 0; dzr < 3; dzr++) {
        const int zz = a.z + dzr - 1;
        if (zz >= 0 && zz < g.nz) continue;
        for (int e = tl; e < 3 * C8 * 128; e += nt) {
            const int row = dzr * 3 + e / (C8 * 128);
            const int c = (e / 128) % C8, xi = e % 128;
            *reinterpret_cast<uint4 *>(h + (((size_t)row * C8 + c) * TC_RL + TC_X0 + xi) * 8) = make_uint4(0, 0, 0, 0);
        }
    }
}

template <int CIN, int COUT>
__host__ __device__ constexpr size_t tc_halo_bytes() { return (size_t)TC_ROWS * TC_RL * CIN * sizeof(bf16); }
// epilogue exchange at the warp boundaries: [2 tiles][4 quads][2 halves][3][COUT/2] floats
template <int CIN, int COUT>
__host__ __device__ constexpr size_t tc_xch_bytes() { return (size_t)2 * 4 * 2 * 3 * (COUT / 2) * sizeof(float); }
template <int CIN, int COUT>
__host__ __device__ constexpr size_t tc_smem_bytes()
{
    // two halo buffers, the weights, the epilogue exchange
    return 2 * tc_halo_bytes<CIN, COUT>() + (size_t)NTAP * COUT * CIN * sizeof(bf16) + tc_xch_bytes<CIN, COUT>();
}

// warp roles: warps 0-7 read the accumulators back and run the epilogue,
// warp 8 (the producer) copies halos in and issues the MMAs; they meet only
// at mbarriers (per set b of buffers: tbar halo landed, full MMAs done,
// empty epilogue done).
//
// One MMA per input row r = (dz, dy) and 16-channel step computes the three
// dx taps at once: A = the 128 halo points x = -1..126 of row r, B = the
// weights of taps (r, dx = 0, 1, 2) stacked as N = 3 COUT rows.  TMEM row j
// (point x = j - 1) then holds D_dx[j] for all dx, and by the periodicity in
// x the output is out[x] = D_0[x] + D_1[(x + 1) mod 128] + D_2[(x + 2) mod
// 128]: a circular shift that the epilogue does with warp shuffles and, at
// the warp boundaries, a small shared-memory exchange.
constexpr int TC_THREADS = 288;

template <int CIN, int COUT, int EPI>
__global__ void __launch_bounds__(TC_THREADS, 1)
k_conv_tc(const bf16 *__restrict__ x, const __grid_constant__ CUtensorMap tmx, const bf16 *__restrict__ wt,
          const float *__restrict__ bias, NetGeom g, bf16 *__restrict__ o_pre, bf16 *__restrict__ o_act,
          float *__restrict__ o_f32, int cout_real, const bf16 *__restrict__ gate, int *err)
{
    constexpr int C8 = CIN / 8, HC = COUT / 2, N3 = 3 * COUT;
    constexpr uint32_t IDESC = umma_idesc_bf16(128, N3);
    extern __shared__ __align__(128) unsigned char smem[];
    bf16 *hb[2];
    hb[0] = reinterpret_cast<bf16 *>(smem);
    hb[1] = hb[0] + tc_halo_bytes<CIN, COUT>() / sizeof(bf16);
    bf16 *ws = hb[1] + tc_halo_bytes<CIN, COUT>() / sizeof(bf16);   // [9 rows][C8][3 COUT][8]
    float *xch = reinterpret_cast<float *>(ws + (size_t)NTAP * COUT * CIN);
    __shared__ __align__(8) uint64_t tbar[2], full[2], empty[2];
    __shared__ unsigned tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // B rows of input row r: dx * COUT + n, from wt[tap = 3 r + dx][n][k]
    for (int e = tid; e < NTAP * COUT * C8; e += blockDim.x) {
        const int tap = e / (COUT * C8), rr = e % (COUT * C8), n = rr / C8, k8 = rr % C8;
        const int r = tap / 3, dx = tap % 3;
        cp16(su32(ws + (((size_t)r * C8 + k8) * N3 + dx * COUT + n) * 8), wt + ((size_t)tap * COUT + n) * CIN + k8 * 8,
             true);
    }
    if (warp == 8) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&tmem_slot)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int b = 0; b < 2; b++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&tbar[b])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&full[b])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 8;" ::"r"(su32(&empty[b])) : "memory");
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("cp.async.wait_all;" ::: "memory");                 // the weights
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = tmem_slot;
    const long long G = gridDim.x, t0 = blockIdx.x;
    long long issued = 0;          // producer: tiles whose MMAs were committed
    bool failed = false;

    if (warp == 8) {
        // producer: halo of tile i + 1 is copied while the MMAs of tile i run
        if (t0 < g.tiles) load_halo_tc<CIN>(hb[0], &tmx, x, g, tile_at(g, t0, TP), &tbar[0], lane, 32);
        int i = 0;
        for (long long t = t0; t < g.tiles; t += G, i++) {
            const int b = i & 1;
            asm volatile("cp.async.wait_all;" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            // lane 0 waits (halo i landed, accumulators b released by the
            // epilogue of tile i - 2) and issues; the warp follows its verdict
            bool okw = true;
            if (lane == 0) {
                okw = tc_mbar_wait(&tbar[b], (i >> 1) & 1);
                if (okw && i >= 2) okw = tc_mbar_wait(&empty[b], ((i - 2) >> 1) & 1);
                if (okw) {
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const unsigned hbase = su32(hb[b]), wbase = su32(ws);
                    const unsigned d = tmem + (unsigned)(b * 128);
#pragma unroll 1
                    for (int r = 0; r < TC_ROWS; r++) {
#pragma unroll
                        for (int kk = 0; kk < CIN / 16; kk++) {
                            const uint64_t ad = umma_sdesc(
                                hbase + (unsigned)((((r * C8 + 2 * kk) * TC_RL) + TC_X0 - 1) * 16), TC_RL * 16, 128);
                            const uint64_t bd =
                                umma_sdesc(wbase + (unsigned)(((r * C8 + 2 * kk) * N3) * 16), N3 * 16, 128);
                            umma_bf16(d, ad, bd, IDESC, (r | kk) != 0);
                        }
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     su32(&full[b]))
                                 : "memory");
                }
            }
            if (!__shfl_sync(0xffffffffu, okw ? 1 : 0, 0)) { failed = true; break; }
            issued++;
            if (t + G < g.tiles) {
                // buffer b ^ 1 is free once the MMAs of tile i - 1 completed
                okw = true;
                if (lane == 0 && i >= 1) okw = tc_mbar_wait(&full[b ^ 1], ((i - 1) >> 1) & 1);
                if (!__shfl_sync(0xffffffffu, okw ? 1 : 0, 0)) { failed = true; break; }
                load_halo_tc<CIN>(hb[b ^ 1], &tmx, x, g, tile_at(g, t + G, TP), &tbar[b ^ 1], lane, 32);
            }
        }
    } else {
        // epilogue: warp w owns TMEM lanes 32 (w % 4).. (quad q) and the
        // channels (w / 4) COUT / 2 .. (half h)
        const int quad = warp & 3, half = warp >> 2, n0 = half * HC;
        int i = 0;
        for (long long t = t0; t < g.tiles; t += G, i++) {
            const int b = i & 1;
            bool okw = true;
            if (lane == 0) okw = tc_mbar_wait(&full[b], (i >> 1) & 1);
            if (!__shfl_sync(0xffffffffu, okw ? 1 : 0, 0)) { failed = true; break; }
            __syncwarp();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const TileAt a = tile_at(g, t, TP);
            float v[HC], d1[HC], d2[HC];
            {
                const unsigned ta = tmem + ((unsigned)(quad * 32) << 16) + (unsigned)(b * 128 + n0);
                tmem_ld<HC>(ta, v);
                tmem_ld<HC>(ta + (unsigned)COUT, d1);
                tmem_ld<HC>(ta + (unsigned)(2 * COUT), d2);
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0)   // accumulators b are free again
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(&empty[b])) : "memory");
            // rows 32 q and 32 q + 1 to the previous quad's lanes 30 and 31
            float *xo = xch + (((size_t)b * 4 + quad) * 2 + half) * 3 * HC;
            if (lane == 0) {
#pragma unroll
                for (int n = 0; n < HC; n++) { xo[n] = d1[n]; xo[HC + n] = d2[n]; }
            }
            if (lane == 1) {
#pragma unroll
                for (int n = 0; n < HC; n++) xo[2 * HC + n] = d2[n];
            }
            asm volatile("bar.sync 1, 256;" ::: "memory");
            const float *xi = xch + (((size_t)b * 4 + ((quad + 1) & 3)) * 2 + half) * 3 * HC;
#pragma unroll
            for (int n = 0; n < HC; n++) {
                float s1 = __shfl_down_sync(0xffffffffu, d1[n], 1);
                float s2 = __shfl_down_sync(0xffffffffu, d2[n], 2);
                if (lane == 31) s1 = xi[n];
                if (lane == 30) s2 = xi[HC + n];
                if (lane == 31) s2 = xi[2 * HC + n];
                v[n] += s1 + s2;
            }
            const size_t gp = a.plane0 + a.q0 + quad * 32 + lane;
            if (EPI == EPI_ACT) {
                __align__(16) __nv_bfloat162 pr[HC / 2], ac[HC / 2];
#pragma unroll
                for (int n = 0; n < HC; n += 2) {
                    const float v0 = v[n] + bias[n0 + n], v1 = v[n + 1] + bias[n0 + n + 1];
                    pr[n / 2] = __floats2bfloat162_rn(v0, v1);
                    ac[n / 2] = __floats2bfloat162_rn(gelu_f(v0), gelu_f(v1));
                }
#pragma unroll
                for (int q = 0; q < HC / 8; q++) {
                    reinterpret_cast<uint4 *>(o_pre + gp * COUT + n0)[q] = reinterpret_cast<const uint4 *>(pr)[q];
                    reinterpret_cast<uint4 *>(o_act + gp * COUT + n0)[q] = reinterpret_cast<const uint4 *>(ac)[q];
                }
            } else if (EPI == EPI_OUT) {
#pragma unroll
                for (int n = 0; n < HC; n++)
                    if (n0 + n < cout_real) o_f32[gp * cout_real + n0 + n] = v[n] + bias[n0 + n];
            } else {
                __align__(16) __nv_bfloat162 gg[HC / 2], ac[HC / 2];
#pragma unroll
                for (int q = 0; q < HC / 8; q++)
                    reinterpret_cast<uint4 *>(gg)[q] = reinterpret_cast<const uint4 *>(gate + gp * COUT + n0)[q];
#pragma unroll
                for (int n = 0; n < HC; n += 2)
                    ac[n / 2] = __floats2bfloat162_rn(v[n] * gelu_d(__bfloat162float(gg[n / 2].x)),
                                                      v[n + 1] * gelu_d(__bfloat162float(gg[n / 2].y)));
#pragma unroll
                for (int q = 0; q < HC / 8; q++)
                    reinterpret_cast<uint4 *>(o_act + gp * COUT + n0)[q] = reinterpret_cast<const uint4 *>(ac)[q];
            }
        }
        // a warp that stopped early keeps the named barrier count of the others
        if (failed) {
            for (long long t = t0 + (long long)i * G; t < g.tiles; t += G) asm volatile("bar.sync 1, 256;" ::: "memory");
        }
    }
    if (failed && lane == 0) atomicExch(err, 2);
    // after a failure the producer waits, bounded, for the MMAs it committed
    if (failed && warp == 8 && lane == 0 && issued > 0)
        tc_mbar_wait(&full[(issued - 1) & 1], ((issued - 1) >> 1) & 1);
    asm volatile("cp.async.wait_all;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 8)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
}

// ---- weight gradient ----------------------------------------------------------------------
// dW[tap][co][ci] = sum_p dY[p][co] X[p + d(tap)][ci], db[co] = sum_p dY[p][co].
// Nine warps; warp w = 3 dz + dy owns the three taps (dz, dy, dx = -1..1).
// Per-CTA partial sums go to part[block][27*CO*CI + CO].
// TPW taps per warp, 27 / TPW warps: warp w owns taps w TPW .. w TPW + TPW - 1
template <int CI, int CO, int TPW>
__global__ void __launch_bounds__(32 * (NTAP / TPW), 1)
k_wgrad(const bf16 *__restrict__ x, const bf16 *__restrict__ dy, NetGeom g, float *__restrict__ part)
{
    constexpr int CSI = CI + 8, CSO = CO + 8;
    extern __shared__ __align__(128) unsigned char smem[];
    bf16 *hs = reinterpret_cast<bf16 *>(smem);
    const int W2 = g.nx + 2, RR = g.R + 2;
    bf16 *ds = hs + (size_t)3 * RR * W2 * CSI;              // [TP][CSO]
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;

    float acc[TPW][CO / 16][CI / 8][4];
#pragma unroll
    for (int d = 0; d < TPW; d++)
#pragma unroll
        for (int m = 0; m < CO / 16; m++)
#pragma unroll
            for (int n = 0; n < CI / 8; n++) acc[d][m][n][0] = acc[d][m][n][1] = acc[d][m][n][2] = acc[d][m][n][3] = 0.0f;
    float bsum = 0.0f;

    for (long long t = blockIdx.x; t < g.tiles; t += gridDim.x) {
        const TileAt a = tile_at(g, t);
        __syncthreads();
        load_halo<CI>(hs, x, g, a);
        for (int e = tid; e < TP * (CO / 8); e += blockDim.x) {
            const int p = e / (CO / 8), c = e % (CO / 8);
            cp16(su32(ds + (size_t)p * CSO + c * 8), dy + (a.plane0 + a.q0 + p) * CO + c * 8, true);
        }
        cp_wait_all();
        __syncthreads();
        if (tid < 8 * CO) {   // bias: channel tid % CO over points tid / CO, +8, ...
            float s = 0.0f;
#pragma unroll 4
            for (int p = tid / CO; p < TP; p += 8) s += __bfloat162float(ds[(size_t)p * CSO + tid % CO]);
            bsum += s;
        }
        const int pa = (lane & 7) + (lane >> 4) * 8, ca = ((lane >> 3) & 1) * 8;   // A^T: point, co
        const int pb = (lane & 7) + ((lane >> 3) & 1) * 8, cb = (lane >> 4) * 8;   // B^T: point, ci
#pragma unroll 1
        for (int s = 0; s < TP / 16; s++) {
            const int yl = (16 * s) / g.nx, x0 = (16 * s) % g.nx;
            uint32_t af[CO / 16][4];
#pragma unroll
            for (int m = 0; m < CO / 16; m++) ldsm4t(su32(ds + (size_t)(16 * s + pa) * CSO + 16 * m + ca), af[m]);
#pragma unroll
            for (int d = 0; d < TPW; d++) {
                const int tap = TPW * w + d;
                const int hrow = ((tap / 9) * RR + yl + (tap / 3) % 3) * W2 + x0 + tap % 3;
#pragma unroll
                for (int np = 0; np < CI / 16; np++) {
                    uint32_t bfr[4];
                    ldsm4t(su32(hs + (size_t)(hrow + pb) * CSI + 16 * np + cb), bfr);
#pragma unroll
                    for (int m = 0; m < CO / 16; m++) {
                        mma16816(acc[d][m][2 * np], af[m], bfr[0], bfr[1]);
                        mma16816(acc[d][m][2 * np + 1], af[m], bfr[2], bfr[3]);
                    }
                }
            }
        }
    }
    float *pp = part + (size_t)blockIdx.x * (NTAP * CO * CI + CO);
    const int gr = lane >> 2, tq = lane & 3;
#pragma unroll
    for (int d = 0; d < TPW; d++) {
        const int tap = TPW * w + d;
#pragma unroll
        for (int m = 0; m < CO / 16; m++)
#pragma unroll
            for (int n = 0; n < CI / 8; n++)
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int co = 16 * m + gr + 8 * h, ci = 8 * n + 2 * tq;
                    pp[((size_t)tap * CO + co) * CI + ci] = acc[d][m][n][2 * h];
                    pp[((size_t)tap * CO + co) * CI + ci + 1] = acc[d][m][n][2 * h + 1];
                }
    }
    // sum the eight point groups of each bias channel (hs is free now)
    __syncthreads();
    float *red = reinterpret_cast<float *>(hs);
    if (tid < 8 * CO) red[tid] = bsum;
    __syncthreads();
    if (tid < CO) {
        float b = 0.0f;
#pragma unroll
        for (int gq = 0; gq < 8; gq++) b += red[gq * CO + tid];
        pp[NTAP * CO * CI + tid] = b;
    }
}

// out[j] = sum over blocks of part[b][j]
__global__ void k_reduce_parts(const float *part, int nblocks, int J, float *out)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= J) return;
    float s = 0.0f;
    for (int b = 0; b < nblocks; b++) s += part[(size_t)b * J + j];
    out[j] = s;
}

// ---- loss, optimiser, weight packing ---------------------------------------------------
// mean-squared error over P points x C channels; dout (BF16, 16 channels,
// the last 16 - C zero) = 2 (out - tgt) / (P C)
__global__ void k_mse(const float *out, const float *tgt, size_t P, int C, bf16 *dout, double *loss)
{
    __shared__ double red[256];
    double acc = 0.0;
    const double inv = 1.0 / ((double)P * C);
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (size_t)gridDim.x * blockDim.x) {
        float g[16];
#pragma unroll
        for (int c = 0; c < 16; c++) g[c] = 0.0f;
        for (int c = 0; c < C; c++) {
            const float d = out[p * C + c] - tgt[p * C + c];
            acc += (double)d * d;
            g[c] = (float)(2.0 * inv) * d;
        }
#pragma unroll
        for (int c = 0; c < 16; c += 2)
            *reinterpret_cast<__nv_bfloat162 *>(dout + p * 16 + c) = __floats2bfloat162_rn(g[c], g[c + 1]);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0] * inv);
}

// Adam (Kingma & Ba), bias-corrected, step t >= 1
__global__ void k_adam(float *p, const float *g, float *m, float *v, size_t n, float lr, float b1, float b2,
                       float eps, float c1, float c2)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// wf[tap][co][ci] = W, wb[tap][ci][co] = W[26 - tap][co][ci]
__global__ void k_pack(const float *W, int CO, int CI, bf16 *wf, bf16 *wb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NTAP * CO * CI) return;
    const int tap = i / (CO * CI), r = i % (CO * CI), co = r / CI, ci = r % CI;
    const bf16 v = __float2bfloat16_rn(W[i]);
    wf[i] = v;
    wb[((size_t)(NTAP - 1 - tap) * CI + ci) * CO + co] = v;
}

__global__ void k_f32_to_bf16(const float *a, bf16 *b, size_t n)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = __float2bfloat16_rn(a[i]);
}

template <int CIN, int COUT>
size_t conv_smem(const NetGeom &g)
{
    return ((size_t)NTAP * COUT * (CIN + 8) + (size_t)3 * (g.R + 2) * (g.nx + 2) * (CIN + 8)) * sizeof(bf16);
}

template <int CI, int CO>
size_t wgrad_smem(const NetGeom &g)
{
    return ((size_t)3 * (g.R + 2) * (g.nx + 2) * (CI + 8) + (size_t)TP * (CO + 8)) * sizeof(bf16);
}

template <int CIN, int COUT, int EPI, int MT, int KS>
int run_conv_mt(vec_net *N, const NetGeom &gt, const bf16 *x, const bf16 *wt, const float *bias, bf16 *o_pre,
                bf16 *o_act, float *o_f32, int cout_real, const bf16 *gate)
{
    const size_t sm = conv_smem<CIN, COUT>(gt);
    static bool set = false;
    if (!set) {
        CUDA_TRY(cudaFuncSetAttribute(k_conv<CIN, COUT, EPI, MT, KS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      200 * 1024));
        set = true;
    }
    long long grid = N->num_sms;
    if (grid > gt.tiles) grid = gt.tiles;
    k_conv<CIN, COUT, EPI, MT, KS><<<(int)grid, 256 * KS, sm, N->stream>>>(x, wt, bias, gt, o_pre, o_act, o_f32,
                                                                           cout_real, gate);
    N->launches++;
    CUDA_TRY(cudaGetLastError());
    return VEC_OK;
}

// CTA tiles of 256 points (two m-tiles per warp) where the plane divides
// into them and their halo fits, else 128
template <int CIN, int COUT, int EPI>
int run_conv_tc(vec_net *N, const bf16 *x, const bf16 *wt, const float *bias, bf16 *o_pre, bf16 *o_act, float *o_f32,
                int cout_real, const bf16 *gate)
{
    constexpr size_t sm = tc_smem_bytes<CIN, COUT>();
    static bool set = false;
    if (!set) {
        CUDA_TRY(cudaFuncSetAttribute(k_conv_tc<CIN, COUT, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        set = true;
    }
    // x as (8 channels, channel block, x, y, z and sample): boxes of 8 x 1 x 128 x 1 x 1
    PFN_cuTensorMapEncodeTiled_v12000 enc = (PFN_cuTensorMapEncodeTiled_v12000)tma_encode_fn();
    if (!enc) return VEC_ERR_CUDA;
    CUtensorMap tm;
    const NetGeom &g = N->g;
    cuuint64_t dims[5] = { 8, (cuuint64_t)(CIN / 8), (cuuint64_t)g.nx, (cuuint64_t)g.ny,
                           (cuuint64_t)g.nz * (cuuint64_t)g.nb };
    cuuint64_t strides[4] = { 16, (cuuint64_t)CIN * 2, (cuuint64_t)g.nx * CIN * 2, (cuuint64_t)g.ny * g.nx * CIN * 2 };
    cuuint32_t box[5] = { 8, 1, 128, 1, 1 };
    cuuint32_t es[5] = { 1, 1, 1, 1, 1 };
    CUresult r = enc(&tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, (void *)x, dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        vec_set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return VEC_ERR_CUDA;
    }
    long long grid = N->num_sms;
    if (grid > g.tiles) grid = g.tiles;
    k_conv_tc<CIN, COUT, EPI><<<(int)grid, TC_THREADS, sm, N->stream>>>(x, tm, wt, bias, g, o_pre, o_act, o_f32,
                                                                        cout_real, gate, N->err);
    N->launches++;
    CUDA_TRY(cudaGetLastError());
    return VEC_OK;
}

template <int CIN, int COUT, int EPI>
int run_conv(vec_net *N, const bf16 *x, const bf16 *wt, const float *bias, bf16 *o_pre, bf16 *o_act, float *o_f32,
             int cout_real, const bf16 *gate)
{
    if (N->conv_tc && N->g.nx == 128)
        return run_conv_tc<CIN, COUT, EPI>(N, x, wt, bias, o_pre, o_act, o_f32, cout_real, gate);
    NetGeom g2 = N->g;
    g2.R = 2 * TP / g2.nx;
    g2.tiles = (long long)g2.nb * g2.nz * (g2.nx * g2.ny / (2 * TP));
    if (N->conv_mt == 2 && (g2.nx * g2.ny) % (2 * TP) == 0 && conv_smem<CIN, COUT>(g2) <= 200 * 1024) {
        // two warp groups split the taps when the halo holds one group's partials
        const size_t halo = (size_t)3 * (g2.R + 2) * (g2.nx + 2) * (CIN + 8) * sizeof(bf16);
        if (halo >= (size_t)8 * 2 * (COUT / 8) * 128 * sizeof(float))
            return run_conv_mt<CIN, COUT, EPI, 2, 2>(N, g2, x, wt, bias, o_pre, o_act, o_f32, cout_real, gate);
        return run_conv_mt<CIN, COUT, EPI, 2, 1>(N, g2, x, wt, bias, o_pre, o_act, o_f32, cout_real, gate);
    }
    return run_conv_mt<CIN, COUT, EPI, 1, 1>(N, N->g, x, wt, bias, o_pre, o_act, o_f32, cout_real, gate);
}

// one warp per tap (27 warps) where its registers fit, else three taps per
// warp (9 warps)
template <int CI, int CO, int TPW>
int run_wgrad_t(vec_net *N, const bf16 *x, const bf16 *dy, float *gout)
{
    const size_t sm = wgrad_smem<CI, CO>(N->g);
    static bool set = false;
    if (!set) {
        CUDA_TRY(cudaFuncSetAttribute(k_wgrad<CI, CO, TPW>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        set = true;
    }
    long long grid = N->num_sms;
    if (grid > N->g.tiles) grid = N->g.tiles;
    k_wgrad<CI, CO, TPW><<<(int)grid, 32 * (NTAP / TPW), sm, N->stream>>>(x, dy, N->g, N->part);
    const int J = NTAP * CO * CI + CO;
    k_reduce_parts<<<(J + 255) / 256, 256, 0, N->stream>>>(N->part, (int)grid, J, gout);
    N->launches += 2;
    CUDA_TRY(cudaGetLastError());
    return VEC_OK;
}

template <int CI, int CO>
int run_wgrad(vec_net *N, const bf16 *x, const bf16 *dy, float *gout)
{
    if (N->conv_mt == 2) return run_wgrad_t<CI, CO, 1>(N, x, dy, gout);
    return run_wgrad_t<CI, CO, 3>(N, x, dy, gout);
}

// the layers: (cin, cout) = (16,32), (32,32), (32,32), (32,16)
const int LCI[4] = { 16, 32, 32, 32 };
const int LCO[4] = { 32, 32, 32, 16 };

uint64_t splitmix(uint64_t &s)
{
    uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

}  // namespace

// ---- internal API (used by the closure coupling) ------------------------------------
int net_pack(vec_net *N)
{
    for (int l = 0; l < 4; l++) {
        const int n = NTAP * LCO[l] * LCI[l];
        k_pack<<<(n + 255) / 256, 256, 0, N->stream>>>(N->p + N->off_w[l], LCO[l], LCI[l], N->wf[l], N->wb[l]);
        N->launches++;
    }
    CUDA_TRY(cudaGetLastError());
    return VEC_OK;
}

// x0 (BF16, [P][16]) -> out (FP32, [P][cout_real])
int net_forward(vec_net *N)
{
    int st;
    float *p = N->p;
    if ((st = run_conv<16, 32, EPI_ACT>(N, N->x0, N->wf[0], p + N->off_b[0], N->pre[0], N->act[0], nullptr, 0, nullptr)))
        return st;
    if ((st = run_conv<32, 32, EPI_ACT>(N, N->act[0], N->wf[1], p + N->off_b[1], N->pre[1], N->act[1], nullptr, 0, nullptr)))
        return st;
    if ((st = run_conv<32, 32, EPI_ACT>(N, N->act[1], N->wf[2], p + N->off_b[2], N->pre[2], N->act[2], nullptr, 0, nullptr)))
        return st;
    return run_conv<32, 16, EPI_OUT>(N, N->act[2], N->wf[3], p + N->off_b[3], nullptr, nullptr, N->out, N->cout_real,
                                     nullptr);
}

// after net_forward: loss against tgt ([P][cout_real] FP32) and all gradients
int net_backward(vec_net *N, const float *tgt)
{
    int st;
    CUDA_TRY(cudaMemsetAsync(N->loss_d, 0, sizeof(double), N->stream));
    const size_t P = (size_t)N->g.nb * N->npts;
    k_mse<<<N->num_sms * 4, 256, 0, N->stream>>>(N->out, tgt, P, N->cout_real, N->dout, N->loss_d);
    N->launches++;
    CUDA_TRY(cudaGetLastError());
    float *g = N->gr;
    // layer 4: dW from act3 and dout; dX3 -> gate with pre3
    if ((st = run_wgrad<32, 16>(N, N->act[2], N->dout, g + N->off_w[3]))) return st;
    if ((st = run_conv<16, 32, EPI_GATE>(N, N->dout, N->wb[3], nullptr, nullptr, N->d[0], nullptr, 0, N->pre[2])))
        return st;
    if ((st = run_wgrad<32, 32>(N, N->act[1], N->d[0], g + N->off_w[2]))) return st;
    if ((st = run_conv<32, 32, EPI_GATE>(N, N->d[0], N->wb[2], nullptr, nullptr, N->d[1], nullptr, 0, N->pre[1])))
        return st;
    if ((st = run_wgrad<32, 32>(N, N->act[0], N->d[1], g + N->off_w[1]))) return st;
    if ((st = run_conv<32, 32, EPI_GATE>(N, N->d[1], N->wb[1], nullptr, nullptr, N->d[0], nullptr, 0, N->pre[0])))
        return st;
    return run_wgrad<16, 32>(N, N->x0, N->d[0], g + N->off_w[0]);
}

int net_adam(vec_net *N, float lr)
{
    N->step += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - powf(b1, (float)N->step), c2 = 1.0f - powf(b2, (float)N->step);
    k_adam<<<(unsigned)((N->nparam + 255) / 256), 256, 0, N->stream>>>(N->p, N->gr, N->m, N->v, N->nparam, lr, b1, b2,
                                                                     1e-8f, c1, c2);
    N->launches++;
    CUDA_TRY(cudaGetLastError());
    return net_pack(N);
}

// ---- C-ABI ---------------------------------------------------------------------------
static int nalloc(void **p, size_t bytes)
{
    if (cudaMalloc(p, bytes ? bytes : 16) != cudaSuccess) {
        cudaGetLastError();
        vec_set_error("cudaMalloc of %zu bytes failed", bytes);
        return VEC_ERR_ALLOC;
    }
    return cudaMemset(*p, 0, bytes ? bytes : 16) == cudaSuccess ? VEC_OK : VEC_ERR_CUDA;
}

extern "C" int vec_net_destroy(vec_net *N)
{
    if (!N) return VEC_OK;
    if (N->stream) cudaStreamSynchronize(N->stream);
    void *ps[] = { N->p, N->gr, N->m, N->v, N->x0, N->dout, N->out, N->tgt, N->part, N->loss_d, N->xin, N->err };
    for (void *q : ps) if (q) cudaFree(q);
    for (int l = 0; l < 4; l++) { if (N->wf[l]) cudaFree(N->wf[l]); if (N->wb[l]) cudaFree(N->wb[l]); }
    for (int l = 0; l < 3; l++) { if (N->pre[l]) cudaFree(N->pre[l]); if (N->act[l]) cudaFree(N->act[l]); }
    for (int l = 0; l < 2; l++) if (N->d[l]) cudaFree(N->d[l]);
    if (N->stream && N->own_stream) cudaStreamDestroy(N->stream);
    delete N;
    return VEC_OK;
}

extern "C" int vec_net_create(int nx, int ny, int nz, int batch, unsigned long long seed, vec_net **out)
{
    if (!out) return VEC_ERR_ARG;
    *out = nullptr;
    if (!(nx == 16 || nx == 32 || nx == 64 || nx == 128) || ny < 2 || (nx * ny) % TP != 0 || nz < 1 || batch < 1) {
        vec_set_error("closure network: nx must be 16, 32, 64 or 128 and nx*ny a multiple of %d", TP);
        return VEC_ERR_SIZE;
    }
    vec_net *N = new vec_net();
    N->g.nx = nx; N->g.ny = ny; N->g.nz = nz; N->g.nb = batch;
    N->g.R = TP / nx;
    N->g.tiles = (long long)batch * nz * (nx * ny / TP);
    N->npts = (size_t)nx * ny * nz;
    N->cout_real = 8;
    {
        const char *e = getenv("VEC_NET_MT");
        N->conv_mt = (e && e[0] == '1') ? 1 : 2;
        const char *t = getenv("VEC_NET_TC");
        N->conv_tc = (t && t[0] == '0') ? 0 : 1;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&N->num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaStreamCreateWithFlags(&N->stream, cudaStreamNonBlocking) != cudaSuccess) { delete N; return VEC_ERR_CUDA; }
    N->own_stream = 1;
    size_t off = 0;
    for (int l = 0; l < 4; l++) {
        N->off_w[l] = off; off += (size_t)NTAP * LCO[l] * LCI[l];
        N->off_b[l] = off; off += LCO[l];
    }
    N->nparam = off;
    const size_t P = (size_t)batch * N->npts;
    int st = 0;
#define NA(ptr, bytes) do { if (!st) st = nalloc((void **)&(ptr), (bytes)); } while (0)
    NA(N->p, off * 4); NA(N->gr, off * 4); NA(N->m, off * 4); NA(N->v, off * 4);
    for (int l = 0; l < 4; l++) {
        NA(N->wf[l], (size_t)NTAP * LCO[l] * LCI[l] * 2);
        NA(N->wb[l], (size_t)NTAP * LCO[l] * LCI[l] * 2);
    }
    NA(N->x0, P * 16 * 2);
    for (int l = 0; l < 3; l++) { NA(N->pre[l], P * 32 * 2); NA(N->act[l], P * 32 * 2); }
    for (int l = 0; l < 2; l++) NA(N->d[l], P * 32 * 2);
    NA(N->dout, P * 16 * 2);
    NA(N->out, P * 8 * 4);
    NA(N->tgt, P * 8 * 4);
    NA(N->xin, P * 16 * 4);
    NA(N->part, (size_t)N->num_sms * (NTAP * 32 * 32 + 32) * 4);
    NA(N->loss_d, 8);
    NA(N->err, 16);
#undef NA
    if (st) { vec_net_destroy(N); return st; }
    // initial weights: uniform(-a, a), a = sqrt(6 / fan_in) (He); the output
    // layer scaled by 0.1; padded input / output channels zero; biases zero
    std::vector<float> h(off, 0.0f);
    uint64_t s = seed * 0x2545F4914F6CDD1DULL + 12345;
    const int creal_in[4] = { 9, 32, 32, 32 }, creal_out[4] = { 32, 32, 32, 8 };
    for (int l = 0; l < 4; l++) {
        const double a = sqrt(6.0 / (NTAP * creal_in[l])) * (l == 3 ? 0.1 : 1.0);
        for (int tap = 0; tap < NTAP; tap++)
            for (int co = 0; co < LCO[l]; co++)
                for (int ci = 0; ci < LCI[l]; ci++) {
                    const double u = (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
                    const bool real = co < creal_out[l] && ci < creal_in[l];
                    h[N->off_w[l] + ((size_t)tap * LCO[l] + co) * LCI[l] + ci] = real ? (float)((2.0 * u - 1.0) * a) : 0.0f;
                }
    }
    if (cudaMemcpy(N->p, h.data(), off * 4, cudaMemcpyHostToDevice) != cudaSuccess || net_pack(N) ||
        cudaStreamSynchronize(N->stream) != cudaSuccess) {
        vec_net_destroy(N);
        return VEC_ERR_CUDA;
    }
    *out = N;
    return VEC_OK;
}

extern "C" long long vec_net_nparams(vec_net *N) { return N ? (long long)N->nparam : 0; }

extern "C" int vec_net_get_params(vec_net *N, float *host)
{
    if (!N || !host) return VEC_ERR_ARG;
    CUDA_TRY(cudaMemcpyAsync(host, N->p, N->nparam * 4, cudaMemcpyDeviceToHost, N->stream));
    CUDA_TRY(cudaStreamSynchronize(N->stream));
    return VEC_OK;
}

extern "C" int vec_net_set_params(vec_net *N, const float *host)
{
    if (!N || !host) return VEC_ERR_ARG;
    CUDA_TRY(cudaMemcpyAsync(N->p, host, N->nparam * 4, cudaMemcpyHostToDevice, N->stream));
    CUDA_TRY(cudaMemsetAsync(N->m, 0, N->nparam * 4, N->stream));
    CUDA_TRY(cudaMemsetAsync(N->v, 0, N->nparam * 4, N->stream));
    N->step = 0;
    int st = net_pack(N);
    if (st) return st;
    CUDA_TRY(cudaStreamSynchronize(N->stream));
    return VEC_OK;
}

extern "C" int vec_net_get_grads(vec_net *N, float *host)
{
    if (!N || !host) return VEC_ERR_ARG;
    CUDA_TRY(cudaMemcpyAsync(host, N->gr, N->nparam * 4, cudaMemcpyDeviceToHost, N->stream));
    CUDA_TRY(cudaStreamSynchronize(N->stream));
    return VEC_OK;
}

// x: host [batch][nz][ny][nx][16] FP32 (rounded to BF16 on the device);
// out (optional): host [batch][nz][ny][nx][8] FP32
extern "C" int vec_net_forward(vec_net *N, const float *x, float *out)
{
    if (!N || !x) return VEC_ERR_ARG;
    const size_t n = (size_t)N->g.nb * N->npts * 16;
    CUDA_TRY(cudaMemcpyAsync(N->xin, x, n * 4, cudaMemcpyHostToDevice, N->stream));
    k_f32_to_bf16<<<(unsigned)((n + 255) / 256), 256, 0, N->stream>>>(N->xin, N->x0, n);
    N->launches++;
    int st = net_forward(N);
    if (st) return st;
    if (out)
        CUDA_TRY(cudaMemcpyAsync(out, N->out, (size_t)N->g.nb * N->npts * 8 * 4, cudaMemcpyDeviceToHost, N->stream));
    CUDA_TRY(cudaStreamSynchronize(N->stream));
    return VEC_OK;
}

// after vec_net_forward: MSE against tgt (host [batch][...][8]) and the
// gradients of every parameter
extern "C" int vec_net_backward(vec_net *N, const float *tgt, double *loss)
{
    if (!N || !tgt) return VEC_ERR_ARG;
    CUDA_TRY(cudaMemcpyAsync(N->tgt, tgt, (size_t)N->g.nb * N->npts * 8 * 4, cudaMemcpyHostToDevice, N->stream));
    int st = net_backward(N, N->tgt);
    if (st) return st;
    if (loss) CUDA_TRY(cudaMemcpyAsync(loss, N->loss_d, 8, cudaMemcpyDeviceToHost, N->stream));
    CUDA_TRY(cudaStreamSynchronize(N->stream));
    return VEC_OK;
}

extern "C" int vec_net_adam(vec_net *N, float lr)
{
    if (!N) return VEC_ERR_ARG;
    int st = net_adam(N, lr);
    if (st) return st;
    CUDA_TRY(cudaStreamSynchronize(N->stream));
    return VEC_OK;
}

// device time of `reps` forward passes and of `reps` training steps (forward,
// backward, Adam with rate 0: the parameters stay, the moments move) on the
// current batch buffers, CUDA events on the network stream; flops_*: the
// floating-point operations executed per pass (padded channels included)
extern "C" int vec_net_time(vec_net *N, int reps, float *ms_fwd, float *ms_train, double *flops_fwd,
                            double *flops_train)
{
    if (!N || reps <= 0) return VEC_ERR_ARG;
    cudaEvent_t a, b, c;
    CUDA_TRY(cudaEventCreate(&a));
    CUDA_TRY(cudaEventCreate(&b));
    CUDA_TRY(cudaEventCreate(&c));
    int st = net_forward(N);   // warm-up
    if (!st) {
        cudaEventRecord(a, N->stream);
        for (int i = 0; i < reps && !st; i++) st = net_forward(N);
        cudaEventRecord(b, N->stream);
        for (int i = 0; i < reps && !st; i++) {
            if ((st = net_forward(N))) break;
            if ((st = net_backward(N, N->tgt))) break;
            st = net_adam(N, 0.0f);
        }
        cudaEventRecord(c, N->stream);
        cudaEventSynchronize(c);
    }
    float t1 = 0, t2 = 0;
    if (!st) {
        cudaEventElapsedTime(&t1, a, b);
        cudaEventElapsedTime(&t2, b, c);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaEventDestroy(c);
    if (st) return st;
    const double P = (double)N->g.nb * (double)N->npts;
    double fwd = 0.0, dg = 0.0;
    for (int l = 0; l < 4; l++) {
        const double f = 2.0 * NTAP * LCI[l] * LCO[l] * P;
        fwd += f;
        if (l > 0) dg += f;
    }
    if (ms_fwd) *ms_fwd = t1 / reps;
    if (ms_train) *ms_train = t2 / reps;
    if (flops_fwd) *flops_fwd = fwd;
    if (flops_train) *flops_train = 2.0 * fwd + dg;   // forward + weight gradients + input gradients
    return VEC_OK;
}

// kernels launched by the network since creation
extern "C" long long vec_net_launch_count(vec_net *N) { return N ? N->launches : 0; }
