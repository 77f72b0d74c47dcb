// lines_ct.cu -- horizontal spectral operators (src/fft.F90) for line
// lengths n = N1*N2 = 2^a or 3*2^a (64..1024), the hot path of the time step.
//
// Per tile a CTA owns 2S real lines of one z-plane (S complex sequences
// z = a + ib).  The tile is brought into shared memory by TMA bulk copies
// (cp.async.bulk + mbarrier): one copy for 2S contiguous x rows, or one
// 2S-wide copy per row for y columns.  CTAs are persistent over tiles and the
// next tile is prefetched into the second buffer while the current one is
// transformed.
//
// Each length-n FFT is a two-level four-step decomposition held in
// registers: n = N1*N2, m = N2*m1 + m2, k = k1 + N1*k2.  Thread m2 does an
// N1-point DFT over m1 (itself a four-step of radix-2/4/8 kernels), applies
// the twiddle W_n^(m2 k1) and hands its results to thread k1 through one
// padded, bank-conflict-free shared-memory exchange; thread k1 then does the
// N2-point DFT over m2 and holds X[k1 + N1 k2] for all k2.  The spectral
// operator (+ik, -k^2, 2/3 truncation, all Hermitian-symmetric multipliers)
// is applied in registers and the inverse runs the same two levels in the
// opposite order, so each transform costs one exchange.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "common.cuh"
#include "engine.h"
#include "tma.cuh"

template <typename R> struct JobPackCT { LineJob<R> j[MAX_JOBS]; };
// one TMA descriptor per job input (y lines: 3-D view nx x ny x nz)
struct TmapPack { CUtensorMap m[MAX_JOBS]; };

// W_32^q = exp(-2 pi i q/32), q = 0..31, and W_96^q (the in-register radix
// kernels; radix-3 factors take their twiddles from the second table)
__constant__ float2 c_tw32f[32];
__constant__ double2 c_tw32d[32];
__constant__ float2 c_tw96f[96];
__constant__ double2 c_tw96d[96];

template <typename C> __device__ __forceinline__ C tw32(int q);
template <> __device__ __forceinline__ float2 tw32<float2>(int q) { return c_tw32f[q]; }
template <> __device__ __forceinline__ double2 tw32<double2>(int q) { return c_tw32d[q]; }
template <typename C> __device__ __forceinline__ C tw96(int q);
template <> __device__ __forceinline__ float2 tw96<float2>(int q) { return c_tw96f[q]; }
template <> __device__ __forceinline__ double2 tw96<double2>(int q) { return c_tw96d[q]; }

// x mod N for x >= 0 (N a compile-time constant)
template <int N> __device__ __forceinline__ int modn(int x) { return (N & (N - 1)) == 0 ? (x & (N - 1)) : x % N; }

template <typename C>
__device__ __forceinline__ C cmul_(C a, C b) { C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r; }
template <typename C>
__device__ __forceinline__ C cadd_(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C>
__device__ __forceinline__ C csub_(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <bool INV, typename C>
__device__ __forceinline__ C rot_(C a) { C r; if (INV) { r.x = -a.y; r.y = a.x; } else { r.x = a.y; r.y = -a.x; } return r; }

// multiply by W_N^e (e compile-time after unrolling); conjugate for INV
template <int N, bool INV, typename C>
__device__ __forceinline__ C twc(C a, int e)
{
    if constexpr (32 % N == 0) {
        const int q = (e * (32 / N)) & 31;
        if (q == 0) return a;
        if (q == 8) return rot_<INV>(a);                           // -i (fwd)
        if (q == 16) { C r; r.x = -a.x; r.y = -a.y; return r; }
        if (q == 24) return rot_<!INV>(a);                         // +i (fwd)
        C w = tw32<C>(q);
        if (INV) w.y = -w.y;
        return cmul_(a, w);
    } else {
        static_assert(96 % N == 0, "radix kernels cover divisors of 32 and 96");
        const int q = (e * (96 / N)) % 96;
        if (q == 0) return a;
        if (q == 24) return rot_<INV>(a);
        if (q == 48) { C r; r.x = -a.x; r.y = -a.y; return r; }
        if (q == 72) return rot_<!INV>(a);
        C w = tw96<C>(q);
        if (INV) w.y = -w.y;
        return cmul_(a, w);
    }
}

// in-register natural-order DFT of N points
template <int N, bool INV> struct RDft;
template <bool INV> struct RDft<1, INV> { template <typename C> static __device__ __forceinline__ void run(C *) {} };
template <bool INV> struct RDft<2, INV> {
    template <typename C> static __device__ __forceinline__ void run(C *v) { C a = v[0], b = v[1]; v[0] = cadd_(a, b); v[1] = csub_(a, b); }
};
// X1,2 = a - (b+c)/2 -+ i (sqrt(3)/2)(b-c) (forward; conjugate for INV)
template <bool INV> struct RDft<3, INV> {
    template <typename C> static __device__ __forceinline__ void run(C *v) {
        using R = decltype(v[0].x);
        const R h = (R)0.8660254037844386;
        C t1 = cadd_(v[1], v[2]), d = csub_(v[1], v[2]);
        C t2; t2.x = v[0].x - (R)0.5 * t1.x; t2.y = v[0].y - (R)0.5 * t1.y;
        C r = rot_<INV>(d);
        r.x *= h; r.y *= h;
        v[0] = cadd_(v[0], t1);
        v[1] = cadd_(t2, r);
        v[2] = csub_(t2, r);
    }
};
template <bool INV> struct RDft<4, INV> {
    template <typename C> static __device__ __forceinline__ void run(C *v) {
        C a0 = cadd_(v[0], v[2]), a1 = csub_(v[0], v[2]);
        C b0 = cadd_(v[1], v[3]), b1 = rot_<INV>(csub_(v[1], v[3]));
        v[0] = cadd_(a0, b0); v[1] = cadd_(a1, b1); v[2] = csub_(a0, b0); v[3] = csub_(a1, b1);
    }
};
// four-step in registers: N = A*B, m = B*m1 + m2, k = k1 + A*k2
template <int A, int B, bool INV, typename C>
__device__ __forceinline__ void reg_ct(C *v)
{
    constexpr int N = A * B;
    C t[N];
#pragma unroll
    for (int m2 = 0; m2 < B; m2++) {
        C a[A];
#pragma unroll
        for (int m1 = 0; m1 < A; m1++) a[m1] = v[B * m1 + m2];
        RDft<A, INV>::run(a);
#pragma unroll
        for (int k1 = 0; k1 < A; k1++) t[m2 * A + k1] = twc<N, INV>(a[k1], m2 * k1);
    }
#pragma unroll
    for (int k1 = 0; k1 < A; k1++) {
        C b[B];
#pragma unroll
        for (int m2 = 0; m2 < B; m2++) b[m2] = t[m2 * A + k1];
        RDft<B, INV>::run(b);
#pragma unroll
        for (int k2 = 0; k2 < B; k2++) v[k1 + A * k2] = b[k2];
    }
}
template <bool INV> struct RDft<8, INV> { template <typename C> static __device__ __forceinline__ void run(C *v) { reg_ct<2, 4, INV>(v); } };
template <bool INV> struct RDft<16, INV> { template <typename C> static __device__ __forceinline__ void run(C *v) { reg_ct<4, 4, INV>(v); } };
template <bool INV> struct RDft<32, INV> { template <typename C> static __device__ __forceinline__ void run(C *v) { reg_ct<8, 4, INV>(v); } };
template <bool INV> struct RDft<6, INV> { template <typename C> static __device__ __forceinline__ void run(C *v) { reg_ct<3, 2, INV>(v); } };
template <bool INV> struct RDft<12, INV> { template <typename C> static __device__ __forceinline__ void run(C *v) { reg_ct<4, 3, INV>(v); } };
template <bool INV> struct RDft<24, INV> { template <typename C> static __device__ __forceinline__ void run(C *v) { reg_ct<8, 3, INV>(v); } };

// ---- TMA helpers (tma.cuh) and the 3-D tiled load of the y tiles -------------------
// 3-D tiled TMA load of one box (c0 innermost) into shared memory
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1, int c2, uint64_t *bar)
{
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
                 ::"r"(smem_u32(dst)), "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar)) : "memory");
}
// rows per TMA box of a y tile: TMA boxes are at most 256 rows, and the box
// must divide the line length
__host__ __device__ constexpr int ybox_rows(int n) { return n <= 256 ? n : (n % 256 == 0 ? 256 : n / 2); }

// ---- the kernel --------------------------------------------------------------------
// DIR 0: x lines (a tile = 2S contiguous rows), DIR 1: y lines (a tile = 2S
// adjacent columns over all ny rows).
//
// WS (x lines with NP dividing 32): the NP threads of a sequence sit in one
// warp, so the exchanges need only warp barriers.  The warps then run
// through their tiles independently; an "empty" mbarrier per tile buffer
// (one arrival per warp once it has read the tile) tells the thread that
// issues the TMA copies when a buffer may be refilled.
// Per-sequence stride of the exchange rows, in complex elements.  The
// forward exchange holds N1 rows of N2 + 1, the inverse one N2 rows of
// N1 + 1, the spectra's separation N + N/32 padded elements: the stride
// covers the largest.  A shared-memory wavefront serves U = 128 /
// sizeof(complex) consecutive elements.  x lines: the threads of a
// half-warp (quarter-warp in FP64) belong to one or two sequences, and a
// stride of 1 mod 16 keeps them on distinct banks.  y lines: thread tid is
// lane tid / S of sequence tid % S, so a wavefront's threads are G = U / S
// lanes of U / G sequences; a stride of G mod U puts them on distinct banks
// (exchange element sidx * stride + lane * 1 or lane * (odd row) + const).
template <typename R, int DIR, int N1, int N2, int S>
__host__ __device__ constexpr int ct_lds()
{
    constexpr int U = 128 / (2 * (int)sizeof(R));
    constexpr int G = U / S > 1 ? U / S : 1;
    constexpr int MF = N1 * (N2 + 1), MI = N2 * (N1 + 1), MS = N1 * N2 + (N1 * N2) / 32 + 1;
    constexpr int M = MF > MI ? (MF > MS ? MF : MS) : (MI > MS ? MI : MS);
    return DIR == 0 ? ((M + 15) / 16) * 16 + 1 : ((M + U - 1) / U) * U + G;
}

// dynamic shared memory of one CTA: two tile buffers, the exchange rows,
// the twiddle table(s) and the three multiplier tables
template <typename R, int DIR, int N1, int N2, int S>
__host__ __device__ constexpr size_t ct_smem_bytes()
{
    constexpr int N = N1 * N2;
    constexpr int LDS = ct_lds<R, DIR, N1, N2, S>();
    return 2 * (size_t)(2 * S * N) * sizeof(R) + ((size_t)S * LDS + (sizeof(R) == 4 ? 2 : 1) * (size_t)N) * 2 * sizeof(R)
           + 3 * (size_t)N * sizeof(R);
}
// two CTAs per SM where their shared memory fits (227 KB per SM), else one
// CTA with the whole register file
template <typename R, int DIR, int N1, int N2, int S>
__host__ __device__ constexpr int ct_min_blocks()
{
    return (S * (N1 > N2 ? N1 : N2) <= 256 && 2 * ct_smem_bytes<R, DIR, N1, N2, S>() <= 232448) ? 2 : 1;
}

template <typename R, int DIR, int N1, int N2, int S, bool WSYNC>
__global__ void __launch_bounds__(S * (N1 > N2 ? N1 : N2), (ct_min_blocks<R, DIR, N1, N2, S>()))
line_ct(JobPackCT<R> jobs, const __grid_constant__ TmapPack tmaps, LineTables<R> tb, int nx, int ny, int nz,
        int tpp, int total, int *err)
{
    PDL_WAIT();
    using C = typename CT<R>::T;
    constexpr int N = N1 * N2;
    constexpr int NP = N1 > N2 ? N1 : N2;
    constexpr int NT = S * NP;
    constexpr int TILE = 2 * S * N;                   // reals per tile
    constexpr int LXF = N2 + 1;                       // padded exchange rows: forward,
    constexpr int LXI = N1 + 1;                       // inverse
    constexpr int LDS = ct_lds<R, DIR, N1, N2, S>();  // per-sequence exchange stride
    constexpr bool WS = WSYNC && DIR == 0 && (32 % NP == 0) && NT % 32 == 0;

    extern __shared__ __align__(128) unsigned char smem[];
    R *tile0 = reinterpret_cast<R *>(smem);
    R *tile1 = tile0 + TILE;
    C *ex = reinterpret_cast<C *>(tile1 + TILE);
    // FP32: twiddles W_N^(m2 k1) as two N1 x N2 tables, one row per value of
    // the loop index, so that the 16 threads of a sequence read consecutive
    // entries (indexed by (m2 k1) mod N, a thread stride of k1 made up to
    // eight-way bank conflicts).  FP64: one table of N (the second would
    // cost the second CTA per SM).
    constexpr bool TW2 = sizeof(R) == 4;
    static_assert(!TW2 || (N1 % 4 == 0 && N2 % 4 == 0), "FP32 twiddles factor the index as 4 a + b");
    C *twf = ex + (size_t)S * LDS;                    // twf[k1 N2 + m2] (FP64: tw[e])
    C *twi = twf + N;                                 // twi[m2 N1 + k1]
    R *sm1 = reinterpret_cast<R *>(twi + (TW2 ? N : 0));   // spectral multipliers
    R *sm2 = sm1 + N;
    R *smda = sm2 + N;
    __shared__ __align__(8) uint64_t bar[4];          // full[2], empty[2]

    const int tid = threadIdx.x;
    const int sidx = DIR == 0 ? tid / NP : tid % S;
    const int lane = DIR == 0 ? tid % NP : tid / S;
    const size_t np = (size_t)nx * ny;
    auto sync = [&]() {
        if constexpr (WS) __syncwarp();
        else __syncthreads();
    };

    for (int e = tid; e < N; e += NT) {
        if constexpr (TW2) {
            const int k1 = e / N2, m2 = e - k1 * N2;
            twf[e] = tb.tw[modn<N>(m2 * k1)];
            const int m2i = e / N1, k1i = e - m2i * N1;
            twi[e] = tb.tw[modn<N>(m2i * k1i)];
        } else {
            twf[e] = tb.tw[e];
        }
        sm1[e] = tb.m1[e];
        sm2[e] = tb.m2[e];
        smda[e] = tb.mda[e];
    }
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init(&bar[2], NT / 32);
        mbar_init(&bar[3], NT / 32);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();

    auto issue = [&](int t, R *dst, uint64_t *b) {
        const int job = t / (nz * tpp);
        const int rem = t - job * (nz * tpp);
        const int plane = rem / tpp;
        const int l0 = (rem - plane * tpp) * 2 * S;
        const R *src = jobs.j[job].in + (size_t)plane * np;
        if (DIR == 0) {
            if (tid == 0) {
                mbar_expect_tx(b, TILE * (unsigned)sizeof(R));
                tma_load(dst, src + (size_t)l0 * nx, TILE * (unsigned)sizeof(R), b);
            }
        } else if (tid == 0) {
            // boxes of 2S columns x (up to 256) rows of this plane
            constexpr int BR = ybox_rows(N);
            mbar_expect_tx(b, TILE * (unsigned)sizeof(R));
#pragma unroll
            for (int c = 0; c < N / BR; c++)
                tma_load_3d(dst + (size_t)c * BR * 2 * S, &tmaps.m[job], l0, c * BR, plane, b);
            (void)src;
        }
    };

    if (blockIdx.x < total) issue(blockIdx.x, tile0, &bar[0]);
    int it = 0;
    for (int t = blockIdx.x; t < total; t += gridDim.x, it++) {
        R *cur = (it & 1) ? tile1 : tile0;
        R *nxt = (it & 1) ? tile0 : tile1;
        bool issued_next = false;
        if (t + (int)gridDim.x < total) {
            if (WS && it >= 1 && tid == 0) {
                // every warp has read buffer nxt (its use in iteration it - 1)
                if (!mbar_wait(&bar[2 + ((it + 1) & 1)], ((it - 1) >> 1) & 1)) {
                    // report, then let this tile's copy (still in flight)
                    // land before the CTA's shared memory is released
                    atomicExch(err, 1);
                    mbar_wait(&bar[it & 1], (it >> 1) & 1);
                    return;
                }
            }
            if (tid == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(t + gridDim.x, nxt, &bar[(it + 1) & 1]);
            issued_next = true;
        }
        if (!mbar_wait(&bar[it & 1], (it >> 1) & 1)) {
            if (tid == 0) {
                // report, then wait (bounded) for the copies this CTA issued
                atomicExch(err, 1);
                mbar_wait(&bar[it & 1], (it >> 1) & 1);
                if (issued_next) mbar_wait(&bar[(it + 1) & 1], ((it + 1) >> 1) & 1);
            }
            return;
        }
        const int job = t / (nz * tpp);
        const int rem = t - job * (nz * tpp);
        const int plane = rem / tpp;
        const int l0 = (rem - plane * tpp) * 2 * S;
        const LineJob<R> &jb = jobs.j[job];
        const size_t pbase = (size_t)plane * np;
        const int op1 = jb.op1, op2 = jb.op2;
        C *ex_s = ex + (size_t)sidx * LDS;

        // element e of sequence sidx in the tile
        auto tile_z = [&](int e) -> C {
            C z;
            if (DIR == 0) { z.x = cur[(2 * sidx) * N + e]; z.y = cur[(2 * sidx + 1) * N + e]; }
            else { z = reinterpret_cast<const C *>(cur)[(size_t)e * S + sidx]; }
            return z;
        };

        // The two sequences a warp holds (x lines, 16 threads each) have rows
        // that start on the same bank; the odd one reads its columns in pairs
        // swapped (index ^ 1), so that the two half-warps hit different banks,
        // and swaps the registers back.  The values are the same.
        constexpr bool XSW = WS && DIR == 0 && NP == 16 && sizeof(R) == 4 && N1 % 2 == 0 && N2 % 2 == 0;
        const int sw = XSW ? (sidx & 1) : 0;
        auto unswap = [&](C *v, int n) {
            if constexpr (XSW) {
#pragma unroll
                for (int i = 0; i < n; i += 2) {
                    const C t0 = v[i], t1 = v[i + 1];
                    v[i] = sw ? t1 : t0;
                    v[i + 1] = sw ? t0 : t1;
                }
            }
        };

        C X[N2];   // thread lane = k1 holds X[k1 + N1 k2], k2 = 0..N2-1
        if (op1 != OP_INV) {
            // forward, first level: thread m2 = lane, N1-point DFT over m1
            if (lane < N2) {
                C a[N1];
#pragma unroll
                for (int m1 = 0; m1 < N1; m1++) a[m1] = tile_z(N2 * (m1 ^ sw) + lane);
                unswap(a, N1);
                RDft<N1, false>::run(a);
                // FP32: W^(lane k1) = W^(lane 4 (k1 / 4)) W^(lane (k1 % 4)): 3 + N1/4 - 1
                // table reads instead of N1 - 1, one product more per twiddle
                C lo[4], hi[N1 / 4];
                if constexpr (TW2) {
#pragma unroll
                    for (int j = 1; j < 4; j++) lo[j] = twf[j * N2 + lane];
#pragma unroll
                    for (int j = 1; j < N1 / 4; j++) hi[j] = twf[4 * j * N2 + lane];
                }
#pragma unroll
                for (int k1 = 0; k1 < N1; k1++) {
                    C w;
                    if constexpr (TW2) {
                        const int ja = k1 >> 2, jb = k1 & 3;
                        w = ja == 0 ? lo[jb] : (jb == 0 ? hi[ja] : cmul_(hi[ja], lo[jb]));
                    } else {
                        w = twf[modn<N>(lane * k1)];
                    }
                    ex_s[k1 * LXF + lane] = k1 == 0 ? a[k1] : cmul_(a[k1], w);
                }
            }
            sync();
            // second level: thread k1 = lane, N2-point DFT over m2
            if (lane < N1) {
#pragma unroll
                for (int m2 = 0; m2 < N2; m2++) X[m2] = ex_s[lane * LXF + m2];
                RDft<N2, false>::run(X);
            }
            sync();
        } else if (lane < N1) {
            // halfcomplex input lines a (re) and b (im): Z_k = A_k + i B_k
#pragma unroll
            for (int k2 = 0; k2 < N2; k2++) {
                const int k = lane + N1 * (k2 ^ sw);
                const int kk = k <= N / 2 ? k : N - k;
                const bool edge = kk == 0 || 2 * kk == N;
                C pa = tile_z(kk);                     // (ha[kk], hb[kk])
                C pb = edge ? C{0, 0} : tile_z(N - kk); // (ha[n-kk], hb[n-kk])
                R ar = pa.x, br = pa.y, ai = k <= N / 2 ? pb.x : -pb.x, bi = k <= N / 2 ? pb.y : -pb.y;
                X[k2].x = ar - bi;
                X[k2].y = ai + br;
            }
            unswap(X, N2);
        }
        if constexpr (WS) {
            // this warp is done with the tile buffer
            __syncwarp();
            if ((tid & 31) == 0) mbar_arrive(&bar[2 + (it & 1)]);
        }

        if (op1 == OP_FWD) {
            // separate Z into the halfcomplex spectra of the two real lines
            if (lane < N1) {
#pragma unroll
                for (int k2 = 0; k2 < N2; k2++) ex_s[lane + N1 * k2 + ((lane + N1 * k2) >> 5)] = X[k2];
            }
            sync();
            for (int p = lane; p < N; p += NP) {
                const int q = p == 0 ? 0 : N - p;
                C zp = ex_s[p + (p >> 5)], zq = ex_s[q + (q >> 5)];
                R va, vb;
                if (2 * p <= N) { va = (R)0.5 * (zp.x + zq.x); vb = (R)0.5 * (zp.y + zq.y); }
                else { va = (R)0.5 * (zq.y - zp.y); vb = (R)0.5 * (zp.x - zq.x); }
                const int la = l0 + 2 * sidx;
                const R ra = jb.alpha1 * va, rb = jb.alpha1 * vb;
                if (DIR == 0) {
                    R *oa = jb.out1 + pbase + (size_t)la * nx + p, *ob = oa + nx;
                    *oa = jb.acc1 ? *oa + ra : ra;
                    *ob = jb.acc1 ? *ob + rb : rb;
                } else {
                    // the two lines are adjacent columns: one vector store
                    C *o = reinterpret_cast<C *>(jb.out1 + pbase + (size_t)p * nx + la);
                    C v = { ra, rb };
                    if (jb.acc1) { const C q = *o; v.x += q.x; v.y += q.y; }
                    *o = v;
                }
            }
            sync();
            continue;
        }

        // one or two outputs: Y = m(X), inverse transform, store (a
        // halfcomplex input takes a second output only for OP_D1: the
        // derivative of its inverse)
        const int nout = (op2 != OP_NONE && (op1 != OP_INV || op2 == OP_D1)) ? 2 : 1;
        for (int o = 0; o < nout; o++) {
            const int op = o == 0 ? op1 : op2;
            R *out = o == 0 ? jb.out1 : jb.out2;
            const R alpha = o == 0 ? jb.alpha1 : jb.alpha2;
            const int acc = o == 0 ? jb.acc1 : jb.acc2;
            if (lane < N1) {
                C Y[N2];
#pragma unroll
                for (int k2 = 0; k2 < N2; k2++) {
                    const int k = lane + N1 * k2;
                    C z = X[k2], y;
                    if (op == OP_D1) { R m = sm1[k]; y.x = -m * z.y; y.y = m * z.x; }
                    else if (op == OP_INV) { y = z; }
                    else { R m = op == OP_D2 ? sm2[k] : smda[k]; y.x = m * z.x; y.y = m * z.y; }
                    Y[k2] = y;
                }
                // inverse, first level: thread k1 = lane, N2-point DFT over k2
                RDft<N2, true>::run(Y);
                // (FP32: the same factorisation of W^(m2 lane), m2 = 4 (m2 / 4) + m2 % 4)
                C lo[4], hi[N2 / 4];
                if constexpr (TW2) {
#pragma unroll
                    for (int j = 1; j < 4; j++) lo[j] = twi[j * N1 + lane];
#pragma unroll
                    for (int j = 1; j < N2 / 4; j++) hi[j] = twi[4 * j * N1 + lane];
                }
#pragma unroll
                for (int m2 = 0; m2 < N2; m2++) {
                    C w;
                    if constexpr (TW2) {
                        const int ja = m2 >> 2, jb = m2 & 3;
                        w = ja == 0 ? lo[jb] : (jb == 0 ? hi[ja] : cmul_(hi[ja], lo[jb]));
                    } else {
                        w = twf[modn<N>(m2 * lane)];
                    }
                    w.y = -w.y;
                    ex_s[m2 * LXI + lane] = m2 == 0 ? Y[m2] : cmul_(Y[m2], w);
                }
            }
            sync();
            // second level: thread m2 = lane, N1-point DFT over k1
            if (lane < N2) {
                C a[N1];
#pragma unroll
                for (int k1 = 0; k1 < N1; k1++) a[k1] = ex_s[lane * LXI + k1];
                RDft<N1, true>::run(a);
                const R sc = op == OP_INV ? (R)1 / (R)N : (R)1;
                const int la = l0 + 2 * sidx;
                R addv = (R)0;
                if (op == OP_INV && jb.addk) addv = (R)jb.addk[plane];
                if (op == OP_INV) addv = addv + (R)jb.addc;
#pragma unroll
                for (int m1 = 0; m1 < N1; m1++) {
                    const int e = lane + N2 * m1;
                    R va = alpha * (a[m1].x * sc), vb = alpha * (a[m1].y * sc);
                    if (DIR == 0) {
                        R *oa = out + pbase + (size_t)la * nx + e, *ob = oa + nx;
                        if (acc) { va = *oa + va; vb = *ob + vb; }
                        if (op == OP_INV) { va = va + addv; vb = vb + addv; }
                        *oa = va;
                        *ob = vb;
                    } else {
                        C *o = reinterpret_cast<C *>(out + pbase + (size_t)e * nx + la);
                        if (acc) { const C q = *o; va = q.x + va; vb = q.y + vb; }
                        if (op == OP_INV) { va = va + addv; vb = vb + addv; }
                        *o = C{ va, vb };
                    }
                }
            }
            sync();
        }
    }
}

// Self-test of the bounded-wait error path: one thread waits on an mbarrier
// that nothing arrives on, gives up after `polls` polls and raises the
// context's error flag exactly as the line kernel does when a tile load does
// not complete.  No copy is in flight, so nothing has to be drained.
__global__ void k_wait_selftest(long long polls, int *err)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x != 0) return;
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (!mbar_wait(&bar, 0, polls)) atomicExch(err, 2);
}

extern "C" int vec_selftest_wait(vec_ctx *c, long long polls)
{
    if (!c || polls < 1 || polls > MBAR_POLLS) return VEC_ERR_ARG;
    Engine &E = engine_of(c);
    k_wait_selftest<<<1, 32, 0, E.stream>>>(polls, E.dev_err);
    CUDA_TRY(cudaGetLastError());
    return VEC_OK;
}

// ---- host side ------------------------------------------------------------------------
int line_ct_configure()
{
    float2 tf[32];
    double2 td[32];
    for (int q = 0; q < 32; q++) {
        // exp(-2 pi i q/32) with exact quadrant values
        double a = 2.0 * M_PI * (double)q / 32.0;
        double c = cos(a), s = sin(a);
        if (q % 8 == 0) {
            c = (q == 0) ? 1.0 : (q == 16 ? -1.0 : 0.0);
            s = (q == 8) ? 1.0 : (q == 24 ? -1.0 : 0.0);
        }
        td[q].x = c; td[q].y = -s;
        tf[q].x = (float)c; tf[q].y = (float)(-s);
    }
    CUDA_TRY(cudaMemcpyToSymbol(c_tw32f, tf, sizeof(tf)));
    CUDA_TRY(cudaMemcpyToSymbol(c_tw32d, td, sizeof(td)));
    float2 uf[96];
    double2 ud[96];
    for (int q = 0; q < 96; q++) {
        double c, s;
        sincos2pi_host(q, 96, &c, &s);
        ud[q].x = c; ud[q].y = -s;
        uf[q].x = (float)c; uf[q].y = (float)(-s);
    }
    CUDA_TRY(cudaMemcpyToSymbol(c_tw96f, uf, sizeof(uf)));
    CUDA_TRY(cudaMemcpyToSymbol(c_tw96d, ud, sizeof(ud)));
    return VEC_OK;
}

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static int get_encoder();

// cuTensorMapEncodeTiled for other translation units (null if unavailable)
void *tma_encode_fn() { return get_encoder() == VEC_OK ? (void *)g_encode : nullptr; }

static int get_encoder()
{
    if (g_encode) return VEC_OK;
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
        cudaGetLastError();
        vec_set_error("cuTensorMapEncodeTiled not available");
        return VEC_ERR_CUDA;
    }
    g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    return VEC_OK;
}

// TMA descriptor of a (nx, ny, nz) field read in boxes of 2S columns x BR rows
template <typename R>
static int encode_ymap(CUtensorMap *m, const R *base, int nx, int ny, int nz, int S, int BR)
{
    cuuint64_t dims[3] = { (cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz };
    cuuint64_t strides[2] = { (cuuint64_t)nx * sizeof(R), (cuuint64_t)nx * ny * sizeof(R) };
    cuuint32_t box[3] = { (cuuint32_t)(2 * S), (cuuint32_t)BR, 1 };
    cuuint32_t es[3] = { 1, 1, 1 };
    CUresult r = g_encode(m, sizeof(R) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3,
                          (void *)base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        vec_set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return VEC_ERR_CUDA;
    }
    return VEC_OK;
}

template <typename R, int DIR, int N1, int N2, int S, bool WSYNC>
static int run_ct(Engine *E, const LineJob<R> *jobs, int nj, const char *name)
{
    using C = typename CT<R>::T;
    constexpr int N = N1 * N2;
    constexpr int NP = N1 > N2 ? N1 : N2;
    constexpr int TILE = 2 * S * N;
    constexpr int LDS = ct_lds<R, DIR, N1, N2, S>();
    static bool attr_set = false;
    const size_t smem = ct_smem_bytes<R, DIR, N1, N2, S>();
    static_assert(ct_smem_bytes<R, DIR, N1, N2, S>() == 2 * TILE * sizeof(R) + ((size_t)S * LDS + (sizeof(R) == 4 ? 2 : 1) * N) * sizeof(C) + 3 * (size_t)N * sizeof(R),
                  "shared memory layout");
    static_assert(ct_smem_bytes<R, DIR, N1, N2, S>() + 128 <= 232448, "tile does not fit one SM's shared memory");
    static_assert(LDS >= N1 * (N2 + 1) && LDS >= N2 * (N1 + 1) && LDS >= N + N / 32 + 1, "exchange rows");
    if (!attr_set) {
        CUDA_TRY(cudaFuncSetAttribute(line_ct<R, DIR, N1, N2, S, WSYNC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
        attr_set = true;
    }
    const int L = DIR == 0 ? E->ny : E->nx;
    const int tpp = L / (2 * S);
    JobPackCT<R> pk;
    memset(&pk, 0, sizeof(pk));
    double fields = 0.0;
    for (int j = 0; j < nj; j++) {
        pk.j[j] = jobs[j];
        fields += 2.0 + (jobs[j].acc1 ? 1.0 : 0.0);
        if (jobs[j].op2 != OP_NONE) fields += 1.0 + (jobs[j].acc2 ? 1.0 : 0.0);
    }
    TmapPack tp;
    memset(&tp, 0, sizeof(tp));
    if (DIR == 1) {
        int st = get_encoder();
        if (st) return st;
        constexpr int BR = ybox_rows(N);
        for (int j = 0; j < nj; j++)
            if ((st = encode_ymap<R>(&tp.m[j], jobs[j].in, E->nx, E->ny, E->nz, S, BR))) return st;
    }
    const int total = nj * E->nz * tpp;
    int per_sm = 1;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, line_ct<R, DIR, N1, N2, S, WSYNC>, S * NP, smem));
    if (per_sm < 1) per_sm = 1;
    int grid = E->num_sms * per_sm;
    if (grid > total) grid = total;
    E->prof_begin(name, fields * (double)E->n * sizeof(R));
    CUDA_TRY(launch_k(*E, line_ct<R, DIR, N1, N2, S, WSYNC>, dim3(grid), dim3(S * NP), smem, pk, tp,
                      E->tables<R>(DIR), E->nx, E->ny, E->nz, tpp, total, E->dev_err));
    E->prof_end();
    CUDA_TRY(cudaGetLastError());
    return VEC_OK;
}

static bool aligned16(const void *p) { return ((uintptr_t)p & 15) == 0; }

// returns 1 if handled by the specialised kernel, 0 if the caller must use
// the generic one, <0 on error
template <typename R>
int launch_lines_ct(Engine *E, int dir, const LineJob<R> *jobs, int njobs)
{
    const int n = dir == 0 ? E->nx : E->ny;
    const int L = dir == 0 ? E->ny : E->nx;
    constexpr bool F = sizeof(R) == 4;
    // sequences per tile
    int S = 0;
    switch (n) {
    case 64: case 96: case 128: case 192: case 256: S = F ? 16 : 8; break;
    case 384: case 512: S = F ? 8 : 4; break;
    // (n >= 768, FP32: 8 sequences make the y tiles' rows 64 bytes wide and
    // give 8 warps per SM; with 4 the 1024-point passes ran at 1.7-1.8 TB/s,
    // with 8 at 3.2-3.4 TB/s, measured at 1024^2 x 17)
    case 768: case 1024: S = F ? 8 : 2; break;
    default: return 0;
    }
    if (F && n <= 256 && E->ct_s == 8) S = 8;    // autotuned alternatives
    if (F && n >= 768 && E->ct_s == 4) S = 4;
    if (L % (2 * S) != 0) return 0;
    if ((E->nx * (int)sizeof(R)) % 16 != 0) return 0;
    for (int j = 0; j < njobs; j++) {
        if (!aligned16(jobs[j].in) || !aligned16(jobs[j].out1) || (jobs[j].out2 && !aligned16(jobs[j].out2)))
            return 0;
    }
    const bool ws = E->ct_warp;
    for (int j0 = 0; j0 < njobs; j0 += MAX_JOBS) {
        const int nj = njobs - j0 < MAX_JOBS ? njobs - j0 : MAX_JOBS;
        const LineJob<R> *jb = jobs + j0;
        const char *name = dir == 0 ? (F ? "line_x_f32" : "line_x_f64") : (F ? "line_y_f32" : "line_y_f64");
        if (E->prof_kinds) {
            // per job kind (profiling aid): forward, inverse, accumulate, derivative pair, other
            static const char *kinds[2][2][5] = {
                { { "line_x_f64_fwd", "line_x_f64_inv", "line_x_f64_acc", "line_x_f64_d12", "line_x_f64_op" },
                  { "line_x_f32_fwd", "line_x_f32_inv", "line_x_f32_acc", "line_x_f32_d12", "line_x_f32_op" } },
                { { "line_y_f64_fwd", "line_y_f64_inv", "line_y_f64_acc", "line_y_f64_d12", "line_y_f64_op" },
                  { "line_y_f32_fwd", "line_y_f32_inv", "line_y_f32_acc", "line_y_f32_d12", "line_y_f32_op" } } };
            const int kd = jb[0].op1 == OP_FWD ? 0 : jb[0].op1 == OP_INV ? 1 : jb[0].acc1 ? 2 : jb[0].op2 != OP_NONE ? 3 : 4;
            name = kinds[dir][F ? 1 : 0][kd];
        }
        int st = -1;
#define CT_CASE(NN, A, B, SS)                                                                       \
    if (n == NN && S == SS)                                                                         \
        st = dir == 1 ? run_ct<R, 1, A, B, SS, false>(E, jb, nj, name)                            \
                      : (ws ? run_ct<R, 0, A, B, SS, true>(E, jb, nj, name)                       \
                            : run_ct<R, 0, A, B, SS, false>(E, jb, nj, name));
        if constexpr (F) {
            CT_CASE(64, 8, 8, 16) CT_CASE(128, 16, 8, 16) CT_CASE(256, 16, 16, 16)
            CT_CASE(64, 8, 8, 8) CT_CASE(128, 16, 8, 8) CT_CASE(256, 16, 16, 8)
            CT_CASE(512, 32, 16, 8) CT_CASE(1024, 32, 32, 4) CT_CASE(1024, 32, 32, 8)
            CT_CASE(96, 8, 12, 16) CT_CASE(192, 16, 12, 16) CT_CASE(96, 8, 12, 8) CT_CASE(192, 16, 12, 8)
            CT_CASE(384, 16, 24, 8) CT_CASE(768, 32, 24, 4) CT_CASE(768, 32, 24, 8)
        } else {
            CT_CASE(64, 8, 8, 8) CT_CASE(128, 16, 8, 8) CT_CASE(256, 16, 16, 8)
            CT_CASE(512, 32, 16, 4) CT_CASE(1024, 32, 32, 2)
            CT_CASE(96, 8, 12, 8) CT_CASE(192, 16, 12, 8) CT_CASE(384, 16, 24, 4) CT_CASE(768, 32, 24, 2)
        }
#undef CT_CASE
        if (st < 0) return 0;
        if (st) return st;
    }
    return 1;
}

template int launch_lines_ct<float>(Engine *, int, const LineJob<float> *, int);
template int launch_lines_ct<double>(Engine *, int, const LineJob<double> *, int);
