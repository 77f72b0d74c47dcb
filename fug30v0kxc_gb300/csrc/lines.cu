// lines.cu -- horizontal spectral operators of src/fft.F90 as batched
// shared-memory FFT kernels for sm_103a.
//
// One CTA takes 2P real lines of one z-plane (rows of nx values for the x
// direction, columns of ny values at stride nx for the y direction), packs
// them pairwise as P complex sequences z = a + i b, and runs a mixed-radix
// (8/4/2/3/5) Stockham FFT on them in shared memory.  Because every
// spectral operator of the reference (+ik, -k^2, the 2/3 truncation) is a
// Hermitian-symmetric multiplier, it acts on Z = A + iB directly and the
// inverse transform returns both real lines at once; only the 2-D
// forward/inverse transforms (halfcomplex storage) separate A and B.
//
// A launch carries up to MAX_JOBS jobs (input field, one or two outputs, an
// operator per output, optional accumulate epilogue); blockIdx.y selects the
// job, so all fields needing the same direction share one launch.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "common.cuh"
#include "engine.h"

template <typename R> struct JobPack { LineJob<R> j[MAX_JOBS]; };

// ---- radix kernels (natural order outputs X_0..X_{R-1}) ----------------------
template <typename C>
__device__ __forceinline__ C cmul(C a, C b) { C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r; }
template <typename C>
__device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C>
__device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
// multiply by -i (forward) or +i (inverse)
template <bool INV, typename C>
__device__ __forceinline__ C rot90(C a) { C r; if (INV) { r.x = -a.y; r.y = a.x; } else { r.x = a.y; r.y = -a.x; } return r; }

template <int RAD, bool INV, typename C> struct Dft;

template <bool INV, typename C> struct Dft<2, INV, C> {
    static __device__ __forceinline__ void run(C *v) { C a = v[0], b = v[1]; v[0] = cadd(a, b); v[1] = csub(a, b); }
};
template <bool INV, typename C> struct Dft<4, INV, C> {
    static __device__ __forceinline__ void run(C *v) {
        C a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
        C b0 = cadd(v[1], v[3]), b1 = rot90<INV>(csub(v[1], v[3]));
        v[0] = cadd(a0, b0); v[1] = cadd(a1, b1); v[2] = csub(a0, b0); v[3] = csub(a1, b1);
    }
};
template <bool INV, typename C> struct Dft<8, INV, C> {
    static __device__ __forceinline__ void run(C *v) {
        using R = decltype(v[0].x);
        const R h = (R)0.70710678118654752440084436210484904;   // sqrt(2)/2
        C a[4], b[4];
#pragma unroll
        for (int j = 0; j < 4; j++) { a[j] = cadd(v[j], v[j + 4]); b[j] = csub(v[j], v[j + 4]); }
        // b_j *= W8^j, W8 = exp(-+ i pi/4)
        {
            C t = b[1];
            if (!INV) { b[1].x = h * (t.x + t.y); b[1].y = h * (t.y - t.x); }
            else      { b[1].x = h * (t.x - t.y); b[1].y = h * (t.y + t.x); }
            b[2] = rot90<INV>(b[2]);
            t = b[3];
            if (!INV) { b[3].x = h * (t.y - t.x); b[3].y = -h * (t.x + t.y); }
            else      { b[3].x = -h * (t.x + t.y); b[3].y = h * (t.x - t.y); }
        }
        Dft<4, INV, C>::run(a);
        Dft<4, INV, C>::run(b);
#pragma unroll
        for (int m = 0; m < 4; m++) { v[2 * m] = a[m]; v[2 * m + 1] = b[m]; }
    }
};
template <bool INV, typename C> struct Dft<3, INV, C> {
    static __device__ __forceinline__ void run(C *v) {
        using R = decltype(v[0].x);
        const R c1 = (R)-0.5;
        const R s1 = INV ? (R)0.86602540378443864676372317075293618 : (R)-0.86602540378443864676372317075293618;
        C t1 = cadd(v[1], v[2]), t2 = csub(v[1], v[2]);
        C x0 = cadd(v[0], t1);
        C m1; m1.x = v[0].x + c1 * t1.x; m1.y = v[0].y + c1 * t1.y;
        // i*s1*t2
        C m2; m2.x = -s1 * t2.y; m2.y = s1 * t2.x;
        v[0] = x0; v[1] = cadd(m1, m2); v[2] = csub(m1, m2);
    }
};
template <bool INV, typename C> struct Dft<5, INV, C> {
    static __device__ __forceinline__ void run(C *v) {
        using R = decltype(v[0].x);
        const R c1 = (R)0.30901699437494742410229341718281906;    // cos(2pi/5)
        const R c2 = (R)-0.80901699437494742410229341718281906;   // cos(4pi/5)
        const R sg = INV ? (R)1 : (R)-1;
        const R s1 = sg * (R)0.95105651629515357211643933337938214;  // sin(2pi/5)
        const R s2 = sg * (R)0.58778525229247312916870595463907277;  // sin(4pi/5)
        C t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
        C d1 = csub(v[1], v[4]), d2 = csub(v[2], v[3]);
        C x0 = cadd(v[0], cadd(t1, t2));
        C a1, a2, b1, b2;
        a1.x = v[0].x + c1 * t1.x + c2 * t2.x; a1.y = v[0].y + c1 * t1.y + c2 * t2.y;
        a2.x = v[0].x + c2 * t1.x + c1 * t2.x; a2.y = v[0].y + c2 * t1.y + c1 * t2.y;
        // b1 = i (s1 d1 + s2 d2), b2 = i (s2 d1 - s1 d2)
        R u1x = s1 * d1.x + s2 * d2.x, u1y = s1 * d1.y + s2 * d2.y;
        R u2x = s2 * d1.x - s1 * d2.x, u2y = s2 * d1.y - s1 * d2.y;
        b1.x = -u1y; b1.y = u1x;
        b2.x = -u2y; b2.y = u2x;
        v[0] = x0; v[1] = cadd(a1, b1); v[4] = csub(a1, b1); v[2] = cadd(a2, b2); v[3] = csub(a2, b2);
    }
};

// ---- one Stockham stage over nseq sequences of length n (stride ld) ----------
// EPT: complex elements held per thread per stage (bounds the register use)
#define EPT 8
template <int RAD, bool INV, typename C>
__device__ __noinline__ void fft_stage(C *buf, int nseq, int ld, int n, int Ns, const C *tw)
{
    constexpr int MAXB = (EPT + RAD - 1) / RAD;
    const int nb = n / RAD, total = nb * nseq;
    const int ts = n / (Ns * RAD);
    C v[MAXB][RAD];
#pragma unroll
    for (int c = 0; c < MAXB; c++) {
        int b = threadIdx.x + c * blockDim.x;
        if (b < total) {
            int s = b / nb, j = b - s * nb;
            int k = j % Ns;
            const C *sq = buf + s * ld;
#pragma unroll
            for (int r = 0; r < RAD; r++) v[c][r] = sq[j + r * nb];
            if (Ns > 1) {
#pragma unroll
                for (int r = 1; r < RAD; r++) {
                    C w = tw[r * k * ts];
                    if (INV) w.y = -w.y;
                    v[c][r] = cmul(v[c][r], w);
                }
            }
            Dft<RAD, INV, C>::run(v[c]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < MAXB; c++) {
        int b = threadIdx.x + c * blockDim.x;
        if (b < total) {
            int s = b / nb, j = b - s * nb;
            int k = j % Ns;
            C *sq = buf + s * ld;
            int d = (j / Ns) * Ns * RAD + k;
#pragma unroll
            for (int r = 0; r < RAD; r++) sq[d + r * Ns] = v[c][r];
        }
    }
    __syncthreads();
}

template <bool INV, typename C>
__device__ void fft_run(C *buf, int nseq, int ld, const LinePlan &pl, const C *tw)
{
    int Ns = 1;
    for (int st = 0; st < pl.nst; st++) {
        switch (pl.radix[st]) {
        case 8: fft_stage<8, INV>(buf, nseq, ld, pl.n, Ns, tw); break;
        case 4: fft_stage<4, INV>(buf, nseq, ld, pl.n, Ns, tw); break;
        case 2: fft_stage<2, INV>(buf, nseq, ld, pl.n, Ns, tw); break;
        case 3: fft_stage<3, INV>(buf, nseq, ld, pl.n, Ns, tw); break;
        default: fft_stage<5, INV>(buf, nseq, ld, pl.n, Ns, tw); break;
        }
        Ns *= pl.radix[st];
    }
}

// ---- the line kernel --------------------------------------------------------
// DIR 0: lines along x (contiguous); DIR 1: lines along y (stride nx).
template <typename R, int DIR>
__global__ void __launch_bounds__(512, 1)
line_kernel(JobPack<R> jobs, LinePlan pl, LineTables<R> tb, int nx, int ny, int nz)
{
    PDL_WAIT();
    using C = typename CT<R>::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = pl.n, P = pl.P, ld = n + 1;
    C *A = reinterpret_cast<C *>(smem_raw);
    C *B = A + (size_t)P * ld;
    C *tw = B + (size_t)P * ld;

    const LineJob<R> &jb = jobs.j[blockIdx.y];
    const int plane = blockIdx.x / pl.tiles;
    const int l0 = (blockIdx.x - plane * pl.tiles) * 2 * P;
    const size_t np = (size_t)nx * ny;
    const size_t pbase = (size_t)plane * np;
    const int L = pl.lines;
    const int tid = threadIdx.x, nt = blockDim.x;

    for (int e = tid; e < n; e += nt) tw[e] = tb.tw[e];

    // element (line l, position e) -> offset in the plane
#define LOFF(l, e) (DIR == 0 ? (size_t)(l) * nx + (e) : (size_t)(e) * nx + (l))

    const int op1 = jb.op1, op2 = jb.op2;
    if (op1 == OP_INV) {
        // assemble Z_k = A_k + i B_k from two halfcomplex lines
        for (int idx = tid; idx < P * n; idx += nt) {
            int s, k;
            if (DIR == 0) { s = idx / n; k = idx - s * n; } else { k = idx / P; s = idx - k * P; }
            int la = l0 + 2 * s, lb = la + 1;
            R ar = 0, ai = 0, br = 0, bi = 0;
            int kk = k <= n / 2 ? k : n - k;
            bool edge = (kk == 0) || (2 * kk == n);
            if (la < L) {
                R x = jb.in[pbase + LOFF(la, kk)];
                R y = edge ? (R)0 : jb.in[pbase + LOFF(la, n - kk)];
                ar = x; ai = k <= n / 2 ? y : -y;
            }
            if (lb < L) {
                R x = jb.in[pbase + LOFF(lb, kk)];
                R y = edge ? (R)0 : jb.in[pbase + LOFF(lb, n - kk)];
                br = x; bi = k <= n / 2 ? y : -y;
            }
            C z; z.x = ar - bi; z.y = ai + br;
            A[s * ld + k] = z;
        }
        // op2 OP_D1: also the derivative of the inverse, B <- m1 * Z
        const bool two = op2 == OP_D1;
        if (two) {
            __syncthreads();
            for (int idx = tid; idx < P * n; idx += nt) {
                const int s = idx / n, k = idx - s * n;
                const C z = A[s * ld + k];
                const R m = tb.m1[k];
                C y; y.x = -m * z.y; y.y = m * z.x;
                B[s * ld + k] = y;
            }
        }
        __syncthreads();
        fft_run<true>(A, two ? 2 * P : P, ld, pl, tw);
        const R sc = (R)1 / (R)n;
        for (int idx = tid; idx < 2 * P * n; idx += nt) {
            int l, e;
            if (DIR == 0) { l = idx / n; e = idx - l * n; } else { e = idx / (2 * P); l = idx - e * (2 * P); }
            int gl = l0 + l;
            if (gl >= L) continue;
            C z = A[(l >> 1) * ld + e];
            R val = (l & 1) ? z.y : z.x;
            val = val * sc;
            R *o = jb.out1 + pbase + LOFF(gl, e);
            R res = jb.alpha1 * val;
            res = jb.acc1 ? *o + res : res;
            if (jb.addk) res = res + (R)jb.addk[plane];
            if (jb.addc != 0.0) res = res + (R)jb.addc;
            *o = res;
            if (two) {
                const C y = B[(l >> 1) * ld + e];
                R *o2 = jb.out2 + pbase + LOFF(gl, e);
                const R r2 = jb.alpha2 * ((l & 1) ? y.y : y.x);
                *o2 = jb.acc2 ? *o2 + r2 : r2;
            }
        }
        return;
    }

    // load 2P real lines as P complex sequences
    for (int idx = tid; idx < 2 * P * n; idx += nt) {
        int l, e;
        if (DIR == 0) { l = idx / n; e = idx - l * n; } else { e = idx / (2 * P); l = idx - e * (2 * P); }
        int gl = l0 + l;
        R val = gl < L ? jb.in[pbase + LOFF(gl, e)] : (R)0;
        R *dst = reinterpret_cast<R *>(&A[(l >> 1) * ld + e]);
        dst[l & 1] = val;
    }
    __syncthreads();
    fft_run<false>(A, P, ld, pl, tw);

    if (op1 == OP_FWD) {
        // separate Z into the halfcomplex spectra of the two real lines
        for (int idx = tid; idx < 2 * P * n; idx += nt) {
            int l, p;
            if (DIR == 0) { l = idx / n; p = idx - l * n; } else { p = idx / (2 * P); l = idx - p * (2 * P); }
            int gl = l0 + l;
            if (gl >= L) continue;
            const C *sq = A + (l >> 1) * ld;
            int q = p == 0 ? 0 : n - p;
            C zp = sq[p], zq = sq[q];
            R val;
            if (2 * p <= n) val = (l & 1) ? (R)0.5 * (zp.y + zq.y) : (R)0.5 * (zp.x + zq.x);
            else            val = (l & 1) ? (R)0.5 * (zp.x - zq.x) : (R)0.5 * (zq.y - zp.y);
            R *o = jb.out1 + pbase + LOFF(gl, p);
            R res = jb.alpha1 * val;
            *o = jb.acc1 ? *o + res : res;
        }
        return;
    }

    // spectral multipliers: A <- m1 * Z, B <- m2 * Z
    const bool two = op2 != OP_NONE;
    for (int idx = tid; idx < P * n; idx += nt) {
        int s = idx / n, k = idx - s * n;
        C z = A[s * ld + k];
        if (two) {
            C y;
            if (op2 == OP_D1) { R m = tb.m1[k]; y.x = -m * z.y; y.y = m * z.x; }
            else { R m = op2 == OP_D2 ? tb.m2[k] : tb.mda[k]; y.x = m * z.x; y.y = m * z.y; }
            B[s * ld + k] = y;
        }
        C y;
        if (op1 == OP_D1) { R m = tb.m1[k]; y.x = -m * z.y; y.y = m * z.x; }
        else { R m = op1 == OP_D2 ? tb.m2[k] : tb.mda[k]; y.x = m * z.x; y.y = m * z.y; }
        A[s * ld + k] = y;
    }
    __syncthreads();
    // A and B are contiguous: one inverse pass over 2P sequences
    fft_run<true>(A, two ? 2 * P : P, ld, pl, tw);

    for (int idx = tid; idx < 2 * P * n; idx += nt) {
        int l, e;
        if (DIR == 0) { l = idx / n; e = idx - l * n; } else { e = idx / (2 * P); l = idx - e * (2 * P); }
        int gl = l0 + l;
        if (gl >= L) continue;
        size_t off = pbase + LOFF(gl, e);
        C z = A[(l >> 1) * ld + e];
        R val = (l & 1) ? z.y : z.x;
        R res = jb.alpha1 * val;
        jb.out1[off] = jb.acc1 ? jb.out1[off] + res : res;
        if (two) {
            C y = B[(l >> 1) * ld + e];
            R v2 = (l & 1) ? y.y : y.x;
            R r2 = jb.alpha2 * v2;
            jb.out2[off] = jb.acc2 ? jb.out2[off] + r2 : r2;
        }
    }
#undef LOFF
}

// ---- host side ------------------------------------------------------------------
// Twiddles exp(-2 pi i e/n) computed on the host in double, exact at
// multiples of n/4 (quadrant reduction of the angle).
void sincos2pi_host(long e, long n, double *c, double *s)
{
    e %= n;
    if (e < 0) e += n;
    long q = (4 * e) / n, r = 4 * e - q * n;
    double cf, sf;
    if (2 * r <= n) { double a = (M_PI / 2.0) * ((double)r / (double)n); cf = cos(a); sf = sin(a); }
    else { double a = (M_PI / 2.0) * ((double)(n - r) / (double)n); cf = sin(a); sf = cos(a); }
    switch (q) {
    case 0: *c = cf; *s = sf; break;
    case 1: *c = -sf; *s = cf; break;
    case 2: *c = -cf; *s = -sf; break;
    default: *c = sf; *s = -cf; break;
    }
}

int line_plan_make(int n, int lines, int elem_bytes, LinePlan *pl, int force_p)
{
    memset(pl, 0, sizeof(*pl));
    pl->n = n;
    int m = n;
    while (m % 8 == 0 && pl->nst < LP_MAXST) { pl->radix[pl->nst++] = 8; m /= 8; }
    while (m % 4 == 0 && pl->nst < LP_MAXST) { pl->radix[pl->nst++] = 4; m /= 4; }
    while (m % 2 == 0 && pl->nst < LP_MAXST) { pl->radix[pl->nst++] = 2; m /= 2; }
    while (m % 3 == 0 && pl->nst < LP_MAXST) { pl->radix[pl->nst++] = 3; m /= 3; }
    while (m % 5 == 0 && pl->nst < LP_MAXST) { pl->radix[pl->nst++] = 5; m /= 5; }
    if (m != 1) return VEC_ERR_SIZE;      // only 2^a 3^b 5^c line lengths
    if (n > 2048) return VEC_ERR_SIZE;
    // P complex sequences per CTA: about 2048 complex elements per buffer
    int P = 2048 / n;
    if (P < 1) P = 1;
    if (P > 16) P = 16;
    if (force_p > 0) P = force_p;
    if (P > lines / 2) P = lines / 2;
    if (P < 1) P = 1;
    pl->P = P;
    pl->lines = lines;
    pl->tiles = (lines + 2 * P - 1) / (2 * P);
    // threads: at most EPT complex elements per thread in every stage
    // (inverse passes may run 2P sequences)
    int th = (2 * P * n + EPT - 1) / EPT;
    th = ((th + 31) / 32) * 32;
    if (th < 64) th = 64;
    if (th > 512) return VEC_ERR_SIZE;
    pl->threads = th;
    pl->smem = (size_t)(2 * P * (n + 1) + n) * 2 * elem_bytes;
    return VEC_OK;
}

// multipliers for a direction: k1 = akx1-like table, k2 = akx2-like table
template <typename R>
int line_tables_make(int n, const double *k1, const double *k2, int icut, LineTables<R> *tb)
{
    using C = typename CT<R>::T;
    C *tw = (C *)malloc(sizeof(C) * n);
    R *m1 = (R *)malloc(sizeof(R) * n), *m2 = (R *)malloc(sizeof(R) * n), *mda = (R *)malloc(sizeof(R) * n);
    const double dn = (double)n;
    for (int e = 0; e < n; e++) {
        double c, s;
        sincos2pi_host(e, n, &c, &s);
        tw[e].x = (R)c;
        tw[e].y = (R)(-s);
        // first derivative: +i k for 0<k<n/2, -i k for k>n/2, 0 at DC / Nyquist
        double d1 = 0.0;
        if (e > 0 && 2 * e < n) d1 = k1[e] / dn;
        else if (2 * e > n) d1 = -k1[e] / dn;
        m1[e] = (R)d1;
        m2[e] = (R)(e == 0 ? 0.0 : k2[e] / dn);
        int kk = e <= n / 2 ? e : n - e;
        mda[e] = (R)(kk >= n / 2 - icut ? 0.0 : 1.0 / dn);
    }
    int st = VEC_OK;
    if (cudaMalloc(&tb->tw, sizeof(C) * n) != cudaSuccess || cudaMalloc(&tb->m1, sizeof(R) * n) != cudaSuccess ||
        cudaMalloc(&tb->m2, sizeof(R) * n) != cudaSuccess || cudaMalloc(&tb->mda, sizeof(R) * n) != cudaSuccess)
        st = VEC_ERR_ALLOC;
    if (!st) {
        cudaMemcpy(tb->tw, tw, sizeof(C) * n, cudaMemcpyHostToDevice);
        cudaMemcpy(tb->m1, m1, sizeof(R) * n, cudaMemcpyHostToDevice);
        cudaMemcpy(tb->m2, m2, sizeof(R) * n, cudaMemcpyHostToDevice);
        cudaMemcpy(tb->mda, mda, sizeof(R) * n, cudaMemcpyHostToDevice);
    }
    free(tw); free(m1); free(m2); free(mda);
    return st;
}

template <typename R>
void line_tables_free(LineTables<R> *tb)
{
    cudaFree(tb->tw); cudaFree(tb->m1); cudaFree(tb->m2); cudaFree(tb->mda);
    memset(tb, 0, sizeof(*tb));
}

template <typename R>
int launch_lines(Engine *E, int dir, const LineJob<R> *jobs, int njobs)
{
    if (njobs <= 0) return VEC_OK;
    if (!E->generic_lines) {
        int h = launch_lines_ct<R>(E, dir, jobs, njobs);
        if (h == 1) return VEC_OK;
        if (h < 0) return h;
    }
    LinePlan pl = dir == 0 ? E->plx : E->ply;
    if (E->ct_s > 0 && E->ct_s != pl.P) {
        // autotuned sequences per CTA for the generic kernel
        LinePlan alt;
        if (line_plan_make(pl.n, pl.lines, sizeof(R), &alt, E->ct_s) == VEC_OK) pl = alt;
    }
    const LineTables<R> &tb = E->tables<R>(dir);
    for (int j0 = 0; j0 < njobs; j0 += MAX_JOBS) {
        JobPack<R> pk;
        memset(&pk, 0, sizeof(pk));
        int nj = njobs - j0 < MAX_JOBS ? njobs - j0 : MAX_JOBS;
        for (int j = 0; j < nj; j++) pk.j[j] = jobs[j0 + j];
        dim3 grid((unsigned)(pl.tiles * E->nz), (unsigned)nj);
        size_t smem = (size_t)(2 * pl.P * (pl.n + 1) + pl.n) * sizeof(typename CT<R>::T);
        const char *name = dir == 0 ? (sizeof(R) == 8 ? "line_x_f64" : "line_x_f32")
                                    : (sizeof(R) == 8 ? "line_y_f64" : "line_y_f32");
        double fields = 0.0;
        for (int j = 0; j < nj; j++) {
            const LineJob<R> &q = pk.j[j];
            fields += 1.0 + 1.0 + (q.acc1 ? 1.0 : 0.0);
            if (q.op2 != OP_NONE) fields += 1.0 + (q.acc2 ? 1.0 : 0.0);
        }
        E->prof_begin(name, fields * (double)E->n * sizeof(R));
        if (dir == 0)
            line_kernel<R, 0><<<grid, pl.threads, smem, E->stream>>>(pk, pl, tb, E->nx, E->ny, E->nz);
        else
            line_kernel<R, 1><<<grid, pl.threads, smem, E->stream>>>(pk, pl, tb, E->nx, E->ny, E->nz);
        E->prof_end();
        CUDA_TRY(cudaGetLastError());
    }
    return VEC_OK;
}

int line_kernels_configure()
{
    int st = line_ct_configure();
    if (st) return st;
    CUDA_TRY(cudaFuncSetAttribute(line_kernel<double, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CUDA_TRY(cudaFuncSetAttribute(line_kernel<double, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CUDA_TRY(cudaFuncSetAttribute(line_kernel<float, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    CUDA_TRY(cudaFuncSetAttribute(line_kernel<float, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    return VEC_OK;
}

template int line_tables_make<double>(int, const double *, const double *, int, LineTables<double> *);
template int line_tables_make<float>(int, const double *, const double *, int, LineTables<float> *);
template void line_tables_free<double>(LineTables<double> *);
template void line_tables_free<float>(LineTables<float> *);
template int launch_lines<double>(Engine *, int, const LineJob<double> *, int);
template int launch_lines<float>(Engine *, int, const LineJob<float> *, int);
