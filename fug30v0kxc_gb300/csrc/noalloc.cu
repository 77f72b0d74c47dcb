// noalloc.cu -- the CFL time-step reduction (src/utils.F90:144-244) as a
// context-free entry point that allocates no memory.
//
// Who needs it: host programs that own all device memory through their own
// arena or pool and forbid any further device allocation once they are set
// up (for example a large coupled simulation driver that hands this solver
// pre-allocated fields), and callers that must not allocate between the
// steps of a long run.  Such callers cannot create a vec_ctx, because
// vec_create allocates every work array with cudaMalloc.
//
// The reduction's scratch (one partial triple per CTA) lives in a file-scope
// __device__ array of fixed size, so the library never allocates for it.
// Every GPU that loads the library holds this array (1.5 MiB) until the
// process exits.  All calls on a device share the array and each call
// overwrites the partials it uses, so calls whose kernels overlap on the GPU
// (different streams, or threads without ordering) race and must be avoided.
#include <math.h>
#include <stdio.h>

#include "common.cuh"

#define NOALLOC_CHUNK 2048                       // grid points per CTA
#define NOALLOC_MAX_BLOCKS 65536                 // CTAs the scratch can hold
#define NOALLOC_MAX_POINTS ((long long)NOALLOC_MAX_BLOCKS * NOALLOC_CHUNK)

// partial (velmxx, velmxz, denmn) per CTA, then one slot for the result
static __device__ __align__(256) double g_calcdt_scratch[3 * NOALLOC_MAX_BLOCKS + 4];

// address of g_calcdt_scratch on each device, found once per device
#define NOALLOC_MAX_DEVICES 64
static double *g_scratch_ptr[NOALLOC_MAX_DEVICES];

__global__ void k_noalloc_partials(const double *u, const double *v, const double *w, const double *r,
                                   const double *t, const double *bx, const double *by, const double *bz,
                                   long long n, double g1, double f, double *scratch)
{
    double mxx = -1.0e-50, mxz = -1.0e-50, mn = 1.0e300;
    const long long base = (long long)blockIdx.x * NOALLOC_CHUNK;
    for (int q = threadIdx.x; q < NOALLOC_CHUNK; q += blockDim.x) {
        long long i = base + q;
        if (i >= n) break;
        double u0 = u[i], v0 = v[i], w0 = w[i], r0 = r[i], t0 = t[i];
        double bz0 = bz[i], bx0 = bx[i], by0 = by[i];
        double bsq0 = bx0 * bx0 + by0 * by0 + bz0 * bz0;
        double xx = sqrt(u0 * u0 + v0 * v0) + g1 * sqrt(t0) + sqrt((bsq0 * f) / r0);
        double xz = sqrt(w0 * w0) + g1 * sqrt(t0) + sqrt((bsq0 * f) / r0);
        mn = fmin(mn, r0);
        mxx = fmax(mxx, xx);
        mxz = fmax(mxz, xz);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mxx = fmax(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
        mxz = fmax(mxz, __shfl_xor_sync(0xffffffffu, mxz, o));
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    }
    __shared__ double sh[3][32];
    const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0) { sh[0][wid] = mxx; sh[1][wid] = mxz; sh[2][wid] = mn; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < nw; k++) {
            mxx = fmax(mxx, sh[0][k]);
            mxz = fmax(mxz, sh[1][k]);
            mn = fmin(mn, sh[2][k]);
        }
        scratch[3 * (size_t)blockIdx.x + 0] = mxx;
        scratch[3 * (size_t)blockIdx.x + 1] = mxz;
        scratch[3 * (size_t)blockIdx.x + 2] = mn;
    }
}

struct NoallocLimits {
    double dd, dz, dtvisc0x, dtvisc0z, dtdiff0x, dtdiff0z, sf, eta_max;
    int var_eta;
};

__global__ void k_noalloc_final(const double *scratch, int nblocks, NoallocLimits L, double *dt_out)
{
    double mxx = -1.0e-50, mxz = -1.0e-50, mn = 1.0e300;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
        mxx = fmax(mxx, scratch[3 * (size_t)b + 0]);
        mxz = fmax(mxz, scratch[3 * (size_t)b + 1]);
        mn = fmin(mn, scratch[3 * (size_t)b + 2]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mxx = fmax(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
        mxz = fmax(mxz, __shfl_xor_sync(0xffffffffu, mxz, o));
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    }
    __shared__ double sh[3][32];
    const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0) { sh[0][wid] = mxx; sh[1][wid] = mxz; sh[2][wid] = mn; }
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int k = 1; k < nw; k++) {
        mxx = fmax(mxx, sh[0][k]);
        mxz = fmax(mxz, sh[1][k]);
        mn = fmin(mn, sh[2][k]);
    }
    // src/utils.F90:223-243, plus the magnetic-diffusion limits of eta(z)
    double m = 0.16 * L.dd / mxx;
    m = fmin(m, 0.3 * L.dz / mxz);
    m = fmin(m, L.dtvisc0x * mn);
    m = fmin(m, L.dtvisc0z * mn);
    m = fmin(m, L.dtdiff0x * mn);
    m = fmin(m, L.dtdiff0z * mn);
    if (L.var_eta) {
        m = fmin(m, 0.1 * L.dd * L.dd / L.eta_max);
        m = fmin(m, 0.2 * L.dz * L.dz / L.eta_max);
    }
    *dt_out = L.sf * m;
}

// Looks up the device address of the scratch array for the current device.
// The first call on each device does this; it must not be the first thing
// the process does inside a stream capture.  With CUDA's lazy module loading
// (the default since CUDA 12.2) this lookup is also what loads this file's
// module onto the device, and with it the 1.5 MiB array: the first call on a
// device therefore needs that much free device memory, and callers whose
// pool later takes the whole device make it at set-up, before the pool
// reserves its memory (or run with CUDA_MODULE_LOADING=EAGER, which loads
// every module when the library's first CUDA call creates the context).
static int noalloc_scratch(double **out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        cudaGetLastError();
        vec_set_error("vec_calcdt_noalloc: no usable current CUDA device");
        return VEC_ERR_CUDA;
    }
    if (!g_scratch_ptr[dev]) {
        double *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void **)&p, g_calcdt_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            vec_set_error("vec_calcdt_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return VEC_ERR_CUDA;
        }
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return VEC_OK;
}

// 1: memory of device dev (device or managed), 0: host memory, -1: memory
// of another device (a kernel on dev would read or write a peer's memory)
static int noalloc_where(const void *p, int dev)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (a.type == cudaMemoryTypeDevice) return a.device == dev ? 1 : -1;
    if (a.type == cudaMemoryTypeManaged) return 1;
    return 0;
}

extern "C" int vec_calcdt_noalloc(const vec_params *p, const double *u, const double *v, const double *w,
                                  const double *r, const double *t, const double *bx, const double *by,
                                  const double *bz, double *dt_out, void *stream)
{
    if (!p || !u || !v || !w || !r || !t || !bx || !by || !bz || !dt_out) {
        vec_set_error("vec_calcdt_noalloc: null argument");
        return VEC_ERR_ARG;
    }
    if (p->nx < 1 || p->ny < 1 || p->nz < 2) {
        vec_set_error("vec_calcdt_noalloc: bad grid %d x %d x %d", p->nx, p->ny, p->nz);
        return VEC_ERR_ARG;
    }
    const long long n = (long long)p->nx * p->ny * p->nz;
    if (n > NOALLOC_MAX_POINTS) {
        vec_set_error("vec_calcdt_noalloc: %lld grid points exceed the fixed scratch limit of %lld points",
                      n, NOALLOC_MAX_POINTS);
        return VEC_ERR_SIZE;
    }
    double *scratch = nullptr;
    int st = noalloc_scratch(&scratch);
    if (st) return st;
    int dev = -1;
    cudaGetDevice(&dev);
    const double *fields[8] = { u, v, w, r, t, bx, by, bz };
    for (int i = 0; i < 8; i++)
        if (noalloc_where(fields[i], dev) != 1) {
            vec_set_error("vec_calcdt_noalloc: field %d is not device memory of the current device %d", i, dev);
            return VEC_ERR_ARG;
        }
    const int out_where = noalloc_where(dt_out, dev);
    if (out_where < 0) {
        vec_set_error("vec_calcdt_noalloc: dt_out is device memory of another device than the current one (%d)", dev);
        return VEC_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    // constants of src/constants.f90:62-107 (only those calcdt reads)
    NoallocLimits L;
    const double dx = p->xmax / (double)p->nx, dy = p->ymax / (double)p->ny;
    L.dz = 1.0 / (double)(p->nz - 1);
    L.dd = dx < dy ? dx : dy;
    L.dtvisc0x = 0.1 * 0.75 * L.dd * L.dd / p->sigma / p->ck;
    L.dtvisc0z = 0.2 * L.dz * L.dz / p->sigma / p->ck * (1.0 + p->theta / 7.0);
    L.dtdiff0x = 0.1 * L.dd * L.dd / p->gamma / p->ck;
    L.dtdiff0z = 0.2 * L.dz * L.dz / p->gamma / p->ck * (1.0 + p->theta / 7.0);
    L.sf = p->sf;
    L.var_eta = p->eta_contrast != 1.0;
    const double zck = p->zeta * p->ck;
    L.eta_max = 0.0;
    for (int k = 0; k < p->nz; k++) {
        double e = zck * (1.0 + (p->eta_contrast - 1.0) * ((double)k * L.dz));
        L.eta_max = e > L.eta_max ? e : L.eta_max;
    }
    const int nblocks = (int)((n + NOALLOC_CHUNK - 1) / NOALLOC_CHUNK);
    k_noalloc_partials<<<nblocks, 256, 0, s>>>(u, v, w, r, t, bx, by, bz, n, sqrt(p->gamma), p->f, scratch);
    const bool dev_out = out_where == 1;
    double *res = dev_out ? dt_out : scratch + 3 * (size_t)NOALLOC_MAX_BLOCKS;
    k_noalloc_final<<<1, 1024, 0, s>>>(scratch, nblocks, L, res);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        vec_set_error("vec_calcdt_noalloc: launch failed: %s", cudaGetErrorString(e));
        return VEC_ERR_CUDA;
    }
    if (!dev_out) {
        e = cudaMemcpyAsync(dt_out, res, sizeof(double), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            vec_set_error("vec_calcdt_noalloc: %s", cudaGetErrorString(e));
            return VEC_ERR_CUDA;
        }
    }
    return VEC_OK;
}
