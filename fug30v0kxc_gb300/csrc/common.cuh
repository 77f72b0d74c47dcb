// common.cuh -- shared types of the GB300 VarElecCond library (internal).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "../../include/vec.h"

// complex type per real precision
template <typename R> struct CT;
template <> struct CT<double> { using T = double2; };
template <> struct CT<float> { using T = float2; };

// ---- line-transform (horizontal FFT) plan -------------------------------
#define LP_MAXST 16
struct LinePlan {
    int n;                  // line length (nx or ny)
    int nst;                // number of Stockham stages
    int radix[LP_MAXST];    // radix of each stage (2,3,4,5,8)
    int P;                  // complex sequences (= pairs of real lines) per CTA
    int lines;              // real lines per plane (ny for x lines, nx for y lines)
    int tiles;              // CTAs per plane = ceil(lines / (2P))
    int threads;            // block size
    size_t smem;            // dynamic shared memory bytes for the precision in use
};

// operations of one line job
enum LineOp {
    OP_NONE = 0,
    OP_D1 = 1,       // first derivative (+ik), DC and Nyquist dropped: src/fft.F90:292-302
    OP_D2 = 2,       // second derivative (-k^2), Nyquist kept: src/fft.F90:442-454
    OP_DEALIAS = 3,  // 2/3-rule truncation: src/fft.F90:618-626
    OP_FWD = 4,      // real -> halfcomplex, unnormalised (rfftw forward)
    OP_INV = 5,      // halfcomplex -> real, divided by n (rfftw backward / n); op2
                     // OP_D1 adds the derivative of that inverse as a second output
};

template <typename R>
struct LineJob {
    const R *in;
    R *out1, *out2;
    R alpha1, alpha2;   // outputs are alpha * result (+ old value when acc)
    int op1, op2;
    int acc1, acc2;
    const double *addk; // OP_INV only: out1 += addk[plane] + addc
    double addc;
};

// line jobs per launch: a batch of 16 members carries up to 96 (five hydro
// jobs, and the Lorentz fluxes' and E's transforms, per member); the job
// and tensor-map packs then take 24 KB of the 32 KB kernel parameter space
#define MAX_JOBS 128

// spectral tables of one direction (device pointers)
template <typename R>
struct LineTables {
    typename CT<R>::T *tw;  // exp(-2 pi i e / n), e = 0..n-1
    R *m1;                  // d1 multiplier (imaginary part, sign and 1/n folded in)
    R *m2;                  // d2 multiplier (k2 / n, DC zeroed)
    R *mda;                 // dealias mask (1/n or 0)
};

// horizontal wavenumber tables in one precision: akx1, aky1 and the
// plane table akx2[i] + aky2[j] (summed in FP64, then rounded once)
template <typename R>
struct HTab {
    const R *kx1, *ky1, *kh2;
    const R *kh2inv;        // 1 / kh2 (0 at the mean, kh2 = 0), rounded once from FP64; FP32 only
};

// ---- per-context derived constants: src/constants.f90:56-109 -----------
struct Consts {
    double dx, dy, dz, dd, xn, xzn, taylt, cpsi, spsi, cor;
    double gck, sck, zck, scko3, sckg, fzckg, thmplus1, fo2, g1, gm1, nusstmp;
    double dtvisc0x, dtvisc0z, dtdiff0x, dtdiff0z;
    double ho12, sc1;
    double f, gamma, theta, sf;
    double eta_max;
    int var_eta;            // eta_contrast != 1
    int icutoffx, icutoffy;
};

// order-preserving keys (see okey in physics.cu) of -DBL_MAX and +DBL_MAX
#define OKEY_NEG_HUGE 0x0010000000000000ull
#define OKEY_POS_HUGE 0xffefffffffffffffull

// time-loop scalars living on the device (src/main.F90:84-103)
struct DevScalars {
    double dt, dt1, dt2, ttime;
    double c0, c1, c2;
    int first, second;
    // reductions
    unsigned long long velmxx, velmxz, denmn;  // order-preserving keys of the reductions
    double res[64];                            // diagnostics results
    // the last calcdt met a non-finite value (NaN or infinity) in the state
    // or in the CFL expression; the time loop reports it as VEC_ERR_NAN
    int nonfinite, pad_nf;
};

// AB3 coefficients of src/main.F90:381-403 from the step sizes (read-only)
__device__ __forceinline__ void ab3_coefs(const DevScalars *ds, double *c)
{
    const double dt = ds->dt;
    if (ds->first) {
        c[0] = dt; c[1] = 0.0; c[2] = 0.0;
    } else if (ds->second) {
        c[0] = dt * (1.0 + 0.5 * (dt / ds->dt1));
        c[1] = -0.5 * dt * (dt / ds->dt1);
        c[2] = 0.0;
    } else {
        const double dt1 = ds->dt1, dt2 = ds->dt2;
        c[0] = dt + (((dt * dt) / (dt1 * dt2)) * ((dt / 3.0) + 0.5 * (dt1 + dt2)));
        c[1] = ((dt * dt) / (dt1 * (dt1 - dt2))) * ((dt / 3.0) + 0.5 * dt2);
        c[2] = -((dt * dt) / (dt2 * (dt1 - dt2))) * ((dt / 3.0) + 0.5 * dt1);
    }
}
// the scalar updates of one step: ttime (:345), the Euler / AB2 start flags
// and dt1, dt2 (:488-489); c are this step's coefficients
__device__ __forceinline__ void ab3_advance(DevScalars *ds, const double *c)
{
    const double dt = ds->dt;
    ds->ttime = ds->ttime + dt;
    if (ds->first) {
        ds->first = 0; ds->second = 1;
        ds->dt1 = 0.0; ds->dt2 = 0.0;
    } else if (ds->second) {
        ds->first = 0; ds->second = 0;
        ds->dt2 = 0.0;
    }
    ds->c0 = c[0]; ds->c1 = c[1]; ds->c2 = c[2];
    ds->dt2 = dt + ds->dt1;
    ds->dt1 = dt;
}

// RHS histories in logical slot order (0 oldest .. 2 newest), kept in device
// memory so that kernels read their slot pointers at run time and a one-
// thread kernel performs the shift of src/main.F90:448-461 by rotating it;
// kernel arguments are then the same on every step (graph capture).
struct HistTable {
    void *p[7][3];          // r, t, u, v, w, pol, tor
    double *bx[3], *by[3];  // bxbardot, bybardot
};

// The arguments of one kernel for each member of a batch: equally sized
// contexts (one grid size of an ensemble) whose step runs as one launch per
// kernel, blockIdx.z picking the member.  A single context is a batch of
// one (NB = 1, member index 0).
#define BATCH_MAX 16
template <typename A, int NB> struct Batch { A a[NB]; };
#define BATCH_MEMBER(bt, NB) ((bt).a[(NB) > 1 ? blockIdx.z : 0])

// First statement of the step's kernels: with programmatic dependent launch
// a kernel may be started while its predecessor in the stream still runs,
// and this waits until every predecessor grid has completed and its memory
// is visible (a no-op for an ordinary launch).
#define PDL_WAIT() asm volatile("griddepcontrol.wait;" ::: "memory")

// ---- error helper --------------------------------------------------------
void vec_set_error(const char *fmt, ...);

#define CUDA_TRY(x)                                                                   \
    do {                                                                              \
        cudaError_t e_ = (x);                                                         \
        if (e_ != cudaSuccess) {                                                      \
            vec_set_error("%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_)); \
            return VEC_ERR_CUDA;                                                      \
        }                                                                             \
    } while (0)
