/*
 * vec.h -- C-ABI of the GB300 (sm_103a) VarElecCond time-step library.
 *
 * The reference (VarElecCond "p3d", Fortran 90) keeps all of its state in
 * module globals (src/arrays.f90:14-74) and exposes argument-light module
 * procedures.  This header replaces those procedures with plain C entry
 * points over an opaque context that owns every device array.
 *
 * Conventions
 *   - Fields are (nx,ny,nz) arrays of double, x fastest, exactly the
 *     Fortran column-major layout of src/arrays.f90:14-74: element
 *     (i,j,k) (1-based) lives at offset (i-1) + nx*((j-1) + ny*(k-1)).
 *     Plane k=1 is the top of the layer (z=0), k=nz the bottom (z=1),
 *     src/main.F90:5-9.
 *   - pol/tor are stored in the reference's 2-D halfcomplex x halfcomplex
 *     order (src/magnetic.f90:123-136, src/fft.F90:687-735).
 *   - Array pointers handed to an entry point may be host or device
 *     pointers: the library asks the CUDA runtime which one it got.  Host
 *     buffers are read/written only during the call; no pointer is kept.
 *   - Every entry point returns an int status: VEC_OK (0) or a negative
 *     code below.  Nothing aborts, traps or exits inside the library.
 *   - One context per host thread; calls on a context are stream-ordered
 *     on the context's own stream and are not re-entrant.
 */
#ifndef VEC_H
#define VEC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (negative, mirroring the reference's iret/abort codes) */
#define VEC_OK              0
#define VEC_ERR_NX         -1   /* odd nx: src/fft.F90:112-115 (also nx<4)  */
#define VEC_ERR_NY         -2   /* odd ny: src/fft.F90:116-119 (also ny<4)  */
#define VEC_ERR_NZ         -4   /* nz<6: src/main.F90:216-219, dbydz :355-358 */
#define VEC_ERR_ALLOC      -5   /* allocation failure: src/fft.F90:150-157  */
#define VEC_ERR_FLAG       -7   /* unknown dflag: src/dbydz.F90:704-707      */
#define VEC_ERR_INPUT      -8   /* unreadable / inconsistent INPUT file      */
#define VEC_ERR_DIVB      -12   /* |div B| > 0.01: src/main.F90:583-590      */
#define VEC_ERR_NAN       -20   /* non-finite value in the state             */
#define VEC_ERR_CUDA      -30   /* CUDA runtime error                        */
#define VEC_ERR_ARG       -31   /* null pointer / bad field id / bad value   */
#define VEC_ERR_SIZE      -32   /* size outside what the kernels support     */

/* ---- precision forms */
#define VEC_PREC_FP64       0   /* plain FP64 drop-in                        */
#define VEC_PREC_SPLIT      1   /* FP32 bulk, FP64 background/state/diagnostics */

/* ---- parameters: the INPUT file (src/initial.F90:142-172), the control
 *      flags hard-coded in src/main.F90:108-116, and the extensions. */
typedef struct vec_params {
    /* physical parameters, src/params.f90:9-28 (after the Ra/Q -> ck/F
     * conversion of src/initial.F90:174-201) */
    double gamma, sigma, theta, ck, cm, f, tayl, psi, zeta, xmax, ymax, sf;
    double rayl, chand;
    /* extensions with no reference counterpart (1.0 / 0 reproduce it) */
    double eta_contrast;   /* eta(z) = zeta*ck*(1 + (eta_contrast-1)*z)     */
    double noise_amp;      /* static IC noise amplitude (reference: 0.1)     */
    /* grid and run control */
    int32_t nx, ny, nz;
    int32_t nframe, ntotal, ndu06, ndu16, ndurestart;
    /* control flags, src/main.F90:108-116 (reference defaults in brackets) */
    int32_t dalias;        /* [1] dealias r,t,u,v,w every 10 steps           */
    int32_t kinematic;     /* [0]                                           */
    int32_t radbc;         /* [0] radiative upper temperature BC            */
    int32_t constflux;     /* [0] fixed-flux lower temperature BC           */
    int32_t perfect;       /* [0] perfectly conducting magnetic BC          */
    int32_t dynamo;        /* [0] seed field inserted by mag_init           */
    /* extensions */
    int32_t kappa_uniform; /* [0] 0: tanh kappa(z) of trans_params.f90:36-62 */
    int32_t seed_base;     /* [1996] RANSET seed base, src/ranset.f90:7      */
    int32_t precision;     /* VEC_PREC_FP64 or VEC_PREC_SPLIT               */
    int32_t diag_cadence;  /* [1] run GlobalAverages/nusselt/checkdivb every ndu06 */
} vec_params;

/* scalars of the time loop, src/main.F90:84-103 */
typedef struct vec_scalars {
    double dt, dt1, dt2, ttime;
    int32_t iter, nit, first, second;
} vec_scalars;

/* diagnostics printed every ndu06 steps, src/main.F90:552-647 */
typedef struct vec_diag_out {
    double ubar, vbar, kenergy, menergy, nusselt;
    double divbmax, divbmin;
    double rmin, rmax, tmin, tmax, umin, umax, vmin, vmax, wmin, wmax;
    double bxmin, bxmax, bymin, bymax, bzmin, bzmax;
    double machmin, machmax, alfvenmin, alfvenmax, rmsmin, rmsmax;
} vec_diag_out;

/* field ids for vec_get_field / vec_set_field (src/arrays.f90:14-74) */
enum vec_field {
    VEC_F_R = 0, VEC_F_T, VEC_F_U, VEC_F_V, VEC_F_W,
    VEC_F_BX, VEC_F_BY, VEC_F_BZ, VEC_F_JSQ, VEC_F_POL, VEC_F_TOR,
    /* RHS histories: slot s (1..3 in the reference) = base + (s-1) */
    VEC_F_RDOT = 16, VEC_F_TDOT = 19, VEC_F_UDOT = 22, VEC_F_VDOT = 25,
    VEC_F_WDOT = 28, VEC_F_POLDOT = 31, VEC_F_TORDOT = 34,
    VEC_F_COUNT = 37
};
/* 1-D mean-field ids for vec_get_mean / vec_set_mean */
enum vec_mean {
    VEC_M_BXBAR = 0, VEC_M_BYBAR,
    VEC_M_BXBARDOT = 2,  /* +0..2 = slots 1..3 */
    VEC_M_BYBARDOT = 5,
    VEC_M_KAPPA = 8, VEC_M_DKAPPA, VEC_M_ETA, VEC_M_DETA,
    VEC_M_COUNT = 12
};

typedef struct vec_ctx vec_ctx;

/* ---- parameters and context ------------------------------------------ */
/* Reference defaults: bin/INPUT values and the flags of src/main.F90:108-116. */
int vec_params_default(vec_params *p);
/* Reads an INPUT file (src/initial.F90:94-201, flag 1 = CK/F, 2 = Ra/Q). */
int vec_params_read_input(const char *path, vec_params *p);
/* Derived constants are set as in src/constants.f90:56-109, wavenumbers as
 * in init_fft (src/fft.F90:88-223), stencil scales as in init_dbydz
 * (src/dbydz.F90:355-362); all arrays of src/arrays.f90:81-300 are
 * allocated on the current CUDA device. */
int vec_create(const vec_params *p, vec_ctx **ctx);
int vec_destroy(vec_ctx *ctx);
const char *vec_last_error(void);
/* the context's CUDA stream (a cudaStream_t) */
void *vec_stream(vec_ctx *ctx);
int vec_sync(vec_ctx *ctx);

/* ---- state I/O --------------------------------------------------------- */
int vec_set_field(vec_ctx *ctx, int field, const double *src);
int vec_get_field(vec_ctx *ctx, int field, double *dst);
int vec_set_mean(vec_ctx *ctx, int mean, const double *src);  /* nz values */
int vec_get_mean(vec_ctx *ctx, int mean, double *dst);
int vec_set_bzbar(vec_ctx *ctx, double bzbar);
int vec_get_bzbar(vec_ctx *ctx, double *bzbar);
int vec_get_scalars(vec_ctx *ctx, vec_scalars *s);
int vec_set_scalars(vec_ctx *ctx, const vec_scalars *s);

/* ---- set-up ------------------------------------------------------------ */
/* static polytrope + seeded noise, src/initial.F90:25-86 with RANSET
 * (src/ranset.f90:1-29), then ini_trans_params (src/main.F90:276-280) */
int vec_static(vec_ctx *ctx);
/* B (real space) -> pol, tor, means, jsq; src/magnetic.f90:5-279 */
int vec_mag_init(vec_ctx *ctx);
/* CFL + diffusive time step, src/utils.F90:144-244; also stored as ctx dt.
 * VEC_ERR_NAN (dt still written) if a term of the CFL expression is not
 * finite. */
int vec_calcdt(vec_ctx *ctx, double *dt);

/* ---- horizontal spectral operators, src/fft.F90:255-799 ---------------- */
int vec_d1bydx(vec_ctx *ctx, const double *fin, double *fout);
int vec_d1bydy(vec_ctx *ctx, const double *fin, double *fout);
int vec_d2bydx(vec_ctx *ctx, const double *fin, double *f1out, double *f2out);
int vec_d2bydy(vec_ctx *ctx, const double *fin, double *f1out, double *f2out);
int vec_dealias(vec_ctx *ctx, double *z);
int vec_forwardfft(vec_ctx *ctx, const double *fin, double *fout);
int vec_inversefft(vec_ctx *ctx, const double *fin, double *fout);

/* ---- vertical finite differences, src/dbydz.F90:1588-3673 -------------- */
int vec_d1bydz(vec_ctx *ctx, const double *fin, double *fout, int dflag);
/* the upwind sign test reads the context's w, as the reference reads the
 * module-global w (src/dbydz.F90:511,559,606) */
int vec_d1upbydz(vec_ctx *ctx, const double *fin, double *fout, int dflag);
int vec_d2bydz(vec_ctx *ctx, const double *fin, double *fout, int dflag);
int vec_d1bydz1d(vec_ctx *ctx, const double *fin, double *fout, int dflag);
int vec_d2bydz1d(vec_ctx *ctx, const double *fin, double *fout, int dflag);

/* ---- FP32 forms of the horizontal operators ------------------------------
 * The line kernels the split form's time step runs (FP32 data, FP32
 * twiddles and multipliers), on caller data: dir 0 transforms along x
 * (d1bydx, d2bydx, ... of src/fft.F90:255-489), dir 1 along y (:329-581).
 * op1: VEC_OP_D1, VEC_OP_D2, VEC_OP_DEALIAS (one direction of
 * src/fft.F90:586-682), VEC_OP_FWD (r2hc), VEC_OP_INV (hc2r divided by n);
 * op2 (a second output from the same forward transform, as d2bydx's f1out /
 * f2out pair): VEC_OP_NONE, VEC_OP_D1 or VEC_OP_D2, with op1 D1, D2 or
 * DEALIAS; or VEC_OP_D1 with op1 INV: the derivative of the inverse, from
 * the same spectrum (how the split bandj takes d(bz)/dx and d(bz)/dy).
 * Arrays are (nx,ny,nz) floats, host or device; any context precision. */
#define VEC_OP_NONE         0
#define VEC_OP_D1           1
#define VEC_OP_D2           2
#define VEC_OP_DEALIAS      3
#define VEC_OP_FWD          4
#define VEC_OP_INV          5
int vec_line_f32(vec_ctx *ctx, int dir, int op1, int op2, const float *fin, float *f1out, float *f2out);

/* ---- physics on the context's state ------------------------------------ */
int vec_hydro_deriv(vec_ctx *ctx);   /* src/hydro_deriv.f90:5-505 -> slot 3 */
int vec_mag_deriv(vec_ctx *ctx);     /* src/magnetic.f90:285-487 -> slot 3  */
int vec_bandj(vec_ctx *ctx);         /* src/magnetic.f90:492-664            */
int vec_magdealias(vec_ctx *ctx);    /* src/magnetic.f90:666-717            */
int vec_boundary(vec_ctx *ctx);      /* src/dbydz.F90:3686-4197             */
int vec_mag_boundary(vec_ctx *ctx);  /* src/dbydz.F90:4205-4791             */
/* AB3 coefficients + update + density floor + history shift + dt1/dt2,
 * src/main.F90:381-489 (uses and advances the context's scalars) */
int vec_ab3_update(vec_ctx *ctx);
/* GlobalAverages (which removes the mean horizontal momentum from u,v),
 * nusselt, checkdivb, sminmax: src/utils.F90:22-371, src/dbydz.F90:4796-4925,
 * src/main.F90:552-647.  Returns VEC_ERR_NAN when r, T, u, v, w, B or div B
 * holds a NaN or an infinity (out is still written), else VEC_ERR_DIVB when
 * |div B| > 0.01. */
int vec_diag(vec_ctx *ctx, vec_diag_out *out);

/* ---- the time loop ----------------------------------------------------- */
/* nsteps iterations of src/main.F90:340-747 (no printing, no snapshots):
 * diagnostics every ndu06 steps, calcdt every 10, dealias every 10.
 * Returns VEC_ERR_DIVB if the div B check of a diagnostics step fails
 * (src/main.F90:583-590).  Returns VEC_ERR_NAN if the state holds a NaN or
 * an infinity: the diagnostics check r, T, u, v, w, B and div B, and calcdt
 * checks the terms of its CFL expression (a negative T or rho counts, as
 * its square root is not finite).  The calcdt check is read back once, at
 * the end of a call whose steps ran calcdt; the steps of that call have
 * then all been executed.  Without a magnetic field (f = 0 and not
 * kinematic) the split form leaves pol and tor as they are: their
 * right-hand side is zero, and the FP64 form's update adds exactly zero. */
int vec_step(vec_ctx *ctx, int nsteps);
/* Steps without diagnostics run as replays of a captured CUDA graph of one
 * step (two variants: plain, and the tenth step with dealias and calcdt);
 * on by default, off while profiling.  on = 0 launches every kernel. */
int vec_use_graphs(vec_ctx *ctx, int on);
/* last diagnostics computed inside vec_step (valid after an ndu06 step) */
int vec_last_diag(vec_ctx *ctx, vec_diag_out *out);

/* ---- snapshots: the NetCDF layout of src/netcdf.F90:39-1287 -------------- */
/* One snapshot in host memory; fields[0..7] = R, T, U, V, W, Bx, By, Bz
 * (caller-owned nx*ny*nz doubles each, Fortran (nx,ny,nz) order). */
typedef struct vec_snapshot {
    int32_t nx, ny, nz, iteration, version, pad_;
    double time, timestep;
    double gamma, sigma, theta, ck, cm, f, tayl, psi, zeta, xmax, ymax;
    char history[80];
    double *fields[8];
} vec_snapshot;
/* Writes a classic (CDF-1) NetCDF file as CreateNetCDF/WriteNetCDF do
 * (src/netcdf.F90:39-585); iprec 4 (float) or 8 (double), cf.
 * src/main.F90:695-704. */
int vec_nc_write(const char *path, const vec_snapshot *s, int iprec);
/* the same with the file format chosen: fmt 1 classic (as above), fmt 2
 * 64-bit offsets (NF_64BIT_OFFSET, the interpolate program's output,
 * interpolate/netcdf.F90:73) */
int vec_nc_write_fmt(const char *path, const vec_snapshot *s, int iprec, int fmt);
/* Reads a classic NetCDF snapshot (OpenNetCDF/ReadNetCDF,
 * src/netcdf.F90:591-1166): sizes, parameters, time, iteration, timestep;
 * fields too when s->fields[i] are set and s->nx/ny/nz match the file. */
int vec_nc_read(const char *path, vec_snapshot *s);
/* The context's state written as a snapshot (time/iteration/timestep from
 * the context's scalars; timestep = dt1 as in src/main.F90:729). */
int vec_write_snapshot(vec_ctx *ctx, const char *path, int iprec, const char *history);
/* Restart (nframe = 1, src/initial.F90:221-230): loads R..Bz, iteration,
 * time and timestep (as dt1); the AB3 histories are not stored, so the next
 * step is an Euler step, as in the reference. */
int vec_read_restart(vec_ctx *ctx, const char *path);

/* ---- allocation-free entry point ---------------------------------------- */
/* No counterpart in the reference.  calcdt (src/utils.F90:144-244) for
 * callers that cannot allocate device memory: programs whose device memory
 * is all handed out by their own arena or pool, and which therefore cannot
 * create a vec_ctx (vec_create allocates).  The caller passes pointers to
 * the eight fields (nx*ny*nz doubles each, sizes taken from p) in memory of
 * the current device, and dt_out (device memory of the current device, or
 * host memory); other pointers return VEC_ERR_ARG.  No memory is allocated
 * by a call: the reduction's scratch is a fixed 1.5 MiB __device__ array
 * inside the library, held until the process exits by every GPU that has
 * loaded it.  The first call on a device looks up that array's address;
 * with CUDA's lazy module loading (the default) that is also when the
 * array is placed on the device, so make the first call on each device at
 * set-up, before any stream capture and before a pool reserves the whole
 * device (or set CUDA_MODULE_LOADING=EAGER).  A host dt_out makes the call
 * synchronise the stream and read the result back, which cannot be
 * captured in a CUDA graph; a device dt_out keeps the call asynchronous.
 * Grids above 2^27 points return VEC_ERR_SIZE.  All calls on a device share
 * the scratch: calls that overlap on the GPU race. */
int vec_calcdt_noalloc(const vec_params *p, const double *u, const double *v, const double *w,
                       const double *r, const double *t, const double *bx, const double *by,
                       const double *bz, double *dt_out, void *stream);

/* ---- batched ensemble (independent instances, uneven grids) ------------- */
typedef struct vec_ens vec_ens;
/* n members with their own parameters (grids and physics may differ) */
int vec_ensemble_create(const vec_params *ps, int n, vec_ens **ens);
int vec_ensemble_destroy(vec_ens *ens);
int vec_ensemble_size(vec_ens *ens);
vec_ctx *vec_ensemble_member(vec_ens *ens, int i);
/* static state, calcdt and mag_init of every member */
int vec_ensemble_start(vec_ens *ens);
/* nsteps time steps of every member; steps without diagnostics replay one
 * captured CUDA graph holding an independent branch per member */
int vec_ensemble_step(vec_ens *ens, int nsteps);
int vec_ensemble_sync(vec_ens *ens);
/* autotuner: per distinct grid, time candidate tile shapes (z-marching
 * chunk, sequences per FFT tile) on a scratch context for `steps` steps and
 * apply the fastest; `cache` (may be NULL) is a text file read first and
 * rewritten with the results */
int vec_ensemble_tune(vec_ens *ens, int steps, const char *cache);
/* the tile shapes in use by a context */
int vec_tunables(vec_ctx *ctx, int *kc, int *s);
/* sets them: kc in {8, 16, 32}; s in {0 (the kernel's default), 4, 8}
 * (FP32 register-FFT lines: 8 selects 8 sequences per tile for n <= 256,
 * 4 selects 4 for n >= 768; the generic kernel takes 4 or 8) */
int vec_set_tunables(vec_ctx *ctx, int kc, int s);

/* ---- learned closure: the network ---------------------------------------
 * No reference counterpart (an addition to the solver).  Four 3x3x3
 * convolutions 9(->16 padded) -> 32 -> 32 -> 32 -> 8 channels with GELU,
 * BF16 weights and activations, FP32 accumulation on the tensor cores,
 * Adam.  Grids: nx in {16, 32, 64, 128}, nx*ny a multiple of 128; periodic
 * in x and y, zero padding in z. */
typedef struct vec_net vec_net;
int vec_net_create(int nx, int ny, int nz, int batch, unsigned long long seed, vec_net **out);
int vec_net_destroy(vec_net *net);
long long vec_net_nparams(vec_net *net);
/* FP32 master parameters: per layer l = 0..3 weights [27][cout][cin] then
 * biases [cout], with (cin, cout) = (16,32), (32,32), (32,32), (32,16) */
int vec_net_get_params(vec_net *net, float *host_out);
int vec_net_set_params(vec_net *net, const float *host);
int vec_net_get_grads(vec_net *net, float *host_out);
/* x: host [batch][nz][ny][nx][16] FP32 (rounded to BF16); out (may be
 * NULL): host [batch][nz][ny][nx][8] FP32 */
int vec_net_forward(vec_net *net, const float *x, float *out);
/* after vec_net_forward: mean-squared error against tgt (host, as out) and
 * the gradient of every parameter */
int vec_net_backward(vec_net *net, const float *tgt, double *loss);
int vec_net_adam(vec_net *net, float lr);
/* device time of reps forward passes and of reps training steps (Adam with
 * rate 0) on the current batch, and the floating-point operations each
 * executes (padded channels included) */
int vec_net_time(vec_net *net, int reps, float *ms_fwd, float *ms_train, double *flops_fwd, double *flops_train);
/* kernels the network launched since creation */
long long vec_net_launch_count(vec_net *net);

/* ---- learned closure: coupling to the solver ----------------------------
 * No reference counterpart.  A closure works on a coarse grid r times
 * coarser than the fine (DNS) grid in x and y, with nz_f - 1 = r (nz_c - 1)
 * (coarse planes on fine planes); r even.  Network inputs: the box-filtered
 * state (u, v, w, rho - rho0(z), T - T0(z), Bx, By, Bz - mean Bz) and the
 * height; outputs: the RHS correction (d/dt of u, v, w, rho, T, Bx, By, Bz)
 * = filtered fine RHS - coarse RHS at the filtered state. */
typedef struct vec_closure vec_closure;
typedef struct {
    int judges;             /* comparisons made */
    int pad_;
    long long coarse_steps, fine_steps;
    long long fallback_step; /* coarse step at which the run fell back, -1 if never */
    double last_err[3];     /* relative error of Nu, kinetic, magnetic energy */
    double max_err[3];
    double end_time;
    int nseries;            /* rows written to the diagnostics series */
    int divb_fail;          /* the coarse run failed the div B check (a fall-back cause) */
    int blowup;             /* the coarse run stopped advancing: non-finite time or step,
                             * or a step below 1e-3 of its first (a fall-back cause) */
    int pad2_;
} vec_closure_report;
/* coarse: the coarse parameters; capacity: training pairs stored (FP32,
 * 64 bytes per coarse point and pair); batch <= 64 */
int vec_closure_create(const vec_params *coarse, int factor, int capacity, int batch, unsigned long long seed,
                       vec_closure **out);
int vec_closure_destroy(vec_closure *cl);
vec_net *vec_closure_net(vec_closure *cl);
/* at inference the normalised network output is limited to +-clip
 * standard deviations of the training targets and the correction scaled by
 * gain (defaults 4 and 1) */
int vec_closure_set_output(vec_closure *cl, float clip, float gain);
/* Nusselt number at the fixed-temperature top (the formula of
 * src/dbydz.F90:4877-4925 mirrored to the top plane); with a fixed-flux
 * bottom the reference's own Nusselt number is identically one */
int vec_top_nusselt(vec_ctx *ctx, double *nu);
int vec_closure_npairs(vec_closure *cl);
/* coarse context state = box-filtered fine state (then pol/tor, B and the
 * boundary conditions as after a time step) */
int vec_box_filter(vec_closure *cl, vec_ctx *fine, vec_ctx *coarse);
/* one training pair from the fine context's current state (coarse is a
 * scratch context whose state is overwritten) */
int vec_closure_add_pair(vec_closure *cl, vec_ctx *fine, vec_ctx *coarse);
int vec_closure_get_pair(vec_closure *cl, int i, float *in, float *tgt);
/* per-channel mean / standard deviation of inputs and targets over pairs
 * [0, n); [32] = input means, input stds, target means, target stds */
int vec_closure_fit_norm(vec_closure *cl, int n);
int vec_closure_get_norm(vec_closure *cl, float *out32);
int vec_closure_set_norm(vec_closure *cl, const float *in32);
/* iters Adam steps (rate lr) on seeded batches from pairs [0, ntrain);
 * losses (may be NULL) gets each iteration's mean-squared error */
int vec_closure_train(vec_closure *cl, int iters, float lr, int ntrain, unsigned long long seed, double *losses);
/* a-priori error on pairs [first, first + count), normalised units:
 * mse_net with the network, mse_zero without (the plain coarse RHS) */
int vec_closure_eval(vec_closure *cl, int first, int count, double *mse_net, double *mse_zero);
/* the RHS correction of a coarse context on (1) or off (0) */
int vec_closure_attach(vec_closure *cl, vec_ctx *coarse, int on);
/* the correction for the coarse context's current state */
int vec_closure_infer(vec_closure *cl, vec_ctx *coarse);
/* nsteps steps, the correction recomputed before each */
int vec_closure_step(vec_closure *cl, vec_ctx *coarse, int nsteps);
/* judged run to time t_end: every `every` coarse steps a plain fine segment
 * of nfine steps from the upsampled coarse state; if the change over the
 * segment of the Nusselt numbers (bottom and top), kinetic or magnetic
 * energy in the coarse run differs from their change in the fine run by
 * more than tol of the fine value (the drift; the offset between the coarse
 * state and the filtered upsampled one at the segment start is not drift),
 * or the coarse state fails the div B check of src/main.F90:583-590, or the coarse run
 * stops advancing (non-finite time or step, or a step below 1e-3 of its
 * first), the run continues on the fine solver from the last state it holds
 * -- the upsampled start of the run, then the end of the last judged
 * segment -- (returning VEC_ERR_NAN if that stops advancing too).  Fine
 * diagnostics are taken of the box-filtered fine state.  With diag_every >
 * 0, rows (time, Nu, kinetic energy, magnetic energy, top Nu) of the running
 * solver are appended to series[cap][5] every diag_every steps. */
int vec_closure_run(vec_closure *cl, vec_ctx *coarse, vec_ctx *fine, double t_end, int every, int nfine, double tol,
                    int diag_every, double *series, int cap, vec_closure_report *rep);

/* ---- spectral upsampling (interpolate/fft.F90:834-927) -------------------- */
/* the reference's expand: in (nx, ny, nz) of coarse -> out (r nx, r ny, nz)
 * of fine (fine has the same nz); host or device arrays */
int vec_expand(vec_ctx *coarse, vec_ctx *fine, const double *in, double *out);
/* fine state from the coarse one: expand of u, v, w, rho, T, B, cubic
 * interpolation between vertex-aligned planes, pol/tor from B, boundary
 * conditions; the fine run restarts its AB3 history at the coarse time */
int vec_upsample(vec_ctx *coarse, vec_ctx *fine);

/* ---- instrumentation --------------------------------------------------- */
/* When on, every kernel launch of the context is bracketed by CUDA events
 * on the context stream and its duration is accumulated per kernel name. */
int vec_profile(vec_ctx *ctx, int on);
/* number of distinct kernels recorded */
int vec_profile_count(vec_ctx *ctx);
/* i-th record: name (<= 63 chars), launches, total milliseconds and total
 * algorithmic bytes (every field the kernel must read or write, once) */
int vec_profile_get(vec_ctx *ctx, int i, char *name, int *launches, double *ms, double *bytes);
int vec_profile_reset(vec_ctx *ctx);
/* kernels launched by this context since creation */
long long vec_launch_count(vec_ctx *ctx);
/* FP64 fused multiply-add throughput of the current device in TFLOP/s (a
 * timed microbenchmark, the best of reps launches): the roofline of the
 * plain FP64 form, whose kernels are bound by the FP64 pipe */
int vec_measure_fp64(int reps, double *tflops);
/* Self-test of the bounded-wait error path: launches, on the context's
 * stream, one kernel that waits on a shared-memory barrier nothing arrives
 * on, gives up after `polls` polls (1 .. 2^24, the line kernels' limit) and
 * raises the context's error flag, as a line kernel does when a tile copy
 * does not complete.  The next vec_sync returns VEC_ERR_CUDA once and clears
 * the flag; the context stays usable. */
int vec_selftest_wait(vec_ctx *ctx, long long polls);

#ifdef __cplusplus
}
#endif
#endif /* VEC_H */
