// engine.h -- the device-resident context behind the C-ABI (internal).
//
// All module-global arrays of src/arrays.f90:14-74 live here, in HBM, for
// the whole run.  Fields are (nx,ny,nz) with x fastest.  In the FP64 form
// every array is double; in the split form the bulk work arrays, RHS
// histories and the FP32 mirrors of the state are float while the state
// itself, the 1-D backgrounds and the diagnostics stay double.
#pragma once
#include <string>
#include <utility>
#include <vector>

#include "common.cuh"

// work-array slots (FP64 form: double; split form: float)
enum WorkSlot {
    // horizontal derivatives of r,t,u,v,w (hydro_deriv)
    W_RX, W_TX, W_TXX, W_UX, W_UXX, W_VX, W_VXX, W_WX, W_WXX,
    W_RY, W_TY, W_TYY, W_UY, W_UYY, W_VY, W_VYY, W_WY, W_WYY,
    // second-level inputs / accumulators
    W_P1, W_P2, W_Q, W_G, W_H, W_P3, W_P4,
    W_RACC, W_UACC, W_VACC, W_WACC,
    // magnetic work (reference: ex, ey, ez, wk1..wk4)
    W_EX, W_EY, W_EZ, W_M1, W_M2, W_M3, W_M4, W_M5, W_M6,
    W_COUNT
};

struct ProfRec {
    std::string name;
    int launches = 0;
    double ms = 0.0;
    double bytes = 0.0;     // algorithmic bytes (fields read + written once)
};

struct Engine {
    vec_params p;
    Consts k;
    int nx, ny, nz;
    size_t np, n;
    int split;                  // VEC_PREC_SPLIT
    cudaStream_t stream = nullptr;
    // mag_deriv runs on stream2, forked from and joined to stream inside the
    // step (it shares no output or work array with hydro_deriv)
    cudaStream_t stream2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int par_mag = 1;            // mag_deriv on stream2 (FP64 form; VEC_SERIAL_MAG=0/1 forces it)
    long long launches = 0;
    int num_sms = 152;
    int *dev_err = nullptr;     // set by kernels whose bounded waits ran out
    int generic_lines = 0;      // force the generic line kernel (VEC_GENERIC_LINES=1)

    LinePlan plx, ply;          // precision of the bulk path
    LinePlan plx64, ply64;      // FP64 plans (per-operator entry points)
    LineTables<double> tx64, ty64;
    LineTables<float> tx32, ty32;

    // FP64 state (src/arrays.f90)
    double *r = nullptr, *t = nullptr, *u = nullptr, *v = nullptr, *w = nullptr;
    double *bx = nullptr, *by = nullptr, *bz = nullptr, *jsq = nullptr, *pol = nullptr, *tor = nullptr;
    // RHS history buffers (physical; their logical order lives in ht)
    void *hbuf[7][3] = {};
    double *bxd_buf[3] = {}, *byd_buf[3] = {};
    HistTable *ht = nullptr;    // device table of logical slots
    // 1-D
    double *bxbar = nullptr, *bybar = nullptr;
    double *kappa = nullptr, *dkappa = nullptr, *eta = nullptr, *deta = nullptr;
    double *akx1 = nullptr, *akx2 = nullptr, *aky1 = nullptr, *aky2 = nullptr;
    HTab<float> hf = {};        // the same wavenumbers in FP32 (kh2: np values)
    HTab<double> hd = {};       // FP64 (kx1, ky1 alias akx1, aky1)
    float *pcf = nullptr;       // split: per-plane FP32 coefficients [PC_COUNT][nz]
    double *w1d = nullptr;      // 1-D scratch (8 nz)
    double bzbar = 0.0;
    // work arrays (bulk precision), carved from one contiguous block
    void *wk[W_COUNT] = {};
    void *wblock = nullptr;
    // FP64 scratch for per-operator entry points and diagnostics
    double *s64[6] = {};
    // split form: FP32 mirrors of the state and FP64 backgrounds
    float *r32 = nullptr, *t32 = nullptr, *u32 = nullptr, *v32 = nullptr, *w32 = nullptr;
    float *bx32 = nullptr, *by32 = nullptr, *bz32 = nullptr, *jsq32 = nullptr;
    float *pol32 = nullptr, *tor32 = nullptr;
    double *rho0 = nullptr, *t0 = nullptr, *hres = nullptr;   // 1-D FP64 background block (split.cu)
    int b32_auth = 0;           // split form: the FP32 B/jsq are newer than the FP64 ones
    // reductions scratch
    double *red = nullptr;      // per-block partials
    float *cdt = nullptr;       // calcdt: 3 global estimate keys (+1 pad), then [3][chunks] estimates
    int red_blocks = 0;
    DevScalars *ds = nullptr;   // device scalars
    DevScalars *hs = nullptr;   // pinned host mirror
    // host counters
    int nit = 0, iter = 0;
    vec_diag_out last_diag;
    int have_diag = 0;

    // CUDA graphs of one time step: [0] plain step, [1] step with dealias and
    // calcdt (nit % 10 == 0); diagnostic steps run without a graph
    int use_graphs = 1;
    cudaGraphExec_t gexec[2] = { nullptr, nullptr };
    int g_b32_after[2] = { 0, 0 };
    long long g_launches[2] = { 0, 0 };
    // learned-closure RHS correction (closure.cu): 7 fields in the history
    // row order (r, t, u, v, w, pol, tor) plus 3 scratch fields, of the RHS
    // precision, and the mean-field corrections; added to the newest RHS
    // slots inside the step while corr_on
    void *corr = nullptr;
    double *corr_bx = nullptr, *corr_by = nullptr;
    int corr_on = 0;
    // tunables (the ensemble autotuner sets them per grid)
    int kc_pass2 = 16;          // planes per z chunk of hydro pass 2 (z-pencil or z-marching kernel)
    int ct_s = 0;               // sequences per line tile (0: default for the size)
    bool ct_warp = true;        // x-line tiles synchronised per warp (VEC_CT_WARP=0: per CTA)
    bool prof_kinds = false;    // VEC_PROF_KINDS=1: line launches profiled per job kind
    bool pdl = true;            // programmatic dependent launches (VEC_PDL=0: ordinary launches)
    bool vec4 = true;           // four-point (16-byte) forms of the split pointwise kernels (VEC_VEC4=0: one point)
    bool zpencil = true;        // split pass 2 with TMA-staged z-pencils (VEC_ZPENCIL=0: per-plane form)
    int zpencil4 = -1;          // the same for pass 4: 1 on, 0 off (four points per thread, per
                                // plane), -1 from np >= 1024^2 on, where its z window of five
                                // fields no longer stays in L2 (VEC_ZPENCIL4)
    bool int_cvt = true;        // FP32/FP64 conversions of the split AB3 update on the integer pipe
                                // (VEC_HW_CVT=1: hardware conversions; the same bits)

    // profiling
    bool prof_on = false;
    std::vector<ProfRec> prof;
    std::vector<cudaEvent_t> ev_pool;
    struct Pending { int rec; cudaEvent_t a, b; double bytes; };
    std::vector<Pending> pending;
    int prof_cur = -1;
    cudaEvent_t prof_a = nullptr;

    template <typename R> const LineTables<R> &tables(int dir) const;
    template <typename R> R *W(int slot) const { return reinterpret_cast<R *>(wk[slot]); }
    // FP64 work array i (i < W_COUNT/2 in the split form, whose block holds
    // W_COUNT float arrays = W_COUNT/2 double arrays)
    double *W64(int i) const { return split ? reinterpret_cast<double *>(wblock) + (size_t)i * n : (double *)wk[i]; }

    void prof_begin(const char *name, double bytes = 0.0);
    void drop_graphs();
    void prof_end();
    int prof_flush();
};

template <> inline const LineTables<double> &Engine::tables<double>(int dir) const { return dir == 0 ? tx64 : ty64; }
// A kernel launch on the engine's stream.  With E.pdl (the default) it is a
// programmatic dependent launch: the launch of the next kernel overlaps the
// end of this one, which hides most of the gap between the step's kernels;
// every kernel launched this way starts with PDL_WAIT().
template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(const Engine &E, void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                            Args &&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = E.stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = E.pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

// One kernel over the members of a batch of equally sized contexts (see
// Batch): make(E) builds a member's arguments; a batch of one launches the
// NB = 1 instance, a larger one the BATCH_MAX instance with one grid layer
// (blockIdx.z) per member.  The launch runs on (and is counted and profiled
// by) the first member; bytes are per member.
template <typename A, typename F>
inline int launch_members(Engine *const *Es, int nE, const char *name, double bytes, dim3 grid, dim3 block,
                          size_t smem, void (*k1)(Batch<A, 1>), void (*kb)(Batch<A, BATCH_MAX>), F make)
{
    Engine *E = Es[0];
    if (nE < 1 || nE > BATCH_MAX) return VEC_ERR_ARG;
    E->prof_begin(name, bytes * nE);
    cudaError_t e;
    if (nE == 1) {
        Batch<A, 1> b;
        b.a[0] = make(Es[0]);
        e = launch_k(*E, k1, grid, block, smem, b);
    } else {
        Batch<A, BATCH_MAX> b;
        for (int i = 0; i < nE; i++) b.a[i] = make(Es[i]);
        grid.z = (unsigned)nE;
        e = launch_k(*E, kb, grid, block, smem, b);
    }
    E->prof_end();
    if (e != cudaSuccess) {
        vec_set_error("%s: launch failed: %s", name, cudaGetErrorString(e));
        return VEC_ERR_CUDA;
    }
    CUDA_TRY(cudaGetLastError());
    return VEC_OK;
}

template <typename R> inline HTab<R> htab(const Engine &E);
// one CTA row of 256 threads per plane (the spectral kernels of magkern.cuh)
inline dim3 plane_grid(const Engine &E) { return dim3((unsigned)((E.np + 255) / 256), (unsigned)E.nz); }
template <> inline HTab<float> htab<float>(const Engine &E) { return E.hf; }
template <> inline HTab<double> htab<double>(const Engine &E) { return E.hd; }
template <> inline const LineTables<float> &Engine::tables<float>(int dir) const { return dir == 0 ? tx32 : ty32; }

// lines.cu
// exp(-2 pi i e/n) on the host in double, exact at multiples of n/4
void sincos2pi_host(long e, long n, double *c, double *s);
int line_plan_make(int n, int lines, int elem_bytes, LinePlan *pl, int force_p = 0);
template <typename R> int line_tables_make(int n, const double *k1, const double *k2, int icut, LineTables<R> *tb);
template <typename R> void line_tables_free(LineTables<R> *tb);
template <typename R> int launch_lines(Engine *E, int dir, const LineJob<R> *jobs, int njobs);
int line_kernels_configure();
// physics.cu: calcdt scratch (floats per context, initialisation of its keys)
int cdt_chunks(size_t n);
int cdt_init(float *cdt);
int line_ct_configure();
template <typename R> int launch_lines_ct(Engine *E, int dir, const LineJob<R> *jobs, int njobs);

template <typename R>
inline LineJob<R> ljob(const R *in, R *out1, int op1, R *out2 = nullptr, int op2 = OP_NONE,
                       int acc1 = 0, int acc2 = 0, R a1 = (R)1, R a2 = (R)1)
{
    LineJob<R> j;
    j.in = in; j.out1 = out1; j.out2 = out2; j.op1 = op1; j.op2 = op2;
    j.acc1 = acc1; j.acc2 = acc2; j.alpha1 = a1; j.alpha2 = a2;
    j.addk = nullptr; j.addc = 0.0;
    return j;
}

// physics.cu (FP64 form)
int op_d1z(Engine *E, const double *in, double *out, int flag, int np, int nz);
int op_d1upz(Engine *E, const double *in, double *out, int flag);
int op_d2z(Engine *E, const double *in, double *out, int flag, int np, int nz);
int phys_hydro64(Engine *E);
int phys_mag64(Engine *E);
int phys_zero_mag_rhs(Engine *E);
int phys_bandj64(Engine *E);
int phys_magdealias(Engine *E);
int phys_boundary(Engine *E);
int phys_mag_boundary(Engine *E);
int phys_boundaries(Engine *E);   // boundary + mag_boundary in one launch
int phys_ab3(Engine *E, int magdealias);
int phys_ab3_coef(Engine *E);
int phys_rotate_hist(Engine *E);
int hist_table_host(Engine *E, HistTable *h);   // synchronous copy of the table
int phys_dealias_state(Engine *E);
int phys_calcdt(Engine *E);
int phys_diag(Engine *E, vec_diag_out *out);
int phys_mag_init(Engine *E);
int phys_static(Engine *E);
int phys_step_prologue(Engine *E);
// capi.cu (used by the ensemble)
int engine_enqueue_step(Engine &E, bool diag_now);
int engine_one_step(Engine &E);
bool engine_diag_due(const Engine &E, int nit);
Engine &engine_of(vec_ctx *c);
// closure.cu
int closure_apply_corr(Engine *E);
// split form (split.cu)
int split_setup(Engine *E);
int split_refresh_coefs(Engine *E);   // after kappa / eta change
const double *split_bg_t0(const Engine *E);   // T0(z), FP64
// FP32 mirrors written by the boundary kernels in the split form (null: FP64 form)
struct BoundaryMirrors {
    float *u32, *v32, *w32, *t32, *pol32, *tor32;
    const double *t0;
};
// with_mag: E = u x B and its forward transforms ride along (the x and y
// line launches carry them); split_mag then runs with spectra_done
int split_hydro(Engine *E, bool with_mag = false);
// In one time step the AB3 coefficient step can ride on the mean-field CTA
// of split_mag's mag_div kernel (ab3_coef) and the history rotation on the
// first kernel of split_bandj (rotate_hist); split_ab3 then runs the update
// alone (folded).
int split_mag(Engine *E, bool ab3_coef = false, bool spectra_done = false);
int split_bandj(Engine *E, bool rotate_hist = false);
int split_refresh(Engine *E);
int split_refresh_field(Engine *E, int field);   // one field's mirror (VEC_F_*)
int split_refresh_planes(Engine *E, int mask);
int split_refresh_uv(Engine *E);
int split_sync_b64(Engine *E);
int split_ab3(Engine *E, int magdealias, bool folded = false);
int split_dealias(Engine *E);
int split_calcdt(Engine *E);

// The same stages for a batch of equally sized split-form contexts (one grid
// of an ensemble): one launch per kernel covers every member (Batch,
// launch_members); line jobs of all members share the line launches.
int phys_zero_mag_rhs_m(Engine *const *Es, int nE);
int phys_boundary_m(Engine *const *Es, int nE);
int phys_boundaries_m(Engine *const *Es, int nE);
int phys_rotate_hist_m(Engine *const *Es, int nE);
int phys_ab3_coef_m(Engine *const *Es, int nE);
int phys_calcdt_m(Engine *const *Es, int nE);
int split_hydro_m(Engine *const *Es, int nE, const bool *with_mag);
int split_emf_m(Engine *const *Es, int nE);
int split_mag_m(Engine *const *Es, int nE, bool ab3_coef, bool spectra_done);
int split_bandj_m(Engine *const *Es, int nE, bool rotate_hist);
int split_ab3_m(Engine *const *Es, int nE, const int *magdealias, const bool *folded);
int split_dealias_m(Engine *const *Es, int nE);
int split_sync_b64_m(Engine *const *Es, int nE);
int split_calcdt_m(Engine *const *Es, int nE);
// capi.cu: one graph step of a batch (no diagnostics, no profiling), and
// whether two contexts can share a batch
int engine_enqueue_step_batch(Engine *const *Es, int nE);
bool engine_batchable(const Engine &a, const Engine &b);
