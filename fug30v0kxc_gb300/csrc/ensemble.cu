// ensemble.cu -- many independent instances (uneven grids and parameters)
// stepped together as one captured CUDA graph.
//
// Every member is a full context (its own arrays and stream).  One ensemble
// step is captured once per step variant (plain, or the tenth step with
// dealias and calcdt).  Members of one grid (and the same kernel forms and
// tile choices) form batches of up to BATCH_MAX: every kernel of the step is
// one launch over all members of a batch (blockIdx.z picks the member, the
// line kernels take all members' jobs), so the ensemble step is a few
// launches per grid rather than per member.  The root stream forks to each
// batch (and each member that fits no batch) through an event and joins them
// again, so the graph holds one branch per batch and the GPU runs them
// concurrently.  Steps with diagnostics (a host read-back) run without the
// graph, member by member.
//
// The autotuner picks, per distinct grid, the planes per z chunk of hydro
// pass 2 and the sequences per tile of the line kernels by
// timing a scratch context of that grid; results can be cached in a text
// file (one line per grid: nx ny nz precision kc s).
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "common.cuh"
#include "engine.h"

struct vec_ens {
    std::vector<vec_ctx *> m;
    cudaStream_t root = nullptr;
    cudaEvent_t ev_root = nullptr;
    std::vector<cudaEvent_t> ev;
    cudaGraphExec_t g[2] = { nullptr, nullptr };
    std::vector<int> b32_after[2];
    std::vector<long long> launches[2];
};

static void drop(vec_ens *e)
{
    for (int v = 0; v < 2; v++)
        if (e->g[v]) { cudaGraphExecDestroy(e->g[v]); e->g[v] = nullptr; }
}

extern "C" int vec_ensemble_destroy(vec_ens *e)
{
    if (!e) return VEC_OK;
    if (e->root) cudaStreamSynchronize(e->root);
    drop(e);
    for (auto c : e->m) vec_destroy(c);
    for (auto ev : e->ev) cudaEventDestroy(ev);
    if (e->ev_root) cudaEventDestroy(e->ev_root);
    if (e->root) cudaStreamDestroy(e->root);
    delete e;
    return VEC_OK;
}

extern "C" int vec_ensemble_create(const vec_params *ps, int n, vec_ens **out)
{
    if (!ps || n <= 0 || !out) return VEC_ERR_ARG;
    *out = nullptr;
    vec_ens *e = new vec_ens();
    for (int i = 0; i < n; i++) {
        vec_ctx *c = nullptr;
        int st = vec_create(&ps[i], &c);
        if (st) { vec_ensemble_destroy(e); return st; }
        e->m.push_back(c);
        cudaEvent_t ev;
        if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) { vec_ensemble_destroy(e); return VEC_ERR_CUDA; }
        e->ev.push_back(ev);
    }
    if (cudaStreamCreateWithFlags(&e->root, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->ev_root, cudaEventDisableTiming) != cudaSuccess) {
        vec_ensemble_destroy(e);
        return VEC_ERR_CUDA;
    }
    for (int v = 0; v < 2; v++) { e->b32_after[v].assign(n, 0); e->launches[v].assign(n, 0); }
    *out = e;
    return VEC_OK;
}

extern "C" int vec_ensemble_size(vec_ens *e) { return e ? (int)e->m.size() : 0; }

extern "C" vec_ctx *vec_ensemble_member(vec_ens *e, int i)
{
    if (!e || i < 0 || i >= (int)e->m.size()) return nullptr;
    return e->m[i];
}

// static state, calcdt and mag_init of every member (src/main.F90:275-333)
extern "C" int vec_ensemble_start(vec_ens *e)
{
    if (!e) return VEC_ERR_ARG;
    drop(e);
    for (auto c : e->m) {
        int st;
        if ((st = vec_static(c))) return st;
        if ((st = vec_calcdt(c, nullptr))) return st;
        Engine &E = engine_of(c);
        if ((E.p.f != 0.0 || E.p.kinematic) && (st = vec_mag_init(c))) return st;
    }
    return VEC_OK;
}

// Work on the member streams must follow the graph replays queued on the
// root stream, and later replays must follow it: join in both directions.
static int root_to_members(vec_ens *e)
{
    CUDA_TRY(cudaEventRecord(e->ev_root, e->root));
    for (auto c : e->m) CUDA_TRY(cudaStreamWaitEvent(engine_of(c).stream, e->ev_root, 0));
    return VEC_OK;
}

static int members_to_root(vec_ens *e)
{
    for (size_t i = 0; i < e->m.size(); i++) {
        CUDA_TRY(cudaEventRecord(e->ev[i], engine_of(e->m[i]).stream));
        CUDA_TRY(cudaStreamWaitEvent(e->root, e->ev[i], 0));
    }
    return VEC_OK;
}

static int ens_eager_step(vec_ens *e)
{
    int st = root_to_members(e);
    if (st) return st;
    for (auto c : e->m) {
        if ((st = engine_one_step(engine_of(c)))) return st;
    }
    return members_to_root(e);
}

extern "C" int vec_ensemble_step(vec_ens *e, int nsteps)
{
    if (!e || nsteps < 0) return VEC_ERR_ARG;
    const int nm = (int)e->m.size();
    int st0 = members_to_root(e);
    if (st0) return st0;
    bool cdt = false;
    for (int s = 0; s < nsteps; s++) {
        // all members advance together, so they share nit
        const int nit = engine_of(e->m[0]).nit + 1;
        cdt = cdt || nit % 10 == 0;
        bool eager = false;
        for (auto c : e->m) {
            Engine &E = engine_of(c);
            if (E.nit + 1 != nit || engine_diag_due(E, nit) || E.prof_on || !E.use_graphs) eager = true;
        }
        if (eager) {
            int st = ens_eager_step(e);
            if (st) return st;
            continue;
        }
        const int v = nit % 10 == 0 ? 1 : 0;
        if (!e->g[v]) {
            // members that can share launches form batches of up to
            // BATCH_MAX (one grid, one launch per kernel for all of them);
            // each batch, and each other member, is one branch of the graph
            std::vector<std::vector<int>> groups;
            for (int i = 0; i < nm; i++) {
                Engine &E = engine_of(e->m[i]);
                bool placed = false;
                for (auto &g : groups) {
                    Engine &L = engine_of(e->m[g[0]]);
                    if ((int)g.size() < BATCH_MAX && engine_batchable(L, E)) { g.push_back(i); placed = true; break; }
                }
                if (!placed) groups.push_back(std::vector<int>{ i });
            }
            CUDA_TRY(cudaStreamBeginCapture(e->root, cudaStreamCaptureModeThreadLocal));
            int st = VEC_OK;
            if (cudaEventRecord(e->ev_root, e->root) != cudaSuccess) st = VEC_ERR_CUDA;
            for (size_t gi = 0; gi < groups.size() && !st; gi++) {
                const std::vector<int> &g = groups[gi];
                Engine &L = engine_of(e->m[g[0]]);
                if (cudaStreamWaitEvent(L.stream, e->ev_root, 0) != cudaSuccess) { st = VEC_ERR_CUDA; break; }
                Engine *Es[BATCH_MAX];
                long long l0[BATCH_MAX];
                for (size_t q = 0; q < g.size(); q++) {
                    Engine &E = engine_of(e->m[g[q]]);
                    E.nit += 1;
                    E.iter += 1;
                    l0[q] = E.launches;
                    Es[q] = &E;
                }
                st = g.size() == 1 ? engine_enqueue_step(L, false) : engine_enqueue_step_batch(Es, (int)g.size());
                for (size_t q = 0; q < g.size(); q++) {
                    e->b32_after[v][g[q]] = Es[q]->b32_auth;
                    e->launches[v][g[q]] = Es[q]->launches - l0[q];
                }
                if (!st && cudaEventRecord(e->ev[g[0]], L.stream) != cudaSuccess) st = VEC_ERR_CUDA;
                if (!st && cudaStreamWaitEvent(e->root, e->ev[g[0]], 0) != cudaSuccess) st = VEC_ERR_CUDA;
            }
            cudaGraph_t g = nullptr;
            cudaError_t ce = cudaStreamEndCapture(e->root, &g);
            if (st) { if (g) cudaGraphDestroy(g); return st; }
            if (ce != cudaSuccess) { vec_set_error("ensemble capture failed: %s", cudaGetErrorString(ce)); return VEC_ERR_CUDA; }
            ce = cudaGraphInstantiate(&e->g[v], g, 0);
            cudaGraphDestroy(g);
            if (ce != cudaSuccess) { vec_set_error("ensemble instantiate failed: %s", cudaGetErrorString(ce)); return VEC_ERR_CUDA; }
        } else {
            for (int i = 0; i < nm; i++) {
                Engine &E = engine_of(e->m[i]);
                E.nit += 1;
                E.iter += 1;
                E.b32_auth = e->b32_after[v][i];
                E.launches += e->launches[v][i];
            }
        }
        CUDA_TRY(cudaGraphLaunch(e->g[v], e->root));
    }
    // whatever the caller does next on a member's stream follows the steps
    int st = root_to_members(e);
    if (st || !cdt) return st;
    // the non-finite check of the calcdt reductions: one 4-byte read-back
    // per member, then one wait per member stream
    for (auto c : e->m) {
        Engine &E = engine_of(c);
        CUDA_TRY(cudaMemcpyAsync(&E.hs->nonfinite, &E.ds->nonfinite, sizeof(int), cudaMemcpyDeviceToHost, E.stream));
    }
    for (int i = 0; i < nm; i++) {
        Engine &E = engine_of(e->m[i]);
        CUDA_TRY(cudaStreamSynchronize(E.stream));
        if (E.hs->nonfinite) {
            vec_set_error("ensemble member %d: non-finite value in the state (calcdt of the time loop)", i);
            return VEC_ERR_NAN;
        }
    }
    return VEC_OK;
}

extern "C" int vec_ensemble_sync(vec_ens *e)
{
    if (!e) return VEC_ERR_ARG;
    CUDA_TRY(cudaStreamSynchronize(e->root));
    for (auto c : e->m) {
        int st = vec_sync(c);
        if (st) return st;
    }
    return VEC_OK;
}

// ---- autotuner -------------------------------------------------------------------
struct TuneKey { int nx, ny, nz, prec; };

static bool same(const TuneKey &a, const TuneKey &b)
{
    return a.nx == b.nx && a.ny == b.ny && a.nz == b.nz && a.prec == b.prec;
}

static int time_config(const vec_params &p, int kc, int s, int steps, float *ms)
{
    vec_ctx *c = nullptr;
    int st = vec_create(&p, &c);
    if (st) return st;
    Engine &E = engine_of(c);
    E.kc_pass2 = kc;
    E.ct_s = s;
    cudaEvent_t a = nullptr, b = nullptr;
    if ((st = vec_static(c)) || (st = vec_calcdt(c, nullptr))) goto out;
    if ((p.f != 0.0 || p.kinematic) && (st = vec_mag_init(c))) goto out;
    if ((st = vec_step(c, 2)) || (st = vec_sync(c))) goto out;   // warm-up and graph capture
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, E.stream);
    if ((st = vec_step(c, steps))) goto out;
    cudaEventRecord(b, E.stream);
    if ((st = vec_sync(c))) goto out;
    cudaEventElapsedTime(ms, a, b);
out:
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    vec_destroy(c);
    return st;
}

// Picks kc (z-marching chunk) and s (sequences per line tile) per distinct
// grid of the ensemble; cache: optional text file read first and rewritten.
extern "C" int vec_ensemble_tune(vec_ens *e, int steps, const char *cache)
{
    if (!e || steps <= 0) return VEC_ERR_ARG;
    struct Entry { TuneKey k; int kc, s; };
    std::vector<Entry> tab;
    if (cache) {
        FILE *fp = fopen(cache, "r");
        if (fp) {
            Entry t;
            while (fscanf(fp, "%d %d %d %d %d %d", &t.k.nx, &t.k.ny, &t.k.nz, &t.k.prec, &t.kc, &t.s) == 6)
                tab.push_back(t);
            fclose(fp);
        }
    }
    for (auto c : e->m) {
        Engine &E = engine_of(c);
        TuneKey k = { E.nx, E.ny, E.nz, E.p.precision };
        const Entry *hit = nullptr;
        for (auto &t : tab) if (same(t.k, k)) { hit = &t; break; }
        if (!hit) {
            // planes per z chunk of hydro pass 2 (the z-pencil kernel's
            // chunk, or the z-marching kernel's where nx % 4 != 0)
            const int kcs[3] = { 8, 16, 32 };
            // sequences per tile: the register-FFT kernel's default, or its
            // alternative (8 for n <= 256, 4 for n >= 768); the generic
            // kernel's default, 4 or 8
            auto ct_len = [](int n) {
                return n == 64 || n == 96 || n == 128 || n == 192 || n == 256 || n == 384 || n == 512 || n == 768 ||
                       n == 1024;
            };
            std::vector<int> ss = { 0 };
            if (ct_len(E.nx) && ct_len(E.ny)) {
                if (E.nx <= 256 || E.ny <= 256) ss.push_back(8);
                if (E.nx >= 768 || E.ny >= 768) ss.push_back(4);
            } else {
                ss = { 0, 4, 8 };
            }
            Entry best = { k, 16, 0 };
            float best_ms = 1e30f;
            for (int kc : kcs)
                for (int s : ss) {
                    float ms = 0.0f;
                    int st = time_config(E.p, kc, s, steps, &ms);
                    if (st) return st;
                    if (ms < best_ms) { best_ms = ms; best.kc = kc; best.s = s; }
                }
            tab.push_back(best);
            hit = &tab.back();
        }
        E.kc_pass2 = hit->kc;
        E.ct_s = hit->s;
        E.drop_graphs();
    }
    drop(e);
    if (cache) {
        FILE *fp = fopen(cache, "w");
        if (fp) {
            for (auto &t : tab) fprintf(fp, "%d %d %d %d %d %d\n", t.k.nx, t.k.ny, t.k.nz, t.k.prec, t.kc, t.s);
            fclose(fp);
        }
    }
    return VEC_OK;
}

extern "C" int vec_tunables(vec_ctx *c, int *kc, int *s)
{
    if (!c) return VEC_ERR_ARG;
    Engine &E = engine_of(c);
    if (kc) *kc = E.kc_pass2;
    if (s) *s = E.ct_s;
    return VEC_OK;
}

extern "C" int vec_set_tunables(vec_ctx *c, int kc, int s)
{
    if (!c || (kc != 8 && kc != 16 && kc != 32) || (s != 0 && s != 4 && s != 8)) return VEC_ERR_ARG;
    Engine &E = engine_of(c);
    E.kc_pass2 = kc;
    E.ct_s = s;
    E.drop_graphs();   // captured steps hold the old launch shapes
    return VEC_OK;
}
