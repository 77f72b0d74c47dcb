// capi.cu -- the extern "C" boundary of include/vec.h.
//
// The context owns every device array (the module globals of
// src/arrays.f90:14-74), the spectral tables (src/fft.F90:60-80, 171-221)
// and the stencil scales (src/dbydz.F90:355-362).  Entry points accept host
// or device pointers; host buffers are staged through context scratch.
#include <ctype.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "common.cuh"
#include "engine.h"

struct vec_ctx {
    Engine E;
};

// ---- error string ------------------------------------------------------------
static thread_local char g_err[512] = "";

void vec_set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

extern "C" const char *vec_last_error(void) { return g_err; }

// ---- profiling ---------------------------------------------------------------------
void Engine::prof_begin(const char *name, double bytes)
{
    launches++;
    if (!prof_on) return;
    int rec = -1;
    for (size_t i = 0; i < prof.size(); i++)
        if (prof[i].name == name) { rec = (int)i; break; }
    if (rec < 0) {
        ProfRec r;
        r.name = name;
        prof.push_back(r);
        rec = (int)prof.size() - 1;
    }
    cudaEvent_t a, b;
    if (ev_pool.size() >= 2) {
        a = ev_pool.back(); ev_pool.pop_back();
        b = ev_pool.back(); ev_pool.pop_back();
    } else {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
    }
    cudaEventRecord(a, stream);
    prof_cur = rec;
    prof_a = a;
    Pending pd;
    pd.rec = rec; pd.a = a; pd.b = b; pd.bytes = bytes;
    pending.push_back(pd);
}

void Engine::prof_end()
{
    if (!prof_on || pending.empty()) return;
    cudaEventRecord(pending.back().b, stream);
}

int Engine::prof_flush()
{
    if (pending.empty()) return VEC_OK;
    CUDA_TRY(cudaStreamSynchronize(stream));
    for (auto &pd : pending) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, pd.a, pd.b);
        prof[pd.rec].launches += 1;
        prof[pd.rec].ms += ms;
        prof[pd.rec].bytes += pd.bytes;
        ev_pool.push_back(pd.a);
        ev_pool.push_back(pd.b);
    }
    pending.clear();
    return VEC_OK;
}

// ---- parameters ---------------------------------------------------------------
static double ck_from_ra(double ra, double theta, double cm, double sigma, double gamma)
{
    // src/initial.F90:194-196
    return sqrt((((cm + 1.0) * theta * theta) / (sigma * ra * gamma)) * (cm + 1.0 - (cm * gamma))
                * pow(1.0 + (0.5 * theta), (2.0 * cm) - 1.0));
}

extern "C" int vec_params_default(vec_params *p)
{
    if (!p) return VEC_ERR_ARG;
    memset(p, 0, sizeof(*p));
    // bin/INPUT
    p->gamma = 1.4; p->sigma = 1.0; p->theta = 10.0; p->cm = 1.0;
    p->tayl = 0.0; p->psi = 1.570796327; p->zeta = 0.2; p->xmax = 4.0; p->ymax = 4.0; p->sf = 0.2;
    p->rayl = 1.0e5; p->chand = 2500.0;
    p->ck = ck_from_ra(p->rayl, p->theta, p->cm, p->sigma, p->gamma);
    p->f = p->chand * (p->zeta * p->sigma * p->ck * p->ck);
    p->nx = 30; p->ny = 30; p->nz = 60;
    p->nframe = 0; p->ntotal = 50000; p->ndu06 = 5000; p->ndu16 = 10000; p->ndurestart = 10000;
    // src/main.F90:108-116
    p->dalias = 1; p->kinematic = 0; p->radbc = 0; p->constflux = 0; p->perfect = 0; p->dynamo = 0;
    // extensions (reference behaviour)
    p->eta_contrast = 1.0; p->noise_amp = 0.1; p->kappa_uniform = 0; p->seed_base = 1996;
    p->precision = VEC_PREC_FP64; p->diag_cadence = 1;
    return VEC_OK;
}

// next line of the file, first whitespace-separated token parsed as a number
static int read_value(FILE *fp, double *v)
{
    char line[512];
    if (!fgets(line, sizeof line, fp)) return -1;
    char *s = line;
    while (*s && isspace((unsigned char)*s)) s++;
    // Fortran list-directed input accepts d exponents
    for (char *c = s; *c && !isspace((unsigned char)*c); c++)
        if (*c == 'd' || *c == 'D') *c = 'e';
    char *end = NULL;
    *v = strtod(s, &end);
    return end == s ? -1 : 0;
}

extern "C" int vec_params_read_input(const char *path, vec_params *p)
{
    if (!path || !p) return VEC_ERR_ARG;
    vec_params_default(p);
    FILE *fp = fopen(path, "r");
    if (!fp) { vec_set_error("cannot open %s", path); return VEC_ERR_INPUT; }
    char line[512];
    double flag, v[20];
    int ok = fgets(line, sizeof line, fp) && fgets(line, sizeof line, fp) && read_value(fp, &flag) == 0
             && fgets(line, sizeof line, fp) && fgets(line, sizeof line, fp);
    for (int i = 0; ok && i < 20; i++) ok = read_value(fp, &v[i]) == 0;
    fclose(fp);
    if (!ok) { vec_set_error("malformed INPUT file %s", path); return VEC_ERR_INPUT; }
    // src/initial.F90:149-171
    p->gamma = v[0]; p->sigma = v[1]; p->theta = v[2]; p->ck = v[3]; p->cm = v[4]; p->f = v[5];
    p->tayl = v[6]; p->psi = v[7]; p->zeta = v[8]; p->xmax = v[9]; p->ymax = v[10]; p->sf = v[11];
    p->nframe = (int)v[12]; p->ntotal = (int)v[13]; p->ndu06 = (int)v[14]; p->ndu16 = (int)v[15];
    p->ndurestart = (int)v[16]; p->nx = (int)v[17]; p->ny = (int)v[18]; p->nz = (int)v[19];
    if ((int)flag == 1) {   // :174-185
        p->chand = p->f / (p->zeta * p->sigma * p->ck * p->ck);
        p->rayl = (((p->cm + 1.0) * p->theta * p->theta) / (p->sigma * p->ck * p->ck * p->gamma))
                  * (p->cm + 1.0 - (p->cm * p->gamma)) * pow(1.0 + (0.5 * p->theta), (2.0 * p->cm) - 1.0);
    } else if ((int)flag == 2) {   // :186-199
        p->rayl = p->ck;
        p->chand = p->f;
        p->ck = ck_from_ra(p->rayl, p->theta, p->cm, p->sigma, p->gamma);
        p->f = p->chand * (p->zeta * p->sigma * p->ck * p->ck);
    } else {
        vec_set_error("unknown input flag %d", (int)flag);
        return VEC_ERR_INPUT;
    }
    if (p->nframe < 0 || p->nframe > 2) { vec_set_error("unknown nframe %d", p->nframe); return VEC_ERR_INPUT; }
    return VEC_OK;
}

// ---- context -------------------------------------------------------------------
static void set_consts(Engine &E)
{
    const vec_params &p = E.p;
    Consts &c = E.k;
    memset(&c, 0, sizeof(c));
    // src/constants.f90:62-107
    c.dx = p.xmax / (double)E.nx;
    c.dy = p.ymax / (double)E.ny;
    c.dz = 1.0 / (double)(E.nz - 1);
    c.dd = c.dx < c.dy ? c.dx : c.dy;
    c.xn = 1.0 / (double)(E.nx * E.ny);
    c.xzn = c.dx * c.dy * c.dz;
    c.taylt = p.tayl / pow(1.0 + p.theta / 2.0, 2.0 * p.cm);
    c.cpsi = cos(p.psi);
    c.spsi = sin(p.psi);
    c.cor = p.ck * p.sigma * sqrt(c.taylt);
    c.gck = p.gamma * p.ck;
    c.sck = p.sigma * p.ck;
    c.zck = p.zeta * p.ck;
    c.scko3 = c.sck / 3.0;
    c.sckg = p.sigma * p.ck * (p.gamma - 1.0);
    c.fzckg = p.f * p.zeta * p.ck * (p.gamma - 1.0);
    c.thmplus1 = p.theta * (p.cm + 1.0);
    c.fo2 = p.f / 2.0;
    c.g1 = sqrt(p.gamma);
    c.gm1 = p.gamma - 1.0;
    c.nusstmp = p.theta * (p.cm + 1.0) * (1.0 - (1.0 / p.gamma));
    c.dtvisc0x = 0.1 * 0.75 * c.dd * c.dd / p.sigma / p.ck;
    c.dtvisc0z = 0.2 * c.dz * c.dz / p.sigma / p.ck * (1.0 + p.theta / 7.0);
    c.dtdiff0x = 0.1 * c.dd * c.dd / p.gamma / p.ck;
    c.dtdiff0z = 0.2 * c.dz * c.dz / p.gamma / p.ck * (1.0 + p.theta / 7.0);
    // src/dbydz.F90:360-361
    c.ho12 = (double)(E.nz - 1) / 12.0;
    c.sc1 = (double)((E.nz - 1) * (E.nz - 1)) / 12.0;
    c.f = p.f; c.gamma = p.gamma; c.theta = p.theta; c.sf = p.sf;
    c.var_eta = p.eta_contrast != 1.0;
    c.icutoffx = (E.nx / 2) / 3;
    c.icutoffy = (E.ny / 2) / 3;
}

static int dev_alloc(void **p, size_t bytes)
{
    if (cudaMalloc(p, bytes ? bytes : 16) != cudaSuccess) {
        cudaGetLastError();
        vec_set_error("cudaMalloc of %zu bytes failed", bytes);
        return VEC_ERR_ALLOC;
    }
    return cudaMemset(*p, 0, bytes ? bytes : 16) == cudaSuccess ? VEC_OK : VEC_ERR_CUDA;
}

#define ALLOC(ptr, bytes)                                              \
    do {                                                               \
        int s_ = dev_alloc((void **)&(ptr), (bytes));                  \
        if (s_) { vec_destroy(c); return s_; }                         \
    } while (0)

static int upload(double *d, const std::vector<double> &h)
{
    CUDA_TRY(cudaMemcpy(d, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice));
    return VEC_OK;
}

extern "C" int vec_create(const vec_params *p, vec_ctx **out)
{
    if (!p || !out) return VEC_ERR_ARG;
    *out = nullptr;
    if (p->nx < 4 || p->nx % 2) { vec_set_error("nx must be even and >= 4"); return VEC_ERR_NX; }
    if (p->ny < 4 || p->ny % 2) { vec_set_error("ny must be even and >= 4"); return VEC_ERR_NY; }
    if (p->nz < 6) { vec_set_error("nz must be >= 6"); return VEC_ERR_NZ; }
    if (p->precision != VEC_PREC_FP64 && p->precision != VEC_PREC_SPLIT) return VEC_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        vec_set_error("no CUDA device");
        return VEC_ERR_CUDA;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    static bool configured[64] = {};
    if (dev >= 0 && dev < 64 && !configured[dev]) {
        int st = line_kernels_configure();
        if (st) return st;
        configured[dev] = true;
    }
    vec_ctx *c = new vec_ctx();
    Engine &E = c->E;
    E.p = *p;
    E.nx = p->nx; E.ny = p->ny; E.nz = p->nz;
    E.np = (size_t)E.nx * E.ny;
    E.n = E.np * E.nz;
    E.split = p->precision == VEC_PREC_SPLIT;
    cudaDeviceGetAttribute(&E.num_sms, cudaDevAttrMultiProcessorCount, dev);
    {
        const char *g = getenv("VEC_GENERIC_LINES");
        E.generic_lines = g && g[0] == '1';
        const char *cw = getenv("VEC_CT_WARP");
        E.ct_warp = !(cw && cw[0] == '0');
        const char *pk = getenv("VEC_PROF_KINDS");
        E.prof_kinds = pk && pk[0] == '1';
        const char *pd = getenv("VEC_PDL");
        E.pdl = !(pd && pd[0] == '0');
        const char *v4 = getenv("VEC_VEC4");
        E.vec4 = !(v4 && v4[0] == '0');
        const char *hc = getenv("VEC_HW_CVT");
        E.int_cvt = !(hc && hc[0] == '1');
        const char *zp = getenv("VEC_ZPENCIL");
        E.zpencil = !(zp && zp[0] == '0');
        const char *z4 = getenv("VEC_ZPENCIL4");
        E.zpencil4 = z4 && (z4[0] == '0' || z4[0] == '1') ? z4[0] - '0' : -1;
    }
    set_consts(E);
    int st;
    if ((st = line_plan_make(E.nx, E.ny, 8, &E.plx)) || (st = line_plan_make(E.ny, E.nx, 8, &E.ply))) {
        vec_set_error("line lengths nx=%d ny=%d are not supported (2^a 3^b 5^c <= 2048)", E.nx, E.ny);
        delete c;
        return st;
    }
    if (cudaStreamCreateWithFlags(&E.stream2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&E.ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&E.ev_join, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return VEC_ERR_CUDA;
    }
    {
        // mag_deriv beside hydro_deriv on a second stream pays off in the FP64
        // form (FP64-pipe bound kernels overlap); in the split form both are
        // HBM bound and the overlap costs more in L2 and DRAM contention than
        // it hides (1.75 against 1.67 ms per 256^2x129 step).  VEC_SERIAL_MAG
        // = 1 / 0 forces one or the other.
        const char *sm = getenv("VEC_SERIAL_MAG");
        E.par_mag = sm ? !(sm[0] == '1') : !E.split;
    }
    if (cudaStreamCreateWithFlags(&E.stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return VEC_ERR_CUDA;
    }
    const size_t n = E.n, nz = E.nz;
    // wavenumbers, src/fft.F90:171-221
    std::vector<double> akx1(E.nx, 0.0), akx2(E.nx, 0.0), aky1(E.ny, 0.0), aky2(E.ny, 0.0);
    {
        double cx = 8.0 * atan(1.0) / p->xmax, cy = 8.0 * atan(1.0) / p->ymax;
        for (int i = 1; i <= E.nx / 2 - 1; i++) {
            akx1[i] = (double)i * cx; akx1[E.nx - i] = (double)i * cx;
            akx2[i] = -(double)i * (double)i * cx * cx; akx2[E.nx - i] = -(double)i * (double)i * cx * cx;
        }
        akx2[E.nx / 2] = -(double)(E.nx / 2) * (double)(E.nx / 2) * cx * cx;
        for (int i = 1; i <= E.ny / 2 - 1; i++) {
            aky1[i] = (double)i * cy; aky1[E.ny - i] = (double)i * cy;
            aky2[i] = -(double)i * (double)i * cy * cy; aky2[E.ny - i] = -(double)i * (double)i * cy * cy;
        }
        aky2[E.ny / 2] = -(double)(E.ny / 2) * (double)(E.ny / 2) * cy * cy;
    }
    if ((st = line_tables_make<double>(E.nx, akx1.data(), akx2.data(), E.k.icutoffx, &E.tx64)) ||
        (st = line_tables_make<double>(E.ny, aky1.data(), aky2.data(), E.k.icutoffy, &E.ty64)) ||
        (st = line_tables_make<float>(E.nx, akx1.data(), akx2.data(), E.k.icutoffx, &E.tx32)) ||
        (st = line_tables_make<float>(E.ny, aky1.data(), aky2.data(), E.k.icutoffy, &E.ty32))) {
        vec_destroy(c);
        return st;
    }
    ALLOC(E.akx1, sizeof(double) * E.nx); ALLOC(E.akx2, sizeof(double) * E.nx);
    ALLOC(E.aky1, sizeof(double) * E.ny); ALLOC(E.aky2, sizeof(double) * E.ny);
    if (upload(E.akx1, akx1) || upload(E.akx2, akx2) || upload(E.aky1, aky1) || upload(E.aky2, aky2)) {
        vec_destroy(c);
        return VEC_ERR_CUDA;
    }
    {
        // the wavenumber tables per precision; kh2 = akx2[i] + aky2[j] per plane point
        std::vector<double> kh2(E.np);
        std::vector<float> kx1f(E.nx), ky1f(E.ny), kh2f(E.np), kh2if(E.np);
        for (int j = 0; j < E.ny; j++)
            for (int i = 0; i < E.nx; i++) {
                const size_t q = (size_t)j * E.nx + i;
                kh2[q] = akx2[i] + aky2[j];
                kh2f[q] = (float)kh2[q];
                kh2if[q] = q == 0 ? 0.0f : (float)(1.0 / kh2[q]);
            }
        for (int i = 0; i < E.nx; i++) kx1f[i] = (float)akx1[i];
        for (int j = 0; j < E.ny; j++) ky1f[j] = (float)aky1[j];
        float *fx = nullptr, *fy = nullptr, *fk = nullptr, *fki = nullptr;
        double *dk = nullptr;
        ALLOC(fx, sizeof(float) * E.nx); E.hf.kx1 = fx;
        ALLOC(fy, sizeof(float) * E.ny); E.hf.ky1 = fy;
        ALLOC(fk, sizeof(float) * E.np); E.hf.kh2 = fk;
        ALLOC(fki, sizeof(float) * E.np); E.hf.kh2inv = fki;
        E.hd.kh2inv = nullptr;
        ALLOC(dk, sizeof(double) * E.np); E.hd.kh2 = dk;
        E.hd.kx1 = E.akx1;
        E.hd.ky1 = E.aky1;
        if (cudaMemcpy(fx, kx1f.data(), sizeof(float) * E.nx, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(fy, ky1f.data(), sizeof(float) * E.ny, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(fk, kh2f.data(), sizeof(float) * E.np, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(fki, kh2if.data(), sizeof(float) * E.np, cudaMemcpyHostToDevice) != cudaSuccess ||
            upload(dk, kh2)) {
            vec_destroy(c);
            return VEC_ERR_CUDA;
        }
    }
    // kappa(z): src/trans_params.f90:36-62; eta(z): the extension
    std::vector<double> kap(nz), dkap(nz), eta(nz), deta(nz);
    double emax = 0.0;
    for (int k = 0; k < E.nz; k++) {
        double z = (double)k * E.k.dz;
        if (p->kappa_uniform) { kap[k] = 1.0; dkap[k] = 0.0; }
        else {
            double constB = 10.0 * (z - 5.0e-1);
            kap[k] = 5.0e-1 * (tanh(constB) + 1);
            dkap[k] = 5.0e-1 * 10.0 * pow(cosh(constB), -2.0);
        }
        eta[k] = E.k.zck * (1.0 + (p->eta_contrast - 1.0) * z);
        deta[k] = E.k.zck * (p->eta_contrast - 1.0);
        emax = eta[k] > emax ? eta[k] : emax;
    }
    E.k.eta_max = emax;
    ALLOC(E.kappa, sizeof(double) * nz); ALLOC(E.dkappa, sizeof(double) * nz);
    ALLOC(E.eta, sizeof(double) * nz); ALLOC(E.deta, sizeof(double) * nz);
    if (upload(E.kappa, kap) || upload(E.dkappa, dkap) || upload(E.eta, eta) || upload(E.deta, deta)) {
        vec_destroy(c);
        return VEC_ERR_CUDA;
    }
    // state
    double **st64[] = { &E.r, &E.t, &E.u, &E.v, &E.w, &E.bx, &E.by, &E.bz, &E.jsq, &E.pol, &E.tor };
    for (auto pp : st64) ALLOC(*pp, sizeof(double) * n);
    const size_t esz = E.split ? sizeof(float) : sizeof(double);
    for (int f = 0; f < 7; f++)
        for (int s = 0; s < 3; s++) ALLOC(E.hbuf[f][s], esz * n);
    ALLOC(E.bxbar, sizeof(double) * nz); ALLOC(E.bybar, sizeof(double) * nz);
    for (int s = 0; s < 3; s++) { ALLOC(E.bxd_buf[s], sizeof(double) * nz); ALLOC(E.byd_buf[s], sizeof(double) * nz); }
    {
        HistTable h;
        for (int f = 0; f < 7; f++) for (int s = 0; s < 3; s++) h.p[f][s] = E.hbuf[f][s];
        for (int s = 0; s < 3; s++) { h.bx[s] = E.bxd_buf[s]; h.by[s] = E.byd_buf[s]; }
        ALLOC(E.ht, sizeof(HistTable));
        CUDA_TRY(cudaMemcpy(E.ht, &h, sizeof(h), cudaMemcpyHostToDevice));
    }
    ALLOC(E.w1d, sizeof(double) * 8 * nz);
    ALLOC(E.wblock, esz * n * W_COUNT);
    for (int i = 0; i < W_COUNT; i++) E.wk[i] = (char *)E.wblock + esz * n * (size_t)i;
    for (int i = 0; i < 3; i++) ALLOC(E.s64[i], sizeof(double) * n);
    E.red_blocks = 152 * 4;
    ALLOC(E.red, sizeof(double) * ((size_t)nz * 8 + 8 + (size_t)E.red_blocks * 25 + 64));
    ALLOC(E.ds, sizeof(DevScalars));
    ALLOC(E.cdt, sizeof(float) * (4 + 3 * (size_t)cdt_chunks(E.n)));
    if ((st = cdt_init(E.cdt))) { vec_destroy(c); return st; }
    ALLOC(E.dev_err, sizeof(int) * 4);
    if (cudaMallocHost(&E.hs, sizeof(DevScalars)) != cudaSuccess) { vec_destroy(c); return VEC_ERR_ALLOC; }
    memset(E.hs, 0, sizeof(DevScalars));
    E.hs->first = 1;
    E.hs->velmxx = OKEY_NEG_HUGE;
    E.hs->velmxz = OKEY_NEG_HUGE;
    E.hs->denmn = OKEY_POS_HUGE;
    CUDA_TRY(cudaMemcpy(E.ds, E.hs, sizeof(DevScalars), cudaMemcpyHostToDevice));
    if (E.split && (st = split_setup(&E))) { vec_destroy(c); return st; }
    CUDA_TRY(cudaDeviceSynchronize());
    *out = c;
    return VEC_OK;
}

extern "C" int vec_destroy(vec_ctx *c)
{
    if (!c) return VEC_OK;
    Engine &E = c->E;
    if (E.stream) cudaStreamSynchronize(E.stream);
    E.drop_graphs();
    void *ptrs[] = { E.r, E.t, E.u, E.v, E.w, E.bx, E.by, E.bz, E.jsq, E.pol, E.tor, E.bxbar, E.bybar,
                     E.kappa, E.dkappa, E.eta, E.deta, E.akx1, E.akx2, E.aky1, E.aky2, E.w1d, E.red, E.ds, E.dev_err, E.cdt,
                     E.r32, E.t32, E.u32, E.v32, E.w32, E.bx32, E.by32, E.bz32, E.jsq32, E.pol32, E.tor32,
                     E.rho0, E.t0, E.hres, E.corr, E.corr_bx };
    for (void *q : ptrs) if (q) cudaFree(q);
    const void *tabs[] = { E.hf.kx1, E.hf.ky1, E.hf.kh2, E.hf.kh2inv, E.hd.kh2, E.pcf };
    for (const void *q : tabs) if (q) cudaFree((void *)q);
    for (int f = 0; f < 7; f++) for (int s = 0; s < 3; s++) if (E.hbuf[f][s]) cudaFree(E.hbuf[f][s]);
    for (int s = 0; s < 3; s++) { if (E.bxd_buf[s]) cudaFree(E.bxd_buf[s]); if (E.byd_buf[s]) cudaFree(E.byd_buf[s]); }
    if (E.ht) cudaFree(E.ht);
    if (E.wblock) cudaFree(E.wblock);
    for (int i = 0; i < 6; i++) if (E.s64[i]) cudaFree(E.s64[i]);
    if (E.tx64.tw) line_tables_free(&E.tx64);
    if (E.ty64.tw) line_tables_free(&E.ty64);
    if (E.tx32.tw) line_tables_free(&E.tx32);
    if (E.ty32.tw) line_tables_free(&E.ty32);
    if (E.hs) cudaFreeHost(E.hs);
    for (auto &pd : E.pending) { cudaEventDestroy(pd.a); cudaEventDestroy(pd.b); }
    for (auto ev : E.ev_pool) cudaEventDestroy(ev);
    if (E.stream2) { cudaStreamSynchronize(E.stream2); cudaStreamDestroy(E.stream2); }
    if (E.ev_fork) cudaEventDestroy(E.ev_fork);
    if (E.ev_join) cudaEventDestroy(E.ev_join);
    if (E.stream) cudaStreamDestroy(E.stream);
    delete c;
    return VEC_OK;
}

extern "C" void *vec_stream(vec_ctx *c) { return c ? (void *)c->E.stream : nullptr; }

extern "C" int vec_sync(vec_ctx *c)
{
    if (!c) return VEC_ERR_ARG;
    CUDA_TRY(cudaStreamSynchronize(c->E.stream));
    int err = 0;
    CUDA_TRY(cudaMemcpy(&err, c->E.dev_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
        // reported once: the flag is cleared, the context stays usable
        CUDA_TRY(cudaMemset(c->E.dev_err, 0, sizeof(int)));
        vec_set_error(err == 2 ? "a bounded device wait ran out (wait self-test)"
                               : "a bounded device wait ran out (TMA tile load did not complete)");
        return VEC_ERR_CUDA;
    }
    return VEC_OK;
}

// ---- host/device staging ---------------------------------------------------------
static bool is_device_ptr(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// copy count doubles from src (host or device) into device dst
static int stage_in(Engine &E, double *dst, const double *src, size_t count)
{
    CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(double) * count,
                             is_device_ptr(src) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, E.stream));
    return VEC_OK;
}
static int stage_out(Engine &E, double *dst, const double *src, size_t count)
{
    CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(double) * count,
                             is_device_ptr(dst) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, E.stream));
    CUDA_TRY(cudaStreamSynchronize(E.stream));
    return VEC_OK;
}

// ---- state I/O ------------------------------------------------------------------
static int hist_index(int field, int *f, int *s)
{
    if (field < VEC_F_RDOT || field >= VEC_F_COUNT) return -1;
    *f = (field - VEC_F_RDOT) / 3;
    *s = (field - VEC_F_RDOT) % 3;
    return 0;
}

static double *state_ptr(Engine &E, int field)
{
    switch (field) {
    case VEC_F_R: return E.r; case VEC_F_T: return E.t; case VEC_F_U: return E.u;
    case VEC_F_V: return E.v; case VEC_F_W: return E.w; case VEC_F_BX: return E.bx;
    case VEC_F_BY: return E.by; case VEC_F_BZ: return E.bz; case VEC_F_JSQ: return E.jsq;
    case VEC_F_POL: return E.pol; case VEC_F_TOR: return E.tor;
    }
    return nullptr;
}

__global__ void k_f2d(const float *a, double *b, size_t n)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (double)a[i];
}
__global__ void k_d2f(const double *a, float *b, size_t n)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

extern "C" int vec_set_field(vec_ctx *c, int field, const double *src)
{
    if (!c || !src) return VEC_ERR_ARG;
    Engine &E = c->E;
    double *d = state_ptr(E, field);
    if (d) {
        int st;
        if (E.split && (st = split_sync_b64(&E))) return st;
        if ((st = stage_in(E, d, src, E.n))) return st;
        if (E.split && (st = split_refresh_field(&E, field))) return st;
        CUDA_TRY(cudaStreamSynchronize(E.stream));
        return VEC_OK;
    }
    int f, s;
    if (hist_index(field, &f, &s)) return VEC_ERR_ARG;
    HistTable h;
    int st = hist_table_host(&E, &h);
    if (st) return st;
    if (!E.split) return stage_in(E, (double *)h.p[f][s], src, E.n) ? VEC_ERR_CUDA : vec_sync(c);
    if ((st = stage_in(E, E.s64[0], src, E.n))) return st;
    k_d2f<<<(unsigned)((E.n + 255) / 256), 256, 0, E.stream>>>(E.s64[0], (float *)h.p[f][s], E.n);
    return vec_sync(c);
}

extern "C" int vec_get_field(vec_ctx *c, int field, double *dst)
{
    if (!c || !dst) return VEC_ERR_ARG;
    Engine &E = c->E;
    double *d = state_ptr(E, field);
    if (d) {
        int st;
        if (E.split && (st = split_sync_b64(&E))) return st;
        return stage_out(E, dst, d, E.n);
    }
    int f, s;
    if (hist_index(field, &f, &s)) return VEC_ERR_ARG;
    HistTable h;
    int st = hist_table_host(&E, &h);
    if (st) return st;
    if (!E.split) return stage_out(E, dst, (const double *)h.p[f][s], E.n);
    k_f2d<<<(unsigned)((E.n + 255) / 256), 256, 0, E.stream>>>((const float *)h.p[f][s], E.s64[0], E.n);
    return stage_out(E, dst, E.s64[0], E.n);
}

static double *mean_ptr(Engine &E, int m)
{
    switch (m) {
    case VEC_M_BXBAR: return E.bxbar; case VEC_M_BYBAR: return E.bybar;
    case VEC_M_KAPPA: return E.kappa; case VEC_M_DKAPPA: return E.dkappa;
    case VEC_M_ETA: return E.eta; case VEC_M_DETA: return E.deta;
    }
    if ((m >= VEC_M_BXBARDOT && m < VEC_M_BXBARDOT + 3) || (m >= VEC_M_BYBARDOT && m < VEC_M_BYBARDOT + 3)) {
        HistTable h;
        if (hist_table_host(&E, &h)) return nullptr;
        if (m < VEC_M_BYBARDOT) return h.bx[m - VEC_M_BXBARDOT];
        return h.by[m - VEC_M_BYBARDOT];
    }
    return nullptr;
}

extern "C" int vec_set_mean(vec_ctx *c, int m, const double *src)
{
    if (!c || !src) return VEC_ERR_ARG;
    double *d = mean_ptr(c->E, m);
    if (!d) return VEC_ERR_ARG;
    int st = stage_in(c->E, d, src, c->E.nz);
    if (!st && c->E.split && (m == VEC_M_KAPPA || m == VEC_M_DKAPPA || m == VEC_M_ETA || m == VEC_M_DETA))
        st = split_refresh_coefs(&c->E);   // their FP32 per-plane copies
    return st ? st : vec_sync(c);
}

extern "C" int vec_get_mean(vec_ctx *c, int m, double *dst)
{
    if (!c || !dst) return VEC_ERR_ARG;
    double *d = mean_ptr(c->E, m);
    if (!d) return VEC_ERR_ARG;
    return stage_out(c->E, dst, d, c->E.nz);
}

extern "C" int vec_set_bzbar(vec_ctx *c, double b)
{
    if (!c) return VEC_ERR_ARG;
    int st;
    if (c->E.split && (st = split_sync_b64(&c->E))) return st;
    c->E.bzbar = b;
    c->E.drop_graphs();
    if (c->E.split && (st = split_refresh(&c->E))) return st;
    return vec_sync(c);
}
extern "C" int vec_get_bzbar(vec_ctx *c, double *b) { if (!c || !b) return VEC_ERR_ARG; *b = c->E.bzbar; return VEC_OK; }

extern "C" int vec_get_scalars(vec_ctx *c, vec_scalars *s)
{
    if (!c || !s) return VEC_ERR_ARG;
    Engine &E = c->E;
    CUDA_TRY(cudaMemcpyAsync(E.hs, E.ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, E.stream));
    CUDA_TRY(cudaStreamSynchronize(E.stream));
    s->dt = E.hs->dt; s->dt1 = E.hs->dt1; s->dt2 = E.hs->dt2; s->ttime = E.hs->ttime;
    s->iter = E.iter; s->nit = E.nit; s->first = E.hs->first; s->second = E.hs->second;
    return VEC_OK;
}

extern "C" int vec_set_scalars(vec_ctx *c, const vec_scalars *s)
{
    if (!c || !s) return VEC_ERR_ARG;
    Engine &E = c->E;
    CUDA_TRY(cudaMemcpyAsync(E.hs, E.ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, E.stream));
    CUDA_TRY(cudaStreamSynchronize(E.stream));
    E.hs->dt = s->dt; E.hs->dt1 = s->dt1; E.hs->dt2 = s->dt2; E.hs->ttime = s->ttime;
    E.hs->first = s->first; E.hs->second = s->second;
    E.iter = s->iter; E.nit = s->nit;
    CUDA_TRY(cudaMemcpyAsync(E.ds, E.hs, sizeof(DevScalars), cudaMemcpyHostToDevice, E.stream));
    CUDA_TRY(cudaStreamSynchronize(E.stream));
    return VEC_OK;
}

// ---- set-up ---------------------------------------------------------------------
extern "C" int vec_static(vec_ctx *c)
{
    if (!c) return VEC_ERR_ARG;
    c->E.b32_auth = 0;
    int st = phys_static(&c->E);
    if (st) return st;
    if (c->E.split) return split_refresh(&c->E);
    return VEC_OK;
}

extern "C" int vec_calcdt(vec_ctx *c, double *dt)
{
    if (!c) return VEC_ERR_ARG;
    Engine &E = c->E;
    int st = E.split ? split_calcdt(&E) : phys_calcdt(&E);
    if (st) return st;
    CUDA_TRY(cudaMemcpyAsync(E.hs, E.ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, E.stream));
    CUDA_TRY(cudaStreamSynchronize(E.stream));
    if (dt) *dt = E.hs->dt;
    if (E.hs->nonfinite) {
        vec_set_error("non-finite value in the state (calcdt)");
        return VEC_ERR_NAN;
    }
    return VEC_OK;
}

extern "C" int vec_mag_init(vec_ctx *c)
{
    if (!c) return VEC_ERR_ARG;
    int st;
    if (c->E.split && (st = split_sync_b64(&c->E))) return st;
    c->E.drop_graphs();
    st = phys_mag_init(&c->E);
    if (st) return st;
    if (c->E.split && (st = split_refresh(&c->E))) return st;
    return vec_sync(c);
}

// ---- per-operator entry points (always FP64) --------------------------------------
static int line_op(vec_ctx *c, int dir, const double *fin, double *f1, int op1, double *f2, int op2)
{
    if (!c || !fin || !f1 || (op2 != OP_NONE && !f2)) return VEC_ERR_ARG;
    Engine &E = c->E;
    int st;
    if ((st = stage_in(E, E.s64[0], fin, E.n))) return st;
    LineJob<double> j = ljob<double>(E.s64[0], E.s64[1], op1, op2 != OP_NONE ? E.s64[2] : nullptr, op2);
    if ((st = launch_lines<double>(&E, dir, &j, 1))) return st;
    if ((st = stage_out(E, f1, E.s64[1], E.n))) return st;
    if (op2 != OP_NONE && (st = stage_out(E, f2, E.s64[2], E.n))) return st;
    return VEC_OK;
}

// FP32 line operators: the kernels the split form's time step runs, on
// caller data (host or device), through the context's scratch
extern "C" int vec_line_f32(vec_ctx *c, int dir, int op1, int op2, const float *fin, float *f1, float *f2)
{
    if (!c || !fin || !f1 || (dir != 0 && dir != 1)) return VEC_ERR_ARG;
    // second outputs: D1 or D2 of a real input, D1 of an inverse
    if (op1 < OP_D1 || op1 > OP_INV || (op2 != OP_NONE && (op2 < OP_D1 || op2 > OP_D2 || op1 == OP_FWD ||
                                                           (op1 == OP_INV && op2 != OP_D1) || !f2)))
        return VEC_ERR_ARG;
    Engine &E = c->E;
    // each FP64 scratch field holds 2n floats
    float *in = reinterpret_cast<float *>(E.s64[0]), *o1 = reinterpret_cast<float *>(E.s64[1]);
    float *o2 = reinterpret_cast<float *>(E.s64[2]);
    const size_t bytes = sizeof(float) * E.n;
    CUDA_TRY(cudaMemcpyAsync(in, fin, bytes, is_device_ptr(fin) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                             E.stream));
    LineJob<float> j = ljob<float>(in, o1, op1, op2 != OP_NONE ? o2 : nullptr, op2);
    int st = launch_lines<float>(&E, dir, &j, 1);
    if (st) return st;
    CUDA_TRY(cudaMemcpyAsync(f1, o1, bytes, is_device_ptr(f1) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                             E.stream));
    if (op2 != OP_NONE)
        CUDA_TRY(cudaMemcpyAsync(f2, o2, bytes, is_device_ptr(f2) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                 E.stream));
    return vec_sync(c);
}

extern "C" int vec_nc_write(const char *path, const vec_snapshot *s, int iprec);
extern "C" int vec_nc_read(const char *path, vec_snapshot *s);

extern "C" int vec_d1bydx(vec_ctx *c, const double *fin, double *fout) { return line_op(c, 0, fin, fout, OP_D1, nullptr, OP_NONE); }
extern "C" int vec_d1bydy(vec_ctx *c, const double *fin, double *fout) { return line_op(c, 1, fin, fout, OP_D1, nullptr, OP_NONE); }
extern "C" int vec_d2bydx(vec_ctx *c, const double *fin, double *a, double *b) { return line_op(c, 0, fin, a, OP_D1, b, OP_D2); }
extern "C" int vec_d2bydy(vec_ctx *c, const double *fin, double *a, double *b) { return line_op(c, 1, fin, a, OP_D1, b, OP_D2); }

extern "C" int vec_dealias(vec_ctx *c, double *z)
{
    if (!c || !z) return VEC_ERR_ARG;
    Engine &E = c->E;
    int st;
    if ((st = stage_in(E, E.s64[0], z, E.n))) return st;
    LineJob<double> j = ljob<double>(E.s64[0], E.s64[0], OP_DEALIAS);
    if ((st = launch_lines<double>(&E, 0, &j, 1)) || (st = launch_lines<double>(&E, 1, &j, 1))) return st;
    return stage_out(E, z, E.s64[0], E.n);
}

extern "C" int vec_forwardfft(vec_ctx *c, const double *fin, double *fout)
{
    if (!c || !fin || !fout) return VEC_ERR_ARG;
    Engine &E = c->E;
    int st;
    if ((st = stage_in(E, E.s64[0], fin, E.n))) return st;
    LineJob<double> jx = ljob<double>(E.s64[0], E.s64[1], OP_FWD);
    LineJob<double> jy = ljob<double>(E.s64[1], E.s64[1], OP_FWD);
    if ((st = launch_lines<double>(&E, 0, &jx, 1)) || (st = launch_lines<double>(&E, 1, &jy, 1))) return st;
    return stage_out(E, fout, E.s64[1], E.n);
}

extern "C" int vec_inversefft(vec_ctx *c, const double *fin, double *fout)
{
    if (!c || !fin || !fout) return VEC_ERR_ARG;
    Engine &E = c->E;
    int st;
    if ((st = stage_in(E, E.s64[0], fin, E.n))) return st;
    LineJob<double> jx = ljob<double>(E.s64[0], E.s64[1], OP_INV);
    LineJob<double> jy = ljob<double>(E.s64[1], E.s64[1], OP_INV);
    if ((st = launch_lines<double>(&E, 0, &jx, 1)) || (st = launch_lines<double>(&E, 1, &jy, 1))) return st;
    return stage_out(E, fout, E.s64[1], E.n);
}

static int zop(vec_ctx *c, const double *fin, double *fout, int flag, int kind, int oned)
{
    if (!c || !fin || !fout) return VEC_ERR_ARG;
    Engine &E = c->E;
    const size_t cnt = oned ? (size_t)E.nz : E.n;
    int np = oned ? 1 : (int)E.np;
    int st;
    if ((st = stage_in(E, E.s64[0], fin, cnt))) return st;
    if (kind == 0) st = op_d1z(&E, E.s64[0], E.s64[1], flag, np, E.nz);
    else if (kind == 1) st = op_d1upz(&E, E.s64[0], E.s64[1], flag);
    else st = op_d2z(&E, E.s64[0], E.s64[1], flag, np, E.nz);
    if (st) return st;
    return stage_out(E, fout, E.s64[1], cnt);
}

extern "C" int vec_d1bydz(vec_ctx *c, const double *fin, double *fout, int dflag) { return zop(c, fin, fout, dflag, 0, 0); }
extern "C" int vec_d1upbydz(vec_ctx *c, const double *fin, double *fout, int dflag) { return zop(c, fin, fout, dflag, 1, 0); }
extern "C" int vec_d2bydz(vec_ctx *c, const double *fin, double *fout, int dflag) { return zop(c, fin, fout, dflag, 2, 0); }
extern "C" int vec_d1bydz1d(vec_ctx *c, const double *fin, double *fout, int dflag) { return zop(c, fin, fout, dflag, 0, 1); }
extern "C" int vec_d2bydz1d(vec_ctx *c, const double *fin, double *fout, int dflag) { return zop(c, fin, fout, dflag, 2, 1); }

// ---- physics entry points -----------------------------------------------------------
static int finish(vec_ctx *c, int st)
{
    if (st) return st;
    return vec_sync(c);
}

static int mag_on(const Engine &E) { return E.p.f != 0.0 || E.p.kinematic; }

extern "C" int vec_hydro_deriv(vec_ctx *c)
{
    if (!c) return VEC_ERR_ARG;
    return finish(c, c->E.split ? split_hydro(&c->E) : phys_hydro64(&c->E));
}
extern "C" int vec_mag_deriv(vec_ctx *c)
{
    if (!c) return VEC_ERR_ARG;
    return finish(c, c->E.split ? split_mag(&c->E) : phys_mag64(&c->E));
}
extern "C" int vec_bandj(vec_ctx *c)
{
    if (!c) return VEC_ERR_ARG;
    return finish(c, c->E.split ? split_bandj(&c->E) : phys_bandj64(&c->E));
}
extern "C" int vec_magdealias(vec_ctx *c)
{
    if (!c) return VEC_ERR_ARG;
    int st = phys_magdealias(&c->E);
    if (!st && c->E.split) st = split_refresh(&c->E);
    return finish(c, st);
}
// (in the split form the boundary kernels also refresh the FP32 mirrors of
// the planes they change)
static int boundary_step(Engine &E) { return phys_boundary(&E); }
static int mag_boundary_step(Engine &E) { return phys_mag_boundary(&E); }
extern "C" int vec_boundary(vec_ctx *c)
{
    if (!c) return VEC_ERR_ARG;
    return finish(c, boundary_step(c->E));
}
extern "C" int vec_mag_boundary(vec_ctx *c)
{
    if (!c) return VEC_ERR_ARG;
    return finish(c, mag_boundary_step(c->E));
}
extern "C" int vec_ab3_update(vec_ctx *c)
{
    if (!c) return VEC_ERR_ARG;
    return finish(c, c->E.split ? split_ab3(&c->E, 0) : phys_ab3(&c->E, 0));
}
static int diag_step(Engine &E, vec_diag_out *out)
{
    int st;
    if (E.split && (st = split_sync_b64(&E))) return st;
    st = phys_diag(&E, out);
    if (E.split) {
        int s2 = split_refresh_uv(&E);   // GlobalAverages changed u and v
        if (!st) st = s2;
    }
    return st;
}
extern "C" int vec_diag(vec_ctx *c, vec_diag_out *out)
{
    if (!c) return VEC_ERR_ARG;
    int st = diag_step(c->E, out);
    int s2 = vec_sync(c);
    return st ? st : s2;
}

void Engine::drop_graphs()
{
    for (int v = 0; v < 2; v++)
        if (gexec[v]) { cudaGraphExecDestroy(gexec[v]); gexec[v] = nullptr; }
}

// device work of one iteration of src/main.F90:340-747 (printing and
// snapshots excluded); host counters are advanced by the caller
static int enqueue_step(Engine &E, bool diag_now)
{
    int st;
    const int mag = mag_on(E);
    const bool par = mag && E.par_mag && !E.prof_on;
    // split form, mag branch after hydro and no closure correction before
    // the update: the AB3 coefficient step rides on the mean-field CTA of
    // mag_div and the history rotation on the first bandj kernel (two
    // launches fewer per step)
    const bool fold = E.split && mag && !par && !E.corr_on;
    // (with per-kernel profiling on, the branches run one after the other so
    // that no two timed kernels overlap)
    if (par) {
        // mag_deriv on stream2 beside hydro_deriv on stream (disjoint outputs
        // and work arrays; both only read the state)
        CUDA_TRY(cudaEventRecord(E.ev_fork, E.stream));
        CUDA_TRY(cudaStreamWaitEvent(E.stream2, E.ev_fork, 0));
        cudaStream_t s0 = E.stream;
        E.stream = E.stream2;
        st = E.split ? split_mag(&E) : phys_mag64(&E);
        E.stream = s0;
        if (st) return st;
        CUDA_TRY(cudaEventRecord(E.ev_join, E.stream2));
        if ((st = E.split ? split_hydro(&E) : phys_hydro64(&E))) return st;
        CUDA_TRY(cudaStreamWaitEvent(E.stream, E.ev_join, 0));
    } else {
        // (split form, magnetic branch after the hydro one: the transforms
        // of E = u x B ride in the hydro derivatives' line launches)
        const bool share = E.split && mag;
        if ((st = E.split ? split_hydro(&E, share) : phys_hydro64(&E))) return st;
        if (mag) st = E.split ? split_mag(&E, fold, share) : phys_mag64(&E);
        else st = phys_zero_mag_rhs(&E);
        if (st) return st;
    }
    if (E.corr_on && (st = closure_apply_corr(&E))) return st;
    const int mdeal = E.p.dalias && mag;
    if ((st = E.split ? split_ab3(&E, mdeal, fold) : phys_ab3(&E, mdeal))) return st;
    const bool dealias_now = E.p.dalias && (E.nit % 10 == 0);
    if (dealias_now && (st = E.split ? split_dealias(&E) : phys_dealias_state(&E))) return st;
    if (mag && (st = E.split ? split_bandj(&E, fold) : phys_bandj64(&E))) return st;
    if (mag) {
        if ((st = phys_boundaries(&E))) return st;   // boundary and mag_boundary (disjoint fields)
    } else if ((st = boundary_step(E))) {
        return st;
    }
    if (diag_now && (st = diag_step(E, nullptr))) return st;
    if (E.nit % 10 == 0 && (st = E.split ? split_calcdt(&E) : phys_calcdt(&E))) return st;
    return VEC_OK;
}

// Whether a and b can step as members of one batch (one launch per kernel):
// split form, the same grid, box, tile choices and kernel forms, the
// four-point and z-pencil kernels, no closure correction, and the magnetic
// branch (if any) after the hydro one.
bool engine_batchable(const Engine &a, const Engine &b)
{
    auto ok = [](const Engine &e) {
        return e.split && !e.corr_on && !e.prof_on && !(mag_on(e) && e.par_mag) && e.nx % 4 == 0 && e.vec4 &&
               e.zpencil && e.np % 512 == 0 && e.nz >= 6;
    };
    return ok(a) && ok(b) && a.nx == b.nx && a.ny == b.ny && a.nz == b.nz && a.p.xmax == b.p.xmax &&
           a.p.ymax == b.p.ymax && a.kc_pass2 == b.kc_pass2 && a.ct_s == b.ct_s && a.pdl == b.pdl &&
           a.int_cvt == b.int_cvt && a.generic_lines == b.generic_lines && a.ct_warp == b.ct_warp &&
           a.zpencil4 == b.zpencil4 &&
           a.p.dalias == b.p.dalias && a.nit == b.nit;
}

// The device work of one time step (no diagnostics) of a batch of members
// that engine_batchable pairs, each kernel one launch over all of them; the
// same stages in the same order as enqueue_step, per member: members with a
// magnetic branch take the folded path (coefficients in mag_div, history
// rotation in bandj), the others zero their magnetic RHS.  Host counters are
// advanced by the caller.
static int enqueue_step_batch_body(Engine *const *Es, int nE);

int engine_enqueue_step_batch(Engine *const *Es, int nE)
{
    if (nE < 1 || nE > BATCH_MAX) return VEC_ERR_ARG;
    // A batched kernel launches on the stream of the first member of the
    // list it is given, and the magnetic and non-magnetic sub-batches below
    // start with other members than the batch.  All of them must land on
    // the first member's stream: under stream capture a launch on any other
    // stream would run once, at capture time, and be missing from the graph.
    cudaStream_t own[BATCH_MAX];
    for (int i = 0; i < nE; i++) {
        own[i] = Es[i]->stream;
        Es[i]->stream = Es[0]->stream;
    }
    const int st = enqueue_step_batch_body(Es, nE);
    for (int i = 0; i < nE; i++) Es[i]->stream = own[i];
    return st;
}

static int enqueue_step_batch_body(Engine *const *Es, int nE)
{
    Engine *mag[BATCH_MAX], *off[BATCH_MAX];
    bool wm[BATCH_MAX], folded[BATCH_MAX];
    int mdeal[BATCH_MAX];
    int nm = 0, no = 0, st;
    for (int i = 0; i < nE; i++) {
        const bool m = mag_on(*Es[i]) != 0;
        wm[i] = m;
        folded[i] = m;
        mdeal[i] = Es[i]->p.dalias && m;
        if (m) mag[nm++] = Es[i];
        else off[no++] = Es[i];
    }
    if ((st = split_hydro_m(Es, nE, wm))) return st;
    if (nm && (st = split_mag_m(mag, nm, true, true))) return st;
    if (no && (st = phys_zero_mag_rhs_m(off, no))) return st;
    if ((st = split_ab3_m(Es, nE, mdeal, folded))) return st;
    const int nit = Es[0]->nit;
    if (Es[0]->p.dalias && nit % 10 == 0 && (st = split_dealias_m(Es, nE))) return st;
    if (nm && (st = split_bandj_m(mag, nm, true))) return st;
    if (nm && (st = phys_boundaries_m(mag, nm))) return st;
    if (no && (st = phys_boundary_m(off, no))) return st;
    if (nit % 10 == 0 && (st = split_calcdt_m(Es, nE))) return st;
    return VEC_OK;
}

static bool diag_due(const Engine &E, int nit)
{
    return E.p.diag_cadence && E.p.ndu06 > 0 && (nit % E.p.ndu06 == 0);
}

// Captures the device work of the next step into graph variant v (or
// replays it).  Returns VEC_OK with *done = 0 when the step must run
// eagerly (diagnostics, profiling, graphs disabled).
static int graph_step(Engine &E, int *done)
{
    *done = 0;
    const int nit = E.nit + 1;
    if (!E.use_graphs || E.prof_on || diag_due(E, nit)) return VEC_OK;
    const int v = (nit % 10 == 0) ? 1 : 0;
    if (!E.gexec[v]) {
        E.nit = nit;
        E.iter += 1;
        cudaGraph_t g = nullptr;
        const long long l0 = E.launches;
        CUDA_TRY(cudaStreamBeginCapture(E.stream, cudaStreamCaptureModeThreadLocal));
        int st = enqueue_step(E, false);
        cudaError_t ce = cudaStreamEndCapture(E.stream, &g);
        if (st) { if (g) cudaGraphDestroy(g); return st; }
        if (ce != cudaSuccess) { vec_set_error("step capture failed: %s", cudaGetErrorString(ce)); return VEC_ERR_CUDA; }
        ce = cudaGraphInstantiate(&E.gexec[v], g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) { vec_set_error("graph instantiate failed: %s", cudaGetErrorString(ce)); return VEC_ERR_CUDA; }
        E.g_b32_after[v] = E.b32_auth;
        E.g_launches[v] = E.launches - l0;
    } else {
        E.nit = nit;
        E.iter += 1;
        E.b32_auth = E.g_b32_after[v];
        E.launches += E.g_launches[v];
    }
    CUDA_TRY(cudaGraphLaunch(E.gexec[v], E.stream));
    *done = 1;
    return VEC_OK;
}

static int one_step(Engine &E)
{
    int done = 0;
    int st = graph_step(E, &done);
    if (st || done) return st;
    E.nit += 1;
    E.iter += 1;
    return enqueue_step(E, diag_due(E, E.nit));
}

// The non-finite check that rides on calcdt: one 4-byte read-back and a
// stream synchronisation, after the steps of a call that ran calcdt.
static int check_nonfinite(Engine &E)
{
    CUDA_TRY(cudaMemcpyAsync(&E.hs->nonfinite, &E.ds->nonfinite, sizeof(int), cudaMemcpyDeviceToHost, E.stream));
    CUDA_TRY(cudaStreamSynchronize(E.stream));
    if (E.hs->nonfinite) {
        vec_set_error("non-finite value in the state (calcdt of the time loop)");
        return VEC_ERR_NAN;
    }
    return VEC_OK;
}

extern "C" int vec_step(vec_ctx *c, int nsteps)
{
    if (!c || nsteps < 0) return VEC_ERR_ARG;
    bool cdt = false;
    for (int s = 0; s < nsteps; s++) {
        cdt = cdt || (c->E.nit + 1) % 10 == 0;
        int st = one_step(c->E);
        if (st) { c->E.prof_flush(); return st; }
    }
    if (c->E.prof_on) {
        int st = c->E.prof_flush();
        if (st) return st;
    }
    return cdt ? check_nonfinite(c->E) : VEC_OK;
}

extern "C" int vec_last_diag(vec_ctx *c, vec_diag_out *out)
{
    if (!c || !out) return VEC_ERR_ARG;
    *out = c->E.last_diag;
    return c->E.have_diag ? VEC_OK : VEC_ERR_ARG;
}

// ---- instrumentation ------------------------------------------------------------------
extern "C" int vec_profile(vec_ctx *c, int on)
{
    if (!c) return VEC_ERR_ARG;
    c->E.prof_flush();
    c->E.prof_on = on != 0;
    return VEC_OK;
}
extern "C" int vec_profile_count(vec_ctx *c)
{
    if (!c) return 0;
    c->E.prof_flush();
    return (int)c->E.prof.size();
}
extern "C" int vec_profile_get(vec_ctx *c, int i, char *name, int *launches, double *ms, double *bytes)
{
    if (!c || i < 0 || i >= (int)c->E.prof.size()) return VEC_ERR_ARG;
    c->E.prof_flush();
    const ProfRec &r = c->E.prof[i];
    if (name) { strncpy(name, r.name.c_str(), 63); name[63] = 0; }
    if (launches) *launches = r.launches;
    if (ms) *ms = r.ms;
    if (bytes) *bytes = r.bytes;
    return VEC_OK;
}
extern "C" int vec_profile_reset(vec_ctx *c)
{
    if (!c) return VEC_ERR_ARG;
    c->E.prof_flush();
    c->E.prof.clear();
    return VEC_OK;
}
extern "C" long long vec_launch_count(vec_ctx *c) { return c ? c->E.launches : 0; }

// ---- snapshots ------------------------------------------------------------------
static const int SNAP_FIELDS[8] = { VEC_F_R, VEC_F_T, VEC_F_U, VEC_F_V, VEC_F_W, VEC_F_BX, VEC_F_BY, VEC_F_BZ };

extern "C" int vec_write_snapshot(vec_ctx *c, const char *path, int iprec, const char *history)
{
    if (!c || !path) return VEC_ERR_ARG;
    Engine &E = c->E;
    vec_scalars sc;
    int st = vec_get_scalars(c, &sc);
    if (st) return st;
    vec_snapshot s;
    memset(&s, 0, sizeof(s));
    s.nx = E.nx; s.ny = E.ny; s.nz = E.nz;
    s.iteration = sc.iter; s.time = sc.ttime; s.timestep = sc.dt1; s.version = 3;
    if (history) strncpy(s.history, history, 79);
    s.gamma = E.p.gamma; s.sigma = E.p.sigma; s.theta = E.p.theta; s.ck = E.p.ck; s.cm = E.p.cm;
    s.f = E.p.f; s.tayl = E.p.tayl; s.psi = E.p.psi; s.zeta = E.p.zeta; s.xmax = E.p.xmax; s.ymax = E.p.ymax;
    std::vector<double> buf(8 * E.n);
    for (int i = 0; i < 8; i++) {
        s.fields[i] = buf.data() + (size_t)i * E.n;
        if ((st = vec_get_field(c, SNAP_FIELDS[i], s.fields[i]))) return st;
    }
    return vec_nc_write(path, &s, iprec);
}

extern "C" int vec_read_restart(vec_ctx *c, const char *path)
{
    if (!c || !path) return VEC_ERR_ARG;
    Engine &E = c->E;
    vec_snapshot s;
    memset(&s, 0, sizeof(s));
    s.nx = E.nx; s.ny = E.ny; s.nz = E.nz;
    std::vector<double> buf(8 * E.n);
    for (int i = 0; i < 8; i++) s.fields[i] = buf.data() + (size_t)i * E.n;
    int st = vec_nc_read(path, &s);
    if (st) return st;
    for (int i = 0; i < 8; i++)
        if ((st = vec_set_field(c, SNAP_FIELDS[i], s.fields[i]))) return st;
    vec_scalars sc;
    if ((st = vec_get_scalars(c, &sc))) return st;
    sc.iter = s.iteration;
    sc.ttime = s.time;
    sc.dt1 = s.timestep;
    sc.nit = 0;
    sc.first = 1;   // src/main.F90:110: the histories are not restored
    sc.second = 0;
    return vec_set_scalars(c, &sc);
}

extern "C" int vec_use_graphs(vec_ctx *c, int on)
{
    if (!c) return VEC_ERR_ARG;
    c->E.use_graphs = on != 0;
    if (!on) c->E.drop_graphs();
    return VEC_OK;
}

int engine_enqueue_step(Engine &E, bool diag_now) { return enqueue_step(E, diag_now); }
int engine_one_step(Engine &E) { return one_step(E); }
bool engine_diag_due(const Engine &E, int nit) { return diag_due(E, nit); }
Engine &engine_of(vec_ctx *c) { return c->E; }
