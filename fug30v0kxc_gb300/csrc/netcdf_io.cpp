// netcdf_io.cpp -- NetCDF classic (CDF-1) snapshots in the layout of the
// reference's T16_NNN.nc / restart.nc files (src/netcdf.F90:39-1287).
//
// libnetcdf is not available, so this is a small codec written from the
// published classic-format specification: big-endian header of dimensions,
// global attributes and variables, followed by the variables' data at their
// 'begin' offsets, each padded to 4 bytes.  The layout written is the one
// CreateNetCDF defines (src/netcdf.F90:77-199): global attributes version,
// history (79 characters), gamma, sigma, theta, ck, cm, f, tayl, psi, zeta,
// xmax, ymax; dimensions nx, ny, nz, one; variables time (units "UNKNOWN"),
// iteration, timestep and R, T, U, V, W, Bx, By, Bz with Fortran shape
// (nx,ny,nz), i.e. netCDF shape (nz,ny,nx), as float (iprec 4) or double
// (iprec 8).
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/vec.h"

void vec_set_error(const char *fmt, ...);

namespace {

enum { NC_BYTE = 1, NC_CHAR = 2, NC_SHORT = 3, NC_INT = 4, NC_FLOAT = 5, NC_DOUBLE = 6 };
enum { TAG_DIM = 0x0A, TAG_VAR = 0x0B, TAG_ATT = 0x0C };
const char *FIELD_NAMES[8] = { "R", "T", "U", "V", "W", "Bx", "By", "Bz" };
const char *ATT_NAMES[11] = { "gamma", "sigma", "theta", "ck", "cm", "f", "tayl", "psi", "zeta", "xmax", "ymax" };

int type_size(int t)
{
    switch (t) {
    case NC_BYTE: case NC_CHAR: return 1;
    case NC_SHORT: return 2;
    case NC_INT: case NC_FLOAT: return 4;
    case NC_DOUBLE: return 8;
    }
    return 0;
}

size_t pad4(size_t n) { return (n + 3) & ~(size_t)3; }

// ---- writer ------------------------------------------------------------------
struct Buf {
    std::vector<unsigned char> b;
    void u32(uint32_t v) { for (int s = 24; s >= 0; s -= 8) b.push_back((unsigned char)(v >> s)); }
    void u64(uint64_t v) { for (int s = 56; s >= 0; s -= 8) b.push_back((unsigned char)(v >> s)); }
    void f64(double d) { uint64_t u; memcpy(&u, &d, 8); u64(u); }
    void f32(float f) { uint32_t u; memcpy(&u, &f, 4); u32(u); }
    void name(const char *s) {
        size_t n = strlen(s);
        u32((uint32_t)n);
        for (size_t i = 0; i < n; i++) b.push_back((unsigned char)s[i]);
        while (b.size() % 4) b.push_back(0);
    }
    void att_f64(const char *n, double v) { name(n); u32(NC_DOUBLE); u32(1); f64(v); }
    void att_i32(const char *n, int32_t v) { name(n); u32(NC_INT); u32(1); u32((uint32_t)v); }
    void att_text(const char *n, const char *txt, size_t len) {
        name(n); u32(NC_CHAR); u32((uint32_t)len);
        for (size_t i = 0; i < len; i++) b.push_back((unsigned char)txt[i]);
        while (b.size() % 4) b.push_back(0);
    }
};

struct VarDef {
    std::string name;
    std::vector<int> dims;
    int type;
    size_t vsize;   // padded bytes
    bool units;
};

// ---- reader --------------------------------------------------------------------
struct Rd {
    const unsigned char *p, *end;
    bool ok = true;
    uint32_t u32() {
        if (end - p < 4) { ok = false; return 0; }
        uint32_t v = ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
        p += 4;
        return v;
    }
    uint64_t u64() { uint64_t hi = u32(); return (hi << 32) | u32(); }
    std::string name() {
        uint32_t n = u32();
        if (!ok || (size_t)(end - p) < pad4(n)) { ok = false; return ""; }
        std::string s((const char *)p, n);
        p += pad4(n);
        return s;
    }
};

double rd_f64(const unsigned char *q) { uint64_t u = 0; for (int i = 0; i < 8; i++) u = (u << 8) | q[i]; double d; memcpy(&d, &u, 8); return d; }
float rd_f32(const unsigned char *q) { uint32_t u = 0; for (int i = 0; i < 4; i++) u = (u << 8) | q[i]; float f; memcpy(&f, &u, 4); return f; }
int32_t rd_i32(const unsigned char *q) { uint32_t u = 0; for (int i = 0; i < 4; i++) u = (u << 8) | q[i]; return (int32_t)u; }

struct Att { std::string name; int type; uint32_t n; const unsigned char *data; };
struct Var { std::string name; std::vector<uint32_t> dims; std::vector<Att> atts; int type; uint64_t vsize, begin; };
struct Header {
    int version = 0;
    std::vector<std::pair<std::string, uint32_t>> dims;
    std::vector<Att> gatts;
    std::vector<Var> vars;
};

bool parse_atts(Rd &r, std::vector<Att> &out)
{
    uint32_t tag = r.u32(), n = r.u32();
    if (tag == 0 && n == 0) return r.ok;
    if (tag != TAG_ATT) return false;
    for (uint32_t i = 0; i < n && r.ok; i++) {
        Att a;
        a.name = r.name();
        a.type = (int)r.u32();
        a.n = r.u32();
        size_t bytes = pad4((size_t)a.n * type_size(a.type));
        if (!type_size(a.type) || (size_t)(r.end - r.p) < bytes) return false;
        a.data = r.p;
        r.p += bytes;
        out.push_back(a);
    }
    return r.ok;
}

bool parse_header(const std::vector<unsigned char> &f, Header &h)
{
    if (f.size() < 8 || f[0] != 'C' || f[1] != 'D' || f[2] != 'F' || (f[3] != 1 && f[3] != 2)) return false;
    h.version = f[3];
    Rd r{ f.data() + 4, f.data() + f.size() };
    r.u32();   // numrecs
    uint32_t tag = r.u32(), n = r.u32();
    if (!(tag == 0 && n == 0)) {
        if (tag != TAG_DIM) return false;
        for (uint32_t i = 0; i < n && r.ok; i++) {
            std::string nm = r.name();
            h.dims.push_back({ nm, r.u32() });
        }
    }
    if (!parse_atts(r, h.gatts)) return false;
    tag = r.u32();
    n = r.u32();
    if (!(tag == 0 && n == 0)) {
        if (tag != TAG_VAR) return false;
        for (uint32_t i = 0; i < n && r.ok; i++) {
            Var v;
            v.name = r.name();
            uint32_t nd = r.u32();
            for (uint32_t d = 0; d < nd; d++) v.dims.push_back(r.u32());
            if (!parse_atts(r, v.atts)) return false;
            v.type = (int)r.u32();
            v.vsize = r.u32();
            v.begin = h.version == 1 ? r.u32() : r.u64();
            h.vars.push_back(v);
        }
    }
    return r.ok;
}

bool read_file(const char *path, std::vector<unsigned char> &out)
{
    FILE *fp = fopen(path, "rb");
    if (!fp) return false;
    fseek(fp, 0, SEEK_END);
    long sz = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    out.resize(sz > 0 ? (size_t)sz : 0);
    bool ok = sz > 0 && fread(out.data(), 1, out.size(), fp) == out.size();
    fclose(fp);
    return ok;
}

const Att *find_att(const std::vector<Att> &v, const char *n)
{
    for (auto &a : v) if (a.name == n) return &a;
    return nullptr;
}

double att_num(const Att *a)
{
    if (!a || a->n < 1) return 0.0;
    switch (a->type) {
    case NC_DOUBLE: return rd_f64(a->data);
    case NC_FLOAT: return rd_f32(a->data);
    case NC_INT: return rd_i32(a->data);
    case NC_SHORT: return (int16_t)((a->data[0] << 8) | a->data[1]);
    case NC_BYTE: return (int8_t)a->data[0];
    }
    return 0.0;
}

}  // namespace

// fmt 1: classic (CDF-1, 32-bit offsets, src/netcdf.F90:74); fmt 2: 64-bit
// offsets (CDF-2, NF_64BIT_OFFSET, interpolate/netcdf.F90:73)
static int nc_write(const char *path, const vec_snapshot *s, int iprec, int fmt)
{
    if (!path || !s || (iprec != 4 && iprec != 8) || (fmt != 1 && fmt != 2)) return VEC_ERR_ARG;
    for (int i = 0; i < 8; i++) if (!s->fields[i]) return VEC_ERR_ARG;
    const size_t n = (size_t)s->nx * s->ny * s->nz;
    Buf h;
    h.b.push_back('C'); h.b.push_back('D'); h.b.push_back('F'); h.b.push_back((unsigned char)fmt);
    h.u32(0);   // numrecs: no record variables
    h.u32(TAG_DIM); h.u32(4);
    h.name("nx"); h.u32((uint32_t)s->nx);
    h.name("ny"); h.u32((uint32_t)s->ny);
    h.name("nz"); h.u32((uint32_t)s->nz);
    h.name("one"); h.u32(1);
    // global attributes in the order of src/netcdf.F90:77-128
    h.u32(TAG_ATT); h.u32(13);
    h.att_i32("version", s->version);
    char his[80];
    memset(his, ' ', 79);
    size_t hl = strnlen(s->history, 79);
    memcpy(his, s->history, hl);
    h.att_text("history", his, 79);
    const double av[11] = { s->gamma, s->sigma, s->theta, s->ck, s->cm, s->f, s->tayl, s->psi, s->zeta, s->xmax, s->ymax };
    for (int i = 0; i < 11; i++) h.att_f64(ATT_NAMES[i], av[i]);
    // variables
    std::vector<VarDef> vars;
    vars.push_back({ "time", { 3 }, NC_DOUBLE, 8, true });
    vars.push_back({ "iteration", { 3 }, NC_INT, 4, false });
    vars.push_back({ "timestep", { 3 }, NC_DOUBLE, 8, false });
    const int ft = iprec == 8 ? NC_DOUBLE : NC_FLOAT;
    for (int i = 0; i < 8; i++) vars.push_back({ FIELD_NAMES[i], { 2, 1, 0 }, ft, pad4(n * (size_t)iprec), false });
    // header size: everything above plus the variable list
    size_t vl = 8;
    for (auto &v : vars) {
        vl += 4 + pad4(v.name.size()) + 4 + 4 * v.dims.size();
        vl += v.units ? 8 + (4 + pad4(5)) + 8 + pad4(7) : 8;
        vl += 4 + 4 + (fmt == 1 ? 4 : 8);
    }
    size_t off = h.b.size() + vl;
    if (fmt == 1 && off + 8 * n * iprec + 64 > 0x7fffffffull) {
        vec_set_error("snapshot larger than the 2 GiB limit of the classic format");
        return VEC_ERR_SIZE;
    }
    h.u32(TAG_VAR); h.u32((uint32_t)vars.size());
    for (auto &v : vars) {
        h.name(v.name.c_str());
        h.u32((uint32_t)v.dims.size());
        for (int d : v.dims) h.u32((uint32_t)d);
        if (v.units) { h.u32(TAG_ATT); h.u32(1); h.att_text("units", "UNKNOWN", 7); }
        else { h.u32(0); h.u32(0); }
        h.u32((uint32_t)v.type);
        h.u32((uint32_t)v.vsize);
        if (fmt == 1) h.u32((uint32_t)off);
        else { h.u32((uint32_t)((uint64_t)off >> 32)); h.u32((uint32_t)off); }
        off += v.vsize;
    }
    // data
    Buf d;
    d.b.reserve(off - h.b.size());
    d.f64(s->time);
    d.u32((uint32_t)s->iteration);
    d.f64(s->timestep);
    for (int i = 0; i < 8; i++) {
        const double *src = s->fields[i];
        if (iprec == 8) for (size_t q = 0; q < n; q++) d.f64(src[q]);
        else for (size_t q = 0; q < n; q++) d.f32((float)src[q]);
        while (d.b.size() % 4) d.b.push_back(0);
    }
    FILE *fp = fopen(path, "wb");
    if (!fp) { vec_set_error("cannot create %s", path); return VEC_ERR_INPUT; }
    bool ok = fwrite(h.b.data(), 1, h.b.size(), fp) == h.b.size() && fwrite(d.b.data(), 1, d.b.size(), fp) == d.b.size();
    ok = (fclose(fp) == 0) && ok;
    if (!ok) { vec_set_error("write to %s failed", path); return VEC_ERR_INPUT; }
    return VEC_OK;
}

extern "C" int vec_nc_write(const char *path, const vec_snapshot *s, int iprec) { return nc_write(path, s, iprec, 1); }

extern "C" int vec_nc_write_fmt(const char *path, const vec_snapshot *s, int iprec, int fmt)
{
    return nc_write(path, s, iprec, fmt);
}

extern "C" int vec_nc_read(const char *path, vec_snapshot *s)
{
    if (!path || !s) return VEC_ERR_ARG;
    std::vector<unsigned char> f;
    if (!read_file(path, f)) { vec_set_error("cannot read %s", path); return VEC_ERR_INPUT; }
    Header h;
    if (!parse_header(f, h)) { vec_set_error("%s is not a classic NetCDF file", path); return VEC_ERR_INPUT; }
    int nx = -1, ny = -1, nz = -1;
    for (auto &d : h.dims) {
        if (d.first == "nx") nx = (int)d.second;
        else if (d.first == "ny") ny = (int)d.second;
        else if (d.first == "nz") nz = (int)d.second;
    }
    if (nx <= 0 || ny <= 0 || nz <= 0) { vec_set_error("%s lacks nx/ny/nz", path); return VEC_ERR_INPUT; }
    // src/netcdf.F90:591-713 (OpenNetCDF): parameters from the attributes
    double *av[11] = { &s->gamma, &s->sigma, &s->theta, &s->ck, &s->cm, &s->f, &s->tayl, &s->psi, &s->zeta,
                       &s->xmax, &s->ymax };
    for (int i = 0; i < 11; i++) *av[i] = att_num(find_att(h.gatts, ATT_NAMES[i]));
    s->version = (int32_t)att_num(find_att(h.gatts, "version"));
    memset(s->history, 0, sizeof(s->history));
    if (const Att *a = find_att(h.gatts, "history"))
        if (a->type == NC_CHAR) memcpy(s->history, a->data, a->n < 79 ? a->n : 79);
    const bool sized = s->nx == nx && s->ny == ny && s->nz == nz;
    s->nx = nx; s->ny = ny; s->nz = nz;
    const size_t n = (size_t)nx * ny * nz;
    for (auto &v : h.vars) {
        const unsigned char *q = f.data() + v.begin;
        const size_t ts = type_size(v.type);
        size_t cnt = 1;
        for (auto d : v.dims) cnt *= h.dims[d].second;
        if (v.begin + cnt * ts > f.size()) { vec_set_error("%s: truncated variable %s", path, v.name.c_str()); return VEC_ERR_INPUT; }
        if (v.name == "time") s->time = v.type == NC_DOUBLE ? rd_f64(q) : rd_f32(q);
        else if (v.name == "timestep") s->timestep = v.type == NC_DOUBLE ? rd_f64(q) : rd_f32(q);
        else if (v.name == "iteration") s->iteration = rd_i32(q);
        else {
            for (int i = 0; i < 8; i++) {
                if (v.name != FIELD_NAMES[i] || !s->fields[i]) continue;
                if (!sized || cnt != n) { vec_set_error("%s: caller buffers do not match the file's grid", path); return VEC_ERR_SIZE; }
                double *dst = s->fields[i];
                if (v.type == NC_DOUBLE) for (size_t k = 0; k < n; k++) dst[k] = rd_f64(q + 8 * k);
                else if (v.type == NC_FLOAT) for (size_t k = 0; k < n; k++) dst[k] = rd_f32(q + 4 * k);
                else { vec_set_error("%s: unsupported type of %s", path, v.name.c_str()); return VEC_ERR_INPUT; }
            }
        }
    }
    return VEC_OK;
}
