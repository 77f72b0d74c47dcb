"""Host-side logic of the library, run without a GPU: exported symbols, the
Fortran / C / Python bindings against each other, the INPUT parser
(src/initial.F90:94-201) and the NetCDF snapshot codec (src/netcdf.F90
layout) against scipy's independent NetCDF reader."""
import os
import re

import numpy as np
import pytest

from fug30v0kxc_gb300 import lib
from fug30v0kxc_gb300.params import ck_from_rayleigh
from fug30v0kxc_gb300.solver import SNAP_ATTRS, SNAP_FIELDS, nc_read, nc_write, read_input

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# the reference's VarElecCond directory, when it is mounted (tests that read
# its files directly skip without it; its INPUT files are also committed as
# a fixture by tests/golden/make_fixtures.py)
REF_DIR = os.environ.get("VEC_REFERENCE_DIR", "")
REF_BIN = os.path.join(REF_DIR, "bin") if REF_DIR else ""


def test_library_exports_every_header_symbol():
    L = lib.load()
    hdr = open(os.path.join(ROOT, "include", "vec.h")).read()
    names = set(re.findall(r"^\s*(?:int|void|const char|long long)\s*\*?\s*(vec_\w+)\s*\(", hdr, re.M))
    assert len(names) > 40
    for n in sorted(names):
        assert hasattr(L, n), n
        assert n in lib.SIGNATURES, f"{n} has no ctypes signature"
    # every ctypes signature takes as many arguments as its C prototype
    hdr_nc = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    for n, (_, args) in lib.SIGNATURES.items():
        proto = re.search(r"\b%s\s*\(([^)]*)\)\s*;" % n, hdr_nc, re.S)
        assert proto, f"{n} is not declared in vec.h"
        ca = [a for a in proto.group(1).split(",") if a.strip() and a.strip() != "void"]
        assert len(ca) == len(args), (n, len(args), len(ca))


INPUT_TEXT = """data file for parallel magnetoconvection program

{flag}\t     INPUT FLAG (1 for CK/F, 2 for Ra/Q)

VALUE        VARIABLE
1.4      GAMMA
1.00          SIGMA
9.0         THETA
{ck}      CK (if FLAG=1) or Ra (if FLAG=2)
1.0          CM
{f}          F (if FLAG=1) or Q (if FLAG=2)
0.0      TAYL (mid layer)
1.570796327         PSI
0.2          ZETA
4.0          XMAX
4.0          YMAX
0.3          SF
0            NFRAME
1000       TOTAL
100          NDU06
1000        NDU16
10            NDURESTART
64\t     NX
64\t     NY
65\t     NZ
"""


def test_input_ra_q_conversion(tmp_path):
    path = tmp_path / "INPUT"
    path.write_text(INPUT_TEXT.format(flag=2, ck="100000", f="100.0"))
    p = read_input(str(path))
    ck = ck_from_rayleigh(1e5, 9.0, 1.0, 1.0, 1.4)
    assert abs(p.ck - ck) < 1e-15 * ck
    assert abs(p.f - 100.0 * 0.2 * ck * ck) < 1e-15
    assert (p.nx, p.ny, p.nz, p.ntotal, p.ndu06) == (64, 64, 65, 1000, 100)
    assert p.rayl == 1e5 and p.chand == 100.0


def test_input_ck_f_and_errors(tmp_path):
    path = tmp_path / "INPUT"
    path.write_text(INPUT_TEXT.format(flag=1, ck="0.05d0", f="2.0"))
    p = read_input(str(path))
    assert p.ck == 0.05 and p.f == 2.0
    assert abs(p.chand - 2.0 / (0.2 * 0.05 * 0.05)) < 1e-9
    path.write_text(INPUT_TEXT.format(flag=3, ck="1", f="1"))
    with pytest.raises(RuntimeError):
        read_input(str(path))
    with pytest.raises(RuntimeError):
        read_input(str(tmp_path / "missing"))


def test_reference_input_files(tmp_path):
    """The reference's own parameter files (bin/INPUT, bin/originalINPUT,
    bin/test1/INPUT, kept as a fixture) through the INPUT reader."""
    import json
    with open(os.path.join(ROOT, "tests", "golden", "reference_inputs.json")) as f:
        texts = json.load(f)
    assert sorted(texts) == ["INPUT", "originalINPUT", "test1/INPUT"]
    for sub, text in texts.items():
        path = tmp_path / sub.replace("/", "_")
        path.write_text(text)
        p = read_input(str(path))
        assert p.nx > 0 and p.ny > 0 and p.nz > 0 and p.ck > 0, sub
    # bin/INPUT: flag 2 (Ra / Q), converted as src/initial.F90:186-199 does
    p = read_input(str(tmp_path / "INPUT"))
    assert p.rayl > 0 and abs(p.f - p.chand * p.zeta * p.sigma * p.ck * p.ck) <= 1e-12 * abs(p.f)


def _snapshot(nx=12, ny=10, nz=7, seed=0):
    rng = np.random.default_rng(seed)
    d = {n: rng.standard_normal((nz, ny, nx)) for n in SNAP_FIELDS}
    d.update(time=13.875, iteration=105000, timestep=1.25e-4, version=3, history="test snapshot")
    d.update({a: float(i) + 0.5 for i, a in enumerate(SNAP_ATTRS)})
    return d


@pytest.mark.parametrize("iprec,fmt", [(4, 1), (8, 1), (8, 2)])
def test_snapshot_roundtrip_and_scipy(tmp_path, iprec, fmt):
    """fmt 1: classic NetCDF (src/netcdf.F90:74); fmt 2: 64-bit offsets
    (the interpolate program's output, interpolate/netcdf.F90:73)."""
    snap = _snapshot()
    path = tmp_path / "T16_001.nc"
    nc_write(path, snap, iprec, fmt)
    assert open(path, "rb").read(4) == b"CDF" + bytes([fmt])
    back = nc_read(path)
    for n in SNAP_FIELDS:
        ref = snap[n].astype(np.float32).astype(np.float64) if iprec == 4 else snap[n]
        assert np.array_equal(back[n], ref), n
    assert back["iteration"] == 105000 and back["time"] == 13.875 and back["timestep"] == 1.25e-4
    # an independent reader sees the reference's layout
    from scipy.io import netcdf_file
    with netcdf_file(str(path), "r", mmap=False) as f:
        assert f.version_byte == fmt
        assert f.dimensions == {"nx": 12, "ny": 10, "nz": 7, "one": 1}
        assert f.variables["R"].shape == (7, 10, 12)
        assert f.variables["R"].typecode() == ("d" if iprec == 8 else "f")
        assert np.array_equal(np.asarray(f.variables["T"][:], dtype=np.float64), back["T"])
        assert f.variables["time"].units == b"UNKNOWN"
        assert int(f.variables["iteration"][0]) == 105000
        assert f.version == 3
        assert len(f.history) == 79
        for i, a in enumerate(SNAP_ATTRS):
            assert getattr(f, a) == float(i) + 0.5


@pytest.mark.skipif(not REF_BIN or not os.path.exists(REF_BIN), reason="set VEC_REFERENCE_DIR to the reference")
def test_reads_reference_restart():
    from scipy.io import netcdf_file
    path = os.path.join(REF_BIN, "restart.nc")
    d = nc_read(path)
    with netcdf_file(path, "r", mmap=False) as f:
        for n in SNAP_FIELDS:
            assert np.array_equal(d[n], np.asarray(f.variables[n][:], dtype=np.float64)), n
        assert d["iteration"] == int(f.variables["iteration"][0])
        assert d["time"] == float(f.variables["time"][0])
        assert d["ck"] == float(f.ck) and d["f"] == float(f.f)


def _c_struct_members(hdr, name):
    """(type, member) pairs of `typedef struct name { ... }` in order."""
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), hdr, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ctype, rest = decl.split(None, 1)
        out += [(ctype, m.strip()) for m in rest.split(",")]
    return out


def _f_type_members(src, name):
    body = re.search(r"type, bind\(C\) :: %s\n(.*?)end type %s" % (name, name), src, re.S).group(1)
    out = []
    for line in body.splitlines():
        m = re.match(r"\s*(real\(c_double\)|integer\(c_int32_t\))\s*::\s*(.*)", line)
        if m:
            ftype = {"real(c_double)": "double", "integer(c_int32_t)": "int32_t"}[m.group(1)]
            out += [(ftype, v.strip()) for v in m.group(2).split(",")]
    return out


def test_fortran_c_and_python_bindings_agree():
    """The drop-in boundary three ways: the Fortran module
    (include/vec_mod.f90), the C header (include/vec.h) and the Python
    ctypes structures must lay out vec_params, vec_scalars and vec_diag_out
    identically, member by member. The field ids must match. Every function
    the Fortran module binds must be declared in the header and exported by
    the library."""
    import ctypes as C
    from fug30v0kxc_gb300 import params as P
    hdr = open(os.path.join(ROOT, "include", "vec.h")).read()
    fsrc = open(os.path.join(ROOT, "include", "vec_mod.f90")).read()
    py = {"vec_params": P.VecParams, "vec_scalars": P.VecScalars, "vec_diag_out": P.VecDiag}
    pytype = {C.c_double: "double", C.c_int32: "int32_t"}
    for name, cls in py.items():
        c = _c_struct_members(hdr, name)
        f = _f_type_members(fsrc, name)
        p = [(pytype[t], n) for n, t in cls._fields_]
        assert c == f, (name, c, f)
        assert c == p, (name, c, p)
    fids = dict((k, int(v)) for k, v in re.findall(r"(VEC_F_[A-Z]+) = (\d+)", fsrc))
    assert fids and all(getattr(P, k[4:]) == v for k, v in fids.items() if hasattr(P, k[4:]))
    assert [fids[f"VEC_F_{n.upper()}"] for n in ("r", "t", "u", "v", "w", "bx", "by", "bz", "jsq", "pol", "tor")] \
        == list(range(11))
    names = re.findall(r"bind\(C, name='(vec_\w+)'\)", fsrc)
    assert len(names) >= 40
    L = lib.load()
    for n in names:
        assert re.search(r"\b%s\s*\(" % n, hdr), n
        assert hasattr(L, n), n
    # argument counts of each bound function against its C prototype
    hdr_nc = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    funcs = re.findall(r"function (vec_\w+)\(([^)]*)\)\s*bind\(C, name='(vec_\w+)'\)", fsrc)
    assert len(funcs) == len(names)
    for _, fargs, cname in funcs:
        fa = [a for a in fargs.replace("&", "").split(",") if a.strip()]
        proto = re.search(r"\b%s\s*\(([^)]*)\)\s*;" % cname, hdr_nc, re.S).group(1)
        ca = [a for a in proto.split(",") if a.strip() and a.strip() != "void"]
        assert len(fa) == len(ca), (cname, len(fa), len(ca))
