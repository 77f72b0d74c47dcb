"""Python mirror of the reference's operator interface, backed by the GPU.

The names follow the reference's module procedures (src/fft.F90,
src/dbydz.F90, src/hydro_deriv.f90, src/magnetic.f90, src/utils.F90,
src/main.F90); arrays are numpy (nz, ny, nx) views of the Fortran
(nx, ny, nz) layout.  Every call goes through the C-ABI of include/vec.h
into the sm_103a kernels; there is no CPU path.
"""
import ctypes as C

import numpy as np

from . import lib as _L
from .params import (FIELD_NAMES, MEAN_NAMES, STATE_FIELDS, STATUS, VecDiag, VecParams,
                     VecScalars, VecSnapshot)


class VecError(RuntimeError):
    def __init__(self, where, status):
        msg = _L.load().vec_last_error().decode(errors="replace")
        super().__init__(f"{where}: status {status} ({STATUS.get(status, '?')}) {msg}")
        self.status = status


def _ptr(a):
    """data pointer of a numpy array, or an int device pointer (torch tensors)."""
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return int(a)


class P3D:
    """One device-resident VarElecCond context (src/arrays.f90 in HBM)."""

    def __init__(self, params: VecParams, handle=None):
        self.L = _L.load()
        self.p = params.copy()
        self.owned = handle is None
        if handle is None:
            h = C.c_void_p()
            st = self.L.vec_create(C.byref(self.p), C.byref(h))
            if st != 0:
                raise VecError("vec_create", st)
            handle = h
        self.h = handle
        self.shape = (self.p.nz, self.p.ny, self.p.nx)

    def close(self):
        if getattr(self, "h", None) and getattr(self, "owned", True):
            self.L.vec_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, st, where):
        if st != 0:
            raise VecError(where, st)

    # -- state ----------------------------------------------------------------
    def get(self, name):
        out = np.empty(self.shape, dtype=np.float64)
        self._chk(self.L.vec_get_field(self.h, FIELD_NAMES[name], out.ctypes.data), name)
        return out

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self.shape)
        self._chk(self.L.vec_set_field(self.h, FIELD_NAMES[name], a.ctypes.data), name)

    def get_mean(self, name):
        out = np.empty(self.p.nz, dtype=np.float64)
        self._chk(self.L.vec_get_mean(self.h, MEAN_NAMES[name], out.ctypes.data), name)
        return out

    def set_mean(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self._chk(self.L.vec_set_mean(self.h, MEAN_NAMES[name], a.ctypes.data), name)

    @property
    def bzbar(self):
        v = C.c_double()
        self.L.vec_get_bzbar(self.h, C.byref(v))
        return v.value

    @bzbar.setter
    def bzbar(self, v):
        self.L.vec_set_bzbar(self.h, float(v))

    def scalars(self):
        s = VecScalars()
        self._chk(self.L.vec_get_scalars(self.h, C.byref(s)), "scalars")
        return s

    def set_scalars(self, s):
        self._chk(self.L.vec_set_scalars(self.h, C.byref(s)), "set_scalars")

    def state(self):
        d = {n: self.get(n) for n in STATE_FIELDS}
        d["bxbar"] = self.get_mean("bxbar")
        d["bybar"] = self.get_mean("bybar")
        return d

    def load_state(self, d, bzbar=None):
        for n in STATE_FIELDS:
            if n in d:
                self.set(n, d[n])
        for n in ("bxbar", "bybar"):
            if n in d:
                self.set_mean(n, d[n])
        if bzbar is not None:
            self.bzbar = bzbar

    # -- src/fft.F90 ---------------------------------------------------------------
    def _o1(self, fn, fin, name):
        fin = np.ascontiguousarray(fin, dtype=np.float64).reshape(self.shape)
        out = np.empty_like(fin)
        self._chk(fn(self.h, fin.ctypes.data, out.ctypes.data), name)
        return out

    def d1bydx(self, f): return self._o1(self.L.vec_d1bydx, f, "d1bydx")
    def d1bydy(self, f): return self._o1(self.L.vec_d1bydy, f, "d1bydy")
    def forwardfft(self, f): return self._o1(self.L.vec_forwardfft, f, "forwardfft")
    def inversefft(self, f): return self._o1(self.L.vec_inversefft, f, "inversefft")

    def d2bydx(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(self.shape)
        a, b = np.empty_like(f), np.empty_like(f)
        self._chk(self.L.vec_d2bydx(self.h, f.ctypes.data, a.ctypes.data, b.ctypes.data), "d2bydx")
        return a, b

    def d2bydy(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(self.shape)
        a, b = np.empty_like(f), np.empty_like(f)
        self._chk(self.L.vec_d2bydy(self.h, f.ctypes.data, a.ctypes.data, b.ctypes.data), "d2bydy")
        return a, b

    def dealias(self, f):
        z = np.array(f, dtype=np.float64).reshape(self.shape)
        self._chk(self.L.vec_dealias(self.h, z.ctypes.data), "dealias")
        return z

    # FP32 line kernels of the split form (VEC_OP_*: 1 d1, 2 d2, 3 dealias, 4 forward, 5 inverse)
    def line_f32(self, direction, op1, f, op2=0):
        f = np.ascontiguousarray(f, dtype=np.float32).reshape(self.shape)
        a = np.empty_like(f)
        b = np.empty_like(f) if op2 else None
        self._chk(self.L.vec_line_f32(self.h, direction, op1, op2, f.ctypes.data, a.ctypes.data,
                                      b.ctypes.data if op2 else None), "line_f32")
        return (a, b) if op2 else a

    def set_tunables(self, kc=16, s=0):
        self._chk(self.L.vec_set_tunables(self.h, kc, s), "set_tunables")

    # -- src/dbydz.F90 ---------------------------------------------------------------
    def _oz(self, fn, f, flag, shape, name):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(shape)
        out = np.empty_like(f)
        self._chk(fn(self.h, f.ctypes.data, out.ctypes.data, flag), name)
        return out

    def d1bydz(self, f, flag): return self._oz(self.L.vec_d1bydz, f, flag, self.shape, "d1bydz")
    def d1upbydz(self, f, flag): return self._oz(self.L.vec_d1upbydz, f, flag, self.shape, "d1upbydz")
    def d2bydz(self, f, flag): return self._oz(self.L.vec_d2bydz, f, flag, self.shape, "d2bydz")
    def d1bydz1d(self, f, flag): return self._oz(self.L.vec_d1bydz1d, f, flag, (self.p.nz,), "d1bydz1D")
    def d2bydz1d(self, f, flag): return self._oz(self.L.vec_d2bydz1d, f, flag, (self.p.nz,), "d2bydz1D")

    # -- physics -------------------------------------------------------------------------
    def static(self): self._chk(self.L.vec_static(self.h), "static")
    def mag_init(self): self._chk(self.L.vec_mag_init(self.h), "mag_init")
    def hydro_deriv(self): self._chk(self.L.vec_hydro_deriv(self.h), "hydro_deriv")
    def mag_deriv(self): self._chk(self.L.vec_mag_deriv(self.h), "mag_deriv")
    def bandj(self): self._chk(self.L.vec_bandj(self.h), "bandj")
    def magdealias(self): self._chk(self.L.vec_magdealias(self.h), "magdealias")
    def boundary(self): self._chk(self.L.vec_boundary(self.h), "boundary")
    def mag_boundary(self): self._chk(self.L.vec_mag_boundary(self.h), "mag_boundary")
    def ab3_update(self): self._chk(self.L.vec_ab3_update(self.h), "ab3_update")

    def calcdt(self):
        dt = C.c_double()
        self._chk(self.L.vec_calcdt(self.h, C.byref(dt)), "calcdt")
        return dt.value

    def diag(self):
        d = VecDiag()
        st = self.L.vec_diag(self.h, C.byref(d))
        return st, d.as_dict()

    def last_diag(self):
        d = VecDiag()
        self.L.vec_last_diag(self.h, C.byref(d))
        return d.as_dict()

    def step(self, n=1):
        """n iterations of the time loop (src/main.F90:340-747); returns the status."""
        return self.L.vec_step(self.h, n)

    def start(self):
        """static IC, calcdt, mag_init (src/main.F90:275-333, nframe=0)."""
        self.static()
        self.calcdt()
        if self.p.f != 0.0 or self.p.kinematic:
            self.mag_init()

    # -- instrumentation -----------------------------------------------------------------
    def stream(self):
        return self.L.vec_stream(self.h)

    def sync(self):
        self._chk(self.L.vec_sync(self.h), "sync")

    def profile(self, on=True):
        self._chk(self.L.vec_profile(self.h, 1 if on else 0), "profile")

    def profile_reset(self):
        self.L.vec_profile_reset(self.h)

    def profile_records(self):
        out = []
        name = C.create_string_buffer(64)
        for i in range(self.L.vec_profile_count(self.h)):
            n, ms, by = C.c_int(), C.c_double(), C.c_double()
            self.L.vec_profile_get(self.h, i, name, C.byref(n), C.byref(ms), C.byref(by))
            out.append((name.value.decode(), n.value, ms.value, by.value))
        return out

    def launch_count(self):
        return self.L.vec_launch_count(self.h)

    def use_graphs(self, on=True):
        self._chk(self.L.vec_use_graphs(self.h, 1 if on else 0), "use_graphs")

    def top_nusselt(self):
        v = C.c_double()
        self._chk(self.L.vec_top_nusselt(self.h, C.byref(v)), "top_nusselt")
        return v.value

    def tunables(self):
        kc, s = C.c_int(), C.c_int()
        self._chk(self.L.vec_tunables(self.h, C.byref(kc), C.byref(s)), "tunables")
        return kc.value, s.value

    # -- snapshots (src/netcdf.F90) -------------------------------------------------
    def write_snapshot(self, path, iprec=8, history=""):
        self._chk(self.L.vec_write_snapshot(self.h, str(path).encode(), iprec, history.encode()),
                  "write_snapshot")

    def read_restart(self, path):
        self._chk(self.L.vec_read_restart(self.h, str(path).encode()), "read_restart")


def read_input(path):
    """Parse a reference INPUT file (src/initial.F90:94-201) via the C-ABI."""
    p = VecParams()
    st = _L.load().vec_params_read_input(path.encode(), C.byref(p))
    if st != 0:
        raise VecError("vec_params_read_input", st)
    return p


SNAP_FIELDS = ("R", "T", "U", "V", "W", "Bx", "By", "Bz")
SNAP_ATTRS = ("gamma", "sigma", "theta", "ck", "cm", "f", "tayl", "psi", "zeta", "xmax", "ymax")


def nc_read(path):
    """Read a reference-layout NetCDF snapshot (no GPU needed): returns a dict
    with the 8 fields as (nz, ny, nx) arrays plus scalars and attributes."""
    L = _L.load()
    s = VecSnapshot()
    st = L.vec_nc_read(str(path).encode(), C.byref(s))
    if st != 0:
        raise VecError("vec_nc_read", st)
    shape = (s.nz, s.ny, s.nx)
    arrs = [np.empty(shape, dtype=np.float64) for _ in SNAP_FIELDS]
    for i, a in enumerate(arrs):
        s.fields[i] = a.ctypes.data
    st = L.vec_nc_read(str(path).encode(), C.byref(s))
    if st != 0:
        raise VecError("vec_nc_read", st)
    out = dict(zip(SNAP_FIELDS, arrs))
    out.update(time=s.time, iteration=s.iteration, timestep=s.timestep, version=s.version,
               history=s.history.decode(errors="replace"))
    out.update({a: getattr(s, a) for a in SNAP_ATTRS})
    return out


def nc_write(path, snap, iprec=8, fmt=1):
    """Write a dict like nc_read's result as a reference-layout snapshot
    (fmt 1: classic NetCDF; fmt 2: 64-bit offsets)."""
    L = _L.load()
    s = VecSnapshot()
    nz, ny, nx = np.asarray(snap["R"]).shape
    s.nx, s.ny, s.nz = nx, ny, nz
    s.time, s.iteration, s.timestep = snap.get("time", 0.0), snap.get("iteration", 0), snap.get("timestep", 0.0)
    s.version = snap.get("version", 3)
    s.history = snap.get("history", "").encode()[:79]
    for a in SNAP_ATTRS:
        setattr(s, a, float(snap.get(a, 0.0)))
    keep = [np.ascontiguousarray(snap[n], dtype=np.float64) for n in SNAP_FIELDS]
    for i, a in enumerate(keep):
        s.fields[i] = a.ctypes.data
    st = L.vec_nc_write_fmt(str(path).encode(), C.byref(s), iprec, fmt)
    if st != 0:
        raise VecError("vec_nc_write", st)


class Ensemble:
    """Independent instances stepped together as one captured CUDA graph."""

    def __init__(self, params_list):
        self.L = _L.load()
        arr = (VecParams * len(params_list))(*[p.copy() for p in params_list])
        h = C.c_void_p()
        st = self.L.vec_ensemble_create(arr, len(params_list), C.byref(h))
        if st != 0:
            raise VecError("vec_ensemble_create", st)
        self.h = h
        self.members = [P3D(params_list[i], handle=C.c_void_p(self.L.vec_ensemble_member(h, i)))
                        for i in range(len(params_list))]

    def close(self):
        if getattr(self, "h", None):
            for m in self.members:
                m.h = None
            self.L.vec_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, st, where):
        if st != 0:
            raise VecError(where, st)

    def start(self):
        self._chk(self.L.vec_ensemble_start(self.h), "ensemble_start")

    def step(self, n=1):
        return self.L.vec_ensemble_step(self.h, n)

    def sync(self):
        self._chk(self.L.vec_ensemble_sync(self.h), "ensemble_sync")

    def tune(self, steps=3, cache=None):
        self._chk(self.L.vec_ensemble_tune(self.h, steps, cache.encode() if cache else None), "ensemble_tune")
