"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
cpu_baseline / --impl reference legs of bench.py, always as the checker.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from fug30v0kxc_gb300.params import (FIELD_NAMES, MEAN_NAMES, STATE_FIELDS, VecDiag,
                                     VecParams, VecScalars)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
_lib = None


def build(force=False):
    if force or not os.path.exists(LIB):
        subprocess.check_call(["make", "-s", "-C", HERE])
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp = C.c_void_p
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        L.or_create.restype = vp
        L.or_create.argtypes = [C.POINTER(VecParams), C.POINTER(C.c_int)]
        L.or_destroy.argtypes = [vp]
        L.or_nthreads.argtypes = [C.c_int]
        for n in ("or_r2hc", "or_hc2r"):
            getattr(L, n).argtypes = [C.c_int, dp, dp]
        L.or_field.argtypes = [vp, C.c_int, C.c_void_p, C.c_void_p]
        L.or_mean.argtypes = [vp, C.c_int, C.c_void_p, C.c_void_p]
        L.or_scalars.argtypes = [vp, C.c_void_p, C.c_void_p]
        L.or_bzbar.argtypes = [vp, C.c_void_p]
        L.or_bzbar.restype = C.c_double
        L.or_calcdt.argtypes = [vp, C.POINTER(C.c_double)]
        for n in ("or_d1bydx", "or_d1bydy", "or_forwardfft", "or_inversefft"):
            getattr(L, n).argtypes = [vp, dp, dp]
        for n in ("or_d2bydx", "or_d2bydy"):
            getattr(L, n).argtypes = [vp, dp, dp, dp]
        L.or_dealias.argtypes = [vp, dp]
        for n in ("or_d1bydz", "or_d1upbydz", "or_d2bydz", "or_d1bydz1d", "or_d2bydz1d"):
            getattr(L, n).argtypes = [vp, dp, dp, C.c_int]
        for n in ("or_static", "or_mag_init", "or_hydro_deriv", "or_mag_deriv", "or_bandj",
                  "or_magdealias", "or_boundary", "or_mag_boundary", "or_ab3_update"):
            getattr(L, n).argtypes = [vp]
        L.or_diag.argtypes = [vp, C.POINTER(VecDiag)]
        L.or_last_diag.argtypes = [vp, C.POINTER(VecDiag)]
        L.or_step.argtypes = [vp, C.c_int]
        _lib = L
    return _lib


def nthreads(n=0):
    return lib().or_nthreads(n)


def r2hc(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    assert lib().or_r2hc(len(x), x, out) == 0
    return out


def hc2r(h):
    h = np.ascontiguousarray(h, dtype=np.float64)
    out = np.empty_like(h)
    assert lib().or_hc2r(len(h), h, out) == 0
    return out


class OracleError(RuntimeError):
    pass


class Oracle:
    """The reference serial path on the CPU, state in module-global style."""

    def __init__(self, params: VecParams):
        self.p = params.copy()
        st = C.c_int(0)
        self.h = lib().or_create(C.byref(self.p), C.byref(st))
        if not self.h:
            raise OracleError(f"or_create failed: {st.value}")
        self.shape = (self.p.nz, self.p.ny, self.p.nx)

    def close(self):
        if self.h:
            lib().or_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _chk(self, st, what):
        if st != 0:
            raise OracleError(f"{what}: status {st}")
        return st

    # -- state -----------------------------------------------------------
    def get(self, name):
        out = np.empty(self.shape, dtype=np.float64)
        self._chk(lib().or_field(self.h, FIELD_NAMES[name], out.ctypes.data, None), name)
        return out

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self.shape)
        self._chk(lib().or_field(self.h, FIELD_NAMES[name], None, a.ctypes.data), name)

    def get_mean(self, name):
        out = np.empty(self.p.nz, dtype=np.float64)
        self._chk(lib().or_mean(self.h, MEAN_NAMES[name], out.ctypes.data, None), name)
        return out

    def set_mean(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self._chk(lib().or_mean(self.h, MEAN_NAMES[name], None, a.ctypes.data), name)

    @property
    def bzbar(self):
        return lib().or_bzbar(self.h, None)

    @bzbar.setter
    def bzbar(self, v):
        x = C.c_double(v)
        lib().or_bzbar(self.h, C.addressof(x))

    def scalars(self):
        s = VecScalars()
        lib().or_scalars(self.h, C.addressof(s), None)
        return s

    def set_scalars(self, s):
        lib().or_scalars(self.h, None, C.addressof(s))

    def state(self):
        d = {n: self.get(n) for n in STATE_FIELDS}
        d["bxbar"] = self.get_mean("bxbar")
        d["bybar"] = self.get_mean("bybar")
        return d

    # -- operators ---------------------------------------------------------
    def _op1(self, fn, fin):
        fin = np.ascontiguousarray(fin, dtype=np.float64).reshape(self.shape)
        out = np.empty_like(fin)
        self._chk(fn(self.h, fin, out), fn.__name__)
        return out

    def d1bydx(self, f): return self._op1(lib().or_d1bydx, f)
    def d1bydy(self, f): return self._op1(lib().or_d1bydy, f)
    def forwardfft(self, f): return self._op1(lib().or_forwardfft, f)
    def inversefft(self, f): return self._op1(lib().or_inversefft, f)

    def d2bydx(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(self.shape)
        a, b = np.empty_like(f), np.empty_like(f)
        self._chk(lib().or_d2bydx(self.h, f, a, b), "d2bydx")
        return a, b

    def d2bydy(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(self.shape)
        a, b = np.empty_like(f), np.empty_like(f)
        self._chk(lib().or_d2bydy(self.h, f, a, b), "d2bydy")
        return a, b

    def dealias(self, f):
        z = np.array(f, dtype=np.float64).reshape(self.shape)
        self._chk(lib().or_dealias(self.h, z), "dealias")
        return z

    def _opz(self, fn, f, flag, shape):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(shape)
        out = np.empty_like(f)
        st = fn(self.h, f, out, flag)
        if st != 0:
            raise OracleError(f"{fn.__name__}: status {st}")
        return out

    def d1bydz(self, f, flag): return self._opz(lib().or_d1bydz, f, flag, self.shape)
    def d1upbydz(self, f, flag): return self._opz(lib().or_d1upbydz, f, flag, self.shape)
    def d2bydz(self, f, flag): return self._opz(lib().or_d2bydz, f, flag, self.shape)
    def d1bydz1d(self, f, flag): return self._opz(lib().or_d1bydz1d, f, flag, (self.p.nz,))
    def d2bydz1d(self, f, flag): return self._opz(lib().or_d2bydz1d, f, flag, (self.p.nz,))

    # -- physics -------------------------------------------------------------
    def static(self): self._chk(lib().or_static(self.h), "static")
    def mag_init(self): self._chk(lib().or_mag_init(self.h), "mag_init")
    def hydro_deriv(self): self._chk(lib().or_hydro_deriv(self.h), "hydro_deriv")
    def mag_deriv(self): self._chk(lib().or_mag_deriv(self.h), "mag_deriv")
    def bandj(self): self._chk(lib().or_bandj(self.h), "bandj")
    def magdealias(self): self._chk(lib().or_magdealias(self.h), "magdealias")
    def boundary(self): self._chk(lib().or_boundary(self.h), "boundary")
    def mag_boundary(self): self._chk(lib().or_mag_boundary(self.h), "mag_boundary")
    def ab3_update(self): self._chk(lib().or_ab3_update(self.h), "ab3_update")

    def calcdt(self):
        dt = C.c_double(0.0)
        self._chk(lib().or_calcdt(self.h, C.byref(dt)), "calcdt")
        return dt.value

    def diag(self):
        d = VecDiag()
        st = lib().or_diag(self.h, C.byref(d))
        return st, d.as_dict()

    def last_diag(self):
        d = VecDiag()
        lib().or_last_diag(self.h, C.byref(d))
        return d.as_dict()

    def step(self, n=1):
        return lib().or_step(self.h, n)

    def start(self):
        """static IC, calcdt, mag_init: src/main.F90:275-333 (nframe=0)."""
        self.static()
        self.calcdt()
        if self.p.f != 0.0 or self.p.kinematic:
            self.mag_init()
