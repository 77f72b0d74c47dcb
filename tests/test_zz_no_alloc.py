"""The allocation-free calcdt entry point against the context-based one.

vec_calcdt_noalloc serves callers that cannot allocate device memory (their
own arena or pool owns the whole device heap), so it takes the caller's
device fields and keeps its reduction scratch in a fixed array inside the
library.  This test compares it with vec_calcdt on calls in a row:

* the first call on a larger grid with large speeds and low density, the
  second on a smaller grid with small speeds: the second call reduces over
  fewer CTAs, so partials the first call left behind would win its maxima
  and minimum if they leaked;
* host and device outputs, the default stream and a torch stream;
* a warm call leaves the device's free memory unchanged;
* pointers that are not device memory of the current device, and grids
  beyond the scratch limit, are rejected.

Tolerance: 1e-14 relative (both reduce with max/min, which are exact).
"""
import ctypes as C

import numpy as np
import pytest

from fug30v0kxc_gb300.params import convection_params
from fug30v0kxc_gb300.solver import P3D
from tests.helpers import smooth_state

pytestmark = pytest.mark.gpu

NAMES = ("u", "v", "w", "r", "t", "bx", "by", "bz")


def _case(torch, grid, speed, density, seed):
    """A context holding a scaled smooth state, its vec_calcdt, and device
    copies of its fields."""
    p = convection_params(*grid, eta_contrast=20.0)
    g = P3D(p)
    s = smooth_state(p, seed=seed)
    for n in ("u", "v", "w"):
        s[n] = s[n] * speed
    s["r"] = s["r"] * density
    for n, a in s.items():
        g.set(n, a)
    dt_ref = g.calcdt()
    d = {n: torch.from_numpy(g.get(n)).cuda() for n in NAMES}
    torch.cuda.synchronize()
    return p, g, dt_ref, d


def _call(L, p, d, out_ptr, stream=None):
    return L.vec_calcdt_noalloc(C.byref(p), *[d[n].data_ptr() for n in NAMES], out_ptr, stream)


def test_calcdt_noalloc_matches_context_calcdt():
    torch = pytest.importorskip("torch")
    # large grid, fast and light (the CFL terms set dt); then a smaller grid,
    # slow and dense, whose dt the first call's partials would shrink
    big = _case(torch, (96, 64, 33), 3000.0, 0.2, seed=1)
    small = _case(torch, (32, 32, 17), 1.0, 1.0, seed=2)
    L = big[1].L
    results = []
    side = torch.cuda.Stream()
    for (p, g, dt_ref, d), dev_out, stream in ((big, False, None), (small, True, None),
                                               (big, True, side), (small, False, side)):
        if dev_out:
            out = torch.zeros(1, dtype=torch.float64, device="cuda")
            ptr = out.data_ptr()
        else:
            out = np.zeros(1)
            ptr = out.ctypes.data
        torch.cuda.synchronize()
        st = _call(L, p, d, ptr, C.c_void_p(stream.cuda_stream) if stream is not None else None)
        assert st == 0, L.vec_last_error()
        torch.cuda.synchronize()
        dt = float(out[0])
        assert abs(dt - dt_ref) <= 1e-14 * dt_ref, (dt, dt_ref, p.nx)
        results.append(dt)
    assert results[0] != results[1]
    for c in (big, small):
        c[1].close()


def test_calcdt_noalloc_warm_call_allocates_nothing():
    torch = pytest.importorskip("torch")
    p, g, dt_ref, d = _case(torch, (64, 48, 33), 1.0, 1.0, seed=3)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert _call(g.L, p, d, out.data_ptr()) == 0     # first call: the scratch is in place
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _call(g.L, p, d, out.data_ptr()) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert abs(float(out[0]) - dt_ref) <= 1e-14 * dt_ref
    g.close()


def test_calcdt_noalloc_rejects_foreign_pointers():
    torch = pytest.importorskip("torch")
    p, g, _, d = _case(torch, (32, 32, 17), 1.0, 1.0, seed=4)
    out = np.zeros(1)
    host_u = g.get("u")
    ptrs = [d[n].data_ptr() for n in NAMES]
    ptrs[0] = host_u.ctypes.data               # a host field
    st = g.L.vec_calcdt_noalloc(C.byref(p), *ptrs, out.ctypes.data, None)
    assert st == -31
    assert b"not device memory" in g.L.vec_last_error()
    g.close()


def test_calcdt_noalloc_rejects_oversize_grid():
    torch = pytest.importorskip("torch")
    p = convection_params(1024, 1024, 129)
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = np.zeros(1)
    from fug30v0kxc_gb300 import lib
    L = lib.load()
    st = L.vec_calcdt_noalloc(C.byref(p), *[x.data_ptr()] * 8, out.ctypes.data, None)
    assert st == -32
    assert b"exceed" in L.vec_last_error()
