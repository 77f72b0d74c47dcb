"""The allocation-free calcdt entry point against the context-based one.

vec_calcdt_noalloc serves callers that cannot allocate device memory (their
own arena or pool owns the whole device heap), so it takes the caller's
device fields and keeps its reduction scratch in a fixed array inside the
library.  This test compares it with vec_calcdt on two calls in a row with
different states (the second call must not see the first call's partials),
once with a host and once with a device output, and checks the size limit.
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


def _device_fields(torch, g):
    return {n: torch.from_numpy(g.get(n)).cuda() for n in NAMES}


def test_calcdt_noalloc_matches_context_calcdt():
    torch = pytest.importorskip("torch")
    p = convection_params(64, 48, 33, eta_contrast=20.0)
    g = P3D(p)
    L = g.L
    results = []
    # the second state has velocities large enough that the CFL limit, not
    # the (state-independent) magnetic diffusion limit, sets dt
    for seed, scale, dev_out in ((1, 1.0, False), (2, 2000.0, True)):
        s = smooth_state(p, seed=seed)
        for n in ("u", "v", "w"):
            s[n] = s[n] * scale
        for n, a in s.items():
            g.set(n, a)
        dt_ref = g.calcdt()
        d = _device_fields(torch, g)
        torch.cuda.synchronize()
        if dev_out:
            out = torch.zeros(1, dtype=torch.float64, device="cuda")
            ptr = out.data_ptr()
        else:
            out = np.zeros(1)
            ptr = out.ctypes.data
        st = L.vec_calcdt_noalloc(C.byref(p), *[d[n].data_ptr() for n in NAMES], ptr, None)
        assert st == 0, L.vec_last_error()
        torch.cuda.synchronize()
        dt = float(out[0])
        assert abs(dt - dt_ref) <= 1e-14 * dt_ref, (dt, dt_ref)
        results.append(dt)
    assert results[0] != results[1]


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
