"""Parity from the reference's own developed state, bin/restart.nc (30x30x60,
iteration 105000; committed as tests/golden/restart_30x30x60.npz), read the
way a restart does (nframe = 1: parameters from the file, histories not
restored, first step Euler): 20 steps on the GPU against the oracle, FP64
(1e-9) and the split form (per-field relative L2 < 1e-4).  Also the NetCDF
snapshot path through the context (vec_write_snapshot / vec_read_restart)."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from fug30v0kxc_gb300.params import VEC_PREC_FP64, VEC_PREC_SPLIT, default_params
from fug30v0kxc_gb300.solver import P3D, SNAP_ATTRS, SNAP_FIELDS, nc_read
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(__file__), "golden", "restart_30x30x60.npz")
MAP = {"R": "r", "T": "t", "U": "u", "V": "v", "W": "w", "Bx": "bx", "By": "by", "Bz": "bz"}


def _params(precision):
    d = np.load(FIX)
    p = default_params()         # bin/INPUT flags: fixed-T bottom, vertical field
    for a in SNAP_ATTRS:
        setattr(p, a, float(d[a]))
    p.nz, p.ny, p.nx = d["R"].shape
    p.precision = precision
    p.ndu06 = 10
    return p, d


def _load(obj, d):
    for n, m in MAP.items():
        obj.set(m, d[n])


@pytest.mark.parametrize("precision", [VEC_PREC_FP64, VEC_PREC_SPLIT])
def test_restart_state_parity(precision):
    p, d = _params(precision)
    g, o = P3D(p), O.Oracle(p)
    _load(g, d)
    _load(o, d)
    o.calcdt(); g.calcdt()
    o.mag_init(); g.mag_init()
    assert g.step(20) == 0 and o.step(20) == 0
    for n in ("r", "t", "u", "v", "w", "pol", "tor", "bx", "by", "bz"):
        a, b = g.get(n), o.get(n)
        if precision == VEC_PREC_FP64:
            assert rel_err(a, b) < 1e-9, n
        else:
            l2 = np.linalg.norm(a - b) / np.linalg.norm(b - (b.mean() if n in ("r", "t", "bz") else 0.0))
            assert l2 < 1e-4, (n, l2)
    dg, do = g.last_diag(), o.last_diag()
    for k in ("kenergy", "menergy", "nusselt"):
        tol = 1e-8 if precision == VEC_PREC_FP64 else 1e-3
        assert abs(dg[k] - do[k]) <= tol * abs(do[k]), k


def test_snapshot_through_context(tmp_path):
    p, d = _params(VEC_PREC_FP64)
    g = P3D(p)
    _load(g, d)
    g.calcdt()
    g.mag_init()
    assert g.step(3) == 0
    path = tmp_path / "T16_000.nc"
    g.write_snapshot(path, iprec=8, history="GPU snapshot")
    snap = nc_read(path)
    for n, m in MAP.items():
        assert np.array_equal(snap[n], g.get(m)), n
    s = g.scalars()
    assert snap["iteration"] == s.iter and snap["time"] == s.ttime and snap["timestep"] == s.dt1
    h = P3D(p)
    h.read_restart(path)
    for n, m in MAP.items():
        assert np.array_equal(h.get(m), g.get(m)), n
    sh = h.scalars()
    assert sh.first == 1 and sh.iter == s.iter and sh.dt1 == s.dt1
