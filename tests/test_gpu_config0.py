"""The reference's CPU-runnable case (64^2 x 65, Ra 1e5, Q 100, eta contrast
5, seeded +-1e-3 temperature noise, 1000 AB3 steps at SF 0.3, diagnostics
every 100 steps) on the GPU against the CPU oracle over the whole run.

* FP64 drop-in: every state field agrees with the oracle to 1e-9 relative L2
  after 1000 steps (only the FFT factorisation and FMA contraction differ;
  measured 1e-15 for r and T, 1e-10 for u, v, pol), except the toroidal
  potential (1e-7; measured 6e-9): it is driven by the vertical vorticity, a
  difference of nearly equal derivatives, so its relative error is the
  rounding of those derivatives over its small norm.  Every diagnostic
  sample agrees to 1e-9 relative.
* Split form: the per-field relative L2 of the deviation from the static
  state stays below 1e-3 (tor: 5e-2, see test_gpu_split), and the time
  averages of the top Nusselt number, the kinetic energy, the magnetic
  energy and the magnetic energy of the field perturbation are within 1 %
  of the FP64 oracle's.  With the fixed-flux bottom of this case the
  reference's own (bottom) Nusselt number is identically one, so the
  fixed-temperature top carries the heat-flux comparison; the uniform seed
  field dominates the magnetic energy, so its perturbation part is
  compared as well.
"""
import numpy as np
import pytest

from oracle import oracle as O
from fug30v0kxc_gb300.params import VEC_PREC_FP64, VEC_PREC_SPLIT, config0
from fug30v0kxc_gb300.solver import P3D
from tests.helpers import perturbation_menergy, top_nusselt

pytestmark = pytest.mark.gpu

FIELDS = ("r", "t", "u", "v", "w", "pol", "tor")


def _rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


@pytest.fixture(scope="module")
def oracle_run():
    p = config0(precision=VEC_PREC_FP64)
    p.ndu06 = 100
    o = O.Oracle(p)
    o.start()
    diags = []
    for _ in range(10):
        assert o.step(100) == 0
        d = o.last_diag()
        d["nusselt_top"] = top_nusselt(p, o.get("t"))
        d["menergy_pert"] = perturbation_menergy(p, o.get("bx"), o.get("by"), o.get("bz"), o.bzbar)
        diags.append(d)
    return p, {n: o.get(n) for n in FIELDS}, diags


def _gpu_run(precision):
    p = config0(precision=precision)
    p.ndu06 = 100
    g = P3D(p)
    g.start()
    diags = []
    for _ in range(10):
        assert g.step(100) == 0
        d = g.last_diag()
        d["nusselt_top"] = g.top_nusselt()
        d["menergy_pert"] = perturbation_menergy(p, g.get("bx"), g.get("by"), g.get("bz"), g.bzbar)
        diags.append(d)
    return g, diags


def test_fp64_1000_steps_match_oracle(oracle_run):
    p, ref, rdiag = oracle_run
    g, gdiag = _gpu_run(VEC_PREC_FP64)
    errs = {n: _rel_l2(g.get(n), ref[n]) for n in FIELDS}
    print("FP64 vs oracle after 1000 steps:", errs)
    for n, e in errs.items():
        assert e < (1e-7 if n == "tor" else 1e-9), (n, e)
    for dg, do in zip(gdiag, rdiag):
        for k in ("nusselt", "nusselt_top", "kenergy", "menergy"):
            assert abs(dg[k] - do[k]) <= 1e-9 * abs(do[k]), (k, dg[k], do[k])
        assert abs(dg["menergy_pert"] - do["menergy_pert"]) <= 1e-6 * abs(do["menergy_pert"])
    g.close()


def test_split_1000_steps_vs_oracle(oracle_run):
    p, ref, rdiag = oracle_run
    g, gdiag = _gpu_run(VEC_PREC_SPLIT)
    z = np.arange(p.nz) / (p.nz - 1)
    t0 = (1.0 + p.theta * z)[:, None, None]
    errs = {}
    for n in FIELDS:
        a, b = g.get(n), ref[n]
        if n in ("r", "t"):
            bg = t0 ** p.cm if n == "r" else t0
            a, b = a - bg, b - bg
        errs[n] = _rel_l2(a, b)
    print("split vs FP64 oracle after 1000 steps:", errs)
    for n, e in errs.items():
        assert e < (5e-2 if n == "tor" else 1e-3), (n, e)
    print("time averages (split, oracle):",
          {k: (np.mean([d[k] for d in gdiag]), np.mean([d[k] for d in rdiag]))
           for k in ("nusselt_top", "kenergy", "menergy", "menergy_pert")})
    for k in ("nusselt_top", "kenergy", "menergy", "menergy_pert"):
        a = np.mean([d[k] for d in gdiag])
        b = np.mean([d[k] for d in rdiag])
        assert abs(a - b) <= 0.01 * abs(b), (k, a, b)
    g.close()


@pytest.mark.parametrize("var,values", [("VEC_SERIAL_MAG", ("0", "1")), ("VEC_PDL", ("1", "0"))])
def test_fp64_step_forms_bit_identical(var, values, monkeypatch):
    """The FP64 step's magnetic branch on a second stream (its default)
    against the serial order, and programmatic dependent launches against
    ordinary ones: 12 steps of the config-0 physics at 64^2 x 33 give the
    same bits."""
    from tests.helpers import smooth_state
    states = []
    for val in values:
        monkeypatch.setenv(var, val)
        p = config0(precision=VEC_PREC_FP64)
        p.nz = 33
        p.ndu06 = 1000
        g = P3D(p)
        for n, a in smooth_state(p, seed=3).items():
            g.set(n, a)
        g.calcdt()
        g.mag_init()
        assert g.step(12) == 0
        states.append({n: g.get(n) for n in ("r", "t", "u", "v", "w", "pol", "tor", "bx", "by", "bz")})
        g.close()
    for n in states[0]:
        assert np.array_equal(states[0][n], states[1][n]), (var, n)
