"""Failure paths, exercised without faulting the GPU.

* A non-finite value injected on the host (a NaN or an infinity in one
  element of one uploaded field) is reported as VEC_ERR_NAN (-20) by
  vec_calcdt, by vec_diag (before the div B check, which fmin/fmax would
  otherwise pass: the reference aborts on div B, src/main.F90:583-590), by
  vec_step through the calcdt it runs every 10 steps, and by the ensemble
  step.  The context stays usable: a finite state uploaded afterwards
  passes both checks again.
* The bounded waits of the line kernels: a self-test kernel waits on a
  barrier nothing arrives on, gives up after a short limit and raises the
  context's error flag; vec_sync reports VEC_ERR_CUDA (-30) once and the
  context keeps working.
"""
import numpy as np
import pytest

from fug30v0kxc_gb300.params import VEC_PREC_FP64, VEC_PREC_SPLIT
from fug30v0kxc_gb300.solver import P3D, Ensemble, VecError
from tests.helpers import small_params

pytestmark = pytest.mark.gpu

NAN_ERR, CUDA_ERR = -20, -30


def _started(precision, **kw):
    p = small_params(32, 32, 17, eta_contrast=5.0, precision=precision, **kw)
    p.ndu06 = 1000
    g = P3D(p)
    g.start()
    assert g.step(3) == 0
    return g


@pytest.mark.parametrize("precision", [VEC_PREC_FP64, VEC_PREC_SPLIT])
@pytest.mark.parametrize("field,value", [("t", np.nan), ("u", np.inf), ("bx", np.nan), ("r", -np.inf)])
def test_injected_nonfinite_is_reported(precision, field, value):
    g = _started(precision)
    good = {n: g.get(n) for n in ("r", "t", "u", "v", "w", "bx", "by", "bz")}
    bad = good[field].copy()
    bad[g.p.nz // 2, 5, 7] = value
    g.set(field, bad)
    with pytest.raises(VecError) as e:
        g.calcdt()
    assert e.value.status == NAN_ERR
    st, _ = g.diag()
    assert st == NAN_ERR
    # the time loop: the calcdt of the tenth step meets it
    assert g.step(10) == NAN_ERR
    # a finite state uploaded afterwards passes both checks again
    for n, a in good.items():
        g.set(n, a)
    g.calcdt()
    st, _ = g.diag()
    assert st == 0
    g.close()


def test_nonfinite_in_div_b_fails_the_diagnostics():
    """NaN in bz only reaches the diagnostics through div B (bz's z
    derivative) and the extrema; it must not pass the |div B| > 0.01 test."""
    g = _started(VEC_PREC_FP64)
    bz = g.get("bz")
    bz[4, 3, 3] = np.nan
    g.set("bz", bz)
    st, d = g.diag()
    assert st == NAN_ERR, (st, d["divbmax"], d["divbmin"])
    g.close()


def test_diagnostics_step_reports_nonfinite():
    """A diagnostics step of the time loop (every ndu06 steps) reports it
    before any calcdt step comes."""
    p = small_params(32, 32, 17, precision=VEC_PREC_SPLIT)
    p.ndu06 = 4
    g = P3D(p)
    g.start()
    assert g.step(1) == 0
    u = g.get("u")
    u[8, 1, 1] = np.nan
    g.set("u", u)
    assert g.step(3) == NAN_ERR
    g.close()


def test_ensemble_step_reports_nonfinite_member():
    ps = [small_params(32, 32, 17, precision=VEC_PREC_SPLIT), small_params(64, 32, 17, precision=VEC_PREC_SPLIT)]
    for p in ps:
        p.ndu06 = 1000
    ens = Ensemble(ps)
    ens.start()
    assert ens.step(2) == 0
    ens.sync()
    m = ens.members[1]
    t = m.get("t")
    t[5, 2, 2] = np.nan
    m.set("t", t)
    assert ens.step(10) == NAN_ERR
    assert b"member 1" in m.L.vec_last_error()
    ens.close()


def test_bounded_wait_runs_out_and_is_reported_once():
    g = _started(VEC_PREC_SPLIT)
    L = g.L
    g.hydro_deriv()
    before = {n: g.get(n) for n in ("rdot3", "tdot3", "udot3", "wdot3")}
    assert L.vec_selftest_wait(g.h, 0) == -31
    assert L.vec_selftest_wait(g.h, 1 << 25) == -31
    assert L.vec_selftest_wait(g.h, 1000) == 0
    assert L.vec_sync(g.h) == CUDA_ERR
    assert b"wait" in L.vec_last_error()
    assert L.vec_sync(g.h) == 0
    # the context still computes, and computes the same
    g.hydro_deriv()
    for n, a in before.items():
        assert np.array_equal(g.get(n), a), n
    assert g.step(12) == 0
    g.close()
