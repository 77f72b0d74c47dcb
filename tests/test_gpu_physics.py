"""GPU parity of the physics entry points and of whole time steps.

Each test loads the same seeded state into the CUDA library and the CPU
oracle, runs the same reference routine on both and compares every output
array.  Tolerances (FP64): single routines 1e-11 relative to each array's
max; 20 full steps 1e-9 (rounding differences of FFT orderings and FMA
contraction, amplified by the time integration).
"""
import numpy as np
import pytest

from oracle import oracle as O
from fug30v0kxc_gb300.params import STATE_FIELDS, VEC_PREC_FP64, convection_params
from fug30v0kxc_gb300.solver import P3D
from tests.helpers import rel_err, smooth_state

pytestmark = pytest.mark.gpu

CASES = [
    dict(nx=32, ny=32, nz=17, eta_contrast=1.0),
    dict(nx=30, ny=20, nz=12, eta_contrast=5.0),
    dict(nx=64, ny=64, nz=33, eta_contrast=20.0),
]


def _setup(case, seed=0, **kw):
    c = dict(case)
    nx, ny, nz = c.pop("nx"), c.pop("ny"), c.pop("nz")
    p = convection_params(nx, ny, nz, **c)
    for k, v in kw.items():
        setattr(p, k, v)
    p.ndu06 = 7
    g, o = P3D(p), O.Oracle(p)
    s = smooth_state(p, seed=seed)
    for n, a in s.items():
        g.set(n, a)
        o.set(n, a)
    o.calcdt()
    g.calcdt()
    o.mag_init()
    g.mag_init()
    return g, o, p


def _cmp(g, o, names, tol):
    for n in names:
        a, b = g.get(n), o.get(n)
        e = rel_err(a, b)
        assert e < tol, f"{n}: {e:.3e}"


@pytest.mark.parametrize("case", CASES)
def test_mag_init(case):
    g, o, p = _setup(case)
    _cmp(g, o, ["pol", "tor", "jsq"], 1e-11)
    for m in ("bxbar", "bybar"):
        assert rel_err(g.get_mean(m), o.get_mean(m)) < 1e-11 or np.abs(o.get_mean(m)).max() < 1e-14
    assert abs(g.bzbar - o.bzbar) < 1e-13


@pytest.mark.parametrize("case", CASES)
def test_hydro_deriv(case):
    g, o, p = _setup(case)
    g.hydro_deriv()
    o.hydro_deriv()
    _cmp(g, o, ["rdot3", "tdot3", "udot3", "vdot3", "wdot3"], 1e-11)


@pytest.mark.parametrize("case", CASES)
def test_mag_deriv(case):
    g, o, p = _setup(case)
    g.mag_deriv()
    o.mag_deriv()
    _cmp(g, o, ["poldot3", "tordot3"], 1e-11)
    for m in ("bxbardot3", "bybardot3"):
        a, b = g.get_mean(m), o.get_mean(m)
        assert np.abs(a - b).max() <= 1e-11 * max(np.abs(b).max(), 1e-300) or np.abs(b).max() < 1e-15


@pytest.mark.parametrize("case", CASES)
def test_bandj(case):
    g, o, p = _setup(case)
    g.bandj()
    o.bandj()
    _cmp(g, o, ["bx", "by", "bz", "jsq"], 1e-11)


@pytest.mark.parametrize("radbc,constflux,perfect", [(0, 1, 0), (1, 0, 1), (0, 0, 0)])
def test_boundaries(radbc, constflux, perfect):
    g, o, p = _setup(CASES[0], radbc=radbc, constflux=constflux, perfect=perfect)
    g.boundary(); o.boundary()
    g.mag_boundary(); o.mag_boundary()
    _cmp(g, o, ["u", "v", "w", "t", "pol", "tor"], 1e-13)
    for m in ("bxbar", "bybar"):
        assert np.abs(g.get_mean(m) - o.get_mean(m)).max() < 1e-13


def test_calcdt_and_diag():
    for case in CASES:
        g, o, p = _setup(case)
        assert abs(g.calcdt() - o.calcdt()) < 1e-14 * o.calcdt()
        sg, dg = g.diag()
        so, do = o.diag()
        assert sg == so
        for k, v in do.items():
            assert abs(dg[k] - v) <= 1e-10 * max(abs(v), 1e-12), k
        _cmp(g, o, ["u", "v"], 1e-12)    # GlobalAverages removes the mean momentum


@pytest.mark.parametrize("case", CASES)
def test_steps_match_oracle(case):
    g, o, p = _setup(case)
    for chunk in (1, 1, 8, 10):          # Euler, AB2, AB3, dealias + calcdt at nit=10, 20
        sg = g.step(chunk)
        so = o.step(chunk)
        assert sg == so == 0
    _cmp(g, o, list(STATE_FIELDS), 1e-9)
    for m in ("bxbar", "bybar"):
        a, b = g.get_mean(m), o.get_mean(m)
        assert np.abs(a - b).max() <= 1e-9 * max(np.abs(b).max(), 1e-12)
    sg, so = g.scalars(), o.scalars()
    assert abs(sg.dt - so.dt) <= 1e-12 * so.dt
    assert abs(sg.ttime - so.ttime) <= 1e-12 * so.ttime
    assert sg.nit == so.nit == 20
    dg, do = g.last_diag(), o.last_diag()
    for k in ("kenergy", "menergy", "nusselt"):
        assert abs(dg[k] - do[k]) <= 1e-8 * max(abs(do[k]), 1e-12), k


def test_config0_static_start_100_steps():
    """The CPU-runnable reference case (64^2 x 65, eta contrast 5) from the
    seeded static state: 100 steps on both sides."""
    p = convection_params(64, 64, 65, eta_contrast=5.0)
    g, o = P3D(p), O.Oracle(p)
    g.start()
    o.start()
    assert g.step(100) == 0
    assert o.step(100) == 0
    _cmp(g, o, ["r", "t", "u", "v", "w", "pol", "tor", "bx", "by", "bz"], 1e-8)


def test_f_zero_skips_magnetics():
    """F=0 (Q=0): no magnetic evolution (src/main.F90:355-376); the seeded
    B is not solenoidal, so both sides stop with the div B check (-12)."""
    g, o, p = _setup(CASES[0], f=0.0)
    assert g.step(12) == o.step(12) == -12
    g, o, p = _setup(CASES[0], f=0.0, diag_cadence=0)
    assert g.step(12) == 0 and o.step(12) == 0
    _cmp(g, o, ["r", "t", "u", "v", "w"], 1e-9)
    assert np.array_equal(g.get("poldot2"), np.zeros_like(g.get("poldot2")))


def _near_tie_state(p, which, seed=3):
    """A state whose CFL (or density) extremum sits among values that agree
    to 1e-9: FP32 estimates cannot tell the points apart, so calcdt must
    evaluate them all in FP64."""
    rng = np.random.default_rng(seed)
    shape = (p.nz, p.ny, p.nx)
    n = p.nx * p.ny * p.nz
    s = smooth_state(p, seed=seed)
    s["bx"] = np.full(shape, 0.3); s["by"] = np.full(shape, 0.2); s["bz"] = np.full(shape, 1.0)
    s["t"] = np.full(shape, 2.0)
    s["r"] = np.full(shape, 1.5)
    jitter = 1.0 + 0.5e-9 * rng.random(shape)
    peak = np.unravel_index(int(rng.integers(n)), shape)
    if which == "xx":
        s["u"] = 1000.0 * jitter; s["v"] = np.zeros(shape); s["w"] = np.zeros(shape)
        s["u"][peak] = 1000.0 * (1.0 + 1e-9)
    elif which == "xz":
        s["u"] = np.zeros(shape); s["v"] = np.zeros(shape); s["w"] = 1000.0 * jitter
        s["w"][peak] = 1000.0 * (1.0 + 1e-9)
    else:
        # no flow, no field, cold: the viscous / diffusive limits times the
        # minimum density set dt
        s["u"] = np.zeros(shape); s["v"] = np.zeros(shape); s["w"] = np.zeros(shape)
        s["bx"] = np.zeros(shape); s["by"] = np.zeros(shape); s["bz"] = np.zeros(shape)
        s["t"] = np.full(shape, 1e-8)
        s["r"] = 1.5 * (2.0 - jitter)
        s["r"][peak] = 1.5 * (1.0 - 1e-9)
    return s


@pytest.mark.parametrize("which", ["xx", "xz", "rho"])
def test_calcdt_near_ties(which):
    """The FP32 pre-pass of calcdt only selects points; the extrema stay the
    FP64 ones (tolerance 1e-14: a wrong pick would be off by ~5e-10)."""
    # 64 x 48 x 33 = 101376 points: 12 full chunks of 8192 and a partial one
    p = convection_params(64, 48, 33, eta_contrast=1.0)
    g, o = P3D(p), O.Oracle(p)
    s = _near_tie_state(p, which)
    for n, a in s.items():
        g.set(n, a)
        o.set(n, a)
    dg, do = g.calcdt(), o.calcdt()
    assert abs(dg - do) <= 1e-14 * do, (dg, do)


@pytest.mark.parametrize("pos", [0, 8191, 8192, 64 * 48 * 33 - 1])
def test_calcdt_spike_at_chunk_edges(pos):
    """One fast point at a chunk boundary of the pre-pass, in a smooth state."""
    p = convection_params(64, 48, 33, eta_contrast=1.0)
    g, o = P3D(p), O.Oracle(p)
    s = smooth_state(p, seed=5)
    shape = s["u"].shape
    idx = np.unravel_index(pos, shape)
    s["u"] = s["u"].copy()
    s["u"][idx] = 50.0
    s["r"] = s["r"].copy()
    s["r"][np.unravel_index((pos + 1) % s["r"].size, shape)] = 0.06
    for n, a in s.items():
        g.set(n, a)
        o.set(n, a)
    dg, do = g.calcdt(), o.calcdt()
    assert abs(dg - do) <= 1e-14 * do, (dg, do)
