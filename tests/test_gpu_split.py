"""The FP32-bulk / FP64-background form against the FP64 oracle.

Single RHS evaluations agree with the FP64 oracle to FP32 accuracy relative
to each array's scale (tolerance 2e-5).  Over 100 steps the per-field
relative L2 error stays below 1e-4, and the top Nusselt number, the kinetic
energy and the magnetic energy of the field perturbation track the FP64
oracle within 1 % (the target stated for the split form), sampled along the
run.  (With the fixed-flux bottom the reference's bottom Nusselt number is
identically one; the uniform seed field dominates the total magnetic energy.)
"""
import numpy as np
import pytest

from oracle import oracle as O
from fug30v0kxc_gb300.params import VEC_PREC_SPLIT, convection_params
from fug30v0kxc_gb300.solver import P3D
from tests.helpers import perturbation_menergy, rel_err, smooth_state, top_nusselt

pytestmark = pytest.mark.gpu


def _pair(nx, ny, nz, eta, seed=0, q=100.0, **kw):
    p = convection_params(nx, ny, nz, q=q, eta_contrast=eta, precision=VEC_PREC_SPLIT)
    for k, v in kw.items():
        setattr(p, k, v)
    p.ndu06 = 10
    g, o = P3D(p), O.Oracle(p)
    s = smooth_state(p, seed=seed)
    for n, a in s.items():
        g.set(n, a)
        o.set(n, a)
    o.calcdt(); g.calcdt()
    o.mag_init(); g.mag_init()
    return g, o, p


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


@pytest.mark.parametrize("eta,grid", [(1.0, (64, 64, 33)), (20.0, (64, 64, 33)), (20.0, (192, 96, 17))])
def test_split_rhs(eta, grid):
    g, o, p = _pair(*grid, eta)
    g.hydro_deriv(); o.hydro_deriv()
    for n in ("rdot3", "tdot3", "udot3", "vdot3", "wdot3"):
        e = rel_err(g.get(n), o.get(n))
        assert e < 2e-5, (n, e)
    g.mag_deriv(); o.mag_deriv()
    for n in ("poldot3", "tordot3"):
        e = rel_err(g.get(n), o.get(n))
        assert e < 2e-5, (n, e)
    g.bandj(); o.bandj()
    for n in ("bx", "by", "jsq"):
        e = rel_err(g.get(n), o.get(n))
        assert e < 2e-5, (n, e)
    bz_g, bz_o = g.get("bz") - o.bzbar, o.get("bz") - o.bzbar
    assert rel_err(bz_g, bz_o) < 2e-5


def test_split_rhs_without_magnetic_field():
    """Q = 0: the split kernels leave out B, J^2 and the Lorentz fluxes (zero
    for f = 0); hydro_deriv still matches the FP64 oracle, which keeps
    them, at FP32 accuracy."""
    g, o, p = _pair(64, 64, 33, 5.0, q=0.0)
    assert p.f == 0.0
    g.hydro_deriv(); o.hydro_deriv()
    for n in ("rdot3", "tdot3", "udot3", "vdot3", "wdot3"):
        e = rel_err(g.get(n), o.get(n))
        assert e < 2e-5, (n, e)


def test_split_30_steps_without_magnetic_field_vs_fp64_oracle():
    """Q = 0, seeded static start, 30 steps (three calcdt and dealias
    steps): relative L2 of r, t (deviations from the polytrope), u, v, w
    against the FP64 oracle below 1e-4."""
    p = convection_params(64, 64, 33, q=0.0, eta_contrast=5.0, precision=VEC_PREC_SPLIT)
    p.ndu06 = 10
    g, o = P3D(p), O.Oracle(p)
    g.start(); o.start()
    assert g.step(30) == 0 and o.step(30) == 0
    z = np.arange(p.nz) / (p.nz - 1)
    t0 = (1.0 + p.theta * z)[:, None, None]
    for n in ("r", "t", "u", "v", "w"):
        a, b = g.get(n), o.get(n)
        if n in ("r", "t"):
            bgd = t0 ** p.cm if n == "r" else t0
            a, b = a - bgd, b - bgd
        e = rel_l2(a, b)
        assert e < 1e-4, (n, e)


def test_split_100_steps_vs_fp64_oracle():
    """64^2 x 65, eta contrast 5, seeded static start (the CPU-runnable case)."""
    p = convection_params(64, 64, 65, eta_contrast=5.0, precision=VEC_PREC_SPLIT)
    p.ndu06 = 10
    g, o = P3D(p), O.Oracle(p)
    g.start(); o.start()
    nus, kes, mes = [], [], []
    for _ in range(10):
        assert g.step(10) == 0 and o.step(10) == 0
        dg, do = g.last_diag(), o.last_diag()
        nus.append((g.top_nusselt(), top_nusselt(p, o.get("t"))))
        kes.append((dg["kenergy"], do["kenergy"]))
        mes.append((perturbation_menergy(p, g.get("bx"), g.get("by"), g.get("bz"), g.bzbar),
                    perturbation_menergy(p, o.get("bx"), o.get("by"), o.get("bz"), o.bzbar)))
    errs = {}
    for n in ("r", "t", "u", "v", "w", "pol", "tor"):
        a, b = g.get(n), o.get(n)
        if n in ("r", "t"):
            # relative L2 of the deviation from the static polytrope
            z = np.arange(p.nz) / (p.nz - 1)
            t0 = (1.0 + p.theta * z)[:, None, None]
            bgd = t0 ** p.cm if n == "r" else t0
            a, b = a - bgd, b - bgd
        errs[n] = rel_l2(a, b)
    print("split vs FP64 oracle, relative L2 after 100 steps:", errs)
    for n, e in errs.items():
        if n == "tor":
            # From rest the toroidal potential (~1e-9 here) is driven by the
            # vertical vorticity, a difference of O(1e-3) FP32 derivatives of
            # u and v: FP32 resolves it to ~1e-11 absolute, i.e. ~1e-2 of tor.
            assert e < 5e-2, (n, e, errs)
        else:
            assert e < 1e-4, (n, e, errs)
    for name, series in (("nusselt_top", nus), ("kenergy", kes), ("menergy_pert", mes)):
        a = np.mean([x for x, _ in series])
        b = np.mean([y for _, y in series])
        assert abs(a - b) <= 0.01 * abs(b), (name, a, b)


@pytest.mark.parametrize("grid", [(64, 64, 33), (96, 48, 17)])
@pytest.mark.parametrize("var,values,tol", [("VEC_HW_CVT", ("1", "0"), 0.0), ("VEC_VEC4", ("0", "1"), 1e-6),
                                            ("VEC_ZPENCIL", ("0", "1"), 1e-6), ("VEC_ZPENCIL4", ("0", "1"), 1e-6),
                                            ("VEC_SERIAL_MAG", ("1", "0"), 0.0), ("VEC_PDL", ("1", "0"), 0.0),
                                            ("VEC_CT_WARP", ("1", "0"), 0.0)])
def test_split_variants_agree(grid, var, values, tol, monkeypatch):
    """Two implementations of the same arithmetic after twelve steps (Euler,
    AB2, AB3, a dealias step and a calcdt at step 10).

    * VEC_HW_CVT: the AB3 update's float/double conversions on the integer
      pipe against the hardware conversions: bit-identical states.
    * VEC_VEC4: the four-point vector forms of the pointwise kernels against
      the one-point forms.  The compiler contracts multiply-adds within one
      expression, not across the vector type's operator functions, so
      single roundings differ; tolerance 1e-6 relative L2 per field.
    * VEC_ZPENCIL: hydro passes 2 and 4 with their z-stencil planes staged
      through shared-memory rings by bulk copies, against the per-plane
      forms that read them from global memory: the same formulas on the
      same values, but the kernels are compiled separately and the compiler
      may fuse different multiply-adds; tolerance 1e-6 relative L2 per
      field.  VEC_ZPENCIL4: the same for pass 4 alone.
    * VEC_SERIAL_MAG: the magnetic branch after the hydro one (E = u x B
      from pass 2, its transforms in the second-level line launches) against
      the branch on a second stream beside hydro (its own emf kernel and
      transforms): bit-identical states.
    * VEC_PDL, VEC_CT_WARP: programmatic dependent launches against ordinary
      ones, warp barriers in the x line tiles against CTA-wide ones; only
      the synchronisation differs, so the states are bit-identical (a
      missing wait would show as a difference).
    """
    states = []
    for val in values:
        monkeypatch.setenv(var, val)
        p = convection_params(*grid, eta_contrast=20.0, precision=VEC_PREC_SPLIT)
        p.ndu06 = 1000
        g = P3D(p)
        s = smooth_state(p, seed=4)
        for n, a in s.items():
            g.set(n, a)
        g.calcdt()
        g.mag_init()
        assert g.step(12) == 0
        states.append({n: g.get(n) for n in ("r", "t", "u", "v", "w", "pol", "tor", "bx", "by", "bz")})
        g.close()
    for n in states[0]:
        if tol == 0.0:
            assert np.array_equal(states[0][n], states[1][n]), n
        else:
            e = rel_l2(states[1][n], states[0][n])
            assert e <= tol, (n, e)


@pytest.mark.parametrize("var", ["VEC_ZPENCIL", "VEC_ZPENCIL4"])
@pytest.mark.parametrize("grid,q", [((64, 64, 33), 100.0), ((96, 48, 17), 100.0), ((128, 32, 40), 100.0),
                                    ((64, 64, 33), 0.0)])
def test_zpencil_passes_match_per_plane_form(grid, q, var, monkeypatch):
    """One hydro_deriv with passes 2 and 4 (VEC_ZPENCIL) or pass 4 alone
    (VEC_ZPENCIL4) fed by the shared-memory z rings against the per-plane
    forms, every RHS at every plane (the wall rows read planes 0..5 and
    nz-6..nz-1; several z chunks per column; Q = 0 leaves g and h out of
    pass 4's ring): largest difference below 1e-6 of the array's largest
    value (single roundings only)."""
    out = []
    for val in ("0", "1"):
        monkeypatch.setenv(var, val)
        p = convection_params(*grid, q=q, eta_contrast=20.0, precision=VEC_PREC_SPLIT)
        g = P3D(p)
        for n, a in smooth_state(p, seed=9).items():
            g.set(n, a)
        g.mag_init()
        g.hydro_deriv()
        out.append({n: g.get(n) for n in ("rdot3", "tdot3", "udot3", "vdot3", "wdot3")})
        g.close()
    for n in out[0]:
        e = rel_err(out[1][n], out[0][n])
        assert e < 1e-6, (n, e)
        # per plane: no row of the ring form is off
        for k in range(grid[2]):
            scale = max(np.abs(out[0][n]).max(), 1e-30)
            assert np.abs(out[1][n][k] - out[0][n][k]).max() / scale < 1e-6, (n, k)
