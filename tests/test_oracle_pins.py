"""Pins of the CPU oracle (the parity checker) against independent truths.

* FFTW-2 rfftw semantics (src/fft.F90:125-136): checked against numpy's
  FFT, an independent implementation of the same DFT.
* The reference's own derivative test, src/test_dbydxy.F90:118-332:
  analytic cos/sin fields for every wavenumber 0..n/2, d1bydx/d2bydx/
  dealias and the y variants; the reference's stated outcome (:4-5) is
  ~0 error except for the top third of modes, which dealias removes.
* z stencils (src/dbydz.F90:366-1558): interior rows exact for quartics,
  boundary rows exact for cubics, with the documented flag semantics.
* The physics, against known answers built from first principles on states
  where the stencils are exact:
  - the AB3 update's polynomial exactness;
  - the boundary conditions, through the d1bydz wall rows;
  - the static polytrope as a discrete equilibrium, and the convergence
    order of its residual;
  - each term of hydro_deriv and mag_deriv on a shear flow, a field, a
    temperature profile, and horizontal and vertical advection;
  - bandj's field construction and its zero divergence, and mag_init as
    its inverse;
  - magdealias as the 2/3 rule;
  - the diagnostics;
  - the whole step loop, which keeps the conductive polytrope fixed and
    commutes with horizontal shifts and reflections.
"""
import numpy as np
import pytest

from oracle import oracle as O
from fug30v0kxc_gb300.params import default_params


@pytest.mark.parametrize("n", [4, 6, 8, 30, 60, 64, 96, 192, 256, 250])
def test_r2hc_matches_numpy(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n)
    h = O.r2hc(x)
    X = np.fft.fft(x)
    ref = np.zeros(n)
    ref[: n // 2 + 1] = X[: n // 2 + 1].real
    for k in range(1, (n + 1) // 2):
        ref[n - k] = X[k].imag
    assert np.abs(h - ref).max() < 1e-13 * max(1.0, np.abs(ref).max())
    # unnormalised backward transform: hc2r(r2hc(x)) = n x
    assert np.abs(O.hc2r(h) / n - x).max() < 1e-14 * n


def _oracle(nx, ny, nz):
    p = default_params()
    p.nx, p.ny, p.nz = nx, ny, nz
    return O.Oracle(p), p


@pytest.mark.parametrize("direction", ["x", "y"])
@pytest.mark.parametrize("func", ["cos", "sin"])
def test_dbydxy_kat(direction, func):
    nx, ny, nz = 30, 24, 6
    o, p = _oracle(nx, ny, nz)
    n = nx if direction == "x" else ny
    L = p.xmax if direction == "x" else p.ymax
    d = L / n
    s = np.arange(n) * d
    icut = (n // 2) // 3
    k3 = np.arange(1, nz + 1)[:, None, None].astype(float)
    for iw in range(0, n // 2 + 1):
        om = iw * 2 * np.pi / L
        if func == "cos":
            g, g1, g2 = np.cos(om * s), -om * np.sin(om * s), -om * om * np.cos(om * s)
        else:
            g, g1, g2 = np.sin(om * s), om * np.cos(om * s), -om * om * np.sin(om * s)
        if direction == "x":
            f = k3 * g[None, None, :] * np.ones((nz, ny, nx))
            e1, e2 = k3 * g1[None, None, :], k3 * g2[None, None, :]
            d1 = o.d1bydx(f)
            a, b = o.d2bydx(f)
        else:
            f = k3 * g[None, :, None] * np.ones((nz, ny, nx))
            e1, e2 = k3 * g1[None, :, None], k3 * g2[None, :, None]
            d1 = o.d1bydy(f)
            a, b = o.d2bydy(f)
        dz = o.dealias(f)
        scale = nz * max(1.0, om * om)
        if iw < n // 2:
            assert np.abs(d1 - e1).max() < 1e-12 * scale, iw
            assert np.abs(a - e1).max() < 1e-12 * scale, iw
            assert np.abs(b - e2).max() < 1e-11 * scale, iw
        else:
            # Nyquist: d1 drops it (:292-302), d2 keeps it (:442-454)
            assert np.abs(d1).max() < 1e-12 * scale
            assert np.abs(b - e2).max() < 1e-11 * scale
        if iw < n // 2 - icut:
            assert np.abs(dz - f).max() < 1e-12 * nz, iw
        else:
            assert np.abs(dz).max() < 1e-12 * nz, iw


def test_forward_inverse_2d_roundtrip():
    o, p = _oracle(30, 20, 6)
    rng = np.random.default_rng(1)
    f = rng.standard_normal((6, 20, 30))
    F = o.forwardfft(f)
    # 2-D halfcomplex x halfcomplex = rfftw along x then along y
    ref = np.apply_along_axis(O.r2hc, 2, f)
    ref = np.apply_along_axis(O.r2hc, 1, ref)
    assert np.abs(F - ref).max() < 1e-12 * np.abs(ref).max()
    assert np.abs(o.inversefft(F) - f).max() < 1e-13


def _poly(nz, deg, rng):
    z = np.arange(nz) / (nz - 1)
    c = rng.standard_normal(deg + 1)
    f = sum(c[i] * z ** i for i in range(deg + 1))
    f1 = sum(i * c[i] * z ** (i - 1) for i in range(1, deg + 1))
    f2 = sum(i * (i - 1) * c[i] * z ** (i - 2) for i in range(2, deg + 1))
    return f, f1, f2


def test_z_stencils_polynomial_exactness():
    nz = 17
    o, p = _oracle(4, 4, nz)
    rng = np.random.default_rng(3)
    # interior rows: 4th order -> exact for quartics (d1 interior is exact
    # to degree 4, d2 interior to degree 5)
    f, f1, f2 = _poly(nz, 4, rng)
    F = np.broadcast_to(f[:, None, None], (nz, 4, 4)).copy()
    d1 = o.d1bydz(F, 5)[:, 0, 0]
    d2 = o.d2bydz(F, 3)[:, 0, 0]
    assert np.abs(d1[2:-2] - f1[2:-2]).max() < 1e-10
    assert np.abs(d2[2:-2] - f2[2:-2]).max() < 1e-8
    # boundary rows: third order -> exact for cubics (flag 5 one-sided)
    f, f1, f2 = _poly(nz, 3, rng)
    F = np.broadcast_to(f[:, None, None], (nz, 4, 4)).copy()
    d1 = o.d1bydz(F, 5)[:, 0, 0]
    assert np.abs(d1 - f1).max() < 1e-10
    d2 = o.d2bydz(F, 3)[:, 0, 0]
    assert np.abs(d2 - f2).max() < 1e-8
    # flag semantics: 0/2 zero the outer rows, flag 0 zeroes d2 at the walls
    assert np.all(o.d1bydz(F, 0)[[0, -1]] == 0.0)
    assert np.all(o.d1bydz(F, 2)[[0, -1]] == 0.0)
    assert np.all(o.d2bydz(F, 0)[[0, -1]] == 0.0)
    # flag 1 ("conserves mass"): top row = ho12*(14f1+36f2-18f3+4f4)
    h = (nz - 1) / 12.0
    top = o.d1bydz(F, 1)[0, 0, 0]
    assert abs(top - h * (14 * f[0] + 36 * f[1] - 18 * f[2] + 4 * f[3])) < 1e-12 * abs(top) + 1e-12
    # 1-D twins are the same stencils
    assert np.allclose(o.d1bydz1d(f, 5), d1, rtol=0, atol=1e-12)


def test_upwind_follows_sign_of_w():
    nz = 12
    o, p = _oracle(4, 4, nz)
    rng = np.random.default_rng(4)
    f = rng.standard_normal((nz, 4, 4))
    h = (nz - 1) / 12.0
    for wsign in (1.0, -1.0):
        o.set("w", np.full((nz, 4, 4), wsign))
        d = o.d1upbydz(f, 5)
        k = 6
        F = f[:, 0, 0]
        if wsign > 0:
            ref = h * (-F[k - 3] + 6 * F[k - 2] - 18 * F[k - 1] + 10 * F[k] + 3 * F[k + 1])
        else:
            ref = h * (F[k + 3] - 6 * F[k + 2] + 18 * F[k + 1] - 10 * F[k] - 3 * F[k - 1])
        assert abs(d[k, 0, 0] - ref) < 1e-12


def test_bad_flag_and_sizes():
    o, p = _oracle(8, 8, 8)
    f = np.zeros((8, 8, 8))
    with pytest.raises(O.OracleError):
        o.d1bydz(f, 3)
    with pytest.raises(O.OracleError):
        o.d2bydz(f, 5)
    for nx, ny, nz in ((7, 8, 8), (8, 9, 8), (8, 8, 5)):
        p2 = default_params()
        p2.nx, p2.ny, p2.nz = nx, ny, nz
        with pytest.raises(O.OracleError):
            O.Oracle(p2)


def test_ran0_sequence():
    """RANSET/ran0 (src/ranset.f90): first draws of layer 1, seed 1996+64."""
    p = default_params()
    p.nx, p.ny, p.nz = 4, 4, 6
    p.noise_amp = 0.5
    o = O.Oracle(p)
    o.static()
    t = o.get("t")
    # Park-Miller with the XOR mask: s0 = seed ^ MASK, s_{n+1} = 16807 s_n mod (2^31-1)
    M, A, MASK = 2147483647, 16807, 123459876
    s = (1996 + 64 * 1) ^ MASK
    vals = []
    for _ in range(16):
        s = (A * s) % M
        vals.append(2.0 * (s * (1.0 / M) - 0.5) * 0.5)
    assert np.array_equal(t[0].ravel(), np.array(vals) + 1.0)


STATE_DOTS = (("r", "rdot"), ("t", "tdot"), ("u", "udot"), ("v", "vdot"), ("w", "wdot"),
              ("pol", "poldot"), ("tor", "tordot"))


@pytest.mark.parametrize("start,order", [("euler", 0), ("ab2", 1), ("ab3", 2)])
def test_ab3_integrates_polynomials_exactly(start, order):
    """Variable-step Adams-Bashforth (src/main.F90:381-403) against exact integrals.

    The coefficients are the integrals over [t_n, t_n + dt] of the Lagrange
    basis through the RHS times t_n, t_n - dt1 and t_n - dt2 (dt2 = t_n -
    t_{n-2}). So one step of the full scheme integrates a right-hand side
    that is quadratic in time exactly, for any step sizes. The start-up
    steps are exact for linear (AB2, dt2 = 0) and constant (Euler) ones.
    Also pinned: the history shift (:448-461) and the dt1/dt2 and start-flag
    updates (:488-489).
    """
    nx, ny, nz = 8, 6, 6
    o, _ = _oracle(nx, ny, nz)
    rng = np.random.default_rng(11 + order)
    dt, dt1, dt2 = 0.0173, 0.0211, 0.0211 + 0.0128
    first, second = {"euler": (1, 0), "ab2": (0, 1), "ab3": (0, 0)}[start]
    s = o.scalars()
    s.dt, s.dt1, s.dt2, s.first, s.second = dt, dt1, dt2, first, second
    o.set_scalars(s)

    def poly(shape):
        c = [rng.uniform(-1.0, 1.0, shape) for _ in range(3)]
        for m in range(order + 1, 3):
            c[m] = np.zeros(shape)
        g = lambda t: c[0] + c[1] * t + c[2] * t * t                        # noqa: E731
        integral = c[0] * dt + c[1] * dt ** 2 / 2.0 + c[2] * dt ** 3 / 3.0   # over [0, dt]
        return g, integral

    # histories sampled at t_n = 0, -dt1, -dt2; slots the scheme does not use
    # hold unrelated values
    times = {3: 0.0, 2: -dt1 if order >= 1 else None, 1: -dt2 if order >= 2 else None}
    shape = (nz, ny, nx)
    expect, hist = {}, {}
    for name, dot in STATE_DOTS:
        y0 = rng.uniform(0.9, 1.1, shape)   # r stays above the 0.05 floor
        g, integral = poly(shape)
        o.set(name, y0)
        for slot, t in times.items():
            h = g(t) if t is not None else rng.uniform(-1.0, 1.0, shape)
            o.set(f"{dot}{slot}", h)
            hist[(dot, slot)] = h
        expect[name] = y0 + integral
    for name in ("bxbar", "bybar"):
        y0 = rng.uniform(-1.0, 1.0, nz)
        g, integral = poly(nz)
        o.set_mean(name, y0)
        for slot, t in times.items():
            h = g(t) if t is not None else rng.uniform(-1.0, 1.0, nz)
            o.set_mean(f"{name}dot{slot}", h)
            hist[(name + "dot", slot)] = h
        expect[name] = y0 + integral

    o.ab3_update()

    for name, dot in STATE_DOTS:
        np.testing.assert_allclose(o.get(name), expect[name], rtol=0, atol=1e-14, err_msg=name)
        # the shift: oldest <- middle <- newest
        assert np.array_equal(o.get(f"{dot}1"), hist[(dot, 2)])
        assert np.array_equal(o.get(f"{dot}2"), hist[(dot, 3)])
    for name in ("bxbar", "bybar"):
        np.testing.assert_allclose(o.get_mean(name), expect[name], rtol=0, atol=1e-14, err_msg=name)
        assert np.array_equal(o.get_mean(f"{name}dot1"), hist[(name + "dot", 2)])
        assert np.array_equal(o.get_mean(f"{name}dot2"), hist[(name + "dot", 3)])
    s = o.scalars()
    prev_dt1 = {"euler": 0.0, "ab2": dt1, "ab3": dt1}[start]
    assert (s.first, s.second) == {"euler": (0, 1), "ab2": (0, 0), "ab3": (0, 0)}[start]
    assert s.dt1 == dt and s.dt2 == dt + prev_dt1


@pytest.mark.parametrize("radbc,constflux", [(0, 0), (1, 1)])
def test_boundary_meets_its_conditions_through_the_stencils(radbc, constflux):
    """boundary (src/dbydz.F90:3686-4197) against the conditions it imposes,
    measured with the independently restated wall rows of d1bydz (flag 5,
    src/dbydz.F90:927 and :626: 2h(-11 f0 + 18 f1 - 9 f2 + 2 f3)):

    * stress-free walls: du/dz = dv/dz = 0, and w = 0;
    * bottom: T = 1, or with radbc the radiative condition dT/dz = theta T^4;
    * top: T = 1 + theta, or with constflux the flux condition dT/dz = theta.
    """
    nx, ny, nz = 6, 4, 9
    p = default_params()
    p.nx, p.ny, p.nz = nx, ny, nz
    p.radbc, p.constflux = radbc, constflux
    o = O.Oracle(p)
    rng = np.random.default_rng(3 + radbc)
    shape = (nz, ny, nx)
    for name in ("u", "v", "w"):
        o.set(name, rng.uniform(-1.0, 1.0, shape))
    zc = np.linspace(0.0, 1.0, nz)[:, None, None]
    o.set("t", 1.0 + p.theta * zc + 0.05 * rng.uniform(-1.0, 1.0, shape))   # near the polytrope
    o.boundary()
    tol = 1e-12
    for name in ("u", "v"):
        d = o.d1bydz(o.get(name), 5)
        assert np.abs(d[0]).max() < tol and np.abs(d[-1]).max() < tol, name
    w = o.get("w")
    assert not w[0].any() and not w[-1].any()
    t = o.get("t")
    dt = o.d1bydz(t, 5)
    if radbc:
        np.testing.assert_allclose(dt[0], p.theta * t[0] ** 4, rtol=1e-11, atol=0)
    else:
        assert np.all(t[0] == 1.0)
    if constflux:
        np.testing.assert_allclose(dt[-1], p.theta, rtol=1e-11, atol=0)
    else:
        assert np.all(t[-1] == 1.0 + p.theta)


@pytest.mark.parametrize("perfect", [0, 1])
def test_mag_boundary_meets_its_conditions_through_the_stencils(perfect):
    """mag_boundary (src/dbydz.F90:4205-4791) against the conditions it
    imposes, measured with the flag-5 wall rows of d1bydz and d1bydz1d:

    * vertical field (:4663-4780): tor = 0, bxbar = bybar = 0 and
      d(pol)/dz = 0 at both walls;
    * perfect conductor (:4407-4560): pol = 0 and d(tor)/dz = d(bxbar)/dz =
      d(bybar)/dz = 0 at both walls.
    """
    nx, ny, nz = 6, 4, 9
    p = default_params()
    p.nx, p.ny, p.nz = nx, ny, nz
    p.perfect = perfect
    o = O.Oracle(p)
    rng = np.random.default_rng(5 + perfect)
    shape = (nz, ny, nx)
    for name in ("pol", "tor"):
        o.set(name, rng.uniform(-1.0, 1.0, shape))
    for name in ("bxbar", "bybar"):
        o.set_mean(name, rng.uniform(-1.0, 1.0, nz))
    o.mag_boundary()
    tol = 1e-12
    pol, tor = o.get("pol"), o.get("tor")
    means = [o.get_mean(n) for n in ("bxbar", "bybar")]

    def walls_zero_slope(d):
        return np.abs(d[0]).max() < tol and np.abs(d[-1]).max() < tol

    if perfect:
        assert not pol[0].any() and not pol[-1].any()
        assert walls_zero_slope(o.d1bydz(tor, 5))
        for m in means:
            assert walls_zero_slope(o.d1bydz1d(m, 5))
    else:
        assert not tor[0].any() and not tor[-1].any()
        for m in means:
            assert m[0] == 0.0 and m[-1] == 0.0
        assert walls_zero_slope(o.d1bydz(pol, 5))


def _static_polytrope(nz, cm, nx=8, ny=8):
    p = default_params()
    p.nx, p.ny, p.nz = nx, ny, nz
    p.noise_amp, p.cm, p.kappa_uniform = 0.0, cm, 1
    o = O.Oracle(p)
    o.static()
    o.bandj()
    return o


def test_static_polytrope_is_a_discrete_equilibrium():
    """With polytropic index m = 1 the static state (src/initial.F90:25-86)
    has T = 1 + theta z, rho = T and p = rho T = T^2: polynomials of degree
    <= 2 in z, on which every z stencil is exact, with a uniform vertical
    field and uniform kappa. Hydrostatic balance (src/hydro_deriv.f90) and
    the induction equation (src/magnetic.f90:285-487) then hold exactly in
    discrete form: every right-hand side vanishes."""
    o = _static_polytrope(17, 1.0)
    o.hydro_deriv()
    o.mag_deriv()
    for d in ("rdot", "tdot", "udot", "vdot", "wdot", "poldot", "tordot"):
        assert np.abs(o.get(f"{d}3")).max() < 1e-12, d
    for m in ("bxbardot3", "bybardot3"):
        assert np.abs(o.get_mean(m)).max() < 1e-12, m


def test_hydrostatic_residual_converges_at_stencil_order():
    """For m = 1.5, p = T^2.5 is no polynomial, and the hydrostatic residual
    in dw/dt is the stencils' truncation error: fourth order at fixed
    interior heights (src/dbydz.F90:371) and third order on the rows next
    to the walls (:776, :1053)."""
    res = {}
    for nz in (33, 65, 129):
        o = _static_polytrope(nz, 1.5)
        o.hydro_deriv()
        w = o.get("wdot3")[:, 0, 0]
        res[nz] = (np.array([w[(nz - 1) // 4], w[(nz - 1) // 2], w[3 * (nz - 1) // 4]]), w[nz - 2])
    for a, b in ((33, 65), (65, 129)):
        interior = np.abs(res[a][0] / res[b][0])
        assert np.all((interior > 15.0) & (interior < 17.5)), (a, b, interior)
    wall = abs(res[65][1] / res[129][1])
    assert 7.0 < wall < 9.5, wall


@pytest.mark.parametrize("eta_contrast", [1.0, 20.0])
def test_induction_diffusion_known_answer(eta_contrast):
    """mag_deriv (src/magnetic.f90:285-487) with u = 0: the EMF vanishes and
    the induction equation is pure diffusion. For one horizontal Fourier mode
    with a cubic z profile f, every z stencil is exact, so with eta(z) =
    zeta ck (1 + (c - 1) z) (c = eta contrast; c = 1 is the reference):

        poldot = eta (-k^2 f + f'')
        tordot = eta (-k^2 f + f'') + eta' f'
        bxbardot = eta f'' + eta' f'   (the horizontal mean, k = 0)

    with k = 2 pi i / xmax or 2 pi j / ymax computed here, independently of
    the oracle's wavenumber tables; every other mode stays zero."""
    nx, ny, nz = 16, 12, 11
    p = default_params()
    p.nx, p.ny, p.nz = nx, ny, nz
    p.eta_contrast = eta_contrast
    o = O.Oracle(p)
    shape = (nz, ny, nx)
    for name in ("u", "v", "w", "bx", "by", "bz"):
        o.set(name, np.zeros(shape))
    z = np.linspace(0.0, 1.0, nz)
    f = 0.3 + 0.7 * z - 1.1 * z ** 2 + 0.9 * z ** 3
    f1 = 0.7 - 2.2 * z + 2.7 * z ** 2
    f2 = -2.2 + 5.4 * z
    i, j = 3, 2
    pol, tor = np.zeros(shape), np.zeros(shape)
    pol[:, 0, i] = f   # x mode i (real part of the halfcomplex pair), y mode 0
    tor[:, j, 0] = f   # y mode j, x mode 0
    o.set("pol", pol)
    o.set("tor", tor)
    o.set_mean("bxbar", f)
    o.set_mean("bybar", np.zeros(nz))
    o.bzbar = 0.0
    o.mag_deriv()
    zck = p.zeta * p.ck
    eta = zck * (1.0 + (eta_contrast - 1.0) * z)
    deta = zck * (eta_contrast - 1.0)
    kx, ky = 2 * np.pi * i / p.xmax, 2 * np.pi * j / p.ymax
    pd, td = o.get("poldot3"), o.get("tordot3")
    tol = 1e-13 * max(1.0, eta_contrast)
    np.testing.assert_allclose(pd[:, 0, i], eta * (-kx * kx * f + f2), rtol=0, atol=tol)
    np.testing.assert_allclose(td[:, j, 0], eta * (-ky * ky * f + f2) + deta * f1, rtol=0, atol=tol)
    pd[:, 0, i] = 0.0
    td[:, j, 0] = 0.0
    assert not pd.any() and not td.any()
    np.testing.assert_allclose(o.get_mean("bxbardot3"), eta * f2 + deta * f1, rtol=0, atol=tol)
    assert not o.get_mean("bybardot3").any()


def test_viscous_shear_flow_known_answer():
    """hydro_deriv (src/hydro_deriv.f90:5-505) on a plane shear flow u = U(z)
    (cubic), v = w = 0, uniform rho = T = 1, no field, no rotation: div u = 0
    and p is uniform, so with the nondimensional numbers sigma ck (viscosity)
    and sigma ck (gamma - 1) (viscous heating), and gravity theta (m + 1):

        udot = sigma ck U''                  (every row: the stencils are exact)
        tdot = sigma ck (gamma - 1) U'^2     (interior; 0 on the fixed-T walls)
        wdot = theta (m + 1)                 (interior; 0 on the walls)
        rdot = vdot = 0
    """
    nx, ny, nz = 8, 6, 11
    p = default_params()
    p.nx, p.ny, p.nz = nx, ny, nz
    p.kappa_uniform = 1
    o = O.Oracle(p)
    shape = (nz, ny, nx)
    z = np.linspace(0.0, 1.0, nz)[:, None, None]
    U = 0.2 + 0.5 * z - 0.8 * z ** 2 + 0.6 * z ** 3
    U1 = 0.5 - 1.6 * z + 1.8 * z ** 2
    U2 = -1.6 + 3.6 * z
    for name in ("v", "w", "bx", "by", "bz", "jsq", "pol", "tor"):
        o.set(name, np.zeros(shape))
    o.set("u", U * np.ones(shape))
    o.set("r", np.ones(shape))
    o.set("t", np.ones(shape))
    o.bzbar = 0.0
    o.hydro_deriv()
    sck = p.sigma * p.ck
    one = np.ones(shape)
    np.testing.assert_allclose(o.get("udot3"), sck * U2 * one, rtol=0, atol=1e-13)
    heat = sck * (p.gamma - 1.0) * U1 ** 2 * one
    heat[0] = heat[-1] = 0.0
    np.testing.assert_allclose(o.get("tdot3"), heat, rtol=0, atol=1e-13)
    grav = p.theta * (p.cm + 1.0) * one
    grav[0] = grav[-1] = 0.0
    np.testing.assert_allclose(o.get("wdot3"), grav, rtol=0, atol=1e-12)
    assert np.abs(o.get("rdot3")).max() == 0.0
    assert np.abs(o.get("vdot3")).max() < 1e-14


def test_lorentz_force_and_ohmic_heating_known_answer():
    """hydro_deriv's Lorentz force, the divergence of the Maxwell stress
    F (B_i B_j - |B|^2 delta_ij / 2) (src/hydro_deriv.f90:139-261), and
    ohmic heating, for B = (beta(z), 0, bz0) with beta quadratic, u = 0,
    rho = T = 1 and J = (0, beta', 0):

        udot = F bz0 beta'                       (every row)
        wdot = theta (m + 1) - F beta beta'      (interior rows, where the
               quartic beta^2 is differentiated exactly; 0 on the walls)
        tdot = F zeta ck (gamma - 1) |J|^2       (every row)
    """
    nx, ny, nz = 8, 6, 11
    p = default_params()
    p.nx, p.ny, p.nz = nx, ny, nz
    p.kappa_uniform = 1
    o = O.Oracle(p)
    shape = (nz, ny, nx)
    one = np.ones(shape)
    z = np.linspace(0.0, 1.0, nz)[:, None, None]
    beta = 0.4 - 0.3 * z + 0.5 * z ** 2
    beta1 = -0.3 + 1.0 * z
    bz0 = 0.7
    for name in ("u", "v", "w", "by", "pol", "tor"):
        o.set(name, np.zeros(shape))
    o.set("bx", beta * one)
    o.set("bz", bz0 * one)
    o.set("jsq", beta1 ** 2 * one)
    o.set("r", one)
    o.set("t", one)
    o.hydro_deriv()
    F = p.f
    np.testing.assert_allclose(o.get("udot3"), F * bz0 * beta1 * one, rtol=0, atol=1e-13)
    wd = o.get("wdot3")
    expect = (p.theta * (p.cm + 1.0) - F * beta * beta1) * one
    np.testing.assert_allclose(wd[2:-2], expect[2:-2], rtol=0, atol=1e-12)
    assert not wd[0].any() and not wd[-1].any()
    heat = p.f * p.zeta * p.ck * (p.gamma - 1.0) * beta1 ** 2 * one
    np.testing.assert_allclose(o.get("tdot3"), heat, rtol=0, atol=1e-13)
    assert np.abs(o.get("vdot3")).max() < 1e-14 and not o.get("rdot3").any()


def test_thermal_conduction_known_answer():
    """hydro_deriv's conduction with the reference's kappa(z) =
    (tanh(10 (z - 1/2)) + 1) / 2 (src/trans_params.f90:15-69), for a cubic
    T(z), rho = 1, u = 0, no field:

        tdot = gamma ck (kappa T'' + kappa' T')   (rows inside the walls)
        wdot = theta (m + 1) - T'                 (p = rho T; 0 on the walls)
    """
    nx, ny, nz = 8, 6, 11
    p = default_params()
    p.nx, p.ny, p.nz = nx, ny, nz
    p.kappa_uniform = 0
    o = O.Oracle(p)
    shape = (nz, ny, nx)
    one = np.ones(shape)
    z = np.linspace(0.0, 1.0, nz)[:, None, None]
    T = 1.0 + p.theta * z + 0.3 * z * (1.0 - z) + 0.2 * z ** 3
    T1 = p.theta + 0.3 - 0.6 * z + 0.6 * z ** 2
    T2 = -0.6 + 1.2 * z
    for name in ("u", "v", "w", "bx", "by", "bz", "jsq", "pol", "tor"):
        o.set(name, np.zeros(shape))
    o.set("r", one)
    o.set("t", T * one)
    o.hydro_deriv()
    kappa = 0.5 * (np.tanh(10.0 * (z - 0.5)) + 1.0)
    dkappa = 5.0 / np.cosh(10.0 * (z - 0.5)) ** 2
    cond = p.gamma * p.ck * (kappa * T2 + dkappa * T1) * one
    np.testing.assert_allclose(o.get("tdot3")[1:-1], cond[1:-1], rtol=0, atol=1e-12)
    wd = o.get("wdot3")
    np.testing.assert_allclose(wd[1:-1], ((p.theta * (p.cm + 1.0) - T1) * one)[1:-1], rtol=0, atol=1e-12)
    assert not wd[0].any() and not wd[-1].any()
    assert not o.get("udot3").any() and not o.get("rdot3").any()


def test_horizontal_advection_and_pressure_known_answer():
    """hydro_deriv with a horizontal density wave rho = 1 + a cos(kx) +
    b sin(ly) carried by a uniform flow (U0, V0, 0) at uniform T = 1. The
    spectral x and y derivatives are exact for resolved modes, with k and l
    computed here, and div u = 0:

        rdot = -(U0 rho_x + V0 rho_y)
        udot = -rho_x / rho,  vdot = -rho_y / rho   (p = rho T)
        tdot = 0,  wdot = theta (m + 1) inside the walls, 0 on them
    """
    nx, ny, nz = 16, 12, 9
    p = default_params()
    p.nx, p.ny, p.nz = nx, ny, nz
    p.kappa_uniform = 1
    o = O.Oracle(p)
    shape = (nz, ny, nx)
    one = np.ones(shape)
    x = (np.arange(nx) * p.xmax / nx)[None, None, :]
    y = (np.arange(ny) * p.ymax / ny)[None, :, None]
    k, l, a, b = 2 * np.pi * 3 / p.xmax, 2 * np.pi * 2 / p.ymax, 0.2, 0.1
    rho = (1.0 + a * np.cos(k * x) + b * np.sin(l * y)) * one
    rx = -a * k * np.sin(k * x) * one
    ry = b * l * np.cos(l * y) * one
    U0, V0 = 0.3, -0.2
    for name in ("w", "bx", "by", "bz", "jsq", "pol", "tor"):
        o.set(name, np.zeros(shape))
    o.set("u", U0 * one)
    o.set("v", V0 * one)
    o.set("r", rho)
    o.set("t", one)
    o.hydro_deriv()
    np.testing.assert_allclose(o.get("rdot3"), -U0 * rx - V0 * ry, rtol=0, atol=1e-13)
    np.testing.assert_allclose(o.get("udot3"), -rx / rho, rtol=0, atol=1e-13)
    np.testing.assert_allclose(o.get("vdot3"), -ry / rho, rtol=0, atol=1e-13)
    assert np.abs(o.get("tdot3")).max() < 1e-13
    wd = o.get("wdot3")
    np.testing.assert_allclose(wd[1:-1], p.theta * (p.cm + 1.0), rtol=0, atol=1e-12)
    assert not wd[0].any() and not wd[-1].any()


@pytest.mark.parametrize("W0", [0.4, -0.4])
def test_vertical_upwind_advection_known_answer(W0):
    """hydro_deriv with a uniform vertical flow W0 through a cubic density
    profile at T = 1 (div u = 0). The upwind z stencils (src/dbydz.F90:485,
    :532, :579; the side follows the sign of w) are exact for cubics:

        rdot = -W0 rho'              (every row inside the walls)
        wdot = -rho'/rho + theta (m + 1)
        tdot = 0

    The w equation is checked away from the walls. Near them its viscous
    term differentiates w with flag 1, which assumes w = 0 on the wall, and
    a uniform W0 does not meet that.
    """
    nx, ny, nz = 8, 6, 11
    p = default_params()
    p.nx, p.ny, p.nz = nx, ny, nz
    p.kappa_uniform = 1
    o = O.Oracle(p)
    shape = (nz, ny, nx)
    one = np.ones(shape)
    z = np.linspace(0.0, 1.0, nz)[:, None, None]
    rho = 1.0 + 0.5 * z - 0.3 * z ** 2 + 0.4 * z ** 3
    rho1 = 0.5 - 0.6 * z + 1.2 * z ** 2
    for name in ("u", "v", "bx", "by", "bz", "jsq", "pol", "tor"):
        o.set(name, np.zeros(shape))
    o.set("w", W0 * one)
    o.set("r", rho * one)
    o.set("t", one)
    o.hydro_deriv()
    np.testing.assert_allclose(o.get("rdot3")[1:-1], (-W0 * rho1 * one)[1:-1], rtol=0, atol=1e-13)
    wexp = (-rho1 / rho + p.theta * (p.cm + 1.0)) * one
    np.testing.assert_allclose(o.get("wdot3")[3:-3], wexp[3:-3], rtol=0, atol=1e-12)
    assert np.abs(o.get("tdot3")[1:-1]).max() < 1e-13


@pytest.mark.parametrize("cm,kappa_uniform", [(1.0, 1), (1.5, 1), (1.0, 0)])
def test_diagnostics_known_answers(cm, kappa_uniform):
    """diag (src/utils.F90:22-371, src/dbydz.F90:4796-4925) on states with
    known values:

    * the conductive static polytrope has Nusselt number 1 (the flux ratio
      it is normalised by), no kinetic energy, T in [1, 1 + theta] and rho
      in [1, (1 + theta)^m];
    * a uniform flow (U0, V0, 0) at rho = 1 has kinetic energy
      (U0^2 + V0^2) / 2 integrated over the xmax x ymax x 1 box, and
      horizontal means U0, V0.
    """
    p = default_params()
    p.nx, p.ny, p.nz = 8, 8, 33
    p.noise_amp, p.cm, p.kappa_uniform = 0.0, cm, kappa_uniform
    o = O.Oracle(p)
    o.static()
    o.bandj()
    st, d = o.diag()
    assert st == 0
    assert abs(d["nusselt"] - 1.0) < 1e-12 and d["kenergy"] == 0.0
    assert d["tmin"] == 1.0 and abs(d["tmax"] - (1.0 + p.theta)) < 1e-12
    assert d["rmin"] == 1.0 and abs(d["rmax"] - (1.0 + p.theta) ** cm) < 1e-12 * (1.0 + p.theta) ** cm
    shape = (p.nz, p.ny, p.nx)
    U0, V0 = 0.3, -0.4
    o.set("r", np.ones(shape))
    o.set("u", U0 * np.ones(shape))
    o.set("v", V0 * np.ones(shape))
    st, d = o.diag()
    assert abs(d["kenergy"] - 0.5 * (U0 ** 2 + V0 ** 2) * p.xmax * p.ymax) < 1e-13
    assert abs(d["ubar"] - U0) < 1e-14 and abs(d["vbar"] - V0) < 1e-14


def test_bandj_field_is_solenoidal():
    """bandj (src/magnetic.f90:492-664) builds B from the poloidal and
    toroidal potentials and the horizontal means, so div B = 0 by
    construction. Discretely the z stencil (per column) commutes with the
    spectral x and y derivatives (per plane). The diagnostics' div B
    (src/utils.F90, d1bydx + d1bydy + d1bydz) then vanishes to rounding for
    random potentials without Nyquist content. The first-derivative
    operator drops the Nyquist mode and the second-derivative one keeps it;
    the 2/3 dealiasing of the magnetic fields removes it in a run.
    """
    nx, ny, nz = 16, 12, 17
    p = default_params()
    p.nx, p.ny, p.nz = nx, ny, nz
    o = O.Oracle(p)
    rng = np.random.default_rng(1)
    shape = (nz, ny, nx)
    for name in ("pol", "tor"):
        a = rng.standard_normal(shape)
        a[:, :, nx // 2] = 0.0
        a[:, ny // 2, :] = 0.0
        o.set(name, a)
    o.set_mean("bxbar", rng.standard_normal(nz))
    o.set_mean("bybar", rng.standard_normal(nz))
    for name in ("u", "v", "w"):
        o.set(name, np.zeros(shape))
    o.set("r", np.ones(shape))
    o.set("t", np.ones(shape))
    o.bandj()
    st, d = o.diag()
    assert st == 0
    bmax = max(np.abs(o.get(n)).max() for n in ("bx", "by", "bz"))
    assert bmax > 10.0
    assert max(abs(d["divbmax"]), abs(d["divbmin"])) < 1e-13 * bmax


def test_bandj_single_mode_known_answer():
    """bandj (src/magnetic.f90:492-664): B = curl curl (pol z) + curl (tor z)
    + means, i.e. bx = d2pol/dxdz + dtor/dy, by = d2pol/dydz - dtor/dx,
    bz = -lap_h pol. For one horizontal mode with a cubic z profile, the
    real-space potential is A(z) cos(kx) (its spectral inverse), and k is
    computed independently of the oracle's tables."""
    nx, ny, nz = 16, 12, 11
    p = default_params()
    p.nx, p.ny, p.nz = nx, ny, nz
    o = O.Oracle(p)
    shape = (nz, ny, nx)
    zc = np.linspace(0.0, 1.0, nz)
    P = 0.3 + 0.7 * zc - 1.1 * zc ** 2 + 0.9 * zc ** 3
    x = (np.arange(nx) * p.xmax / nx)[None, None, :]
    y = (np.arange(ny) * p.ymax / ny)[None, :, None]
    i, j = 3, 2
    k, l = 2 * np.pi * i / p.xmax, 2 * np.pi * j / p.ymax
    o.set_mean("bxbar", np.zeros(nz))
    o.set_mean("bybar", np.zeros(nz))
    o.bzbar = 0.0
    zero = np.zeros(shape)

    def run(pol, tor):
        o.set("pol", pol)
        o.set("tor", tor)
        o.bandj()
        return o.get("bx"), o.get("by"), o.get("bz")

    def mode(jj, ii):
        a = np.zeros(shape)
        a[:, jj, ii] = P
        real = o.inversefft(a)
        return real, real[:, 0:1, 0:1]   # A(z) at x = y = 0

    tol = 1e-15
    # poloidal, x mode i: pol = A cos(kx)
    pol = np.zeros(shape)
    pol[:, 0, i] = P
    pr, A = mode(0, i)
    assert np.abs(pr - A * np.cos(k * x)).max() < tol
    dA = o.d1bydz(A * np.ones(shape), 5)[:, 0:1, 0:1]   # A is cubic: exact
    bx, by, bz = run(pol, zero)
    np.testing.assert_allclose(bz, k * k * pr, rtol=0, atol=tol)
    np.testing.assert_allclose(bx, -k * dA * np.sin(k * x) * np.ones(shape), rtol=0, atol=10 * tol)
    assert not by.any()
    # toroidal, y mode j: tor = A cos(ly) gives bx = dtor/dy, by = bz = 0
    tr, A = mode(j, 0)
    tor = np.zeros(shape)
    tor[:, j, 0] = P
    bx, by, bz = run(zero, tor)
    np.testing.assert_allclose(bx, -l * A * np.sin(l * y) * np.ones(shape), rtol=0, atol=tol)
    assert not by.any() and not bz.any()
    # toroidal, x mode i: by = -dtor/dx
    tr, A = mode(0, i)
    tor = np.zeros(shape)
    tor[:, 0, i] = P
    bx, by, bz = run(zero, tor)
    np.testing.assert_allclose(by, k * A * np.sin(k * x) * np.ones(shape), rtol=0, atol=tol)
    assert not bx.any() and not bz.any()


@pytest.mark.parametrize("nx,ny", [(30, 24), (32, 26), (48, 36)])
def test_magdealias_is_the_two_thirds_rule(nx, ny):
    """magdealias (src/magnetic.f90:666-717) on the spectral potentials
    keeps exactly the modes with 3|kx| < nx and 3|ky| < ny: the 2/3 rule,
    under which the product of two kept modes aliases only onto removed
    ones. Checked two ways:

    * on random fields, against a numpy FFT low-pass with that mask;
    * dealiasing the grid product of two kept-band fields gives the
      truncated exact product, computed on a grid that holds it unaliased.
    """
    nz = 6
    o, _ = _oracle(nx, ny, nz)
    rng = np.random.default_rng(nx + ny)
    kx = np.abs(np.fft.fftfreq(nx, 1.0 / nx))[None, None, :]
    ky = np.abs(np.fft.fftfreq(ny, 1.0 / ny))[None, :, None]
    keep = (3 * kx < nx) & (3 * ky < ny)

    def oracle_dealias(f):
        o.set("pol", o.forwardfft(f))
        o.set("tor", np.zeros_like(f))
        o.magdealias()
        return o.inversefft(o.get("pol"))

    def lowpass(f):
        return np.fft.ifft2(np.fft.fft2(f, axes=(1, 2)) * keep, axes=(1, 2)).real

    f = rng.standard_normal((nz, ny, nx))
    assert np.abs(oracle_dealias(f) - lowpass(f)).max() < 1e-12
    # aliasing: a, b band-limited to the kept modes; their exact product has
    # modes up to twice as high, held without aliasing on a 2x finer grid
    a, b = lowpass(rng.standard_normal((nz, ny, nx))), lowpass(rng.standard_normal((nz, ny, nx)))

    def fine(g):   # exact trigonometric interpolation onto the 2x grid
        G = np.fft.fft2(g, axes=(1, 2))
        H = np.zeros((nz, 2 * ny, 2 * nx), complex)
        iy = np.fft.fftfreq(ny, 1.0 / ny).astype(int)
        ix = np.fft.fftfreq(nx, 1.0 / nx).astype(int)
        H[:, iy[:, None] % (2 * ny), ix[None, :] % (2 * nx)] = G
        return np.fft.ifft2(H, axes=(1, 2)).real * 4.0

    P = np.fft.fft2(fine(a) * fine(b), axes=(1, 2)) / 4.0
    iy = np.fft.fftfreq(ny, 1.0 / ny).astype(int)
    ix = np.fft.fftfreq(nx, 1.0 / nx).astype(int)
    exact_kept = np.fft.ifft2(P[:, iy[:, None] % (2 * ny), ix[None, :] % (2 * nx)] * keep, axes=(1, 2)).real
    assert np.abs(oracle_dealias(a * b) - exact_kept).max() < 1e-12


def test_mag_init_inverts_bandj():
    """mag_init (src/magnetic.f90:5-279) recovers the potentials from B:
    pol from bz = -lap_h pol, tor from the vertical current, and the means
    from the horizontal averages. bandj (src/magnetic.f90:492-664) builds B
    from them. Starting from random potentials inside the 2/3 band (mag_init
    truncates B's spectra) without a horizontal mean mode, bandj then
    mag_init returns them, the means, bzbar and |J|^2 to rounding. Wall
    planes are excluded, since mag_init ends with mag_boundary."""
    nx, ny, nz = 16, 12, 11
    o, _ = _oracle(nx, ny, nz)
    rng = np.random.default_rng(2)
    shape = (nz, ny, nx)
    ix = np.array([i if i <= nx // 2 else nx - i for i in range(nx)])
    iy = np.array([j if j <= ny // 2 else ny - j for j in range(ny)])

    def in_band(a):
        a = a.copy()
        a[:, :, 3 * ix >= nx] = 0.0
        a[:, 3 * iy >= ny, :] = 0.0
        a[:, 0, 0] = 0.0
        return a

    pol, tor = in_band(rng.standard_normal(shape)), in_band(rng.standard_normal(shape))
    bxbar, bybar, bzbar = rng.standard_normal(nz), rng.standard_normal(nz), 0.7
    o.set("pol", pol)
    o.set("tor", tor)
    o.set_mean("bxbar", bxbar)
    o.set_mean("bybar", bybar)
    o.bzbar = bzbar
    o.bandj()
    jsq = o.get("jsq")
    zero = np.zeros(shape)
    o.set("pol", zero)
    o.set("tor", zero)
    o.set_mean("bxbar", np.zeros(nz))
    o.set_mean("bybar", np.zeros(nz))
    o.bzbar = 0.0
    o.mag_init()
    tol = 1e-13
    assert np.abs(o.get("pol")[1:-1] - pol[1:-1]).max() < tol * np.abs(pol).max()
    assert np.abs(o.get("tor")[1:-1] - tor[1:-1]).max() < tol * np.abs(tor).max() * 10
    assert np.abs(o.get_mean("bxbar")[1:-1] - bxbar[1:-1]).max() < tol
    assert np.abs(o.get_mean("bybar")[1:-1] - bybar[1:-1]).max() < tol
    assert abs(o.bzbar - bzbar) < tol
    assert np.abs(o.get("jsq")[1:-1] - jsq[1:-1]).max() < tol * np.abs(jsq).max()


def test_global_averages_remove_mean_momentum():
    """GlobalAverages (src/utils.F90:22-139): ubar, vbar are the density-
    weighted means int(rho u) / int(rho), trapezoidal in z (half weight on
    the wall planes), and the diagnostics step subtracts them from u and v.
    Afterwards int(rho u) = int(rho v) = 0, so a second call reports zero."""
    nx, ny, nz = 8, 6, 9
    o, _ = _oracle(nx, ny, nz)
    rng = np.random.default_rng(8)
    shape = (nz, ny, nx)
    r = rng.uniform(0.5, 2.0, shape)
    u, v = rng.standard_normal(shape) + 0.3, rng.standard_normal(shape) - 0.2
    for name, a in (("r", r), ("u", u), ("v", v), ("w", rng.standard_normal(shape)),
                    ("t", np.ones(shape)), ("bx", np.zeros(shape)), ("by", np.zeros(shape)),
                    ("bz", np.zeros(shape))):
        o.set(name, a)
    wz = np.ones(nz)
    wz[0] = wz[-1] = 0.5
    mean = lambda a: np.sum(wz[:, None, None] * r * a) / np.sum(wz[:, None, None] * r)   # noqa: E731
    st, d = o.diag()
    assert abs(d["ubar"] - mean(u)) < 1e-14 and abs(d["vbar"] - mean(v)) < 1e-14
    np.testing.assert_allclose(o.get("u"), u - d["ubar"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(o.get("v"), v - d["vbar"], rtol=0, atol=1e-15)
    st, d = o.diag()
    assert abs(d["ubar"]) < 1e-15 and abs(d["vbar"]) < 1e-15


@pytest.mark.parametrize("perfect,radbc,constflux", [(0, 0, 0), (1, 0, 0), (0, 1, 1)])
def test_static_polytrope_is_a_fixed_point_of_the_step(perfect, radbc, constflux):
    """The whole step loop (src/main.F90:340-747: RHS, AB3, dealias, bandj,
    boundaries, diagnostics, calcdt) keeps the m = 1 conductive polytrope
    with a uniform field unchanged. Every RHS is zero, the boundary
    conditions hold for a linear T (radbc: T = 1 is the root of the
    radiative condition; constflux: the top flux is theta), and the uniform
    field is its own potential decomposition. Time advances by the step
    count times dt, across the 10-step dealias and calcdt cadence and the
    diagnostics every 5 steps."""
    p = default_params()
    p.nx, p.ny, p.nz = 8, 8, 17
    p.noise_amp, p.cm, p.kappa_uniform = 0.0, 1.0, 1
    p.perfect, p.radbc, p.constflux, p.ndu06 = perfect, radbc, constflux, 5
    o = O.Oracle(p)
    o.static()
    o.mag_init()
    dt = o.calcdt()
    s0 = o.state()
    assert o.step(25) == 0
    s1 = o.state()
    for name in s0:
        assert np.abs(s1[name] - s0[name]).max() < 1e-12, name
    sc = o.scalars()
    assert sc.iter == 25 and abs(sc.ttime - 25 * dt) < 1e-15


@pytest.mark.parametrize("sym", ["shift", "mirror_x", "mirror_y"])
def test_step_commutes_with_horizontal_symmetries(sym):
    """The whole step loop (hydrodynamic, F = 0, no rotation) commutes with
    the symmetries of the periodic horizontal domain: a shift by whole grid
    points, and the reflections x -> -x (u -> -u) and y -> -y (v -> -v).
    Spectral derivatives, per-column z stencils and pointwise terms all
    commute with them, so 12 steps from a noisy state agree to rounding."""
    fields = ("r", "t", "u", "v", "w")

    def act(name, a):
        if sym == "shift":
            return np.roll(a, (2, 3), axis=(1, 2))
        if sym == "mirror_x":
            b = np.roll(a[:, :, ::-1], 1, axis=2)
            return -b if name == "u" else b
        b = np.roll(a[:, ::-1, :], 1, axis=1)
        return -b if name == "v" else b

    def run(transform):
        p = default_params()
        p.nx, p.ny, p.nz = 16, 12, 13
        p.noise_amp, p.f, p.chand = 0.1, 0.0, 0.0
        o = O.Oracle(p)
        o.static()
        if transform:
            for n in fields:
                o.set(n, act(n, o.get(n)))
        o.calcdt()
        assert o.step(12) == 0
        return {n: o.get(n) for n in fields}, o.scalars().ttime

    a, ta = run(False)
    b, tb = run(True)
    assert ta == tb
    for n in fields:
        scale = max(1.0, np.abs(a[n]).max())
        assert np.abs(act(n, a[n]) - b[n]).max() < 1e-14 * scale * 10, n


def test_magnetic_step_commutes_with_horizontal_shifts():
    """The MHD step loop (mag_init's seed field, induction, bandj, the
    mean-field equations) commutes with a horizontal grid shift. The
    spectral potentials are shifted through the inverse and forward
    transforms. 12 steps agree to rounding, B measured against its
    largest component."""
    shift = (2, 3)
    real = ("r", "t", "u", "v", "w", "bx", "by", "bz", "jsq")

    def run(shifted):
        p = default_params()
        p.nx, p.ny, p.nz = 16, 12, 13
        p.noise_amp, p.dynamo = 0.1, 1
        o = O.Oracle(p)
        o.static()
        o.mag_init()
        if shifted:
            for n in real:
                o.set(n, np.roll(o.get(n), shift, axis=(1, 2)))
            for n in ("pol", "tor"):
                o.set(n, o.forwardfft(np.roll(o.inversefft(o.get(n)), shift, axis=(1, 2))))
        o.calcdt()
        assert o.step(12) == 0
        out = {n: o.get(n) for n in real}
        out["pol"], out["tor"] = o.inversefft(o.get("pol")), o.inversefft(o.get("tor"))
        return out, o.get_mean("bxbar"), o.get_mean("bybar")

    a, axb, ayb = run(False)
    b, bxb, byb = run(True)
    bscale = max(np.abs(a[n]).max() for n in ("bx", "by", "bz"))
    for n in a:
        scale = bscale if n in ("bx", "by", "bz") else np.abs(a[n]).max()
        assert np.abs(np.roll(a[n], shift, axis=(1, 2)) - b[n]).max() <= 1e-12 * scale, n
    for m, mm in ((axb, bxb), (ayb, byb)):
        assert np.abs(m - mm).max() <= 1e-12 * np.abs(m).max()
