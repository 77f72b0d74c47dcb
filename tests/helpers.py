"""Shared test helpers: seeded smooth states and comparison utilities."""
import numpy as np

from fug30v0kxc_gb300.params import STATE_FIELDS, config0, convection_params, default_params


def small_params(nx=32, ny=32, nz=17, **kw):
    p = convection_params(nx, ny, nz, **kw)
    p.ndu06 = 5
    return p


def smooth_state(p, seed=0, amp=1e-2, bamp=5e-2):
    """A seeded, smooth, non-trivial state: velocities vanish at the walls,
    T and rho are the polytrope plus perturbations, B has a horizontal
    structure (pol/tor are obtained by the caller via mag_init)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = p.nx, p.ny, p.nz
    x = np.arange(nx) * (p.xmax / nx)
    y = np.arange(ny) * (p.ymax / ny)
    z = np.arange(nz) / (nz - 1)
    X, Y = np.meshgrid(x, y)          # (ny, nx)

    def horiz(nmodes=4):
        f = np.zeros((ny, nx))
        for _ in range(nmodes):
            kx = rng.integers(0, max(1, nx // 6)) * 2 * np.pi / p.xmax
            ky = rng.integers(0, max(1, ny // 6)) * 2 * np.pi / p.ymax
            ph = rng.uniform(0, 2 * np.pi)
            f += rng.normal() * np.cos(kx * X + ky * Y + ph)
        return f

    prof = np.sin(np.pi * z)[:, None, None]
    t0 = (1.0 + p.theta * z)[:, None, None]
    s = {}
    s["u"] = amp * prof * np.stack([horiz() * (1 + 0.3 * zz) for zz in z])
    s["v"] = amp * prof * np.stack([horiz() * (1 - 0.2 * zz) for zz in z])
    s["w"] = amp * prof * np.stack([horiz() for _ in z])
    s["t"] = t0 + amp * prof * np.stack([horiz() for _ in z])
    s["r"] = t0 ** p.cm * (1.0 + amp * prof * np.stack([horiz() for _ in z]))
    s["bx"] = bamp * np.stack([horiz() * np.cos(np.pi * zz) for zz in z])
    s["by"] = bamp * np.stack([horiz() * np.cos(np.pi * zz) for zz in z])
    s["bz"] = 1.0 + bamp * np.stack([horiz() for _ in z])
    return {k: np.ascontiguousarray(v) for k, v in s.items()}


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)


def top_nusselt(p, t):
    """Nusselt number at the fixed-temperature top plane: the formula of
    src/dbydz.F90:4877-4925 with its one-sided derivative mirrored to the
    top, (-11 T1 + 18 T2 - 9 T3 + 2 T4) / (6 dz) averaged over the plane.
    With the fixed-flux bottom of these configurations the reference's own
    (bottom) Nusselt number is identically one, so this is the live one."""
    dz = 1.0 / (p.nz - 1)
    tz = (-11.0 * t[0] + 18.0 * t[1] - 9.0 * t[2] + 2.0 * t[3]) / (6.0 * dz)
    nusstmp = p.theta * (p.cm + 1.0) * (1.0 - 1.0 / p.gamma)
    return (float(tz.mean()) - nusstmp) / (p.theta - nusstmp)


def perturbation_menergy(p, bx, by, bz, bzbar):
    """Magnetic energy of the field perturbation: the diagnostic's
    F * (1/2) int |B|^2 (trapezium in z, src/utils.F90:22-139) with the
    uniform seed field bzbar taken out of bz before squaring, so that the
    small perturbation energy is not a difference of two large numbers."""
    e = (bx * bx + by * by + (bz - bzbar) ** 2).sum(axis=(1, 2))
    wz = np.ones(p.nz)
    wz[0] = wz[-1] = 0.5
    dxdydz = (p.xmax / p.nx) * (p.ymax / p.ny) / (p.nz - 1)
    return float(p.f * 0.5 * (wz * e).sum() * dxdydz)
