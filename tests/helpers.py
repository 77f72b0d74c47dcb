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
