"""A size-independent property at the benchmark grid, 256^2 x 129.

The static polytrope with polytropic index 1 is a fixed point of the whole
time step (src/main.F90:340-747). T = 1 + theta z, rho = T and p = T^2 are
polynomials of degree <= 2 in z, on which every z stencil is exact. With
uniform kappa and a uniform vertical field, every right-hand side vanishes,
and the boundary conditions hold. The oracle keeps this state bit for bit
(tests/test_oracle_pins.py). The library, in the FP64 and split forms, may
move it only by rounding: about 1e-14 here, against the O(dt) ~ 1e-4 of
any real imbalance. Run for 25 steps, past the 10-step dealias and calcdt
cadence, with diagnostics every 5 steps.

The same body runs on the oracle at a small size in the CPU suite.
"""
import numpy as np
import pytest

from oracle import oracle as O
from fug30v0kxc_gb300.params import VEC_PREC_FP64, VEC_PREC_SPLIT, default_params

STEPS = 25


def fixed_point_drift(make, nx, ny, nz, precision):
    """Largest change of each state field over STEPS steps, relative to
    max(1, the field's scale), the iterations and model time the run
    advanced, and dt."""
    p = default_params()
    p.nx, p.ny, p.nz = nx, ny, nz
    p.noise_amp, p.cm, p.kappa_uniform, p.ndu06 = 0.0, 1.0, 1, 5
    p.precision = precision
    s = make(p)
    s.static()
    s.mag_init()
    dt = s.calcdt()
    s0, c0 = s.state(), s.scalars()
    assert s.step(STEPS) == 0
    s1, c1 = s.state(), s.scalars()
    drift = {n: float(np.abs(s1[n] - s0[n]).max() / max(1.0, np.abs(s0[n]).max())) for n in s0}
    return drift, c1.iter - c0.iter, c1.ttime - c0.ttime, dt


def test_oracle_fixed_point_small():
    drift, iters, elapsed, dt = fixed_point_drift(O.Oracle, 16, 16, 17, VEC_PREC_FP64)
    assert all(d == 0.0 for d in drift.values()), drift
    assert iters == STEPS and abs(elapsed - STEPS * dt) <= 1e-12 * STEPS * dt


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [VEC_PREC_FP64, VEC_PREC_SPLIT])
def test_fixed_point_at_benchmark_grid(precision):
    from fug30v0kxc_gb300.solver import P3D
    drift, iters, elapsed, dt = fixed_point_drift(P3D, 256, 256, 129, precision)
    print("drift over", STEPS, "steps:", drift)
    assert all(d < 1e-8 for d in drift.values()), drift
    assert iters == STEPS and abs(elapsed - STEPS * dt) <= 1e-9 * STEPS * dt
