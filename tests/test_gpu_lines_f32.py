"""The FP32 line kernels of the split form against the FP64 oracle.

The split time step runs its horizontal derivatives, dealiasing and 2-D
transforms (src/fft.F90:255-799) through the FP32 instances of the line
kernels: the TMA-fed register FFT for n = 2^a and 3*2^a (64..1024, two tile
shapes for n <= 256: 16 and 8 sequences per tile) and the generic Stockham
kernel for the other lengths.  vec_line_f32 runs exactly those kernels on
caller data (two tile shapes for n >= 768 too: 8 and 4 sequences).  Every
instance is compared on seeded random data with the
oracle's FP64 operators; a wrong twiddle, multiplier or index gives O(1)
errors, FP32 rounding gives ~1e-7.

Tolerance: largest difference over the largest reference value below 1e-5
(the transforms' rounding grows like log2 n times the FP32 unit roundoff).
"""
import numpy as np
import pytest

from oracle import oracle as O
from fug30v0kxc_gb300.params import default_params
from fug30v0kxc_gb300.solver import P3D
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

D1, D2, DEALIAS, FWD, INV = 1, 2, 3, 4, 5
TOL = 1e-5
LENGTHS = [64, 96, 128, 192, 256, 384, 512, 768, 1024]


def _pair(nx, ny, nz=6):
    p = default_params()
    p.nx, p.ny, p.nz = nx, ny, nz
    return P3D(p), O.Oracle(p)


def _check_direction(g, o, direction, f):
    """Every operator of one direction: d1, the (d1, d2) pair from one
    forward transform, dealias, and forward / inverse transforms."""
    ref_d1 = o.d1bydx(f) if direction == 0 else o.d1bydy(f)
    ref_d1b, ref_d2 = o.d2bydx(f) if direction == 0 else o.d2bydy(f)
    errs = {"d1": rel_err(g.line_f32(direction, D1, f), ref_d1)}
    a, b = g.line_f32(direction, D1, f, op2=D2)
    errs["d2.f1"] = rel_err(a, ref_d1b)
    errs["d2.f2"] = rel_err(b, ref_d2)
    # the oracle's dealias and 2-D transforms run x then y; with the other
    # direction's FP32 pass the composition is the same operator
    other = 1 - direction
    f32 = f.astype(np.float32)
    da = g.line_f32(other, DEALIAS, g.line_f32(direction, DEALIAS, f32))
    errs["dealias"] = rel_err(da, o.dealias(f))
    F = g.line_f32(other, FWD, g.line_f32(direction, FWD, f32))
    ref_F = o.forwardfft(f)
    errs["forward"] = rel_err(F, ref_F)
    back = g.line_f32(other, INV, g.line_f32(direction, INV, ref_F.astype(np.float32)))
    ref_back = o.inversefft(ref_F)
    errs["inverse"] = rel_err(back, ref_back)
    # an inverse with the derivative of the inverse as its second output
    # (the split bandj's d(bz)/dx, d(bz)/dy): completed by the other
    # direction's inverse, the second output is the derivative of the 2-D
    # inverse transform
    a, b = g.line_f32(direction, INV, ref_F.astype(np.float32), op2=D1)
    errs["inv+d1.inv"] = rel_err(g.line_f32(other, INV, a), ref_back)
    ref_dback = o.d1bydx(ref_back) if direction == 0 else o.d1bydy(ref_back)
    errs["inv+d1.d1"] = rel_err(g.line_f32(other, INV, b), ref_dback)
    return errs


CASES = [(n, 0) for n in LENGTHS] + [(n, 8) for n in LENGTHS if n <= 256] + [(n, 4) for n in LENGTHS if n >= 768]


@pytest.mark.parametrize("n,tile", CASES)
def test_f32_line_kernels_match_fp64_oracle(n, tile):
    """x lines of length n on an (n, 64, 6) grid and y lines of length n on
    a (64, n, 6) grid; tile 8 selects the 8-sequence tile for n <= 256 and
    tile 4 the 4-sequence tile for n >= 768; 0 is the kernel's default."""
    rng = np.random.default_rng(n + tile)
    for direction, (nx, ny) in ((0, (n, 64)), (1, (64, n))):
        g, o = _pair(nx, ny)
        g.set_tunables(16, tile)
        f = rng.standard_normal((6, ny, nx))
        errs = _check_direction(g, o, direction, f)
        assert max(errs.values()) < TOL, (n, tile, direction, errs)
        g.close()
        o.close()


@pytest.mark.parametrize("nx,ny", [(80, 48), (60, 100)])
def test_f32_generic_line_kernel_matches_fp64_oracle(nx, ny):
    """Lengths outside the register kernel's set (2^a 3^b 5^c) run the
    generic Stockham kernel in FP32."""
    rng = np.random.default_rng(nx * ny)
    g, o = _pair(nx, ny)
    f = rng.standard_normal((6, ny, nx))
    for direction in (0, 1):
        errs = _check_direction(g, o, direction, f)
        assert max(errs.values()) < TOL, (nx, ny, direction, errs)


def test_f32_line_rejects_bad_operators():
    g, _ = _pair(64, 64)
    f = np.zeros((6, 64, 64), np.float32)
    out = np.empty_like(f)
    for d, op1, op2 in ((2, D1, 0), (0, 0, 0), (0, 6, 0), (0, FWD, D2), (0, D1, DEALIAS), (0, INV, D2)):
        st = g.L.vec_line_f32(g.h, d, op1, op2, f.ctypes.data, out.ctypes.data, out.ctypes.data)
        assert st == -31, (d, op1, op2, st)
