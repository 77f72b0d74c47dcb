"""GPU parity of the per-operator entry points against the CPU oracle.

Tolerances (FP64): horizontal spectral operators and z stencils agree with
the oracle to 1e-12 relative to the field's max (different FFT
factorisations and FMA contraction change the rounding only); the initial
state is integer arithmetic plus exactly rounded operations and must be
bit-identical.
"""
import numpy as np
import pytest

from oracle import oracle as O
from fug30v0kxc_gb300.params import default_params
from fug30v0kxc_gb300.solver import P3D, VecError
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

SIZES = [(30, 30, 8), (64, 48, 7), (4, 4, 6), (96, 60, 9), (256, 256, 6), (10, 250, 6),
         (128, 128, 6), (512, 64, 6), (64, 1024, 6), (1024, 32, 6), (64, 64, 7),
         (192, 96, 6), (384, 64, 6), (96, 768, 6)]
TOL = 1e-12


def _pair(nx, ny, nz, **kw):
    p = default_params()
    p.nx, p.ny, p.nz = nx, ny, nz
    for k, v in kw.items():
        setattr(p, k, v)
    return P3D(p), O.Oracle(p)


@pytest.mark.parametrize("nx,ny,nz", SIZES)
def test_horizontal_operators(nx, ny, nz):
    g, o = _pair(nx, ny, nz)
    rng = np.random.default_rng(nx * 1000 + ny)
    f = rng.standard_normal((nz, ny, nx))
    assert rel_err(g.d1bydx(f), o.d1bydx(f)) < TOL
    assert rel_err(g.d1bydy(f), o.d1bydy(f)) < TOL
    for a, b in zip(g.d2bydx(f), o.d2bydx(f)):
        assert rel_err(a, b) < TOL
    for a, b in zip(g.d2bydy(f), o.d2bydy(f)):
        assert rel_err(a, b) < TOL
    assert rel_err(g.dealias(f), o.dealias(f)) < TOL
    F = g.forwardfft(f)
    assert rel_err(F, o.forwardfft(f)) < TOL
    assert rel_err(g.inversefft(F), o.inversefft(F)) < TOL
    assert rel_err(g.inversefft(F), f) < 1e-13


@pytest.mark.parametrize("nx,ny,nz", [(8, 8, 6), (16, 8, 7), (8, 4, 33)])
def test_z_operators(nx, ny, nz):
    g, o = _pair(nx, ny, nz)
    rng = np.random.default_rng(nz)
    f = rng.standard_normal((nz, ny, nx))
    w = rng.standard_normal((nz, ny, nx))
    g.set("w", w)
    o.set("w", w)
    for fl in (0, 1, 2, 5):
        assert rel_err(g.d1bydz(f, fl), o.d1bydz(f, fl)) < TOL
        assert rel_err(g.d1upbydz(f, fl), o.d1upbydz(f, fl)) < TOL
        assert rel_err(g.d1bydz1d(f[:, 0, 0], fl), o.d1bydz1d(f[:, 0, 0], fl)) < TOL
    for fl in (0, 3):
        assert rel_err(g.d2bydz(f, fl), o.d2bydz(f, fl)) < TOL
        assert rel_err(g.d2bydz1d(f[:, 0, 0], fl), o.d2bydz1d(f[:, 0, 0], fl)) < TOL
    for bad in (3, 4, -1):
        with pytest.raises(VecError) as e:
            g.d1bydz(f, bad)
        assert e.value.status == -7
    with pytest.raises(VecError) as e:
        g.d2bydz(f, 5)
    assert e.value.status == -7


def test_device_pointers():
    torch = pytest.importorskip("torch")
    g, o = _pair(64, 64, 8)
    rng = np.random.default_rng(7)
    f = rng.standard_normal((8, 64, 64))
    fd = torch.from_numpy(f).cuda()
    od = torch.empty_like(fd)
    assert g.L.vec_d1bydx(g.h, fd.data_ptr(), od.data_ptr()) == 0
    torch.cuda.synchronize()
    assert rel_err(od.cpu().numpy(), o.d1bydx(f)) < TOL


@pytest.mark.parametrize("perfect", [0, 1])
def test_static_ic_bit_exact(perfect):
    g, o = _pair(64, 32, 9, noise_amp=1e-3, theta=9.0, perfect=perfect)
    g.static()
    o.static()
    for n in ("r", "t", "u", "v", "w", "bx", "by", "bz"):
        assert np.array_equal(g.get(n), o.get(n)), n


def test_bad_sizes():
    for nx, ny, nz, code in ((7, 8, 8, -1), (8, 9, 8, -2), (8, 8, 5, -4), (14, 8, 8, -32)):
        p = default_params()
        p.nx, p.ny, p.nz = nx, ny, nz
        with pytest.raises(VecError) as e:
            P3D(p)
        assert e.value.status == code


@pytest.mark.parametrize("nx,ny,nz", [(256, 256, 7), (64, 128, 6), (1024, 64, 6), (128, 512, 6),
                                      (192, 192, 7), (96, 384, 6), (768, 96, 6)])
def test_specialised_lines_match_generic(nx, ny, nz, monkeypatch):
    """The 2^a / 3*2^a line kernel (TMA-fed, register four-step FFT) and the
    generic shared-memory Stockham kernel agree on every operator."""
    rng = np.random.default_rng(nx + ny)
    f = rng.standard_normal((nz, ny, nx))
    p = default_params()
    p.nx, p.ny, p.nz = nx, ny, nz
    fast = P3D(p)
    monkeypatch.setenv("VEC_GENERIC_LINES", "1")
    slow = P3D(p)
    for name in ("d1bydx", "d1bydy", "dealias", "forwardfft"):
        a, b = getattr(fast, name)(f), getattr(slow, name)(f)
        assert rel_err(a, b) < 1e-13, name
    for name in ("d2bydx", "d2bydy"):
        for a, b in zip(getattr(fast, name)(f), getattr(slow, name)(f)):
            assert rel_err(a, b) < 1e-13, name
    F = fast.forwardfft(f)
    assert rel_err(fast.inversefft(F), slow.inversefft(F)) < 1e-13
