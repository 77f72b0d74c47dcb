"""The closure network's CUDA kernels against the numpy oracle.

Forward output, loss and every parameter gradient are compared with the
oracle run in its BF16-emulating mode (same roundings as the GPU, float64
accumulation where the GPU accumulates in FP32).  Remaining differences come
from FP32 accumulation order flipping a BF16 rounding now and then, so the
tolerance is 2e-2 of the largest magnitude of each array (BF16 has 8
significant bits).  One Adam step matches the float32 oracle to 1e-6, and a
short training run on a learnable target cuts the loss fourfold."""
import numpy as np
import pytest

from oracle import closure_oracle as CO
from fug30v0kxc_gb300.closure import Net

pytestmark = pytest.mark.gpu


def _case(nx, ny, nz, nb, seed):
    rng = np.random.default_rng(seed)
    p = CO.init_params(seed=seed, out_scale=1.0)
    lay, n = CO.layout()
    for ow, ob, ci, co in lay:
        p[ob:ob + min(co, 32)] = (0.1 * rng.standard_normal(co)).astype(np.float32)
    p[lay[3][1] + 8:lay[3][1] + 16] = 0.0
    x = np.zeros((nb, nz, ny, nx, 16), np.float32)
    x[..., :9] = rng.standard_normal((nb, nz, ny, nx, 9))
    tgt = rng.standard_normal((nb, nz, ny, nx, 8)).astype(np.float32)
    return p, x, tgt


def _close(a, b, tol):
    scale = max(np.abs(b).max(), 1e-30)
    return np.abs(a - b).max() <= tol * scale


@pytest.mark.parametrize("nx,ny,nz,nb,mt", [(16, 16, 5, 2, "2"), (32, 8, 4, 1, "2"), (64, 4, 3, 2, "2"),
                                             (128, 2, 3, 1, "2"), (16, 16, 5, 2, "1"), (128, 3, 3, 1, "2"),
                                             (128, 2, 3, 1, "tc"), (128, 4, 5, 2, "tc")])
def test_forward_backward_match_oracle(nx, ny, nz, nb, mt, monkeypatch):
    """mt: m-tiles per warp in the mma.sync convolution kernels (the
    128 x 3 plane does not divide into 256-point tiles and takes the one-tile
    path); "tc": forward and input gradient on tcgen05 (nx = 128)."""
    monkeypatch.setenv("VEC_NET_MT", "2" if mt == "tc" else mt)
    monkeypatch.setenv("VEC_NET_TC", "1" if mt == "tc" else "0")
    p, x, tgt = _case(nx, ny, nz, nb, seed=nx + nz)
    net = Net(nx, ny, nz, nb)
    net.set_params(p)
    out = net.forward(x)
    loss = net.backward(tgt)
    g = net.grads()
    ro, cache = CO.forward(p, x, exact=False)
    rl, rg = CO.backward(p, cache, ro, tgt, exact=False)
    assert _close(out, ro, 2e-2)
    assert abs(loss - rl) <= 1e-2 * rl
    lay, _ = CO.layout()
    for l, (ow, ob, ci, co) in enumerate(lay):
        assert _close(g[ow:ob], rg[ow:ob], 2e-2), l
        assert _close(g[ob:ob + co], rg[ob:ob + co], 2e-2), l
    net.close()


def test_adam_step_matches_oracle():
    p, x, tgt = _case(16, 16, 5, 2, seed=7)
    net = Net(16, 16, 5, 2)
    net.set_params(p)
    net.forward(x)
    net.backward(tgt)
    g = net.grads()
    net.adam(1e-3)
    p1 = net.params()
    rp, _, _ = CO.adam(p, g, np.zeros_like(p), np.zeros_like(p), 1, 1e-3)
    assert np.abs(p1 - rp).max() <= 1e-6
    net.close()


def test_training_reduces_loss():
    """Target: a fixed random 3x3x3 linear map of the inputs (learnable)."""
    rng = np.random.default_rng(11)
    nx, ny, nz, nb = 32, 32, 6, 4
    Wt = 0.05 * rng.standard_normal((27, 8, 16))
    Wt[:, :, 9:] = 0.0
    net = Net(nx, ny, nz, nb, seed=5)
    losses = []
    for it in range(300):
        x = np.zeros((nb, nz, ny, nx, 16), np.float32)
        x[..., :9] = rng.standard_normal((nb, nz, ny, nx, 9))
        tgt = CO.conv(x.astype(np.float64), Wt).astype(np.float32)
        net.forward(x)
        losses.append(net.backward(tgt))
        net.adam(1e-3)
    assert np.mean(losses[-20:]) < 0.25 * np.mean(losses[:5]), (losses[:5], losses[-5:])
    net.close()
