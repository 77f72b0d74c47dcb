"""CPU pins of the closure oracle (oracle/closure_oracle.py): BF16 rounding
known answers, the adjoint identity of the convolution pair, and the float64
backward pass against central finite differences."""
import numpy as np

from oracle import closure_oracle as CO


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 1.0 + 2.0 ** -9, -2.5, 3.0e38, 1.0e-30],
                 np.float32)
    r = CO.bf16(x)
    # ties go to even: 1 + 2^-8 -> 1, 1 + 3*2^-8 -> 1 + 2^-6
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2.0 ** -6 and r[3] == 1.0
    assert r[4] == -2.5
    assert abs(r[5] / 3.0e38 - 1) < 2 ** -8 and abs(r[6] / 1e-30 - 1) < 2 ** -8


def test_conv_adjoint():
    rng = np.random.default_rng(1)
    X = rng.standard_normal((2, 4, 8, 16, 16))
    Y = rng.standard_normal((2, 4, 8, 16, 32))
    W = rng.standard_normal((27, 32, 16))
    lhs = np.sum(CO.conv(X, W) * Y)
    rhs = np.sum(X * CO.conv_input_grad(Y, W))
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs)


def test_backward_finite_differences():
    rng = np.random.default_rng(2)
    p = CO.init_params(seed=3, out_scale=1.0).astype(np.float64)
    lay, n = CO.layout()
    for ow, ob, ci, co in lay:
        p[ob:ob + co] = 0.1 * rng.standard_normal(co)
    x = np.zeros((1, 3, 8, 16, 16))
    x[..., :9] = rng.standard_normal((1, 3, 8, 16, 9))
    tgt = rng.standard_normal((1, 3, 8, 16, 8))
    out, cache = CO.forward(p, x, exact=True)
    loss, g = CO.backward(p, cache, out, tgt, exact=True)
    # probe real (non-padded) weights and biases of every layer
    idx = []
    creal_in, creal_out = (9, 32, 32, 32), (32, 32, 32, 8)
    for l, (ow, ob, ci, co) in enumerate(lay):
        for _ in range(5):
            t, o, i = rng.integers(27), rng.integers(creal_out[l]), rng.integers(creal_in[l])
            idx.append(ow + (t * co + o) * ci + i)
        idx.append(ob + int(rng.integers(creal_out[l])))
    h = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        lp = np.mean((CO.forward(pp, x)[0] - tgt) ** 2)
        lm = np.mean((CO.forward(pm, x)[0] - tgt) ** 2)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g).max()), (k, fd, g[k])
