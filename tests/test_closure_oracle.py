"""CPU pins of the closure oracle (oracle/closure_oracle.py): BF16 rounding
known answers, the adjoint identity of the convolution pair, the float64
backward pass against central finite differences, the spectral upsampler on
band-limited fields and the box filter's transfer function."""
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


def test_expand_is_exact_for_band_limited_fields():
    """The spectral upsampler (interpolate/fft.F90:834-927) returns a field
    made of modes below the coarse Nyquist frequency exactly at the fine
    grid points, for r = 2 and 4 (x first, then y)."""
    nz, ny, nx = 3, 8, 12
    xs = lambda n: 2 * np.pi * np.arange(n) / n   # noqa: E731  (unit-period grid)

    def field(ny_, nx_):
        f = np.zeros((nz, ny_, nx_))
        X, Y = np.meshgrid(xs(nx_), xs(ny_))
        for kx, ky, a, b in ((1, 0, 0.7, -0.2), (2, 3, 0.3, 0.5), (5, 1, -0.4, 0.1), (0, 2, 0.25, 0.0)):
            f += (a * np.cos(kx * X + ky * Y) + b * np.sin(kx * X - ky * Y))[None]
        return f

    coarse = field(ny, nx)
    for r in (2, 4):
        fine = CO.expand(coarse, r)
        assert fine.shape == (nz, r * ny, r * nx)
        assert np.abs(fine - field(r * ny, r * nx)).max() < 1e-13


def test_box_filter_transfer_function():
    """The box filter's weights (1, 2, ..., 2, 1) / 2r over 2r + 1 fine points
    per horizontal axis sum to 1. On a mode cos(k x) it therefore returns
    H(k) cos(k x) at the coarse points, with the transfer function
    H(k) = (1/r)(sum_{|j| < r/2} cos(k j dx) + cos(k r dx / 2)) per axis.
    Planes the z weights combine, all equal here, are left unchanged."""
    r = 4
    nzf, nyf, nxf = 2 * r + 1, 16, 32
    dx = 1.0
    kx, ky = 2 * np.pi * 3 / nxf, 2 * np.pi * 2 / nyf
    X, Y = np.meshgrid(np.arange(nxf) * dx, np.arange(nyf) * dx)
    f = np.broadcast_to((np.cos(kx * X) * np.cos(ky * Y))[None], (nzf, nyf, nxf)).copy()
    g = CO.box_filter(f, r)
    h = r // 2

    def H(k):
        return (sum(np.cos(k * j * dx) for j in range(-h + 1, h)) + np.cos(k * h * dx)) / r

    expect = H(kx) * H(ky) * (np.cos(kx * X) * np.cos(ky * Y))[::r, ::r]
    for kc in range(g.shape[0]):
        assert np.abs(g[kc] - expect).max() < 1e-13
    const = CO.box_filter(np.full((nzf, nyf, nxf), 2.5), r)
    assert np.abs(const - 2.5).max() < 1e-14
