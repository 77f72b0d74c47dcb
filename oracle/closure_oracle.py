"""CPU oracle of the learned closure (numpy).

TEST INFRASTRUCTURE ONLY: used by tests/ as the checker of the GPU closure
network, box filter and spectral upsampler, never on the product path.

The closure has no reference counterpart: it is a 4-layer 3x3x3
convolutional network (9 real input channels padded to 16 -> 32 -> 32 -> 32
-> 8 output channels padded to 16, GELU with the Gaussian CDF between
layers) on channel-last fields [batch][nz][ny][nx][channel], periodic in x
and y and zero-padded in z.  Tap t = 9(dz+1) + 3(dy+1) + (dx+1) multiplies
X[x+dx, y+dy, z+dz].  Two modes:

* exact=True: float64 throughout (pinned by central finite differences);
* exact=False: rounds to BF16 (round-to-nearest-even) where the GPU stores
  BF16 -- inputs, weights, pre-activations, activations, gradients -- and
  accumulates in float64 where the GPU accumulates in FP32.
"""
import numpy as np
from scipy.special import erf

NTAP = 27
LCI = (16, 32, 32, 32)
LCO = (32, 32, 32, 16)
COUT_REAL = 8


def bf16(a):
    """Round float32 values to the nearest BF16 (ties to even)."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32).astype(np.float64)


def layout():
    """Offsets of each layer's weights [27][cout][cin] and biases [cout]."""
    off, out = 0, []
    for ci, co in zip(LCI, LCO):
        ow = off
        off += NTAP * co * ci
        ob = off
        off += co
        out.append((ow, ob, ci, co))
    return out, off


def unpack(p):
    lay, _ = layout()
    Ws, bs = [], []
    for ow, ob, ci, co in lay:
        Ws.append(np.asarray(p[ow:ow + NTAP * co * ci], np.float64).reshape(NTAP, co, ci))
        bs.append(np.asarray(p[ob:ob + co], np.float64))
    return Ws, bs


def taps():
    for t in range(NTAP):
        yield t, t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1


def shift(X, dz, dy, dx):
    """S[b, z, y, x] = X[b, z+dz, y+dy, x+dx]; periodic in x, y, zero in z."""
    S = np.roll(X, shift=(-dy, -dx), axis=(2, 3))
    out = np.zeros_like(S)
    nz = X.shape[1]
    lo, hi = max(0, -dz), min(nz, nz - dz)
    if hi > lo:
        out[:, lo:hi] = S[:, lo + dz:hi + dz]
    return out


def conv(X, W, b=None):
    """Y[p, co] = sum_t sum_ci W[t, co, ci] X[p + d_t, ci] (+ b[co])."""
    Y = np.zeros(X.shape[:-1] + (W.shape[1],))
    for t, dz, dy, dx in taps():
        Y += shift(X, dz, dy, dx) @ W[t].T
    if b is not None:
        Y += b
    return Y


def conv_input_grad(dY, W):
    """dX[q, ci] = sum_t sum_co W[t, co, ci] dY[q - d_t, co]."""
    dX = np.zeros(dY.shape[:-1] + (W.shape[2],))
    for t, dz, dy, dx in taps():
        dX += shift(dY, -dz, -dy, -dx) @ W[t]
    return dX


def conv_weight_grad(X, dY):
    """dW[t, co, ci] = sum_p dY[p, co] X[p + d_t, ci]; db[co] = sum_p dY[p, co]."""
    co, ci = dY.shape[-1], X.shape[-1]
    dW = np.zeros((NTAP, co, ci))
    dYf = dY.reshape(-1, co)
    for t, dz, dy, dx in taps():
        dW[t] = dYf.T @ shift(X, dz, dy, dx).reshape(-1, ci)
    return dW, dYf.sum(axis=0)


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_d(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def forward(p, x, exact=True):
    """x: [B, nz, ny, nx, 16]; returns (out [.., 8], cache)."""
    r = (lambda a: a) if exact else bf16
    Ws, bs = unpack(p)
    Wr = [r(W) for W in Ws]
    a = r(x)
    cache = {"x": a, "pre": [], "act": [], "W": Wr}
    for l in range(3):
        pre = conv(a, Wr[l], bs[l])
        a = r(gelu(pre))
        cache["pre"].append(r(pre))
        cache["act"].append(a)
    out = conv(a, Wr[3], bs[3])[..., :COUT_REAL]
    return out, cache


def backward(p, cache, out, tgt, exact=True):
    """MSE loss and the flat gradient vector (same layout as p)."""
    r = (lambda a: a) if exact else bf16
    Wr = cache["W"]
    cnt = out.size
    loss = float(np.sum((out - tgt) ** 2) / cnt)
    dout = np.zeros(out.shape[:-1] + (16,))
    dout[..., :COUT_REAL] = 2.0 * (out - tgt) / cnt
    dout = r(dout)
    lay, n = layout()
    g = np.zeros(n)
    ins = [cache["x"]] + cache["act"]
    d = dout
    for l in (3, 2, 1, 0):
        dW, db = conv_weight_grad(ins[l], d)
        ow, ob, ci, co = lay[l]
        g[ow:ow + dW.size] = dW.ravel()
        g[ob:ob + co] = db
        if l > 0:
            d = r(conv_input_grad(d, Wr[l]) * gelu_d(cache["pre"][l - 1]))
    return loss, g


def init_params(seed=0, out_scale=0.1):
    """He-uniform weights on the real channels, zero elsewhere, zero biases."""
    rng = np.random.default_rng(seed)
    lay, n = layout()
    p = np.zeros(n, np.float32)
    creal_in, creal_out = (9, 32, 32, 32), (32, 32, 32, 8)
    for l, (ow, ob, ci, co) in enumerate(lay):
        a = np.sqrt(6.0 / (NTAP * creal_in[l])) * (out_scale if l == 3 else 1.0)
        W = np.zeros((NTAP, co, ci), np.float32)
        W[:, :creal_out[l], :creal_in[l]] = rng.uniform(-a, a, (NTAP, creal_out[l], creal_in[l]))
        p[ow:ow + W.size] = W.ravel()
    return p


def adam(p, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One bias-corrected Adam step in float32 (returns new p, m, v)."""
    p, g, m, v = (np.asarray(a, np.float32) for a in (p, g, m, v))
    m = np.float32(b1) * m + np.float32(1 - b1) * g
    v = np.float32(b2) * v + np.float32(1 - b2) * g * g
    c1, c2 = np.float32(1 - b1 ** t), np.float32(1 - b2 ** t)
    p = p - np.float32(lr) * (m / c1) / (np.sqrt(v / c2) + np.float32(eps))
    return p, m, v


# ---- the spectral upsampler (interpolate/fft.F90:834-927) ----------------------------
def _hc(x, axis):
    """FFTW halfcomplex forward transform along axis (unnormalised, sign -1):
    r0, r1, ..., r_{n/2}, i_{(n-1)/2}, ..., i_1."""
    n = x.shape[axis]
    X = np.fft.rfft(x, axis=axis)
    X = np.moveaxis(X, axis, -1)
    h = np.zeros(X.shape[:-1] + (n,))
    h[..., :n // 2 + 1] = X.real[..., :n // 2 + 1]
    for k in range(1, (n - 1) // 2 + 1):
        h[..., n - k] = X.imag[..., k]
    return np.moveaxis(h, -1, axis)


def _hc_inv(h, axis):
    """FFTW halfcomplex backward transform along axis (unnormalised)."""
    n = h.shape[axis]
    H = np.moveaxis(h, axis, -1)
    X = np.zeros(H.shape[:-1] + (n // 2 + 1,), complex)
    X.real[..., :n // 2 + 1] = H[..., :n // 2 + 1]
    for k in range(1, (n - 1) // 2 + 1):
        X.imag[..., k] = H[..., n - k]
    x = np.fft.irfft(X, n=n, axis=-1) * n
    return np.moveaxis(x, -1, axis)


def expand_axis(f, axis, r):
    """One axis of expand: modes 0..n/2 (Nyquist real part included) keep
    their index, imaginary parts move from n - k to N - k, N = r n; the
    backward transform of length N is divided by n."""
    n = f.shape[axis]
    N = r * n
    H = np.moveaxis(_hc(f, axis), axis, -1)
    G = np.zeros(H.shape[:-1] + (N,))
    G[..., :n // 2 + 1] = H[..., :n // 2 + 1]
    for k in range(1, n // 2):
        G[..., N - k] = H[..., n - k]
    g = _hc_inv(np.moveaxis(G, -1, axis), axis) / n
    return g


def expand(f, r=2):
    """f[nz, ny, nx] -> [nz, r ny, r nx]: x first, then y, as the reference."""
    return expand_axis(expand_axis(f, 2, r), 1, r)


# ---- the box filter ---------------------------------------------------------------
def box_filter(f, r):
    """f[nz_f, ny_f, nx_f] -> [nz_c, ny_c, nx_c]: weights (1, 2, ..., 2, 1)/2r
    over 2r+1 points per axis (periodic in x, y); wall planes taken alone."""
    h = r // 2
    w = np.array([0.5 if abs(j) == h else 1.0 for j in range(-h, h + 1)]) / r
    nzf, nyf, nxf = f.shape
    nzc = (nzf - 1) // r + 1
    g = np.zeros((nzf, nyf // r, nxf // r))
    for dj, wy in zip(range(-h, h + 1), w):
        for di, wx in zip(range(-h, h + 1), w):
            g += wy * wx * np.roll(f, (-dj, -di), axis=(1, 2))[:, ::r, ::r]
    out = np.zeros((nzc, nyf // r, nxf // r))
    out[0] = g[0]
    out[-1] = g[-1]
    for kc in range(1, nzc - 1):
        out[kc] = sum(wz * g[r * kc + dk] for dk, wz in zip(range(-h, h + 1), w))
    return out
