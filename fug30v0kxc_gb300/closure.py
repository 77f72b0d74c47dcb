"""The learned closure (no reference counterpart): host side of the GPU
network, dataset and coupling (include/vec.h, vec_net_* / vec_closure_*)."""
import ctypes as C

import numpy as np

from . import lib as _L
from .params import VecClosureReport
from .solver import VecError


class Net:
    """Four 3x3x3 convolutions (16 -> 32 -> 32 -> 32 -> 8 channels, GELU),
    BF16 weights / activations with FP32 accumulation on the GPU, Adam."""

    def __init__(self, nx, ny, nz, batch, seed=0):
        self.L = _L.load()
        h = C.c_void_p()
        st = self.L.vec_net_create(nx, ny, nz, batch, seed, C.byref(h))
        if st != 0:
            raise VecError("vec_net_create", st)
        self.h = h
        self.shape_in = (batch, nz, ny, nx, 16)
        self.shape_out = (batch, nz, ny, nx, 8)
        self.n = int(self.L.vec_net_nparams(h))

    def close(self):
        if getattr(self, "h", None):
            self.L.vec_net_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, st, where):
        if st != 0:
            raise VecError(where, st)

    def params(self):
        p = np.empty(self.n, np.float32)
        self._chk(self.L.vec_net_get_params(self.h, p.ctypes.data), "vec_net_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.n
        self._chk(self.L.vec_net_set_params(self.h, p.ctypes.data), "vec_net_set_params")

    def grads(self):
        g = np.empty(self.n, np.float32)
        self._chk(self.L.vec_net_get_grads(self.h, g.ctypes.data), "vec_net_get_grads")
        return g

    def forward(self, x):
        x = np.ascontiguousarray(x, np.float32)
        assert x.shape == self.shape_in, (x.shape, self.shape_in)
        out = np.empty(self.shape_out, np.float32)
        self._chk(self.L.vec_net_forward(self.h, x.ctypes.data, out.ctypes.data), "vec_net_forward")
        return out

    def backward(self, tgt):
        tgt = np.ascontiguousarray(tgt, np.float32)
        assert tgt.shape == self.shape_out
        loss = C.c_double()
        self._chk(self.L.vec_net_backward(self.h, tgt.ctypes.data, C.byref(loss)), "vec_net_backward")
        return loss.value

    def adam(self, lr=1e-3):
        self._chk(self.L.vec_net_adam(self.h, lr), "vec_net_adam")


class _NetView(Net):
    """The network owned by a Closure (not destroyed by this object)."""

    def __init__(self, L, h, nx, ny, nz, batch):
        self.L, self.h = L, h
        self.shape_in = (batch, nz, ny, nx, 16)
        self.shape_out = (batch, nz, ny, nx, 8)
        self.n = int(L.vec_net_nparams(h))

    def close(self):
        self.h = None


class Closure:
    """Training data, training, inference and the judged run of the learned
    closure on a coarse grid `factor` times coarser than the fine grid."""

    def __init__(self, coarse_params, factor=4, capacity=64, batch=8, seed=0):
        self.L = _L.load()
        h = C.c_void_p()
        st = self.L.vec_closure_create(C.byref(coarse_params), factor, capacity, batch, seed, C.byref(h))
        if st != 0:
            raise VecError("vec_closure_create", st)
        self.h = h
        self.p = coarse_params.copy()
        self.batch = batch
        self.npc = coarse_params.nx * coarse_params.ny * coarse_params.nz
        self.net = _NetView(self.L, C.c_void_p(self.L.vec_closure_net(h)), coarse_params.nx, coarse_params.ny,
                            coarse_params.nz, batch)

    def close(self):
        if getattr(self, "h", None):
            self.L.vec_closure_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, st, where):
        if st != 0:
            raise VecError(where, st)

    def npairs(self):
        return self.L.vec_closure_npairs(self.h)

    def box_filter(self, fine, coarse):
        self._chk(self.L.vec_box_filter(self.h, fine.h, coarse.h), "vec_box_filter")

    def add_pair(self, fine, coarse_scratch):
        self._chk(self.L.vec_closure_add_pair(self.h, fine.h, coarse_scratch.h), "vec_closure_add_pair")

    def pair(self, i):
        a = np.empty((self.npc, 8), np.float32)
        b = np.empty((self.npc, 8), np.float32)
        self._chk(self.L.vec_closure_get_pair(self.h, i, a.ctypes.data, b.ctypes.data), "vec_closure_get_pair")
        return a, b

    def fit_norm(self, n=None):
        self._chk(self.L.vec_closure_fit_norm(self.h, n or self.npairs()), "vec_closure_fit_norm")

    def norm(self):
        a = np.empty(32, np.float32)
        self._chk(self.L.vec_closure_get_norm(self.h, a.ctypes.data), "vec_closure_get_norm")
        return a

    def set_norm(self, a):
        a = np.ascontiguousarray(a, np.float32)
        self._chk(self.L.vec_closure_set_norm(self.h, a.ctypes.data), "vec_closure_set_norm")

    def train(self, iters, lr=1e-3, ntrain=None, seed=0):
        losses = np.zeros(max(iters, 1))
        self._chk(self.L.vec_closure_train(self.h, iters, lr, ntrain or self.npairs(), seed, losses.ctypes.data),
                  "vec_closure_train")
        return losses[:iters]

    def evaluate(self, first, count):
        a, b = C.c_double(), C.c_double()
        self._chk(self.L.vec_closure_eval(self.h, first, count, C.byref(a), C.byref(b)), "vec_closure_eval")
        return a.value, b.value

    def attach(self, coarse, on=True):
        self._chk(self.L.vec_closure_attach(self.h, coarse.h, 1 if on else 0), "vec_closure_attach")

    def infer(self, coarse):
        self._chk(self.L.vec_closure_infer(self.h, coarse.h), "vec_closure_infer")

    def step(self, coarse, n=1):
        return self.L.vec_closure_step(self.h, coarse.h, n)

    def run(self, coarse, fine, t_end, every, nfine, tol):
        rep = VecClosureReport()
        self._chk(self.L.vec_closure_run(self.h, coarse.h, fine.h, t_end, every, nfine, tol, C.byref(rep)),
                  "vec_closure_run")
        return {"judges": rep.judges, "coarse_steps": rep.coarse_steps, "fine_steps": rep.fine_steps,
                "fallback_step": rep.fallback_step, "last_err": list(rep.last_err), "max_err": list(rep.max_err),
                "end_time": rep.end_time}


def expand(coarse, fine, f):
    """The reference's expand of one field (coarse (nz, ny, nx) -> fine)."""
    L = _L.load()
    f = np.ascontiguousarray(f, np.float64)
    out = np.empty(fine.shape, np.float64)
    st = L.vec_expand(coarse.h, fine.h, f.ctypes.data, out.ctypes.data)
    if st != 0:
        raise VecError("vec_expand", st)
    return out


def upsample(coarse, fine):
    L = _L.load()
    st = L.vec_upsample(coarse.h, fine.h)
    if st != 0:
        raise VecError("vec_upsample", st)
