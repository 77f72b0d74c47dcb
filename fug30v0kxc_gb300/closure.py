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

    def launch_count(self):
        return int(self.L.vec_net_launch_count(self.h))

    def time(self, reps=10):
        """(ms per forward, ms per training step, flops per forward, flops per
        training step) on the current batch buffers."""
        a, b = C.c_float(), C.c_float()
        fa, fb = C.c_double(), C.c_double()
        self._chk(self.L.vec_net_time(self.h, reps, C.byref(a), C.byref(b), C.byref(fa), C.byref(fb)),
                  "vec_net_time")
        return a.value, b.value, fa.value, fb.value


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

    def set_output(self, clip=4.0, gain=1.0):
        self._chk(self.L.vec_closure_set_output(self.h, clip, gain), "vec_closure_set_output")

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

    def run(self, coarse, fine, t_end, every, nfine, tol, diag_every=0, cap=0):
        """The judged run; with diag_every > 0 the report holds a series of
        rows (time, Nu, kinetic energy, magnetic energy, top Nu)."""
        rep = VecClosureReport()
        series = np.zeros((max(cap, 1), 5))
        self._chk(self.L.vec_closure_run(self.h, coarse.h, fine.h, t_end, every, nfine, tol, diag_every,
                                         series.ctypes.data, cap, C.byref(rep)), "vec_closure_run")
        return {"judges": rep.judges, "coarse_steps": rep.coarse_steps, "fine_steps": rep.fine_steps,
                "fallback_step": rep.fallback_step, "last_err": list(rep.last_err), "max_err": list(rep.max_err),
                "end_time": rep.end_time, "divb_fail": rep.divb_fail, "blowup": rep.blowup,
                "series": series[:rep.nseries].copy()}


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


def top_nusselt(g):
    """Nusselt number at the fixed-temperature top of a solver."""
    L = _L.load()
    v = C.c_double()
    st = L.vec_top_nusselt(g.h, C.byref(v))
    if st != 0:
        raise VecError("vec_top_nusselt", st)
    return v.value


def _tavg(series, col):
    """Time average (trapezoid rule) of one column of the rows (t, ...)."""
    s = np.asarray(series, dtype=np.float64)
    if len(s) < 2:
        return float(s[0, col]) if len(s) else float("nan")
    t, v = s[:, 0], s[:, col]
    return float(np.sum(0.5 * (v[1:] + v[:-1]) * np.diff(t)) / (t[-1] - t[0]))


def advance_to(g, t_end, chunk=100):
    """Step a solver until its time reaches t_end; returns False (and stops)
    if the time stops advancing by finite steps not below 1e-3 of the first."""
    s = g.scalars()
    dt0 = s.dt
    while s.ttime < t_end:
        if g.step(chunk) != 0:
            return False
        s2 = g.scalars()
        if not (np.isfinite(s2.ttime) and np.isfinite(s2.dt)) or s2.ttime <= s.ttime or s2.dt < 1e-3 * dt0:
            return False
        s = s2
    return True


def _row(g):
    st, d = g.diag()
    return [g.scalars().ttime, d["nusselt"], d["kenergy"], d["menergy"], top_nusselt(g)], st


def run_workload(nxf=512, nyf=512, nzf=257, factor=4, ra=1.0e6, q=1.0e3, eta=20.0, noise=0.05, pre_time=1.5,
                 spinup=2000, pairs=2000, pair_every=4, iters=2000, batch=8, lr=1e-3, window=8000, diag_every=100,
                 judge_every=2000, nfine=50, tol=0.03, seed=0, log=None):
    """The learned-closure workload.  Convection develops on the coarse grid
    (the plain solver from the seeded noise state to time pre_time), is
    upsampled to the fine grid (the reference's interpolate step) and spun up
    for `spinup` fine steps; then box-filtered training pairs from the
    split-form DNS and training; then, over `window` DNS steps, the filtered
    DNS statistics against the judged closure run and the plain coarse run
    (same physical time).  Statistics: time averages of the top Nusselt
    number and the kinetic and magnetic energies (the reference's bottom
    Nusselt number is identically one with a fixed-flux bottom).  Returns a
    dict of relative errors and wall times (seconds, runs synchronised)."""
    import time
    from .params import VEC_PREC_SPLIT, convection_params
    from .solver import P3D

    def say(*a):
        if log:
            log(" ".join(str(x) for x in a))

    def params(nx, ny, nz):
        p = convection_params(nx, ny, nz, ra=ra, q=q, eta_contrast=eta, noise=noise, precision=VEC_PREC_SPLIT)
        p.ndu06 = 10 ** 9
        return p

    pf, pc = params(nxf, nyf, nzf), params(nxf // factor, nyf // factor, (nzf - 1) // factor + 1)
    res = {"fine": [nxf, nyf, nzf], "coarse": [pc.nx, pc.ny, pc.nz], "ra": ra, "q": q, "eta_contrast": eta}
    C0 = P3D(pc)
    C0.start()
    t0 = time.perf_counter()
    ok = advance_to(C0, pre_time)
    res["pre_s"] = time.perf_counter() - t0
    res["pre_ok"] = ok
    res["pre_steps"] = C0.scalars().iter
    r0, _ = _row(C0)
    res["pre_nutop"], res["pre_kenergy"] = r0[4], r0[2]
    say("coarse pre-run to t =", pre_time, "ok" if ok else "STOPPED", res["pre_steps"], "steps",
        round(res["pre_s"], 1), "s, top Nu", r0[4], "KE", r0[2])
    if not ok:
        C0.close()
        res["error"] = "the coarse pre-run stopped advancing"
        return res
    F = P3D(pf)
    upsample(C0, F)
    C0.close()
    t0 = time.perf_counter()
    assert F.step(spinup) == 0
    F.sync()
    res["spinup_s"] = time.perf_counter() - t0
    r0, _ = _row(F)
    res["spinup_nutop"], res["spinup_kenergy"] = r0[4], r0[2]
    say("DNS spin-up", spinup, "steps", round(res["spinup_s"], 1), "s, top Nu", r0[4], "KE", r0[2])
    cl = Closure(pc, factor=factor, capacity=pairs, batch=batch, seed=seed)
    S = P3D(pc)
    t0 = time.perf_counter()
    for _ in range(pairs):
        cl.add_pair(F, S)
        assert F.step(pair_every) == 0
    F.sync()
    res["pairs_s"] = time.perf_counter() - t0
    say("pairs", pairs, round(res["pairs_s"], 1), "s")
    ntrain = max(1, int(0.9 * pairs))
    cl.fit_norm(pairs)
    t0 = time.perf_counter()
    losses = cl.train(iters, lr=lr, ntrain=ntrain, seed=seed + 1)
    res["train_s"] = time.perf_counter() - t0
    res["loss_first"] = float(np.mean(losses[:10]))
    res["loss_last"] = float(np.mean(losses[-10:]))
    mse_net, mse_zero = cl.evaluate(ntrain, pairs - ntrain) if pairs > ntrain else cl.evaluate(0, pairs)
    res["apriori_mse_net"], res["apriori_mse_zero"] = mse_net, mse_zero
    ms_f, ms_t, fl_f, fl_t = cl.net.time(10)
    res["net_ms_fwd_batch"], res["net_ms_train_step"] = ms_f, ms_t
    res["net_tflops_fwd"], res["net_tflops_train"] = fl_f / ms_f * 1e-9, fl_t / ms_t * 1e-9
    say("trained", iters, "iterations", round(res["train_s"], 1), "s; a-priori mse", mse_net, "vs", mse_zero,
        "; network", round(res["net_tflops_train"], 1), "TFLOP/s")

    # the window: the coarse runs start from the filtered DNS state
    sc = F.scalars()
    C1, C2 = P3D(pc), P3D(pc)
    for c in (C1, C2):
        cl.box_filter(F, c)
        s = c.scalars()
        s.ttime = sc.ttime
        s.first, s.second = 1, 0
        c.set_scalars(s)
        c.calcdt()
    tstart = sc.ttime

    def filtered_row():
        # (t, Nu, KE, ME, top Nu) of the filtered state, then the DNS's own
        # top Nusselt number (the plane-averaged wall flux, which the
        # horizontal part of the filter leaves unchanged; the 3-D box filter
        # also averages four fine levels next to the wall, which biases the
        # wall-normal gradient of the filtered state)
        cl.box_filter(F, S)
        s = S.scalars()
        s.ttime = F.scalars().ttime
        S.set_scalars(s)
        return _row(S)[0] + [top_nusselt(F)]

    dns = [filtered_row()]
    tdns = 0.0
    dt0 = F.scalars().dt
    res["dns_blowup"] = 0
    nstep = 0
    for _ in range(0, window, diag_every):
        F.sync()
        t0 = time.perf_counter()
        st = F.step(diag_every)
        F.sync()
        tchunk = time.perf_counter() - t0
        s = F.scalars()
        # the window ends where the DNS stops advancing by finite steps not
        # below 1e-3 of its first (an unstable DNS)
        if st != 0 or not (np.isfinite(s.ttime) and np.isfinite(s.dt)) or s.ttime <= dns[-1][0] \
                or s.dt < 1e-3 * dt0:
            res["dns_blowup"] = 1
            break
        tdns += tchunk
        nstep += diag_every
        dns.append(filtered_row())
    tend = dns[-1][0]
    res["window_time"] = tend - tstart
    res["dns_steps"] = nstep
    res["dns_s"] = tdns
    say("DNS window", nstep, "steps", round(tdns, 1), "s, model time", tend - tstart,
        "(stopped: the DNS stopped advancing)" if res["dns_blowup"] else "")
    if nstep == 0:
        res["error"] = "the DNS stopped advancing at the start of the window"
        for o in (F, S, C1, C2):
            o.close()
        cl.close()
        return res
    F2 = P3D(pf)
    r1, st1 = _row(C1)
    res["coarse_initial_divb_status"] = st1
    t0 = time.perf_counter()
    rep = cl.run(C1, F2, tend, every=judge_every, nfine=nfine, tol=tol, diag_every=max(1, diag_every // factor),
                 cap=200000)
    res["closure_s"] = time.perf_counter() - t0
    rows = [r1] + rep["series"].tolist()
    res["judge"] = {k: rep[k] for k in ("judges", "coarse_steps", "fine_steps", "fallback_step", "max_err",
                                        "divb_fail", "blowup")}
    say("closure run", rep["coarse_steps"], "coarse steps", rep["fine_steps"], "fine steps",
        round(res["closure_s"], 1), "s", res["judge"])
    r2, _ = _row(C2)
    plain = [r2]
    t0 = time.perf_counter()
    n, divb_plain = 0, 0
    s0 = C2.scalars()
    dt0, tp = s0.dt, s0.ttime
    res["plain_blowup"] = 0
    while True:
        s = C2.scalars()
        if s.ttime >= tend:
            break
        # the judged run's progress test: finite time advancing by steps not
        # below 1e-3 of the first, within 100 x the steps the first implies
        if (not (np.isfinite(s.ttime) and np.isfinite(s.dt)) or (n > 0 and s.ttime <= tp)
                or s.dt < 1e-3 * dt0 or n > 100 * (tend - tstart) / dt0 + 1000):
            res["plain_blowup"] = 1
            break
        tp = s.ttime
        if C2.step(1) != 0:
            res["plain_blowup"] = 1
            break
        n += 1
        if n % max(1, diag_every // factor) == 0:
            r, st = _row(C2)
            divb_plain += int(st == -12)
            plain.append(r)
    res["plain_s"] = time.perf_counter() - t0
    res["plain_steps"] = n
    res["plain_divb_fail_samples"] = divb_plain
    say("plain coarse run", n, "steps", round(res["plain_s"], 1), "s, blow-up", res["plain_blowup"])
    names = ("nusselt", "kenergy", "menergy", "nusselt_top")
    res["dns"] = {nm: _tavg(dns, j + 1) for j, nm in enumerate(names)}
    res["dns"]["nusselt_top_dns"] = _tavg(dns, 5)
    res["dns"]["nusselt_top_dns_first"], res["dns"]["nusselt_top_filtered_first"] = dns[0][5], dns[0][4]
    for tag, ser in (("closure", rows), ("plain", plain)):
        res[tag] = {}
        for j, nm in enumerate(names):
            a, b = _tavg(ser, j + 1), res["dns"][nm]
            res[tag][nm] = a
            res[tag][nm + "_err"] = abs(a - b) / max(abs(b), 1e-300)
        b = res["dns"]["nusselt_top_dns"]
        res[tag]["nusselt_top_dns_err"] = abs(res[tag]["nusselt_top"] - b) / max(abs(b), 1e-300)
        res[tag]["max_err"] = max(res[tag][nm + "_err"] for nm in ("kenergy", "menergy", "nusselt_top"))
        res[tag]["max_err_dns_wall_flux"] = max(res[tag][nm] for nm in ("kenergy_err", "menergy_err",
                                                                        "nusselt_top_dns_err"))
    res["speedup_vs_dns"] = tdns / res["closure_s"] if res["closure_s"] > 0 else None
    for o in (F, F2, S, C1, C2):
        o.close()
    cl.close()
    return res
