"""Benchmark: grid-point-steps/s of the VarElecCond time step on one GB300.

Workload: 256 x 256 x 129, Ra 1e5, Q 100, m=1, theta 9 (density contrast
10), gamma 1.4, zeta 0.2, fixed-flux bottom, vertical seed field, eta(z)
contrast 20, seeded +-1e-3 temperature noise (synthetic state), SF 0.3.
One step = one iteration of the time loop (src/main.F90:340-747): RHS,
AB3 update, dealias every 10 steps, bandj, boundary conditions, calcdt
every 10 steps.  The state (>1 GB) is far larger than L2, so no explicit
L2 flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  Under torchrun every rank runs an independent
replica (the path does not shard: replicas only); rank 0 prints.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NX, NY, NZ = 256, 256, 129
WORKLOAD = "VarElecCond 256x256x129 Ra1e5 Q100 eta-contrast-20"
METRIC = "grid-point-steps/s at 256^2x129"
LARGE = {"on": False}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.lines = []
        self.gpu = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def make_params(precision):
    from fug30v0kxc_gb300.params import config1, config4
    p = (config4 if LARGE["on"] else config1)(precision=precision)
    p.nx, p.ny, p.nz = NX, NY, NZ
    p.ndu06 = 1000000          # diagnostics printing cadence of bin/INPUT is 5000 steps
    return p


def time_gpu(args, precision):
    """Device-resident timed region: W warmup steps, then K timed steps
    replayed from the step's CUDA graph with nothing else on the streams.

    The per-kernel durations come from a second pass of K steps right after
    it, with a CUDA event pair around every launch on the stream it is
    launched on (this pass runs eagerly and runs the magnetic branch on the
    library stream after the hydro branch, so no two timed kernels overlap).
    """
    import torch
    from fug30v0kxc_gb300.solver import P3D
    g = P3D(make_params(precision))
    g.start()
    stream = torch.cuda.ExternalStream(g.stream())
    st = g.step(args.warmup)
    assert st == 0, f"warmup step failed: {st}"
    g.sync()
    launches0 = g.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(torch.cuda.current_device())
    clk.start()
    ev0.record(stream)
    st = g.step(args.steps)
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    assert st == 0, f"timed step failed: {st}"
    ms = ev0.elapsed_time(ev1)
    launches = g.launch_count() - launches0
    ms = reduce_max(ms)
    # per-kernel pass
    g.profile(True)
    g.profile_reset()
    st = g.step(args.steps)
    assert st == 0, f"profiled step failed: {st}"
    prof = g.profile_records()
    g.profile(False)
    return g, ms, launches, prof, clocks


def time_e2e(g, args):
    """Through the C-ABI with host buffers: upload the state from pinned host
    memory, K calls of vec_step(1) each reading the step's scalars back, then
    download the state; every copy is inside the timed region.  Returns the
    total time, the copied bytes, the scalars' bytes per step and the three
    phases' times."""
    import numpy as np
    import torch
    from fug30v0kxc_gb300.params import FIELD_NAMES, VecScalars
    names = ("r", "t", "u", "v", "w", "bx", "by", "bz", "pol", "tor")
    host = {}
    for n in names:
        a = torch.empty(g.shape, dtype=torch.float64, pin_memory=True).numpy()
        a[...] = g.get(n)
        host[n] = a
    sc = VecScalars()
    L = g.L
    # one untimed round trip through the fresh pinned buffers (their first
    # DMA use pays a one-time mapping cost that is not part of a step)
    for n in names:
        assert L.vec_set_field(g.h, FIELD_NAMES[n], host[n].ctypes.data) == 0
    for n in names:
        assert L.vec_get_field(g.h, FIELD_NAMES[n], host[n].ctypes.data) == 0
    # the timed region three times (each a full upload, K steps and download);
    # the median is reported, all three totals are listed
    runs = []
    for _ in range(3):
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for n in names:
            assert L.vec_set_field(g.h, FIELD_NAMES[n], host[n].ctypes.data) == 0
        t1 = time.perf_counter()
        for _ in range(args.steps):
            assert L.vec_step(g.h, 1) == 0
            assert L.vec_get_scalars(g.h, C.byref(sc)) == 0
        t2 = time.perf_counter()
        for n in names:
            assert L.vec_get_field(g.h, FIELD_NAMES[n], host[n].ctypes.data) == 0
        t3 = time.perf_counter()
        runs.append((reduce_max((t3 - t0) * 1e3) / 1e3, t1 - t0, t2 - t1, t3 - t2))
    runs.sort(key=lambda r: r[0])
    dt, up, st, down = runs[1]
    nbytes = sum(host[n].nbytes for n in names)
    phases = {"upload_ms": round(up * 1e3, 2), "steps_ms": round(st * 1e3, 2), "download_ms": round(down * 1e3, 2),
              "repetitions_ms": [round(r[0] * 1e3, 2) for r in runs], "statistic": "median of 3"}
    return dt, nbytes, C.sizeof(VecScalars), phases


def time_ensemble(args):
    """The 48-member ensemble (16 x 64^2x65, 16 x 128^2x97, 16 x 192^2x129,
    split form) stepped as one captured graph after the autotuner picked the
    tile shapes per grid.  Aggregate grid-point-steps/s over all members."""
    import torch
    from fug30v0kxc_gb300.params import config2_members
    from fug30v0kxc_gb300.solver import Ensemble
    ps = config2_members()
    npts = sum(p.nx * p.ny * p.nz for p in ps)
    ens = Ensemble(ps)
    ens.start()
    t0 = time.perf_counter()
    ens.tune(steps=3)
    tune_s = time.perf_counter() - t0
    assert ens.step(args.warmup) == 0
    ens.sync()
    m0 = ens.members[0]
    stream = torch.cuda.ExternalStream(m0.stream())
    launches0 = sum(m.launch_count() for m in ens.members)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(torch.cuda.current_device())
    clk.start()
    # the ensemble step joins every member stream into its root stream
    # first and forks back at the end, so events on member 0's stream
    # bracket all members' work
    ev0.record(stream)
    st = ens.step(args.steps)
    ev1.record(stream)
    ens.sync()
    torch.cuda.synchronize()
    clocks = clk.stop()
    assert st == 0, f"ensemble step failed: {st}"
    ms = reduce_max(ev0.elapsed_time(ev1))
    launches = sum(m.launch_count() for m in ens.members) - launches0
    tun = sorted({(m.p.nx, m.p.nz) + tuple(m.tunables()) for m in ens.members})
    ens.close()
    return npts, ms, launches, clocks, tune_s, tun


def ensemble_line(args, ws, hbm, pk):
    npts, ms, launches, clocks, tune_s, tun = time_ensemble(args)
    value = npts * args.steps * ws / (ms * 1e-3)
    alg = 196
    return {"value": value, "unit": "grid-point-steps/s", "ms_per_step": ms / args.steps,
            "members": 48, "points": npts, "gpu_launches": launches, "clocks": clocks,
            "step_roofline": {"alg_bytes_per_gps": alg, "achieved_gbs": round(value / ws * alg / 1e9, 1),
                              "peak": hbm, "frac": round(value / ws * alg / 1e9 / hbm, 4), "peak_kind": pk},
            "autotune_s": round(tune_s, 2),
            "tunables": [{"n": t[0], "nz": t[1], "kc": t[2], "s": t[3]} for t in tun]}


def closure_line(args, ws):
    """The learned closure against the filtered DNS (Ra 1e6, Q 1e3, eta
    contrast 20, split form): errors of the time-averaged top Nusselt number
    and energies of the judged closure run and of the plain coarse run, and
    the wall time of the closure run against the DNS over the same time."""
    from fug30v0kxc_gb300.closure import run_workload
    if args.closure_scale == "full":
        kw = dict(nxf=512, nyf=512, nzf=257, pre_time=args.closure_pre_time, spinup=2000, pairs=2000,
                  pair_every=4, iters=2000, window=40000, diag_every=100, judge_every=args.closure_judge_every,
                  nfine=50)
    else:
        kw = dict(nxf=256, nyf=256, nzf=129, pre_time=args.closure_pre_time, spinup=1000, pairs=200, pair_every=4,
                  iters=500, window=2000, diag_every=50, judge_every=min(args.closure_judge_every, 100), nfine=50)
    if args.closure_window > 0:
        kw["window"] = args.closure_window
    r = run_workload(log=lambda m: print("#", m, file=sys.stderr, flush=True), **kw)
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak, pk = float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        peak, pk = 1900.0, "fallback"
    ach = r.get("net_tflops_train")
    value = r["closure"]["max_err"] if "closure" in r else None
    # the DNS wall time is the time of the steps it completed
    return {"metric": "closure: max relative error of the time-averaged top Nusselt number, kinetic and "
                      "magnetic energy vs the filtered DNS",
            "value": value, "unit": "fraction", "n_gpus": ws,
            "steps": r.get("judge", {}).get("coarse_steps"), "warmup": 0, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16 network / f32-f64 solver",
            "data": "synthetic (seeded static polytrope + uniform +-0.05 T noise, developed on the coarse grid, "
                    "upsampled, spun up)",
            "config": {"workload": "closure %dx%dx%d DNS -> %dx%dx%d, Ra 1e6, Q 1e3, eta contrast 20"
                                   % tuple(r["fine"] + r["coarse"]), **kw},
            "roofline": {"bound": "tensor", "kernel": "closure network training step (BF16: forward and input gradient on "
                                   "tcgen05 at nx = 128, weight gradient on mma.sync)",
                         "achieved": round(ach, 2) if ach else None, "peak": peak, "peak_kind": pk, "unit": "TFLOP/s",
                         "frac": round(ach / peak, 4) if ach else None, "traffic": None},
            "closure": r}


def net_line(args, ws):
    """The closure network alone: forward pass and training step (forward,
    input and weight gradients, Adam) on a seeded synthetic batch of 8 at
    the coarse grid of the closure workload (128^2x65; --grid overrides),
    CUDA events on the network's stream."""
    import numpy as np
    from fug30v0kxc_gb300.closure import Net
    nx, ny, nz = (int(v) for v in args.grid.split(",")) if args.grid else (128, 128, 65)
    nb = 8
    net = Net(nx, ny, nz, nb, seed=1)
    rng = np.random.default_rng(0)
    x = np.zeros((nb, nz, ny, nx, 16), np.float32)
    x[..., :9] = rng.standard_normal((nb, nz, ny, nx, 9))
    net.forward(x)
    net.backward(rng.standard_normal((nb, nz, ny, nx, 8)).astype(np.float32))
    net.time(args.warmup)
    l0 = net.launch_count()
    ms_f, ms_t, fl_f, fl_t = net.time(args.steps)
    launches = net.launch_count() - l0
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak, pk = float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        peak, pk = 1900.0, "fallback"
    ach = fl_t / ms_t * 1e-9
    pts = nb * nx * ny * nz
    net.close()
    return {"metric": "closure network training steps/s (batch 8)", "value": 1e3 / ms_t, "unit": "steps/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_t, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (fp32 accumulate)",
            "data": "synthetic (seeded normal inputs and targets)",
            "config": {"workload": "closure network 4x Conv3d 3x3x3, 16-32-32-32-16 channels, batch 8, %dx%dx%d"
                                   % (nx, ny, nz), "points_per_batch": pts,
                       "l2": "no flush: one activation buffer is %.2f GB" % (pts * 2 * 32 / 1e9)},
            "roofline": {"bound": "tensor", "kernel": "training step (conv forward, input and weight gradients)",
                         "achieved": round(ach, 2), "peak": peak, "peak_kind": pk, "unit": "TFLOP/s",
                         "frac": round(ach / peak, 4), "traffic": None},
            "forward": {"ms": ms_f, "tflops": fl_f / ms_f * 1e-9, "frac": fl_f / ms_f * 1e-9 / peak},
            "gpu_launches": launches}


def accuracy_line(args, ws):
    """The split form's accuracy at 256^2x129 (eta contrast 20) against the
    FP64 form, the drop-in whose every kernel is parity-checked against the
    oracle: both start from the same seeded static state and run the time
    loop with diagnostics every --acc-every steps (GlobalAverages, nusselt,
    checkdivb at their reference cadence, src/main.F90:552-647).

    Reported: per-field relative L2 of the split state against the FP64
    state after 100 steps (r and T as deviations from the static polytrope),
    and the time averages over the second half of the run of the top
    Nusselt number (the fixed-flux bottom makes the reference's bottom one
    identically 1), the kinetic energy, the magnetic energy and the energy
    of the field perturbation, with their relative differences."""
    import numpy as np
    from fug30v0kxc_gb300.params import VEC_PREC_FP64, VEC_PREC_SPLIT, config1
    from fug30v0kxc_gb300.solver import P3D
    total, every = args.acc_steps, args.acc_every
    runs = {}
    for name, prec in (("split", VEC_PREC_SPLIT), ("fp64", VEC_PREC_FP64)):
        p = config1(precision=prec)
        p.ndu06 = every
        g = P3D(p)
        g.start()
        t0 = time.perf_counter()
        assert g.step(100) == 0
        z = np.arange(p.nz) / (p.nz - 1)
        bg = (1.0 + p.theta * z)[:, None, None]
        s100 = {n: g.get(n) - (bg ** p.cm if n == "r" else bg if n == "t" else 0.0)
                for n in ("r", "t", "u", "v", "w", "pol", "tor")}
        rows = []
        done = 100
        while done < total:
            n = every - done % every
            st = g.step(n)
            assert st == 0, f"{name}: step status {st} at {done + n}"
            done += n
            d = g.last_diag()
            bx, by, bz = g.get("bx"), g.get("by"), g.get("bz")
            e = (bx * bx + by * by + (bz - g.bzbar) ** 2).sum(axis=(1, 2))
            e[0] *= 0.5
            e[-1] *= 0.5
            mep = p.f * 0.5 * e.sum() * (p.xmax / p.nx) * (p.ymax / p.ny) / (p.nz - 1)
            rows.append((done, g.scalars().ttime, g.top_nusselt(), d["kenergy"], d["menergy"], mep, d["nusselt"]))
        g.sync()
        runs[name] = {"s100": s100, "rows": np.array(rows), "wall_s": time.perf_counter() - t0}
        g.close()
    rel_l2 = {n: float(np.linalg.norm((runs["split"]["s100"][n] - runs["fp64"]["s100"][n]).ravel())
                       / max(np.linalg.norm(runs["fp64"]["s100"][n].ravel()), 1e-300))
              for n in runs["fp64"]["s100"]}
    half = total // 2
    avgs = {}
    for name in runs:
        r = runs[name]["rows"]
        sel = r[r[:, 0] > half]
        avgs[name] = {"nusselt_top": float(sel[:, 2].mean()), "kenergy": float(sel[:, 3].mean()),
                      "menergy": float(sel[:, 4].mean()), "menergy_perturbation": float(sel[:, 5].mean()),
                      "nusselt_bottom": float(sel[:, 6].mean()), "samples": int(len(sel)),
                      "model_time": [float(sel[0, 1]), float(sel[-1, 1])]}
    diffs = {k: abs(avgs["split"][k] - avgs["fp64"][k]) / max(abs(avgs["fp64"][k]), 1e-300)
             for k in ("nusselt_top", "kenergy", "menergy", "menergy_perturbation")}
    series = {name: [[float(x) for x in row[:6]] for row in runs[name]["rows"][:: max(1, len(runs[name]["rows"]) // 20)]]
              for name in runs}
    value = max(diffs.values())
    return {"metric": "split vs FP64 at 256^2x129: max relative difference of the time-averaged top Nusselt "
                      "number, kinetic, magnetic and perturbation magnetic energy over the second half of the run",
            "value": value, "unit": "fraction", "n_gpus": ws, "steps": total, "warmup": 0,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64 vs f64",
            "data": "synthetic (seeded static polytrope + uniform +-1e-3 T noise)",
            "config": {"workload": WORKLOAD + " accuracy", "nx": NX, "ny": NY, "nz": NZ, "steps": total,
                       "diag_every": every, "average_over_steps": [half, total]},
            "within_1pct": bool(value <= 0.01),
            "rel_l2_after_100_steps": rel_l2, "time_averages": avgs, "relative_differences": diffs,
            "wall_s": {k: round(v["wall_s"], 1) for k, v in runs.items()},
            "series_columns": ["step", "time", "nusselt_top", "kenergy", "menergy", "menergy_perturbation"],
            "series": series}


def cpu_baseline(nsteps, precision_note=""):
    """The oracle (plain C restatement, OpenMP over planes) on the host cores."""
    from oracle import oracle as O
    threads = O.nthreads(os.cpu_count() or 1)
    o = O.Oracle(make_params(0))
    o.start()
    o.step(1)
    t0 = time.perf_counter()
    assert o.step(nsteps) == 0
    dt = time.perf_counter() - t0
    return NX * NY * NZ * nsteps / dt, threads, dt


_dist = {"on": False}


def barrier():
    if _dist["on"]:
        import torch.distributed as dist
        dist.barrier()


def reduce_max(x):
    if not _dist["on"]:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dominant_roofline(prof, hbm_peak, peak_kind):
    """Dominant kernel = largest share of the timed region's device time.
    achieved = its algorithmic bytes per launch (every field it must read or
    write, once; recorded per launch by the library) / its mean launch time
    measured with CUDA events on the library stream."""
    total = sum(r[2] for r in prof) or 1.0
    name, launches, ms, nbytes = max(prof, key=lambda r: r[2])
    avg_ms = ms / launches
    per_launch = nbytes / launches
    achieved = per_launch / (avg_ms * 1e-3) / 1e9
    return {"kernel": name, "bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak,
            "unit": "GB/s", "frac": round(achieved / hbm_peak, 4), "peak_kind": peak_kind,
            "traffic": TRAFFIC.get(name), "share": round(ms / total, 4),
            "avg_launch_ms": round(avg_ms, 4), "launches": launches,
            "alg_bytes_per_launch": per_launch}


# dram__bytes_read.sum + dram__bytes_write.sum per launch of the split step's
# kernels, from one-kernel ncu captures at 256x256x65 scaled by the points to
# 256x256x129 (profiles/dram_traffic_split_256x256x65.md; the line kernels'
# figures are the mean over a step's three launches); other workloads: null
_SCALE_129_65 = 129.0 / 65.0
TRAFFIC_256x256x129 = {k: v * _SCALE_129_65 for k, v in {
    "ab3_update_split": 900.9e6, "hydro_pass2_f32": 667.2e6, "hydro_pass4_f32": 344.8e6,
    "mag_final_f32": 119.5e6, "line_x_f32": (294.2e6 + 55.6e6 + 145.5e6) / 3,
    "line_y_f32": (279.2e6 + 53.3e6 + 139.6e6) / 3}.items()}
TRAFFIC = {}
# operation count of one grid-point-step at n = 256 (formula: ~72 real
# transform passes x 2.5 log2 n, ~200 for the z stencils, ~300 pointwise,
# ~40 for AB3) and GB300's nominal FP64 rate
FP64_FLOP_PER_GPS_256 = 1.9e3
FP64_NOMINAL_TFLOPS = 1.25


def fp64_peak():
    """The FP64 FMA rate measured on this GPU (DFMA chains timed with CUDA
    events, vec_measure_fp64), or the nominal rate if that fails."""
    from fug30v0kxc_gb300 import lib
    v = C.c_double()
    if lib.load().vec_measure_fp64(5, C.byref(v)) == 0 and v.value > 0:
        return v.value, "measured (DFMA microbenchmark)"
    return FP64_NOMINAL_TFLOPS, "nominal"


def run_reference(args):
    """--impl reference: the reference's CPU path.  The Fortran reference
    cannot be built here (no Fortran compiler, MPI, FFTW 2 or netCDF), so
    this times the oracle port of its serial path on all host cores."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    threads = O.nthreads(os.cpu_count() or 1)
    o = O.Oracle(make_params(0))
    o.start()
    assert o.step(args.warmup) == 0
    t0 = time.perf_counter()
    assert o.step(args.steps) == 0
    dt = time.perf_counter() - t0
    v = NX * NY * NZ * args.steps / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "grid-point-steps/s",
            "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded static polytrope + noise)",
            "config": {"workload": WORKLOAD, "nx": NX, "ny": NY, "nz": NZ, "precision": "fp64",
                       "l2": "state >1 GB, larger than L2"},
            "cpu_baseline": {"value": v, "unit": "grid-point-steps/s", "cores": threads,
                             "kind": "port",
                             "sample": f"{args.steps} steps of the full 256x256x129 workload after "
                                       f"{args.warmup} warm-up steps (reference Fortran unbuildable: "
                                       "oracle port of its serial path)"},
            "e2e": {"value": v, "unit": "grid-point-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def measure(args, precision, ws, hbm, pk, with_e2e):
    g, ms, launches, prof, clocks = time_gpu(args, precision)
    npts = NX * NY * NZ
    value = npts * args.steps * ws / (ms * 1e-3)
    res = {"value": value, "ms_per_step": ms / args.steps, "launches": launches, "clocks": clocks,
           "roofline": dominant_roofline(prof, hbm, pk)}
    alg_step = 280 if precision == 0 else 196
    res["step_roofline"] = {"alg_bytes_per_gps": alg_step,
                            "achieved_gbs": round(value / ws * alg_step / 1e9, 1),
                            "frac": round(value / ws * alg_step / 1e9 / hbm, 4)}
    total_ms = sum(r[2] for r in prof) or 1.0
    # the kernels' own time per step (profiled pass) beside the replayed step
    # time: the difference is launch gaps and ramp-up/drain between kernels
    res["kernel_ms_per_step"] = round(total_ms / args.steps, 4)
    res["kernels"] = sorted(({"kernel": n, "launches": l, "ms": round(m, 3), "share": round(m / total_ms, 4),
                              "gbs": round(b / (m * 1e-3) / 1e9, 1) if m > 0 else None}
                             for n, l, m, b in prof), key=lambda d: -d["ms"])[:12]
    if with_e2e:
        e2e_s, e2e_bytes, sc_bytes, phases = time_e2e(g, args)
        res["e2e"] = {"value": npts * args.steps * ws / e2e_s, "unit": "grid-point-steps/s",
                      "h2d_bytes_per_step": e2e_bytes / args.steps,
                      "d2h_bytes_per_step": e2e_bytes / args.steps + sc_bytes, **phases}
    g.close()
    return res


def main():
    global NX, NY, NZ, WORKLOAD, METRIC
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="both", choices=["both", "fp64", "split"])
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--grid", default=None, help="NX,NY,NZ (smaller cases for ncu captures)")
    ap.add_argument("--closure-scale", default="full", choices=["full", "small"],
                    help="closure workload: full = DNS 512^2x257 -> 128^2x65, 2000 pairs; small = 256^2x129 "
                         "-> 64^2x33, 200 pairs")
    ap.add_argument("--closure-pre-time", type=float, default=1.5,
                    help="closure workload: model time the coarse solver develops convection before the DNS")
    ap.add_argument("--closure-window", type=int, default=0,
                    help="closure workload: DNS steps of the comparison window (0: 40000 full, which holds the "
                         "judge after 2000 coarse steps; 2000 small)")
    ap.add_argument("--closure-judge-every", type=int, default=2000,
                    help="closure workload: coarse steps between judged fine segments")
    ap.add_argument("--acc-steps", type=int, default=20000, help="accuracy workload: steps of each run")
    ap.add_argument("--acc-every", type=int, default=100, help="accuracy workload: diagnostics cadence")
    ap.add_argument("--workload", default="single",
                    choices=["single", "ensemble", "large", "closure", "net", "accuracy"],
                    help="ensemble: the 48-member batched ensemble as the headline line; "
                         "large: one 1024^2x513 instance, Ra 1e7, Q 1e4, eta contrast 50 (split); "
                         "accuracy: split against FP64 at 256^2x129 over --acc-steps steps")
    ap.add_argument("--no-e2e", action="store_true",
                    help="skip the host-buffer measurement (very large grids)")
    ap.add_argument("--no-ensemble", action="store_true",
                    help="skip the ensemble sub-measurement of the single-instance line")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.grid:
        NX, NY, NZ = (int(x) for x in args.grid.split(","))
        WORKLOAD = f"VarElecCond {NX}x{NY}x{NZ} Ra1e5 Q100 eta-contrast-20"
        METRIC = f"grid-point-steps/s at {NX}x{NY}x{NZ}"

    if (NX, NY, NZ) == (256, 256, 129) and args.workload == "single":
        TRAFFIC.update(TRAFFIC_256x256x129)
    if args.workload == "large":
        LARGE["on"] = True
        NX, NY, NZ = 1024, 1024, 513
        WORKLOAD = "VarElecCond 1024x1024x513 Ra1e7 Q1e4 eta-contrast-50 theta19"
        METRIC = "grid-point-steps/s at 1024^2x513"
        args.precision, args.no_e2e, args.no_ensemble, args.no_cpu = "split", True, True, True
    ws, rank, local = dist_env()
    if ws > 1:
        import torch
        import torch.distributed as dist
        if args.impl == "ours":
            torch.cuda.set_device(local)
        dist.init_process_group(backend="nccl" if args.impl == "ours" else "gloo")
        _dist["on"] = True
    if args.impl == "reference":
        run_reference(args)
        if _dist["on"]:
            import torch.distributed as dist
            dist.barrier()
            dist.destroy_process_group()
        return

    import torch
    torch.cuda.set_device(local)
    from fug30v0kxc_gb300.params import VEC_PREC_FP64, VEC_PREC_SPLIT
    hbm, pk = peaks()
    if args.workload in ("closure", "net", "accuracy"):
        line = {"closure": closure_line, "net": net_line, "accuracy": accuracy_line}[args.workload](args, ws)
        if rank == 0:
            print(json.dumps(line), flush=True)
        if _dist["on"]:
            import torch.distributed as dist
            dist.barrier()
            dist.destroy_process_group()
        return
    if args.workload == "ensemble":
        e = ensemble_line(args, ws, hbm, pk)
        line = {"metric": "aggregate grid-point-steps/s, 48-instance ensemble", "value": e["value"],
                "unit": e["unit"], "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": e["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32/f64",
                "data": "synthetic (seeded static polytropes + uniform +-1e-3 T noise)",
                "config": {"workload": "ensemble 16x64^2x65 + 16x128^2x97 + 16x192^2x129, Ra log-uniform "
                                       "[1e4,1e6], Q {0,100,1000}, eta contrast {1,5,20}, split",
                           "parallelism": f"replicas{ws}", "l2": "no flush: resident state ~100 GB"},
                "roofline": {"bound": "hbm", "achieved": e["step_roofline"]["achieved_gbs"], "peak": hbm,
                             "unit": "GB/s", "frac": e["step_roofline"]["frac"], "traffic": None,
                             "basis": "196 B/gps compulsory state traffic of the whole step"},
                "clocks": e["clocks"], "gpu_launches": e["gpu_launches"], "ensemble": e}
        if rank == 0:
            print(json.dumps(line), flush=True)
        if _dist["on"]:
            import torch.distributed as dist
            dist.barrier()
            dist.destroy_process_group()
        return
    head_prec = VEC_PREC_FP64 if args.precision == "fp64" else VEC_PREC_SPLIT
    head = measure(args, head_prec, ws, hbm, pk, with_e2e=not args.no_e2e)
    line = {
        "metric": METRIC, "value": head["value"], "unit": "grid-point-steps/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if head_prec == VEC_PREC_FP64 else "f32/f64",
        "data": "synthetic (seeded static polytrope + uniform +-1e-3 T noise)",
        "config": {"workload": WORKLOAD, "nx": NX, "ny": NY, "nz": NZ,
                   "precision": "fp64" if head_prec == VEC_PREC_FP64 else "split (FP32 bulk, FP64 state)",
                   "parallelism": f"replicas{ws}",
                   "l2": "no flush: resident state >1 GB, larger than L2"},
        "roofline": head["roofline"],
        "step_roofline": head["step_roofline"],
        "clocks": head["clocks"],
        "e2e": head.get("e2e"),
        "gpu_launches": head["launches"],
        "kernel_ms_per_step": head["kernel_ms_per_step"],
        "kernels": head["kernels"],
    }
    if args.precision == "both":
        f64 = measure(args, VEC_PREC_FP64, ws, hbm, pk, with_e2e=not args.no_e2e)
        line["fp64"] = {"value": f64["value"], "ms_per_step": f64["ms_per_step"],
                        "roofline": f64["roofline"], "step_roofline": f64["step_roofline"],
                        "clocks": f64["clocks"], "gpu_launches": f64["launches"], "e2e": f64.get("e2e"),
                        "kernels": f64["kernels"][:6]}
        # The FP64 form is bound by GB300's FP64 pipe, not by HBM: its rate in
        # FLOP/s, with the step's operation count from the formula for n = 256
        # (transform passes x 2.5 log2 n + stencils + pointwise + AB3, about
        # 1.9 kflop per grid-point-step), against the FP64 FMA rate measured
        # on this GPU by the library's microbenchmark (vec_measure_fp64)
        if NX == 256 and NY == 256:
            achieved = FP64_FLOP_PER_GPS_256 * f64["value"] / ws / 1e12
            peak64, kind64 = fp64_peak()
            line["fp64"]["fp64_roofline"] = {"bound": "fp64", "achieved": round(achieved, 3),
                                             "peak": round(peak64, 3), "unit": "TFLOP/s",
                                             "frac": round(achieved / peak64, 3), "peak_kind": kind64,
                                             "flop_per_gps": FP64_FLOP_PER_GPS_256}
        line["split_over_fp64"] = head["value"] / f64["value"]
    if not args.no_ensemble and not args.grid:
        try:
            line["ensemble"] = ensemble_line(args, ws, hbm, pk)
        except Exception as ex:  # reported, never hides the headline
            line["ensemble"] = {"error": f"{type(ex).__name__}: {ex}"}
    if rank == 0 and not args.no_cpu:
        v, cores, dt = cpu_baseline(args.cpu_steps)
        line["cpu_baseline"] = {"value": v, "unit": "grid-point-steps/s", "cores": cores, "kind": "port",
                                "sample": f"{args.cpu_steps} steps of the full 256x256x129 workload "
                                          f"({dt:.1f} s) by the oracle port, FP64, OpenMP over planes"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if _dist["on"]:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
