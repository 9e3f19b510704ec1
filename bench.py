#!/usr/bin/env python
"""Benchmark: blastwave-steps/s of the comoving radiation step (synchrotron +
SSC + SSA) on the 21-layer Gaussian jet with forward and reverse shocks
(42 blastwaves x 1000 burster times, 201 gamma x 128 nu), on one GB300.

One bench "step" is one pass of the whole batch through the step: every
blastwave evolved over its 1000-time history (all valid blastwave-steps).
The inputs are, by default, the reference program's own run of that jet: the
dynamics its blastwave driver saved (tests/golden/refdrv_gaussian.npz,
recorded by tests/golden/make_reference_run.py), turned into step records
exactly as the driver passes them to its radiation step, so that the step
mix (valid steps, cooling regimes, substep counts) is the reference's own;
--inputs thin-shell uses the seeded thin-shell histories instead.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0). Under torchrun each rank runs its own replica
of the jet on its own GPU (blastwaves are independent; no collective on the
data path) and the line reports the whole-job rate over the slowest rank.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "blastwave-steps/s (sync+SSC) on 1 GB300"
UNIT = "blastwave-steps/s"
WORKLOAD = "gaussian-jet-21-layers-fs-rs-syn-ssc-ssa-201x128-ntb1000"
L2_FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-sample-seconds", type=float, default=15.0)
    ap.add_argument("--workload", default="gaussian-jet",
                    choices=["gaussian-jet", "contraction", "uneven-sweep", "surrogate", "eats-lc", "bw-rhs"],
                    help="gaussian-jet: the step benchmark (default); contraction: the emissivity-"
                         "contraction microbenchmark (65536 states, 256 gamma x 256 nu); uneven-sweep: a "
                         "seeded sample of the 4096-set parameter sweep with uneven step counts; surrogate: train "
                         "the SSC surrogate on states of the sweep, time it against the exact contraction and "
                         "deploy it on the Gaussian jet; eats-lc: the adaptive EATS light curve of the Gaussian jet "
                         "from the step's device-resident histories; bw-rhs: the blastwave ODE right-hand side "
                         "over a large batch of blastwave states")
    ap.add_argument("--inputs", default="driver", choices=["driver", "thin-shell"],
                    help="driver: step records from the reference program's own Gaussian-jet run (default); "
                         "thin-shell: seeded thin-shell histories")
    ap.add_argument("--subset", default="all", choices=["all", "chang-cooper", "rest"],
                    help="gaussian-jet workload, a timing aid: all (default); chang-cooper: only the blastwaves with "
                         "Chang-Cooper steps, up to their last one; rest: every other valid record as a one-step "
                         "blastwave (histories.split_chain)")
    ap.add_argument("--sets", type=int, default=64, help="parameter sets of the uneven-sweep workload")
    ap.add_argument("--train-states", type=int, default=1000000, help="training states of the surrogate workload")
    ap.add_argument("--epochs", type=int, default=8, help="training epochs of the surrogate workload")
    ap.add_argument("--tol", type=float, default=0.01, help="error-estimate tolerance of the surrogate")
    ap.add_argument("--states", type=int, default=65536)
    ap.add_argument("--fp32-states", type=int, default=4096,
                    help="states of the FP32 CUDA-core variant of the contraction benchmark")
    ap.add_argument("--check-states", type=int, default=64,
                    help="states checked against the FP64 oracle in the contraction benchmark")
    ap.add_argument("--lc-times", type=int, default=32, help="observer times of the eats-lc workload")
    ap.add_argument("--quad", default="cadre", choices=["cadre", "trap"], help="quadrature of the eats-lc workload")
    ap.add_argument("--rhs-states", type=int, default=1 << 20, help="blastwave states of the bw-rhs workload")
    ap.add_argument("--profile", type=int, default=0,
                    help="run this many device passes of the workload and exit (for ncu captures)")
    return ap.parse_args()


from pyblastafterglowmag_gb300.replicas import dist_info  # noqa: E402
from pyblastafterglowmag_gb300 import replicas  # noqa: E402


DRIVER_RUN = os.path.join(ROOT, "tests", "golden", "refdrv_gaussian.npz")
INPUTS = {"driver": "the reference program's own run of the jet: the dynamics its blastwave driver saved "
                    "(refdrv_gaussian.npz), step records rebuilt as the driver passes them to its step",
          "thin-shell": "seeded synthetic blastwave histories (thin-shell dynamics)"}


def driver_run():
    from pyblastafterglowmag_gb300 import histories as H
    return H.DriverRun(DRIVER_RUN)


def workload(inputs, tables=None):
    """The Gaussian jet's step records from `inputs` (INPUTS). tables:
    what builds the grids and the shock scalars - the library (default) or,
    for the CPU arm, the oracle, which produces the same bytes without
    loading the library."""
    from pyblastafterglowmag_gb300 import histories as H
    if tables is None:
        from pyblastafterglowmag_gb300 import _lib as tables
    cfg = H.config_gaussian_ssc()
    if inputs == "driver":
        run = driver_run()
        assert (run.grid.ngam, run.grid.nfreq, run.nlayers) == (cfg.ngam, cfg.nfreq, cfg.nlayers)
        recs, off, prm = run.records(tables)
        grid = run.grid
    else:
        recs, off, prm, grid = H.make_batch(tables, cfg)
    return cfg, recs, off, prm, grid


def config_dict(cfg, recs, prm, inputs, extra=None):
    d = {"workload": WORKLOAD, "blastwaves": int(len(prm)), "layers": cfg.nlayers,
         "shocks": "forward+reverse", "ngam": cfg.ngam, "nfreq": cfg.nfreq, "ntb": cfg.ntb,
         "valid_blastwave_steps_per_pass": int((recs["mode"] != 0).sum()),
         "radiation": "synchrotron(CSYN)+SSA+SSC", "solve": "Chang-Cooper, FP64 state, double-float substeps",
         "ssc_contraction": "FP32 accumulate, per-blastwave power-of-two scaling",
         "l2": "flushed with a 256 MiB device write before every timed pass",
         "inputs": INPUTS[inputs]}
    if extra:
        d.update(extra)
    return d


def algorithmic_bytes_per_bw_step(grid, outputs):
    """Bytes one blastwave-step must move at minimum (FP64): N(gamma) in and
    out (2G), photon field in and out (2F), ~20 step scalars, and the history
    rows the caller asked for (F values each; j and a are the totals). The
    evolve kernel does all of it (it completes the previous step too)."""
    G, F = grid.ngam, grid.nfreq
    return 8 * (2 * G + 2 * F + 20 + len(outputs) * F)


def contraction_flops_per_bw_step(grid):
    """Algorithmic FLOPs of the emissivity contractions of one blastwave-step:
    the SSC bilinear form 2 F^2 G and the synchrotron quadrature 2 F G."""
    G, F = grid.ngam, grid.nfreq
    return 2 * F * F * G + 2 * F * G


# ---------------------------------------------------------------- clocks ---
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.samples, self._stop = index, [], threading.Event()
        self._t = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 3 + i and s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# ---------------------------------------------------------- cpu baseline ---
def cpu_sample(recs, off, prm, grid, seconds, threads, inner=0):
    """Time the oracle port on a bounded sample of the workload: windows of
    consecutive steps spread over every blastwave's history, each window
    re-initialised at its first step. threads: blastwaves in parallel, one per
    thread; inner > 0: the reference's own arrangement instead, blastwaves one
    after another with the inner loops on `inner` threads (its num_threads(4)
    OpenMP loops). Returns (bw-steps/s, description, seconds)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from pyblastafterglowmag_gb300 import abi
    orc = pyoracle.Oracle()
    nbw = len(prm)

    def make(nwin, wlen):
        rr, lens, pp = [], [], []
        for b in range(nbw):
            n = int(off[b + 1] - off[b])
            for s0 in np.linspace(0, n - wlen, nwin).astype(int):
                r = recs[off[b] + s0: off[b] + s0 + wlen]
                rr.append(r)
                lens.append(len(r))
                pp.append(prm[b])
        o = np.zeros(len(lens) + 1, dtype=np.int64)
        o[1:] = np.cumsum(lens)
        return np.concatenate(rr), o, np.array(pp, dtype=abi.SHOCK_PARAMS_DTYPE)

    kw = (dict(flags=pyoracle.ORC_INNER_OMP, outer_threads=1, inner_threads=inner) if inner > 0
          else dict(flags=0, outer_threads=threads))
    # calibrate on a small sample, then size the sample to ~`seconds`
    r, o, p = make(1, 4)
    t0 = time.perf_counter()
    orc.run(grid, r, o, p, **kw)
    t1 = time.perf_counter() - t0
    per_step = max(t1 / max(int((r["mode"] != 0).sum()), 1), 1e-6)
    budget_steps = seconds / per_step
    # long windows: the first step of each is the (cheaper) initialisation
    wlen = 25
    nwin = int(max(1, min(16, budget_steps / (wlen * nbw))))
    r, o, p = make(nwin, wlen)
    t0 = time.perf_counter()
    rc, where, _ = orc.run(grid, r, o, p, **kw)
    dt = time.perf_counter() - t0
    n = int((r["mode"] != 0).sum())
    how = (f"blastwaves one after another, inner loops on {inner} threads as in the reference" if inner > 0
           else "one blastwave per thread")
    desc = (f"{nbw} blastwaves x {nwin} windows x {wlen} consecutive steps spread over the 1000-step "
            f"histories ({n} valid blastwave-steps), FP64 oracle port in the reference's loop structure "
            f"(cooling terms recomputed every substep), {how}")
    return n / dt, desc, dt


def reference_arm(args):
    """The reference's CPU path alone: the oracle port (the reference's loop
    structure, bit-exact against the compiled reference) builds the records and
    runs the step; the GPU library is neither built nor loaded."""
    rank, world, local = dist_info()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build_oracle()
    cfg, recs, off, prm, grid = workload(args.inputs, pyoracle.Oracle())
    threads = os.cpu_count() or 1
    per_step = max(10.0, min(60.0, 150.0 / max(args.steps + args.warmup, 1)))
    vals, dts, desc = [], [], ""
    for i in range(args.warmup + args.steps):
        v, desc, dt = cpu_sample(recs, off, prm, grid, per_step, threads)
        if i >= args.warmup:
            vals.append(v)
            dts.append(dt)
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.median(dts),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": config_dict(cfg, recs, prm, args.inputs, {"sample": desc}),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------- gb300 arm ---
def gb300_arm(args):
    import torch
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    replicas.init(world)
    from pyblastafterglowmag_gb300 import _lib, abi, build, histories as H
    build.build()
    cfg, recs, off, prm, grid = workload(args.inputs)
    if args.subset != "all":
        gam, _ = _lib.grids(grid)
        chain, rest = H.split_chain(recs, off, prm, gam)
        recs, off, prm = chain if args.subset == "chang-cooper" else rest
    nvalid = int((recs["mode"] != 0).sum())
    nrec, nbw, F = len(recs), len(prm), grid.nfreq
    ctx = _lib.Context(grid, device=local, ssc=True)
    dev = torch.device("cuda", local)

    # device-resident inputs and outputs
    d_recs = torch.from_numpy(recs.view(np.uint8).copy()).to(dev)
    d_prm = torch.from_numpy(prm.view(np.uint8).copy()).to(dev)
    outs = ("j_all", "a_all", "f_all", "i_all")
    d_out = {k: torch.empty((nrec, F), dtype=torch.float64, device=dev) for k in outs}
    d_ptrs = {k: v.data_ptr() for k, v in d_out.items()}
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def barrier():
        replicas.barrier(world, dev)

    def one_pass():
        ctx.run_device(d_prm.data_ptr(), nbw, off, d_recs.data_ptr(), d_ptrs)

    if args.profile:
        for _ in range(args.profile):
            one_pass()
        torch.cuda.synchronize(dev)
        print(json.dumps({"profile_passes": args.profile, "launches_per_pass": ctx.last_launch_count()}))
        return
    for _ in range(args.warmup):
        flush.zero_()
        one_pass()
    barrier()
    # timed region: K passes, device time of each pass with CUDA events
    launches = 0
    ev_ms = []
    with ClockSampler(local) as clk:
        barrier()
        t_wall = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize(dev)
            e0.record(stream)
            one_pass()  # synchronous: returns after the batch finished on the device
            e1.record(stream)
            e1.synchronize()
            ev_ms.append(e0.elapsed_time(e1))
            launches += ctx.last_launch_count()
        barrier()
        t_wall = time.perf_counter() - t_wall
    # per-kernel device times: one more pass with a CUDA event pair around
    # every launch on the library's stream (direct launches instead of the
    # captured graph, same kernels and data)
    ctx.set_timing(True)
    flush.zero_()
    one_pass()
    timing = ctx.timing()
    ctx.set_timing(False)
    prof_passes = 1
    total_ms = replicas.max_over_ranks(float(sum(ev_ms)), world)
    value = replicas.job_rate(nvalid * args.steps, total_ms * 1e-3, world)

    # end to end through the host-buffer entry point (pinned host memory)
    h_recs = torch.from_numpy(recs.view(np.uint8).copy()).pin_memory()
    h_prm = torch.from_numpy(prm.view(np.uint8).copy()).pin_memory()
    h_out = {k: torch.empty((nrec, F), dtype=torch.float64).pin_memory() for k in outs}
    out_struct = abi.Outputs()
    import ctypes as C
    for k in abi.OUTPUT_FIELDS:
        setattr(out_struct, k, C.cast(C.c_void_p(h_out[k].data_ptr()), C.POINTER(C.c_double))
                if k in h_out else C.POINTER(C.c_double)())
    lib = _lib.load()
    off_c = np.ascontiguousarray(off, dtype=np.int64)

    def e2e_pass():
        st = abi.Status()
        rc = lib.pbag_run_batch(ctx.handle, C.c_void_p(h_prm.data_ptr()), nbw,
                                off_c.ctypes.data_as(C.POINTER(C.c_int64)), C.c_void_p(h_recs.data_ptr()),
                                C.byref(out_struct), C.byref(st))
        if rc != 0:
            raise _lib.PbagError(rc, "pbag_run_batch", st.bw, st.step, st.site)

    for _ in range(max(1, args.warmup)):
        e2e_pass()
    barrier()
    e2e_t = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        e2e_pass()
        e2e_t.append(time.perf_counter() - t0)
    e2e_total = replicas.max_over_ranks(sum(e2e_t), world)
    e2e_value = replicas.job_rate(nvalid * args.steps, e2e_total, world)
    h2d = int(recs.nbytes + prm.nbytes + off_c.nbytes)
    d2h = int(nrec * F * 8 * len(outs))

    if rank != 0:
        return
    # roofline of the dominant kernel class
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    tc_peak = float(peaks.get("bf16_tflops", 1900.0))
    dominant = max(timing, key=lambda k: timing[k][0])
    share = {k: v[0] / max(sum(x[0] for x in timing.values()), 1e-12) for k, v in timing.items()}
    traffic = {}
    try:
        traffic = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
    except Exception:
        pass
    # the evolve kernel (Chang-Cooper solve + completion of the previous step): HBM roofline
    ms_e, nl_e = timing["evolve"]
    bw_steps_per_launch = nvalid / max(nl_e, 1)
    bytes_per_launch = bw_steps_per_launch * algorithmic_bytes_per_bw_step(grid, outs)
    achieved = bytes_per_launch / (ms_e / nl_e * 1e-3) / 1e9 if nl_e else None
    roofline = {"bound": "hbm", "kernel": "evolve", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak if achieved else None,
                "traffic": traffic.get("evolve_bytes_per_launch"),
                "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
                "bytes_per_launch": bytes_per_launch,
                "bytes_per_blastwave_step": algorithmic_bytes_per_bw_step(grid, outs),
                "avg_launch_us": 1e3 * ms_e / nl_e if nl_e else None,
                "dominant_kernel_class": dominant,
                "kernel_share": share,
                "kernel_ms_per_pass": {k: v[0] / prof_passes for k, v in timing.items()},
                "kernel_timing": "CUDA events around every launch on the library stream, one extra pass of the same workload with direct launches"}
    # the emissivity contractions (tensor-core SSC + synchrotron/SSA): tensor roofline
    ms_c, nl_c = timing["ssc"]
    flops_per_launch = nvalid / max(nl_c, 1) * contraction_flops_per_bw_step(grid)
    tflops = flops_per_launch / (ms_c / nl_c * 1e-3) / 1e12 if nl_c else None
    roofline_c = {"bound": "tensor", "kernel": "ssc+radiation", "achieved": tflops, "peak": tc_peak,
                  "unit": "TFLOP/s", "frac": tflops / tc_peak if tflops else None,
                  "traffic": traffic.get("ssc_bytes_per_launch"),
                  "flops_per_blastwave_step": contraction_flops_per_bw_step(grid),
                  "avg_launch_us": 1e3 * ms_c / nl_c if nl_c else None,
                  "peak_source": "measured" if "bf16_tflops" in peaks else "fallback"}
    bws = [b for b in (0, 1, 10, 11, 16, 17, 40) if b < nbw] if args.subset == "all" else list(range(min(nbw, 6)))
    parity = output_check(recs, off, prm, grid, {k: v.numpy() for k, v in h_out.items()}, bws=tuple(bws))
    threads = os.cpu_count() or 1
    if args.subset == "all":
        cpu_v, cpu_desc, _ = cpu_sample(recs, off, prm, grid, args.cpu_sample_seconds, threads)
        # the reference's own arrangement (blastwaves serial, inner loops on 4 threads)
        asis_v, asis_desc, _ = cpu_sample(recs, off, prm, grid, min(8.0, args.cpu_sample_seconds), threads, inner=4)
    else:  # a timing aid on part of the batch: no CPU sample
        cpu_v = asis_v = None
        cpu_desc = asis_desc = f"not sampled (--subset {args.subset})"
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64/f32", "data": "synthetic",
            "config": config_dict(cfg, recs, prm, args.inputs, {"parallelism": f"replicas{world}",
                                                                 "subset": args.subset}),
            "clocks": clk.summary(),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": int(launches),
            "roofline": roofline,
            "roofline_contraction": roofline_c,
            "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": threads, "kind": "port", "sample": cpu_desc,
                             "as_is": {"value": asis_v, "unit": UNIT, "cores": 4, "sample": asis_desc}},
            "parity": parity,
            "wall_s_timed_region": t_wall}
    print(json.dumps(line), flush=True)


def output_check(recs, off, prm, grid, got, bws=(0, 1, 10, 11, 16, 17, 40), tol=1e-4):
    """The histories of the last end-to-end pass against the FP64 oracle on a
    sample of whole blastwaves (each blastwave's history is independent, so a
    subset runs exactly as in the batch): per-row relative L2 of every timed
    output, its maximum per history."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from pyblastafterglowmag_gb300 import abi
    orc = pyoracle.Oracle()
    rows = np.concatenate([np.arange(off[b], off[b + 1]) for b in bws])
    lens = [int(off[b + 1] - off[b]) for b in bws]
    o = np.zeros(len(bws) + 1, dtype=np.int64)
    o[1:] = np.cumsum(lens)
    p = np.array([prm[b] for b in bws], dtype=abi.SHOCK_PARAMS_DTYPE)
    rc, where, ref = orc.run(grid, recs[rows], o, p, outputs=tuple(got), outer_threads=len(bws))
    worst = {}
    for k, r in ref.items():
        g = got[k][rows]
        num = np.sqrt(((g - r) ** 2).sum(axis=1))
        den = np.sqrt((r ** 2).sum(axis=1))
        rel = num[den > 0] / den[den > 0]
        zero_bad = int(((den == 0) & (num > 0)).sum())
        worst[k] = float(rel.max()) if rel.size else 0.0
        if zero_bad:
            worst[k] = float("inf")
    return {"blastwaves": list(bws), "rows": int(len(rows)), "oracle_status": int(rc),
            "max_rel_l2": worst, "tol": tol, "ok": bool(rc == 0 and max(worst.values()) <= tol)}


# ------------------------------------------------------ contraction arm ---
def contraction_arm(args):
    """Emissivity-contraction microbenchmark: pbag_contract (synchrotron sums
    in FP32 + SSC contraction) on seeded states, for every SSC precision, each
    checked against the FP64 oracle on a sample of states."""
    import ctypes as C
    import torch
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    from pyblastafterglowmag_gb300 import _lib, abi, build, contraction as CT
    build.build()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    dev = torch.device("cuda", local)
    n = args.states
    g = CT.grid_desc(256, 256)
    G, F = g.ngam, g.nfreq
    gam, freq = _lib.grids(g)
    f, B = CT.states(gam, n)
    ctx = _lib.Context(g, local, ssc=True)
    d_f = torch.from_numpy(f).to(dev)
    d_B = torch.from_numpy(B).to(dev)
    d_js = torch.zeros((n, F), dtype=torch.float64, device=dev)
    d_jc = torch.zeros((n, F), dtype=torch.float64, device=dev)
    # seed photons: the states' own synchrotron spectra
    ctx.contract_device(n, d_f.data_ptr(), d_B.data_ptr(), 0, abi.PBAG_SYN_CSYN, abi.PBAG_PREC_FP32,
                        d_js.data_ptr(), 0)
    nu = torch.from_numpy(np.asarray(freq[:F])).to(dev)
    d_n = (d_js / (CT.H_PL * nu[None, :])).contiguous()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    flops_state = 2 * F * F * G + 2 * F * G
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    tc_peak = float(peaks.get("bf16_tflops", 1900.0))
    orc = pyoracle.Oracle()
    ns = min(args.check_states, n)
    sample = np.linspace(0, n - 1, ns).astype(int)
    threads = os.cpu_count() or 1
    variants = {}
    with ClockSampler(local) as clk:
        for prec in (abi.PBAG_PREC_SPLIT_BF16, abi.PBAG_PREC_BF16, abi.PBAG_PREC_TF32, abi.PBAG_PREC_FP32):
            nn = n if prec != abi.PBAG_PREC_FP32 else min(n, args.fp32_states)

            def run(ssc_only=False):
                ctx.contract_device(nn, d_f.data_ptr(), d_B.data_ptr(), d_n.data_ptr(), abi.PBAG_SYN_CSYN, prec,
                                    0 if ssc_only else d_js.data_ptr(), d_jc.data_ptr())

            def timed(ssc_only):
                for _ in range(args.warmup):
                    flush.zero_()
                    run(ssc_only)
                ms = []
                for _ in range(args.steps):
                    flush.zero_()
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    torch.cuda.synchronize(dev)
                    e0.record()
                    run(ssc_only)
                    e1.record()
                    e1.synchronize()
                    ms.append(e0.elapsed_time(e1))
                return statistics.median(ms)

            ms_all = timed(False)
            ms_ssc = timed(True)
            run(False)
            js = d_js[sample[sample < nn]].cpu().numpy()
            jc = d_jc[sample[sample < nn]].cpu().numpy()
            idx = sample[sample < nn]
            ojs, ojc = orc.contract(g, f[idx], B=B[idx], nph=d_n[idx].cpu().numpy(), threads=threads)

            def rel(x, y):
                num = np.sqrt(((x - y) ** 2).sum(axis=1))
                den = np.sqrt((y ** 2).sum(axis=1))
                r = num[den > 0] / den[den > 0]
                return float(r.max()), float(np.percentile(r, 99))

            es, ec = rel(js, ojs), rel(jc, ojc)
            tflops = nn * flops_state / (ms_all * 1e-3) / 1e12
            variants[abi.PRECISION_NAMES[prec]] = {
                "states": int(nn), "ms_per_pass": ms_all, "states_per_s": nn / (ms_all * 1e-3),
                "ssc_only_ms_per_pass": ms_ssc,
                "tflops_algorithmic": tflops, "frac_of_bf16_peak": tflops / tc_peak,
                "ssc_tflops_algorithmic": nn * 2 * F * F * G / (ms_ssc * 1e-3) / 1e12,
                "rel_l2_jsyn_max": es[0], "rel_l2_jssc_max": ec[0], "rel_l2_jssc_p99": ec[1],
                "checked_states": int(len(idx))}
    best = variants["split-bf16"]
    # end to end through the C ABI with host buffers: states in, spectra out
    h_f = torch.from_numpy(f).pin_memory()
    h_B = torch.from_numpy(B).pin_memory()
    h_n = d_n.cpu().pin_memory()
    h_js = torch.empty((n, F), dtype=torch.float64).pin_memory()
    h_jc = torch.empty((n, F), dtype=torch.float64).pin_memory()

    def e2e():
        d_f.copy_(h_f, non_blocking=True)
        d_B.copy_(h_B, non_blocking=True)
        d_n.copy_(h_n, non_blocking=True)
        torch.cuda.current_stream(dev).synchronize()
        ctx.contract_device(n, d_f.data_ptr(), d_B.data_ptr(), d_n.data_ptr(), abi.PBAG_SYN_CSYN,
                            abi.PBAG_PREC_SPLIT_BF16, d_js.data_ptr(), d_jc.data_ptr())
        h_js.copy_(d_js)
        h_jc.copy_(d_jc)

    e2e()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e()
    e2e_s = (time.perf_counter() - t0) / args.steps
    if rank != 0:
        return
    line = {"metric": "contraction states/s (synchrotron + SSC, split-BF16) on 1 GB300", "value": best["states_per_s"],
            "unit": "states/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": best["ms_per_pass"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16x3/f32", "data": "synthetic",
            "config": {"workload": "contraction-microbench-65536-states-256x256", "states": n, "ngam": G, "nfreq": F,
                       "inputs": "seeded power laws with exponential cutoff; seed photons = own synchrotron spectra",
                       "l2": "flushed with a 256 MiB device write before every timed pass"},
            "clocks": clk.summary(),
            "e2e": {"value": n / e2e_s, "unit": "states/s", "h2d_bytes_per_step": int(f.nbytes + B.nbytes + h_n.numel() * 8),
                    "d2h_bytes_per_step": int(2 * n * F * 8)},
            "roofline": {"bound": "tensor", "kernel": "k_ssc_tc (split-bf16) + prep + synchrotron sums",
                         "achieved": best["tflops_algorithmic"], "peak": tc_peak, "unit": "TFLOP/s",
                         "frac": best["frac_of_bf16_peak"], "traffic": None,
                         "flops_per_state": flops_state,
                         "peak_source": "measured" if "bf16_tflops" in peaks else "fallback"},
            "variants": variants}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------- uneven-sweep arm ---
def sweep_arm(args):
    """A seeded sample of the batched parameter sweep (top-hat and Gaussian jets
    of 1-41 layers x FS+RS, uneven 200-2000 step histories) as one batch: one
    captured graph over the longest history, blastwaves drop out as their
    histories end."""
    import torch
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    replicas.init(world)
    from pyblastafterglowmag_gb300 import _lib, abi, build, histories as H
    build.build()
    # rank r runs sets r*sets .. (r+1)*sets-1 of the seeded sweep (weak scaling)
    recs, off, prm, grid = H.sweep_batch(_lib, args.sets, seed=3, workers=os.cpu_count() or 1,
                                         first=rank * args.sets)
    nvalid = int((recs["mode"] != 0).sum())
    nrec, nbw, F = len(recs), len(prm), grid.nfreq
    dev = torch.device("cuda", local)
    ctx = _lib.Context(grid, device=local, ssc=True)
    d_recs = torch.from_numpy(recs.view(np.uint8).copy()).to(dev)
    d_prm = torch.from_numpy(prm.view(np.uint8).copy()).to(dev)
    outs = ("j_all", "a_all")
    d_out = {k: torch.empty((nrec, F), dtype=torch.float64, device=dev) for k in outs}
    d_ptrs = {k: v.data_ptr() for k, v in d_out.items()}
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    status = {"code": 0}

    def one_pass():
        try:
            ctx.run_device(d_prm.data_ptr(), nbw, off, d_recs.data_ptr(), d_ptrs)
        except _lib.PbagError as e:  # the reference would stop this run; the batch completes
            status.update(code=e.code, blastwave=e.bw, step=e.step)

    if args.profile:
        for _ in range(args.profile):
            one_pass()
        torch.cuda.synchronize(dev)
        print(json.dumps({"profile_passes": args.profile, "launches_per_pass": ctx.last_launch_count(),
                          "blastwaves": nbw}))
        return
    for _ in range(args.warmup):
        flush.zero_()
        one_pass()
    ms = []
    replicas.barrier(world, dev)
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize(dev)
            e0.record()
            one_pass()
            e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
    replicas.barrier(world, dev)
    # per-kernel-class device time: one more pass with a CUDA event pair
    # around every launch (direct launches instead of the captured graph)
    ctx.set_timing(True)
    flush.zero_()
    one_pass()
    timing = ctx.timing()
    ctx.set_timing(False)
    t = replicas.max_over_ranks(sum(ms) / len(ms), world)
    value = replicas.job_rate(nvalid, t * 1e-3, world)
    if rank != 0:
        return
    lens = np.diff(off)
    line = {"metric": "blastwave-steps/s (sync+SSC) on 1 GB300, uneven sweep", "value": value,
            "unit": "blastwave-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64/f32",
            "data": "synthetic",
            "config": {"workload": f"uneven-sweep-{args.sets}-sets-201x128", "sets": args.sets, "blastwaves": nbw,
                       "records": int(nrec), "valid_blastwave_steps_per_pass": nvalid,
                       "steps_per_blastwave": [int(lens.min()), int(lens.max())],
                       "launch": "one captured graph over the longest history",
                       "l2": "flushed with a 256 MiB device write before every timed pass",
                       "outputs": list(outs)},
            "clocks": clk.summary(), "status": status, "gpu_launches": ctx.last_launch_count(),
            "kernel_ms_per_pass": {k: v[0] for k, v in timing.items()},
            "kernel_launches_per_pass": {k: v[1] for k, v in timing.items()},
            "kernel_timing": "CUDA events around every launch on the library stream, one extra pass with direct launches"}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------- surrogate arm ---
def surrogate_profile(args, dev, n=100_000):
    """Kernel passes for ncu captures of the surrogate's kernels: n seeded
    states on the 201 x 128 grid (seed photons = their own synchrotron
    spectra), a random-init network with no fallback (the same kernels and
    shapes as a trained one), args.profile surrogate passes, then as many
    exact split-BF16 contractions."""
    import torch
    from pyblastafterglowmag_gb300 import _lib, abi, contraction as CT, surrogate as SG
    g = CT.grid_desc(ngam=201, nfreq=128)
    gam, freq = _lib.grids(g)
    f, B = CT.states(gam, n, seed=4)
    ctx = _lib.Context(g, dev.index, ssc=True)
    d_f = torch.from_numpy(f).to(dev)
    d_B = torch.from_numpy(B).to(dev)
    d_js = torch.zeros((n, g.nfreq), dtype=torch.float64, device=dev)
    ctx.contract_device(n, d_f.data_ptr(), d_B.data_ptr(), 0, abi.PBAG_SYN_CSYN, abi.PBAG_PREC_FP32,
                        d_js.data_ptr(), 0)
    nph = torch.from_numpy(CT.seed_photons(d_js.cpu().numpy(), freq)).to(dev)
    SG.configure(ctx)
    tr = SG.Trainer(g.nfreq, dev.index, seed=0)
    SG.configure(ctx, tr.net, tr.mean, tr.std, tol=1e30)
    j = torch.zeros((n, g.nfreq), dtype=torch.float64, device=dev)
    for _ in range(args.profile):
        SG.contract(ctx, n, d_f.data_ptr(), d_B.data_ptr(), nph.data_ptr(), j.data_ptr())
    for _ in range(args.profile):
        ctx.contract_device(n, d_f.data_ptr(), d_B.data_ptr(), nph.data_ptr(), abi.PBAG_SYN_CSYN,
                            abi.PBAG_PREC_SPLIT_BF16, 0, j.data_ptr())
    torch.cuda.synchronize(dev)
    print(json.dumps({"profile_passes": args.profile, "states": n, "workload": "surrogate-kernels-201x128"}))


def surrogate_arm(args):
    """SSC surrogate: trained on states of a seeded sweep (the plain GPU step),
    evaluated on held-out states against the exact contraction (split BF16),
    timed against it, and deployed on the Gaussian jet with the error estimate
    and exact fallback."""
    import torch
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    from pyblastafterglowmag_gb300 import _lib, abi, build, histories as H, surrogate as SG
    build.build()
    dev = torch.device("cuda", local)
    if args.profile:
        return surrogate_profile(args, dev)
    cfg, recs, off, prm, g = workload(args.inputs)
    _, freq = _lib.grids(g)
    ctx = _lib.Context(g, device=local, ssc=True)
    SG.configure(ctx)
    t0 = time.perf_counter()
    f, B, nph = SG.sweep_states(ctx, g, nsets=max(args.sets, 8), seed=5, workers=os.cpu_count() or 1, device=local,
                                max_states=args.train_states)
    t_gen = time.perf_counter() - t0
    n = f.shape[0]
    X = torch.zeros((n, SG.NIN), dtype=torch.float32, device=dev)
    proj = torch.zeros((n, SG.NPROJ), dtype=torch.float64, device=dev)
    base = torch.zeros((n, g.nfreq), dtype=torch.float32, device=dev)
    SG.features(ctx, n, f.data_ptr(), B.data_ptr(), nph.data_ptr(), X.data_ptr(), proj.data_ptr(), base.data_ptr())
    jex = SG.exact_ssc(ctx, f, B, nph)
    T, M = SG.make_targets(jex, proj, freq, base)
    ntr, ncal = int(0.85 * n), int(0.05 * n)
    tr = SG.Trainer(g.nfreq, local, seed=0)
    Xs = tr.standardise(X.clone())
    t0 = time.perf_counter()
    loss = tr.fit(Xs[:ntr], T[:ntr], M[:ntr], epochs=args.epochs, batch=4096, lr=2e-3)
    torch.cuda.synchronize(dev)
    t_train = time.perf_counter() - t0
    cal = slice(ntr, ntr + ncal)
    scale = SG.calibrate(ctx, tr, f[cal].contiguous(), B[cal].contiguous(), nph[cal].contiguous(),
                         jex[cal].contiguous())
    va = slice(ntr + ncal, n)
    fv, Bv, nv, jv = f[va].contiguous(), B[va].contiguous(), nph[va].contiguous(), jex[va].contiguous()
    nv_states = fv.shape[0]
    # accuracy without fallback, the error estimate, and with the tolerance
    cfg_sur = lambda tol: SG.configure(ctx, tr.net, tr.mean, tr.std, tol=tol, est_scale=scale)
    cfg_sur(1e30)
    j = torch.zeros_like(jv)
    est = torch.zeros(nv_states, dtype=torch.float32, device=dev)
    SG.contract(ctx, nv_states, fv.data_ptr(), Bv.data_ptr(), nv.data_ptr(), j.data_ptr(), est.data_ptr())
    err = SG.rel_l2(j, jv)
    err_rows = SG.rel_l2_rows(j, jv)
    err_base = SG.rel_l2(SG.band_baseline(proj[va], freq, base[va]), jv)
    cfg_sur(args.tol)
    jt = torch.zeros_like(jv)
    nfb = SG.contract(ctx, nv_states, fv.data_ptr(), Bv.data_ptr(), nv.data_ptr(), jt.data_ptr())
    err_t = SG.rel_l2(jt, jv)
    accepted = (est <= args.tol) & torch.isfinite(err_rows)
    q = lambda e, p: float(e.quantile(p)) if e.numel() <= 16_000_000 else float(e.float().quantile(p))

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        ms = []
        for _ in range(args.steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize(dev)
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return statistics.median(ms)

    jj = torch.zeros_like(jv)
    ms_exact = timed(lambda: ctx.contract_device(nv_states, fv.data_ptr(), Bv.data_ptr(), nv.data_ptr(),
                                                 abi.PBAG_SYN_CSYN, abi.PBAG_PREC_SPLIT_BF16, 0, jj.data_ptr()))
    ms_exact_bf16 = timed(lambda: ctx.contract_device(nv_states, fv.data_ptr(), Bv.data_ptr(), nv.data_ptr(),
                                                      abi.PBAG_SYN_CSYN, abi.PBAG_PREC_BF16, 0, jj.data_ptr()))
    cfg_sur(1e30)
    ms_sur = timed(lambda: SG.contract(ctx, nv_states, fv.data_ptr(), Bv.data_ptr(), nv.data_ptr(), jj.data_ptr()))
    cfg_sur(args.tol)
    ms_sur_fb = timed(lambda: SG.contract(ctx, nv_states, fv.data_ptr(), Bv.data_ptr(), nv.data_ptr(), jj.data_ptr()))
    # deployment on the Gaussian jet: surrogate step vs plain step
    outs = ("j_all", "a_all", "f_all", "i_all")
    plain = ctx.run(recs, off, prm, outputs=outs)
    ctx.set_ssc_path(abi.PBAG_SSC_SURROGATE)
    sur = ctx.run(recs, off, prm, outputs=outs)
    t_sur = min(timeit_run(ctx, recs, off, prm) for _ in range(3))
    ctx.set_ssc_path(abi.PBAG_SSC_AUTO)
    t_plain = min(timeit_run(ctx, recs, off, prm) for _ in range(3))
    num = np.sqrt(((sur["j_all"] - plain["j_all"]) ** 2).sum(axis=1))
    den = np.sqrt((plain["j_all"] ** 2).sum(axis=1))
    rows = den > 0
    dep = num[rows] / den[rows]
    nvalid = int((recs["mode"] != 0).sum())
    if rank != 0:
        return
    line = {"metric": "SSC surrogate speed-up over the exact contraction (states/s ratio)",
            "value": ms_exact / ms_sur_fb, "unit": "x", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_sur_fb, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 MLP and projections / bf16x3 fallback", "data": "synthetic",
            "config": {"workload": "ssc-surrogate-201x128", "train_states": ntr, "val_states": nv_states,
                       "epochs": args.epochs, "net": [SG.NIN, *SG.HIDDEN, g.nfreq], "tol": args.tol,
                       "train_source": "seeded parameter sweep (seed 5), plain GPU step",
                       "calibration_states": ncal, "est_scale": scale},
            "timing": {"generate_s": t_gen, "train_s": t_train, "final_loss": loss,
                       "exact_ms": ms_exact, "exact_bf16_ms": ms_exact_bf16,
                       "surrogate_ms_no_fallback": ms_sur, "surrogate_ms_with_fallback": ms_sur_fb,
                       "states_per_s_exact": nv_states / (ms_exact * 1e-3),
                       "states_per_s_surrogate": nv_states / (ms_sur_fb * 1e-3),
                       "speedup_no_fallback": ms_exact / ms_sur,
                       "speedup_vs_exact_bf16": ms_exact_bf16 / ms_sur_fb},
            "accuracy": {"rel_l2_median": q(err, 0.5), "rel_l2_p90": q(err, 0.9), "rel_l2_p99": q(err, 0.99),
                         "baseline_rel_l2_median": q(err_base, 0.5),
                         "with_fallback_rel_l2_median": q(err_t, 0.5), "with_fallback_rel_l2_p99": q(err_t, 0.99),
                         "with_fallback_rel_l2_max": float(err_t.max()),
                         "fallback_fraction": nfb / nv_states,
                         "accepted_true_error_p99": q(err_rows[accepted], 0.99) if bool(accepted.any()) else None,
                         "accepted_true_error_max": float(err_rows[accepted].max()) if bool(accepted.any())
                         else None,
                         "accepted_above_tol_fraction": float((err_rows[accepted] > args.tol).float().mean())
                         if bool(accepted.any()) else None},
            "deployment_gaussian_jet": {"j_all_rel_l2_vs_plain_median": float(np.median(dep)),
                                        "j_all_rel_l2_vs_plain_p99": float(np.percentile(dep, 99)),
                                        "blastwave_steps_per_s_surrogate": nvalid / t_sur,
                                        "blastwave_steps_per_s_plain": nvalid / t_plain}}
    print(json.dumps(line), flush=True)

# ------------------------------------------------------------ eats-lc arm ---
def eats_arm(args):
    """The adaptive EATS light curve of the 21-layer Gaussian jet (forward and
    reverse shocks, theta_obs = 20.8 deg, nu = 1e15 Hz, args.lc_times observer
    times in [3e3, 1e9] s, CADRE with rtol 1e-6 or TRAP_FIXED 100 x 100): the
    GPU step leaves the histories on the device, pbag_eats_flux_a integrates
    them there. The CPU figure is the oracle's restatement of the reference's
    EATS integrator on one host core over a sample of the queries; the
    line's parity compares the GPU light curve with the oracle's on that
    sample (same histories). With the default inputs (the reference
    program's run) the layers, dynamics and EATS options are the run's, and
    the parity also holds the GPU light curve at the run's own observer
    times against the light curve the reference program wrote."""
    import torch
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from pyblastafterglowmag_gb300 import _lib, abi, build, histories as H
    build.build()
    pyoracle.build_oracle()
    orc = pyoracle.Oracle()
    cfg, recs, off, prm, grid = workload(args.inputs)
    dev = torch.device("cuda", 0)
    ctx = _lib.Context(grid, device=0, ssc=True)
    nrec = len(recs)
    d_recs = torch.from_numpy(recs.view(np.uint8).copy()).to(dev)
    d_prm = torch.from_numpy(prm.view(np.uint8).copy()).to(dev)
    d_out = {k: torch.zeros((nrec, grid.nfreq), dtype=torch.float64, device=dev) for k in ("j_all", "a_all")}
    ctx.run_device(d_prm.data_ptr(), len(prm), off, d_recs.data_ptr(), {k: v.data_ptr() for k, v in d_out.items()})
    run = None
    if args.inputs == "driver":
        # the reference run's layers, dynamics and parfile EATS options
        run = driver_run()
        layers, dyn, q_run = run.eats()
        o = run.eats_opts()
    else:
        layers, dyn = H.eats_inputs(cfg, recs, off)
        o = abi.EatsOpts()
        o.theta_obs, o.z, o.d_l = np.deg2rad(20.8), 0.0, 3.09e26
        o.rtol_theta = o.rtol_phi = 1e-6
        o.counter_jet = 1
        o.flux.shock_vel, o.flux.method_ne = abi.PBAG_VEL_SHOCK, abi.PBAG_NE_USE_NE
        o.flux.method_tau = abi.PBAG_TAU_APPROX
    o.method_quad = abi.PBAG_QUAD_CADRE if args.quad == "cadre" else abi.PBAG_QUAD_TRAP_FIXED
    o.nmax_theta = o.nmax_phi = 1000 if args.quad == "cadre" else 100
    t_obs = np.logspace(np.log10(3e3), np.log10(1e9), args.lc_times)
    q = np.zeros(len(layers) * len(t_obs), dtype=abi.EATS_QUERY_DTYPE)
    q["layer"] = np.repeat(np.arange(len(layers)), len(t_obs))
    q["t_obs"] = np.tile(t_obs, len(layers))
    q["nu_obs"] = 1e15
    d_dyn = torch.from_numpy(np.ascontiguousarray(dyn)).to(dev)
    d_q = torch.from_numpy(q.view(np.uint8).copy()).to(dev)
    d_f = torch.zeros(len(q), dtype=torch.float64, device=dev)

    def one_pass():
        _lib.eats_flux_a(ctx, o, layers, d_dyn.data_ptr(), dyn.shape[-1], off, d_out["j_all"].data_ptr(),
                         d_out["a_all"].data_ptr(), len(q), d_q.data_ptr(), d_f.data_ptr())

    for _ in range(args.warmup):
        one_pass()
    ms = []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize(dev)
            e0.record()
            one_pass()
            e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
    t = statistics.median(ms)
    got = d_f.cpu().numpy()
    # the oracle on a sample: every 4th observer time of every layer
    sel = np.flatnonzero(np.tile(np.arange(len(t_obs)) % 4 == 0, len(layers)))
    j, a = d_out["j_all"].cpu().numpy(), d_out["a_all"].cpu().numpy()
    t0 = time.perf_counter()
    rc, fail, ref = orc.eats_flux(grid, o, layers, dyn, off, j, a, q[sel])
    cpu_s = time.perf_counter() - t0
    rel = np.abs(got[sel] - ref) / ref
    parity = {"max_rel": float(rel.max()), "oracle_status": int(rc), "tol": 1e-5,
              "ok": bool(rc == 0 and rel.max() <= 1e-5)}
    if run is not None and args.quad == "cadre":
        # the reference program's own light curve of the run (every layer at
        # its recorded observer times), from the GPU step's histories
        d_qr = torch.from_numpy(q_run.view(np.uint8).copy()).to(dev)
        d_fr = torch.zeros(len(q_run), dtype=torch.float64, device=dev)
        _lib.eats_flux_a(ctx, o, layers, d_dyn.data_ptr(), dyn.shape[-1], off, d_out["j_all"].data_ptr(),
                         d_out["a_all"].data_ptr(), len(q_run), d_qr.data_ptr(), d_fr.data_ptr())
        lc = run.lc.ravel()
        parity["vs_reference_program"] = {"points": int(len(lc)),
                                          "max_rel": float(np.max(np.abs(d_fr.cpu().numpy() - lc) / lc)),
                                          "tol": 1e-4}
    line = {"metric": "EATS light-curve points/s (adaptive quadrature) on 1 GB300", "value": len(q) / (t * 1e-3),
            "unit": "points/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"eats-lc-gaussian-jet-21-layers-fs-rs-{args.quad}",
                       "layers": len(layers), "lc_times": len(t_obs), "queries": len(q), "theta_obs_deg": 20.8,
                       "nu_obs": 1e15, "quadrature": args.quad, "nmax": o.nmax_phi, "rtol": o.rtol_phi,
                       "counter_jet": True, "histories": "the GPU step's, device-resident",
                       "inputs": INPUTS[args.inputs]},
            "clocks": clk.summary(),
            "cpu_baseline": {"value": len(sel) / cpu_s, "unit": "points/s", "cores": 1, "kind": "port",
                             "sample": f"{len(sel)} of the {len(q)} queries (every 4th observer time), the oracle's "
                                       "restatement of the reference's EATS integrator (equal to it bit for bit)"},
            "parity": parity}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------- bw-rhs arm ---
def bw_rhs_arm(args):
    """The blastwave ODE right-hand side (rhs_fs / rhs_fsrs with the
    radiative-loss term) over args.rhs_states blastwave states on the GPU, one
    thread per state: the Gaussian jet's right-hand-side evaluations as the
    reference program sampled them (refdrv_gaussian.npz: forward-shock and
    forward+reverse-shock layers), drawn with replacement and perturbed
    (R, Gamma, Eint2, M2 by 1e-3 relative), resident in HBM. The CPU figure is
    the same restatement on the host (pbag_bw_rhs) on a sample, one core; the
    parity compares a sample of the GPU's derivatives with the host's and the
    reference's own sampled evaluations with the GPU's."""
    import torch
    from pyblastafterglowmag_gb300 import _lib, abi, build
    build.build()
    z = np.load(DRIVER_RUN)
    P, B, A, D = z["rhs_pars"], z["rhs_before"], z["rhs_after"], z["rhs_dydt"]
    rng = np.random.default_rng(11)
    n = args.rhs_states
    idx = rng.integers(0, len(P), n)
    P2, B2 = P[idx].copy(), B[idx].copy()
    for q in ("R", "Gamma", "Eint2", "M2"):
        k = abi.BW_Q.index(q)
        B2["Y"][:, k] *= 1.0 + 1e-3 * rng.standard_normal(n)
    gk = abi.BW_Q.index("Gamma")
    B2["Y"][:, gk] = np.maximum(B2["Y"][:, gk], 1.0 + 1e-6)
    dev = torch.device("cuda", 0)
    ctx = _lib.Context(driver_run().grid, device=0, ssc=False)
    d_p = torch.from_numpy(P2.view(np.uint8).copy()).to(dev)
    h_s = torch.from_numpy(B2.view(np.uint8).copy())
    d_s0 = h_s.to(dev)
    d_s = d_s0.clone()
    d_y = torch.zeros((n, abi.PBAG_Y_N), dtype=torch.float64, device=dev)

    def one_pass():
        d_s.copy_(d_s0)  # the carried members start from the same values every pass
        _lib.bw_rhs_device(ctx, n, d_p.data_ptr(), d_s.data_ptr(), d_y.data_ptr())

    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    for _ in range(args.warmup):
        one_pass()
    ms = []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize(dev)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            one_pass()
            e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
    t = statistics.median(ms)
    # end to end: host states in (pinned), derivatives and states out
    h_p = torch.from_numpy(P2.view(np.uint8).copy()).pin_memory()
    h_s = h_s.pin_memory()
    h_y = torch.empty((n, abi.PBAG_Y_N), dtype=torch.float64).pin_memory()
    h_s_out = torch.empty_like(h_s).pin_memory()

    def e2e_pass():
        d_p.copy_(h_p, non_blocking=True)
        d_s.copy_(h_s, non_blocking=True)
        _lib.bw_rhs_device(ctx, n, d_p.data_ptr(), d_s.data_ptr(), d_y.data_ptr())
        h_y.copy_(d_y, non_blocking=True)
        h_s_out.copy_(d_s, non_blocking=True)
        torch.cuda.synchronize(dev)

    e2e_pass()
    e2e = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        e2e_pass()
        e2e.append(time.perf_counter() - t0)
    e2e_s = statistics.median(e2e)
    # parity: the host restatement on a sample of the batch, the reference's own evaluations
    sel = rng.integers(0, n, 20000)
    t0 = time.perf_counter()
    ref_y, ref_after = _lib.bw_rhs(P2[sel], B2[sel])
    cpu_s = time.perf_counter() - t0
    got = d_y.cpu().numpy()[sel]
    writes = np.zeros((len(sel), abi.PBAG_Y_N), dtype=bool)
    for t_, names in ((abi.PBAG_BW_FS, abi.BW_Q_FS), (abi.PBAG_BW_FSRS, abi.BW_Q_FSRS)):
        for q in names:
            writes[P2["type"][sel] == t_, abi.BW_Q.index(q)] = True
    den = np.abs(ref_y)
    rel = np.where(den > 0, np.abs(got - ref_y) / np.where(den > 0, den, 1.0), np.abs(got))[writes]
    d_p1 = torch.from_numpy(P.view(np.uint8).copy()).to(dev)
    d_s1 = torch.from_numpy(B.view(np.uint8).copy()).to(dev)
    d_y1 = torch.zeros((len(P), abi.PBAG_Y_N), dtype=torch.float64, device=dev)
    _lib.bw_rhs_device(ctx, len(P), d_p1.data_ptr(), d_s1.data_ptr(), d_y1.data_ptr())
    g1 = d_y1.cpu().numpy()
    w1 = np.zeros_like(g1, dtype=bool)
    for t_, names in ((abi.PBAG_BW_FS, abi.BW_Q_FS), (abi.PBAG_BW_FSRS, abi.BW_Q_FSRS)):
        for q in names:
            w1[P["type"] == t_, abi.BW_Q.index(q)] = True
    den1 = np.abs(D)
    rel1 = np.where(den1 > 0, np.abs(g1 - D) / np.where(den1 > 0, den1, 1.0), np.abs(g1))[w1]
    ctx.close()
    bytes_per = abi.BW_RHS_PARS_DTYPE.itemsize + 2 * abi.BW_RHS_STATE_DTYPE.itemsize + 2 * 8 * abi.PBAG_Y_N
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = n * bytes_per / (t * 1e-3) / 1e9
    line = {"metric": "blastwave ODE right-hand-side evaluations/s on 1 GB300", "value": n / (t * 1e-3),
            "unit": "evaluations/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "bw-rhs-gaussian-jet-fs-fsrs", "states": n,
                       "fsrs_fraction": float(np.mean(P2["type"] == abi.PBAG_BW_FSRS)),
                       "inputs": "the reference program's sampled right-hand-side evaluations of the 21-layer "
                                 "Gaussian jet, drawn with replacement, R/Gamma/Eint2/M2 perturbed by 1e-3",
                       "l2": "flushed with a 256 MiB device write before every timed pass"},
            "clocks": clk.summary(),
            "e2e": {"value": n / e2e_s, "unit": "evaluations/s",
                    "h2d_bytes_per_step": int(h_p.numel() + h_s.numel()),
                    "d2h_bytes_per_step": int(h_y.numel() * 8 + h_s_out.numel())},
            "gpu_launches": args.steps,
            "roofline": {"bound": "hbm", "kernel": "k_bw_rhs", "achieved": achieved, "peak": hbm_peak,
                         "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": None,
                         "bytes_per_state": bytes_per,
                         "note": "FP64-bound in practice (transcendentals per state); the HBM figure is the "
                                 "algorithmic bytes of one evaluation"},
            "cpu_baseline": {"value": len(sel) / cpu_s, "unit": "evaluations/s", "cores": 1, "kind": "port",
                             "sample": f"{len(sel)} of the {n} states through pbag_bw_rhs on one host core (the "
                                       "restatement equal bit for bit to the reference's rhs_fs evaluations)"},
            "parity": {"max_rel_vs_host": float(rel.max()), "max_rel_vs_reference": float(rel1.max()),
                       "reference_evaluations": int(len(P)), "tol": 1e-9,
                       "ok": bool(rel.max() <= 1e-9 and rel1.max() <= 1e-9)}}
    print(json.dumps(line), flush=True)


def timeit_run(ctx, recs, off, prm):
    t0 = time.perf_counter()
    ctx.run(recs, off, prm, outputs=("j_all", "a_all", "f_all", "i_all"))
    return time.perf_counter() - t0


def main():
    args = parse()
    if args.workload == "surrogate":
        surrogate_arm(args)
        return
    if args.workload == "eats-lc":
        eats_arm(args)
        return
    if args.workload == "bw-rhs":
        bw_rhs_arm(args)
        return
    if args.workload == "contraction":
        contraction_arm(args)
    elif args.workload == "uneven-sweep":
        sweep_arm(args)
    elif args.impl == "reference":
        reference_arm(args)
    else:
        gb300_arm(args)


if __name__ == "__main__":
    main()
