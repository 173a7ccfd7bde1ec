#!/usr/bin/env python
"""Benchmark of the Chebyshev propagation step on GB300.

A step is one Chebyshev iteration of every partial wave of the workload: H psi
(difs), the damped three-term update, CoefEcheby and the flux/Cvj/norm
accumulators (SRC/main_madwave3.f:324-352).  The metric is stored grid
points x iterations per second, a stored point being one entry of the
reference's compressed state vector (one Omega/electronic block at one grid
point kept below Vcut).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]
                  [--workload NAME] [--precision mixed|fp64]

--impl reference times the CPU restatement of the same step (oracle/, all host
threads) on the same workload.  With --gpus N > 1 (torchrun) the partial waves
are independent, so each rank propagates its own replica of the workload
("replicas only": the path has no exchange step on one node).
"""
import argparse
import datetime
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

L2_BYTES = 129 * 1024 * 1024
FP64_NOMINAL_TFLOPS = 1.25
# FP32 CUDA-core rate at the maximum SM clock: 152 SMs x 128 lanes x 2 flop x 2.07 GHz
FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12

# DRAM bytes per stored point and launch of the mixed path's top kernels, from
# one ncu capture (dram__bytes_read.sum + dram__bytes_write.sum) of the J=0..4
# sweep; the per-block structure of the full sweep is the same, so the traffic
# scales with the stored points (the ncu summaries of each kernel on that sweep)
TRAFFIC_PER_POINT = {"dst_R": 16.0, "angular": 16.6, "update": 27.9}

WORKLOADS = {
    # partial-wave sweep J=0..40, Omega=0..min(J,6): 266 blocks on 256 R x 128 r x 60 angles
    "jsweep0-40_256x128x60": dict(case="j0_256x128x60", sweep=list(range(0, 41))),
    # the first five partial waves of that sweep (15 blocks): a profiling-sized case
    "jsweep0-4_256x128x60": dict(case="j0_256x128x60", sweep=list(range(0, 5))),
    # J=0, one Omega block, one state: 256 R x 128 r x 60 angles (synthetic LEPS)
    "j0_256x128x60": dict(case="j0_256x128x60", sweep=None),
    # J=0 at 512 R x 256 r x 120 angles
    "j0_512x256x120": dict(case="j0_512x256x120", sweep=None),
    # J=10 with Omega=0..10 Coriolis-coupled: 11 blocks on 256 R x 128 r x 60 angles
    "j10_256x128x60": dict(case="j10_256x128x60", sweep=None),
    # three diabatic states, J=2 with Omega=0..2, 384 R x 192 r x 80 angles, started from the
    # lowest J=1 bound state of the ground surface times a constant transition dipole of 1 a.u.
    "e3_384x192x80_photo": dict(case="e3_384x192x80", sweep=None, photo=True),
}
DEFAULT_WORKLOAD = "jsweep0-40_256x128x60"


def metric_name():
    return "Chebyshev Hψ grid-pt·iter/s, mixed/batched vs FP64 plain at |ΔP(E)|≤1e-4"


def load_peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p.get("hbm_gbs", 6800.0), p.get("bf16_tflops", 1900.0), "of measured"
    except Exception:
        return 6800.0, 1900.0, "of fallback"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def case_runs(workload, rank):
    from madwave3_gb300.host import generator, setup
    w = WORKLOADS[workload]
    base = os.environ.get("MW3_CASES", os.path.join(tempfile.gettempdir(), "mw3_cases_r%d" % rank))
    if w.get("photo"):
        from madwave3_gb300 import workloads
        return [workloads.photodissociation(base, w["case"])[0]]
    d = os.path.join(base, w["case"])
    if not os.path.exists(os.path.join(d, "pot", "cont.pot")):
        generator.write_case(d, **generator.CASES[w["case"]])
    if w["sweep"] is None:
        return [setup.load(os.path.join(d, "input.dat"))]
    return setup.load_sweep(os.path.join(d, "input.dat"), w["sweep"], generator.jsweep_inputs)


def sample_waves(runs, n=5):
    """Waves spread over a sweep (first, last and evenly between) for CPU samples."""
    if len(runs) <= n:
        return list(runs)
    idx = sorted(set(int(round(x)) for x in np.linspace(0, len(runs) - 1, n)))
    return [runs[i] for i in idx]


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 50 ms from before
    the warm-up; the summary keeps the samples whose timestamps fall inside the
    timed region (marked by start() and end(), 100 ms of slack each side)."""

    def __init__(self, gpu_index):
        self.path = os.path.join(tempfile.gettempdir(), "mw3_clocks_%d_%d.csv" % (os.getpid(), gpu_index))
        q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        self.t0 = self.t1 = None
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + q,
                                       "--format=csv,noheader,nounits", "-lms", "50"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def wait_first(self, timeout=5.0):
        """Until the first sample is written (nvidia-smi takes a moment to start)."""
        t = time.time()
        while self.p is not None and time.time() - t < timeout:
            if os.path.getsize(self.path) > 0:
                return
            time.sleep(0.05)

    def start(self):
        self.t0 = datetime.datetime.now()

    def end(self):
        self.t1 = datetime.datetime.now()

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.15)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 10:
                    continue
                try:
                    ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f")
                    rows.append((ts, float(parts[2]), float(parts[3]), parts[6:10]))
                except ValueError:
                    continue
        os.unlink(self.path)
        slack = datetime.timedelta(seconds=0.1)
        inside = [r for r in rows if self.t0 is not None and self.t1 is not None
                  and self.t0 - slack <= r[0] <= self.t1 + slack]
        use = inside or rows
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in use for n, v in zip(names, r[3]) if v.lower() == "active"})
        return {"sm_mhz": float(np.median([r[1] for r in use])) if use else None,
                "sm_max_mhz": float(max(r[2] for r in use)) if use else None,
                "reasons": reasons, "samples": len(use),
                "window": "timed region" if inside else "whole run (no sample inside the timed region)"}


def stage_model(runs, prop, kin):
    """Algorithmic work of each stage of one iteration (flops or bytes).

    The angular stage is counted as bytes when the mixed path runs it as the
    factorised tensor-core contraction (kin["tc_angular"]; the l^2 stage then
    measures ~0): psi read at every stored point in FP32 and H read and written,
    20 bytes per stored point.  The explicit form is counted in flops."""
    r0 = runs[0]
    i = r0.inp
    n1, n2, na = i.npun1, i.npun2, i.nangu
    tsz = 8 if prop.precision == "fp64" else 4
    rows = 0
    rows_sq = 0
    nsto = 0
    for w, r in enumerate(runs):
        nopr1 = prop.tables(w)["nopr1"].astype(np.int64)
        rows += r.ncan * int(nopr1.sum())
        rows_sq += r.ncan * int((nopr1 ** 2).sum())
        nsto += r.ntot
    ne = r0.nelec
    fused = prop.precision != "fp64" and kin["tc_angular"]
    return {
        # the fused radial kernel does all four DST products in stage 0
        "dst_R": ("flop", 4.0 * rows * n2 * n2 + 4.0 * rows_sq * n2) if kin["tc_dst_fused"]
        else ("flop", 2.0 * rows * n2 * n2),
        "dst_r_pair": ("flop", 4.0 * rows_sq * n2),
        "dst_R_gather": ("flop", 2.0 * rows * n2 * n2),
        "angular": (("byte", 20.0 * nsto) if fused else ("flop", 2.0 * na * nsto)),
        "angular_l2": ("flop", 2.0 * na * nsto * 3),
        # FP64 path: psi_k, psi_k-1, H read, psi_k+1 written, V row, rectangle store, two
        # grid indices.  Mixed path: two grid indices, H (FP32), per source the FP32
        # potential and FP32 psi_k, psi_k-1 (FP64), psi_k+1 (FP64 and FP32), rectangle (FP32)
        "update": ("byte", nsto * (8 * 4 + 8 * ne + tsz + 8)) if prop.precision == "fp64"
        else ("byte", nsto * (8 + 4 + 8 * ne + 8 + 8 + 4 + 4)),
        "accumulators": ("byte", sum(prop.nflux(w) * r.inp.netot * 2 * 2 * 16 for w, r in enumerate(runs))),
    }


def dominant_roofline(stages, nrec, model, kin, precision, nsto, peaks):
    """Roofline of the stage that takes the most time per iteration, against the
    unit that executes it: the FP64 pipe (FP64 path), the tensor cores (mixed-path
    DSTs on tcgen05), the FP32 CUDA cores (mixed-path CUDA-core DSTs and explicit
    angular kernels) or HBM (stages counted in bytes).  stages: total ms per
    stage over nrec iterations; model: stage_model's (kind, work) per stage."""
    hbm, tf, src = peaks
    dom = max(stages, key=lambda k: stages[k])
    kind, work = model[dom]
    t_launch = stages[dom] / max(nrec, 1) * 1e-3
    on_tensor = dom.startswith("dst") and kin["tc_dst"]
    traffic = None
    if precision == "mixed" and kin["tc_dst_fused"] and kin["tc_angular"] and dom in TRAFFIC_PER_POINT:
        traffic = TRAFFIC_PER_POINT[dom] * nsto
    flops = ("algorithmic flops of the stage's dense products (DST along R: 2 nopr1 npun2^2 per slab%s; "
             "r1 pair: 4 nopr1^2 npun2; explicit angular: 2 nangu per stored point, the l^2 stage for up "
             "to three coupled blocks)")
    if kind == "flop" and precision == "fp64":
        # the FP64 path's transforms run on the FP64 pipe: against its nominal rate
        # (the measured peaks hold no FP64 figure)
        achieved = work / t_launch / 1e12
        return {"bound": "fp64", "achieved": achieved, "peak": FP64_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                "frac": achieved / FP64_NOMINAL_TFLOPS, "traffic": traffic, "kernel": dom,
                "peak_source": "nominal GB300 FP64 rate (not measured)",
                "work": flops % ", run as a Rader FFT with fewer flops when npun2 = 256"}
    if kind == "flop" and not on_tensor:
        achieved = work / t_launch / 1e12
        return {"bound": "fp32", "achieved": achieved, "peak": FP32_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                "frac": achieved / FP32_NOMINAL_TFLOPS, "traffic": traffic, "kernel": dom,
                "peak_source": "nominal GB300 FP32 CUDA-core rate at 2070 MHz (not measured)",
                "work": flops % ""}
    if kind == "flop":
        achieved = work / t_launch / 1e12
        return {"bound": "tensor", "achieved": achieved, "peak": tf, "unit": "TFLOP/s",
                "frac": achieved / tf, "traffic": traffic, "kernel": dom, "peak_source": src,
                "work": "algorithmic DST flops (4 nopr1 npun2^2 + 4 nopr1^2 npun2 per slab); the kernel issues "
                        + ("3 FP16 products per flop (split FP16, kind::f16 at the bf16 rate)" if kin.get("dst_f16")
                           else "3 TF32 products per flop (3xTF32, kind::tf32 at half the bf16 rate)")
                        + ", and the peak is the dense bf16 one"}
    achieved = work / t_launch / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "traffic": traffic, "kernel": dom, "peak_source": src}


RING = 32   # iterations in one cycle of the Cvj ring and in one captured CUDA-graph block


def warmup_count(it_now, warmup, steps):
    """Untimed iterations before the timed window: at least ``warmup``, then up to
    the iteration where the window must start.  A window of a multiple of 32
    steps starts at an iteration that is a multiple of 32 (whole ring cycles,
    replayed as CUDA graphs; one block is run first so the graph is captured
    outside the timing); a shorter or ragged window ends on the iteration
    congruent to 31 mod 32, so the once-per-cycle Cvj flush falls inside it."""
    target = 0 if steps % RING == 0 else (RING - 1 - steps) % RING
    w = warmup
    while (it_now + w) % RING != target:
        w += 1
    if steps >= RING and steps % RING == 0:
        w += RING
    return w


# context counts (one CUDA stream and one host thread each) the end-to-end leg
# tries when it splits the waves, so that copies and kernels of different
# contexts overlap; which is faster depends on the box (measured: 4 gave 9.3 ms
# and 8 gave 12.7 ms on one, 13.2 and 9.0 ms on another)
E2E_CONTEXTS = (4, 8)


def run_e2e(runs, precision, nctx, steps, choices=None):
    """End to end through the C-ABI with host buffers: the host owns every wave's
    psi_k (pinned) and each step hands it in, runs one iteration and reads the
    new psi_k back (psi_k-1 stays the device's own).  The waves are split over
    nctx contexts, each driven by its own host thread (the library's calls
    release the interpreter lock and wait on their own stream), so one context's
    copies overlap the other contexts' kernels and the two directions of the
    host link overlap each other.  Host wall time over the steps of all
    contexts; returns (ms per step, contexts)."""
    import threading
    import torch
    from madwave3_gb300 import Propagator, replicas

    parts = replicas.partition([float(r.ntot) for r in runs], nctx) if nctx > 1 else [list(range(len(runs)))]
    props, bufs, its = [], [], []
    for part in parts:
        if not part:
            continue
        p = Propagator([runs[i] for i in part], precision)
        if choices:
            p.set_choices(choices)
        p.start()
        p.run(RING)
        _, k, it = p.state_all()
        props.append(p)
        bufs.append([torch.from_numpy(k).pin_memory(), torch.empty(k.size, dtype=torch.float64).pin_memory()])
        its.append(it)
    errors = []

    def drive(i):
        try:
            p, (a, b) = props[i], bufs[i]
            for s in range(steps):
                p.upload_state_all(None, a.numpy(), its[i] + s)
                p.run(1)
                p.state_k_all(b.numpy())
                a, b = b, a
        except Exception as e:      # re-raised on the main thread
            errors.append(e)

    torch.cuda.synchronize()
    threads = [threading.Thread(target=drive, args=(i,)) for i in range(len(props))]
    t0 = time.perf_counter()
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    ms = (time.perf_counter() - t0) * 1e3 / steps
    for p in props:
        p.close()
    if errors:
        raise errors[0]
    return ms, len(props)


def run_gpu(args, rank, world, local):
    import torch
    from madwave3_gb300 import Propagator, replicas

    torch.cuda.set_device(local)
    all_runs = case_runs(args.workload, rank)
    nsto_job = sum(r.ntot for r in all_runs)
    if world > 1 and len(all_runs) >= world:
        # the partial waves are independent: each rank propagates its share of the
        # sweep (longest-processing-time split by stored points), no exchange
        part = replicas.partition([float(r.ntot) for r in all_runs], world)
        runs = [all_runs[i] for i in part[rank]]
        scaling, parallelism = "strong", "partial waves split over %d GPUs" % world
    else:
        runs = all_runs
        scaling = "weak"
        parallelism = "replicas" if world > 1 else "single GPU"
        nsto_job = world * nsto_job
    nsto = sum(r.ntot for r in runs)
    prop = Propagator(runs, args.precision)
    tune = None
    if args.autotune != "none":
        # the project's autotuner: every distinct path of the scope timed over 64
        # synthetic iterations of this workload, the fastest kept (before the start)
        t0 = time.perf_counter()
        choice, ms_tuned = prop.autotune(iterations=64, scope=args.autotune)
        tune = {"scope": args.autotune, "choice": choice, "ms_per_iteration": ms_tuned,
                "seconds": time.perf_counter() - t0}
    prop.start()
    working_set = nsto * 8 * 4
    flush = working_set < 2 * L2_BYTES
    nwarm = warmup_count(1, args.warmup, args.steps) if not flush else args.warmup
    clocks = ClockSampler(local)
    clocks.wait_first()
    prop.run(nwarm)
    prop.sync()
    it0 = 1 + nwarm
    stream = torch.cuda.ExternalStream(prop.stream())
    fbuf = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda") if flush else None
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = prop.kernel_launches()
    clocks.start()
    if flush:
        # a small workload: L2 flushed before every step, each step timed alone
        evs = []
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                fbuf.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            prop.run(1)
            e1.record(stream)
            evs.append((e0, e1))
        prop.sync()
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in evs)
    else:
        # inputs larger than L2: the K steps back to back as the production loop
        # runs them (whole ring cycles replay as CUDA graphs)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        prop.run(args.steps)
        e1.record(stream)
        prop.sync()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
    clocks.end()
    clk = clocks.stop()
    launches = prop.kernel_launches() - launches0
    t = torch.tensor([ms], dtype=torch.float64, device="cuda")
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.barrier()
    ms_max = float(t.item())
    ms_step = ms_max / args.steps
    value = nsto_job * args.steps / (ms_max * 1e-3)

    # stage breakdown: one more ring cycle with per-stage events (untimed; event
    # recording switches graph replay off)
    prop.profile(True)
    prop.run(RING)
    stages, nrec = prop.stage_times()
    prop.profile(False)

    # roofline of the dominant stage, against the unit that executes it
    hbm, tf, src = load_peaks()
    kin = out_kernels = prop.path()
    roof = dominant_roofline(stages, nrec, stage_model(runs, prop, kin), kin, args.precision, nsto,
                             (hbm, tf, src))
    # the whole iteration against HBM (the fused ideal's bytes: psi_k-1 and psi_k
    # read, psi_k+1 written, the V rows a state's Omega blocks share) and the angular
    # DVR <-> basis transforms as tensor work (dense contractions over the rectangles,
    # split products counted once), as the hot-path scope defines them
    b_iter = sum(r.ntot * 8.0 * (3.0 + r.nelec / max(1.0, r.ncan / r.nelec)) for r in runs)
    i0 = runs[0].inp
    f_ang = 4.0 * sum(r.ncan for r in runs) * i0.npun1 * i0.npun2 * float(i0.nangu) ** 2
    t_ang = (stages.get("angular", 0.0) + stages.get("angular_l2", 0.0)) / max(nrec, 1) * 1e-3
    scope = {
        "iteration_hbm": {"bytes": b_iter, "achieved": b_iter / (ms_step * 1e-3) / 1e9, "peak": hbm,
                          "unit": "GB/s", "frac": b_iter / (ms_step * 1e-3) / 1e9 / hbm},
        "angular_tensor": {"flop": f_ang, "achieved": f_ang / t_ang / 1e12 if t_ang > 0 else None, "peak": tf,
                           "unit": "TFLOP/s", "frac": f_ang / t_ang / 1e12 / tf if t_ang > 0 else None},
    }
    out = {
        "metric": metric_name(), "value": value, "unit": "grid-pt*iter/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": scaling, "vs_baseline": None,
        "dtype": "f64 recursion, f32 transforms" if args.precision == "mixed" else "f64",
        "data": "synthetic LEPS surface, generated on the fly",
        "config": {"workload": args.workload, "precision": args.precision,
                   "stored_points": nsto_job if scaling == "strong" else nsto,
                   "waves": len(all_runs), "blocks": sum(r.ncan for r in all_runs),
                   "grid": [runs[0].inp.npun2, runs[0].inp.npun1, runs[0].inp.nangu],
                   "netot": runs[0].inp.netot,
                   "l2": "flushed before every timed step" if flush else "working set larger than L2",
                   "window": {"iterations": [it0 + 1, it0 + args.steps], "untimed_warmup_iterations": nwarm,
                              "graph_blocks": (not flush) and args.steps % RING == 0},
                   "parallelism": parallelism},
        "gpu_launches": launches,
        "stages_ms_per_step": {k: v / max(nrec, 1) for k, v in stages.items()},
        "roofline": roof,
        "scope_rooflines": scope,
        "clocks": clk,
    }
    out["config"]["kernels"] = out_kernels
    if tune:
        out["config"]["autotune"] = tune
    prop.close()
    del prop

    # end to end (after the device-resident context is released).  The host link is
    # shared with the rest of the node, so each context count runs three times; the
    # line reports the better count's median and lists every run
    e2e_steps = max(1, min(args.steps, 10))
    e2e_runs = {}
    for n in sorted({min(k, len(runs)) for k in E2E_CONTEXTS}):
        e2e_runs[n] = [run_e2e(runs, args.precision, n, e2e_steps, tune and tune["choice"])[0] for _ in range(3)]
    e2e_ctx = min(e2e_runs, key=lambda n: sorted(e2e_runs[n])[1])
    e2e_ms = sorted(e2e_runs[e2e_ctx])[1]
    if world > 1:
        te = torch.tensor([e2e_ms], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(te, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(te.item())
    e2e_value = nsto_job / (e2e_ms * 1e-3) if scaling == "strong" else world * nsto / (e2e_ms * 1e-3)
    out["e2e"] = {"value": e2e_value, "unit": "grid-pt*iter/s",
                  "h2d_bytes_per_step": int(8 * nsto), "d2h_bytes_per_step": int(8 * nsto),
                  "ms_per_step": e2e_ms, "contexts": e2e_ctx,
                  "ms_per_step_runs": {str(n): v for n, v in e2e_runs.items()},
                  "how": "host-owned psi_k (pinned) in and psi_k+1 out every step through mw3_upload_state_all / "
                         "mw3_run / mw3_download_state_all; waves split over the contexts, one host thread and "
                         "CUDA stream each, host wall time; median of three runs of the steps for each "
                         "context count, the better count reported"}
    if args.precision == "mixed" and args.fp64_steps > 0:
        fp = fp64_plain(runs, args.fp64_steps)
        fp["speedup_mixed_over_fp64"] = nsto * args.steps / (ms_max * 1e-3) / fp["value"]
        out["fp64_plain"] = fp
    if rank == 0 and world == 1 and args.gate_iterations > 0 and args.precision == "mixed":
        out["gate"] = precision_gate(args.gate_iterations)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(sample_waves(runs), seconds=args.cpu_seconds)
    return out


def precision_gate(iterations, case="j0_256x128x60"):
    """|Delta P(E)| of the mixed path against FP64 after a full propagation of the
    J=0 wave on the sweep's grid (the metric's gate); both paths on this GPU."""
    from madwave3_gb300 import gate
    res = gate.run_gate(case, iterations)[0]
    keep = ("case", "iterations", "max_abs_dP", "at_energy_ev", "max_P", "pass_1e-4", "seconds_fp64",
            "seconds_mixed")
    return {k: res[k] for k in keep}


def fp64_plain(runs, steps, warmup=3):
    """The plain FP64 path on the same waves (this GPU's share), for the
    mixed/FP64 ratio."""
    import torch
    from madwave3_gb300 import Propagator
    prop = Propagator(runs, "fp64")
    prop.start()
    for _ in range(warmup):
        prop.run(1)
    prop.sync()
    stream = torch.cuda.ExternalStream(prop.stream())
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    prop.run(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    prop.close()
    nsto = sum(r.ntot for r in runs)
    return {"value": nsto * steps / (ms * 1e-3), "unit": "grid-pt*iter/s",
            "ms_per_step": ms / steps, "steps": steps, "warmup": warmup}


def cpu_baseline(runs, seconds=15.0):
    """The oracle (CPU restatement of the same step), all host threads, bounded sample."""
    from oracle.mw3ref import Oracle
    cores = os.cpu_count() or 1
    total_pts, total_t, its_done = 0, 0.0, 0
    per_wave = seconds / len(runs)
    for r in runs:
        o = Oracle(r, threads=cores)
        o.start(r.psi0)
        t = time.time()
        o.run_iters(1)
        t1 = time.time() - t
        n = max(1, min(200, int(per_wave / max(t1, 1e-6))))
        t = time.time()
        o.run_iters(n)
        dt = time.time() - t
        total_pts += r.ntot * n
        total_t += dt
        its_done += n
        del o
    return {"value": total_pts / total_t, "unit": "grid-pt*iter/s", "cores": cores, "kind": "port",
            "sample": "%d Chebyshev iterations in total, after one warm-up iteration each, over the waves J=%s "
                      "of the workload" % (its_done, ",".join(str(r.inp.Jtot) for r in runs))}


def run_reference(args, rank, world, local):
    if rank != 0:
        return None
    from oracle.mw3ref import Oracle
    runs = sample_waves(case_runs(args.workload, rank))
    cores = os.cpu_count() or 1
    oracles = []
    for r in runs:
        o = Oracle(r, threads=cores)
        o.start(r.psi0)
        oracles.append(o)
    for _ in range(args.warmup):
        for o in oracles:
            o.run_iters(1)
    t = time.time()
    for _ in range(args.steps):
        for o in oracles:
            o.run_iters(1)
    dt = time.time() - t
    nsto = sum(r.ntot for r in runs)
    value = nsto * args.steps / dt
    return {
        "impl": "reference", "metric": metric_name(), "value": value, "unit": "grid-pt*iter/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic LEPS surface, generated on the fly",
        "config": {"workload": args.workload, "stored_points_per_step": nsto, "waves_per_step": len(runs)},
        "cpu_baseline": {"value": value, "unit": "grid-pt*iter/s", "cores": cores, "kind": "port",
                         "sample": "%d timed Chebyshev iterations after %d warm-up, each over the waves J=%s"
                                   % (args.steps, args.warmup, ",".join(str(r.inp.Jtot) for r in runs))},
        "e2e": {"value": value, "unit": "grid-pt*iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fp64-steps", type=int, default=3,
                    help="timed steps of the plain FP64 path on the same workload (0: skip)")
    ap.add_argument("--gate-iterations", type=int, default=2000,
                    help="iterations of the |dP(E)| gate of the mixed path against FP64 on the J=0 wave (0: skip)")
    ap.add_argument("--autotune", default="none", choices=["none", "layout", "form", "all"],
                    help="run the library's autotuner over this scope before the timed context starts")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = dist_env()
    if world > 1:
        import torch
        backend = "gloo" if args.impl == "reference" else "nccl"
        if backend == "nccl":
            torch.cuda.set_device(local)
        torch.distributed.init_process_group(backend=backend)
    if args.impl == "reference":
        out = run_reference(args, rank, world, local)
    else:
        out = run_gpu(args, rank, world, local)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
