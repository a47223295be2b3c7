"""Benchmark of the GB300 monodomain hot path (driver contract).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload (one bench "step" = one whole solve on one GPU): fk_holes_1024 —
Fenton-Karma 3V in FP32 on a 1024x1024 grid, 20,000 explicit Euler steps,
300 circular holes (r ~ U[2,6] cells), 12 S2 patches of 40x40 at seeded
positions and times ~ U[200,400] ms, seeded u ~ U(-0.01, 0.01), v = w = 1,
S1 on columns 0-9 (synthetic: there is no dataset).

Metric: Gcell-steps/s (1024^2 cells x 20,000 steps per solve). The state is
re-initialised from a device copy at the start of every solve and a 256 MB
buffer (> the 129 MB L2) is written between solves; within one solve the
12.6 MB state stays resident in L2, which is the physical behaviour of this
workload, so the HBM roofline fraction computed on algorithmic bytes can
exceed 1 (see `roofline` and the ncu traffic).

N > 1 (torchrun): every rank runs its own replica (the path does not shard);
value = all ranks' cell-steps / the max time over ranks.

--impl reference: the reference has no CPU implementation of this path; its
step semantics are timed as the FP32 C/OpenMP transcription in oracle/ (the
CPU restatement of the reference kernels), on all host cores, on a bounded
sample of the same workload, same metric and unit.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gcell-steps/s"
L2_FLUSH_BYTES = 256 << 20


def env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(key):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/traffic.json), or None."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    v = d.get(key)
    return None if v is None else float(v)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(wl, seconds=10.0):
    """The FP32 C/OpenMP transcription of the step (oracle/, the CPU
    restatement of the reference kernels) on all host cores: a bounded
    sample of the workload's first steps, about `seconds` long."""
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    st = wl.state0()
    steps, elapsed = 0, 0.0
    n = 4
    while elapsed < seconds:
        t0 = time.perf_counter()
        st = O.run(wl.p, wl.model, wl.fk, st, n, wl.stims, wl.solid,
                   step0=steps, dtype=np.float32)
        elapsed += time.perf_counter() - t0
        steps += n
        n = min(n * 2, 256)
    value = wl.cells * steps / elapsed / 1e9
    return {"value": round(value, 4), "unit": METRIC, "cores": cores,
            "kind": "port",
            "sample": "%s: first %d of %d steps (%dx%d with holes), FP32, "
                      "OpenMP %d threads, %.1f s" % (
                          wl.name, steps, wl.nsteps, wl.p.nx, wl.p.ny, cores,
                          elapsed)}


def issue_roofline(key, gcs, clocks, sms=152):
    """The instruction-issue bound of the dominant kernel: warp instructions
    per cell-step from its ncu capture (profiles/traffic.json,
    "warp_inst_per_cell_step") x cell-steps/s, against the issue ceiling of
    one warp instruction per cycle per scheduler (4 per SM) at the SM clock
    sampled during the timed region."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        w = json.load(f).get("warp_inst_per_cell_step", {}).get(key)
    mhz = clocks.get("sm_mhz") if clocks else None
    if w is None or not mhz:
        return None
    achieved = gcs * 1e9 * w
    peak = sms * 4 * mhz * 1e6
    return {"warp_inst_per_cell_step": w,
            "thread_inst_per_cell_step": round(32 * w, 1),
            "achieved_warp_inst_per_s": round(achieved / 1e12, 4),
            "peak_warp_inst_per_s": round(peak / 1e12, 4), "unit": "T/s",
            "frac": round(achieved / peak, 4), "sm_mhz": mhz,
            "note": "warp instructions per cell-step from ncu x cell-steps/s "
                    "over %d SMs x 4 schedulers x 1 issue/cycle at the "
                    "sampled SM clock" % sms}


def config_of(wl, args, tb, autotuned=False, engine="cpu"):
    state_mb = 12.0 * wl.cells / 2 ** 20
    return {"workload": wl.name, "grid": [wl.p.nx, wl.p.ny],
            "steps_per_solve": wl.nsteps, "model": "FK3V",
            "holes": 0 if wl.solid is None else int(round(300 * wl.cells / 2 ** 20)),
            "s2_patches": len(wl.stims),
            "cells": wl.cells, "dt_ms": wl.p.dt, "dx_cm": wl.p.hx,
            "engine": engine, "time_block": tb, "engine_autotuned": autotuned,
            "l2": "256 MB write between solves; %.1f MB state%s within a solve" % (
                state_mb, " L2-resident" if 2 * state_mb < 100 else ""),
            "parallelism": "replicas x%d" % args.gpus}


def max_over_ranks(x, dist, device):
    """The largest of one float per rank (the job's time is its slowest
    rank's); x itself without a process group."""
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(cells, nsteps, solves, world, seconds):
    """Whole-job Gcell-steps/s: every rank advances its own replica of
    `cells` cells by nsteps steps, `solves` times, in `seconds` (the
    slowest rank's time)."""
    return cells * nsteps * solves * world / seconds / 1e9


def reference_gpu(n=1024, steps=200, warmup=20):
    """The reference's own reactionDiffusion_kernel (built from its sources
    into oracle/_ref, launched headless with its 16x16 blocks, one launch per
    step as reactionDiffusion_wrapper does) on the GB300: REF2V in FP64, the
    reference's model and precision (it has no FK3V), n x n cells, the
    reference's default parameters and cross-field initial condition. None
    without a GPU or without the built reference."""
    try:
        import torch
        from oracle import refgpu as R
    except Exception:
        return None
    if not torch.cuda.is_available() or not R.available():
        return None
    from yolohtli_gb300 import _abi as A
    from yolohtli_gb300 import workloads as W
    p = A.param_defaults(n, n)
    p.Lx = p.Ly = 3.0
    p.hx = p.hy = 3.0 / (n - 1)
    p = A.param_derive(p)
    st = W.ref2v_cross(n, n)
    a = [torch.tensor(np.asarray(x, np.float64), device="cuda") for x in st]
    b = [torch.zeros_like(a[0]) for _ in range(2)]
    J = [torch.zeros_like(a[0]) for _ in range(2)]
    vt = [torch.zeros_like(a[0]) for _ in range(2)]
    R.set_params(p)
    for k in range(warmup + steps):
        if k == warmup:
            R.sync()
            t0 = time.perf_counter()
        R.rd(p, b, a, J, vt)
        a, b = b, a
    R.sync()
    dt = time.perf_counter() - t0
    return {"value": round(n * n * steps / dt / 1e9, 3), "unit": METRIC,
            "kernel": "reactionDiffusion_kernel (the reference's own, "
                      "compiled from its sources for sm_103a)",
            "model": "REF2V FP64 (the reference's model; it has no FK3V)",
            "grid": [n, n], "steps": steps,
            "launch": "16x16 blocks, one launch per step, host-timed over "
                      "%d launches after %d warm-up" % (steps, warmup)}


def dropin_gpu(n=1024, steps=200, warmup=20):
    """This library's FP64 drop-in of reactionDiffusion_wrapper (the
    reference's C++ symbol, include/yolohtli_compat.h) on the case and loop
    of reference_gpu: REF2V FP64, n x n cells, one call per step, host-timed.
    None without a GPU."""
    try:
        import torch
        from yolohtli_gb300 import _abi as A
        from yolohtli_gb300 import workloads as W
        from yolohtli_gb300.compat import B2, G2, Compat, Int2, sv
    except Exception:
        return None
    if not torch.cuda.is_available():
        return None
    p = A.param_defaults(n, n)
    p.Lx = p.Ly = 3.0
    p.hx = p.hy = 3.0 / (n - 1)
    p = A.param_derive(p)
    cp = Compat()
    cp.set_params(p)
    st = W.ref2v_cross(n, n)
    a = [torch.tensor(np.asarray(x, np.float64), device="cuda") for x in st]
    b = [torch.zeros_like(a[0]) for _ in range(2)]
    J = [torch.zeros_like(a[0]) for _ in range(2)]
    vt = [torch.zeros_like(a[0]) for _ in range(2)]
    rd = cp.f["rd"]
    for k in range(warmup + steps):
        if k == warmup:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
        rd(0, G2, B2, sv(*b), sv(*a), sv(*J), sv(*vt), False, None, False,
           None, False, Int2(0, 0))
        a, b = b, a
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    if cp.err() != 0:
        return {"unavailable": "drop-in returned status %d" % cp.err()}
    return {"value": round(n * n * steps / dt / 1e9, 3), "unit": METRIC,
            "kernel": "rd_step_scalar<REF2V, double> through the drop-in "
                      "reactionDiffusion_wrapper",
            "model": "REF2V FP64", "grid": [n, n], "steps": steps,
            "launch": "one call per step, host-timed over %d calls after %d "
                      "warm-up (as reference_gpu)" % (steps, warmup)}


def run_reference(args, wl):
    rank = env_int("RANK", 0)
    if rank != 0:
        return
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    # consecutive windows of the solve: bench step k advances the state by
    # the next sample_steps steps (stimulus events included), so the sample
    # covers the first (warmup + steps) x sample_steps steps of the run
    sample_steps = 256
    st = wl.state0()
    times = []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        st = O.run(wl.p, wl.model, wl.fk, st, sample_steps, wl.stims, wl.solid,
                   step0=k * sample_steps, dtype=np.float32)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(dt)
    total = sum(times)
    value = wl.cells * sample_steps * len(times) / total / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4),
        "unit": METRIC, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * total / len(times), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": config_of(wl, args, 1),
        "cpu_baseline": {
            "value": round(value, 4), "unit": METRIC, "cores": cores,
            "kind": "port",
            "sample": "each step: the next %d steps of %s (steps 0-%d over "
                      "the run, the S2 patches included) on the host cores, "
                      "FP32 C/OpenMP transcription of the reference step "
                      "(the reference has no CPU path)" % (
                          sample_steps, wl.name,
                          (args.warmup + args.steps) * sample_steps)},
        "e2e": {"value": round(value, 4), "unit": METRIC,
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    rg = reference_gpu()
    if rg is not None:
        line["reference_gpu"] = rg
    print(json.dumps(line), flush=True)


def batch_measure(nsteps, solves, warmup, dist, world, loops=True,
                  engine="auto"):
    """The batched workload (fk_batch_256: 256 FK3V grids of 128^2 .. 768^2,
    `nsteps` steps): the batched solver (schedule autotuned on the initial
    state), then, with `loops`, a loop of single-grid solvers on one shared
    stream and on one stream per grid, all on this GPU. Returns a dict."""
    import torch
    from yolohtli_gb300 import _abi as A
    from yolohtli_gb300 import workloads as W
    from yolohtli_gb300.batch import Batch
    from yolohtli_gb300.solver import Monodomain
    bw = W.fk_batch_256(seed=0, nsteps=nsteps)
    insts = bw.instances
    b = Batch([w.p for w in insts], [w.fk for w in insts],
              [w.solid for w in insts])
    dev0 = [[torch.tensor(x, device="cuda") for x in w.state0()] for w in insts]
    lib = b.lib

    def events():
        base = b.step_count()
        return [(k, W.stim(s.step + base, s.i0, s.j0, s.i1, s.j1, s.value))
                for k, s in bw.stims()]

    def restore():  # the initial state from device copies (not timed)
        for k in range(len(insts)):
            lib.yh_batch_set_state(b.h, k, *[C.c_void_p(x.data_ptr())
                                             for x in dev0[k]])
        b.synchronize()

    restore()
    if engine == "auto":
        tuned = b.autotune(256)
    elif engine == "instance":  # one two-step launch sequence per instance
        b.set_schedule(0, 8)
        b.set_depth(2)
        tuned = (0, 8, 2)
    else:  # the wavefront engine with that many CTAs per instance
        b.set_wave(int(engine[4:]))
        tuned = (0, int(engine[4:]), 0)
    for _ in range(warmup):
        restore()
        b.run(bw.nsteps, events())
    b.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(env_int("LOCAL_RANK", 0))
    clocks.start()
    launches0 = b.launch_count()
    sec = 0.0
    for k in range(solves):
        restore()
        ev = events()
        if k == 0:  # the range `ncu --profile-from-start off` captures
            torch.cuda.profiler.start()
        t0 = time.perf_counter()
        b.run(bw.nsteps, ev)
        b.synchronize()
        sec += time.perf_counter() - t0
        if k == 0:
            torch.cuda.profiler.stop()
    clk = clocks.stop()
    launches = b.launch_count() - launches0
    sec = max_over_ranks(sec, dist, "cuda")
    value = job_value(bw.cells, bw.nsteps, solves, world, sec)

    # end to end: host buffers in, u of every grid out, every solve, through
    # yh_batch_run_host (each instance's copies on its own stream under the
    # per-instance schedule)
    hst = [[torch.tensor(x).pin_memory() for x in w.state0()] for w in insts]
    outs = [(torch.empty(w.cells, dtype=torch.float32).pin_memory(), None, None)
            for w in insts]
    b.synchronize()
    t0 = time.perf_counter()
    for _ in range(solves):
        b.run_host(bw.nsteps, hst, outs, events())
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist, "cuda")
    e2e = {"value": round(job_value(bw.cells, bw.nsteps, solves, world, e2e_s), 3),
           "unit": METRIC, "h2d_bytes_per_step": 12 * bw.cells,
           "d2h_bytes_per_step": 4 * bw.cells}
    # the wavefront engine (one persistent launch per solve) beside the
    # autotuner's pick: a warm-up solve, then a timed one, per cluster size
    wave = {}
    if engine == "auto" and loops:
        for cl in (1, 2):
            b.set_wave(cl)
            restore()
            b.run(bw.nsteps, events())
            restore()
            ev = events()
            l0 = b.launch_count()
            t0 = time.perf_counter()
            b.run(bw.nsteps, ev)
            b.synchronize()
            dt = max_over_ranks(time.perf_counter() - t0, dist, "cuda")
            wave["cta_per_instance_%d" % cl] = {
                "value": round(job_value(bw.cells, bw.nsteps, 1, world, dt), 3),
                "gpu_launches_per_solve": b.launch_count() - l0}
    b.close()
    del dev0, hst, outs
    torch.cuda.empty_cache()

    # loops of single-grid solvers (step engine): one shared stream, then
    # one stream per grid; a warm-up solve, then the timed one
    lp = {}
    if loops:
        for mode in ("one_stream", "stream_per_grid"):
            s0 = torch.cuda.Stream() if mode == "one_stream" else None
            ms = [Monodomain(w.p, w.model, w.fk, solid=w.solid,
                             stream=s0.cuda_stream if s0 else None) for w in insts]
            for m in ms:
                m.set_engine(A.YH_ENGINE_STEP, 1)
            sec_l = 0.0
            for rep in range(2):
                for m, w in zip(ms, insts):
                    m.set_state(*w.state0())
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                for m, w in zip(ms, insts):
                    base = m.step_count()
                    m.run(bw.nsteps, [W.stim(x.step + base, x.i0, x.j0, x.i1,
                                             x.j1, x.value) for x in w.stims])
                for m in ms:
                    m.synchronize()
                sec_l = time.perf_counter() - t0
            for m in ms:
                m.close()
            lp[mode] = round(job_value(bw.cells, bw.nsteps, 1, world,
                                       max_over_ranks(sec_l, dist, "cuda")), 3)
    return {"bw": bw, "value": value, "sec": sec, "solves": solves,
            "tuned": tuned, "launches": launches, "clocks": clk, "e2e": e2e,
            "loops": lp, "wave": wave}


def batch_config(bw, tuned, world):
    if tuned[2] == 0:
        sched = ("wavefront engine: one persistent launch per solve, %d CTA(s) "
                 "per instance" % tuned[1])
    elif tuned[0] == 0:
        sched = ("autotuned: every instance its own sequence of single-grid "
                 "launches (64-step graphs, %d step(s) per launch), on %d "
                 "streams" % (tuned[2], tuned[1]))
    else:
        sched = ("autotuned: groups of ~%d cells on %d streams, %d steps per "
                 "launch" % tuned[:3])
    return {"workload": bw.name, "instances": len(bw.instances),
            "cells": bw.cells, "steps_per_solve": bw.nsteps,
            "sizes": "n ~ U{128,160,...,768}, square",
            "schedule": sched, "parallelism": "replicas x%d" % world}


WAVE_NOTE = ("the wavefront engine (rd_batch_wave_kernel): every instance "
             "on a cluster of CTAs, K steps per pass in shared memory, one "
             "launch per solve; timed beside the autotuner's pick")


def batch_summary(r):
    """The batched workload's figures as one object of the headline line."""
    lp = r["loops"]
    out = {"metric": METRIC, "value": round(r["value"], 3), "unit": METRIC,
           "config": batch_config(r["bw"], r["tuned"], 1),
           "solves_timed": r["solves"], "e2e": r["e2e"],
           "gpu_launches_per_solve": round(r["launches"] / r["solves"], 1),
           "loop_baselines": dict(lp, unit=METRIC)}
    if r["wave"]:
        out["wave_engine"] = dict(r["wave"], unit=METRIC, note=WAVE_NOTE)
    for k, v in lp.items():
        out["x_vs_" + k] = round(r["value"] / v, 3) if v else None
    return out


def run_batch(args):
    """The batched workload's own line (see batch_measure)."""
    import torch
    rank, world = env_int("RANK", 0), env_int("WORLD_SIZE", 1)
    torch.cuda.set_device(env_int("LOCAL_RANK", 0))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device(
            "cuda", env_int("LOCAL_RANK", 0)))
    r = batch_measure(args.nsteps, args.steps, args.warmup, dist, world,
                      engine=args.batch_engine)
    if rank == 0:
        peak, peak_kind = measured_peaks()
        value = r["value"]
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": METRIC,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * r["sec"] / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": batch_config(r["bw"], r["tuned"], world),
            "roofline": {"bound": "hbm", "achieved": round(25.0 * value, 1),
                         "peak": peak, "unit": "GB/s",
                         "frac": round(25.0 * value / peak, 4), "traffic": None,
                         "peak_kind": peak_kind, "alg_bytes_per_cell_step": 25,
                         "note": "achieved = 25 B x cell-steps/s over the whole "
                                 "run; state on chip, so frac > 1 is possible"},
            "cpu_baseline": None, "e2e": r["e2e"],
            "loop_baselines": dict(r["loops"], unit=METRIC,
                                   note="the same 256 grids run one by one "
                                        "through single-grid solver handles "
                                        "(step engine, graphs)"),
            "gpu_launches": int(r["launches"]), "clocks": r["clocks"],
        }
        if r["wave"]:
            line["wave_engine"] = dict(r["wave"], unit=METRIC, note=WAVE_NOTE)
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def sr_start(tau_d=0.25):
    """The re-entry that seeds the symmetry-reduced workload
    (fk_sr_512(tau_d): S1 at 0 ms, the tau_d's S2, 20,000 steps of 0.05 ms
    on 512^2). Returns (p, fk, state, tips)."""
    from yolohtli_gb300 import workloads as W
    from yolohtli_gb300.solver import Monodomain
    wl = W.fk_sr_512(seed=0, tau_d=tau_d)
    n = wl.p.nx
    q = wl.p.copy()
    q.tipx = q.tipy = n / 2  # tips anywhere in the tissue
    q.tipOffsetX = q.tipOffsetY = n // 2
    m = Monodomain(q, wl.model, wl.fk)
    m.set_state(*wl.state0())
    m.run(wl.nsteps - 1, wl.stims)
    m.run(1)
    m.track_tips()
    tips = m.get_tips()
    st = m.get_state()
    m.close()
    return wl.p, wl.fk, st, tips


def nearest_tip(tips, n):
    k = int(np.argmin(np.hypot(tips[:, 0] - n / 2, tips[:, 1] - n / 2)))
    return float(tips[k, 0]), float(tips[k, 1])


def sr_params(p, tip, radius=160):
    """SR parameters: dt halved as the reference does in SR mode
    (main.cu:148), the tip disc centred on the spiral's tip."""
    from yolohtli_gb300 import _abi as A
    q = p.copy()
    q.dt *= 0.5
    A.param_derive(q)
    q.tipx, q.tipy = tip
    q.tipOffsetX = q.tipOffsetY = radius
    return q


def sr_roofline(rate, cells):
    """The SR step against HBM: 84 algorithmic bytes per cell-step (RD 24,
    BFECC 24, the integral pass's state reads 12, the frozen template's
    derivative fields 24) x cells x SR steps/s."""
    peak, kind = measured_peaks()
    achieved = 84.0 * cells * rate / 1e9
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
            "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": None,
            "peak_kind": kind, "alg_bytes_per_cell_step": 84,
            "kernel": "the SR step (4 kernels and a memset)",
            "note": "latency-bound: four dependent launches of 0.1-0.26 M "
                    "cells per step; see profiles/sr_step_fk3v_512.md"}


def run_sr(args):
    """The symmetry-reduced spiral: FK3V FP32 on 512^2, every step RD, tips,
    slices, the 12 phase-condition integrals (float-float sums, FP64 from
    the integrals on), the FP64 3x3 solve, the comoving field and BFECC,
    all on the device; 40,000 SR steps of dt/2 = 0.025 ms (1000 ms).
    Template re-taken every step (the reference's behaviour); a run that
    ends with a singular solve or without a tip has no rate. tau_d = 0.25
    (the value) and 0.30; 0.35 and 0.45 have no re-entry on 512^2
    (workloads.SR_PROTOCOLS). The frozen template (the start state) is run
    beside it and reported by where its phase conditions became singular.
    The REF2V FP64 drop-in of the reference's own symbols, driven in its
    own sequence (main.cu:894-954), is reported beside it."""
    import torch
    from yolohtli_gb300 import _abi as A
    from yolohtli_gb300 import workloads as W
    from yolohtli_gb300.compat import Compat, sr_driver
    from yolohtli_gb300.ops import YolohtliError
    from yolohtli_gb300.solver import Monodomain
    nsr, K = args.nsteps, args.steps
    starts = {td: sr_start(td) for td in sorted(W.SR_PROTOCOLS)}
    n = 512
    N = n * n

    def run(m, k, profile=False):
        """k calls of nsr SR steps; (wall s, launches, ms per call,
        calls that saw a singular solve)."""
        torch.cuda.synchronize()
        l0 = m.launch_count()
        if profile:  # the range `ncu --profile-from-start off` captures
            torch.cuda.profiler.start()
        t0 = time.perf_counter()
        marks, sing = [], 0
        for _ in range(k):
            try:
                m.sr_step(nsr)
            except YolohtliError as e:
                if e.status != A.YH_ESINGULAR:
                    raise
                sing += 1
            m.synchronize()
            marks.append(time.perf_counter())
        wall = time.perf_counter() - t0
        if profile:
            torch.cuda.profiler.stop()
        per = [1e3 * (b - a) for a, b in zip([t0] + marks[:-1], marks)]
        return wall, m.launch_count() - l0, per, sing

    def handle(td, mode, stream=None):
        p, fk, st, tips = starts[td]
        q = sr_params(p, nearest_tip(tips, n))
        m = Monodomain(q, A.YH_MODEL_FK3V, fk, stream=stream)
        m.set_state(*st)
        m.sr_begin(mode, template=st if mode == A.YH_TEMPLATE_FROZEN else None)
        return m, q, st, fk

    runs, launches, clk, step_ms = {}, 0, None, []
    for td in sorted(starts):
        # warm-up on a handle of its own (graph capture), then the timed run
        # of the whole 40,000 steps from the start state
        m, q, st, fk = handle(td, A.YH_TEMPLATE_CURRENT)
        for _ in range(args.warmup):
            try:
                m.sr_step(nsr // 4)
            except YolohtliError:
                pass
        m.close()
        m, q, st, fk = handle(td, A.YH_TEMPLATE_CURRENT)
        if td == 0.25:
            clocks = ClockSampler(env_int("LOCAL_RANK", 0))
            clocks.start()
        wall, nl, per, sing = run(m, K, profile=td == 0.25)
        if td == 0.25:
            clk = clocks.stop()
            launches = nl
            step_ms = [round(x, 2) for x in per]
        sym = m.get_sym()
        ok = sing == 0 and sym.nsingular == 0 and sym.ntips >= 1
        runs[td] = dict(rate=K * nsr / wall, valid=ok, status=sym.status,
                        nsingular=sym.nsingular, ntips_end=sym.ntips,
                        c=[round(x, 6) for x in sym.c],
                        phi=[round(x, 5) for x in sym.phi],
                        start_tips=len(starts[td][3]))
        m.close()
    # the frozen template: SR steps in segments of 1,000 until a solve is
    # singular (the phase conditions lose rank once the pattern leaves the
    # template's shape)
    frozen = {}
    for td in sorted(starts):
        m, q, st, fk = handle(td, A.YH_TEMPLATE_FROZEN)
        done, first = 0, None
        while done < K * nsr:
            try:
                m.sr_step(1000)
            except YolohtliError as e:
                if e.status != A.YH_ESINGULAR:
                    raise
                first = done
                break
            done += 1000
        s = m.get_sym()
        frozen[str(td)] = {"singular_within_steps": None if first is None else
                           [first, first + 1000], "ntips": s.ntips,
                           "nsingular": s.nsingular}
        m.close()
    # the tau_d runs at once, one handle and stream each
    streams = [torch.cuda.Stream() for _ in starts]
    hs = [handle(td, A.YH_TEMPLATE_CURRENT, sm.cuda_stream)[0]
          for td, sm in zip(sorted(starts), streams)]
    for m in hs:
        m.sr_step(nsr // 4)
        m.synchronize()
    t0 = time.perf_counter()
    for _ in range(K):  # both runs' steps enqueued, nothing waited for
        for m in hs:
            m.sr_enqueue(nsr)
    for m in hs:
        try:
            m.sr_status()
        except YolohtliError as e:
            if e.status != A.YH_ESINGULAR:
                raise
    concurrent = len(hs) * K * nsr / (time.perf_counter() - t0)
    for m in hs:
        m.close()
    # end to end: the state from pinned host memory, the state and the
    # drift/rotation read back, every nsr steps
    m, q, st, fk = handle(0.25, A.YH_TEMPLATE_CURRENT)
    hst = [torch.from_numpy(np.ascontiguousarray(x, np.float32)).pin_memory()
           for x in st]
    t0 = time.perf_counter()
    for _ in range(K):
        m.set_state(*[x.numpy() for x in hst])
        try:
            m.sr_step(nsr)
        except YolohtliError:
            pass
        m.get_state()
        m.get_sym()
    e2e = K * nsr / (time.perf_counter() - t0)
    m.close()
    # like for like with the reference: REF2V FP64 through the drop-in
    r = A.param_defaults(n, n)
    r.Lx = r.Ly = 3.0 * n / 256
    r.hx = r.hy = r.Lx / (n - 1)
    r = sr_params(r, (n / 2, n / 2))
    u, v = W.ref2v_cross(n, n)
    cp = Compat()
    cp.set_params(r)
    gin = [torch.tensor(np.asarray(x, np.float64), device="cuda") for x in (u, v)]
    sr_driver(cp, r, gin, 5)
    torch.cuda.synchronize()
    k = 60
    t0 = time.perf_counter()
    sr_driver(cp, r, gin, k, count0=5)
    torch.cuda.synchronize()
    compat_rate = k / (time.perf_counter() - t0)
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        p, fk, st, tips = starts[0.25]
        q = sr_params(p, nearest_tip(tips, n))
        m0 = O.SR(q, A.YH_MODEL_FK3V, fk, st)
        t0 = time.perf_counter()
        ks = 0
        while time.perf_counter() - t0 < 10.0:
            m0.step(5)
            ks += 5
        cpu = {"value": round(ks / (time.perf_counter() - t0), 3),
               "unit": "SR steps/s", "cores": os.cpu_count() or 1,
               "kind": "port",
               "sample": "%d SR steps of the same 512^2 FK3V case in FP64 "
                         "(the oracle's SR sequence, OpenMP)" % ks}
    head = runs[0.25]
    v = head["rate"] if head["valid"] else None
    line = {
        "metric": "SR steps/s", "value": None if v is None else round(v, 2),
        "unit": "SR steps/s", "n_gpus": 1, "steps": K, "warmup": args.warmup,
        "ms_per_step": None if v is None else round(1e3 * nsr / v, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 state, f64 integrals and solve", "data": "synthetic",
        "config": {"workload": "fk_sr_512", "grid": [n, n], "model": "FK3V",
                   "tau_d": 0.25, "sr_steps_per_step": nsr,
                   "sr_steps_timed": K * nsr,
                   "template": "re-taken every step (the reference's)",
                   "start": "the state at 1000 ms of S1 + S2 on the lower "
                            "half at 585 ms (tau_d 0.25), on the lower-left "
                            "quadrant at 615 ms (tau_d 0.30)",
                   "disc_radius_cells": 160,
                   "dt_ms": sr_params(starts[0.25][0], (0, 0)).dt,
                   "l2": "state 3 MB: L2-resident (SR steps are latency-bound)",
                   "parallelism": "replicas x1"},
        "valid": head["valid"],
        "gcell_steps_per_s": None if v is None else round(v * N / 1e9, 3),
        "step_ms": step_ms,
        "tau_d_runs": {str(k): x for k, x in runs.items()},
        "tau_d_without_reentry": {
            "0.35": "no S2 time (180-705 ms, quadrant or half) sustains "
                    "activity past 850 ms on 512^2",
            "0.45": "as 0.35"},
        "frozen_template": frozen,
        "tau_d_concurrent": {"value": round(concurrent, 2),
                             "unit": "SR steps/s (sum of the tau_d runs)",
                             "note": "one handle and stream per run, the steps of both enqueued by yh_sr_enqueue, the status read once at the end"},
        "compat_fp64_reference_sequence": {
            "value": round(compat_rate, 2), "unit": "SR steps/s",
            "model": "REF2V FP64",
            "sequence": "main.cu:894-954 through the drop-in symbols from "
                        "Python: 12 integral read-backs and a host solve "
                        "per step, as the reference"},
        "roofline": None if v is None else sr_roofline(v, N),
        "cpu_baseline": cpu,
        "e2e": {"value": round(e2e, 2), "unit": "SR steps/s",
                "h2d_bytes_per_step": 3 * 4 * N,
                "d2h_bytes_per_step": 3 * 4 * N + C.sizeof(A.SymState)},
        "gpu_launches": int(launches), "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def run_sr_reference(args):
    """--impl reference for the symmetry-reduced workload: the reference's
    SR step sequence (main.cu:894-954) as the CPU restatement runs it (the
    oracle port, FP64, OpenMP over the host cores) on this arm's case: the
    fk_sr_512 start at tau_d = 0.25 (built on the CPU too), the same disc,
    the template re-taken every step. The reference's own GPU kernels in
    their sequence (REF2V FP64, the model it has) are reported beside it
    as reference_gpu."""
    if env_int("RANK", 0) != 0:
        return
    from oracle import oracle as O
    from yolohtli_gb300 import _abi as A
    from yolohtli_gb300 import workloads as W
    wl = W.fk_sr_512(seed=0)
    n = wl.p.nx
    t_start = time.perf_counter()
    pre = O.run(wl.p, wl.model, wl.fk, wl.state0(), wl.nsteps - 1, wl.stims,
                dtype=np.float64)
    st = O.run(wl.p, wl.model, wl.fk, pre, 1, wl.stims, step0=wl.nsteps - 1,
               dtype=np.float64)
    whole = wl.p.copy()
    whole.tipx = whole.tipy = n / 2
    whole.tipOffsetX = whole.tipOffsetY = n // 2
    tips = O.tips(whole, pre[0], st[0])
    tip = nearest_tip(tips, n) if len(tips) else (n / 2, n / 2)
    q = sr_params(wl.p, tip)
    start_s = time.perf_counter() - t_start
    sr = O.SR(q, A.YH_MODEL_FK3V, wl.fk, st)
    sample = 25  # SR steps per bench step
    times = []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        sr.step(sample)
        if k >= args.warmup:
            times.append(time.perf_counter() - t0)
    rate = sample * len(times) / sum(times)
    cores = os.cpu_count() or 1
    line = {
        "impl": "reference", "metric": "SR steps/s", "value": round(rate, 3),
        "unit": "SR steps/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * sum(times) / len(times), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": "fk_sr_512", "grid": [n, n], "model": "FK3V",
                   "tau_d": 0.25, "template": "re-taken every step (the reference's)",
                   "disc_radius_cells": 160,
                   "dt_ms": q.dt, "start_tips": int(len(tips)),
                   "parallelism": "host cores"},
        "cpu_baseline": {
            "value": round(rate, 3), "unit": "SR steps/s", "cores": cores,
            "kind": "port",
            "sample": "each step: %d SR steps (RD, tips, slices + integrals, "
                      "solve, comoving field, BFECC) of the 512^2 FK3V case, "
                      "FP64 C/OpenMP restatement of the reference's sequence; "
                      "start state built on the CPU in %.1f s" % (sample, start_s)},
        "e2e": {"value": round(rate, 3), "unit": "SR steps/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    try:
        import torch
        from oracle import refgpu as R
        if torch.cuda.is_available() and R.available():
            r = A.param_defaults(n, n)
            r.Lx = r.Ly = 3.0 * n / 256
            r.hx = r.hy = r.Lx / (n - 1)
            r = sr_params(r, (n / 2, n / 2))
            u, v = W.ref2v_cross(n, n)
            gin = [torch.tensor(np.asarray(x, np.float64), device="cuda")
                   for x in (u, v)]
            R.sr_driver(r, gin, 5, O.solve)
            k = 60
            t0 = time.perf_counter()
            R.sr_driver(r, gin, k, O.solve, count0=5)
            line["reference_gpu"] = {
                "value": round(k / (time.perf_counter() - t0), 2),
                "unit": "SR steps/s", "model": "REF2V FP64 (the reference's)",
                "sequence": "main.cu:894-954 on the reference's kernels "
                            "(sm_103a, headless): RD, tips, slices, 12 trapz "
                            "launches each read back, host solve, Cxy, BFECC"}
    except Exception as e:  # the GPU leg is optional beside the CPU value
        line["reference_gpu"] = {"unavailable": str(e)[:200]}
    print(json.dumps(line), flush=True)


ADJ_BYTES = {"sqrt_n": 104, "store_all": 76}


def adjoint_roofline(grads_per_s, cells, nsteps, mode="sqrt_n"):
    """Algorithmic bytes of one gradient per cell-step: the forward step
    reads D, u, v, w and writes u, v, w (28 B); the reverse step reads D,
    u, v, w, the adjoint state lu, lv, lw, writes lu, lv, lw and updates
    the D gradient (48 B). sqrt(N) checkpoints run every forward step twice
    (the pass that records the checkpoints, the segment recompute; the
    last segment's once): 2 x 28 + 48 = 104 B; with every state kept,
    28 + 48 = 76 B."""
    peak, kind = measured_peaks()
    b = ADJ_BYTES[mode]
    achieved = grads_per_s * b * cells * nsteps / 1e9
    trip = profiled_traffic("adjoint512_step_triplet") if cells == 512 * 512 else None
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
            "unit": "GB/s", "frac": round(achieved / peak, 4),
            "traffic": trip if mode == "sqrt_n" else None,
            "traffic_note": "DRAM bytes of one forward + recompute + reverse "
                            "step (ncu, cold L2)" if trip and mode == "sqrt_n" else None,
            "peak_kind": kind, "alg_bytes_per_cell_step": b,
            "note": "achieved = %d B x cells x steps per gradient x "
                    "gradients/s (forward %s + reverse)" % (
                        b, "+ recompute" if mode == "sqrt_n" else "")}


def adjoint_cpu_baseline(p, fk, D, state0, target, nsteps, frame, spacing,
                         smooth, sample_steps=200):
    """The FP64 tangent-linear oracle (oracle/yh_oracle_tlm.c, dual numbers,
    one directional derivative per run) on the host cores, on the first
    `sample_steps` steps of the workload; scaled to the whole horizon."""
    from oracle import oracle as O
    from yolohtli_gb300 import _abi as A
    dfk = A.FKParams()
    dD = np.asarray(D, np.float32) * 0.01
    t0 = time.perf_counter()
    O.adj_tlm(p, fk, dfk, smooth, sample_steps, frame, spacing, D, dD, state0,
              target)
    sec = (time.perf_counter() - t0) * nsteps / sample_steps
    return {"value": round(1.0 / sec, 5), "unit": "directional derivatives/s",
            "cores": os.cpu_count() or 1, "kind": "port",
            "sample": "FP64 tangent-linear model (dual numbers) of the same "
                      "forward map, first %d of %d steps on %dx%d, scaled to "
                      "the horizon; a full gradient by this route takes "
                      "%d directional derivatives (D and the 13 parameters)"
                      % (sample_steps, nsteps, p.nx, p.ny, p.nx * p.ny + 13)}


def adjoint_measure(nsteps, steps, warmup, dist, world, full=False):
    """The adjoint workload (fk_adjoint_512: 512^2 FK3V, D(x, y) of 8
    Gaussian bumps in [5e-4, 1.5e-3], `nsteps` steps, the loss on a 32 x 32
    probe lattice every 20 steps, target from the true D, gradient at
    1.1 D; the model's switches as tanh ramps of width 0.01, without which
    the loss's derivative is not usable at this horizon). A gradient is the
    full one: dLoss/dD and dLoss/d(13 FK parameters). Returns gradients per
    second with sqrt(N) checkpoints and the ratio to the forward run; with
    `full` also every state kept, 16 instances in one handle, and the
    accuracy checks (FP32 against FP64, FP64 against central differences
    along 20 random directions of (D, FK parameters))."""
    import torch
    from yolohtli_gb300 import _abi as A
    from yolohtli_gb300 import workloads as W
    from yolohtli_gb300.adjoint import Adjoint, fk_array, fk_struct
    n = 512
    frame, spacing = 20, 16
    ck = max(1, int(round(nsteps ** 0.5)))
    p = A.fk_tissue_params(n, n)
    D_true, state0 = W.fk_adjoint_case(n, seed=0)
    smooth = 0.01
    fk0 = A.fk_defaults()

    def make(fp64, nst, ckpt, batch=1):
        a = Adjoint(p, fk0, nst, frame, spacing, ckpt, fp64=fp64,
                    smooth=smooth, batch=batch)
        st = [torch.tensor(x, device="cuda").repeat(batch) for x in state0]
        Dt = torch.tensor(D_true, device="cuda").repeat(batch)
        tgt = torch.empty(a.target_shape, dtype=torch.float32, device="cuda")
        a.record(Dt, st, tgt)
        a.set_target(tgt)
        return a, st, Dt * 1.1, tgt

    def timed(a, st, D, k, grad=True):
        g = torch.empty_like(D) if grad else None
        gfk = (A.FKParams * a.batch)() if grad else None
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(k):
            loss = a.run(D, st, g, gfk)
        return time.perf_counter() - t0, loss, g, gfk

    adj, st, D, tgt = make(False, nsteps, ck)
    # both sequences (gradient, loss only) captured and run once before
    # either is timed
    timed(adj, st, D, 1, grad=False)
    for _ in range(warmup):
        timed(adj, st, D, 1)
    if dist:
        dist.barrier()
    torch.cuda.profiler.start()  # one gradient: the range ncu captures
    timed(adj, st, D, 1)
    torch.cuda.profiler.stop()
    clocks = ClockSampler(env_int("LOCAL_RANK", 0))
    clocks.start()
    sec, loss, g, gfk = timed(adj, st, D, steps)
    clk = clocks.stop()
    fwd, _, _, _ = timed(adj, st, D, steps, grad=False)
    sec = max_over_ranks(sec, dist, "cuda")
    value = world * steps / sec
    # end to end: D from the host, both gradients back, every gradient
    Dh = D.cpu().pin_memory()
    gh = torch.empty_like(Dh).pin_memory()
    Dd = torch.empty_like(D)
    gfk_h = A.FKParams()
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    for _ in range(steps):
        Dd.copy_(Dh, non_blocking=True)
        adj.run(Dd, st, g, gfk_h)
        gh.copy_(g)
    e2e_s = max_over_ranks(time.perf_counter() - t2, dist, "cuda")
    out = {"value": value, "sec": sec, "loss": float(loss),
           "forward_ratio": sec / fwd, "clocks": clk,
           "checkpoint_steps": ck, "smooth": smooth, "n": n, "frame": frame,
           "spacing": spacing,
           "e2e": {"value": round(world * steps / e2e_s, 3),
                   "unit": "gradients/s", "h2d_bytes_per_step": 4 * n * n,
                   "d2h_bytes_per_step": 4 * n * n + 13 * 8},
           "roofline": adjoint_roofline(value / world, n * n, nsteps)}
    if env_int("RANK", 0) == 0 and world == 1:
        out["cpu_baseline"] = adjoint_cpu_baseline(
            p, fk0, (D.cpu().numpy()), state0, tgt.cpu().numpy(), nsteps,
            frame, spacing, smooth)
    if not full:
        del adj
        torch.cuda.empty_cache()
        return out
    # every state kept (31 GB at this size): no recompute
    del adj
    torch.cuda.empty_cache()
    a1, st1, D1, _ = make(False, nsteps, 1)
    timed(a1, st1, D1, 1)
    timed(a1, st1, D1, 1, grad=False)
    s1, _, _, _ = timed(a1, st1, D1, steps)
    f1, _, _, _ = timed(a1, st1, D1, steps, grad=False)
    del a1
    torch.cuda.empty_cache()
    out["store_all_states"] = {
        "value": round(steps / s1, 3), "unit": "gradients/s",
        "forward_ratio": round(s1 / f1, 3),
        "memory_gb": round(3 * 4 * n * n * nsteps / 1e9, 1),
        "roofline": adjoint_roofline(steps / s1, n * n, nsteps, "store_all")}
    # 16 instances, one handle
    B = 16
    ab, stb, Db, _ = make(False, nsteps, ck, batch=B)
    timed(ab, stb, Db, 1)
    sb, _, _, _ = timed(ab, stb, Db, max(1, steps // 2))
    batch_rate = B * max(1, steps // 2) / sb
    del ab
    torch.cuda.empty_cache()
    out["batched_16"] = {"value": round(batch_rate, 3),
                         "unit": "instance gradients/s", "checkpoint_steps": ck,
                         "note": "16 instances in one handle, one launch per step",
                         "roofline": adjoint_roofline(batch_rate, n * n, nsteps)}
    # the batched fit: 16 instances (true D of seeds 0..15, the FK3V
    # parameters shared), Adam on log D and log parameters from the true
    # values + 10 %, 20 iterations, one batched gradient each
    from yolohtli_gb300.adjoint import fit
    af = Adjoint(p, fk0, nsteps, frame, spacing, ck, smooth=smooth, batch=B)
    Dt = torch.cat([torch.tensor(W.fk_adjoint_case(n, seed=k)[0], device="cuda")
                    for k in range(B)])
    stf = [torch.tensor(x, device="cuda").repeat(B) for x in state0]
    tgt = torch.empty(af.target_shape, dtype=torch.float32, device="cuda")
    af.record(Dt, stf, tgt)
    af.set_target(tgt)
    Df = Dt * 1.1
    e0 = float((Df - Dt).norm() / Dt.norm())
    t4 = time.perf_counter()
    th, losses = fit(af, Df, stf, fk_array(fk0) * 1.1, iters=20, lr=0.01)
    fit_s = time.perf_counter() - t4
    e1 = float((Df - Dt).norm() / Dt.norm())
    th_true = fk_array(fk0)
    out["fit"] = {
        "instances": B, "iterations": 20, "optimizer": "Adam on log D and "
        "log parameters (second moments shared per instance's D and over "
        "the 13 parameters), lr 0.01", "seconds": round(fit_s, 2),
        "loss_total": [float(x) for x in losses.sum(axis=1)],
        "loss_ratio_per_instance": [round(float(x), 4) for x in
                                    losses[-1] / losses[0]],
        "D_rel_error": [round(e0, 5), round(e1, 5)],
        "fk_rel_error_max": [0.1, round(float(np.abs(th / th_true - 1).max()), 4)],
        "note": "start: true D and FK parameters + 10 %; target: probes of the "
                "run with the true values"}
    del af, Dt, stf, tgt, Df
    torch.cuda.empty_cache()
    # accuracy at the full size
    b64, st64, D64, _ = make(True, nsteps, ck)
    g64 = torch.empty_like(D64)
    f64 = A.FKParams()
    t3 = time.perf_counter()
    b64.run(D64, st64, g64, f64)
    out["fp64_gradients_per_s"] = round(1.0 / (time.perf_counter() - t3), 3)
    th0 = fk_array(fk0)
    rng = np.random.default_rng(3)
    ndir = 20
    fd_err = {1e-3: 0.0, 1e-5: 0.0}
    for _ in range(ndir):
        d = torch.tensor(rng.standard_normal(n * n).astype(np.float32), device="cuda") * D64
        dth = rng.standard_normal(13) * th0
        for hrel in fd_err:
            Dp, Dm = D64 + hrel * d, D64 - hrel * d
            stp = (Dp.double() - Dm.double()) / 2
            b64.set_fk(fk_struct(th0 + hrel * dth))
            Lp = b64.run(Dp, st64)
            b64.set_fk(fk_struct(th0 - hrel * dth))
            Lm = b64.run(Dm, st64)
            ad = 2 * (float((g64.double() * stp).sum()) +
                      hrel * float(np.dot(fk_array(f64), dth)))
            fd_err[hrel] = max(fd_err[hrel], abs((Lp - Lm) - ad) / max(abs(ad), 1e-300))
    b64.set_fk(fk0)
    out["fd_check"] = {"directions": ndir,
                       "max_rel_err": {"h_rel 1e-3": fd_err[1e-3],
                                       "h_rel 1e-5": fd_err[1e-5]},
                       "note": "directional derivatives of the FP64 adjoint "
                               "along random directions of D (relative) and "
                               "all 13 FK parameters (relative) against "
                               "central differences of the FP64 loss, full "
                               "size; the error falling as h^2 is the "
                               "differences' truncation"}
    out["fp32_vs_fp64_gradient_rel_l2"] = float(
        (g.double() - g64.double()).norm() / g64.double().norm())
    out["fp32_vs_fp64_fk_gradient_rel_max"] = float(
        np.abs(fk_array(gfk[0]) - fk_array(f64)).max() / np.abs(fk_array(f64)).max())
    return out


def adjoint_config(r, nsteps, world):
    n = r["n"]
    return {"workload": "fk_adjoint_512", "grid": [n, n],
            "steps_per_gradient": nsteps, "frames": nsteps // r["frame"],
            "probes": [n // r["spacing"], n // r["spacing"]],
            "checkpoint_steps": r["checkpoint_steps"],
            "gradient": "dLoss/dD (512^2) and dLoss/d(13 FK parameters)",
            "D": "8 Gaussian bumps in [5e-4, 1.5e-3]",
            "switches": "FK3V's H(u - u_c), H(u - u_v) as tanh ramps of "
                        "width %g" % r["smooth"],
            "estimate": "1.1 x the true D",
            "parallelism": "replicas x%d" % world}


def run_adjoint(args):
    """The adjoint workload's own line (see adjoint_measure)."""
    import torch
    rank, world = env_int("RANK", 0), env_int("WORLD_SIZE", 1)
    torch.cuda.set_device(env_int("LOCAL_RANK", 0))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device(
            "cuda", env_int("LOCAL_RANK", 0)))
    r = adjoint_measure(args.nsteps, args.steps, args.warmup, dist, world,
                        full=True)
    if rank == 0:
        line = {
            "metric": "adjoint gradients/s", "value": round(r["value"], 3),
            "unit": "gradients/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": round(1e3 * r["sec"] / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": adjoint_config(r, args.nsteps, world),
            "loss": r["loss"], "forward_ratio": round(r["forward_ratio"], 3),
            "roofline": r["roofline"], "cpu_baseline": r.get("cpu_baseline"),
            "e2e": r["e2e"], "gpu_launches": None, "clocks": r["clocks"]}
        for k in ("store_all_states", "batched_16", "fit", "fd_check",
                  "fp32_vs_fp64_gradient_rel_l2",
                  "fp32_vs_fp64_fk_gradient_rel_max", "fp64_gradients_per_s"):
            line[k] = r[k]
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def adjoint_summary(r, nsteps):
    return {"metric": "adjoint gradients/s", "value": round(r["value"], 3),
            "unit": "gradients/s", "config": adjoint_config(r, nsteps, 1),
            "forward_ratio": round(r["forward_ratio"], 3),
            "roofline": r["roofline"], "cpu_baseline": r.get("cpu_baseline"),
            "e2e": r["e2e"]}


def run_spiral(args):
    """Config 0 (fk_spiral_256): FK3V 256^2, 10,000 steps, S1 columns 0-9 at
    t = 0, S2 on the lower-left quadrant at 320 ms, tips every sampleIt =
    40 steps (param.sample = 2 ms, main.cu:156,961-964). One bench step = one
    solve with its tip trajectory. With --out DIR the last solve's final
    state goes to DIR/raw_data.dat, its tips to DIR/dataTip.dat and
    DIR/dataTipSize.dat and the parameters to DIR/dataparamcsv.csv, the
    reference's own formats (printFunctions.cu:58-78,149-197,266-403)."""
    import torch
    rank, world = env_int("RANK", 0), env_int("WORLD_SIZE", 1)
    torch.cuda.set_device(env_int("LOCAL_RANK", 0))
    from yolohtli_gb300 import _abi as A
    from yolohtli_gb300 import refio
    from yolohtli_gb300 import workloads as W
    from yolohtli_gb300.solver import Monodomain
    wl = W.fk_spiral_256(nsteps=args.nsteps)
    sample_it = 40
    m = Monodomain(wl.p, wl.model, wl.fk)
    m.set_state(*wl.state0())
    engine, tb = m.autotune(256)

    def solve():
        base = m.step_count()
        stims = [W.stim(s.step + base, s.i0, s.j0, s.i1, s.j1, s.value)
                 for s in wl.stims]
        m.set_state(*wl.state0())
        tips = []
        for _ in range(wl.nsteps // sample_it):
            m.run(sample_it, stims)
            m.track_tips()
            t = m.get_tips()
            t[:, 4] = wl.p.dt * (m.step_count() - base)
            tips.append(t)
        return tips

    for _ in range(args.warmup):
        solve()
    m.synchronize()
    clocks = ClockSampler(env_int("LOCAL_RANK", 0))
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        tips = solve()
    m.synchronize()
    sec = time.perf_counter() - t0
    clk = clocks.stop()
    u, v, w = m.get_state()
    value = job_value(wl.cells, wl.nsteps, args.steps, world, sec)
    ntips = sum(len(t) for t in tips)
    if args.out:
        os.makedirs(args.out, exist_ok=True)
        refio.write_raw_data(os.path.join(args.out, "raw_data.dat"), wl.p, u, v)
        tp, sz = (os.path.join(args.out, f) for f in ("dataTip.dat",
                                                      "dataTipSize.dat"))
        for f in (tp, sz):
            if os.path.exists(f):
                os.unlink(f)
        for t in tips:
            refio.write_tips(tp, sz, t, append=True)
        refio.write_param_csv(os.path.join(args.out, "dataparamcsv.csv"), wl.p)
    m.close()
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": round(value, 3), "unit": METRIC,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * sec / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": wl.name, "grid": [wl.p.nx, wl.p.ny],
                       "steps_per_solve": wl.nsteps, "model": "FK3V",
                       "tips_every_steps": sample_it, "engine":
                           A.ENGINE_NAMES[engine], "time_block": tb,
                       "parallelism": "replicas x%d" % world},
            "tips": {"samples": len(tips), "total": ntips,
                     "samples_with_tips": sum(1 for t in tips if len(t)),
                     "last_tip_ms": max([float(t[0, 4]) for t in tips if len(t)]
                                        or [None])},
            "final_u": {"max": float(u.max()), "mean": float(u.mean()),
                        "cells_above_0.5": int((u > 0.5).sum())},
            "outputs": args.out, "clocks": clk}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--engine", default="auto",
                    choices=["auto", "step", "blocked", "resident"],
                    help="how the solver advances (auto: the library's "
                         "autotuner picks engine and depth before timing)")
    ap.add_argument("--time-block", type=int, default=4,
                    help="steps per launch of the blocked engine")
    ap.add_argument("--nsteps", type=int, default=None,
                    help="explicit steps per solve (default: the workload's, "
                         "20,000 for fk_holes_1024, 5,000 for batch256)")
    ap.add_argument("--workload", default="holes1024",
                    choices=["holes1024", "batch256", "adjoint512", "sr512",
                             "spiral256"],
                    help="holes1024: one 1024^2 grid with 300 holes (the "
                         "headline); batch256: 256 grids of 128^2..768^2 "
                         "through the batched solver")
    ap.add_argument("--grid", type=int, default=1024,
                    help="grid side (1024 = the benchmark; larger sides are "
                         "for profiling beyond the L2, holes scaled by area)")
    ap.add_argument("--batch-engine", default="auto",
                    choices=["auto", "instance", "wave1", "wave2", "wave4"],
                    help="batch256: the autotuner's pick (and the wavefront "
                         "engine timed beside it), one two-step launch "
                         "sequence per instance on 8 streams, or the "
                         "wavefront engine with 1, 2 or 4 CTAs per instance")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--out", default=None,
                    help="spiral256: directory for the final state and the "
                         "tip trajectory in the reference's file formats")
    ap.add_argument("--no-extras", action="store_true",
                    help="the headline workload alone (without the batched "
                         "and adjoint figures the default line carries)")
    args = ap.parse_args()

    from yolohtli_gb300 import workloads as W
    if args.workload == "spiral256":
        if args.nsteps is None:
            args.nsteps = 10000
        if args.impl == "reference":
            run_reference(args, W.fk_spiral_256(nsteps=args.nsteps))
        else:
            run_spiral(args)
        return
    if args.workload == "sr512":
        if args.nsteps is None:
            args.nsteps = 8000  # x 5 steps = the 40,000 SR steps of the case
        if args.impl == "reference":
            run_sr_reference(args)
        else:
            run_sr(args)
        return
    if args.workload == "adjoint512":
        if args.nsteps is None:
            args.nsteps = 10000
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable":
                              "the reference computes no gradients"}), flush=True)
        else:
            run_adjoint(args)
        return
    if args.workload == "batch256":
        if args.nsteps is None:
            args.nsteps = 5000
        if args.impl == "reference":
            # the CPU transcription on a sample: the largest grid of the batch
            bw = W.fk_batch_256(seed=0, nsteps=args.nsteps)
            run_reference(args, max(bw.instances, key=lambda w: w.cells))
        else:
            run_batch(args)
        return
    if args.nsteps is None:
        args.nsteps = 20000
    scale = (args.grid / 1024.0) ** 2
    wl = W.fk_holes_1024(seed=0, n=args.grid, nsteps=args.nsteps,
                         nholes=int(round(300 * scale)))

    if args.impl == "reference":
        run_reference(args, wl)
        return

    import torch
    rank, world = env_int("RANK", 0), env_int("WORLD_SIZE", 1)
    local = env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from yolohtli_gb300 import _abi as A
    from yolohtli_gb300.solver import Monodomain

    stream = torch.cuda.Stream()
    m = Monodomain(wl.p, wl.model, wl.fk, solid=wl.solid, stream=stream.cuda_stream)
    ic = [torch.tensor(x, device="cuda") for x in wl.state0()]
    autotuned = args.engine == "auto"
    if autotuned:
        # the library's autotuner, on the workload's initial state (restored)
        m.set_state(*wl.state0())
        engine, tb = m.autotune(512)
    else:
        engine = {"step": A.YH_ENGINE_STEP, "blocked": A.YH_ENGINE_BLOCKED,
                  "resident": A.YH_ENGINE_RESIDENT}[args.engine]
        m.set_engine(engine, args.time_block)
        engine, tb = m.engine()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    lib = m.lib

    # One handle serves every solve (a fresh handle would re-upload the mask):
    # its step counter keeps running, so the stimulus schedule is shifted by
    # the steps already taken; each solve re-initialises the state from the
    # device copy of the initial condition.
    base = [0]

    def solve_shifted():
        stims = []
        for s in wl.stims:
            q = A.Stim()
            q.step, q.i0, q.j0, q.i1, q.j1, q.value = (
                s.step + base[0], s.i0, s.j0, s.i1, s.j1, s.value)
            stims.append(q)
        lib.yh_set_state(m.h, *[C.c_void_p(t.data_ptr()) for t in ic])
        m.run(wl.nsteps, stims)
        base[0] += wl.nsteps

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            solve_shifted()
            flush.fill_(1.0)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        clocks = ClockSampler(local)
        clocks.start()
        launches0 = m.launch_count()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for k in range(args.steps):
            solve_shifted()
            if k + 1 < args.steps:
                flush.fill_(1.0)
        ev1.record(stream)
        torch.cuda.synchronize()
        launches = m.launch_count() - launches0
        ms = ev0.elapsed_time(ev1)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        clk = clocks.stop()

    ms_max = max_over_ranks(ms, dist, "cuda")
    cell_steps = wl.cells * wl.nsteps * args.steps * world
    value = job_value(wl.cells, wl.nsteps, args.steps, world, ms_max * 1e-3)

    # Dominant kernel: the RD step (the stimulus kernels of the events that
    # fire are the only other launches; the resident engine applies the
    # events inside its own launch). Algorithmic bytes: 25 B per cell-step
    # (u, v, w read + write in FP32 and the 1-byte hole mask); one launch
    # advances all cells by steps_per_launch steps. The mean launch time is
    # taken over the whole timed region, so it also carries the stimulus
    # kernels, the L2 flushes and the gaps between launches.
    fired = sum(1 for s in wl.stims if s.step < wl.nsteps)
    stim_launches = 0 if engine == A.YH_ENGINE_RESIDENT else fired
    rd_launches = max(1, launches - args.steps * stim_launches)
    steps_per_launch = wl.nsteps * args.steps / rd_launches
    avg_launch_s = ms * 1e-3 / rd_launches
    bytes_alg = 25.0 * wl.cells * steps_per_launch
    achieved = bytes_alg / avg_launch_s / 1e9
    peak, peak_kind = measured_peaks()
    key = "%s_%s%d" % (wl.name, A.ENGINE_NAMES[engine], tb)
    traffic = profiled_traffic(key)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4),
                "traffic": traffic, "peak_kind": peak_kind,
                "alg_bytes_per_cell_step": 25,
                "steps_per_launch": round(steps_per_launch, 3),
                "mean_launch_us": round(avg_launch_s * 1e6, 3),
                "kernel": {A.YH_ENGINE_STEP: "rd_step_vec4",
                           A.YH_ENGINE_BLOCKED: "rd_tb_kernel",
                           A.YH_ENGINE_RESIDENT: "rd_resident_kernel"}[engine],
                "note": "achieved = 25 B x cells x steps_per_launch / mean launch "
                        "time; frac > 1 is possible: the state stays in L2 and "
                        "temporal blocking re-reads it once per steps_per_launch"}
    if traffic is not None:
        roofline["dram_bytes_per_launch"] = traffic
        roofline["dram_gbs"] = round(traffic / avg_launch_s / 1e9, 1)
    roofline["issue"] = issue_roofline(key, value / world, clk)

    # end to end through the public C ABI with pinned host buffers
    e2e = None
    if rank == 0 or world > 1:
        hst = [torch.tensor(x).pin_memory() for x in wl.state0()]
        out_u = torch.empty(wl.cells, dtype=torch.float32).pin_memory()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(args.steps):
            stims = []
            for s in wl.stims:
                q = A.Stim()
                q.step, q.i0, q.j0, q.i1, q.j1, q.value = (
                    s.step + base[0], s.i0, s.j0, s.i1, s.j1, s.value)
                stims.append(q)
            lib.yh_set_state(m.h, *[C.c_void_p(x.data_ptr()) for x in hst])
            m.run(wl.nsteps, stims)
            base[0] += wl.nsteps
            lib.yh_get_state(m.h, C.c_void_p(out_u.data_ptr()), None, None)
        e2e_s = time.perf_counter() - t0
        e2e_max = max_over_ranks(e2e_s, dist, "cuda")
        e2e = {"value": round(job_value(wl.cells, wl.nsteps, args.steps, world,
                                        e2e_max), 3),
               "unit": METRIC, "h2d_bytes_per_step": 3 * 4 * wl.cells,
               "d2h_bytes_per_step": 4 * wl.cells}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(wl)

    m.close()
    del ic, flush
    torch.cuda.empty_cache()
    extras = {}
    if not args.no_extras and args.grid == 1024:
        # the batched and adjoint workloads, shortened to a few solves each:
        # their own lines come from --workload batch256 / adjoint512
        extras["batched"] = batch_summary(batch_measure(5000, 2, 1, dist, world))
        extras["adjoint"] = adjoint_summary(
            adjoint_measure(10000, 2, 1, dist, world), 10000)
        # like for like with the reference's own kernel (reference_gpu of
        # the reference arm's line): REF2V FP64, 1024^2, through the drop-in
        extras["fp64_dropin"] = dropin_gpu()
    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": METRIC,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms_max / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": config_of(wl, args, tb, autotuned,
                                A.ENGINE_NAMES[engine]),
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": int(launches), "clocks": clk,
        }
        line.update(extras)
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
