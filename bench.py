"""Benchmark: cell-updates/s of the time-step hot path on one GB300.

A step is one accepted time step of IntegrateTo (the fused hydraulic passes plus the
activation check) over the whole active domain.  One cell-update is one active cell
advanced by one accepted hydraulic dt (a morphodynamic Strang step counts 2).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

- value:   device-timed throughput (CUDA events on the library's stream around each
           step; L2 flushed by a 256 MiB write between timed steps, outside the timed
           intervals).
- e2e:     the same metric through the public C ABI, host clock: K kg_step calls after
           the same spin-up (each returns its statistics to the host, with the library's
           own count of its host<->device bytes), then the conserved fields of every
           active tile read back to host memory.  e2e_job: the whole job from kg_create
           with the settings and bed uploaded, through the spin-up, to the read-back.
- roofline: the fused hydraulic pass; algorithmic bytes per cell-update (FP64 hydraulic
           step: 368 B over its 4 passes) over the measured pass time, against the
           measured HBM copy bandwidth.  roofline_fp64: the same pass against its FP64
           pipe, the bound it meets on GB300.
- cpu_baseline: the CPU oracle (a serial C++ restatement of the reference, which is
           itself serial; the Fortran cannot be built here) on a bounded sample of the
           same workload, on one of the host's cores.
Under torchrun (N > 1) each rank advances an independent replica (replicas only).
"""
from __future__ import annotations

import argparse
import ctypes as C
import faulthandler
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic bytes per cell-update (minimal traffic: each stage's inputs read once, its
# outputs written once; the bed is the two vertex fields).  A hydraulic step is 4 fused
# passes over 46 field accesses per cell; a morphodynamic Strang step H.M.H counts 2
# cell-updates and adds the 36 accesses of the M operator.
ALG_BYTES = {"fp64_hydro": 368.0, "fp64_morpho": 512.0, "fp32_hydro": 252.0, "fp32_morpho": 366.0}
# One fused hydraulic pass: a quarter of the hydraulic step, per cell of the pass.
ALG_PASS_BYTES = {"fp64": ALG_BYTES["fp64_hydro"] / 4.0, "fp32": ALG_BYTES["fp32_hydro"] / 4.0}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def measured_sm_max_mhz():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["sm_max_mhz"])
    except Exception:
        return 2070.0


def profile_figure(kernel: str, workload: str, key: str):
    """A per-cell figure (`key: value` line) from the committed ncu summary of this kernel
    and workload under profiles/, or None."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    if not os.path.exists(path):
        return None
    m = re.search(re.escape(key) + r":\s*([0-9.eE+]+)", open(path).read())
    return float(m.group(1)) if m else None


def profile_traffic(kernel: str, workload: str, cells: float):
    """DRAM bytes per pass, scaled to `cells` active cells from the bytes per cell and pass
    recorded in the ncu summary (the `dram_bytes_per_cell_pass:` line): the capture may run
    a smaller active set of the same workload, and traffic grows with the cells processed."""
    per_cell = profile_figure(kernel, workload, "dram_bytes_per_cell_pass")
    return per_cell * cells if per_cell is not None else None


def fp64_pipe_roofline(kernel: str, workload: str, cells: float, pass_ms: float, sm_mhz, n_sm: int):
    """The bound the pass actually meets on GB300: its FP64 pipe (2 FP64 lanes per SM per
    clock).  `achieved` = the FP64-pipe busy cycles one pass needs (the per-cell figure from
    the ncu capture, `fp64_pipe_cycles_per_cell_pass:`, times the cells of the pass) over
    the measured pass time; `peak` = every SM's FP64 pipe busy every cycle at `sm_mhz` (the
    median SM clock sampled during the main timed region; the GPU's maximum clock for the
    FP64 twin, which is not sampled)."""
    per_cell = profile_figure(kernel, workload, "fp64_pipe_cycles_per_cell_pass")
    if per_cell is None or not pass_ms or not sm_mhz or not n_sm:
        return None
    achieved = per_cell * cells / (pass_ms / 1e3)
    peak = n_sm * sm_mhz * 1e6
    return {"bound": "fp64_pipe", "achieved": achieved, "peak": peak, "unit": "FP64-pipe cycles/s",
            "frac": achieved / peak, "pipe_cycles_per_cell_pass": per_cell, "cells_per_pass": cells,
            "sm_mhz": sm_mhz, "n_sm": n_sm, "kernel": kernel,
            "source": f"profiles/{kernel}_{workload}.md (per-cell FP64-pipe cycles: sm__pipe_fp64_cycles_active "
                      f"x sm__cycles_active over the SMs, divided by the cells of the captured launch)"}


class ClockSampler:
    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return

        def rd():
            for line in self.proc.stdout:
                self.samples.append([x.strip() for x in line.split(",")])

        self.thread = threading.Thread(target=rd, daemon=True)
        self.thread.start()

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[0]))
                mx = float(s[1])
                for n, v in zip(names, s[2:6]):
                    if v.lower() in ("active", "1", "yes"):
                        reasons.add(n)
            except Exception:
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(params, b0=None, seconds=15.0, max_steps=100000, snapshot=None):
    """Oracle timed on a bounded sample: accepted steps until ~`seconds`, from t = 0 or,
    with a snapshot (the GPU run's state at the end of its spin-up), from that state."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle
    from kestrel_gb300 import abi
    from kestrel_gb300.solver import Simulation
    L = _oracle.load()
    if snapshot is not None:
        sim = Simulation(L, "ko", params, b0=b0, load_sources=False)
        sim.load_state(*snapshot)
    else:
        sim = _oracle.simulation(params, b0=b0)
    t_start = sim.time[0]
    total_cu, total_s, steps = 0, 0.0, 0
    rc = C.c_int32(0)
    while total_s < seconds and steps < max_steps:
        st = abi.StepStats()
        dt = L.ko_timed_steps(sim.h, 1, C.byref(st), C.byref(rc))
        if rc.value != 0:
            break
        total_cu += st.cell_updates
        total_s += dt
        steps += st.steps
        if sim.time[0] >= params.tend:
            break
    return {"value": total_cu / total_s if total_s > 0 else None, "unit": "cell-updates/s", "cores": 1,
            "host_cores": os.cpu_count(), "kind": "port", "sample": f"{steps} accepted steps from t={t_start:.3f} s to {sim.time[0]:.3f} s"
            + (f" (from the GPU run's state at the end of its spin-up, {len(snapshot[0])} tiles)" if snapshot else "") + ", "
            f"{total_cu} cell-updates in {total_s:.2f} s, serial C++ restatement (oracle)"}


def run_reference(args, wl):
    from kestrel_gb300 import abi  # noqa: F401
    made = wl["params"]()
    p, b0 = made if isinstance(made, tuple) else (made, None)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle
    from kestrel_gb300.solver import Simulation
    L = _oracle.load()
    spin = wl.get("spinup", 0.0) if args.spinup is None else args.spinup
    start = "t=0"
    snap = None
    if spin > 0.0:
        # The same window as the GPU arm: the state at the end of the spin-up, integrated by
        # the GPU's FP64 plain path (equal to the oracle within 1e-10 on the parity tests),
        # is loaded into the oracle (ko_load_state, LoadInitialCondition) and the oracle's
        # own steps are timed from there.  Without a GPU the oracle starts at t = 0.
        try:
            from kestrel_gb300 import abi as A0, lib
            g = lib.simulation(p, precision=A0.PREC_FP64, b0=b0)
            g.integrate_to(spin)
            snap = take_snapshot(g)
            g.close()
            start = (f"t={snap[3]:.3f} s ({len(snap[0])} tiles): the state integrated to the end of the spin-up by the "
                     f"FP64 GPU path and loaded into the oracle")
        except Exception as e:  # no GPU: time the same configuration from its start
            start = f"t=0 (no spin-up state: {e!r})"
    if snap is not None:
        sim = Simulation(L, "ko", p, b0=b0, load_sources=False)
        sim.load_state(*snap)
    else:
        sim = _oracle.simulation(p, b0=b0)
    rc = C.c_int32(0)
    from kestrel_gb300 import abi as A
    for _ in range(args.warmup):
        st = A.StepStats()
        L.ko_timed_steps(sim.h, 1, C.byref(st), C.byref(rc))
    cu, secs, n = 0, 0.0, 0
    for _ in range(args.steps):
        st = A.StepStats()
        secs += L.ko_timed_steps(sim.h, 1, C.byref(st), C.byref(rc))
        cu += st.cell_updates
        n += st.steps
    v = cu / secs if secs > 0 else None
    line = {"metric": "cell-updates/s", "value": v, "unit": "cell-updates/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * secs / max(n, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": args.workload, "desc": wl["desc"], "active_cells_end": len(sim.active_tiles()) * p.nXpertile * p.nYpertile,
                       "l2": "n/a (CPU)", "parallelism": "single"},
            "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": 1, "host_cores": os.cpu_count(), "kind": "port",
                             "sample": f"{n} accepted steps after {args.warmup} warm-up steps from {start}, serial C++ "
                                       f"restatement (oracle)"},
            "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_reference_members(args):
    """The reference arm for the batched and served forms: the oracle (serial, one core)
    advancing the first members of the same ensemble or request stream one after another,
    a bounded sample of about 20 s of CPU work; cell-updates per second over the sample."""
    from kestrel_gb300 import abi as A, workloads
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle
    L = _oracle.load()
    if args.workload == "ensemble_fp32":
        members = [(p, b0) for p, b0, _ in workloads.ensemble(8)]
    else:
        members = [(p, b0) for _, p, b0, _ in workloads.serve_requests(8, rate=args.rate,
                                                                       tend_range=(args.tend_min, args.tend_max))]
    rc = C.c_int32(0)
    cu, secs, n, used = 0, 0.0, 0, 0
    for p, b0 in members:
        if secs >= 20.0:
            break
        sim = _oracle.simulation(p, b0=b0)
        used += 1
        while secs < 20.0 * used / len(members) and sim.time[0] < p.tend:
            st = A.StepStats()
            secs += L.ko_timed_steps(sim.h, 1, C.byref(st), C.byref(rc))
            cu += st.cell_updates
            n += st.steps
        sim.close()
    v = cu / secs if secs > 0 else None
    sample = f"{n} accepted steps of the first {used} members, serial C++ restatement (oracle)"
    print(json.dumps({"metric": "cell-updates/s", "value": v, "unit": "cell-updates/s", "n_gpus": args.gpus,
                      "steps": n, "warmup": 0, "ms_per_step": 1e3 * secs / max(n, 1), "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
                      "config": {"workload": args.workload},
                      "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": 1, "host_cores": os.cpu_count(), "kind": "port", "sample": sample},
                      "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def run_ensemble(args):
    """The batched ensemble: N members (grid sides log-uniform in [128, 1024]
    at dx = 5 m, own fractal terrain, cap or flux source of 1e3-1e6 m^3, Chezy / Voellmy /
    Manning drag, morphodynamics on for half), tile sides from the autotuner, all advanced
    together; value = member cell-updates per second of device time over the timed batch
    steps (CUDA events on the batch stream, L2 flushed between steps)."""
    import torch
    from kestrel_gb300 import autotune, lib, workloads
    from kestrel_gb300.batch import Batch
    L = lib.load()
    t0 = time.perf_counter()
    cache = os.path.join(ROOT, "kestrel_gb300", "_build", "autotune.json")
    tuned = autotune.tune(cache=cache, log=lambda m: print(m, file=sys.stderr))
    t_tune = time.perf_counter() - t0
    members = workloads.ensemble(args.members, tiles=lambda side: autotune.tile_for(side, tuned))
    b = Batch(args.members, graphs=bool(args.batch_graphs))
    t1 = time.perf_counter()
    ids = [b.add(p, b0) for p, b0, _ in members]
    t_add = time.perf_counter() - t1
    sims = [b.member(i) for i in ids]
    cnt = (C.c_int64 * 3)()

    def cells():
        tot = 0
        for s in sims:
            L.kg_get_counters(s.h, cnt)
            tot += cnt[2]
        return tot
    for _ in range(args.spinup_steps):
        b.step()
    stream = torch.cuda.ExternalStream(b.stream())
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        b.step()
    torch.cuda.synchronize()
    c0 = cells()
    l0, r0 = b.stats()
    clocks = ClockSampler(0)
    clocks.start()
    evs, wall0 = [], time.perf_counter()
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        b.step()
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    ms = sum(a.elapsed_time(e) for a, e in evs)
    cu = cells() - c0
    l1, r1 = b.stats()
    hbm = sum(L.kg_device_bytes(s.h) for s in sims)
    sides = [d["side"] for _, _, d in members]
    line = {"metric": "cell-updates/s", "value": cu / (ms / 1e3), "unit": "cell-updates/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "ensemble_fp32", "members": args.members, "sides": [min(sides), max(sides)],
                       "tiles": {str(k): v for k, v in tuned.items()}, "morpho_members": sum(d["morpho"] for _, _, d in members),
                       "spinup_batch_steps": args.spinup_steps,
                       "l2": "flushed (256 MiB write) between timed batch steps, outside the timed intervals"},
            "e2e": {"value": cu / wall, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                    "note": "host clock around the same batch steps (control words only cross per step)"},
            "batch": {"kernel_launches_per_step": (l1 - l0) / args.steps, "rounds_per_step": (r1 - r0) / args.steps,
                      "device_gb": hbm / 1e9, "autotune_s": t_tune, "add_s": t_add, "graphs": bool(args.batch_graphs),
                      "graph_launches_updates_instantiations_replays": list(b.graph_stats())},
            "clocks": clk}
    b.close()
    return line


def run_serve(args):
    """The served stream: requests arrive as a Poisson process (--rate per s),
    grid sides uniform over {256, 512, 1024, 2048}, end times uniform over
    [--tend-min, --tend-max] s, admitted by the HBM budget into one continuously batched
    engine; reports p50/p99 latency, solves/s and cell-updates/s (host clock)."""
    from kestrel_gb300 import autotune, serve, workloads
    cache = os.path.join(ROOT, "kestrel_gb300", "_build", "autotune.json")
    tuned = autotune.tune(cache=cache)
    reqs = [serve.Request(arrival=t, params=p, b0=b0, desc=d) for t, p, b0, d in
            workloads.serve_requests(args.requests, rate=args.rate, tend_range=(args.tend_min, args.tend_max),
                                     tiles=lambda side: autotune.tile_for(side, tuned))]
    srv = serve.Server(hbm_budget=args.budget_gb * 1e9, max_members=min(256, args.requests), keep_state=False,
                       graphs=bool(args.serve_graphs))
    clocks = ClockSampler(0)
    clocks.start()
    try:
        rep = srv.run(reqs, max_wall_s=getattr(args, "serve_max_wall", None))
    finally:
        clk = clocks.stop()
        srv.close()
    line = {"metric": "cell-updates/s", "value": rep["cell_updates_per_s"], "unit": "cell-updates/s", "n_gpus": 1,
            "steps": rep["batch_steps"], "warmup": 0, "ms_per_step": 1e3 * rep["makespan_s"] / max(rep["batch_steps"], 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "serve_fp32", "requests": args.requests, "rate_per_s": args.rate,
                       "tend_s": [args.tend_min, args.tend_max], "hbm_budget_gb": args.budget_gb,
                       "sides": [256, 512, 1024, 2048], "graphs": bool(args.serve_graphs)},
            "serve": rep, "clocks": clk}
    return line


def extras_ensemble(args):
    """The batched ensemble beside the headline: --members members (128^2-1024^2), its
    device-timed and host-clock throughput and round shape."""
    import copy
    a = copy.copy(args)
    a.steps, a.warmup = 20, 3
    r = run_ensemble(a)
    return {"workload": r["config"]["workload"], "value": r["value"], "unit": r["unit"], "e2e": r["e2e"]["value"],
            "ms_per_round": r["ms_per_step"], "rounds": r["steps"], "members": r["config"]["members"],
            "morpho_members": r["config"]["morpho_members"], "sides": r["config"]["sides"], "tiles": r["config"]["tiles"],
            "batch": r["batch"], "dtype": "f32", "clocks": r.get("clocks")}


def extras_serve(args):
    """The served request stream beside the headline (Poisson arrivals at
    --rate per s, sides 256-2048, HBM budget --budget-gb), with the end times scaled by
    --serve-tend-scale so that the whole stream is served within the default run."""
    import copy
    a = copy.copy(args)
    a.tend_min, a.tend_max = args.tend_min * args.serve_tend_scale, args.tend_max * args.serve_tend_scale
    a.serve_max_wall = 300.0
    r = run_serve(a)
    rep = r["serve"]
    return {"workload": "serve_fp32", "requests": a.requests, "rate_per_s": a.rate,
            "tend_s": [a.tend_min, a.tend_max], "tend_scale": args.serve_tend_scale,
            "latency_p50_s": rep.get("latency_p50_s"), "latency_p99_s": rep.get("latency_p99_s"),
            "solves_per_s": rep.get("solves_per_s"), "cell_updates_per_s": rep.get("cell_updates_per_s"),
            "makespan_s": rep.get("makespan_s"), "peak_members": rep.get("peak_members"),
            "peak_budget_gb": rep.get("peak_budget_gb"), "hbm_budget_gb": a.budget_gb, "dtype": "f32",
            "note": "host clock from the first arrival; end times of the configuration ([60, 600] s) scaled by "
                    f"{args.serve_tend_scale} so that the stream is served within the default run"}


EXTRAS = {"sparse_8192_fp32": lambda a: run_sparse_window(a, t_window=a.sparse_window, deadline_s=240.0),
          "ensemble_fp32": lambda a: extras_ensemble(a),
          "serve_fp32": lambda a: extras_serve(a)}


def run_extra(key: str, args, timeout_s: float = 600.0):
    """One secondary figure beside the headline, run as `bench.py --extra key` in a child
    process; returns its JSON, or {"error": ...} when it fails, crashes or runs out of time."""
    cmd = [sys.executable, os.path.abspath(__file__), "--extra", key, "--sparse-window", str(args.sparse_window),
           "--members", str(args.members), "--requests", str(args.requests), "--rate", str(args.rate),
           "--tend-min", str(args.tend_min), "--tend-max", str(args.tend_max), "--budget-gb", str(args.budget_gb),
           "--serve-tend-scale", str(args.serve_tend_scale), "--batch-graphs", str(args.batch_graphs),
           "--serve-graphs", str(args.serve_graphs)]
    try:
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=timeout_s)
    except subprocess.TimeoutExpired:
        return {"error": f"no result within {timeout_s:.0f} s"}
    sys.stderr.write(r.stderr)
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    if r.returncode == 0 and lines:
        return json.loads(lines[-1])
    return {"error": f"exit code {r.returncode}", "stderr_tail": r.stderr[-600:]}


def run_sparse_window(args, t_window: float = 200.0, steps: int = 20, deadline_s=None):
    """The large sparse configuration (8192^2 cells in 16,384 tiles of 64^2, three seeded
    flux sources, Pouliquen drag, morphodynamics; FP32 form): an untimed spin-up to
    t_window (the active-tile count recorded every 20 s), then `steps` accepted steps
    device-timed as the headline (CUDA events on the library's stream, L2 flushed between
    steps).  Beside the headline the window is t = 200 s (about 3% of the tiles active, a
    spin-up of about 1.5 minutes); the configuration reaches 5% at its end time, t = 300 s,
    which --sparse-window 290 times after a spin-up of about 5 minutes."""
    import torch
    from kestrel_gb300 import lib, workloads
    L = lib.load()
    wl = workloads.WORKLOADS["sparse_8192_fp32"]
    p, b0 = wl["params"]()
    t0 = time.perf_counter()
    sim = lib.simulation(p, precision=wl["prec"], b0=b0)
    try:
        timeline = spin_up(sim, p, t_window, 20.0, deadline_s=deadline_s)
    except TimeoutError as e:
        n_st = (C.c_int64 * 3)()
        L.kg_get_counters(sim.h, n_st)
        sim.close()
        return {"workload": "sparse_8192_fp32", "error": str(e), "active_timeline": getattr(e, "timeline", None),
                "steps_accepted_refused": [n_st[0], n_st[1]]}
    spin_s = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(L.kg_stream(sim.h))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    for _ in range(3):
        sim.step(p.tend)
    torch.cuda.synchronize()
    evs, cu, n = [], 0, 0
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        st = sim.step(p.tend)
        e1.record(stream)
        evs.append((e0, e1))
        cu += st.cell_updates
        n += st.steps
        if sim.time[0] >= p.tend:
            break
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in evs)
    act = len(sim.active_tiles())
    t_end = sim.time[0]
    sim.close()
    total = p.nXtiles * p.nYtiles
    return {"workload": "sparse_8192_fp32", "value": cu / (ms / 1e3) if ms > 0 else None, "unit": "cell-updates/s",
            "steps": n, "ms_per_step": ms / max(n, 1), "t_window": [t_window, round(t_end, 3)],
            "active_tiles": act, "active_percent": round(100.0 * act / total, 3), "active_timeline": timeline,
            "spinup_wall_s": spin_s, "dtype": "f32",
            "note": "device-timed steps after an untimed spin-up to the window; L2 flushed between steps"}


def reduce_replicas(seconds, cell_updates, dist=None, device="cpu"):
    """Replicas (one simulation per rank, no exchange between them): the job's time is the
    slowest rank's and its work the sum of the ranks' cell-updates.  Returns (seconds, cell
    updates) for the whole job; without a process group, the rank's own."""
    if not dist:
        return float(seconds), float(cell_updates)
    import torch
    tt = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    cc = torch.tensor([float(cell_updates)], dtype=torch.float64, device=device)
    dist.all_reduce(cc)
    return float(tt.item()), float(cc.item())


def spin_up(sim, p, spin, every=None, deadline_s=None):
    """Untimed integration to t = spin; with `every`, the active-tile count is recorded at
    each multiple of `every` seconds: [[t, active tiles, percent of all tiles], ...] (and
    printed to stderr as it goes).  With `deadline_s`, the integration runs step by step and
    raises TimeoutError once that much wall time has passed (a secondary figure must not
    hold up the bench line)."""
    out = []
    if spin <= 0.0:
        return out
    if not every and not deadline_s:
        sim.integrate_to(spin)
        return out
    total = p.nXtiles * p.nYtiles
    t, t0 = 0.0, time.perf_counter()
    every = every or spin
    while t < spin:
        t = min(spin, t + every)
        if deadline_s:
            while sim.time[0] < t:
                sim.step(t)
                if time.perf_counter() - t0 > deadline_s:
                    n = len(sim.active_tiles())
                    out.append([round(sim.time[0], 3), n, round(100.0 * n / total, 3)])
                    e = TimeoutError(f"spin-up reached t={sim.time[0]:.3f} s of {spin} s in {deadline_s:.0f} s of wall time")
                    e.timeline = out
                    raise e
        else:
            sim.integrate_to(t)
        n = len(sim.active_tiles())
        out.append([round(sim.time[0], 3), n, round(100.0 * n / total, 3)])
        print(f"spin-up t={sim.time[0]:.1f} s: {n} active tiles, {time.perf_counter() - t0:.1f} s wall", file=sys.stderr, flush=True)
    return out


def take_snapshot(sim):
    """(tile ids, state (n, 4, nY, nX), vertex bt (n, nY+1, nX+1), t) of a running simulation."""
    import numpy as np
    ids = sim.active_tiles()
    state = np.stack([np.stack([sim.field(t, f) for f in (1, 2, 3, 4)]) for t in ids])
    btv = np.stack([sim.vertex(t, 1) for t in ids])
    return ids, state, btv, sim.time[0]


def run_dem(args):
    """Raster topography ingestion on the 2048^2 configuration: kg_upload_raster computes
    every tile's vertex heights (1024 tiles x 65^2 vertices, four bicubic samples each)
    from a 2.5 m raster of the domain (4128^2 pixels).  value = vertex heights per second
    of device time (CUDA events on the context's stream around the call, which includes
    the raster's host-to-device copy); e2e = the same through the host clock.  The CPU
    baseline is the oracle computing the heights of the tiles its set-up activates."""
    from kestrel_gb300 import abi, workloads
    p, r = workloads.dem_2048()
    nvt = (p.nXpertile + 1) * (p.nYpertile + 1)
    if args.impl == "reference":
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import _oracle
        t1 = time.perf_counter()
        o = _oracle.simulation(p, raster=r)
        secs = time.perf_counter() - t1
        nt = len(o.active_tiles()) + len(o.ghost_tiles())
        v = nt * nvt / secs
        print(json.dumps({"metric": "vertex-heights/s", "value": v, "unit": "vertex-heights/s", "n_gpus": args.gpus,
                          "steps": 1, "warmup": 0, "ms_per_step": 1e3 * secs, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
                          "config": {"workload": "dem_2048"},
                          "cpu_baseline": {"value": v, "unit": "vertex-heights/s", "cores": 1, "host_cores": os.cpu_count(), "kind": "port",
                                           "sample": f"oracle set-up: raster copy, sources and the heights of its {nt} active and ghost tiles"},
                          "e2e": {"value": v, "unit": "vertex-heights/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    import torch
    from kestrel_gb300 import lib
    from kestrel_gb300.solver import Simulation
    L = lib.load()
    sim = Simulation(L, "kg", p, precision=abi.PREC_FP64, load_sources=False)
    stream = torch.cuda.ExternalStream(L.kg_stream(sim.h))
    for _ in range(args.warmup):
        sim.upload_raster(**r)
    torch.cuda.synchronize()
    steps = min(args.steps, 20)
    clocks = ClockSampler(0)
    clocks.start()
    evs, t0 = [], time.perf_counter()
    for _ in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.upload_raster(**r)
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    ms = sum(a.elapsed_time(b) for a, b in evs)
    nv = p.nXtiles * p.nYtiles * nvt
    sim.close()
    line = {"metric": "vertex-heights/s", "value": nv * steps / (ms / 1e3), "unit": "vertex-heights/s", "n_gpus": 1,
            "steps": steps, "warmup": args.warmup, "ms_per_step": ms / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "dem_2048", "raster": list(r["values"].shape), "pixel_m": r["pixel"][0],
                       "tiles": p.nXtiles * p.nYtiles, "vertices_per_tile": (p.nXpertile + 1) * (p.nYpertile + 1),
                       "l2": "inputs (136 MB raster) larger than L2; not flushed"},
            "e2e": {"value": nv * steps / wall, "unit": "vertex-heights/s", "h2d_bytes_per_step": int(r["values"].nbytes),
                    "d2h_bytes_per_step": 4 * p.nXtiles * p.nYtiles},
            "gpu_launches": steps, "clocks": clk}
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import _oracle
        t1 = time.perf_counter()
        o = _oracle.simulation(p, raster=r)
        secs = time.perf_counter() - t1
        nt = len(o.active_tiles()) + len(o.ghost_tiles())
        line["cpu_baseline"] = {"value": nt * (p.nXpertile + 1) * (p.nYpertile + 1) / secs, "unit": "vertex-heights/s",
                                "cores": 1, "host_cores": os.cpu_count(), "kind": "port",
                                "sample": f"oracle set-up: raster copy, sources and the heights of its {nt} active and ghost tiles, {secs:.2f} s"}
    print(json.dumps(line))


def run_fp32_error(args):
    """The FP32 form's depth error on the 2048^2 morphodynamic configuration against the
    FP64 path, set beside the configuration's own sensitivity to its inputs: the FP64 path
    run again with the hydrograph's peak inflow scaled by (1 + 2^-52) (one FP64 rounding)
    and by (1 + 2^-24) (one FP32 rounding).  At each checkpoint every run is compared with
    the unperturbed FP64 run over the tiles active in either (an inactive tile is dry):
    relative L-inf of the depth Hn and its 99th percentile over the cells wet in either run,
    both relative to the largest FP64 depth, with the accepted and refused step counts."""
    import numpy as np
    import torch
    from kestrel_gb300 import abi, lib, workloads
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    times = [float(x) for x in args.error_times.split(",")]
    runs = [("fp64", abi.PREC_FP64, 0.0), ("fp64_inflow_2^-52", abi.PREC_FP64, 2.0 ** -52),
            ("fp64_inflow_2^-24", abi.PREC_FP64, 2.0 ** -24), ("fp32", abi.PREC_FP32, 0.0)]
    sims, stats = {}, {}
    for name, prec, eps in runs:
        p, b0 = workloads.morpho_flux_2048()
        p.sources[0].flux[1] = p.sources[0].flux[1] * (1.0 + eps)
        sims[name] = lib.simulation(p, precision=prec, b0=b0)
        stats[name] = [0, 0]
    nX, nY = p.nXpertile, p.nYpertile

    def depth(sim):
        return {t: sim.field(t, 5) for t in sim.active_tiles()}

    rows = []
    t0 = time.perf_counter()
    for tc in times:
        hs = {}
        for name, _, _ in runs:
            st = sims[name].integrate_to(tc)
            stats[name][0] += st.steps
            stats[name][1] += st.rejected
            hs[name] = depth(sims[name])
        ref = hs["fp64"]
        scale = max(float(np.max(np.abs(v))) for v in ref.values())
        row = {"t": tc, "fp64_steps": stats["fp64"][0], "fp64_active_tiles": len(ref), "max_depth": scale}
        zero = np.zeros((nY, nX))
        for name, _, _ in runs[1:]:
            h = hs[name]
            tiles = sorted(set(ref) | set(h))
            a = np.concatenate([ref.get(t, zero).ravel() for t in tiles])
            b = np.concatenate([h.get(t, zero).ravel() for t in tiles])
            d = np.abs(a - b)
            wet = (a > 0) | (b > 0)
            row[name] = {"linf": float(d.max() / scale), "p99": float(np.percentile(d[wet], 99) / scale) if wet.any() else 0.0,
                         "steps": stats[name][0], "rejected": stats[name][1], "active_tiles": len(h)}
        rows.append(row)
        print(json.dumps(row), file=sys.stderr, flush=True)
    for s in sims.values():
        s.close()
    print(json.dumps({"workload": "fp32_error_2048",
                      "desc": "depth of the FP32 form and of FP64 runs with the peak inflow scaled by (1 + 2^-52) and "
                              "(1 + 2^-24), against the unperturbed FP64 run on the 2048^2 morphodynamic configuration; "
                              "linf and p99 relative to the largest FP64 depth, over the tiles active in either run",
                      "seconds": time.perf_counter() - t0, "checkpoints": rows}))


def fp64_plain(args, wname, snapshot=None):
    """The plain FP64 drop-in on the same configuration, device-timed the same way (for the
    FP32-vs-FP64 comparison of the headline line).  With a snapshot, the FP64 context is
    restarted from the FP32 run's state at the end of its spin-up (kg_load_state) instead of
    integrating the spin-up again."""
    import torch
    from kestrel_gb300 import lib, workloads
    from kestrel_gb300.solver import Simulation
    L = lib.load()
    wl = workloads.WORKLOADS[wname]
    made = wl["params"]()
    p, b0 = made if isinstance(made, tuple) else (made, None)
    if snapshot is not None:
        sim = Simulation(L, "kg", p, precision=wl["prec"], b0=b0, load_sources=False)
        sim.load_state(*snapshot)
    else:
        sim = lib.simulation(p, precision=wl["prec"], b0=b0)
        spin = wl.get("spinup", 0.0) if args.spinup is None else args.spinup
        if spin > 0.0:
            sim.integrate_to(spin)
    own_snapshot = take_snapshot(sim)  # the FP64 state the CPU baseline starts from
    stream = torch.cuda.ExternalStream(L.kg_stream(sim.h))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        sim.step(p.tend)
    torch.cuda.synchronize()
    timed = L.kg_set_kernel_timing(sim.h, 1) == 0  # pass times, as in the main leg
    evs, cu, n = [], 0, 0
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        st = sim.step(p.tend)
        e1.record(stream)
        evs.append((e0, e1))
        cu += st.cell_updates
        n += st.steps
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in evs)
    # end to end through the C ABI: the same number of steps on the host clock (each
    # returns its statistics), then the conserved fields of every active tile read back
    xb0 = (C.c_int64 * 2)()
    L.kg_get_transfer_bytes(sim.h, xb0)
    cu_e, n_e = 0, 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st = sim.step(p.tend)
        cu_e += st.cell_updates
        n_e += st.steps
    sim.get_state()  # the conserved fields and bed change of every active tile, one call
    e2e_s = time.perf_counter() - t0
    xb1 = (C.c_int64 * 2)()
    L.kg_get_transfer_bytes(sim.h, xb1)
    active = len(sim.active_tiles())
    pass_ms = None
    if timed:
        kms, kpasses = C.c_double(), C.c_int64()
        if L.kg_get_kernel_time(sim.h, C.byref(kms), C.byref(kpasses)) == 0 and kpasses.value > 0:
            pass_ms = kms.value / kpasses.value
    sim.close()
    out = {"workload": wname, "value": cu / (ms / 1e3), "unit": "cell-updates/s", "steps": n, "ms_per_step": ms / max(n, 1),
           "active_tiles_end": active, "pass_ms": pass_ms,
           "e2e": {"value": cu_e / e2e_s if e2e_s > 0 else None, "unit": "cell-updates/s",
                   "h2d_bytes_per_step": (xb1[0] - xb0[0]) / max(n_e, 1), "d2h_bytes_per_step": (xb1[1] - xb0[1]) / max(n_e, 1),
                   "note": f"host clock around {n_e} further kg_step calls, then the read-back of the conserved fields "
                           f"and bed change (kg_get_state)"}}
    try:  # the FP64 pass against its FP64 pipe; the clock is the GPU's maximum (not sampled here)
        cells = cu / max(n, 1) / (2.0 if p.MorphodynamicsOn else 1.0)
        n_sm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        out["roofline_fp64"] = fp64_pipe_roofline("k_hydro", wname, cells, pass_ms, measured_sm_max_mhz(), n_sm)
    except Exception as e:
        out["roofline_fp64"] = {"error": repr(e)}
    if snapshot is not None:
        out["start"] = f"restarted from the FP32 run's state at t={snapshot[3]:.3f} s ({len(snapshot[0])} tiles)"
    out["_snapshot"] = own_snapshot
    return out


def main():
    faulthandler.enable()  # a native crash prints the Python stack to stderr
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="morpho_flux_2048_fp32")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 plain measurement beside an FP32 workload")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--spinup", type=float, default=None, help="override the workload's untimed spin-up (s)")
    ap.add_argument("--profile", action="store_true", help="cudaProfilerStart/Stop around the timed steps")
    ap.add_argument("--members", type=int, default=256, help="ensemble: members")
    ap.add_argument("--spinup-steps", type=int, default=20, help="ensemble: untimed batch steps")
    ap.add_argument("--requests", type=int, default=24, help="serve: requests")
    ap.add_argument("--rate", type=float, default=20.0, help="serve: arrivals per second")
    ap.add_argument("--tend-min", type=float, default=60.0)
    ap.add_argument("--tend-max", type=float, default=600.0)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--serve-tend-scale", type=float, default=0.1, help="served stream beside the headline: end-time scale")
    ap.add_argument("--no-extras", action="store_true", help="headline only (no sparse, ensemble and served keys)")
    ap.add_argument("--batch-graphs", type=int, default=1, help="ensemble: replay the rounds through CUDA graphs")
    ap.add_argument("--serve-graphs", type=int, default=0,
                    help="served stream: replay the rounds through CUDA graphs (off: members joining and leaving "
                         "have ended in a host-side crash with graphs)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end legs (profiling runs)")
    ap.add_argument("--sparse-window", type=float, default=200.0,
                    help="sparse configuration beside the headline: spin-up end (s) of its timed window")
    ap.add_argument("--fused-morpho", type=int, default=1,
                    help="FP32 form: one launch per morphodynamic stage (1) or three (0); same results")
    ap.add_argument("--dry-skip", type=int, default=1,
                    help="FP32 form: skip the flux work of blocks with no water (1) or run every block (0)")
    ap.add_argument("--error-times", default="5,10,20,40,80,120",
                    help="fp32_error_2048: checkpoints (s) of the depth comparison")
    ap.add_argument("--extra", default=None, choices=sorted(EXTRAS), help=argparse.SUPPRESS)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    if args.extra:  # one secondary figure, in the child process run_extra starts
        try:
            print(json.dumps(EXTRAS[args.extra](args)))
        except Exception as e:
            print(json.dumps({"error": repr(e)}))
        return

    if args.workload == "fp32_error_2048":
        if int(os.environ.get("RANK", "0")) != 0 or args.impl == "reference":
            return
        return run_fp32_error(args)

    if args.workload in ("ensemble_fp32", "serve_fp32") and args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        return run_reference_members(args)
    if args.workload == "ensemble_fp32" and args.impl == "ours":
        print(json.dumps(run_ensemble(args)))
        return
    if args.workload == "serve_fp32" and args.impl == "ours":
        print(json.dumps(run_serve(args)))
        return
    if args.workload == "dem_2048":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        return run_dem(args)
    from kestrel_gb300 import workloads
    wl = workloads.WORKLOADS[args.workload]
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args, wl)
        return

    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from kestrel_gb300 import abi, lib
    L = lib.load()
    made = wl["params"]()
    p, b0 = made if isinstance(made, tuple) else (made, None)

    # ---- device-timed throughput ----
    sim = lib.simulation(p, precision=wl["prec"], b0=b0)
    L.kg_set_fused_morpho(sim.h, args.fused_morpho)
    L.kg_set_dry_skip(sim.h, args.dry_skip)
    spin = wl.get("spinup", 0.0) if args.spinup is None else args.spinup
    timeline = spin_up(sim, p, spin, wl.get("timeline"))
    stream = torch.cuda.ExternalStream(L.kg_stream(sim.h))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > L2
    for _ in range(args.warmup):
        sim.step(p.tend)
    torch.cuda.synchronize()
    snapshot = take_snapshot(sim) if (wl.get("twin_restart") or spin > 0.0) else None
    L.kg_set_kernel_timing(sim.h, 1)
    launches0 = L.kg_kernel_launches(sim.h)
    clocks = ClockSampler(local)
    if rank == 0:
        clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    if args.profile:
        torch.cuda.cudart().cudaProfilerStart()
    total_ms, cu, nsteps = 0.0, 0, 0
    evs = []
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        st = sim.step(p.tend)
        e1.record(stream)
        evs.append((e0, e1))
        cu += st.cell_updates
        nsteps += st.steps
        if sim.time[0] >= p.tend:
            break
    torch.cuda.synchronize()
    if args.profile:
        torch.cuda.cudart().cudaProfilerStop()
    total_ms = sum(a.elapsed_time(b) for a, b in evs)
    if dist:
        dist.barrier()
    clk = clocks.stop() if rank == 0 else None
    launches = L.kg_kernel_launches(sim.h) - launches0
    kms, kpasses = C.c_double(), C.c_int64()
    L.kg_get_kernel_time(sim.h, C.byref(kms), C.byref(kpasses))
    t_s = total_ms / 1e3
    t_s, cu_all = reduce_replicas(t_s, cu, dist, "cuda")
    value = cu_all / t_s
    active_cells = len(sim.active_tiles()) * p.nXpertile * p.nYpertile
    sim.close()

    # ---- end to end through the C ABI ----
    # (1) e2e: the same kind of steps as `value` (after the same untimed spin-up and
    # warm-up), host clock around kg_step calls that return their statistics to the host
    # every step, plus the read-back of the conserved fields of every active tile at the
    # end; the bytes are the library's own count of its host<->device copies.
    # (2) e2e_job: the whole job from kg_create (settings and the bed grid uploaded) through
    # the spin-up and the same steps to the final read-back.
    e2e_s = job_s = 0.0
    cu2 = n2 = cu_job = fields_bytes = 0
    xb0, xb1 = (C.c_int64 * 2)(), (C.c_int64 * 2)()
    if not args.no_e2e:
        t_job = time.perf_counter()
        sim2 = lib.simulation(p, precision=wl["prec"], b0=b0)
        cu_job = 0
        if spin > 0.0:
            cu_job += sim2.integrate_to(spin).cell_updates
        for _ in range(args.warmup):
            cu_job += sim2.step(p.tend).cell_updates
        xb0 = (C.c_int64 * 2)()
        L.kg_get_transfer_bytes(sim2.h, xb0)
        cu2, n2 = 0, 0
        t0 = time.perf_counter()
        for _ in range(args.steps):
            st = sim2.step(p.tend)
            cu2 += st.cell_updates
            n2 += st.steps
            if sim2.time[0] >= p.tend:
                break
        # the state a host reads back at the end: every active tile's conserved fields and
        # vertex bed change in one call (kg_get_state: one gather, one copy per array)
        _, st_fields, st_bt, _ = sim2.get_state()
        fields_bytes = st_fields.nbytes + st_bt.nbytes
        t1 = time.perf_counter()
        xb1 = (C.c_int64 * 2)()
        L.kg_get_transfer_bytes(sim2.h, xb1)
        e2e_s = t1 - t0
        job_s = t1 - t_job
        cu_job += cu2
        sim2.close()

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    key = "fp64_hydro" if wl["prec"] == abi.PREC_FP64 else "fp32_hydro"
    if p.MorphodynamicsOn:
        key = key.replace("hydro", "morpho")
    alg = ALG_BYTES[key]
    pass_ms = kms.value / max(kpasses.value, 1)
    kname = "k_hydro" if wl["prec"] == abi.PREC_FP64 else "k_hydro32"
    # cells of one pass: a Strang step advances each active cell by two cell-updates
    cells_pass = cu / max(nsteps, 1) / (2.0 if p.MorphodynamicsOn else 1.0)
    # algorithmic bytes of one pass: 92 B (FP64) or 63 B (FP32 form) per cell of the pass
    alg_pass = ALG_PASS_BYTES["fp64" if wl["prec"] == abi.PREC_FP64 else "fp32"] * cells_pass
    achieved = alg_pass / (pass_ms / 1e3) / 1e9 if pass_ms > 0 else None
    peak, peak_kind = measured_peaks()
    traffic = profile_traffic(kname, args.workload, cells_pass)
    # the whole step: algorithmic bytes per cell-update times the cell-updates of a step
    step_gbs = alg * (cu / max(nsteps, 1)) / (total_ms / max(nsteps, 1) / 1e3) / 1e9 if total_ms > 0 else None
    line = {
        "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": world, "steps": nsteps,
        "warmup": args.warmup, "ms_per_step": total_ms / max(nsteps, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if wl["prec"] == abi.PREC_FP64 else "f32", "data": "synthetic",
        "config": {"workload": args.workload, "desc": wl["desc"], "active_cells_end": active_cells,
                   "l2": "flushed (256 MiB write) between timed steps, outside the timed intervals",
                   "parallelism": "replicas" if world > 1 else "single",
                   "fused_morpho": bool(args.fused_morpho), "dry_skip": bool(args.dry_skip),
                   "dry_skip_note": "FP32 form: 16x16 blocks whose cells and 2-cell halo hold no water carry their "
                                    "state with a zero RHS (the full computation changes them only by round-off; "
                                    "A/B on this workload: 0.808 -> 0.772 ms per step with the fused M stages)"},
        "e2e": {"value": cu2 / e2e_s if e2e_s > 0 else None, "unit": "cell-updates/s", "h2d_bytes_per_step": (xb1[0] - xb0[0]) / max(n2, 1),
                "d2h_bytes_per_step": (xb1[1] - xb0[1]) / max(n2, 1),
                "note": f"host clock around {n2} kg_step calls after the same spin-up, then the read-back of the "
                        f"conserved fields and bed change of every active tile with kg_get_state ({fields_bytes} B, "
                        f"counted in d2h)"},
        "e2e_job": {"value": cu_job / job_s if job_s > 0 else None, "unit": "cell-updates/s", "seconds": job_s,
                    "note": "kg_create with the settings and bed grid uploaded, spin-up, warm-up and the same steps, "
                            "final read-back"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if achieved else None, "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": kname, "pass_ms": pass_ms, "cells_per_pass": cells_pass,
                     "alg_bytes_per_pass": alg_pass,
                     "traffic_over_alg": traffic / alg_pass if traffic and alg_pass else None,
                     "step": {"alg_bytes_per_cell_update": alg, "achieved": step_gbs,
                              "frac": step_gbs / peak if step_gbs else None},
                     "note": "achieved = algorithmic bytes of one fused hydraulic pass (" +
                             f"{alg_pass / max(cells_pass, 1):.0f} B per cell of the pass: a quarter of the "
                             "hydraulic step's bytes per cell-update) over the pass time from CUDA events on the "
                             "library's stream; traffic = DRAM bytes per pass from the committed ncu capture, scaled "
                             "to the pass's cells; step = the form's bytes per cell-update times the cell-updates of "
                             "a step over the device-timed step"},
        "gpu_launches": launches,
        "clocks": clk,
    }
    try:
        mhz = (clk or {}).get("sm_mhz") or measured_sm_max_mhz()
        n_sm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        line["roofline_fp64"] = fp64_pipe_roofline(kname, args.workload, cells_pass, pass_ms, mhz, n_sm)
    except Exception as e:  # a secondary figure: never lose the bench line for it
        line["roofline_fp64"] = {"error": repr(e)}
    if timeline:
        line["config"]["active_timeline"] = timeline
    if wl["prec"] == abi.PREC_FP32 and not args.no_fp64:
        twin = args.workload.replace("_fp32", "_fp64")
        if twin in workloads.WORKLOADS:
            f64 = fp64_plain(args, twin, snapshot if wl.get("twin_restart") else None)
            snap64 = f64.pop("_snapshot", None)
            if snap64 is not None and not wl.get("twin_restart"):
                # the oracle (FP64) starts from the FP64 path's state of the same window: the
                # FP32 form's state can hold the slightly negative thin-film solids that the
                # reference's excess-deposition test refuses over and over
                snapshot = snap64
            line["fp64_plain"] = f64
            line["fp32_over_fp64"] = line["value"] / f64["value"] if f64["value"] else None
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(p, b0, snapshot=snapshot)
    if args.workload == "morpho_flux_2048_fp32" and not args.no_extras:
        # the other forms of the metric on their own configurations, under their own keys;
        # each runs in a process of its own, so an error or a crash in one never loses the
        # headline line
        for key in ("sparse_8192_fp32", "ensemble_fp32", "serve_fp32"):
            line[key] = run_extra(key, args)

    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
