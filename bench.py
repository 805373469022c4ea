"""Benchmark of GOM's per-timestep core on GB300 through the C ABI.

Workload: the baroclinic estuary (about 150k cells: 600 x 250 squares of 100 m plus a 4-row
triangle strip, 20 z-layers, river 500 m3/s, ocean boundary with M2 0.6 m and S/T series,
TVD limiter on, wind stress 0.1 Pa, dt = 60 s), generated from a fixed seed.  A step is one
timestep of the core (main.f90:94-272).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

value          cell-layer-steps/s with the state resident in HBM: per step the host forcing
               (a few kB) is uploaded and gom_step_all replays the captured timestep graph;
               timed with CUDA events on the library's stream.
e2e            the same through the public API end to end: host forcing computed per step,
               uploaded from pinned memory, and the step's result (status, PCG iterations and
               the FP64 volume/salt sums) read back every step.
roofline       the dominant kernel (the transport column solve) timed alone with CUDA events,
               algorithmic bytes / time against the measured HBM copy bandwidth; traffic is
               the DRAM bytes per launch of that kernel from an ncu capture (a constant below,
               with the capture it came from).
cpu_baseline   the CPU restatement of the reference (oracle/), built with OpenMP over every
               host thread, on a bounded sample of the same workload.
e2e_device_series
               the e2e loop with the boundary forcing held on the device
               (gom_set_boundary_series): no forcing upload per step.
serving        a bounded storm-surge serving run (16 Poisson requests, quarter-scale meshes):
               p50 / p99 latency and throughput of packed mixed precision against plain FP64
               serving one request at a time on the same GPU (--no-serving skips it).
ensemble       the 96-run storm-surge ensemble at full size, packed mixed precision against plain
               FP64 one run at a time over the same 10 steps (--no-ensemble skips it).

N > 1 runs independent replicas (the single-run path does not shard): value is the sum over
ranks of cell-layer-steps divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import dataclasses
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-layer-steps/s; batched-ensemble p50/p99 latency vs plain FP64 on same GPU"
UNIT = "cell-layer-steps/s"
ORACLE_SO = ROOT / "oracle" / "_build" / "libgomoracle.so"
ORACLE_OMP_SO = ROOT / "oracle" / "_build" / "libgomoracle_omp.so"   # same loops, OpenMP-parallel

# algorithmic bytes per active unit and phase (FP64 state read once and written once per phase,
# integer topology counted once); the unit is stated beside each figure
PHASE_BYTES_PER_CELL_LAYER = {
    "advection": 100, "momentum": 208, "velocities": 120, "layers": 64, "node_velocity": 96,
    "density": 80, "bottom_friction": 2, "boundary_velocity": 0, "swap": 0,
}
TRANSPORT_BYTES_PER_CELL_LAYER_SUBCYCLE = 168
TRANSPORT_BYTES_PER_CELL_LAYER_AVERAGING = 72
PCG_BYTES_PER_CELL_ITERATION = 120
FS_ASSEMBLY_BYTES_PER_CELL_LAYER = 64


def make_deck(size: str, precision: str = "fp64", transport_solver: int = 1):
    import dataclasses
    from gom_release_gb300.deck import estuary
    if size == "small":
        d = estuary(nx=120, ny=50, dx=100.0, n_layers=20)
    elif size == "medium":
        d = estuary(nx=300, ny=125, dx=100.0, n_layers=20)
    else:
        d = estuary()
    if precision == "mixed":
        d = dataclasses.replace(d, params=dataclasses.replace(d.params, precision=1))
    if transport_solver == 2:
        # the ELM transport has no subcycles
        d = dataclasses.replace(d, params=dataclasses.replace(d.params, transport_solver=2, trans_sub_iter=1))
    return d


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.samples: list[list[str]] = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self) -> dict:
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def kernel_launches_per_step(deck) -> int:
    p = deck.params
    n = 1                                   # bottom friction
    n += 1 if deck.n_qb else 0              # river boundary velocity
    n += (3 if p.elm_backtrace_flag == 1 else 1) if p.advection_flag else 1
    n += 2                                  # momentum (dry-face clear + columns)
    n += 4                                  # assembly, PCG, node eta (wet, dry)
    n += 2                                  # face velocities, cell w
    n += 4                                  # layers: cells, faces, nodes, check
    n += 2                                  # face levels, node u/v/w
    if p.transport_flag:
        nt = max(1, p.trans_sub_iter)
        lim = p.h_flux_limiter > 0 or p.v_flux_limiter > 0
        per = (1 if deck.n_ob + deck.n_qb else 0) + 2 + (2 if lim else 0) + 1
        n += 1 + nt * per + 2
    if p.baroclinic_flag == 1:
        n += 3 if p.ana_density == 0 else 2
    if p.turbulence_flag:
        n += 2                              # closure: face columns, cell diffusivities
    return n


def stream_events(core):
    import torch
    stream = torch.cuda.ExternalStream(core.stream_handle())
    return torch, stream


def time_steps(run, forcings, torch, stream) -> float:
    """K steps (state resident, host forcing precomputed), CUDA events on the library stream."""
    core = run.core
    core.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for f in forcings:
        core.set_forcing(f)
        core.step_all()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / 1e3


def time_phases(deck, st_snapshot, lib, forcing, torch, reps: int = 3) -> dict:
    """Each phase timed alone with CUDA events on the library stream, from the same snapshot."""
    from gom_release_gb300.core import GomCore, TIME_LOOP
    core = GomCore(deck, lib=lib)
    core.load_state(st_snapshot)
    stream = torch.cuda.ExternalStream(core.stream_handle())
    out = {}
    for ph in TIME_LOOP:
        ts = []
        core.load_state(st_snapshot)
        core.set_forcing(forcing)
        for _ in range(reps):
            core.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            core.step(ph)
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3)
        out[ph] = min(ts)
    core.close()
    return out


# transport column solve, per active cell-layer and launch: tracers read (2 x 8) and written
# (2 x 8), face flux, diffusion and limiter coefficients of about two faces (2 x (8 + 8 + 2 x 8)),
# interface flux, diffusion and limiter (8 + 8 + 2 x 8), old and new thickness (2 x 8); FP32
# storage halves each term
TR_SOLVE_BYTES_PER_CELL_LAYER = {"fp64": 144, "mixed": 72}


# DRAM bytes per active cell-layer and launch of the transport solve: dram__bytes_read.sum +
# dram__bytes_write.sum of one ncu capture of the solve on the medium estuary (--size medium) over
# that case's active cell-layers.  The solve reads and writes a fixed set of arrays per wet
# cell-layer, so a launch's traffic is this figure times the workload's active cell-layers.
SOLVE_TRAFFIC_PER_CELL_LAYER = {
    "k_tr_solve fp64": 393.5,
    "k_tr_solve mixed": 257.7,
    "k_tr_rows64_sorted + k_tr_thomas_col fp64": 333.5 + 87.2,
}


# FP64 instructions (DADD + DMUL + DFMA, ncu smsp__sass_thread_inst_executed_op_d{add,mul,fma}_pred_on.sum)
# per active cell-layer and launch of the FP64 transport solve, from one ncu capture of the medium
# estuary (359,706 active cell-layers; the count per cell-layer does not depend on the mesh size)
SOLVE_FP64_INSTR_PER_CELL_LAYER = {
    "k_tr_rows64_sorted + k_tr_thomas_col": 157.3 + 32.0,
    "k_tr_solve": 186.5,
}

# FP64 warp instructions (ncu smsp__inst_executed_pipe_fp64.sum) per active cell-layer and launch,
# same capture.  GB300's FP64 pipe takes a warp instruction at one cost however many of its lanes
# are active, so its issue peak is the thread peak / 32 and this count, not the thread count, is
# what the pipe spends its time on.
SOLVE_FP64_WARP_INSTR_PER_CELL_LAYER = {
    "k_tr_rows64_sorted + k_tr_thomas_col": 5.620 + 1.157,
}


def solve_traffic(kernel: str, precision: str, ncl: int):
    """ncu DRAM bytes per launch of the transport solve on a workload of ncl active cell-layers."""
    per = SOLVE_TRAFFIC_PER_CELL_LAYER.get(f"{kernel} {precision}")
    return per * ncl if per is not None else None


def phase_bytes(deck, ncl: int, pcg_iters: float) -> dict:
    p = deck.params
    nt = max(1, p.trans_sub_iter)
    b = {ph: v * ncl for ph, v in PHASE_BYTES_PER_CELL_LAYER.items()}
    b["transport"] = ncl * (TRANSPORT_BYTES_PER_CELL_LAYER_SUBCYCLE * nt + TRANSPORT_BYTES_PER_CELL_LAYER_AVERAGING)
    b["free_surface"] = ncl * FS_ASSEMBLY_BYTES_PER_CELL_LAYER + deck.n_cells * PCG_BYTES_PER_CELL_ITERATION * pcg_iters
    return b


def measured_peak() -> tuple[float, str]:
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            return float(json.loads(f.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def time_oracle(deck, st, max_steps: int, budget_s: float):
    """Steps of the OpenMP build of the CPU restatement on every host core: one untimed step,
    then timed steps until max_steps or budget_s seconds.  Returns (steps, seconds, threads)."""
    from gom_release_gb300.core import GomCore
    from gom_release_gb300.driver import Run
    if not ORACLE_OMP_SO.exists():
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    core = GomCore(deck, lib_path=ORACLE_OMP_SO)
    core.lib.gom_oracle_threads.argtypes = [ctypes.c_int32]
    threads = core.lib.gom_oracle_threads(int(os.environ.get("OMP_NUM_THREADS", host_threads())))
    run = Run(deck, core, st)
    run.advance(1)
    n = 0
    t0 = time.perf_counter()
    while n < max_steps and (n == 0 or time.perf_counter() - t0 < budget_s):
        run.advance(1)
        n += 1
    return n, time.perf_counter() - t0, threads


def cpu_baseline(deck, st, ncl: int, max_steps: int = 20, budget_s: float = 15.0) -> dict:
    n, dt, threads = time_oracle(deck, st, max_steps, budget_s)
    return {"value": ncl * n / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": (f"{n} timesteps (after 1 untimed) of the same estuary workload, FP64 CPU restatement of "
                       f"the reference built with OpenMP over {threads} host threads"),
            "seconds": dt}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local


def reduce_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_reference(args, world, rank):
    """The reference's CPU algorithm for this path on the host cores: the reference is Fortran and
    no Fortran compiler exists here, so its FP64 restatement (oracle/gom_oracle.cpp) runs, built
    with OpenMP over the same loops the reference parallelises, on every host thread."""
    if rank != 0:
        return
    from gom_release_gb300.deck import active_cell_layers, initial_state
    deck = make_deck(args.size, "fp64", args.transport_solver)
    st = initial_state(deck)
    ncl = active_cell_layers(deck, st)
    k, dt, threads = time_oracle(deck, st, max(1, args.steps), 20.0)
    value = ncl * k / dt
    sample = (f"{k} timesteps (after 1 untimed, bounded to about 20 s) of the estuary workload, FP64 CPU "
              f"restatement built with OpenMP on {threads} host threads (the reference is Fortran and no "
              "Fortran compiler exists here)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": k,
        "warmup": 1, "ms_per_step": dt / k * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"estuary {deck.n_cells} cells x {deck.n_layers} layers, {ncl} active cell-layers",
                   "sample": sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def snapshot_overlap(run, k: int, ms_plain: float, every: int = 5) -> dict:
    """The e2e loop again with the restart fields snapshotted every `every` steps
    (gom_snapshot_begin: staged on the device, transferred to pinned memory while the next
    steps run), against a synchronous read of the same fields (gom_get_field)."""
    from gom_release_gb300.output import RESTART_FIELDS, Snapshot
    core = run.core
    snap = Snapshot(core, RESTART_FIELDS)
    nbytes = sum(b.nbytes for b in snap.buffers)
    core.synchronize()
    t0 = time.perf_counter()
    for i in range(k):
        run.it += 1
        core.set_forcing(run.forcing.step(run.it))
        core.step_all()
        core.conservation()
        if i % every == every - 1:
            snap.wait()
            snap.begin()
    snap.wait()
    wall = time.perf_counter() - t0
    t1 = time.perf_counter()
    core.state(RESTART_FIELDS)
    sync_read = time.perf_counter() - t1
    snap.close()
    return {"fields": "write_restart.f90 set", "bytes": nbytes, "every_steps": every,
            "wall_ms_per_step_with_snapshots": wall / k * 1e3, "wall_ms_per_step_without": ms_plain * 1e3,
            "sync_get_field_ms": sync_read * 1e3}


def e2e_device_series(run, deck, ncl: int, k: int, torch_mod, stream, world) -> dict:
    """The e2e loop with the boundary forcing held on the device (gom_set_boundary_series of the
    deck's tide, river and boundary tracers, the same values the host forcing computes): every
    step is one gom_step_all plus the conservation read, with no forcing upload."""
    from gom_release_gb300.series import from_synthetic
    core = run.core
    bs = from_synthetic(deck)
    bs.step, bs.julian_day = run.it, run.forcing.julian_day
    core.set_boundary_series(bs)
    core.step_all()                     # captures the step graph with the series kernels
    run.it += 1
    run.forcing.step(run.it)
    core.synchronize()
    t0 = time.perf_counter()
    e0 = torch_mod.cuda.Event(enable_timing=True)
    e1 = torch_mod.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(k):
        core.step_all()
        core.conservation()
    e1.record(stream)
    e1.synchronize()
    secs = reduce_max(e0.elapsed_time(e1) / 1e3, world)
    wall = time.perf_counter() - t0
    for _ in range(k):                  # the host clock follows the device's
        run.it += 1
        run.forcing.step(run.it)
    return {"value": ncl * k * world / secs, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 16 + 20,
            "wall_s": wall, "steps": k,
            "forcing": "gom_set_boundary_series: harmonic tide, river discharge and boundary tracers on the device"}


def time_core_steps(core, k: int) -> float:
    """k steps of a context with device-side forcing, CUDA events on its stream."""
    import torch
    stream = torch.cuda.ExternalStream(core.stream_handle())
    core.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(k):
        core.step_launch()
    e1.record(stream)
    e1.synchronize()
    core.step_wait()
    return e0.elapsed_time(e1) / 1e3


def phase_times_in_place(core) -> dict:
    """One step run phase by phase (the context's own forcing kernels excluded), each phase timed
    with CUDA events on the context stream."""
    import torch
    from gom_release_gb300.core import TIME_LOOP
    stream = torch.cuda.ExternalStream(core.stream_handle())
    out = {}
    for ph in TIME_LOOP:
        core.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        core.step(ph)
        e1.record(stream)
        e1.synchronize()
        out[ph] = e0.elapsed_time(e1)
    return out


def bench_ensemble(args):
    """Storm-surge ensemble: every run packed into one mixed-precision context (one launch per
    phase for all runs, per-run PCG, device-side forcing) against the plain FP64 path serving
    the same runs one at a time on the same GPU."""
    from gom_release_gb300.core import load_core
    from gom_release_gb300.ensemble import ensemble_decks, pack
    from gom_release_gb300.serve import active_cell_layers, storm_context
    lib = load_core()
    t0 = time.perf_counter()
    decks = ensemble_decks(n_runs=args.runs, seed=7, min_cells=max(200, int(5000 * args.scale)),
                           max_cells=max(400, int(400000 * args.scale)))
    gen_s = time.perf_counter() - t0
    storms = [d.meta["storm"] for d in decks]
    pk = pack(decks)
    k = args.steps
    w = max(3, args.warmup, int(round(args.warm_hours * 3600.0 / pk.params.dt)))
    if args.profile_step:
        # for kernel profiles: warm up, autotune, then one step phase by phase inside an NVTX
        # range named prof_step (ncu --nvtx --nvtx-include "prof_step/")
        import torch
        from gom_release_gb300.core import TIME_LOOP
        core = storm_context(lib, pk, 1, storms)
        time_core_steps(core, w)
        tune = core.autotune(reps=2)
        core.synchronize()
        torch.cuda.nvtx.range_push("prof_step")
        for ph in TIME_LOOP:
            core.step(ph)
        core.synchronize()
        torch.cuda.nvtx.range_pop()
        print(json.dumps({"profile_step": "done", "cells": pk.n_cells, "warm_steps": w, "autotune": tune}))
        return
    res = {}
    with ClockSampler(0) as clocks:
        for label, prec in (("mixed_packed", 1), ("fp64_packed", 0)):
            if label == "fp64_packed" and args.skip_fp64_packed:
                continue
            core = storm_context(lib, pk, prec, storms)
            ncl = active_cell_layers(core, pk)
            nbytes = core.device_bytes()
            time_core_steps(core, w)
            tune = core.autotune(reps=2)
            time_core_steps(core, 1)
            secs = time_core_steps(core, k)
            res[label] = {"value": ncl * k / secs, "ms_per_step": secs / k * 1e3, "device_gb": nbytes / 1e9,
                          "active_cell_layers": ncl, "pcg_iters_total": core.pcg_iterations_total(),
                          "autotune": tune, "phase_ms": phase_times_in_place(core)}
            if args.day and label == "mixed_packed":
                res["mixed_packed_day"] = day = rest_of_day(core, ncl, w + 1 + k)
                if day["failure"] is not None and 0 <= day["failure"]["run"] < len(decks):
                    r = day["failure"]["run"]
                    day["failure"]["run_deck"] = {"cells": decks[r].n_cells, "layers": decks[r].meta["n_layers_run"],
                                                  "storm": dataclasses.asdict(storms[r])}
            core.close()
        # each run alone, timed over the same steps of the storm as the packed context (warm-up,
        # autotune, one step, then k timed steps)
        for label, prec in (("fp64_one_at_a_time", 0), ("mixed_one_at_a_time", 1)):
            if label == "mixed_one_at_a_time" and args.skip_mixed_alone:
                continue
            work = 0
            tsum = 0.0
            for d, s in zip(decks, storms):
                core = storm_context(lib, d, prec, [s])
                ncl = active_cell_layers(core, d)
                time_core_steps(core, w)
                core.autotune(reps=2)
                time_core_steps(core, 1)
                tsum += time_core_steps(core, k)
                work += ncl * k
                core.close()
            res[label] = {"value": work / tsum, "steps_per_run": k, "seconds": tsum}
    cells = [d.n_cells for d in decks]
    layers = [d.meta["n_layers_run"] for d in decks]
    line = {
        "metric": METRIC, "value": res["mixed_packed"]["value"], "unit": UNIT, "n_gpus": 1, "steps": k, "warmup": w,
        "ms_per_step": res["mixed_packed"]["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": (f"storm-surge ensemble: {len(decks)} runs, {sum(cells)} cells "
                                f"(log-uniform {min(cells)}-{max(cells)}), deepest water {min(layers)}-{max(layers)} "
                                f"of {pk.n_layers} shared 1 m levels, Holland vortex + M2 tide forcing on the "
                                f"device, dt={pk.params.dt:g} s"),
                   "generation_s": gen_s, "l2": "state larger than L2",
                   "timed_steps": f"{w + 2}-{w + k + 1} of the 1440-step day (spin-up ramp 6 h)"},
        "ensemble": res,
        "speedup_vs_fp64_one_at_a_time": res["mixed_packed"]["value"] / res["fp64_one_at_a_time"]["value"],
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)


def bounded_ensemble(lib, steps: int = 10, warm: int = 5) -> dict:
    """The ensemble comparison at full size for the default benchmark line: the 96 storm-surge
    runs packed into one mixed-precision context against the plain FP64 path stepping every run
    alone, each arm warmed up `warm` steps, autotuned, stepped once, then timed over `steps` steps
    with CUDA events (the same steps of the storms for both arms)."""
    from gom_release_gb300.ensemble import ensemble_decks, pack
    from gom_release_gb300.serve import active_cell_layers, storm_context
    t0 = time.perf_counter()
    decks = ensemble_decks(n_runs=96, seed=7)
    storms = [d.meta["storm"] for d in decks]
    pk = pack(decks)
    core = storm_context(lib, pk, 1, storms)
    ncl = active_cell_layers(core, pk)
    time_core_steps(core, warm)
    tune = core.autotune(reps=2)
    time_core_steps(core, 1)
    secs = time_core_steps(core, steps)
    packed = {"value": ncl * steps / secs, "ms_per_step": secs / steps * 1e3, "active_cell_layers": ncl,
              "device_gb": core.device_bytes() / 1e9, "autotune": tune, "status": int(core.status().code)}
    core.close()
    work, tsum = 0, 0.0
    for d, st in zip(decks, storms):
        c = storm_context(lib, d, 0, [st])
        n = active_cell_layers(c, d)
        time_core_steps(c, warm)
        c.autotune(reps=2)
        time_core_steps(c, 1)
        tsum += time_core_steps(c, steps)
        work += n * steps
        c.close()
    fp64 = {"value": work / tsum, "seconds": tsum}
    cells = [d.n_cells for d in decks]
    return {"workload": (f"{len(decks)} storm-surge runs, {sum(cells)} cells (log-uniform {min(cells)}-{max(cells)}), "
                         f"steps {warm + 2}-{warm + steps + 1} of the storms"),
            "packed_mixed": packed, "fp64_one_at_a_time": fp64, "ratio": packed["value"] / fp64["value"],
            "wall_s": time.perf_counter() - t0}


def serving_record(lib, n_requests: int, scale: float, horizon_scale: float, pool_size: int, servers=None):
    """Poisson stream of storm-surge requests (rate 2/s, horizons U(6, 48) h scaled by
    horizon_scale), meshes drawn from an ensemble-like pool: continuous batching in one packed
    mixed-precision context (and optionally one mixed context per run) under a 150 GB
    device-memory budget, against the plain FP64 path serving the same requests one at a time on
    the same GPU.  Returns per-server latency percentiles and throughput."""
    import dataclasses as dc
    from gom_release_gb300.ensemble import ensemble_decks
    from gom_release_gb300.serve import Request, poisson_arrivals, serve, serve_fifo, serve_packed
    servers = servers or ("packed", "contexts", "fifo")
    t0 = time.perf_counter()
    pool = ensemble_decks(n_runs=pool_size, seed=5, min_cells=max(200, int(5000 * scale)),
                          max_cells=max(400, int(400000 * scale)))
    gen_s = time.perf_counter() - t0
    arrivals = poisson_arrivals(n_requests, 2.0, seed=3)

    def make_requests():
        out = []
        r2 = np.random.default_rng(17)
        for i, t in enumerate(arrivals):
            d = pool[int(r2.integers(len(pool)))]
            st = dc.replace(d.meta["storm"], dp=float(r2.uniform(20e2, 80e2)), rmax=float(r2.uniform(20e3, 60e3)),
                            b=float(r2.uniform(1.0, 1.8)), speed=float(r2.uniform(3.0, 8.0)))
            hours = float(r2.uniform(6.0, 48.0)) * horizon_scale
            steps = max(1, int(round(hours * 3600.0 / d.params.dt)))
            out.append(Request(rid=i, deck=d, storm=st, steps=steps, arrival=float(t)))
        return out

    res = {}
    if "packed" in servers:
        res["serving_packed_mixed"] = serve_packed(lib, make_requests(), budget_bytes=150e9, precision=1)
    if "contexts" in servers:
        res["serving_contexts_mixed"] = serve(lib, make_requests(), budget_bytes=150e9, precision=1)
    if "fifo" in servers:
        res["serving_fp64_one_at_a_time"] = serve_fifo(lib, make_requests(), precision=0)
    workload = (f"serving: {n_requests} Poisson requests (rate 2/s), horizons U(6,48) h x {horizon_scale:g}, "
                f"meshes from a pool of {len(pool)} storm-surge runs "
                f"({min(d.n_cells for d in pool)}-{max(d.n_cells for d in pool)} cells), HBM budget 150 GB")
    return res, workload, gen_s


def rest_of_day(core, ncl: int, done: int, day_steps: int = 1440) -> dict:
    """Step a storm context through the rest of the 24 h day an hour (60 steps) at a time, timed
    with CUDA events, checking the status after every hour: the storms' full strength and
    landfall included."""
    hours = []
    left = day_steps - done
    secs = 0.0
    while left > 0:
        n = min(60, left)
        try:
            t = time_core_steps(core, n)
        except Exception as exc:   # a run failed: the library's error, with the status it read
            st = core.status()
            hours.append({"steps": n, "ms_per_step": float("nan"), "status": -1, "error": str(exc),
                          "failure": {k: getattr(st, k) for k, _ in st._fields_}})
            break
        st = core.status()
        hours.append({"steps": n, "ms_per_step": t / n * 1e3, "status": int(st.code)})
        secs += t
        left -= n
        if st.code:
            break
    steps = sum(h["steps"] for h in hours if h["status"] == 0)
    return {"steps": steps, "value": ncl * steps / secs if secs > 0 else 0.0, "failed": any(h["status"] for h in hours),
            "last_step": done + steps, "ms_per_step_by_hour": [round(h["ms_per_step"], 2) for h in hours],
            "failure": next((dict(h["failure"], error=h["error"]) for h in hours if "failure" in h), None),
            "pcg_iters_total": core.pcg_iterations_total()}


def bench_serving(args):
    """The serving workload alone (serving_record at the command line's sizes)."""
    from gom_release_gb300.core import load_core
    lib = load_core()
    with ClockSampler(0) as clocks:
        res, workload, gen_s = serving_record(lib, args.requests, args.scale, args.horizon_scale, args.pool)
    packed, fifo = res["serving_packed_mixed"], res["serving_fp64_one_at_a_time"]
    line = {
        "metric": METRIC, "value": packed["throughput"], "unit": UNIT, "n_gpus": 1, "steps": None, "warmup": 0,
        "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic",
        "config": {"workload": workload, "generation_s": gen_s},
        **res,
        "latency_p50_s": packed["latency_p50_s"], "latency_p99_s": packed["latency_p99_s"],
        "throughput_vs_fp64_one_at_a_time": packed["throughput"] / fifo["throughput"],
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)


def bounded_serving(lib) -> dict:
    """The serving comparison at a bounded size for the default benchmark line: 16 requests,
    quarter-scale meshes (1,250-100,000 cells), horizons 0.6-4.8 h; packed mixed precision against
    plain FP64 one request at a time, p50 / p99 latency and throughput of each."""
    t0 = time.perf_counter()
    res, workload, _ = serving_record(lib, 16, 0.25, 0.1, 12, servers=("packed", "fifo"))
    packed, fifo = res["serving_packed_mixed"], res["serving_fp64_one_at_a_time"]
    keep = ("latency_p50_s", "latency_p99_s", "latency_mean_s", "throughput", "failed", "repacks",
            "repack_s_mean", "peak_in_flight")

    def short(r):
        return {k: r[k] for k in keep if k in r}

    return {"workload": workload, "packed_mixed": short(packed), "fp64_one_at_a_time": short(fifo),
            "p50_ratio_fp64_over_packed": fifo["latency_p50_s"] / packed["latency_p50_s"],
            "p99_ratio_fp64_over_packed": fifo["latency_p99_s"] / packed["latency_p99_s"],
            "throughput_ratio": packed["throughput"] / fifo["throughput"],
            "wall_s": time.perf_counter() - t0}


def bench_precision(args):
    """The tidal-basin generator scaled up (default 2M cells x 40 layers), run in plain FP64 and
    in mixed precision from the same cold start for the same steps: per-field max and RMS error
    of the mixed run against the FP64 run (which tracks the CPU restatement to 1e-8), volume and
    salt-mass difference, and both throughputs."""
    import dataclasses as dc
    from gom_release_gb300.core import GomCore, load_core
    from gom_release_gb300.deck import HostForcing, tidal_basin
    from gom_release_gb300.serve import active_cell_layers
    lib = load_core()
    ny = int(round(math.sqrt(args.cells / 1.5)))
    nx = int(round(args.cells / ny))
    t0 = time.perf_counter()
    deck = tidal_basin(nx=nx, ny=ny, dx=250.0, n_layers=args.layers, dt=60.0)
    gen_s = time.perf_counter() - t0
    out = {}
    fields = ("eta_cell", "un_face", "vn_face", "wn_cell", "u_node", "w_node", "salt_cell", "temp_cell", "dz_cell")
    snaps = {}
    for label, prec in (("fp64", 0), ("mixed", 1)):
        d = dc.replace(deck, params=dc.replace(deck.params, precision=prec))
        core = GomCore(d, lib=lib)
        p = d.params
        core.cold_start(p.ref_salt, p.ref_temp, p.av_0, p.kv_0)
        core.step("density")
        ncl = active_cell_layers(core, d)
        hf = HostForcing(d)
        v0, s0 = core.conservation()
        secs = 0.0
        import torch
        stream = torch.cuda.ExternalStream(core.stream_handle())
        for it in range(1, args.steps + 1):
            core.set_forcing(hf.step(it))
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            core.step_launch()
            e1.record(stream)
            core.step_wait()
            if it > 3:
                secs += e0.elapsed_time(e1) / 1e3
        v1, s1 = core.conservation()
        snaps[label] = {f: core.get_field(f) for f in fields}
        out[label] = {"value": ncl * (args.steps - 3) / secs, "ms_per_step": secs / (args.steps - 3) * 1e3,
                      "device_gb": core.device_bytes() / 1e9, "active_cell_layers": ncl, "volume": v1,
                      "salt_mass": s1, "volume_change_rel": (v1 - v0) / v0, "pcg_iters_total": core.pcg_iterations_total()}
        core.close()
    err = {}
    for f in fields:
        a, b = snaps["mixed"][f], snaps["fp64"][f]
        scale = max(float(np.abs(b).max()), 1e-30)
        err[f] = {"max_abs": float(np.abs(a - b).max()), "rms_abs": float(np.sqrt(np.mean((a - b) ** 2))),
                  "max_rel_to_field_max": float(np.abs(a - b).max()) / scale}
    line = {
        "metric": METRIC, "value": out["mixed"]["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps - 3,
        "warmup": 3, "ms_per_step": out["mixed"]["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": (f"precision: tidal basin {deck.n_cells} cells x {deck.n_layers} layers, "
                                f"dt=60 s, {args.steps} steps from a cold start, FP64 vs mixed"), "generation_s": gen_s},
        "precision": out, "mixed_vs_fp64_error": err,
        "volume_diff_rel": abs(out["mixed"]["volume"] - out["fp64"]["volume"]) / out["fp64"]["volume"],
        "salt_mass_diff_rel": abs(out["mixed"]["salt_mass"] - out["fp64"]["salt_mass"]) / out["fp64"]["salt_mass"],
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", default="full", choices=["full", "medium", "small"],
                    help="full: the benchmark workload; medium (38k cells) and small (6k cells) for profiling")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true",
                    help="estuary: skip the bounded serving record (packed mixed vs FP64 latency) of the line")
    ap.add_argument("--no-ensemble", action="store_true",
                    help="estuary: skip the ensemble record (96 runs packed mixed vs FP64 one at a time) of the line")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--tuning", default=None,
                    help="launch variants per tunable site, e.g. 1,3,3,1 (set instead of autotuning)")
    ap.add_argument("--no-phases", action="store_true", help="skip the per-phase timing pass")
    ap.add_argument("--e2e-steps", type=int, default=0)
    ap.add_argument("--workload", default="estuary", choices=["estuary", "ensemble", "serving", "precision"],
                    help="estuary: the single-run benchmark; ensemble: packed storm-surge ensemble; "
                         "serving: Poisson request stream with continuous batching")
    ap.add_argument("--requests", type=int, default=48, help="serving: number of requests")
    ap.add_argument("--cells", type=int, default=2_000_000, help="precision: cell count")
    ap.add_argument("--layers", type=int, default=40, help="precision: z-layers")
    ap.add_argument("--pool", type=int, default=16, help="serving: distinct meshes")
    ap.add_argument("--horizon-scale", type=float, default=1.0, help="serving: scale of the 6-48 h horizons")
    ap.add_argument("--runs", type=int, default=96, help="ensemble: number of runs")
    ap.add_argument("--scale", type=float, default=1.0, help="ensemble: cell-count scale (1 = 5k-400k)")
    ap.add_argument("--skip-fp64-packed", action="store_true")
    ap.add_argument("--warm-hours", type=float, default=0.0,
                    help="ensemble: simulated hours stepped before timing (the storms ramp up over 6 h)")
    ap.add_argument("--skip-mixed-alone", action="store_true", help="ensemble: skip the mixed one-at-a-time arm")
    ap.add_argument("--day", action="store_true",
                    help="ensemble: after its timed window, step the packed mixed context through the rest of the "
                         "24 h day and report its throughput and status hour by hour")
    ap.add_argument("--profile-step", action="store_true",
                    help="ensemble: warm up, autotune and run one packed step phase by phase in an NVTX range "
                         "prof_step (for ncu), then exit")
    ap.add_argument("--transport-solver", type=int, default=1, choices=[1, 2],
                    help="estuary: 1 TVD transport (the configuration), 2 ELM transport (transport_solver 2)")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"],
                    help="fp64: the drop-in path (bit-for-bit with the CPU restatement); mixed: FP32 layered state")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.workload == "ensemble":
        if rank == 0:
            bench_ensemble(args)
        return
    if args.workload == "serving":
        if rank == 0:
            bench_serving(args)
        return
    if args.workload == "precision":
        if rank == 0:
            bench_precision(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    import torch
    from gom_release_gb300.core import GomCore, load_core
    from gom_release_gb300.deck import HostForcing, active_cell_layers, initial_state
    from gom_release_gb300.driver import Run

    deck = make_deck(args.size, args.precision, args.transport_solver)
    st = initial_state(deck)
    ncl = active_cell_layers(deck, st)
    lib = load_core()
    run = Run(deck, GomCore(deck, lib=lib), st)
    torch_mod, stream = stream_events(run.core)
    run.advance(args.warmup)
    if args.tuning:
        tune = [int(v) for v in args.tuning.split(",")]
        run.core.set_tuning(tune)
    else:
        tune = run.core.autotune(reps=3) if not args.no_autotune else None
    # ---- value: K steps, state resident in HBM, host forcing precomputed
    hf = HostForcing(deck)
    hf.julian_day = run.forcing.julian_day
    hf.first = False
    forcings = [hf.step(run.it + 1 + i) for i in range(args.steps)]
    barrier(world)
    with ClockSampler(local) as clocks:
        secs = time_steps(run, forcings, torch_mod, stream)
    run.it += args.steps
    run.forcing = hf
    secs = reduce_max(secs, world)
    pcg_total = run.core.pcg_iterations_total()
    # ---- e2e: the public API with host buffers, forcing computed and result read every step
    ke = args.e2e_steps or max(10, args.steps // 4)
    run.core.synchronize()
    t0 = time.perf_counter()
    e0 = torch_mod.cuda.Event(enable_timing=True)
    e1 = torch_mod.cuda.Event(enable_timing=True)
    e0.record(stream)
    h2d = 0
    for _ in range(ke):
        run.it += 1
        f = run.forcing.step(run.it)
        h2d = sum(np.asarray(v).nbytes for v in f.values() if isinstance(v, np.ndarray)) + 32
        run.core.set_forcing(f)
        run.core.step_all()
        run.core.conservation()
    e1.record(stream)
    e1.synchronize()
    e2e_secs = reduce_max(e0.elapsed_time(e1) / 1e3, world)
    wall_e2e = time.perf_counter() - t0
    snapshot = snapshot_overlap(run, ke, wall_e2e / ke)
    e2e_series = e2e_device_series(run, deck, ncl, ke, torch_mod, stream, world)
    # ---- per-phase timing for the roofline
    snap = run.core.state()
    f = dict(run.forcing.step(run.it + 1))
    f.update(wind_stress_normal=run.forcing.wind_normal, wind_stress_tangnt=run.forcing.wind_tangnt,
             gamma_t=run.forcing.gamma_t)
    pcg_mean = (pcg_total / max(1, args.warmup + args.steps))
    peak, peak_kind = measured_peak()
    # dominant kernel: the transport column solve (one launch per subcycle), timed alone; with the
    # ELM transport (no TVD solve) the ELM walk of the advection instead
    tvd = deck.params.transport_solver != 2
    if tvd:
        solve_ms = run.core.profile_kernel(run.core.KERNEL_TRANSPORT_SOLVE, reps=5)
        solve_bytes = TR_SOLVE_BYTES_PER_CELL_LAYER[args.precision] * ncl
        # FP64 solve variant 3 runs the solve as two kernels (rows per wet cell-layer, column Thomas)
        list_solve = args.precision == "fp64" and tune is not None and tune[2] == 3
        solve_kernel = "k_tr_rows64_sorted + k_tr_thomas_col" if list_solve else "k_tr_solve"
        traffic = solve_traffic(solve_kernel, args.precision, ncl)
        kernel_label = f"transport solve, one subcycle ({solve_kernel})"
    else:
        solve_ms = run.core.profile_kernel(run.core.KERNEL_ELM_WALK, reps=5)
        solve_bytes = PHASE_BYTES_PER_CELL_LAYER["advection"] * ncl
        solve_kernel, traffic, kernel_label = "ELM walk", None, "ELM walk of the advection (k_elm_faces / k_elm_list)"
    achieved = solve_bytes / (solve_ms * 1e-3) / 1e9
    # FP64 roofline of the same launch: FP64 instructions per second against the measured issue
    # peak (the library's FMA-chain kernel; an FMA is one instruction and two flops)
    roof_fp64 = None
    if args.precision == "fp64" and tvd:
        from gom_release_gb300.core import measure_fp64_peak
        peak_gflops = measure_fp64_peak(lib)
        instr = SOLVE_FP64_INSTR_PER_CELL_LAYER[solve_kernel] * ncl
        ach = instr / (solve_ms * 1e-3) / 1e9
        roof_fp64 = {"bound": "fp64", "kernel": solve_kernel, "achieved": ach, "peak": peak_gflops / 2.0,
                     "unit": "G FP64 instructions/s", "frac": ach / (peak_gflops / 2.0),
                     "instructions_per_cell_layer": SOLVE_FP64_INSTR_PER_CELL_LAYER[solve_kernel],
                     "peak_fma_gflops": peak_gflops,
                     "peak_source": "measured: gom_measure_fp64_peak (independent FMA chains, CUDA events)"}
        warp = SOLVE_FP64_WARP_INSTR_PER_CELL_LAYER.get(solve_kernel)
        if warp is not None:
            # the pipe's issue rate: warp instructions against the measured warp-instruction rate
            # (all lanes active, and one lane per warp active for the cost of a divergent warp)
            from gom_release_gb300.core import measure_fp64_issue
            wpeak = measure_fp64_issue(lib, 32) / 1e9
            wone = measure_fp64_issue(lib, 1) / 1e9
            wach = warp * ncl / (solve_ms * 1e-3) / 1e9
            roof_fp64["warp_issue"] = {"achieved": wach, "peak": wpeak, "peak_one_lane": wone,
                                       "unit": "G FP64 warp instructions/s", "frac": wach / wpeak,
                                       "warp_instructions_per_cell_layer": warp,
                                       "peak_source": "measured: gom_measure_fp64_issue (FMA chains, 32 and 1 "
                                                      "active lanes per warp, CUDA events)"}
    if args.no_phases:
        phases = {}
    else:
        phases = time_phases(deck, snap, lib, f, torch_mod)
    if rank != 0:
        barrier(world)
        return
    value = ncl * args.steps * world / secs
    # the single-GPU comparisons of the serving form (run once, at N = 1, on the full workload)
    serving = ensemble = None
    if not args.no_serving and args.size == "full" and world == 1:
        serving = bounded_serving(lib)
    if not args.no_ensemble and args.size == "full" and world == 1:
        ensemble = bounded_ensemble(lib)
    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_baseline(deck, st, ncl)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic",
        "config": {
            "precision": args.precision,
            "workload": (f"estuary: {deck.n_cells} cells ({deck.meta['nx']}x{deck.meta['ny']} squares of "
                         f"{deck.meta['dx']:g} m + {deck.meta['tri_rows']}-row triangle strip), {deck.n_faces} faces, "
                         f"{deck.n_nodes} nodes, {deck.n_layers} layers, {ncl} active cell-layers, dt={deck.params.dt:g} s, "
                         + (f"TVD limiter, {deck.params.trans_sub_iter} transport subcycles, "
                            if deck.params.transport_solver != 2 else "ELM transport (transport_solver 2), ") +
                         f"baroclinic, "
                         f"turbulence closure {deck.params.turbulence_flag}"),
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
            "l2": "state larger than L2 (each phase streams its arrays from HBM)",
            "simulated_hours_per_wall_s": deck.params.dt * args.steps / secs / 3600.0,
            "autotune": tune,
            "pcg_iters_mean": pcg_mean,
        },
        "roofline": {"bound": "hbm", "kernel": kernel_label,
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": traffic, "algorithmic_bytes": solve_bytes,
                     "ms_per_launch": solve_ms,
                     "phase_ms": {k: v * 1e3 for k, v in phases.items()},
                     "phase_algorithmic_gbs": {k: phase_bytes(deck, ncl, pcg_mean).get(k, 0) / v / 1e9
                                               for k, v in phases.items() if v > 0}},
        "roofline_fp64": roof_fp64,
        "cpu_baseline": cpu,
        "e2e": {"value": ncl * ke * world / e2e_secs, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": 16 + 20, "wall_s": wall_e2e},
        "gpu_launches": kernel_launches_per_step(deck) * args.steps,
        "clocks": clocks.summary(),
        "snapshot": snapshot,
        "serving": serving,
        "ensemble": ensemble,
        "e2e_device_series": e2e_series,
    }
    print(json.dumps(line), flush=True)
    barrier(world)


if __name__ == "__main__":
    main()
