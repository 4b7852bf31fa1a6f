"""Benchmark: D3Q27 cumulant step throughput (MLUPS) and its HBM roofline.

Workload: the uniform lattice-Mach-0.1 NACA0012 case (384 x 256 x 8 cells, 12 x 8
chords, leading edge at (128, 128), chord 32 cells, AoA 4 deg, Re 30000,
characteristic farfield on all x/y faces, seeded 1e-4 perturbation, z periodic).
The reference's own minimum span is 8 cells, used here so the same case runs
in both arms.  Inputs are larger than L2 for the FP64 form (2 x 185 MB of
populations); the reduced-storage forms are timed step by step with an L2
flush (a 512 MB device write) between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One JSON line on rank 0.  Under torchrun each rank advances its own replica of
the case (independent cases do not exchange data), timed between barriers; the
slowest rank's time is used.
"""
import argparse
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

METRIC = "D3Q27 MLUPS & %HBM peak"
CELLS_PER_CHORD = 32
WORKLOAD = "uniform NACA0012 384x256x8, chord 32, AoA 4, Re 3e4, Ma 0.1, characteristic farfield"
BYTES_PER_CELL = {"f64": 27 * 2 * 8, "f32": 27 * 2 * 4, "f16": 27 * 2 * 2}


def case_parts():
    from aerokinetic_gb300 import Flow, Grid, Section, naca0012
    section = Section((naca0012(),))
    flow = Flow(reynolds=30000, alpha_deg=4, lattice_speed=0.1 / math.sqrt(3))
    grid = Grid(cells_per_chord=CELLS_PER_CHORD, upstream_chords=4.0, downstream_chords=6.9867,
                transverse_chords=3.9266, span_chords=0.125, farfield="characteristic_transport_v1",
                memory_limit_gib=64)
    return section, flow, grid


def peaks():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        data = json.loads(path.read_text())
        return float(data["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.reader = threading.Thread(target=self._read, daemon=True)
            self.reader.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def oracle_case(threads):
    from aerokinetic_gb300 import Plan
    from oracle import oracle as O
    section, flow, grid = case_parts()
    plan = Plan.create(section, flow, grid)
    lead = O.leading_edge([e.xy for e in section.elements], section.moment_reference, section.chord,
                          flow.alpha_deg)
    case = O.AirfoilCase([c.xy for c in section.normalized(flow.alpha_deg)], plan.shape, plan.origin, plan.dx,
                         plan.span, plan.relaxation_rate, flow.lattice_speed, grid.cells_per_chord, grid.farfield,
                         flow.perturbation, flow.seed, lead, threads)
    return plan, case


def oracle_run(case, steps, budget_s):
    """Up to `steps` oracle steps (loads every 8), stopping after budget_s."""
    done, start = 0, time.perf_counter()
    while done < steps:
        done += 1
        case.step(sample=done % 8 == 0)
        if time.perf_counter() - start >= budget_s:
            break
    return done, time.perf_counter() - start


def oracle_sample(budget_s=15.0):
    """The CPU oracle (C restatement, FP64, OpenMP on all host cores) on the
    same case for a bounded sample of steps; returns MLUPS and the sample."""
    cores = cpu_cores()
    plan, case = oracle_case(cores)
    case.step(sample=True)  # boundary set-up outside the timing
    steps, elapsed = oracle_run(case, 10**9, budget_s)
    cells = math.prod(plan.shape)
    return {"value": cells * steps / elapsed / 1e6, "unit": "MLUPS", "cores": cores, "kind": "port",
            "sample": f"{steps} steps of the same {plan.shape} case on {cores} host threads "
                      f"(FP64 oracle, loads every 8 steps), {elapsed:.1f} s"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    cores = cpu_cores()
    plan, case = oracle_case(cores)
    oracle_run(case, args.warmup, 20.0)
    steps, elapsed = oracle_run(case, args.steps, 120.0)
    cells = math.prod(plan.shape)
    value = cells * steps / elapsed / 1e6
    sample = (f"{steps} of {args.steps} requested steps of the {plan.shape} case on {cores} host threads "
              f"(FP64 oracle, loads every 8 steps), {elapsed:.1f} s, capped at 120 s")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "MLUPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed * 1e3 / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "engine": "CPU oracle (C restatement of the reference step)",
                       "l2": "host run"},
            "cpu_baseline": {"value": value, "unit": "MLUPS", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "reference_as_published": {"value": 20.0, "unit": "MLUPS",
                                       "note": "lbmpy 1.4 CPU, 1 thread, 176x101x16 (profile_threads1.json)"}}
    print(json.dumps(line), flush=True)


def flush_l2(buf, stream):
    import torch
    with torch.cuda.stream(stream):
        buf.add_(1)


def measure_form(storage, steps, warmup, flush):
    """Per-step timing of the stream-collide kernel of one storage form."""
    import torch
    from aerokinetic_gb300.solver import Solver
    section, flow, grid = case_parts()
    solver = Solver(section, flow, grid, storage=storage)
    lib = solver._lib
    stream = torch.cuda.ExternalStream(lib.ak_case_stream(solver._case))
    buf = torch.zeros(128 * 2**20, dtype=torch.float32, device="cuda")
    ms = np.zeros(4)
    lib.ak_step_timed(solver._case, max(1, warmup), ms.ctypes.data_as(ctypes.c_void_p))
    bulk = total = 0.0
    for _ in range(steps):
        if flush:
            flush_l2(buf, stream)
        ms[:] = 0
        code = lib.ak_step_timed(solver._case, 1, ms.ctypes.data_as(ctypes.c_void_p))
        if code:
            raise RuntimeError(lib.ak_last_error())
        total += ms[0]
        bulk += ms[1]
    info = solver.info
    solver.close()
    return {"cells": info["cells"], "fluid_cells": info["fluid_cells"], "bulk_ms": bulk / steps,
            "step_ms": total / steps}


def run_engine(args, rank, world, local_rank):
    import torch
    from aerokinetic_gb300 import _native
    from aerokinetic_gb300.solver import Solver
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
    lib = _native.load()
    section, flow, grid = case_parts()

    # ---- headline: plain FP64 form, K steps in the timed region
    solver = Solver(section, flow, grid, storage="f64")
    case = solver._case
    ms = np.zeros(4)
    ptr = ms.ctypes.data_as(ctypes.c_void_p)
    _native.check(lib.ak_step_timed(case, max(3, args.warmup), ptr))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches0 = lib.ak_kernel_launches(case)
    with ClockSampler(local_rank) as clocks:
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        ms[:] = 0
        _native.check(lib.ak_step_timed(case, args.steps, ptr))
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    launches = lib.ak_kernel_launches(case) - launches0
    elapsed_ms = float(ms[0])
    bulk_ms = float(ms[1]) / args.steps
    if dist:
        t = torch.tensor([elapsed_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms = float(t.item())
    info = solver.info
    cells = info["cells"]
    value = world * cells * args.steps / (elapsed_ms / 1e3) / 1e6
    solver.close()
    if rank != 0:
        return

    # ---- end to end through the public API: case set-up from the host
    # description, the reference's compute loop (loads every 8 steps plus
    # diagnostics), results back on the host
    e2e_steps = max(64, min(args.steps, 2000))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s = Solver(section, flow, grid, storage="f64")
    samples = 0
    for i in range(e2e_steps // 8):
        s.advance(8, sample_last=True)
        s.diagnostics()
        samples += 1
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    s.close()
    h2d = 8 * sum(len(c.xy) * 2 for c in section.normalized(flow.alpha_deg)) + 128
    d2h = samples * (5 * 8 + 5 * 8)

    # ---- the reduced-storage forms, step by step with an L2 flush
    forms = {}
    hbm, peak_kind = peaks()
    for storage in ("f64", "f32", "f16"):
        m = measure_form(storage, steps=min(args.steps, 100), warmup=args.warmup, flush=True)
        bytes_launch = m["fluid_cells"] * BYTES_PER_CELL[storage]
        achieved = bytes_launch / (m["bulk_ms"] / 1e3) / 1e9
        forms[storage] = {"mlups": m["cells"] / (m["step_ms"] / 1e3) / 1e6,
                          "kernel_mlups": m["cells"] / (m["bulk_ms"] / 1e3) / 1e6,
                          "bulk_kernel_ms": m["bulk_ms"], "achieved_gbs": achieved,
                          "frac_of_" + peak_kind: achieved / hbm, "bytes_per_cell": BYTES_PER_CELL[storage]}

    bytes_launch = info["fluid_cells"] * BYTES_PER_CELL["f64"]
    achieved = bytes_launch / (bulk_ms / 1e3) / 1e9
    traffic = None
    summary = ROOT / "profiles" / "stream_collide_f64_uniform_384x256x8.txt"
    if summary.exists():
        for line in summary.read_text().splitlines():
            if line.startswith("dram_bytes_per_launch:"):
                traffic = float(line.split(":", 1)[1].split()[0])
    cpu = oracle_sample(budget_s=15.0)
    line = {"metric": METRIC, "value": value, "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cells": cells, "fluid_cells": info["fluid_cells"],
                       "storage": "f64 populations, two copies (pull A->B)",
                       "l2": "inputs larger than L2 (2 x 185 MB); reduced forms flushed between steps",
                       "parallelism": f"replicas x{world}"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": traffic, "peak_source": peak_kind,
                         "kernel": "k_stream_collide<double>", "bytes_per_launch": bytes_launch,
                         "kernel_ms": bulk_ms},
            "forms": forms,
            "cpu_baseline": cpu,
            "e2e": {"value": cells * e2e_steps / e2e_s / 1e6, "unit": "MLUPS", "steps": e2e_steps,
                    "h2d_bytes_per_step": h2d / e2e_steps, "d2h_bytes_per_step": d2h / e2e_steps,
                    "includes": "case set-up from host description, loads + diagnostics every 8 steps"},
            "gpu_launches": int(launches),
            "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def main():
    parser = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    parser.add_argument("--gpus", type=int, default=1)
    parser.add_argument("--steps", type=int, default=2000)
    parser.add_argument("--warmup", type=int, default=20)
    parser.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    args = parser.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", args.gpus if "RANK" in os.environ else 1))
    local_rank = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    run_engine(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
