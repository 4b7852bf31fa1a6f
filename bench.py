"""Benchmark: D3Q27 cumulant step throughput (MLUPS) and its HBM roofline.

Headline workload (the two-level case): NACA0012 at AoA 8 deg, Re 30000,
lattice Mach 0.1; coarse level 512 x 384 x 8 cells (16 x 12 chords, chord 32
coarse cells), fine level at twice the resolution (chord 64) over
x in [-0.5c, 2c], y in [-0.6c, 0.6c] around the section: 160 x 76 x 16 fine
cells.  Legacy outer boundary (the reference's refined solver accepts no
other), FP64 (the reference's dtype).  MLUPS counts coarse cells + 2 x fine
cells per coarse step, as the reference does for two-level runs.  Inputs are
larger than L2 (2 x 340 MB of coarse populations).

Also reported: the reduced-precision forms (FP32 arithmetic with FP32 or FP16
shifted storage) of the same case, and the uniform 384 x 256 x 8 case with the
characteristic farfield (the reference's CPU-runnable configuration).

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
WORKLOAD = ("two-level NACA0012, coarse 512x384x8 (chord 32) + fine 160x76x16 (chord 64) over "
            "x in [-0.5c, 2c], y in [-0.6c, 0.6c], AoA 8, Re 3e4, Ma 0.1, legacy farfield")
UNIFORM = "uniform NACA0012 384x256x8, chord 32, AoA 4, Re 3e4, Ma 0.1, characteristic farfield"
BYTES_PER_CELL = {"f64": 27 * 2 * 8, "f32": 27 * 2 * 4, "f16": 27 * 2 * 2, "df64": 27 * 2 * 8}
# coarse steps after which the reduced forms' coefficients are compared with
# the FP64 form's (the start-up transient is over by then at chord 32)
FORM_ERROR_STEPS = 2000
# coarse steps of the end-to-end solve (set-up from the host description
# included; the benchmark case itself is a 10000-step run)
E2E_STEPS = 1000
# DRAM bytes (read + write) of the coarse k_stream_collide<double> over one
# coarse step of the two-level case, from the ncu capture summarised in
# profiles/stream_collide_f64_refined_512x384x8.txt: the graphed step runs it
# as a far launch (347383040 + 284257536 B) and a near launch (8960512 +
# 8704 B); the eager step that kernel_ms times covers the same cells in one
# launch.  The algorithmic figure is 1572864 cells x 432 B = 679477248 B.
TRAFFIC_BYTES_PER_LAUNCH = 347383040 + 284257536 + 8960512 + 8704


def case_parts(farfield="characteristic_transport_v1", sgs="none"):
    from aerokinetic_gb300 import Flow, Grid, Section, naca0012
    section = Section((naca0012(),))
    flow = Flow(reynolds=30000, alpha_deg=4, lattice_speed=0.1 / math.sqrt(3), sgs=sgs)
    grid = Grid(cells_per_chord=CELLS_PER_CHORD, upstream_chords=4.0, downstream_chords=6.9867,
                transverse_chords=3.9266, span_chords=0.125, farfield=farfield, memory_limit_gib=64)
    return section, flow, grid


def refined_parts():
    from aerokinetic_gb300 import Flow, Grid, Project, Section, naca0012
    from aerokinetic_gb300.refined_plan import RefinementSettings
    section = Section((naca0012(),))
    flow = Flow(reynolds=30000, alpha_deg=8, lattice_speed=0.1 / math.sqrt(3))
    grid = Grid(cells_per_chord=CELLS_PER_CHORD, upstream_chords=5.0, downstream_chords=9.9938,
                transverse_chords=5.9056, span_chords=0.25, memory_limit_gib=64)
    refinement = RefinementSettings(upstream_chords=0.5, downstream_chords=1.0, transverse_chords=0.5)
    return Project(section, flow, grid), refinement


def fine_passes(fine_storage):
    """Passes over the fine block per coarse step, each reading and writing
    every cell once: the first fine step's collision, its streaming fused
    with the second step's collision, the second step's streaming (the band's
    own collision in the second step is not counted)."""
    return 3


def refined_cells(plan):
    fine = math.prod(2 * n for n in plan.box.shape)
    return math.prod(plan.shape) + 2 * fine


def fma_peak(lib, precision):
    """Measured FMA throughput of the device, TFLOP/s (0 FP64, 1 FP32)."""
    from aerokinetic_gb300 import _native
    out = ctypes.c_double()
    _native.check(lib.ak_fma_peak(precision, ctypes.byref(out)))
    return out.value


def collision_flops(lib, storage):
    """Algorithmic FLOPs of one cell's collision in the storage form's arithmetic."""
    from aerokinetic_gb300 import _native
    counts = np.zeros(4)
    _native.check(lib.ak_collision_flops(_native.STORAGE[storage], counts.ctypes.data_as(ctypes.c_void_p)))
    return float(counts[3])


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


def oracle_uniform(threads):
    from aerokinetic_gb300 import Plan
    from oracle import oracle as O
    section, flow, grid = case_parts()
    plan = Plan.create(section, flow, grid)
    lead = O.leading_edge([e.xy for e in section.elements], section.moment_reference, section.chord,
                          flow.alpha_deg)
    case = O.AirfoilCase([c.xy for c in section.normalized(flow.alpha_deg)], plan.shape, plan.origin, plan.dx,
                         plan.span, plan.relaxation_rate, flow.lattice_speed, grid.cells_per_chord, grid.farfield,
                         flow.perturbation, flow.seed, lead, threads)
    return math.prod(plan.shape), case


def oracle_refined(threads):
    from aerokinetic_gb300.refined_plan import RefinedPlan
    from oracle import oracle as O
    from oracle.refined import RefinedCase
    project, refinement = refined_parts()
    plan = RefinedPlan.create(project, refinement)
    sec, flow = project.section, project.flow
    lead = O.leading_edge([e.xy for e in sec.elements], sec.moment_reference, sec.chord, flow.alpha_deg)
    case = RefinedCase([c.xy for c in sec.normalized(flow.alpha_deg)], plan.shape, plan.origin,
                       plan.coarse_level.dx, plan.coarse_level.dt, plan.coarse_level.tau_shear,
                       plan.coarse_level.tau_bulk, plan.box.lower, plan.box.upper, flow.lattice_speed,
                       flow.perturbation, flow.seed, lead, plan.span, threads)
    return refined_cells(plan), case


def oracle_run(case, steps, budget_s):
    """Up to `steps` oracle steps, stopping after budget_s; a two-level step
    closes its mass and momentum budget as the reference's step does."""
    step = getattr(case, "step_with_budget", case.step)
    done, start = 0, time.perf_counter()
    while done < steps:
        done += 1
        step()
        if time.perf_counter() - start >= budget_s:
            break
    return done, time.perf_counter() - start


def oracle_sample(budget_s=15.0, refined=True):
    """The CPU oracle (C restatement + numpy, FP64, OpenMP on all host cores)
    on the same case for a bounded sample of steps; returns MLUPS and the sample."""
    cores = cpu_cores()
    cells, case = (oracle_refined if refined else oracle_uniform)(cores)
    case.step()  # first-step set-up outside the timing
    steps, elapsed = oracle_run(case, 10**9, budget_s)
    what = "two-level" if refined else "uniform"
    return {"value": cells * steps / elapsed / 1e6, "unit": "MLUPS", "cores": cores, "kind": "port",
            "sample": f"{steps} steps of the same {what} case (budget closed every step) on {cores} host threads "
                      f"(FP64 oracle), {elapsed:.1f} s"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    cores = cpu_cores()
    cells, case = oracle_refined(cores)
    oracle_run(case, args.warmup, 30.0)
    steps, elapsed = oracle_run(case, args.steps, 120.0)
    value = cells * steps / elapsed / 1e6
    sample = (f"{steps} of {args.steps} requested coarse steps of the two-level case, each closing its mass and "
              f"momentum budget, on {cores} host threads (FP64 oracle), {elapsed:.1f} s, capped at 120 s")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "MLUPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed * 1e3 / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "engine": "CPU oracle (restatement of the reference step)",
                       "step": "loads and the mass/momentum budget every coarse step (the reference's step)",
                       "l2": "host run"},
            "cpu_baseline": {"value": value, "unit": "MLUPS", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "reference_as_published": {"value": 0.53, "unit": "MLUPS",
                                       "note": "lbmpy 1.4 CPU two-level step, 1 thread, coarse 128x69x16 + "
                                               "fine 136x58x32 (BENCHMARK_CPU_CHECK.json)"}}
    print(json.dumps(line), flush=True)


def reduce_max(value, dist):
    """The largest of every rank's value (the slowest replica's time): on the
    GPU for NCCL, on the host for gloo."""
    import torch
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_mlups(cells, steps, elapsed_ms, world):
    """Whole-job MLUPS of `world` replicas that each advanced `cells` cell
    updates per step for `steps` steps in `elapsed_ms` (the slowest rank's)."""
    return world * cells * steps / (elapsed_ms / 1e3) / 1e6


def flush_l2(buf, stream):
    import torch
    with torch.cuda.stream(stream):
        buf.add_(1)


def measure_form(storage, steps, warmup, flush, farfield="characteristic_transport_v1", sgs="none",
                 measure_static=False):
    """Per-step timing of the uniform case's stream-collide kernel in one storage form."""
    import torch
    from aerokinetic_gb300.solver import Solver
    section, flow, grid = case_parts(farfield, sgs)
    solver = Solver(section, flow, grid, storage=storage)
    lib = solver._lib
    stream = torch.cuda.ExternalStream(lib.ak_case_stream(solver._case))
    buf = torch.zeros(128 * 2**20, dtype=torch.float32, device="cuda")
    ms = np.zeros(4)
    lib.ak_step_timed(solver._case, max(1, warmup), ms.ctypes.data_as(ctypes.c_void_p))
    bulk = total = outer = 0.0
    for _ in range(steps):
        if flush:
            flush_l2(buf, stream)
        ms[:] = 0
        code = lib.ak_step_timed(solver._case, 1, ms.ctypes.data_as(ctypes.c_void_p))
        if code:
            raise RuntimeError(lib.ak_last_error())
        total += ms[0]
        bulk += ms[1]
        outer += ms[3]
    # the step as Solver.advance runs it (ak_step: graph replay where the
    # outer boundary allows), L2 flushed before each step
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    graph = 0.0
    lib.ak_step(solver._case, 2, None)
    for _ in range(steps):
        if flush:
            flush_l2(buf, stream)
        start.record(stream)
        code = lib.ak_step(solver._case, 1, None)
        end.record(stream)
        end.synchronize()
        if code:
            raise RuntimeError(lib.ak_last_error())
        graph += start.elapsed_time(end)
    info = solver.info
    out = {"cells": info["cells"], "fluid_cells": info["fluid_cells"], "bulk_ms": bulk / steps,
           "eager_step_ms": total / steps, "step_ms": graph / steps, "outer_ms": outer / steps}
    if measure_static:
        # a sampled step through ak_step (graph replay, lazily allocated
        # partial sums) and through ak_step_loads_static (eager, static scratch)
        loads = np.zeros((len(solver.contours), 5))
        ptr = loads.ctypes.data_as(ctypes.c_void_p)
        handle = lib.ak_case_stream(solver._case)
        k = max(5, min(steps, 20))
        out["sampled_step_ms"] = sum(stream_ms(lib, handle, lambda: lib.ak_step(solver._case, 1, ptr))
                                     for _ in range(k)) / k
        out["static_loads_step_ms"] = sum(
            stream_ms(lib, handle, lambda: lib.ak_step_loads_static(solver._case, 1, ptr)) for _ in range(k)) / k
    solver.close()
    return out


def measure_form_at(cells_per_chord, storage, **kw):
    """measure_form on the uniform case at another resolution."""
    global CELLS_PER_CHORD
    keep, CELLS_PER_CHORD = CELLS_PER_CHORD, cells_per_chord
    try:
        return measure_form(storage, **kw)
    finally:
        CELLS_PER_CHORD = keep


def batch_case_parts(i, base_seed=2026):
    """Case i of the polar-sweep batch: chord cells from {24, 32, 48, 64}, a
    12c x 8c domain with a periodic span of 4 cells (the plan's minimum of 8),
    AoA U[-4, 16] deg, Re log-uniform on [1e4, 1e5], drawn from
    default_rng(base_seed + i); the perturbation phase from the case's seed."""
    from aerokinetic_gb300 import Flow, Grid, Section, naca0012
    rng = np.random.default_rng(base_seed + i)
    chord = int(rng.choice([24, 32, 48, 64]))
    flow = Flow(reynolds=float(10 ** rng.uniform(4, 5)), alpha_deg=float(rng.uniform(-4, 16)),
                lattice_speed=0.1 / math.sqrt(3), seed=base_seed + i)
    grid = Grid(cells_per_chord=chord, upstream_chords=4.0, downstream_chords=7.0, transverse_chords=3.9,
                span_chords=4 / chord, farfield="characteristic_transport_v1", memory_limit_gib=64)
    return Section((naca0012(81),)), flow, grid


def stream_ms(lib, stream_handle, fn):
    """Milliseconds of fn() measured by CUDA events on the given stream."""
    import torch
    stream = torch.cuda.ExternalStream(stream_handle)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    fn()
    b.record(stream)
    torch.cuda.synchronize()
    return float(a.elapsed_time(b))


# the reduced forms of the two-level case compared with the FP64 form:
# (label, coarse storage, fine storage)
REFINED_FORMS = (("df64", "df64", "df64"), ("f32", "f32", "f32"), ("f16", "f16", "f32"), ("f16_all", "f16", "f16"))


def form_errors(project, refinement, steps=2000, every=10, early=400):
    """The two-level case's reduced forms against the FP64 form from the same
    initial state: Cl, Cd, Cm sampled every `every` coarse steps; errors
    relative to the FP64 value (floor 0.05) at step `early` (before the wake
    turns unsteady), at the last step, and of the means over the second half
    (the unsteady phase, where single samples diverge chaotically); mean
    density over the owned cells and the velocity field's relative L2 over
    both levels at the last step."""
    from aerokinetic_gb300.refined import RefinedSolver
    runs = {}
    for label, storage, fine in (("f64", "f64", "f64"),) + REFINED_FORMS:
        solver = RefinedSolver(project, refinement, storage=storage, fine_storage=fine, budget=False)
        series = []
        for _ in range(steps // every):
            rec = solver.advance(every)
            series.append([rec["cl"], rec["cd"], rec["cm"]])
        integrals = solver.conserved_integrals()
        volume = (solver.coarse_owned_cells * solver.coarse_level.dx ** 3
                  + solver.fine_fluid_cells * solver.fine_level.dx ** 3)
        (rc, uc), (rf, uf) = solver.level_macros()
        box = solver.plan.box
        owned = np.ones(rc.shape, bool)
        owned[box.lower[0]:box.upper[0], box.lower[1]:box.upper[1]] = False
        fluid = np.broadcast_to(~solver._fine_solid_xy()[:, :, None], rf.shape)
        runs[label] = (np.array(series), integrals["mass"] / volume, uc[owned], uf[fluid])
        solver.close()
    ref = runs["f64"]
    half = len(ref[0]) // 2
    k_early = early // every - 1

    def rel(a, b):
        return {k: float(abs(a[i] - b[i]) / max(abs(b[i]), 0.05)) for i, k in enumerate(("cl", "cd", "cm"))}
    out = {"coarse_steps": steps, "sample_every": every, "early_step": early,
           "mean_window": [int((half + 1) * every), steps], "error_floor": 0.05}
    for label, storage, fine in REFINED_FORMS:
        series, mean_rho, uc, uf = runs[label]
        du = np.sum((uc - ref[2]) ** 2) + np.sum((uf - ref[3]) ** 2)
        norm = np.sum(ref[2] ** 2) + np.sum(ref[3] ** 2)
        window = rel(series[half:].mean(axis=0), ref[0][half:].mean(axis=0))
        out[label] = {"coarse_storage": storage, "fine_storage": fine,
                      "at_early_step": rel(series[k_early], ref[0][k_early]), "at_last_step": rel(series[-1], ref[0][-1]),
                      "window_mean": window, "max_window_mean": max(window.values()),
                      "mean_rho_abs": abs(mean_rho - ref[1]), "u_l2_rel": float(np.sqrt(du / norm))}
    out["f64_values"] = {"cl": ref[0][-1][0], "cd": ref[0][-1][1], "cm": ref[0][-1][2], "mean_rho": ref[1],
                         "window_mean": dict(zip(("cl", "cd", "cm"), ref[0][half:].mean(axis=0).tolist()))}
    return out


def coefficient_series(solver, steps, every):
    """Cl, Cd, Cm of a uniform case every `every` steps."""
    out = []
    for _ in range(steps // every):
        rec = solver.advance(every, sample_last=True)
        out.append([rec["cl"], rec["cd"], rec["cm"]])
    return np.array(out)


def series_errors(low, ref, floor=0.05):
    """Relative errors (floor) of the last sample and of the second half's mean."""
    half = len(ref) // 2
    names = ("cl", "cd", "cm")
    last = {k: float(abs(low[-1][i] - ref[-1][i]) / max(abs(ref[-1][i]), floor)) for i, k in enumerate(names)}
    lm, rm = low[half:].mean(axis=0), ref[half:].mean(axis=0)
    window = {k: float(abs(lm[i] - rm[i]) / max(abs(rm[i]), floor)) for i, k in enumerate(names)}
    return last, window


def batch_errors(parts, storage="f16", steps=2000, every=20, per_chord=2):
    """Cl/Cd/Cm of the batch's reduced form against the plain FP64 form on
    `per_chord` cases of each chord: every case's bits in a batch equal the
    same case stepped alone (tests/test_batch.py), so each is stepped alone
    here in both forms."""
    from aerokinetic_gb300.solver import Solver
    chosen, seen = [], {}
    for i, p in enumerate(parts):
        chord = p[2].cells_per_chord
        if seen.get(chord, 0) < per_chord:
            seen[chord] = seen.get(chord, 0) + 1
            chosen.append(i)
    worst_last, worst_window, cases = {}, {}, []
    for i in chosen:
        series = {}
        for form in (storage, "f64"):
            solver = Solver(*parts[i], storage=form)
            series[form] = coefficient_series(solver, steps, every)
            solver.close()
        last, window = series_errors(series[storage], series["f64"])
        cases.append({"case": i, "chord": parts[i][2].cells_per_chord, "alpha_deg": parts[i][1].alpha_deg,
                      "at_last_step": last, "window_mean": window})
        for k in last:
            worst_last[k] = max(worst_last.get(k, 0.0), last[k])
            worst_window[k] = max(worst_window.get(k, 0.0), window[k])
    return {"form": storage, "steps": steps, "sample_every": every, "error_floor": 0.05,
            "max_at_last_step": worst_last, "max_window_mean": worst_window, "cases": cases}


def run_batch(steps, n_cases=64, solve_steps=5000):
    """Batched polar sweep (64 uneven cases) against the same cases solved one
    after another in the plain FP64 form.  Throughputs are measured over
    `steps` batch steps and scaled to solve_steps per case."""
    from aerokinetic_gb300 import Plan
    from aerokinetic_gb300.batch import Batch
    from aerokinetic_gb300.solver import Solver
    lib = None
    parts = [batch_case_parts(i) for i in range(n_cases)]
    cells = [math.prod(Plan.create(*p).shape) for p in parts]
    out = {"workload": f"{n_cases} NACA0012 cases, chord cells in {{24, 32, 48, 64}}, 12c x 8c x 8 (span 4 "
                       "requested, plan minimum 8), AoA U[-4, 16], Re log-U[1e4, 1e5], characteristic farfield",
           "cases": n_cases, "cells": int(sum(cells)), "solve_steps": solve_steps, "measured_steps": steps}
    for storage in ("f16", "f32"):
        solvers = [Solver(*p, storage=storage) for p in parts]
        with Batch(solvers) as batch:
            lib = batch._lib
            batch.advance(3, sample_last=False)
            schedule = batch.tune(trials=3)
            batch.advance(3, sample_last=False)
            launches0 = batch.launches
            ms = stream_ms(lib, batch.stream, lambda: batch.advance(steps, sample_last=False))
            launches = batch.launches - launches0
        for solver in solvers:
            solver.close()
        step_ms = ms / steps
        out[storage] = {"ms_per_step": step_ms, "mlups": sum(cells) / (step_ms / 1e3) / 1e6,
                        "solves_per_hour": n_cases / (solve_steps * step_ms / 1e3) * 3600,
                        "launches_per_step": launches / steps, "schedule": schedule,
                        "achieved_gbs": sum(cells) * BYTES_PER_CELL[storage] / (step_ms / 1e3) / 1e9,
                        # the batched stream-collide launch alone (the tuner's timing of it)
                        "bulk_achieved_gbs": sum(cells) * BYTES_PER_CELL[storage] / (schedule["ms_per_launch"] / 1e3)
                                             / 1e9}
    # plain form, one case at a time: per-step time of one case of each chord,
    # set-up time included once per case
    per_chord = {}
    for i, p in enumerate(parts):
        chord = p[2].cells_per_chord
        if chord in per_chord:
            continue
        t0 = time.perf_counter()
        solver = Solver(*p, storage="f64")
        solver.advance(3)
        setup_s = time.perf_counter() - t0
        k = max(10, min(steps, 40))
        ms = stream_ms(solver._lib, solver._lib.ak_case_stream(solver._case), lambda: solver.advance(k))
        per_chord[chord] = (ms / k, setup_s)
        solver.close()
    total_s = sum(per_chord[p[2].cells_per_chord][0] * solve_steps / 1e3 + per_chord[p[2].cells_per_chord][1]
                  for p in parts)
    out["plain_sequential"] = {"solves_per_hour": n_cases / total_s * 3600, "form": "f64, one case at a time",
                               "ms_per_step_by_chord": {str(c): v[0] for c, v in sorted(per_chord.items())}}
    out["speedup_f16_vs_plain"] = out["f16"]["solves_per_hour"] / out["plain_sequential"]["solves_per_hour"]
    out["speedup_f32_vs_plain"] = out["f32"]["solves_per_hour"] / out["plain_sequential"]["solves_per_hour"]
    out["error_vs_f64"] = {form: batch_errors(parts, form) for form in ("f16", "f32")}
    return out


def large_parts():
    """The large two-level case: NACA0012 main element (chord 64 coarse, 128
    fine cells) with a NACA0012 flap of 0.3c deflected 20 deg, 0.02c gap and
    0.01c overlap at the main trailing edge; Re 1e5, lattice Mach 0.1, AoA 6,
    span 32 coarse cells; coarse 3281 x 2195 x 32 and fine 866 x 422 x 64
    (254 M cells, 277 M cell updates per coarse step)."""
    from aerokinetic_gb300 import Flow, Grid, Project
    from aerokinetic_gb300.refined_plan import RefinementSettings
    from aerokinetic_gb300.serve import flapped_section
    section = flapped_section(0.0, 0.0, 0.12, 20.0, n_side=161)
    flow = Flow(reynolds=1e5, alpha_deg=6.0, lattice_speed=0.1 / math.sqrt(3))
    grid = Grid(cells_per_chord=64, upstream_chords=16.0, downstream_chords=34.0, transverse_chords=17.0,
                span_chords=0.5, memory_limit_gib=250)
    return Project(section, flow, grid), RefinementSettings(upstream_chords=1.5, downstream_chords=4.0,
                                                            transverse_chords=1.5)


def run_large(steps=8, error_steps=100):
    """The large two-element two-level case in the plain FP64 form and the FP16
    storage form: graph-replayed coarse steps timed by CUDA events; the FP16
    form's Cl, Cd, Cm against the FP64 form's after error_steps coarse steps."""
    import torch
    from aerokinetic_gb300 import _native
    from aerokinetic_gb300.refined import RefinedSolver
    project, refinement = large_parts()
    out = {"workload": "two-element NACA0012 + 0.3c flap at 20 deg, chord 64/128, Re 1e5, AoA 6, span 32, "
                       "legacy farfield"}
    lib = _native.load()
    coefficients = {}
    for storage in ("f64", "f16"):
        t0 = time.perf_counter()
        solver = RefinedSolver(project, refinement, storage=storage, budget=False)
        setup_s = time.perf_counter() - t0
        # timing group 2 is the coarse streaming fused with the collision
        assert solver.coarse_post_collision().any(), "the fine box must lie three coarse cells inside"
        cells = refined_cells(solver.plan)
        fine_padded = math.prod((2 * solver.plan.box.shape[0] + 4, 2 * solver.plan.box.shape[1] + 4,
                                 2 * solver.plan.box.shape[2]))
        _native.check(lib.ak_refined_step(solver._handle, 2, None))
        ms = stream_ms(lib, lib.ak_case_stream(solver._coarse),
                       lambda: _native.check(lib.ak_refined_step(solver._handle, steps, None)))
        groups = np.zeros(6)
        _native.check(lib.ak_refined_step_timed(solver._handle, 2, groups.ctypes.data_as(ctypes.c_void_p)))
        # the coarse streaming fused with the collision plus the fine passes
        collide_ms = (groups[2] + groups[3] + groups[4]) / 2
        collide_bytes = (math.prod(solver.plan.shape) * BYTES_PER_CELL[storage]
                         + fine_passes(solver.fine_storage) * fine_padded * BYTES_PER_CELL[solver.fine_storage])
        out.setdefault("coarse_shape", list(solver.plan.shape))
        out.setdefault("fine_shape", list(solver.fine_shape))
        out.setdefault("cell_updates_per_step", cells)
        out[storage] = {"mlups": cells * steps / (ms / 1e3) / 1e6, "ms_per_step": ms / steps,
                        "collide_achieved_gbs": collide_bytes / (collide_ms / 1e3) / 1e9,
                        "setup_s": setup_s, "device_gib": solver.plan.estimated_memory_gib, "steps": steps,
                        "fine_storage": solver.fine_storage}
        done = lib.ak_refined_steps_done(solver._handle)
        rec = solver.advance(error_steps - done) if error_steps > done else None
        coefficients[storage] = rec
        solver.close()
        torch.cuda.synchronize()
    ref, low = coefficients["f64"], coefficients["f16"]
    if ref is not None and low is not None:
        out["f16_error_vs_f64"] = {"coarse_steps": error_steps, "error_floor": 0.05,
                                   **{k: abs(low[k] - ref[k]) / max(abs(ref[k]), 0.05) for k in ("cl", "cd", "cm")}}
    return out


def run_serving(n_requests=16, rate_per_s=2.0, seed=7, budget_gib=120.0, chunk=500, error_budget_s=40.0,
                farfield="legacy"):
    """Continuous batching of the serving workload as specified: NACA 4-digit
    sections (m U[0, 0.04], p U[0.3, 0.5], t U[0.09, 0.15]), half with a 0.3c
    flap deflected U[0, 25] deg, chord 24-96 cells, span 4-32 cells, AoA
    U[-4, 14] deg, Re log-U[1e4, 1e5], 1000-20000 steps or until Cl changes by
    less than 1e-4 over 1000 steps; Poisson arrivals, a fixed HBM budget,
    FP32 compute and FP32 storage.  The outer boundary is the reference's
    default (legacy UBB and outflow): on the characteristic farfield every
    request that runs past ~5000 steps diverges, as the reference's own
    characteristic-farfield record does (it failed at step 5192).  Against the plain FP64 form one request
    at a time: each request's set-up and per-step time measured in the plain
    form and scaled to the steps it was served; the served coefficients
    compared with full FP64 solves of the smallest requests (as many as fit
    error_budget_s)."""
    import torch
    from aerokinetic_gb300.serve import Server, poisson_arrivals, random_requests
    from aerokinetic_gb300.solver import Solver
    requests = random_requests(n_requests, seed=seed, farfield=farfield)
    arrivals = poisson_arrivals(rate_per_s, n_requests, seed=seed)
    server = Server(memory_budget_gib=budget_gib, storage="f32", chunk=chunk)
    results = server.run(requests, arrivals)
    by_name = {r.name: r for r in requests}
    plain_s, per_step = 0.0, {}
    for res in results:
        req = by_name[res.name]
        t0 = time.perf_counter()
        solver = Solver(req.section, req.flow, req.grid, storage="f64")
        solver.advance(2)
        torch.cuda.synchronize()
        setup = time.perf_counter() - t0
        k = 20
        ms = stream_ms(solver._lib, solver._lib.ak_case_stream(solver._case), lambda: solver.advance(k))
        solver.close()
        per_step[res.name] = ms / k
        plain_s += setup + res.steps * ms / k / 1e3
    # full FP64 solves of the cheapest requests for the served form's error
    worst, checked, spent = {"cl": 0.0, "cd": 0.0, "cm": 0.0}, [], 0.0
    for res in sorted(results, key=lambda r: per_step[r.name] * r.steps):
        if spent + per_step[res.name] * res.steps / 1e3 > error_budget_s:
            break
        req = by_name[res.name]
        t0 = time.perf_counter()
        solver = Solver(req.section, req.flow, req.grid, storage="f64")
        solver.advance(res.steps - 1)
        ref = solver.advance(1, sample_last=True)
        solver.close()
        spent += time.perf_counter() - t0
        errors = {k: abs(getattr(res, k) - ref[k]) / max(abs(ref[k]), 0.05) for k in worst}
        checked.append({"request": res.name, "steps": res.steps, "status": res.status, **errors})
        for k in worst:
            worst[k] = max(worst[k], errors[k])
    stats = dict(server.stats)
    plain_rate = len(results) / plain_s * 3600
    stats.update({"workload": f"{n_requests} requests, Poisson arrivals at {rate_per_s}/s, NACA 4-digit m U[0, 0.04], "
                              "p U[0.3, 0.5], t U[0.09, 0.15], half with a 0.3c flap at U[0, 25] deg, chord 24-96 "
                              "cells, span 4-32 cells (plan minimum 8), AoA U[-4, 14], Re log-U[1e4, 1e5], "
                              "1000-20000 steps or Cl settled to 1e-4 over 1000 steps, " + farfield + " outer boundary",
                  "memory_budget_gib": budget_gib, "chunk": chunk,
                  "statuses": {s_: sum(r.status == s_ for r in results) for s_ in ("converged", "step_limit",
                                                                                   "failed")},
                  "converged": sum(r.converged for r in results),
                  "plain_sequential_solves_per_hour": plain_rate,
                  "plain_sequential": "FP64, one request at a time: measured set-up + measured per-step time x "
                                      "the steps each request was served",
                  "speedup_vs_plain": stats["solves_per_hour"] / plain_rate,
                  "max_relative_error_vs_f64": worst, "error_floor": 0.05, "error_checked": checked})
    return stats


def run_engine(args, rank, world, local_rank):
    import torch
    from aerokinetic_gb300 import _native
    from aerokinetic_gb300.refined import RefinedSolver
    from aerokinetic_gb300.solver import Solver
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
    lib = _native.load()
    project, refinement = refined_parts()

    # ---- headline: the two-level case in FP64, K coarse steps in the timed
    # region, each the reference's whole step: the walls' loads, and the mass
    # and momentum budget (outer-face flux, integrals of the state the step
    # leaves) computed every step (refined_solver.py:311-343)
    solver = RefinedSolver(project, refinement, storage="f64", budget=True)
    # timing group 2 is the coarse streaming fused with the collision
    assert solver.coarse_post_collision().any(), "the fine box must lie three coarse cells inside"
    plan = solver.plan
    cells = refined_cells(plan)
    ms = np.zeros(6)
    ptr = ms.ctypes.data_as(ctypes.c_void_p)
    _native.check(lib.ak_refined_step_timed(solver._handle, max(3, args.warmup), ptr))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    # the timed region replays the captured budget step (ak_refined_step_budget),
    # timed by CUDA events on the case's stream
    stream = torch.cuda.ExternalStream(lib.ak_case_stream(solver._coarse))
    loads, outer, stats = np.zeros((len(solver.contours), 5)), np.zeros(8), np.zeros(16)
    budget_args = [loads.ctypes.data_as(ctypes.c_void_p), outer.ctypes.data_as(ctypes.c_void_p),
                   stats.ctypes.data_as(ctypes.c_void_p)]
    _native.check(lib.ak_refined_step_budget(solver._handle, max(3, args.warmup), *budget_args))
    launches0 = lib.ak_kernel_launches(solver._coarse)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clocks:
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        start.record(stream)
        _native.check(lib.ak_refined_step_budget(solver._handle, args.steps, *budget_args))
        end.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    launches = lib.ak_kernel_launches(solver._coarse) - launches0
    elapsed_ms = float(start.elapsed_time(end))
    # per-group split from an eager run with events between the groups
    group_steps = min(args.steps, 200)
    ms[:] = 0
    _native.check(lib.ak_refined_step_timed(solver._handle, group_steps, ptr))
    groups = {"coarse_transfer_block_collide_ms": ms[1] / group_steps,
              "coarse_stream_collide_ms": ms[2] / group_steps,
              "fine_collide_ms": ms[3] / group_steps, "fine_stream_ms": ms[4] / group_steps,
              "interface_and_boundaries_ms": ms[5] / group_steps, "eager_step_ms": ms[0] / group_steps}
    if dist:
        elapsed_ms = reduce_max(elapsed_ms, dist)
    value = replica_mlups(cells, args.steps, elapsed_ms, world)
    fine_padded = math.prod(n for n in (2 * plan.box.shape[0] + 4, 2 * plan.box.shape[1] + 4, 2 * plan.box.shape[2]))
    coarse_cells = math.prod(plan.shape)
    solver.close()
    # the same step without the budget (loads only), for the budget's cost
    bare = RefinedSolver(project, refinement, storage="f64", budget=False)
    _native.check(lib.ak_refined_step(bare._handle, max(3, args.warmup), None))
    bare_ms = stream_ms(lib, lib.ak_case_stream(bare._coarse),
                        lambda: _native.check(lib.ak_refined_step(bare._handle, max(args.steps, 20), None)))
    bare_ms /= max(args.steps, 20)
    bare.close()
    if rank != 0:
        return
    hbm, peak_kind = peaks()
    # the dominant kernel: the coarse k_stream_collide<double>, the coarse
    # streaming fused with the next collision (every coarse cell read and
    # written once; the transfer block's cells streamed only).  It is bound by
    # GB300's FP64 pipe: its roofline is the measured FP64 FMA throughput,
    # against the collision's algorithmic FLOPs per cell
    fp64_peak = fma_peak(lib, 0)
    # the collision's forward sums (the chimera additions that take the 27
    # populations to their ten moments) run as exact integer additions on the
    # device: of the algorithmic FLOPs per cell these never reach the FP64 pipe
    forward_sums_per_cell = 66
    fp32_peak = fma_peak(lib, 1)
    fp32x2_peak = fma_peak(lib, 2)
    flops_cell = collision_flops(lib, "f64")
    xfer_cells = (plan.box.shape[0] + 6) * (plan.box.shape[1] + 6) * plan.shape[2]
    kernel_ms = groups["coarse_stream_collide_ms"]
    kernel_flops = (coarse_cells - xfer_cells) * flops_cell
    kernel_bytes = coarse_cells * BYTES_PER_CELL["f64"]
    achieved_tflops = kernel_flops / (kernel_ms / 1e3) / 1e12
    achieved_gbs = kernel_bytes / (kernel_ms / 1e3) / 1e9
    # the same for the collision launches of one coarse step (the fused coarse
    # pass and the fine block's passes)
    collide_bytes = (coarse_cells + fine_passes("f64") * fine_padded) * BYTES_PER_CELL["f64"]
    collide_ms = groups["coarse_stream_collide_ms"] + groups["fine_collide_ms"] + groups["fine_stream_ms"]
    achieved = collide_bytes / (collide_ms / 1e3) / 1e9

    # ---- end to end through the public API: case set-up from the host
    # description, every coarse step returning its loads to the host
    e2e_steps = E2E_STEPS
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s = RefinedSolver(project, refinement, storage="f64")
    for _ in range(e2e_steps):
        s.step()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    s.close()
    h2d = 8 * sum(len(c.xy) * 2 for c in project.section.normalized(project.flow.alpha_deg)) + 256

    # ---- reduced-precision forms of the two-level case
    forms = {}
    for label, storage, fine in REFINED_FORMS:
        r = RefinedSolver(project, refinement, storage=storage, fine_storage=fine, budget=False)
        fst = torch.cuda.ExternalStream(lib.ak_case_stream(r._coarse))
        _native.check(lib.ak_refined_step(r._handle, max(3, args.warmup), None))
        k = min(args.steps, 400)
        torch.cuda.synchronize()
        start.record(fst)
        _native.check(lib.ak_refined_step(r._handle, k, None))
        end.record(fst)
        torch.cuda.synchronize()
        step_ms = float(start.elapsed_time(end)) / k
        m = np.zeros(6)
        _native.check(lib.ak_refined_step_timed(r._handle, k, m.ctypes.data_as(ctypes.c_void_p)))
        r.close()
        # the coarse stream-collide and the fine block's passes
        cb = coarse_cells * BYTES_PER_CELL[storage] + fine_passes(fine) * fine_padded * BYTES_PER_CELL[fine]
        cms = (m[2] + m[3] + m[4]) / k
        forms[label] = {"coarse_storage": storage, "fine_storage": fine,
                          "mlups": cells / (step_ms / 1e3) / 1e6, "ms_per_step": step_ms,
                          "collide_achieved_gbs": cb / (cms / 1e3) / 1e9,
                          "collide_frac_of_" + peak_kind: cb / (cms / 1e3) / 1e9 / hbm,
                          # the same bytes over the whole replayed step
                          "step_achieved_gbs": cb / (step_ms / 1e3) / 1e9,
                          "step_frac_of_" + peak_kind: cb / (step_ms / 1e3) / 1e9 / hbm,
                          "groups_ms": {"coarse_transfer_block_collide": m[1] / k, "coarse_stream_collide": m[2] / k,
                                        "fine_collide": m[3] / k, "fine_stream": m[4] / k,
                                        "interface_and_boundaries": m[5] / k, "eager_step": m[0] / k}}

    # ---- the uniform case (the reference's CPU-runnable configuration)
    uniform = {}
    for storage in ("f64", "df64", "f32", "f16"):
        m = measure_form(storage, steps=min(args.steps, 100), warmup=args.warmup, flush=True,
                         measure_static=storage == "f64")
        bytes_launch = m["fluid_cells"] * BYTES_PER_CELL[storage]
        a = bytes_launch / (m["bulk_ms"] / 1e3) / 1e9
        uniform[storage] = {"mlups": m["cells"] / (m["step_ms"] / 1e3) / 1e6, "eager_step_ms": m["eager_step_ms"],
                            "kernel_mlups": m["cells"] / (m["bulk_ms"] / 1e3) / 1e6,
                            "stream_collide_ms": m["bulk_ms"], "achieved_gbs": a, "frac_of_" + peak_kind: a / hbm}
        if storage == "f64":
            uniform["f64"].update(sampled_step_ms=m["sampled_step_ms"],
                                  static_loads_step_ms=m["static_loads_step_ms"])
    # the same case with the other outer boundaries and with the Smagorinsky
    # subgrid rate (FP64 and the FP32 form)
    for label, farfield, sgs in (("exterior", "exterior_regularized_fd_v1", "none"),
                                 ("legacy", "legacy", "none"),
                                 ("smagorinsky", "characteristic_transport_v1", "smagorinsky")):
        for storage in ("f64", "f32"):
            m = measure_form(storage, steps=min(args.steps, 50), warmup=args.warmup, flush=True, farfield=farfield,
                             sgs=sgs)
            a = m["fluid_cells"] * BYTES_PER_CELL[storage] / (m["bulk_ms"] / 1e3) / 1e9
            uniform[f"{label}_{storage}"] = {"mlups": m["cells"] / (m["step_ms"] / 1e3) / 1e6,
                                             "eager_step_ms": m["eager_step_ms"],
                                             "kernel_mlups": m["cells"] / (m["bulk_ms"] / 1e3) / 1e6,
                                             "stream_collide_ms": m["bulk_ms"], "outer_boundary_ms": m["outer_ms"],
                                             "achieved_gbs": a, "frac_of_" + peak_kind: a / hbm}
    # the pair kernels on the same case at chord 64, whose copies exceed the
    # 129 MB L2 in both forms (170 MB per FP16 copy, 340 MB per FP32 copy)
    uniform["chord64"] = {"workload": "uniform NACA0012 768x512x8, chord 64, otherwise as above"}
    for storage in ("f32", "f16"):
        m = measure_form_at(64, storage, steps=min(args.steps, 50), warmup=args.warmup, flush=True)
        a = m["fluid_cells"] * BYTES_PER_CELL[storage] / (m["bulk_ms"] / 1e3) / 1e9
        uniform["chord64"][storage] = {"kernel_mlups": m["cells"] / (m["bulk_ms"] / 1e3) / 1e6,
                                       "stream_collide_ms": m["bulk_ms"], "achieved_gbs": a,
                                       "frac_of_" + peak_kind: a / hbm}

    forms["error_vs_f64"] = form_errors(project, refinement, steps=FORM_ERROR_STEPS)
    batch = run_batch(steps=min(args.steps, 100))
    serving = run_serving()
    large = run_large()

    cpu = oracle_sample(budget_s=15.0, refined=True)
    line = {"metric": METRIC, "value": value, "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "coarse_cells": coarse_cells,
                       "fine_cells": math.prod(2 * n for n in plan.box.shape),
                       "cell_updates_per_step": cells, "storage": "f64 populations, two copies per level",
                       "step": "loads and the mass/momentum budget every coarse step (the reference's step)",
                       "l2": "inputs larger than L2 (coarse 2 x 340 MB); uniform forms flushed between steps",
                       "parallelism": f"replicas x{world}"},
            "roofline": {"bound": "fp64", "achieved": achieved_tflops, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": achieved_tflops / fp64_peak, "traffic": TRAFFIC_BYTES_PER_LAUNCH,
                         "peak_source": "measured in this run (ak_fma_peak: FP64 FMA chains, 2 FLOPs per FMA)",
                         "kernel": "coarse k_stream_collide<double> (streaming fused with the collision)",
                         "flops_per_cell": flops_cell, "cells_collided_per_launch": coarse_cells - xfer_cells,
                         "integer_pipe_flops_per_cell": forward_sums_per_cell,
                         "frac_fp64_pipe": (flops_cell - forward_sums_per_cell) * (coarse_cells - xfer_cells)
                                           / (kernel_ms / 1e3) / 1e12 / fp64_peak,
                         "kernel_ms": kernel_ms, "bytes_per_launch": kernel_bytes,
                         "hbm": {"achieved": achieved_gbs, "peak": hbm, "unit": "GB/s", "frac": achieved_gbs / hbm,
                                 "peak_source": peak_kind},
                         "collision_launches_per_step": {"bytes": collide_bytes, "ms": collide_ms,
                                                         "achieved_gbs": achieved, "frac_of_hbm": achieved / hbm},
                         "fp32_fma_peak_tflops": fp32_peak, "fp32x2_fma_peak_tflops": fp32x2_peak},
            "groups_ms": groups,
            "budget": {"step_ms_with_budget": elapsed_ms / args.steps, "step_ms_without_budget": bare_ms,
                       "cost_fraction": (elapsed_ms / args.steps) / bare_ms - 1.0,
                       "includes": "outer-face flux and the integrals of the state each step leaves, every step; "
                                   "the coarse integrals from the fused stream-collide pass"},
            "forms": forms,
            "uniform": {"workload": UNIFORM, **uniform},
            "cpu_baseline": cpu,
            "e2e": {"value": cells * e2e_steps / e2e_s / 1e6, "unit": "MLUPS", "steps": e2e_steps,
                    "h2d_bytes_per_step": h2d / e2e_steps, "d2h_bytes_per_step": 5 * 8 + 4,
                    "includes": "case set-up from the host description; every coarse step returns its loads and "
                                "closes the mass/momentum budget (RefinedSolver.step)"},
            "batch": batch,
            "serving": serving,
            "large": large,
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
