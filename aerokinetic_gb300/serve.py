"""Continuous batching of uniform solves on one GPU.

The reference answers one project per process; a polar sweep or a design loop
queues many.  Server keeps every admitted case's lattice resident in HBM and
advances all of them as one Batch (batch.py), admitting new requests as they
arrive and as device memory frees up, and retiring each case when its lift
coefficient settles or its step limit is reached.  Scheduling happens only at
chunk boundaries, every case is stepped by the same batched kernels whatever
its neighbours, and its convergence test reads only its own samples, so a
request's result is the same whether it ran alone or in any mix.  An
admitted request's case is built (plan, geometry, device set-up on its own
stream) by a host worker thread while the GPU advances the running batch; it
joins the batch at the next chunk boundary after it is ready.
"""
from concurrent.futures import ThreadPoolExecutor, wait, FIRST_COMPLETED
from dataclasses import dataclass, field
import math
import time

import numpy as np

from .config import Flow, Grid, Plan
from .geometry import Contour, Section, naca4_parametric

__all__ = ["SolveRequest", "SolveResult", "Server", "flapped_section", "random_requests", "poisson_arrivals"]


@dataclass(frozen=True)
class SolveRequest:
    """One solve.  It ends when |Cl(n) - Cl(n - window)| < cl_tolerance at a
    step n that is a multiple of window (from 2 windows on), or at max_steps
    (rounded up to the server's chunk)."""
    section: Section
    flow: Flow
    grid: Grid
    max_steps: int = 20000
    window: int = 1000
    cl_tolerance: float = 1e-4
    name: str = ""

    def __post_init__(self):
        if type(self.max_steps) is not int or self.max_steps < 1:
            raise ValueError("max_steps must be a positive integer")
        if type(self.window) is not int or self.window < 1:
            raise ValueError("window must be a positive integer")
        if not math.isfinite(self.cl_tolerance) or self.cl_tolerance <= 0:
            raise ValueError("cl_tolerance must be finite and positive")


@dataclass
class SolveResult:
    name: str
    cl: float
    cd: float
    cm: float
    steps: int
    converged: bool
    status: str           # "converged", "step_limit" or "failed"
    arrival_s: float
    admitted_s: float
    finished_s: float
    cells: int

    @property
    def latency_s(self):
        return self.finished_s - self.arrival_s


@dataclass(eq=False)
class _Live:
    request: SolveRequest
    solver: object
    arrival: float
    admitted: float
    device_bytes: int
    history: dict = field(default_factory=dict)


class Server:
    """memory_budget_gib: device memory the resident cases may hold; storage:
    the population form of every case ("f16", "f32" or "f64"); chunk: steps
    between scheduling points (each request's window is a multiple of it)."""

    def __init__(self, memory_budget_gib=200.0, storage="f32", chunk=250, tune_trials=0, max_cases=512,
                 clock=time.monotonic, sleep=time.sleep):
        if not math.isfinite(memory_budget_gib) or memory_budget_gib <= 0:
            raise ValueError("memory_budget_gib must be finite and positive")
        if type(chunk) is not int or chunk < 1:
            raise ValueError("chunk must be a positive integer")
        self.budget = int(memory_budget_gib * 2**30)
        self.storage, self.chunk, self.tune_trials, self.max_cases = storage, chunk, tune_trials, max_cases
        self.clock, self.sleep = clock, sleep
        self.stats = {}

    def footprint(self, request):
        """Device bytes a request will hold (the plan's estimate, set-up included)."""
        plan = Plan.create(request.section, request.flow, request.grid, self.storage)
        return int(plan.estimated_memory_gib * 2**30)

    def run(self, requests, arrivals=None):
        """Serve requests arriving at the given seconds after the start (all at
        once when None); returns their results in completion order."""
        from .batch import Batch
        from .solver import Solver
        requests = list(requests)
        arrivals = [0.0] * len(requests) if arrivals is None else [float(a) for a in arrivals]
        if len(arrivals) != len(requests):
            raise ValueError("one arrival time per request")
        for r in requests:
            if r.window % self.chunk:
                raise ValueError(f"window {r.window} of {r.name!r} is not a multiple of the chunk {self.chunk}")
            if self.footprint(r) > self.budget:
                raise MemoryError(f"request {r.name!r} alone exceeds the memory budget")
        order = sorted(range(len(requests)), key=lambda i: arrivals[i])
        pending = [(arrivals[i], requests[i]) for i in order]
        resident, results, building = [], [], []
        batch, used = None, 0
        peak_cases = peak_bytes = 0
        batch_steps = rebuilds = 0
        cell_updates = 0
        pool = ThreadPoolExecutor(max_workers=1, thread_name_prefix="admission")
        start = self.clock()
        try:
            while pending or resident or building:
                now = self.clock() - start
                changed = False
                # admission in arrival order while the footprint fits: the
                # memory is reserved now, the case is built by the worker
                while pending and pending[0][0] <= now and len(resident) + len(building) < self.max_cases:
                    arrival, request = pending[0]
                    need = self.footprint(request)
                    if used + need > self.budget:
                        break
                    pending.pop(0)
                    future = pool.submit(Solver, request.section, request.flow, request.grid, storage=self.storage)
                    building.append((future, arrival, need, request))
                    used += need
                if building and not resident:
                    # nothing to step: wait for a case (or the next arrival)
                    timeout = None if not pending else max(0.0, pending[0][0] - (self.clock() - start))
                    wait([b[0] for b in building], timeout=timeout, return_when=FIRST_COMPLETED)
                for item in [b for b in building if b[0].done()]:
                    building.remove(item)
                    future, arrival, need, request = item
                    resident.append(_Live(request, future.result(), arrival, self.clock() - start, need))
                    changed = True
                peak_cases = max(peak_cases, len(resident))
                peak_bytes = max(peak_bytes, used)
                if not resident:
                    if not building and pending:
                        self.sleep(max(0.0, pending[0][0] - (self.clock() - start)))
                    continue
                if changed or batch is None:
                    if batch is not None:
                        batch.close()
                    batch = Batch([live.solver for live in resident], tune_trials=self.tune_trials)
                    rebuilds += 1
                records = batch.advance(self.chunk)
                batch_steps += self.chunk
                cell_updates += self.chunk * sum(int(np.prod(l.solver.plan.shape)) for l in resident)
                finished = self.clock() - start
                keep = []
                for live, record in zip(resident, records):
                    steps = live.solver.steps
                    cl = record["cl"]
                    live.history[steps] = cl
                    status = None
                    if not all(math.isfinite(record[k]) for k in ("cl", "cd", "cm")):
                        status = "failed"
                    elif (steps % live.request.window == 0 and steps >= 2 * live.request.window
                          and abs(cl - live.history[steps - live.request.window]) < live.request.cl_tolerance):
                        status = "converged"
                    elif steps >= live.request.max_steps:
                        status = "step_limit"
                    if status is None:
                        keep.append(live)
                        continue
                    results.append(SolveResult(live.request.name, float(record["cl"]), float(record["cd"]),
                                               float(record["cm"]), steps, status == "converged", status,
                                               live.arrival, live.admitted, finished,
                                               int(np.prod(live.solver.plan.shape))))
                    used -= live.device_bytes
                if len(keep) != len(resident):
                    batch.close()
                    batch = None
                    for live in resident:
                        if live not in keep:
                            live.solver.close()
                    resident = keep
        finally:
            pool.shutdown(wait=True)
            for future, _, _, _ in building:
                if future.done() and future.exception() is None:
                    future.result().close()
            if batch is not None:
                batch.close()
            for live in resident:
                live.solver.close()
        makespan = self.clock() - start
        latencies = np.array([r.latency_s for r in results]) if results else np.zeros(1)
        self.stats = {"requests": len(requests), "completed": len(results), "makespan_s": makespan,
                      "solves_per_hour": len(results) / makespan * 3600 if makespan > 0 else float("inf"),
                      "latency_p50_s": float(np.percentile(latencies, 50)),
                      "latency_p95_s": float(np.percentile(latencies, 95)),
                      "latency_p99_s": float(np.percentile(latencies, 99)),
                      "peak_resident_cases": peak_cases, "peak_resident_gib": peak_bytes / 2**30,
                      "batch_rebuilds": rebuilds, "chunks": batch_steps // self.chunk,
                      "cell_updates": cell_updates, "storage": self.storage}
        return results


def flapped_section(m, p, thickness, flap_deg, flap_chord=0.3, gap=0.02, overlap=0.01, n_side=81):
    """Main NACA 4-digit element (unit chord) plus a NACA0012 flap of
    flap_chord, its leading edge at (1 - overlap, y_te - gap) below the main
    trailing edge and deflected flap_deg trailing edge down about it.  The
    reference has no flap builder; this follows the multi-element pattern of
    tests/test_multi_and_les.py:8-10 (scaled, rotated, translated contours).
    Reference chord 1, moment reference at the main element's quarter chord."""
    main = naca4_parametric(m, p, thickness, n_side, name="main")
    te = main.xy[np.isclose(main.xy[:, 0], main.xy[:, 0].max(), rtol=0, atol=1e-12)].mean(axis=0)
    flap = naca4_parametric(0.0, 0.0, 0.12, n_side, name="flap").xy * flap_chord
    a = -math.radians(flap_deg)
    rotation = np.array([[math.cos(a), -math.sin(a)], [math.sin(a), math.cos(a)]])
    flap = flap @ rotation.T + np.array([1.0 - overlap, te[1] - gap])
    return Section((main, Contour(flap, "flap")), chord=1.0, moment_reference=(0.25, 0.0))


def poisson_arrivals(rate_per_s, n, seed=0):
    """n arrival times (seconds) of a Poisson process of the given rate."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate_per_s, n)).tolist()


def random_requests(n, seed=0, chord=(24, 96), span=(4, 32), steps=(1000, 20000), window=1000,
                    flap_probability=0.5, cl_tolerance=1e-4, lattice_speed=0.1 / math.sqrt(3),
                    farfield="characteristic_transport_v1"):
    """Synthetic solve requests with the distributions of the serving workload:
    camber U[0, 0.04], camber position U[0.3, 0.5], thickness U[0.09, 0.15],
    optional 0.3c flap deflected U[0, 25] deg, chord cells in `chord`, span
    cells in `span`, AoA U[-4, 14] deg, Re log-uniform on [1e4, 1e5], step
    limits in `steps` (multiples of window), on the given outer boundary."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        m, p, t = rng.uniform(0, 0.04), rng.uniform(0.3, 0.5), rng.uniform(0.09, 0.15)
        if rng.uniform() < flap_probability:
            section = flapped_section(m, p, t, rng.uniform(0, 25))
        else:
            section = Section((naca4_parametric(m, p, t, 81, name="main"),))
        n_chord = int(rng.integers(chord[0], chord[1] + 1))
        n_span = int(rng.integers(span[0], span[1] + 1))
        flow = Flow(reynolds=float(10 ** rng.uniform(4, 5)), alpha_deg=float(rng.uniform(-4, 14)),
                    lattice_speed=lattice_speed, seed=int(rng.integers(0, 2**31 - 1)))
        grid = Grid(cells_per_chord=n_chord, upstream_chords=4.0, downstream_chords=7.0, transverse_chords=3.9,
                    span_chords=n_span / n_chord, farfield=farfield, memory_limit_gib=64)
        limit = int(rng.integers(steps[0] // window, steps[1] // window + 1)) * window
        out.append(SolveRequest(section, flow, grid, max_steps=max(limit, window), window=window,
                                cl_tolerance=cl_tolerance, name=f"request{i:04d}"))
    return out
