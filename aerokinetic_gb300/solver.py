"""Solver: the reference's uniform Solver interface over the GB300 engine.

Same constructor, attributes and methods as src/aerokinetic/solver.py:33-537
(step, diagnostics, save_frame, run); the lattice lives on the GPU and every
numerical operation of a step runs in the engine's sm_103a kernels through the
C ABI of include/aerokinetic_gb300.h.  There is no CPU path.
"""
import csv
import ctypes
from dataclasses import asdict
import hashlib
import json
import math
import os
from pathlib import Path
import shutil
import time
import uuid

import numpy as np

from . import _native
from ._native import NumericalFailure, check
from .config import EXTERIOR_FARFIELD, Flow, Grid, Plan
from .geometry import Section
from .project import Project, RunSettings, write_json

__all__ = ["Solver", "NumericalFailure", "coefficients"]


def coefficients(force, moment_z, speed, chord_cells, span_cells):
    """Force on the solid: +Cl up, +Cd downstream, +Cm nose up (solver.py:27-30)."""
    q_area = 0.5 * speed**2 * chord_cells * span_cells
    return float(force[1] / q_area), float(force[0] / q_area), float(-moment_z / (q_area * chord_cells))


def _leading_edge(section, alpha_deg):
    """Rotated leading edge in chord units about the moment reference (solver.py:172-177)."""
    original = np.concatenate([e.xy for e in section.elements])
    leading = original[np.argmin(original[:, 0])]
    angle = -np.deg2rad(alpha_deg)
    rotation = np.array([[np.cos(angle), -np.sin(angle)], [np.sin(angle), np.cos(angle)]])
    return rotation @ ((leading - np.asarray(section.moment_reference)) / section.chord)


def _ptr(array):
    return array.ctypes.data_as(ctypes.c_void_p)


class Solver:
    """Uniform D3Q27 cumulant lattice around a fixed extruded section.

    storage selects the population format: "f64" is the reference's plain
    double-precision form; "f32" and "f16" keep FP32 arithmetic and store the
    shifted populations f - w in 32 or 16 bits.
    """

    def __init__(self, section: Section, flow: Flow = Flow(), grid: Grid = Grid(), progress=None, storage="f64"):
        if storage not in _native.STORAGE:
            raise ValueError(f"storage must be one of {sorted(_native.STORAGE)}")
        if grid.farfield not in _native.FARFIELD:
            raise ValueError(f"farfield {grid.farfield!r} is not provided by this engine")
        self.section, self.flow, self.grid, self.storage = section, flow, grid, storage
        self.plan = Plan.create(section, flow, grid, storage)
        self.contours = section.normalized(flow.alpha_deg)
        if self.plan.estimated_memory_gib > grid.memory_limit_gib:
            raise MemoryError(f"Estimated {self.plan.estimated_memory_gib:.2f} GiB exceeds the explicit "
                              f"limit {grid.memory_limit_gib:.2f} GiB. Inspect Plan before choosing a larger limit.")
        self._progress = progress or (lambda message: None)
        self._progress("Building the D3Q27 cumulant case on the GPU")
        self._lib = _native.load()
        self._case = None
        # exterior_regularized_fd_v1 pads the physical core by one auxiliary
        # cell in x and y, the engine's ghost layer (solver.py:36-41)
        self._exterior = grid.farfield == EXTERIOR_FARFIELD
        self._padding = (1, 1, 0) if self._exterior else (0, 0, 0)
        self._storage_shape = tuple(n + 2 * p for n, p in zip(self.plan.shape, self._padding))
        self._storage_origin = tuple(x - p * self.plan.dx for x, p in zip(self.plan.origin, self._padding[:2]))
        self._wall_mass_exchange = 0.0
        self._wall_mass_total = 0.0
        self._exterior_report = None
        self._exterior_source_total = np.zeros(4)
        self._build()
        self.steps = 0
        self.last_loads = None
        self._initialize()

    # --------------------------------------------------------------- set-up
    def _build(self):
        nx, ny, nz = self.plan.shape
        sizes = np.array([len(c.xy) for c in self.contours], dtype=np.int32)
        xy = np.ascontiguousarray(np.concatenate([c.xy for c in self.contours]), dtype=np.float64)
        self._poly = (sizes, xy)
        desc = _native.CaseDesc(nx, ny, nz, self.plan.origin[0], self.plan.origin[1], self.plan.dx,
                                self.plan.relaxation_rate, 1.0, self.flow.lattice_speed,
                                _native.FARFIELD[self.grid.farfield], _native.STORAGE[self.storage],
                                len(self.contours), sizes.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                xy.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                self.flow.smagorinsky_constant if self.flow.sgs == "smagorinsky" else 0.0)
        handle = ctypes.c_void_p()
        check(self._lib.ak_case_create(ctypes.byref(desc), ctypes.byref(handle)))
        self._case = handle
        info = _native.CaseInfo()
        check(self._lib.ak_case_get_info(self._case, ctypes.byref(info)))
        self.info = {name: getattr(info, name) for name, _ in info._fields_}
        self.wall_fallback_links = int(info.fallback_links)
        flags = np.zeros((nx, ny), dtype=np.uint8)
        check(self._lib.ak_get_flags(self._case, _ptr(flags)))
        self._solid_xy = flags != 0
        self._fluid = np.broadcast_to(~self._solid_xy[:, :, None], self.plan.shape)

    def _initialize(self):
        """Freestream plus the seeded divergence-free perturbation (solver.py:157-202)."""
        rng = np.random.default_rng(self.flow.seed)
        phase_y, phase_z = rng.uniform(0, 2 * np.pi, 2)
        leading = _leading_edge(self.section, self.flow.alpha_deg)
        amp = self.flow.perturbation * self.flow.lattice_speed
        check(self._lib.ak_init_perturbed(self._case, amp, phase_y, phase_z, float(leading[0]), float(leading[1]),
                                          self.plan.span))

    def set_fields(self, rho, velocity):
        """Equilibrium populations for given rho (nx,ny,nz) and u (nx,ny,nz,3)."""
        rho = np.ascontiguousarray(np.broadcast_to(rho, self.plan.shape), dtype=np.float64)
        velocity = np.ascontiguousarray(np.broadcast_to(velocity, self.plan.shape + (3,)), dtype=np.float64)
        check(self._lib.ak_init_fields(self._case, _ptr(rho), _ptr(velocity)))

    # --------------------------------------------------------------- stepping
    def _coefficients(self, per_element):
        total = per_element.sum(axis=0)
        cl, cd, cm = coefficients(total[:3], total[3], self.flow.lattice_speed, self.grid.cells_per_chord,
                                  self.plan.shape[2])
        return {"cl": cl, "cd": cd, "cm": cm, "element_lattice_loads": per_element[:, :4].copy(),
                "wall_mass_exchange_lattice": float(total[4])}

    def advance(self, nsteps, sample_last=False):
        """Run nsteps steps in one engine call; sample loads on the last one if asked."""
        out = np.zeros((len(self.contours), 5)) if sample_last else None
        check(self._lib.ak_step(self._case, int(nsteps), _ptr(out) if out is not None else None))
        self.steps += int(nsteps)
        if self._exterior:
            self._read_exterior()
        if out is None:
            return None
        self.last_loads = self._record(out)
        if self._exterior:
            # solver.py:264-271: the wall mass of every step accumulates
            self.last_loads.update(wall_mass_exchange_lattice=self._wall_mass_exchange,
                                   wall_mass_exchange_accumulated=self._wall_mass_total,
                                   exterior_source_mass_lattice=self._exterior_report["exterior_source_mass_momentum"][0],
                                   exterior_source_mass_accumulated=float(self._exterior_source_total[0]))
        return self.last_loads

    def _read_exterior(self):
        """The exterior boundary's bookkeeping after the last step (exterior.py:186-200)."""
        out = np.zeros(11)
        check(self._lib.ak_exterior_report(self._case, _ptr(out)))
        self._exterior_source_total = out[4:8].copy()
        self._wall_mass_exchange = float(out[8])
        self._wall_mass_total = float(out[9])
        self._exterior_report = {"step": self.steps, "reconstruction_moment_error": float(out[10]),
                                 "exterior_source_mass_momentum": out[0:4].tolist()} if self.steps else None

    def boundary_diagnostics(self):
        """Numerical exchanges of the exterior farfield, in lattice mass per step
        (solver.py:299-310); None for the other outer boundaries.  The engine
        stores post-collision populations, so pdf_stage differs from the
        reference's pre-collision storage."""
        if not self._exterior:
            return None
        self._read_exterior()
        return {"model": EXTERIOR_FARFIELD, "pdf_stage": "post_collision",
                "physical_shape": tuple(self.plan.shape), "storage_shape": self._storage_shape,
                "storage_origin": self._storage_origin,
                "wall_mass_exchange_lattice": self._wall_mass_exchange,
                "wall_mass_exchange_accumulated": self._wall_mass_total,
                "exterior_source_mass_momentum_accumulated": self._exterior_source_total.tolist(),
                "last_exterior_step": self._exterior_report,
                "definition": "Wall incoming-minus-outgoing mass and explicit auxiliary PDF source; a closed "
                              "bookkeeping budget does not prove zero wall mass flux or accuracy."}

    def _record(self, per_element):
        """The sample-step record of solver.py:262-279 from per-element lattice loads."""
        loads = self._coefficients(per_element)
        loads.update(step=self.steps, t_star=(self.steps - 0.5) * self.plan.dt_convective)
        if self.plan.dt_seconds is not None:
            loads["time_s"] = (self.steps - 0.5) * self.plan.dt_seconds
        return loads

    def step(self, sample=False):
        """One step; with sample=True the loads of its boundary stage (solver.py:252-279)."""
        return self.advance(1, sample_last=sample)

    def diagnostics(self):
        diag = np.zeros(5)
        code = self._lib.ak_diagnostics(self._case, _ptr(diag))
        check(code)
        return {"local_mach_max": float(diag[0]), "density_mean": float(diag[1]),
                "density_error_max": float(diag[2]), "wall_fallback_links": self.wall_fallback_links}

    # --------------------------------------------------------------- fields
    def macros(self):
        rho = np.empty(self.plan.shape)
        u = np.empty(self.plan.shape + (3,))
        check(self._lib.ak_macros(self._case, _ptr(rho), _ptr(u)))
        return rho, u

    def population_tensor(self):
        """The current population array as a torch tensor viewing the engine's
        device memory (no copy): shape (27, nz, ny + 2, pitch) in the storage's
        dtype (df64: a trailing (hi, lo) axis of float32), x and y offset by one
        ghost layer.  Valid until the next step swaps the two copies."""
        return population_view(self._lib, self._case, self.storage)

    def pdf(self):
        """Interior populations g = f - w as (nx, ny, nz, 27) doubles."""
        out = np.empty(self.plan.shape + (27,))
        check(self._lib.ak_get_pdf(self._case, _ptr(out)))
        return out

    def set_pdf(self, pdf):
        pdf = np.ascontiguousarray(pdf, dtype=np.float64)
        if pdf.shape != self.plan.shape + (27,):
            raise ValueError("populations must have shape (nx, ny, nz, 27)")
        check(self._lib.ak_set_pdf(self._case, _ptr(pdf)))

    def wall_links(self):
        """Distinct cut links: rows (element, x, y, direction) and their q."""
        n = self.info["wall_keys"]
        rows = np.zeros((n, 4), dtype=np.int32)
        q = np.zeros(n)
        check(self._lib.ak_get_wall_links(self._case, _ptr(rows), _ptr(q)))
        return rows, q

    def save_frame(self, path, max_pixels=800):
        """Mid-span speed, vorticity and Cp slice as .npz (solver.py:312-334)."""
        nx, ny, nz = self.plan.shape
        stride = max(1, math.ceil(max(nx, ny) / max_pixels))
        rho, velocity = self.macros()
        velocity = velocity[::stride, ::stride, nz // 2]
        rho = rho[::stride, ::stride, nz // 2]
        speed = np.linalg.norm(velocity, axis=-1) / self.flow.lattice_speed
        omega_z = (np.gradient(velocity[..., 1], stride * self.plan.dx, axis=0)
                   - np.gradient(velocity[..., 0], stride * self.plan.dx, axis=1)) / self.flow.lattice_speed
        cp = (rho - 1) / (1.5 * self.flow.lattice_speed**2)
        mask = self._solid_xy[::stride, ::stride]
        for array in (speed, omega_z, cp):
            array[mask] = np.nan
        path = Path(path)
        tmp = path.with_name(path.name + ".tmp")
        with open(tmp, "wb") as handle:
            np.savez_compressed(handle, speed=speed, omega_z=omega_z, cp=cp, mask=mask, origin=self.plan.origin,
                                dx=self.plan.dx * stride, t_star=self.steps * self.plan.dt_convective)
        tmp.replace(path)

    # --------------------------------------------------------------- checkpoints
    def save_checkpoint(self, path, context=None):
        from .checkpoint import save_checkpoint
        return save_checkpoint(self, path, context)

    @classmethod
    def from_checkpoint(cls, path, progress=None):
        from .checkpoint import restore_checkpoint
        return restore_checkpoint(cls, path, progress)

    @classmethod
    def resume_run(cls, output, callback=None, stop_event=None, progress=None, residual_callback=None):
        """Continue an interrupted run from output/checkpoint.npz (solver.py:345-351)."""
        output = Path(output)
        metadata = json.loads((output / "metadata.json").read_text(encoding="utf-8"))
        solver = cls.from_checkpoint(output / "checkpoint.npz", progress)
        run = dict(metadata["run"])
        return solver.run(output=output, callback=callback, stop_event=stop_event, residual_callback=residual_callback,
                          resume=True, **run)

    # --------------------------------------------------------------- run loop
    def run(self, duration_convective, output, sample_every=20, frame_every=200, average_after=0.0,
            check_every=100, callback=None, stop_event=None, checkpoint_every=1000, resume=False,
            termination=None, residual_callback=None):
        """Advance t* = t U / c and write history.csv, metadata.json, summary.json,
        frames and checkpoint.npz (solver.py:353-537): sampling, guards, frames,
        the callback/stop_event contract, checkpoints every checkpoint_every
        steps and at the end, resume from the last checkpoint (resume_run), and
        the failed-run report.  Steps between samples are one engine call.
        """
        from .project import StopCriteria
        if isinstance(termination, dict):
            termination = StopCriteria(**termination)
        settings = RunSettings(duration_convective, sample_every, frame_every, check_every, average_after,
                               checkpoint_every, termination or StopCriteria())
        project = Project(self.section, self.flow, self.grid, settings,
                          "+".join(e.name for e in self.section.elements))
        output = Path(output)
        if not resume and output.exists() and any(output.iterdir()):
            raise FileExistsError("Use a new/empty output directory to avoid mixing histories")
        output.mkdir(parents=True, exist_ok=True)
        (output / "frames").mkdir(exist_ok=resume)
        history = output / "history.csv"
        end_step = self.steps + _duration_steps(duration_convective, self.plan.dt_convective)
        metadata = {"version": "aerokinetic_gb300", "flow": asdict(self.flow), "grid": asdict(self.grid),
                    "plan": self.plan.as_dict(), "reference_chord_input_units": self.section.chord,
                    "moment_reference_input_units": self.section.moment_reference,
                    "contours": [{"name": e.name, "xy": e.xy.tolist()} for e in self.section.elements],
                    "coefficient_convention": "Cl up; Cd downstream; Cm nose-up about moment_reference; area=c*periodic_span",
                    "force_time": "midpoint of boundary momentum-transfer interval", "status": "running",
                    "experimental_validation": "not_performed", "case_fingerprint": project.case_fingerprint,
                    "run": asdict(settings), "start_step": self.steps,
                    "start_t_star": self.steps * self.plan.dt_convective, "storage": self.storage,
                    "resume_supported": True}
        names = ["step", "t_star", "time_s", "cl", "cd", "cm", "local_mach_max", "density_error_max"]
        if self._exterior:
            names.extend(("wall_mass_exchange_lattice", "wall_mass_exchange_accumulated",
                          "exterior_source_mass_lattice", "exterior_source_mass_accumulated"))
            metadata["boundary_model"] = self.boundary_diagnostics()
        rows = []
        if resume:
            old = json.loads((output / "metadata.json").read_text(encoding="utf-8"))
            metadata["start_step"] = old.get("start_step", 0)
            metadata["start_t_star"] = metadata["start_step"] * self.plan.dt_convective
            metadata["resumed_from_version"] = old.get("version")
            context = getattr(self, "_checkpoint_context", {})
            saved_project = Project.load(output / "project.json")
            if (saved_project.case_fingerprint != project.case_fingerprint
                    or asdict(saved_project.run) != asdict(settings)):
                raise ValueError("Saved project or run settings changed; resume requires the original project")
            if (old.get("case_fingerprint") != project.case_fingerprint
                    or context.get("case_fingerprint") != project.case_fingerprint):
                raise ValueError("Resume requires the original project, settings and checkpoint")
            if old.get("status") == "completed":
                raise ValueError("This run has already completed")
            end_step = context["end_step"]
            prefix = context["history_bytes"]
            if _file_hash(history, prefix) != context["history_sha256"]:
                raise ValueError("History before the checkpoint has changed; refusing to mix results")
            # samples and frames written after the last durable checkpoint are
            # kept aside, then the same timeline continues from the checkpoint
            future = [p for p in (output / "frames").glob("frame_*.npz") if int(p.stem.split("_")[-1]) > self.steps]
            if history.stat().st_size > prefix or future:
                recovery = output / "recovery" / uuid.uuid4().hex
                recovery.mkdir(parents=True)
                shutil.copy2(history, recovery / "history_before_resume.csv")
                with history.open("r+b") as handle:
                    handle.truncate(prefix)
                for path in future:
                    shutil.move(str(path), str(recovery / path.name))
            with history.open(newline="", encoding="utf-8") as handle:
                rows = list(csv.DictReader(handle))
            for row in rows:
                row["step"] = int(row["step"])
                for name in ("t_star", "cl", "cd", "cm"):
                    row[name] = float(row[name])
            if rows and rows[-1]["step"] > self.steps:
                raise ValueError("History extends beyond the checkpoint")
        else:
            project.save(output / "project.json")
        if self.steps > end_step:
            raise ValueError("Checkpoint is past the requested end time")
        from .convergence import RunControl
        control = RunControl(self, settings, output, resume=resume, callback=residual_callback,
                             start_step=metadata["start_step"])
        metadata["end_step"] = end_step
        metadata["residual_definition"] = ("Volume-weighted L2/Linf of d(rho,j_common)/dt*, owned fluid only; "
                                           "stationary-flow residual, not a turbulence-accuracy measure")
        write_json(output / "metadata.json", metadata)
        state, reason = "completed", "duration_reached"
        start = time.monotonic()
        try:
            self.diagnostics()
            self.save_frame(output / "frames" / f"frame_{self.steps:010d}.npz")
            with history.open("a" if resume else "w", newline="", encoding="utf-8") as handle:
                writer = csv.DictWriter(handle, names)
                if not resume:
                    writer.writeheader()

                def checkpoint():
                    handle.flush()
                    os.fsync(handle.fileno())
                    context = {"case_fingerprint": project.case_fingerprint, "end_step": end_step,
                               "history_bytes": history.stat().st_size, "history_sha256": _file_hash(history)}
                    context.update(control.checkpoint_context())
                    self.save_checkpoint(output / "checkpoint.npz", context)

                while self.steps < end_step:
                    if stop_event is not None and stop_event.is_set():
                        state, reason = "stopped", "user_stopped"
                        break
                    # next step that samples, checks, writes a frame or a checkpoint
                    nxt = end_step
                    for every in (sample_every, check_every, frame_every, checkpoint_every):
                        if every:
                            nxt = min(nxt, (self.steps // every + 1) * every)
                    if settings.termination.max_steps:
                        nxt = min(nxt, max(self.steps + 1, control.run_start_step + settings.termination.max_steps))
                    sample = nxt % sample_every == 0
                    record = self.advance(nxt - self.steps, sample_last=sample)
                    diagnostic = None
                    if self.steps % check_every == 0 or self.steps == end_step or sample:
                        diagnostic = self.diagnostics()
                    if self.steps % check_every == 0:
                        control.observe()
                    if self.steps % frame_every == 0 or self.steps == end_step:
                        self.save_frame(output / "frames" / f"frame_{self.steps:010d}.npz")
                    if record is not None:
                        if not all(math.isfinite(record[k]) for k in ("cl", "cd", "cm")):
                            raise NumericalFailure("Non-finite loads; the run is invalid")
                        row = {k: record.get(k, "") for k in names}
                        row.update({k: diagnostic[k] for k in ("local_mach_max", "density_error_max")})
                        writer.writerow(row)
                        handle.flush()
                        rows.append(row)
                        if callback is not None and callback(self, record) is False:
                            state, reason = "stopped", "user_stopped"
                            break
                    stop = control.stop_reason()
                    if stop:
                        reason = stop
                        if stop == "wall_time_limit":
                            state = "stopped"
                        break
                    if checkpoint_every and self.steps % checkpoint_every == 0:
                        checkpoint()
                self.diagnostics()
                self.save_frame(output / "frames" / f"frame_{self.steps:010d}.npz")
                checkpoint()
        except BaseException as error:
            state, reason = "failed", "failed"
            metadata["failure"] = f"{type(error).__name__}: {error}"
            raise
        finally:
            selected = np.array([[float(r["cl"]), float(r["cd"]), float(r["cm"])] for r in rows
                                 if float(r["t_star"]) >= average_after])
            ok = len(selected) and state != "failed"
            summary = {"status": state, "steps": self.steps, "t_star": self.steps * self.plan.dt_convective,
                       "wall_clock_seconds": time.monotonic() - start, "samples": len(rows),
                       "averaging_samples": len(selected), "average_after_t_star": average_after,
                       "mean": dict(zip(("cl", "cd", "cm"), selected.mean(axis=0))) if ok else None,
                       "rms_fluctuation": dict(zip(("cl", "cd", "cm"), selected.std(axis=0))) if ok else None,
                       "wall_fallback_links": self.wall_fallback_links, "experimental_validation": "not_performed"}
            summary.update(control.summary(reason))
            control.close()
            if self._exterior:
                boundary = json.loads(json.dumps(self.boundary_diagnostics(), allow_nan=True),
                                      parse_constant=lambda value: None)
                summary["boundary_diagnostics"] = boundary
                metadata["boundary_model"] = boundary
            metadata["status"] = state
            metadata["termination_reason"] = reason
            write_json(output / "metadata.json", metadata)
            write_json(output / "summary.json", summary)
        return summary

    # --------------------------------------------------------------- lifetime
    def close(self):
        if getattr(self, "_case", None):
            self._lib.ak_case_destroy(self._case)
            self._case = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class _DeviceArray:
    """__cuda_array_interface__ of engine-owned device memory."""

    def __init__(self, pointer, shape, typestr, owner):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (pointer, False),
                                         "version": 3, "strides": None}
        self._owner = owner


def population_view(lib, handle, storage):
    import torch
    current, other = ctypes.c_void_p(), ctypes.c_void_p()
    dims = (ctypes.c_int64 * 4)()
    size = ctypes.c_int32()
    check(lib.ak_case_buffers(handle, ctypes.byref(current), ctypes.byref(other), dims, ctypes.byref(size)))
    shape = list(dims)
    typestr = {"f64": "<f8", "f32": "<f4", "f16": "<f2", "df64": "<f4"}[storage]
    if storage == "df64":
        shape.append(2)
    return torch.as_tensor(_DeviceArray(current.value, shape, typestr, handle), device="cuda")


def _file_hash(path, limit=None):
    """sha256 of a file's first `limit` bytes (all of it without a limit)."""
    digest = hashlib.sha256()
    remaining = None if limit is None else int(limit)
    with Path(path).open("rb") as handle:
        while remaining is None or remaining > 0:
            block = handle.read(1 << 20 if remaining is None else min(1 << 20, remaining))
            if not block:
                break
            digest.update(block)
            if remaining is not None:
                remaining -= len(block)
    return digest.hexdigest()


def _duration_steps(duration, dt):
    """Whole steps covering duration, snapping round-off near an integer (timing.py:5-21)."""
    if not math.isfinite(duration) or not math.isfinite(dt) or duration <= 0 or dt <= 0:
        raise ValueError('Duration and time step must be finite and positive')
    q = duration / dt
    if not math.isfinite(q):
        raise ValueError('Requested step count overflows')
    nearest = round(q)
    if nearest >= 1 and abs(q - nearest) <= min(4 * math.ulp(q), 1e-8):
        return int(nearest)
    return max(1, math.ceil(q))
