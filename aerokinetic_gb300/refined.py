"""RefinedSolver: the reference's two-level (2:1) airfoil solver on the GB300 engine.

Same construction and step interface as src/aerokinetic/refined_solver.py:115-345
(RefinedSolver(project, refinement).step() -> {"step", "t_star", "cl", "cd",
"cm"}), with both levels resident on the GPU and every operation of a step
(collisions, streaming, outer boundary, walls, donors, face fluxes, reflux,
restriction) in the engine's sm_103a kernels (include/aerokinetic_gb300.h,
ak_refined_*).
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
import uuid

import numpy as np

from . import _native
from ._native import check
from .project import write_json
from .refined_plan import RefinedPlan, RefinementSettings, refined_project_dict
from .solver import _duration_steps, _file_hash, _leading_edge, _ptr

__all__ = ["RefinedSolver", "RefinementSettings", "RefinedPlan"]


def _jsonable(value):
    """Plan dictionaries hold dataclasses and tuples: plain JSON values."""
    if isinstance(value, dict):
        return {k: _jsonable(v) for k, v in value.items()}
    if isinstance(value, (list, tuple)):
        return [_jsonable(v) for v in value]
    if isinstance(value, np.generic):
        return value.item()
    return value


def post_collision_columns(plan):
    """(nx, ny) coarse columns whose populations the engine stores
    post-collision: all but the transfer block (the fine box and three coarse
    cells around it) when that block lies inside the lattice, else none."""
    nx, ny, _ = plan.shape
    lo, hi = plan.box.lower, plan.box.upper
    mask = np.zeros((nx, ny), dtype=bool)
    if lo[0] >= 3 and hi[0] + 3 <= nx and lo[1] >= 3 and hi[1] + 3 <= ny:
        mask[:, :] = True
        mask[lo[0] - 3:hi[0] + 3, lo[1] - 3:hi[1] + 3] = False
    return mask


class RefinedSolver:
    """Two-level solver.  budget=True (the reference's behaviour) closes the
    mass and momentum budget of every step() (refined_solver.py:311-343);
    budget=False skips the per-step integrals and outer-face fluxes."""
    pad = 2

    def __init__(self, project, refinement=RefinementSettings(), progress=None, storage="f64", budget=True,
                 fine_storage=None):
        if storage not in _native.STORAGE:
            raise ValueError(f"storage must be one of {sorted(_native.STORAGE)}")
        # the FP16 form keeps the fine level, which holds the walls, in FP32:
        # the FP16 significand is spent on the far field's small departures
        # from the free stream, while the wall region's populations keep FP32's
        if fine_storage is None:
            fine_storage = "f32" if storage == "f16" else storage
        if fine_storage != storage and (storage, fine_storage) != ("f16", "f32"):
            raise ValueError("fine_storage must equal storage, or be 'f32' (or 'f16') under storage='f16'")
        self.project, self.refinement, self.storage = project, refinement, storage
        self.fine_storage = fine_storage
        self.budget = bool(budget)
        self.section, self.flow, self.grid = project.section, project.flow, project.grid
        self.plan = RefinedPlan.create(project, refinement)
        if self.plan.estimated_memory_gib > self.grid.memory_limit_gib:
            raise MemoryError(f"Estimated {self.plan.estimated_memory_gib:.2f} GiB exceeds the explicit limit "
                              f"{self.grid.memory_limit_gib:.2f} GiB")
        self.coarse_level, self.fine_level = self.plan.coarse_level, self.plan.fine_level
        self.contours = self.section.normalized(self.flow.alpha_deg)
        (progress or (lambda m: None))("Building the two-level case on the GPU")
        self._lib = _native.load()
        self._handle = None
        self._step_buffers = None
        self._build()
        self.steps = 0
        self.last_loads = None
        self.initialize_flow()

    def _build(self):
        nx, ny, nz = self.plan.shape
        sizes = np.array([len(c.xy) for c in self.contours], dtype=np.int32)
        xy = np.ascontiguousarray(np.concatenate([c.xy for c in self.contours]), dtype=np.float64)
        self._poly = (sizes, xy)
        coarse = _native.CaseDesc(nx, ny, nz, self.plan.origin[0], self.plan.origin[1], self.coarse_level.dx,
                                  1 / self.coarse_level.tau_shear, 1 / self.coarse_level.tau_bulk,
                                  self.flow.lattice_speed, _native.FARFIELD["legacy"], _native.STORAGE[self.storage],
                                  len(self.contours), sizes.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                  xy.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        box = self.plan.box
        desc = _native.RefinedDesc(coarse, self.coarse_level.tau_shear, self.coarse_level.tau_bulk,
                                   self.coarse_level.dt, self.plan.span, (ctypes.c_int32 * 3)(*box.lower),
                                   (ctypes.c_int32 * 3)(*box.upper), _native.STORAGE[self.fine_storage])
        handle = ctypes.c_void_p()
        check(self._lib.ak_refined_create(ctypes.byref(desc), ctypes.byref(handle)))
        self._handle = handle
        self._coarse = ctypes.c_void_p(self._lib.ak_refined_level(handle, 0))
        self._fine = ctypes.c_void_p(self._lib.ak_refined_level(handle, 1))
        self.fine_shape = tuple(2 * n for n in box.shape)
        check(self._lib.ak_refined_track_budget(handle, int(self.budget)))
        info = _native.CaseInfo()
        check(self._lib.ak_case_get_info(self._fine, ctypes.byref(info)))
        self.wall_fallback_links = int(info.fallback_links)
        self.fine_fluid_cells = int(info.fluid_cells) - self._band_cells()
        self.coarse_owned_cells = (nx * ny - box.shape[0] * box.shape[1]) * nz

    def _band_cells(self):
        fx, fy, fz = self.fine_shape
        return ((fx + 2 * self.pad) * (fy + 2 * self.pad) - fx * fy) * fz

    def initialize_flow(self):
        """Free stream plus the seeded perturbation on both levels (refined_solver.py:224-269)."""
        rng = np.random.default_rng(self.flow.seed)
        phase_y, phase_z = rng.uniform(0, 2 * np.pi, 2)
        leading = _leading_edge(self.section, self.flow.alpha_deg)
        amp = self.flow.perturbation * self.flow.lattice_speed
        check(self._lib.ak_refined_init_perturbed(self._handle, amp, phase_y, phase_z, float(leading[0]),
                                                  float(leading[1])))
        self.steps = 0
        self.initialized = True
        self.last_loads, self.last_budget = None, {}
        self._integrals = self._initial_integrals = self.conserved_integrals()

    def _record(self, raw):
        # element sums once, then scalar arithmetic in the same order as the
        # array expressions (sum * volume * unit, ...): the same doubles
        tot = raw.sum(axis=0).tolist()
        f = self.fine_level
        volume, unit = f.dx ** 3, f.lattice_velocity_unit
        dt = self.coarse_level.dt
        moment = tot[3] * f.dx * volume * unit
        q_area = 0.5 * self.plan.span
        record = {"step": self.steps, "t_star": (self.steps - 0.5) * dt,
                  "cl": (tot[1] * volume * unit / dt) / q_area, "cd": (tot[0] * volume * unit / dt) / q_area,
                  "cm": -(moment / dt) / q_area,
                  "wall_mass_exchange": tot[4] * volume}
        if self.plan.dt_seconds is not None:
            record["time_s"] = (self.steps - 0.5) * self.plan.dt_seconds
        return record

    # ------------------------------------------------------------ stepping
    def advance(self, nsteps):
        """nsteps coarse steps; loads (and, with budget, the budget) of the last one."""
        nsteps = int(nsteps)
        if nsteps < 1:
            raise ValueError("nsteps must be >= 1")
        if not self.initialized:
            raise RuntimeError("The refined state is invalid; initialize_flow() first")
        try:
            if nsteps > 1:
                check(self._lib.ak_refined_step(self._handle, nsteps - 1, None))
                self.steps += nsteps - 1
                self._integrals = None
            before = self._integrals if self._integrals is not None else (
                self.conserved_integrals() if self.budget else None)
            # the step's output arrays and their pointers, made once and
            # rewritten by every step (nothing below keeps a reference)
            if self._step_buffers is None:
                arrays = (np.zeros((len(self.contours), 5)), np.zeros(8), np.zeros(16))
                self._step_buffers = arrays + tuple(_ptr(a) for a in arrays)
            raw, flux, stats, praw, pflux, pstats = self._step_buffers
            if self.budget:
                # the step returns its loads, outer-face flux and integrals at once
                check(self._lib.ak_refined_step_budget(self._handle, 1, praw, pflux, pstats))
            else:
                check(self._lib.ak_refined_step(self._handle, 1, praw))
            self.steps += 1
        except Exception:
            self.initialized = False
            raise
        record = self._record(raw)
        if self.budget:
            self._close_budget(before, raw, flux, self._integrals_of(stats[:8], stats[8:]))
        self.last_loads = record
        return record

    def step(self):
        return self.advance(1)

    def _close_budget(self, before, raw, flux, after):
        """refined_solver.py:329-339 from the engine's integrals and outer-face flux."""
        # scalar arithmetic in the order of the array expressions it replaces
        f = self.fine_level
        self._integrals = after
        unit = f.lattice_velocity_unit
        tot = raw.sum(axis=0).tolist()
        ext = flux[:4].tolist()
        external = [ext[0]] + [e * unit for e in ext[1:]]
        dx3 = f.dx ** 3
        impulse = [tot[k] * dx3 * unit for k in range(3)]
        wall_mass = tot[4] * dx3
        mass_residual = after["mass"] - before["mass"] - external[0] - wall_mass
        momentum_residual = [after["momentum"][k] - before["momentum"][k] - external[1 + k] + impulse[k]
                             for k in range(3)]
        volume = self.coarse_owned_cells * self.coarse_level.dx ** 3 + self.fine_fluid_cells * dx3
        self.last_budget = {"mass_residual_per_volume": mass_residual / volume,
                            "momentum_residual_per_volume": [m / volume for m in momentum_residual],
                            "wall_mass_exchange": wall_mass, "external_mass_in": external[0],
                            "wall_impulse": impulse, "external_impulse_in": external[1:]}

    # ------------------------------------------------------------ integrals, validity
    def _stats(self):
        out = np.zeros(16)
        check(self._lib.ak_refined_integrals(self._handle, _ptr(out)))
        return out[:8], out[8:]

    def conserved_integrals(self):
        """Mass and momentum of the coarse cells outside the fine box and the
        fine fluid cells (refined_solver.py:291-299), common units."""
        return self._integrals_of(*self._stats())

    def _integrals_of(self, coarse, fine):
        mass, impulse = 0.0, [0.0, 0.0, 0.0]
        for st, level in zip((coarse, fine), (self.coarse_level, self.fine_level)):
            st = st.tolist()
            if st[7]:
                return {"mass": float("nan"), "momentum": [float("nan")] * 3}
            volume = level.dx ** 3
            mass += (st[6] + st[2]) * volume
            unit = level.lattice_velocity_unit
            impulse = [impulse[k] + st[3 + k] * volume * unit for k in range(3)]
        return {"mass": mass, "momentum": impulse}

    @property
    def cumulative_wall_impulse(self):
        cum = self._cumulative_loads()
        return cum[:, :3].sum(axis=0) * self.fine_level.dx ** 3 * self.fine_level.lattice_velocity_unit

    @property
    def cumulative_wall_mass_exchange(self):
        return float(self._cumulative_loads()[:, 4].sum() * self.fine_level.dx ** 3)

    @property
    def cumulative_external_in(self):
        flux = np.zeros(8)
        check(self._lib.ak_refined_outer_flux(self._handle, _ptr(flux)))
        out = flux[4:].copy()
        out[1:] *= self.fine_level.lattice_velocity_unit
        return out

    def _cumulative_loads(self):
        cum = np.zeros((len(self.contours), 5))
        check(self._lib.ak_refined_cumulative_loads(self._handle, _ptr(cum)))
        return cum

    def diagnostics(self):
        """Local Mach and density guards over both leaves (refined_solver.py:347-361)."""
        mach = density_error = 0.0
        for st in self._stats():
            if st[7]:
                mach = density_error = float("nan")
                break
            mach = max(mach, math.sqrt(st[0]) * math.sqrt(3))
            density_error = max(density_error, float(st[1]))
        if not (mach <= 0.3 and density_error <= 0.1):
            raise RuntimeError(f"Refined low-Mach state invalid: max Ma={mach:.5g}, density deviation={density_error:.5g}")
        wall_mass = self.cumulative_wall_mass_exchange
        return {"local_mach_max": mach, "density_error_max": density_error,
                "wall_fallback_links_including_donors": self.wall_fallback_links,
                "coarse_boundary_calls": self.coarse_boundary_calls, "fine_boundary_calls": self.fine_boundary_calls,
                "cumulative_wall_mass_exchange": wall_mass,
                "cumulative_wall_mass_exchange_over_initial_mass": wall_mass / self._initial_integrals["mass"],
                "last_budget": self.last_budget}

    @property
    def fine_steps(self):
        return 2 * self.steps

    @property
    def coarse_boundary_calls(self):
        return self.steps

    @property
    def fine_boundary_calls(self):
        return 2 * self.steps

    @property
    def time(self):
        return self.steps * self.coarse_level.dt

    @property
    def case_fingerprint(self):
        data = {"project_case": self.project.case_fingerprint, "refinement": asdict(self.refinement)}
        return hashlib.sha256(json.dumps(data, sort_keys=True, separators=(",", ":")).encode()).hexdigest()

    def coarse_post_collision(self):
        """(nx, ny) columns where states() holds post-collision coarse
        populations: outside the transfer block (the fine box and three coarse
        cells around it), whose coarse streaming is fused with the next step's
        collision, when that block lies inside the lattice.  The reference
        stores pre-collision populations everywhere; collision conserves mass
        and momentum, so macroscopic fields and integrals agree."""
        return post_collision_columns(self.plan)

    def states(self):
        """Pre-collision populations of the coarse lattice (covered cells
        virtual) and of the physical fine block, (x, y, z, 27) each, as the
        reference's states() returns them (interface.py:354-358).  Where the
        engine holds the coarse level post-collision (coarse_post_collision())
        the pre-collision state is rebuilt from the copy the last step read."""
        nx, ny, nz = self.plan.shape
        coarse = np.empty((nx, ny, nz, 27))
        fx, fy, fz = self.fine_shape
        padded = np.empty((fx + 2 * self.pad, fy + 2 * self.pad, fz, 27))
        check(self._lib.ak_refined_states(self._handle, _ptr(coarse), _ptr(padded)))
        return coarse, padded[self.pad:-self.pad, self.pad:-self.pad]

    def held_states(self):
        """The populations as the engine holds them (post-collision in the
        coarse_post_collision() columns), the representation checkpoints store."""
        nx, ny, nz = self.plan.shape
        coarse = np.empty((nx, ny, nz, 27))
        check(self._lib.ak_get_pdf(self._coarse, _ptr(coarse)))
        fx, fy, fz = self.fine_shape
        padded = np.empty((fx + 2 * self.pad, fy + 2 * self.pad, fz, 27))
        check(self._lib.ak_get_pdf(self._fine, _ptr(padded)))
        return coarse, padded[self.pad:-self.pad, self.pad:-self.pad]

    # ------------------------------------------------------------ frames and runs
    def level_macros(self):
        """(rho, u) of both levels in lattice units: the coarse lattice and the
        physical fine block, each (nx, ny, nz) and (nx, ny, nz, 3)."""
        out = []
        for handle, shape, crop in ((self._coarse, tuple(self.plan.shape), 0),
                                    (self._fine, tuple(self.fine_shape), self.pad)):
            full = (shape[0] + 2 * crop, shape[1] + 2 * crop, shape[2])
            rho, u = np.empty(full), np.empty(full + (3,))
            check(self._lib.ak_macros(handle, _ptr(rho), _ptr(u)))
            if crop:
                rho, u = rho[crop:-crop, crop:-crop], u[crop:-crop, crop:-crop]
            out.append((rho, u))
        return out

    def slice_data(self, z_plane=None):
        """Mid-span (or z_plane) section of both levels, the keys of
        interface_visualization.py:16-42 with zero background velocity."""
        z_plane = self.plan.span / 2 if z_plane is None else float(z_plane)
        unit = self.coarse_level.lattice_velocity_unit
        saved = {"time": self.time, "z_plane": z_plane, "background_velocity_lattice": np.zeros(3),
                 "velocity_unit": unit}
        box = self.plan.box
        origins = ((self.plan.origin[0], self.plan.origin[1]),
                   (self.plan.origin[0] + box.lower[0] * self.coarse_level.dx,
                    self.plan.origin[1] + box.lower[1] * self.coarse_level.dx))
        solid = self._fine_solid_xy()
        for label, (rho, u), (ox, oy), dx in zip(("coarse", "fine"), self.level_macros(), origins,
                                                  (self.coarse_level.dx, self.fine_level.dx)):
            nx, ny, nz = rho.shape
            zz = (np.arange(nz) + 0.5) * dx
            if not zz[0] <= z_plane <= zz[-1]:
                raise ValueError("Slice plane needs bracketing cell centres on both levels; extrapolation is unsupported")
            upper = min(nz - 1, max(1, int(np.searchsorted(zz, z_plane))))
            lower = upper - 1
            fraction = (z_plane - zz[lower]) / (zz[upper] - zz[lower])
            r = (1 - fraction) * rho[:, :, lower] + fraction * rho[:, :, upper]
            j = (1 - fraction) * (rho * u.transpose(3, 0, 1, 2))[..., lower] + fraction * (
                rho * u.transpose(3, 0, 1, 2))[..., upper]
            velocity = np.moveaxis(j / r, 0, -1) * unit
            if label == "coarse":
                mask = np.zeros((nx, ny), bool)
                mask[box.lower[0]:box.upper[0], box.lower[1]:box.upper[1]] = True
            else:
                mask = solid
            saved[f"{label}_speed"] = np.linalg.norm(velocity, axis=-1)
            saved[f"{label}_velocity_perturbation"] = velocity
            saved[f"{label}_rho"] = r
            saved[f"{label}_mask"] = mask
            saved[f"{label}_dx"] = dx
            saved[f"{label}_x_edges"] = ox + np.arange(nx + 1) * dx
            saved[f"{label}_y_edges"] = oy + np.arange(ny + 1) * dx
        return saved

    def _fine_solid_xy(self):
        if getattr(self, "_solid_cache", None) is None:
            flags = np.zeros((self.fine_shape[0] + 2 * self.pad, self.fine_shape[1] + 2 * self.pad), dtype=np.uint8)
            check(self._lib.ak_get_flags(self._fine, _ptr(flags)))
            self._solid_cache = flags[self.pad:-self.pad, self.pad:-self.pad] != 0
        return self._solid_cache

    def save_frame(self, path):
        """Mid-span section of both levels as .npz (refined_visualization.py:13-38)."""
        data = self.slice_data()
        data.update(format="aerokinetic_refined_slice", t_star=self.time,
                    contours_json=json.dumps([c.xy.tolist() for c in self.contours]),
                    fine_cells_per_chord=2 * self.grid.cells_per_chord)
        if self.flow.physical_speed is not None:
            data["physical_speed"] = self.flow.physical_speed
            data["physical_dynamic_pressure"] = 0.5 * self.flow.atmosphere.rho * self.flow.physical_speed ** 2
        for level in ("coarse", "fine"):
            mask = data[f"{level}_mask"]
            velocity = data[f"{level}_velocity_perturbation"].copy()
            if level == "fine":
                velocity[mask] = np.nan
            cp = (data[f"{level}_rho"] - 1) / (1.5 * self.flow.lattice_speed ** 2)
            cp[mask] = np.nan
            dx = float(data[f"{level}_dx"])
            omega = np.gradient(velocity[..., 1], dx, axis=0) - np.gradient(velocity[..., 0], dx, axis=1)
            omega[mask] = np.nan
            data[f"{level}_cp"] = cp
            data[f"{level}_omega_z"] = omega
            data[f"{level}_speed"][mask] = np.nan
        path = Path(path)
        tmp = path.with_name(path.name + ".tmp")
        with open(tmp, "wb") as handle:
            np.savez_compressed(handle, **data)
        tmp.replace(path)
        return path

    # ------------------------------------------------------------ checkpoints
    def _padded_shape(self):
        fx, fy, fz = self.fine_shape
        return (fx + 2 * self.pad, fy + 2 * self.pad, fz)

    def save_checkpoint(self, path, context=None):
        from .checkpoint import save_refined_checkpoint
        return save_refined_checkpoint(self, path, context)

    @classmethod
    def from_checkpoint(cls, path, progress=None):
        from .checkpoint import restore_refined_checkpoint
        return restore_refined_checkpoint(cls, path, progress)

    @classmethod
    def resume_run(cls, output, **kwargs):
        """Continue an interrupted run from output/checkpoint.npz (refined_run.py:159-163)."""
        output = Path(output)
        solver = cls.from_checkpoint(output / "checkpoint.npz", progress=kwargs.pop("progress", None))
        return solver.run(output, resume=True, **kwargs)

    def run(self, output, *, callback=None, stop_event=None, resume=False, residual_callback=None):
        """Run the project's RunSettings and write project.json, history.csv,
        metadata.json, summary.json, frames and checkpoint.npz
        (refined_run.py:19-156): checks, samples, frames, checkpoints every
        checkpoint_every steps and at the end, resume from the last checkpoint,
        the callback/stop_event contract and the failed-run report."""
        from .refined_plan import load_refined_project
        settings = self.project.run
        output = Path(output)
        if not resume and output.exists() and any(output.iterdir()):
            raise FileExistsError("Use a new/empty refined result directory")
        output.mkdir(parents=True, exist_ok=True)
        (output / "frames").mkdir(exist_ok=resume)
        history = output / "history.csv"
        columns = ["step", "t_star", "cl", "cd", "cm"]
        if self.plan.dt_seconds is not None:
            columns.append("time_s")
        end_step = self.steps + _duration_steps(settings.duration_convective, self.coarse_level.dt)
        if resume:
            metadata = json.loads((output / "metadata.json").read_text(encoding="utf-8"))
            context = getattr(self, "_checkpoint_context", {})
            metadata["resumed_with_version"] = "aerokinetic_gb300"
            original, refinement = load_refined_project(output / "project.json")
            if (original.case_fingerprint != self.project.case_fingerprint or refinement != self.refinement
                    or original.run != settings or metadata["case_fingerprint"] != self.case_fingerprint
                    or context.get("case_fingerprint") != self.case_fingerprint):
                raise ValueError("Refined project/run settings changed; cannot mix histories")
            if metadata["status"] == "completed":
                raise ValueError("The requested refined run has already completed")
            end_step = context["end_step"]
            prefix = context["history_bytes"]
            if _file_hash(history, prefix) != context["history_sha256"]:
                raise ValueError("Refined history before checkpoint changed")
            future = [p for p in (output / "frames").glob("frame_*.npz") if int(p.stem.split("_")[-1]) > self.steps]
            if history.stat().st_size > prefix or future:
                recovery = output / "recovery" / uuid.uuid4().hex
                recovery.mkdir(parents=True)
                shutil.copy2(history, recovery / "history_before_resume.csv")
                with history.open("r+b") as handle:
                    handle.truncate(prefix)
                for path in future:
                    shutil.move(str(path), str(recovery / path.name))
        else:
            metadata = {"format": "aerokinetic_refined_run", "version": "aerokinetic_gb300",
                        "case_fingerprint": self.case_fingerprint, "flow": asdict(self.flow),
                        "grid": asdict(self.grid), "refinement": asdict(self.refinement),
                        "plan": _jsonable(self.plan.as_dict()), "run": asdict(settings), "start_step": self.steps,
                        "contours": [{"name": e.name, "xy": e.xy.tolist()} for e in self.section.elements],
                        "coefficient_convention": "Cl up; Cd downstream; Cm nose-up about the chosen reference; area=c*periodic_span",
                        "force_time": "average of both fine momentum-transfer intervals; timestamp at coarse interval midpoint",
                        "experimental_validation": "not_performed", "resume_supported": True,
                        "storage": self.storage, "fine_storage": self.fine_storage,
                        "reference_chord_input_units": self.section.chord,
                        "moment_reference_input_units": self.section.moment_reference}
            write_json(output / "project.json", refined_project_dict(self.project, self.refinement))
            with history.open("w", newline="", encoding="utf-8") as handle:
                csv.DictWriter(handle, fieldnames=columns).writeheader()
            self.save_frame(output / "frames" / f"frame_{self.steps:09d}.npz")
        from .convergence import RunControl
        control = RunControl(self, settings, output, resume=resume, callback=residual_callback,
                             start_step=metadata.get("start_step", self.steps))
        metadata.update(status="running", target_steps=end_step)
        metadata["residual_definition"] = ("Volume-weighted L2/Linf of d(rho,j_common)/dt*, owned fluid only; "
                                           "integral balance defects of the last coarse step are a separate diagnostic")
        write_json(output / "metadata.json", metadata)
        status, error, reason = "completed", None, "duration_reached"

        def checkpoint(handle):
            handle.flush()
            os.fsync(handle.fileno())
            context = {"case_fingerprint": self.case_fingerprint, "end_step": end_step,
                       "history_bytes": history.stat().st_size, "history_sha256": _file_hash(history)}
            context.update(control.checkpoint_context())
            self.save_checkpoint(output / "checkpoint.npz", context)

        try:
            with history.open("a", newline="", encoding="utf-8") as handle:
                writer = csv.DictWriter(handle, fieldnames=columns)
                while self.steps < end_step:
                    if stop_event is not None and stop_event.is_set():
                        status, reason = "stopped", "user_stopped"
                        break
                    # steps up to the next one that checks, samples, writes a frame or a checkpoint
                    nxt = end_step
                    for every in (settings.check_every, settings.sample_every, settings.frame_every,
                                  settings.checkpoint_every):
                        if every:
                            nxt = min(nxt, (self.steps // every + 1) * every)
                    if settings.termination.max_steps:
                        nxt = min(nxt, max(self.steps + 1, control.run_start_step + settings.termination.max_steps))
                    record = self.advance(nxt - self.steps)
                    if self.steps % settings.check_every == 0:
                        self.diagnostics()
                        control.observe()
                    if self.steps % settings.sample_every == 0:
                        writer.writerow({k: record[k] for k in columns})
                        handle.flush()
                        if callback is not None and callback(self, record) is False:
                            status, reason = "stopped", "user_stopped"
                    if self.steps % settings.frame_every == 0:
                        self.save_frame(output / "frames" / f"frame_{self.steps:09d}.npz")
                    if settings.checkpoint_every and self.steps % settings.checkpoint_every == 0:
                        checkpoint(handle)
                    if status == "stopped":
                        break
                    stop = control.stop_reason()
                    if stop:
                        reason = stop
                        if stop == "wall_time_limit":
                            status = "stopped"
                        break
                self.diagnostics()
                self.save_frame(output / "frames" / f"frame_{self.steps:09d}.npz")
                checkpoint(handle)
        except Exception as failure:
            status, error, reason = "failed", f"{type(failure).__name__}: {failure}", "failed"
        with history.open(newline="", encoding="utf-8") as handle:
            rows = list(csv.DictReader(handle))
        selected = [r for r in rows if float(r["t_star"]) >= settings.average_after]
        mean = {n: float(np.mean([float(r[n]) for r in selected])) for n in ("cl", "cd", "cm")} if selected else None
        rms = {n: float(np.std([float(r[n]) for r in selected])) for n in ("cl", "cd", "cm")} if selected else None
        final = {"state": "invalid"}
        if self.initialized:
            try:
                final = self.diagnostics()
            except Exception as failure:
                status, error, reason = "failed", f"{type(failure).__name__}: {failure}", "failed"
                self.initialized = False
        summary = {"status": status, "steps": self.steps, "fine_steps": self.fine_steps, "t_star": self.time,
                   "average_after_t_star": settings.average_after, "samples": len(rows),
                   "averaging_samples": len(selected), "mean": mean, "rms": rms,
                   "experimental_validation": "not_performed", "statistical_convergence": "not_established",
                   "diagnostics": final}
        summary.update(control.summary(reason))
        control.close()
        if error:
            summary["error"] = error
        metadata.update(status=status, completed_steps=self.steps, termination_reason=reason)
        write_json(output / "metadata.json", metadata)
        write_json(output / "summary.json", summary)
        if error:
            raise RuntimeError(error)
        return summary

    def close(self):
        if getattr(self, "_handle", None):
            self._lib.ak_refined_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
