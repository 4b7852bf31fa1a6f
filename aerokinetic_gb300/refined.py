"""RefinedSolver: the reference's two-level (2:1) airfoil solver on the GB300 engine.

Same construction and step interface as src/aerokinetic/refined_solver.py:115-345
(RefinedSolver(project, refinement).step() -> {"step", "t_star", "cl", "cd",
"cm"}), with both levels resident on the GPU and every operation of a step
(collisions, streaming, outer boundary, walls, donors, face fluxes, reflux,
restriction) in the engine's sm_103a kernels (include/aerokinetic_gb300.h,
ak_refined_*).
"""
import ctypes

import numpy as np

from . import _native
from ._native import check
from .refined_plan import RefinedPlan, RefinementSettings
from .solver import _leading_edge, _ptr

__all__ = ["RefinedSolver", "RefinementSettings", "RefinedPlan"]


class RefinedSolver:
    pad = 2

    def __init__(self, project, refinement=RefinementSettings(), progress=None, storage="f64"):
        if storage not in _native.STORAGE:
            raise ValueError(f"storage must be one of {sorted(_native.STORAGE)}")
        self.project, self.refinement, self.storage = project, refinement, storage
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
                                   (ctypes.c_int32 * 3)(*box.upper))
        handle = ctypes.c_void_p()
        check(self._lib.ak_refined_create(ctypes.byref(desc), ctypes.byref(handle)))
        self._handle = handle
        self._coarse = ctypes.c_void_p(self._lib.ak_refined_level(handle, 0))
        self._fine = ctypes.c_void_p(self._lib.ak_refined_level(handle, 1))
        self.fine_shape = tuple(2 * n for n in box.shape)

    def initialize_flow(self):
        """Free stream plus the seeded perturbation on both levels (refined_solver.py:224-269)."""
        rng = np.random.default_rng(self.flow.seed)
        phase_y, phase_z = rng.uniform(0, 2 * np.pi, 2)
        leading = _leading_edge(self.section, self.flow.alpha_deg)
        amp = self.flow.perturbation * self.flow.lattice_speed
        check(self._lib.ak_refined_init_perturbed(self._handle, amp, phase_y, phase_z, float(leading[0]),
                                                  float(leading[1])))
        self.steps = 0

    def _record(self, raw):
        f = self.fine_level
        volume, unit = f.dx ** 3, f.lattice_velocity_unit
        impulse = raw[:, :3].sum(axis=0) * volume * unit
        moment = raw[:, 3].sum() * f.dx * volume * unit
        q_area = 0.5 * self.plan.span
        force = impulse / self.coarse_level.dt
        record = {"step": self.steps, "t_star": (self.steps - 0.5) * self.coarse_level.dt,
                  "cl": float(force[1] / q_area), "cd": float(force[0] / q_area),
                  "cm": float(-(moment / self.coarse_level.dt) / q_area),
                  "wall_mass_exchange": float(raw[:, 4].sum() * volume)}
        if self.plan.dt_seconds is not None:
            record["time_s"] = (self.steps - 0.5) * self.plan.dt_seconds
        return record

    def advance(self, nsteps):
        """nsteps coarse steps in one engine call; loads of the last one."""
        raw = np.zeros((len(self.contours), 5))
        check(self._lib.ak_refined_step(self._handle, int(nsteps), _ptr(raw)))
        self.steps += int(nsteps)
        self.last_loads = self._record(raw)
        return self.last_loads

    def step(self):
        return self.advance(1)

    def states(self):
        """Coarse populations (covered cells virtual) and the physical fine block, (x, y, z, 27)."""
        nx, ny, nz = self.plan.shape
        coarse = np.empty((nx, ny, nz, 27))
        check(self._lib.ak_get_pdf(self._coarse, _ptr(coarse)))
        fx, fy, fz = self.fine_shape
        padded = np.empty((fx + 2 * self.pad, fy + 2 * self.pad, fz, 27))
        check(self._lib.ak_get_pdf(self._fine, _ptr(padded)))
        return coarse, padded[self.pad:-self.pad, self.pad:-self.pad]

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
