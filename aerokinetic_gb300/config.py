"""Flow, grid and plan: the case parameters of one uniform lattice.

Mirrors the reference's config.py (Atmosphere 11-33, Flow 36-75, Grid 78-102,
Plan 106-166): same fields, defaults, validation messages and derived numbers
(shape, origin, dx, viscosity, relaxation rate, convective time step).  The
memory estimate describes this engine's device footprint instead of lbmpy's.
"""
from dataclasses import asdict, dataclass, field
import math

import numpy as np

EXTERIOR_FARFIELD = "exterior_regularized_fd_v1"
CHARACTERISTIC_FARFIELD = "characteristic_transport_v1"
FARFIELDS = ("legacy", CHARACTERISTIC_FARFIELD, EXTERIOR_FARFIELD)
STORAGE_MODES = ("f64", "f32", "f16", "df64")


@dataclass(frozen=True)
class Atmosphere:
    """ISA sea-level dry air; dimensional time also needs a physical chord."""
    temperature_k: float = 288.15
    pressure_pa: float = 101325.0
    gas_constant: float = 287.05287
    dynamic_viscosity: float = 1.7894e-5

    def __post_init__(self):
        if any(not math.isfinite(v) or v <= 0 for v in asdict(self).values()):
            raise ValueError("Atmospheric quantities must be finite and positive")

    @property
    def rho(self):
        return self.pressure_pa / (self.gas_constant * self.temperature_k)

    @property
    def nu(self):
        return self.dynamic_viscosity / self.rho

    @property
    def speed_of_sound(self):
        return math.sqrt(1.4 * self.gas_constant * self.temperature_k)


@dataclass(frozen=True)
class Flow:
    reynolds: float = 10000.0
    alpha_deg: float = 0.0
    lattice_speed: float = 0.04
    physical_chord_m: float | None = None
    atmosphere: Atmosphere = field(default_factory=Atmosphere)
    sgs: str = "none"
    smagorinsky_constant: float = 0.10
    perturbation: float = 1e-4
    seed: int = 31

    def __post_init__(self):
        if not 10000 <= self.reynolds <= 100000 or not math.isfinite(self.reynolds):
            raise ValueError("This module targets 10000 <= Re <= 100000")
        if not math.isfinite(self.alpha_deg) or abs(self.alpha_deg) >= 90:
            raise ValueError("Use an angle strictly between -90 and 90 degrees")
        if not 0 < self.lattice_speed <= 0.08:
            raise ValueError("Lattice speed must be in (0,0.08]; local Mach is monitored")
        if self.sgs not in ("none", "smagorinsky"):
            raise ValueError("sgs must be none or smagorinsky")
        if not 0 < self.smagorinsky_constant < 0.3:
            raise ValueError("Smagorinsky constant must be in (0,0.3)")
        if not 0 <= self.perturbation <= 0.01 or not math.isfinite(self.perturbation):
            raise ValueError("Initial perturbation must be in [0,0.01] relative to U")
        if self.physical_chord_m is not None:
            if not math.isfinite(self.physical_chord_m) or self.physical_chord_m <= 0:
                raise ValueError("Physical chord must be positive")
            if self.physical_mach > 0.15:
                raise ValueError("Physical Mach exceeds 0.15: this low-Mach model is unsuitable")

    @property
    def physical_speed(self):
        if self.physical_chord_m is None:
            return None
        return self.reynolds * self.atmosphere.nu / self.physical_chord_m

    @property
    def physical_mach(self):
        speed = self.physical_speed
        return None if speed is None else speed / self.atmosphere.speed_of_sound


@dataclass(frozen=True)
class Grid:
    cells_per_chord: int = 128
    upstream_chords: float = 6.0
    downstream_chords: float = 12.0
    transverse_chords: float = 6.0
    span_chords: float = 0.5
    memory_limit_gib: float = 8.0
    target: str = "cpu"
    openmp_threads: int = 1
    farfield: str = "legacy"

    def __post_init__(self):
        if not isinstance(self.cells_per_chord, int) or self.cells_per_chord < 16:
            raise ValueError("cells_per_chord must be an integer >=16")
        if self.target not in ("cpu", "gpu"):
            raise ValueError("target must be cpu or gpu")
        for key in ("upstream_chords", "downstream_chords", "transverse_chords", "span_chords",
                    "memory_limit_gib"):
            value = getattr(self, key)
            if not math.isfinite(value) or value <= 0:
                raise ValueError(f"{key} must be finite and positive")
        if type(self.openmp_threads) is not int or self.openmp_threads < 1:
            raise ValueError("openmp_threads must be a positive integer")
        if self.farfield not in FARFIELDS:
            raise ValueError("farfield must be one of " + ", ".join(FARFIELDS))


def device_bytes_per_cell(storage="f64"):
    """Bytes of HBM one lattice cell occupies in this engine (two population
    copies plus the per-column flag byte amortised over the span)."""
    size = {"f64": 8, "f32": 4, "f16": 2, "df64": 8}[storage]
    return 2 * 27 * size


@dataclass(frozen=True)
class Plan:
    shape: tuple
    origin: tuple
    dx: float
    span: float
    viscosity: float
    relaxation_rate: float
    dt_convective: float
    dt_seconds: float | None
    estimated_memory_gib: float
    notes: tuple

    @classmethod
    def create(cls, section, flow, grid, storage="f64"):
        contours = section.normalized(flow.alpha_deg)
        p = np.concatenate([e.xy for e in contours])
        xmin, ymin = p.min(axis=0)
        xmax, ymax = p.max(axis=0)
        n = grid.cells_per_chord
        shape = (math.ceil((xmax - xmin + grid.upstream_chords + grid.downstream_chords) * n),
                 math.ceil((ymax - ymin + 2 * grid.transverse_chords) * n),
                 max(8, math.ceil(grid.span_chords * n)))
        # the bounding box is centred transversely; x starts `upstream` ahead
        origin = (xmin - grid.upstream_chords, (ymin + ymax) / 2 - shape[1] / (2 * n))
        memory = (math.prod(v + 2 for v in shape[:2]) * shape[2] * device_bytes_per_cell(storage)
                  * 1.05 + 64 * 2**20) / 2**30
        nu = flow.lattice_speed * n / flow.reynolds
        tau = 0.5 + 3 * nu
        dt = flow.lattice_speed / n
        dt_s = None if flow.physical_speed is None else dt * flow.physical_chord_m / flow.physical_speed
        notes = ["One lattice spacing everywhere; walls by interpolated bounce-back, without a wall model "
                 "(two-level refinement is a separate RefinedSolver case).",
                 "The coefficients are lattice results: convergence in grid, domain, span, Mach number and averaging "
                 "window, and agreement with experiment, are for the user to establish.",
                 "The seeded spanwise perturbation only breaks the initial symmetry; it models no inflow turbulence."]
        if grid.farfield != "legacy":
            if min(grid.upstream_chords, grid.downstream_chords, grid.transverse_chords) * n < 2:
                raise ValueError("Characteristic farfield needs at least two fluid cells between body bounds and exterior")
            if grid.farfield == EXTERIOR_FARFIELD:
                if flow.sgs != "none":
                    raise ValueError("Exterior FD currently supports molecular viscosity with sgs=none only")
                notes.append("exterior_regularized_fd_v1: the physical lattice keeps its shape; one auxiliary ring of "
                             "cells in x and y is rebuilt every step from a predicted state, and the source this adds "
                             "is reported. Uniform grids only; its airfoil accuracy is not established.")
            else:
                notes.append("characteristic_transport_v1: per-link Riemann invariants with a linearised transverse "
                             "term, not a viscous characteristic boundary; its airfoil accuracy is not established.")
        if n < 256:
            notes.append("Below 256 cells per chord the boundary layer is not resolved; treat results as development runs.")
        if tau < 0.501:
            notes.append("The relaxation time is within 1e-3 of 0.5: shear modes are barely damped, so watch the Mach "
                         "and density guards and the resolution.")
        if flow.physical_speed is None:
            notes.append("No physical chord given: time is reported as t* = t U / c only.")
        else:
            atm = flow.atmosphere
            mean_free_path = atm.dynamic_viscosity / atm.pressure_pa * math.sqrt(
                math.pi * atm.gas_constant * atm.temperature_k / 2)
            if mean_free_path / flow.physical_chord_m > 1e-3:
                raise ValueError("Kn > 1e-3: the no-slip low-Kn model needs reconsideration")
        return cls(shape, origin, 1 / n, shape[2] / n, nu, 1 / tau, dt, dt_s, memory, tuple(notes))

    def as_dict(self):
        return asdict(self)
