"""Two-level (2:1) case description: refinement settings and the refined plan.

Mirrors the reference's refined_solver.py:23-112 (RefinementSettings,
RefinedPlan.create, the "aerokinetic_refined_project" JSON) and
refinement.py:23-65 (AcousticLevel): same fields, validation and box
placement, so refined project files load unchanged.
"""
from dataclasses import asdict, dataclass
import json
import math
from pathlib import Path

import numpy as np

from .project import Project


@dataclass(frozen=True)
class AcousticLevel:
    """dx and dt in one common system; relaxation times in lattice units."""
    dx: float
    dt: float
    tau_shear: float
    tau_bulk: float

    def __post_init__(self):
        for name in ("dx", "dt", "tau_shear", "tau_bulk"):
            value = getattr(self, name)
            if isinstance(value, (bool, np.bool_)) or not math.isfinite(value) or value <= 0:
                raise ValueError(f"{name} must be finite and positive")
        if self.tau_shear <= 0.5 or self.tau_bulk <= 0.5:
            raise ValueError("Relaxation times must be strictly above 0.5")

    @property
    def lattice_velocity_unit(self):
        return self.dx / self.dt

    def refined(self):
        """Two fine steps per coarse step at fixed physical viscosities."""
        return AcousticLevel(self.dx / 2, self.dt / 2, 0.5 + 2 * (self.tau_shear - 0.5),
                             0.5 + 2 * (self.tau_bulk - 0.5))


@dataclass(frozen=True)
class FineBox:
    """Half-open coarse-cell bounds of the fine region."""
    lower: tuple
    upper: tuple

    def __post_init__(self):
        for values in (self.lower, self.upper):
            if len(values) != 3 or any(isinstance(v, (bool, np.bool_)) or not isinstance(v, (int, np.integer))
                                       for v in values):
                raise ValueError("Fine-box bounds must be three integer indices")
        if any(lo < 0 or hi <= lo for lo, hi in zip(self.lower, self.upper)):
            raise ValueError("Fine-box bounds must have 0 <= lower < upper")
        object.__setattr__(self, "lower", tuple(int(v) for v in self.lower))
        object.__setattr__(self, "upper", tuple(int(v) for v in self.upper))

    @property
    def shape(self):
        return tuple(hi - lo for lo, hi in zip(self.lower, self.upper))


@dataclass(frozen=True)
class RefinementSettings:
    upstream_chords: float = 0.375
    downstream_chords: float = 0.75
    transverse_chords: float = 0.375
    guard_coarse_cells: int = 4
    coarse_bulk_relaxation_time: float = 1.0

    def __post_init__(self):
        for name in ("upstream_chords", "downstream_chords", "transverse_chords"):
            value = getattr(self, name)
            if not math.isfinite(value) or value <= 0:
                raise ValueError(f"Refinement {name} must be finite and positive")
        if type(self.guard_coarse_cells) is not int or self.guard_coarse_cells < 4:
            raise ValueError("At least four coarse cells must separate every wall from the fine interface")
        if not math.isfinite(self.coarse_bulk_relaxation_time) or self.coarse_bulk_relaxation_time <= .5:
            raise ValueError("Coarse bulk relaxation time must be finite and above 0.5")


@dataclass(frozen=True)
class RefinedPlan:
    shape: tuple
    origin: tuple
    box: FineBox
    coarse_level: AcousticLevel
    fine_level: AcousticLevel
    span: float
    dt_seconds: float | None
    estimated_memory_gib: float
    minimum_wall_interface_distance_coarse_cells: float
    notes: tuple

    @classmethod
    def create(cls, project, refinement):
        if project.grid.farfield != "legacy":
            raise ValueError("Characteristic farfield is not yet verified on refined grids; use a uniform grid explicitly")
        if project.flow.sgs != "none":
            raise ValueError("Refined SGS is not implemented; select sgs=none explicitly")
        base = project.plan()
        points = np.concatenate([e.xy for e in project.section.normalized(project.flow.alpha_deg)])
        lower, upper = points.min(axis=0), points.max(axis=0)
        margins_low = np.array([refinement.upstream_chords, refinement.transverse_chords])
        margins_high = np.array([refinement.downstream_chords, refinement.transverse_chords])
        lo = np.floor((lower - margins_low - base.origin) / base.dx + 1e-12).astype(int)
        hi = np.ceil((upper + margins_high - base.origin) / base.dx - 1e-12).astype(int)
        if np.any(lo < 1) or np.any(hi > np.array(base.shape[:2]) - 1):
            raise ValueError("The refined box must fit strictly inside the external x/y domain")
        distances = np.r_[(lower - (base.origin + lo * base.dx)) / base.dx,
                          ((base.origin + hi * base.dx) - upper) / base.dx]
        if distances.min() < refinement.guard_coarse_cells - 1e-10:
            raise ValueError("Wall/interface guard too small; enlarge the refinement margins")
        box = FineBox((*map(int, lo), 0), (*map(int, hi), base.shape[2]))
        coarse = AcousticLevel(base.dx, base.dt_convective, 1 / base.relaxation_rate,
                               refinement.coarse_bulk_relaxation_time)
        fine = coarse.refined()
        padded = tuple(2 * n + 4 for n in box.shape)
        cells = math.prod(n + 2 for n in base.shape) + math.prod(n for n in padded)
        memory = (cells * 2 * 27 * 8 * 1.1 + 64 * 2**20) / 2**30
        return cls(base.shape, base.origin, box, coarse, fine, base.span, base.dt_seconds, memory,
                   float(distances.min()),
                   ("Static two-level grid; fine cells/chord = 2 * coarse cells/chord.",
                    "All walls on the fine level; no SGS, wall model or compressible-energy model.",
                    "Bulk relaxation is an explicit numerical parameter."))

    def as_dict(self):
        data = asdict(self)
        data.update(dx=self.coarse_level.dx, dt_convective=self.coarse_level.dt,
                    coarse_cells_per_chord=round(1 / self.coarse_level.dx),
                    fine_cells_per_chord=round(1 / self.fine_level.dx),
                    fine_shape=tuple(2 * n for n in self.box.shape))
        return data


def refined_project_dict(project, refinement):
    return {"format": "aerokinetic_refined_project", "schema_version": 1,
            "project": project.as_dict(), "refinement": asdict(refinement)}


def load_refined_project(path_or_dict, base_directory=Path(".")):
    if isinstance(path_or_dict, dict):
        data = path_or_dict
    else:
        path = Path(path_or_dict)
        data = json.loads(path.read_text(encoding="utf-8-sig"))
        base_directory = path.resolve().parent
    if data.get("format") != "aerokinetic_refined_project" or data.get("schema_version") != 1:
        raise ValueError("This command requires an aerokinetic_refined_project, not a uniform project")
    return Project.from_dict(data["project"], base_directory), RefinementSettings(**data["refinement"])
