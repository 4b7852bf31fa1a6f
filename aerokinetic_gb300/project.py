"""Case JSON ("aerokinetic_project", schema 1) and run settings.

Mirrors the reference's project.py:14-92 and convergence.py:26-50 (StopCriteria):
the same keys, defaults, validation and the SHA-256 case fingerprint over
geometry, flow and grid, so a project file written by either program loads in
the other with the same fingerprint.
"""
from dataclasses import asdict, dataclass, field
import hashlib
import json
import math
import os
from pathlib import Path
import tempfile

from .config import Atmosphere, Flow, Grid, Plan
from .geometry import Contour, Section, naca0012, naca4


@dataclass(frozen=True)
class StopCriteria:
    mode: str = 'time'
    mass_tolerance: float = 1e-5
    momentum_x_tolerance: float = 1e-5
    momentum_y_tolerance: float = 1e-5
    momentum_z_tolerance: float = 1e-5
    minimum_t_star: float = 1.
    consecutive_checks: int = 10
    max_steps: int = 0
    wall_time_limit_s: float = 0.

    def __post_init__(self):
        if self.mode not in ('time', 'steady'):
            raise ValueError('Stop mode must be time or steady')
        for name in ('mass_tolerance', 'momentum_x_tolerance', 'momentum_y_tolerance',
                     'momentum_z_tolerance'):
            if not math.isfinite(getattr(self, name)) or getattr(self, name) <= 0:
                raise ValueError(f'{name} must be finite and positive')
        for name in ('minimum_t_star', 'wall_time_limit_s'):
            if not math.isfinite(getattr(self, name)) or getattr(self, name) < 0:
                raise ValueError(f'{name} must be finite and nonnegative')
        for name, minimum in (('consecutive_checks', 1), ('max_steps', 0)):
            if type(getattr(self, name)) is not int or getattr(self, name) < minimum:
                raise ValueError(f'{name} must be an integer >= {minimum}')

    @property
    def thresholds(self):
        return (self.mass_tolerance, self.momentum_x_tolerance, self.momentum_y_tolerance, self.momentum_z_tolerance)


@dataclass(frozen=True)
class RunSettings:
    duration_convective: float = 0.2
    sample_every: int = 10
    frame_every: int = 20
    check_every: int = 10
    average_after: float = 0.1
    checkpoint_every: int = 1000
    termination: StopCriteria = field(default_factory=StopCriteria)

    def __post_init__(self):
        if isinstance(self.termination, dict):
            object.__setattr__(self, 'termination', StopCriteria(**self.termination))
        if not isinstance(self.termination, StopCriteria):
            raise ValueError('termination must contain stop criteria')
        if not math.isfinite(self.duration_convective) or self.duration_convective <= 0:
            raise ValueError("duration_convective must be finite and positive")
        if not math.isfinite(self.average_after) or self.average_after < 0:
            raise ValueError("average_after must be finite and nonnegative")
        for name in ("sample_every", "frame_every", "check_every", "checkpoint_every"):
            value = getattr(self, name)
            lowest = 0 if name == "checkpoint_every" else 1
            if type(value) is not int or value < lowest:
                raise ValueError(f"{name} has to be an integer >= {lowest}")


def write_json(path, data):
    """Atomic JSON write: temporary file in the same directory, then rename."""
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=path.parent, prefix=path.name, suffix=".tmp")
    try:
        with os.fdopen(fd, "w", encoding="utf-8") as handle:
            json.dump(data, handle, indent=2)
            handle.write("\n")
        os.replace(tmp, path)
    except BaseException:
        if os.path.exists(tmp):
            os.unlink(tmp)
        raise


@dataclass(frozen=True)
class Project:
    section: Section
    flow: Flow = field(default_factory=Flow)
    grid: Grid = field(default_factory=Grid)
    run: RunSettings = field(default_factory=RunSettings)
    title: str = "NACA0012"

    @classmethod
    def from_dict(cls, data, base_directory=Path(".")):
        if data.get("format", "aerokinetic_project") != "aerokinetic_project" or data.get("schema_version", 1) != 1:
            raise ValueError("Unsupported project format or schema version")
        geometry = data.get("geometry", {})
        if "elements" in geometry:
            elements = []
            for i, item in enumerate(geometry["elements"]):
                if "file" in item:
                    elements.append(Contour.from_dat(Path(base_directory) / item["file"]))
                else:
                    elements.append(Contour(item["xy"], item.get("name", f"element_{i}")))
            elements = tuple(elements)
        elif "naca4" in geometry:
            elements = (naca4(**geometry["naca4"]),)
        else:
            elements = (naca0012(**geometry.get("naca0012", {})),)
        flow = dict(data.get("flow", {}))
        flow["atmosphere"] = Atmosphere(**flow.get("atmosphere", {}))
        return cls(Section(elements, geometry.get("chord"), geometry.get("moment_reference")),
                   Flow(**flow), Grid(**data.get("grid", {})), RunSettings(**data.get("run", {})),
                   data.get("title", elements[0].name))

    @classmethod
    def load(cls, path):
        path = Path(path)
        return cls.from_dict(json.loads(path.read_text(encoding="utf-8-sig")), path.resolve().parent)

    def as_dict(self):
        grid = asdict(self.grid)
        # an absent farfield key means the legacy boundary; omitting the default
        # keeps the fingerprints of older project files unchanged
        if grid["farfield"] == "legacy":
            del grid["farfield"]
        return {"format": "aerokinetic_project", "schema_version": 1, "title": self.title,
                "geometry": {"elements": [{"name": e.name, "xy": e.xy.tolist()} for e in self.section.elements],
                             "chord": self.section.chord, "moment_reference": self.section.moment_reference},
                "flow": asdict(self.flow), "grid": grid, "run": asdict(self.run)}

    def save(self, path):
        write_json(path, self.as_dict())

    def plan(self):
        return Plan.create(self.section, self.flow, self.grid)

    @property
    def case_fingerprint(self):
        data = self.as_dict()
        case = {k: data[k] for k in ("geometry", "flow", "grid")}
        return hashlib.sha256(json.dumps(case, sort_keys=True, separators=(",", ":")).encode()).hexdigest()
