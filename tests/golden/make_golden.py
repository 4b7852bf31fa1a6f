"""Regenerate the golden fixtures of tests/golden/ from the reference checkout.

Run in a container that has the reference sources (read-only) at
/root/reference:

    python tests/golden/make_golden.py [--reference /root/reference]

Two kinds of fixture are written:

* recorded outputs of the reference's own runs, copied verbatim from its
  docs/ tree (acoustic probe records, Cl/Cd/Cm histories with their project
  files, the 272-step known answer);
* geometry produced by importing the reference's pure-numpy modules
  (aerokinetic.geometry, aerokinetic.config) and calling them: plans,
  normalised polygons, solid flags, and Bouzidi fractions from the
  reference's own link callback (solver.py:100-122), driven on a stub index
  list that holds every (fluid cell, direction) pair whose neighbour is solid.

Nothing at test time reads the reference checkout.
"""
import argparse
import csv
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

D3Q27 = [(0, 0, 0), (0, 1, 0), (0, -1, 0), (-1, 0, 0), (1, 0, 0), (0, 0, 1), (0, 0, -1), (-1, 1, 0), (1, 1, 0),
         (-1, -1, 0), (1, -1, 0), (0, 1, 1), (0, -1, 1), (-1, 0, 1), (1, 0, 1), (0, 1, -1), (0, -1, -1),
         (-1, 0, -1), (1, 0, -1), (1, 1, 1), (-1, 1, 1), (1, -1, 1), (-1, -1, 1), (1, 1, -1), (-1, 1, -1),
         (1, -1, -1), (-1, -1, -1)]

HISTORIES = {
    "failure_capture_n16": ("docs/verification_failure_capture_20261107", None),
    "characteristic_down3": ("docs/verification_farfield_20261107/airfoil/characteristic_down3", 120),
    "legacy_corrected32": ("docs/verification_stage1_20261106/corrected32_t12", 120),
    "legacy_down6": ("docs/verification_farfield_20261107/airfoil/legacy_down6", 120),
    "exterior_down3": ("docs/verification_exterior_library_20261108/raw/matched_airfoils/airfoil_down3", 60),
}
EXTERIOR_COLUMNS = ("wall_mass_exchange_lattice", "wall_mass_exchange_accumulated", "exterior_source_mass_lattice",
                    "exterior_source_mass_accumulated")

# Geometry cases: (name, project kwargs) built with the reference's classes.
GEOMETRY_CASES = {
    "kat272": dict(naca=("0012", 81), chord=1.0, ref=(0.25, 0.0),
                   flow=dict(reynolds=30000, alpha_deg=4, physical_chord_m=0.15),
                   grid=dict(cells_per_chord=32, upstream_chords=1.5, downstream_chords=3,
                             transverse_chords=1.5, span_chords=0.5, memory_limit_gib=2)),
    "uniform_c1": dict(naca=("0012", 161), chord=None, ref=None,
                       flow=dict(reynolds=30000, alpha_deg=4, lattice_speed=0.1 / np.sqrt(3)),
                       grid=dict(cells_per_chord=32, upstream_chords=4.0, downstream_chords=6.9867,
                                 transverse_chords=3.9266, span_chords=0.125,
                                 farfield="characteristic_transport_v1", memory_limit_gib=64)),
    "failure_capture_n16": dict(naca=("0012", 31), chord=None, ref=None,
                                flow=dict(reynolds=30000, alpha_deg=0, lattice_speed=0.04, perturbation=0),
                                grid=dict(cells_per_chord=16, upstream_chords=1, downstream_chords=2,
                                          transverse_chords=1, memory_limit_gib=2)),
    "two_element": dict(naca=None, chord=None, ref=None,
                        flow=dict(reynolds=30000, alpha_deg=6, lattice_speed=0.05),
                        grid=dict(cells_per_chord=48, upstream_chords=1.0, downstream_chords=1.5,
                                  transverse_chords=0.8, span_chords=0.2, memory_limit_gib=8)),
}


def read_history(path, limit):
    with open(path, newline="", encoding="utf-8") as handle:
        rows = list(csv.DictReader(handle))
    rows = rows if limit is None else rows[:limit]
    keep = ("step", "cl", "cd", "cm", "local_mach_max", "density_error_max")
    keep += tuple(k for k in EXTERIOR_COLUMNS if rows and k in rows[0])
    return [{k: (int(r[k]) if k == "step" else float(r[k])) for k in keep} for r in rows]


class _Stub:
    """Minimal stand-in for the index-list object the reference's callback receives."""

    def __init__(self, links):
        self.index_array = {"x": links[:, 0], "y": links[:, 1], "z": links[:, 2], "dir": links[:, 3]}
        self.offset = (-1, -1, -1)
        self.values = {}

    def link_offsets(self):
        return np.array(D3Q27, dtype=np.int64)[self.index_array["dir"]]

    def __setitem__(self, key, value):
        self.values[key] = np.asarray(value)


def geometry_fixture(ak, spec):
    from aerokinetic.geometry import naca4, Section, Contour
    from aerokinetic.config import Flow, Grid, Plan
    from aerokinetic.solver import Solver
    if spec["naca"] is None:
        main = naca4("0012", 81)
        flap_xy = naca4("0012", 41).xy * 0.3
        angle = -np.deg2rad(20.0)
        rot = np.array([[np.cos(angle), -np.sin(angle)], [np.sin(angle), np.cos(angle)]])
        flap_xy = flap_xy @ rot.T + np.array([0.99, -0.035])
        elements = (main, Contour(flap_xy, "flap"))
    else:
        elements = (naca4(spec["naca"][0], spec["naca"][1]),)
    section = Section(elements, spec["chord"], spec["ref"])
    flow, grid = Flow(**spec["flow"]), Grid(**spec["grid"])
    plan = Plan.create(section, flow, grid)
    contours = section.normalized(flow.alpha_deg)
    nx, ny, nz = plan.shape
    # solid flags of the padded (x, y) plane exactly as solver.py:93-98 evaluates them
    mid_x = np.arange(-1, nx + 1) + 0.5
    mid_y = np.arange(-1, ny + 1) + 0.5
    X, Y = np.meshgrid(mid_x, mid_y, indexing="ij")
    flags = np.zeros(X.shape, np.int8)
    for k, contour in enumerate(contours):
        inside = contour.contains(X * plan.dx + plan.origin[0], Y * plan.dx + plan.origin[1])
        flags[inside] = k + 1
    solver = Solver.__new__(Solver)
    solver.plan = plan
    solver._storage_origin = plan.origin
    solver.contours = contours
    solver.wall_fallback_links = 0
    c = np.array(D3Q27)
    links_out = []
    for k, contour in enumerate(contours):
        rows = []
        for x in range(1, nx + 1):
            for y in range(1, ny + 1):
                if flags[x, y] != 0:
                    continue
                for d in range(1, 27):
                    if c[d][2] != 0:
                        continue
                    if flags[x + c[d][0], y + c[d][1]] == k + 1:
                        rows.append((x, y, 1, d))
        links = np.array(rows, dtype=np.int64)
        stub = _Stub(links)
        solver._distance_callback(contour)(stub)
        q = stub.values["q"]
        for (x, y, _, d), qq in zip(links, q):
            links_out.append([k, int(x) - 1, int(y) - 1, int(c[d][0]), int(c[d][1]), float(qq)])
    return {
        "section": {"elements": [e.xy.tolist() for e in section.elements], "names": [e.name for e in section.elements],
                    "chord": section.chord, "moment_reference": list(section.moment_reference)},
        "flow": spec["flow"], "grid": spec["grid"],
        "plan": {"shape": [int(v) for v in plan.shape], "origin": list(plan.origin), "dx": plan.dx, "span": plan.span,
                 "viscosity": plan.viscosity, "relaxation_rate": plan.relaxation_rate,
                 "dt_convective": plan.dt_convective},
        "normalized": [e.xy.tolist() for e in contours],
        "solid_xy": [[int(v) for v in row] for row in flags[1:-1, 1:-1]],
        "wall_links_2d": links_out,
        "wall_fallback_links_2d": int(sum(1 for r in links_out if r[5] == -1.0)),
    }


def main():
    parser = argparse.ArgumentParser()
    parser.add_argument("--reference", default="/root/reference")
    args = parser.parse_args()
    ref = Path(args.reference)
    sys.path.insert(0, str(ref / "src"))
    import aerokinetic as ak

    acoustic = {}
    for name in ("ubb", "extrapolation"):
        with open(ref / "docs/verification_stage1_20261106/acoustics" / f"{name}.csv", newline="") as handle:
            acoustic[name] = [{k: float(v) for k, v in r.items() if k != "step"} | {"step": int(r["step"])}
                              for r in csv.DictReader(handle)]
    (HERE / "acoustic_probe.json").write_text(json.dumps(acoustic) + "\n")

    histories = {}
    for name, (path, limit) in HISTORIES.items():
        base = ref / path
        project = json.loads((base / "project.json").read_text())
        histories[name] = {"project": project, "history": read_history(base / "history.csv", limit),
                           "source": path}
    for name, (path, limit) in {"refined_startup": ("docs/verification_040", 12)}.items():
        base = ref / path
        project = json.loads((base / "startup_project.json").read_text())
        with open(base / "startup_history.csv", newline="", encoding="utf-8") as handle:
            rows = list(csv.DictReader(handle))[:limit]
        histories[name] = {"project": project, "source": path,
                           "history": [{k: (int(r[k]) if k == "step" else float(r[k]))
                                        for k in ("step", "cl", "cd", "cm")} for r in rows]}
    # the recorded Smagorinsky (sgs="smagorinsky") run: demo_wake/ was written
    # from examples/naca0012_wake_demo.json (demo_wake/README_RU.md)
    project = json.loads((ref / "examples/naca0012_wake_demo.json").read_text())
    histories["smagorinsky_wake"] = {"project": project, "source": "demo_wake; examples/naca0012_wake_demo.json",
                                     "history": read_history(ref / "demo_wake/history.csv", None)}
    (HERE / "histories.json").write_text(json.dumps(histories) + "\n")

    profile = json.loads((ref / "docs/verification_stage1_20261106/profile_threads1.json").read_text())
    kat = {"source": "tools/profile_stage1.py; docs/verification_stage1_20261106/profile_threads1.json",
           "steps": profile["warmup_steps"] + profile["timed_steps"], "shape": profile["shape"],
           "last_sample": profile["last_sample"]}
    (HERE / "kat272.json").write_text(json.dumps(kat, indent=1) + "\n")

    geometry = {name: geometry_fixture(ak, spec) for name, spec in GEOMETRY_CASES.items()}
    (HERE / "geometry.json").write_text(json.dumps(geometry) + "\n")
    print("wrote", sorted(p.name for p in HERE.glob("*.json")))


if __name__ == "__main__":
    main()
