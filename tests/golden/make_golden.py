"""Regenerate the golden fixtures of tests/golden/ from the reference checkout.

Run where a checkout of the reference sources is available, naming it:

    python tests/golden/make_golden.py --reference <path to the checkout>

Two kinds of fixture are written:

* recorded outputs of the reference's own runs, copied verbatim from its
  docs/ tree (acoustic probe records, Cl/Cd/Cm histories with their project
  files, the 272-step known answer);
* geometry produced by importing the reference's pure-numpy modules
  (aerokinetic.geometry, aerokinetic.config) and calling them: plans,
  normalised polygons, solid flags, and Bouzidi fractions from the
  reference's own link callback (solver.py:100-122), driven on a stub index
  list that holds every (fluid cell, direction) pair whose neighbour is solid;
* two-level plans from the reference's RefinedPlan.create
  (refined_solver.py:42-99) for the two-level benchmark cases (refined_plans.json);
* unit vectors of the reference's level-transfer algebra on seeded inputs:
  D3Q27Transfer.moments / populations / _rescale_stress,
  prolong_cell_averages, restrict_cell_averages (refinement.py:78-254) and
  StreamingFaceFlux (interface.py:44-104) (transfer.json).

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


# Two-level benchmark cases, described by the parameters both sides build them
# from: the headline case (coarse 512 x 384 x 8 at chord 32, AoA 8) and the
# large two-element case (main element + 0.3c flap at 20 deg, chord 64).
REFINED_PLAN_CASES = {
    "two_level_512x384x8": dict(
        flap=None, flow=dict(reynolds=30000, alpha_deg=8, lattice_speed=0.1 / np.sqrt(3)),
        grid=dict(cells_per_chord=32, upstream_chords=5.0, downstream_chords=9.9938, transverse_chords=5.9056,
                  span_chords=0.25, memory_limit_gib=64),
        refinement=dict(upstream_chords=0.5, downstream_chords=1.0, transverse_chords=0.5)),
    "two_element_large": dict(
        flap=dict(m=0.0, p=0.0, thickness=0.12, flap_deg=20.0, n_side=161),
        flow=dict(reynolds=1e5, alpha_deg=6.0, lattice_speed=0.1 / np.sqrt(3)),
        grid=dict(cells_per_chord=64, upstream_chords=16.0, downstream_chords=34.0, transverse_chords=17.0,
                  span_chords=0.5, memory_limit_gib=1000),
        refinement=dict(upstream_chords=1.5, downstream_chords=4.0, transverse_chords=1.5)),
}


def refined_section(ak_geometry, spec):
    """The case's section as reference Contours.  The reference has no flap
    builder: the flapped polygon comes from this repository's
    serve.flapped_section (the same function the engine's cases use) and is
    handed to the reference as plain vertex arrays."""
    if spec["flap"] is None:
        return ak_geometry.Section((ak_geometry.naca4("0012", 161),))
    sys.path.insert(0, str(HERE.parents[1]))
    from aerokinetic_gb300.serve import flapped_section
    mine = flapped_section(**spec["flap"])
    elements = tuple(ak_geometry.Contour(np.array(e.xy), e.name) for e in mine.elements)
    return ak_geometry.Section(elements, mine.chord, mine.moment_reference)


def refined_plan_fixtures():
    """RefinedPlan.create of the reference (refined_solver.py:42-99) for the
    two-level benchmark cases."""
    from aerokinetic import geometry as G
    from aerokinetic.config import Flow, Grid
    from aerokinetic.project import Project
    from aerokinetic.refined_solver import RefinedPlan, RefinementSettings
    out = {}
    for name, spec in REFINED_PLAN_CASES.items():
        project = Project(refined_section(G, spec), Flow(**spec["flow"]), Grid(**spec["grid"]))
        plan = RefinedPlan.create(project, RefinementSettings(**spec["refinement"]))
        level = lambda L: {"dx": L.dx, "dt": L.dt, "tau_shear": L.tau_shear, "tau_bulk": L.tau_bulk}
        out[name] = {"spec": spec, "shape": list(plan.shape), "origin": list(plan.origin),
                     "box_lower": list(plan.box.lower), "box_upper": list(plan.box.upper),
                     "coarse_level": level(plan.coarse_level), "fine_level": level(plan.fine_level),
                     "span": plan.span,
                     "minimum_wall_interface_distance_coarse_cells":
                         plan.minimum_wall_interface_distance_coarse_cells}
    return out


def transfer_inputs(rng, shape):
    """Seeded pre-collision populations near a slow equilibrium: rho in
    [0.98, 1.02], |u| < 0.05, stress perturbations ~1e-3 of the weights, so
    the transfer's positivity and Mach checks pass."""
    w = np.prod(np.where(np.array(D3Q27) == 0, 2 / 3, 1 / 6), axis=1)
    c = np.array(D3Q27, dtype=float)
    rho = 1 + 0.02 * (2 * rng.random(shape) - 1)
    u = 0.05 / np.sqrt(3) * (2 * rng.random(shape + (3,)) - 1)
    cu = u @ c.T
    usq = np.sum(u * u, axis=-1)[..., None]
    feq = rho[..., None] * w * (1 + 3 * cu + 4.5 * cu ** 2 - 1.5 * usq)
    noise = 1e-3 * w * (2 * rng.random(shape + (27,)) - 1)
    return feq + noise - w  # zero-centred


def transfer_fixtures():
    """The reference's transfer algebra (refinement.py:78-254,
    interface.py:44-104) applied to seeded inputs; every array is stored in
    full so the tests need only numpy."""
    from aerokinetic.interface import StreamingFaceFlux
    from aerokinetic.refinement import (AcousticLevel, D3Q27Transfer, prolong_cell_averages,
                                        restrict_cell_averages)
    rng = np.random.default_rng(20261204)
    coarse = AcousticLevel(1 / 32, 0.1 / np.sqrt(3) / 32, 0.5 + 3 * 0.1 / np.sqrt(3) * 32 / 30000, 1.0)
    t = D3Q27Transfer(D3Q27, coarse, zero_centered=True, pdf_stage="pre_collision")
    cells = transfer_inputs(rng, (12,))
    moments = t.moments(cells)
    fields = moments.copy()
    fields[:, 4:] += 1e-4 * (2 * rng.random((12, 6)) - 1)
    block = transfer_inputs(rng, (6, 6, 5))
    block_moments = t.moments(block)
    fine = transfer_inputs(rng, (4, 6, 4))
    lattice = transfer_inputs(rng, (5, 6, 4))
    fluxes = []
    for axis, index, ranges in ((0, 1, ((1, 4), (0, 4))), (1, 2, ((0, 5), (1, 3))), (2, 0, ((1, 4), (2, 5)))):
        flux = StreamingFaceFlux((5, 6, 4), D3Q27, axis, index, ranges, periodic=True)
        fluxes.append({"axis": axis, "index": index, "ranges": [list(r) for r in ranges],
                       "flux": flux(lattice).tolist()})
    return {
        "stencil": D3Q27,
        "coarse_level": {"dx": coarse.dx, "dt": coarse.dt, "tau_shear": coarse.tau_shear,
                         "tau_bulk": coarse.tau_bulk},
        "cells": cells.tolist(), "moments": moments.tolist(),
        "fields": fields.tolist(), "populations": t.populations(fields).tolist(),
        "rescale_to_fine": t._rescale_stress(fields, t.coarse, t.fine).tolist(),
        "rescale_to_coarse": t._rescale_stress(fields, t.fine, t.coarse).tolist(),
        "block": block.tolist(), "prolonged_moments": prolong_cell_averages(block_moments).tolist(),
        "prolonged_in_time": t.prolong_in_time(block, block[::-1], 0.5).tolist(),
        "fine": fine.tolist(), "restricted_moments": restrict_cell_averages(t.moments(fine)).tolist(),
        "restricted": t.restrict(fine).tolist(),
        "lattice": lattice.tolist(), "face_fluxes": fluxes,
    }


def main():
    parser = argparse.ArgumentParser()
    parser.add_argument("--reference", required=True, help="path of the reference checkout")
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
    (HERE / "refined_plans.json").write_text(json.dumps(refined_plan_fixtures()) + "\n")
    (HERE / "transfer.json").write_text(json.dumps(transfer_fixtures()) + "\n")
    print("wrote", sorted(p.name for p in HERE.glob("*.json")))


if __name__ == "__main__":
    main()
