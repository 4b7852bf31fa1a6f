"""The host-side case layer (geometry, plan, project JSON) against the reference.

Fixtures in tests/golden/geometry.json were produced by the reference's own
numpy code (tests/golden/make_golden.py): plans, normalised polygons, solid
flags and Bouzidi fractions.  Flags, link sets and fractions are compared for
exact equality, as the engine must reproduce them bit for bit.
"""
import json

import numpy as np
import pytest

from aerokinetic_gb300.config import Flow, Grid, Plan
from aerokinetic_gb300.geometry import Contour, Section, naca0012, naca4
from aerokinetic_gb300.project import Project

O = pytest.importorskip("oracle.oracle")

CASES = ["kat272", "uniform_c1", "failure_capture_n16", "two_element"]


def rebuild(fixture):
    s = fixture["section"]
    elements = tuple(Contour(np.array(xy), name) for xy, name in zip(s["elements"], s["names"]))
    section = Section(elements, s["chord"], tuple(s["moment_reference"]))
    flow, grid = Flow(**fixture["flow"]), Grid(**fixture["grid"])
    return section, flow, grid


@pytest.mark.parametrize("name", CASES)
def test_plan_and_normalised_polygon_bit_exact(golden, name):
    fixture = golden["geometry"][name]
    section, flow, grid = rebuild(fixture)
    plan = Plan.create(section, flow, grid)
    ref = fixture["plan"]
    assert list(plan.shape) == ref["shape"]
    assert list(plan.origin) == ref["origin"]
    for key in ("dx", "span", "viscosity", "relaxation_rate", "dt_convective"):
        assert getattr(plan, key) == ref[key], key
    for mine, theirs in zip(section.normalized(flow.alpha_deg), fixture["normalized"]):
        assert np.array_equal(mine.xy, np.array(theirs))


def test_naca_points_match_reference_project(golden):
    """The project files of the reference embed naca4 polygons verbatim."""
    record = golden["histories"]["characteristic_down3"]["project"]
    xy = np.array(record["geometry"]["elements"][0]["xy"])
    assert np.array_equal(naca4("0012", 81).xy, xy)


@pytest.mark.parametrize("name", CASES)
def test_oracle_flags_and_fractions_bit_exact(golden, name):
    fixture = golden["geometry"][name]
    plan = fixture["plan"]
    nx, ny, _ = plan["shape"]
    contours = [np.array(c) for c in fixture["normalized"]]
    cx = (np.arange(nx) + 0.5) * plan["dx"] + plan["origin"][0]
    cy = (np.arange(ny) + 0.5) * plan["dx"] + plan["origin"][1]
    flags = np.zeros((nx, ny), np.int64)
    for k, c in enumerate(contours):
        flags[O.contains(c, cx[:, None], cy[None, :])] = k + 1
    assert np.array_equal(flags, np.array(fixture["solid_xy"]))
    # oracle link set and fractions, through its own lattice set-up at nz=1 rows
    case = O.AirfoilCase(contours, (nx, ny, 8), plan["origin"], plan["dx"], plan["span"],
                         plan["relaxation_rate"], 0.04, 32, "legacy", 0.0, 31, (0.0, 0.0), 1)
    rows = case.wall_links()
    mine = {(int(r[0]), int(r[1]), int(r[3]), int(r[4])): r[6] for r in rows if r[2] == 0 and r[5] == 0}
    theirs = {(r[1], r[2], r[3], r[4]): r[5] for r in fixture["wall_links_2d"]}
    assert mine.keys() == theirs.keys()
    for key, q in theirs.items():
        assert mine[key] == q, key


def test_project_round_trip_and_fingerprint(golden, tmp_path):
    record = golden["histories"]["characteristic_down3"]["project"]
    project = Project.from_dict(record)
    assert project.as_dict()["geometry"]["elements"][0]["xy"] == record["geometry"]["elements"][0]["xy"]
    path = tmp_path / "p.json"
    project.save(path)
    again = Project.load(path)
    assert again.case_fingerprint == project.case_fingerprint
    assert json.loads(path.read_text())["format"] == "aerokinetic_project"
    with pytest.raises(ValueError):
        Project.from_dict({"format": "other"})


def test_vectorised_intersection_tests_agree_with_the_pairwise_test():
    """Contour and Section validation evaluate segments_intersect (the
    reference's closed-segment test, geometry.py:112-123) over all edge pairs
    with numpy; on random polygons, including collinear and touching edges on
    a half-integer lattice, the outcome equals the pair-by-pair loop."""
    from aerokinetic_gb300.geometry import _any_segments_intersect, _pairs_intersect, segments_intersect
    rng = np.random.default_rng(7)
    for trial in range(200):
        n = int(rng.integers(3, 12))
        p = rng.normal(size=(n, 2))
        q = rng.normal(size=(5, 2))
        if trial % 3 == 0:
            p, q = np.round(p * 2) / 2, np.round(q * 2) / 2
        pn, qn = np.roll(p, -1, axis=0), np.roll(q, -1, axis=0)
        self_ref = any(segments_intersect(p[i], pn[i], p[j], pn[j])
                       for i in range(n) for j in range(i + 2, n) if not (i == 0 and j == n - 1))
        assert _any_segments_intersect(p, pn) == self_ref
        i, j = np.meshgrid(np.arange(n), np.arange(5), indexing="ij")
        pair_ref = [segments_intersect(p[a], pn[a], q[b], qn[b]) for a, b in zip(i.ravel(), j.ravel())]
        assert list(_pairs_intersect(p[i.ravel()], pn[i.ravel()], q[j.ravel()], qn[j.ravel()])) == pair_ref


def test_validation_errors_match_the_reference_messages():
    square = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], dtype=float)
    bowtie = np.array([[0, 0], [2, 2], [2, 0], [0, 1]], dtype=float)
    with pytest.raises(ValueError, match="Self-intersection"):
        Contour(bowtie, "bowtie")
    with pytest.raises(ValueError, match="touch or overlap"):
        Section((Contour(square, "a"), Contour(square + [0.5, 0.0], "b")))
    Section((Contour(square, "a"), Contour(square + [2.0, 0.0], "b")))


def test_post_collision_columns_follow_the_transfer_block(golden):
    """The coarse columns whose populations the engine stores post-collision:
    all but the fine box and three coarse cells around it, and none when that
    block reaches the lattice's edge (the unfused form)."""
    from types import SimpleNamespace

    from aerokinetic_gb300.refined import post_collision_columns
    from aerokinetic_gb300.refined_plan import RefinedPlan, load_refined_project
    project, refinement = load_refined_project(golden["histories"]["refined_startup"]["project"])
    plan = RefinedPlan.create(project, refinement)
    lo, hi = plan.box.lower, plan.box.upper
    mask = post_collision_columns(plan)
    assert mask.shape == tuple(plan.shape[:2])
    assert not mask[lo[0] - 3:hi[0] + 3, lo[1] - 3:hi[1] + 3].any()
    assert mask.sum() == mask.size - (hi[0] - lo[0] + 6) * (hi[1] - lo[1] + 6)
    edge = SimpleNamespace(shape=plan.shape, box=SimpleNamespace(lower=(2, lo[1], lo[2]), upper=hi))
    assert not post_collision_columns(edge).any()


def test_refined_fine_storage_choices_are_validated_before_any_device_work():
    """storage='f16' keeps the walls' fine level in FP32 unless told
    otherwise; any other mixture is refused up front."""
    import pytest
    from aerokinetic_gb300.refined import RefinedSolver
    from aerokinetic_gb300.refined_plan import RefinementSettings
    from aerokinetic_gb300 import Flow, Grid, Project, Section, naca0012
    project = Project(Section((naca0012(41),)), Flow(), Grid(cells_per_chord=16, memory_limit_gib=1))
    for storage, fine in (("f32", "f16"), ("f64", "f32"), ("f16", "f64")):
        with pytest.raises(ValueError, match="fine_storage"):
            RefinedSolver(project, RefinementSettings(), storage=storage, fine_storage=fine)


def test_normalized_contours_are_computed_once_and_read_only():
    """Section.normalized returns the same contours for the same angle (the
    plan and the solver both ask for them) and they cannot be modified."""
    section = Section((naca0012(41),))
    first = section.normalized(4.0)
    assert section.normalized(4) is first
    assert section.normalized(5.0) is not first
    with pytest.raises(ValueError):
        first[0].xy[0, 0] = 1.0
