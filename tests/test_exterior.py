"""exterior_regularized_fd_v1 on the GPU against the oracle and the reference's record.

The engine stores post-collision populations; the oracle (like the reference)
stores pre-collision ones, so the engine's state after step n is compared
with the oracle's state after step n collided once more.  Bars as for the
other outer boundaries: populations within 2e-12 per step, loads within
2e-10, the exterior source (a sum of ~2.4e5 rebuilt-minus-streamed
differences of order 1e-3) within 5e-12 per step, its running sum within
5e-12 times the step count.  The df64 form stores populations to 48 bits and
its collision differs from FP64 by up to ~5e-15 per population, so the same
sum over the ring carries up to ~1e-9 of that difference in the worst case;
it is held to 2e-10 per step.
"""
import json

import numpy as np
import pytest

from aerokinetic_gb300.config import Plan
from aerokinetic_gb300.project import Project
from tests.conftest import oracle_threads

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

O = pytest.importorskip("oracle.oracle")


@pytest.fixture(scope="module", autouse=True)
def _needs_device():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def exterior_pair(project, storage="f64"):
    from aerokinetic_gb300.solver import Solver
    from oracle.exterior import ExteriorCase
    plan = Plan.create(project.section, project.flow, project.grid)
    lead = O.leading_edge([e.xy for e in project.section.elements], project.section.moment_reference,
                          project.section.chord, project.flow.alpha_deg)
    oracle = ExteriorCase([c.xy for c in project.section.normalized(project.flow.alpha_deg)], plan.shape,
                          plan.origin, plan.dx, plan.span, plan.relaxation_rate, project.flow.lattice_speed,
                          project.grid.cells_per_chord, project.flow.perturbation, project.flow.seed, lead,
                          oracle_threads())
    solver = Solver(project.section, project.flow, project.grid, storage=storage)
    return solver, oracle


def ring_cells(NX, NY):
    """The engine's ring order: row y = 0, row y = NY - 1, column x = 0, column x = NX - 1."""
    xs = list(range(NX)) + list(range(NX)) + [0] * (NY - 2) + [NX - 1] * (NY - 2)
    ys = [0] * NX + [NY - 1] * NX + list(range(1, NY - 1)) * 2
    return np.array(xs), np.array(ys)


def engine_ring(solver):
    """The engine's ring populations (post-collision) as (x, y, z, 27) in ring order."""
    from aerokinetic_gb300.checkpoint import boundary_state
    _, values = boundary_state(solver._lib, solver._case)
    NX, NY, nz = solver._storage_shape
    nring = 2 * NX + 2 * (NY - 2)
    return values[1:1 + nring * nz * 27].reshape(nz, nring, 27).transpose(1, 0, 2)


def golden_project(golden):
    return Project.from_dict(golden["histories"]["exterior_down3"]["project"])


@pytest.mark.parametrize("storage", ["f64", "df64"])
def test_exterior_case_matches_oracle(golden, storage):
    """176x101x16 NACA0012 case of the reference's record: the core and the
    rebuilt ring after every 8 steps, loads and the exterior bookkeeping
    (wall mass, exterior source, reconstruction moment error) every step."""
    solver, oracle = exterior_pair(golden_project(golden), storage)
    try:
        NX, NY, nz = solver._storage_shape
        rx, ry = ring_cells(NX, NY)
        fluid = oracle.lattice.fluid[1:-1, 1:-1]
        pdf_tol = 2e-12 if storage == "f64" else 4e-12
        src_tol = 5e-12 if storage == "f64" else 2e-10
        for s in range(1, 25):
            mine = solver.step(sample=True)
            theirs = oracle.step(sample=True)
            for k in ("cl", "cd", "cm"):
                assert mine[k] == pytest.approx(theirs[k], abs=2e-10), (s, k)
            np.testing.assert_allclose(mine["element_lattice_loads"], theirs["element_lattice_loads"][:, :4],
                                       rtol=0, atol=2e-10)
            for k in ("wall_mass_exchange_lattice", "wall_mass_exchange_accumulated"):
                assert mine[k] == pytest.approx(theirs[k], abs=2e-12), (s, k)
            assert mine["exterior_source_mass_lattice"] == pytest.approx(oracle.source_last[0], abs=src_tol)
            assert mine["exterior_source_mass_accumulated"] == pytest.approx(oracle.source_total[0], abs=src_tol * s)
            report = solver.boundary_diagnostics()
            np.testing.assert_allclose(report["last_exterior_step"]["exterior_source_mass_momentum"],
                                       oracle.source_last, rtol=0, atol=src_tol)
            assert 0.0 <= report["last_exterior_step"]["reconstruction_moment_error"] < 1e-13
            if s % 8 == 0:
                core = np.abs(solver.pdf() - oracle.post_collision())[fluid].max()
                assert core <= pdf_tol * s, (s, core)
                ring = oracle.lattice.interior()[rx, ry]
                expected = O.collide(ring, oracle.omega, 1.0)
                assert np.abs(engine_ring(solver) - expected).max() <= pdf_tol * s, s
        diag, theirs = solver.diagnostics(), oracle.diagnostics()
        for k in ("local_mach_max", "density_mean", "density_error_max"):
            assert diag[k] == pytest.approx(theirs[k], rel=1e-12, abs=1e-14), k
    finally:
        solver.close()


def test_exterior_history_on_gpu(golden):
    """The reference's recorded exterior airfoil run (docs/verification_exterior_
    library_20261108/raw/matched_airfoils/airfoil_down3/history.csv): loads,
    wall mass, exterior source and guards of the first 24 samples (192 steps)."""
    from aerokinetic_gb300.solver import Solver
    record = golden["histories"]["exterior_down3"]
    project = Project.from_dict(record["project"])
    solver = Solver(project.section, project.flow, project.grid)
    try:
        assert solver.plan.shape == (176, 101, 16)
        for row in record["history"][:24]:
            loads = solver.advance(row["step"] - solver.steps, sample_last=True)
            for k in ("cl", "cd", "cm"):
                assert loads[k] == pytest.approx(row[k], abs=2e-12), (row["step"], k)
            for k in ("wall_mass_exchange_lattice", "wall_mass_exchange_accumulated"):
                assert loads[k] == pytest.approx(row[k], abs=2e-12), (row["step"], k)
            assert loads["exterior_source_mass_lattice"] == pytest.approx(row["exterior_source_mass_lattice"],
                                                                          abs=5e-12)
            # from step ~70 the start-up wave crosses the ring and the source
            # grows to O(1) per step: the running sum is held to 5e-12 a step
            assert loads["exterior_source_mass_accumulated"] == pytest.approx(
                row["exterior_source_mass_accumulated"], abs=5e-12 * row["step"])
            diag = solver.diagnostics()
            for k in ("local_mach_max", "density_error_max"):
                assert diag[k] == pytest.approx(row[k], abs=1e-12), (row["step"], k)
    finally:
        solver.close()


@pytest.mark.parametrize("storage,tol", [("f32", 5e-4), ("f16", 1e-2)])
def test_exterior_precision_forms_track_fp64(golden, storage, tol):
    """FP32 arithmetic with FP32 / FP16 shifted storage (ring arithmetic in
    FP64) against the FP64 form over 160 steps: Cl/Cd/Cm differences relative
    to max|C| below tol, and the exterior source of the same order."""
    from aerokinetic_gb300.solver import Solver
    project = golden_project(golden)
    ref = Solver(project.section, project.flow, project.grid, storage="f64")
    low = Solver(project.section, project.flow, project.grid, storage=storage)
    try:
        a, b = [], []
        for _ in range(8):
            ra = ref.advance(20, sample_last=True)
            rb = low.advance(20, sample_last=True)
            a.append([ra["cl"], ra["cd"], ra["cm"]])
            b.append([rb["cl"], rb["cd"], rb["cm"]])
        a, b = np.array(a), np.array(b)
        scale = np.abs(a).max()
        assert np.abs(a - b).max() <= tol * scale, np.abs(a - b).max() / scale
        src_a = ref.boundary_diagnostics()["exterior_source_mass_momentum_accumulated"][0]
        src_b = low.boundary_diagnostics()["exterior_source_mass_momentum_accumulated"][0]
        assert np.isfinite(src_b) and abs(src_b - src_a) <= max(abs(src_a), 1e-6)
    finally:
        ref.close()
        low.close()


def test_exterior_run_writes_boundary_bookkeeping(golden, tmp_path):
    """Solver.run in exterior mode: the history carries the wall-mass and
    exterior-source columns, metadata and summary the boundary model
    (solver.py:437-445, 519-533)."""
    import csv
    from aerokinetic_gb300.solver import Solver
    project = golden_project(golden)
    solver = Solver(project.section, project.flow, project.grid)
    try:
        dt = solver.plan.dt_convective
        summary = solver.run(48 * dt, tmp_path / "run", sample_every=8, frame_every=48, check_every=16,
                             checkpoint_every=0)
        with (tmp_path / "run" / "history.csv").open() as handle:
            rows = list(csv.DictReader(handle))
        assert len(rows) == 6 and rows[-1]["step"] == "48"
        for k in ("wall_mass_exchange_lattice", "wall_mass_exchange_accumulated", "exterior_source_mass_lattice",
                  "exterior_source_mass_accumulated"):
            assert all(r[k] != "" for r in rows), k
        record = golden["histories"]["exterior_down3"]["history"]
        for mine, theirs in zip(rows, record[:6]):
            assert float(mine["cl"]) == pytest.approx(theirs["cl"], abs=2e-12)
            assert float(mine["exterior_source_mass_accumulated"]) == pytest.approx(
                theirs["exterior_source_mass_accumulated"], abs=5e-12 * theirs["step"])
        boundary = summary["boundary_diagnostics"]
        assert boundary["model"] == "exterior_regularized_fd_v1"
        assert tuple(boundary["storage_shape"]) == (178, 103, 16)
        metadata = json.loads((tmp_path / "run" / "metadata.json").read_text())
        assert metadata["boundary_model"]["last_exterior_step"]["step"] == 48
    finally:
        solver.close()
