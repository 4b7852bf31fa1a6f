"""sgs="smagorinsky" (solver.py:74-77) on the GPU against the oracle and the reference's record.

The bulk collision takes each cell's Smagorinsky shear rate from its
non-equilibrium second moments; the walls, outer boundaries and loads are
unchanged.  Bars as for molecular viscosity: populations within 2e-12 per
step and loads within 2e-10 of the oracle; the reference's recorded run
(demo_wake, written by its 0.1.0 release) within its 2e-10 load gate.
"""
import dataclasses

import numpy as np
import pytest

from aerokinetic_gb300.project import Project
from tests.test_gpu_parity import compare_run, kat_project, solver_for

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _needs_device():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def with_sgs(project, constant=0.1):
    flow = dataclasses.replace(project.flow, sgs="smagorinsky", smagorinsky_constant=constant)
    return dataclasses.replace(project, flow=flow)


def wake_project(golden):
    return Project.from_dict(golden["histories"]["smagorinsky_wake"]["project"])


@pytest.mark.parametrize("storage", ["f64", "df64"])
def test_smagorinsky_wake_case_matches_oracle(golden, storage):
    """The recorded wake case (176x102x16, legacy outer boundary, C = 0.1) over
    40 steps in the plain and the df64 forms."""
    compare_run(wake_project(golden), steps=40, sample_every=8, storage=storage)


def test_smagorinsky_characteristic_case_matches_oracle():
    """The characteristic farfield with C = 0.2, where the subgrid rate departs
    furthest from the molecular one."""
    compare_run(with_sgs(kat_project("characteristic_transport_v1"), 0.2), steps=40, sample_every=8)


def test_smagorinsky_history_on_gpu(golden):
    """demo_wake/history.csv: Cl/Cd/Cm of the first 12 samples (480 steps)."""
    record = golden["histories"]["smagorinsky_wake"]
    solver = solver_for(Project.from_dict(record["project"]))
    try:
        for row in record["history"][:12]:
            loads = solver.advance(row["step"] - solver.steps, sample_last=True)
            for k in ("cl", "cd", "cm"):
                assert loads[k] == pytest.approx(row[k], abs=2e-10), (row["step"], k)
    finally:
        solver.close()


@pytest.mark.parametrize("storage,tol", [("f32", 5e-4), ("f16", 1e-2)])
def test_smagorinsky_precision_forms_track_fp64(golden, storage, tol):
    """FP32 arithmetic (FP32 / FP16 storage) with the subgrid rate against the
    FP64 form over 200 steps of the wake case: Cl/Cd/Cm relative to max|C|."""
    project = wake_project(golden)
    ref, low = solver_for(project, "f64"), solver_for(project, storage)
    try:
        a, b = [], []
        for _ in range(10):
            ra, rb = ref.advance(20, sample_last=True), low.advance(20, sample_last=True)
            a.append([ra["cl"], ra["cd"], ra["cm"]])
            b.append([rb["cl"], rb["cd"], rb["cm"]])
        a, b = np.array(a), np.array(b)
        assert np.abs(a - b).max() <= tol * np.abs(a).max(), np.abs(a - b).max() / np.abs(a).max()
    finally:
        ref.close()
        low.close()


def test_smagorinsky_is_rejected_where_the_reference_rejects_it(golden):
    """Exterior and refined cases keep molecular viscosity (config.py:147-148,
    refined_solver.py:61-62)."""
    from aerokinetic_gb300.config import Grid
    project = wake_project(golden)
    grid = dataclasses.replace(project.grid, farfield="exterior_regularized_fd_v1")
    with pytest.raises(ValueError, match="sgs=none"):
        solver_for(dataclasses.replace(project, grid=grid))
    assert isinstance(grid, Grid)
