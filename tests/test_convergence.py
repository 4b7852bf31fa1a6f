"""Stationarity residuals on the device and the run loops' stop criteria
(convergence.py:20-176)."""
import csv
import math

import numpy as np
import pytest

from aerokinetic_gb300 import Flow, Grid, Section, StopCriteria, naca4


def _parts():
    section = Section((naca4("0012", 41),))
    flow = Flow(reynolds=2e4, alpha_deg=6.0, lattice_speed=0.05, seed=11)
    grid = Grid(cells_per_chord=16, upstream_chords=2.0, downstream_chords=3.0, transverse_chords=1.5,
                span_chords=0.25, farfield="characteristic_transport_v1", memory_limit_gib=8)
    return section, flow, grid


def test_stop_criteria_thresholds_and_validation():
    criteria = StopCriteria(mode="steady", mass_tolerance=1e-3, momentum_y_tolerance=2e-3)
    assert criteria.thresholds == (1e-3, 1e-5, 2e-3, 1e-5)
    with pytest.raises(ValueError):
        StopCriteria(mode="forever")


@pytest.mark.gpu
def test_device_residuals_match_host_differences(tmp_path):
    """L2 and Linf of d(rho, j/U)/dt* from the device snapshot equal the same
    norms computed from two host copies of the populations."""
    from aerokinetic_gb300.convergence import RunControl
    from aerokinetic_gb300.project import RunSettings
    from aerokinetic_gb300.solver import Solver
    solver = Solver(*_parts())
    try:
        solver.advance(5)
        control = RunControl(solver, RunSettings(), tmp_path)
        before = solver.pdf()
        solver.advance(7)
        after = solver.pdf()
        record = control.observe()
        control.close()
        c = np.array([[0, 0, 0], [0, 1, 0], [0, -1, 0], [-1, 0, 0], [1, 0, 0], [0, 0, 1], [0, 0, -1], [-1, 1, 0],
                      [1, 1, 0], [-1, -1, 0], [1, -1, 0], [0, 1, 1], [0, -1, 1], [-1, 0, 1], [1, 0, 1], [0, 1, -1],
                      [0, -1, -1], [-1, 0, -1], [1, 0, -1], [1, 1, 1], [-1, 1, 1], [1, -1, 1], [-1, -1, 1],
                      [1, 1, -1], [-1, 1, -1], [1, -1, -1], [-1, -1, -1]], dtype=float)
        fluid = solver._fluid

        def sample(pdf):
            q = np.empty(pdf.shape[:-1] + (4,))
            q[..., 0] = pdf.sum(axis=-1) + 1
            q[..., 1:] = pdf @ c / solver.flow.lattice_speed
            return q[fluid]
        d = (sample(after) - sample(before)) / (7 * solver.plan.dt_convective)
        l2 = np.sqrt((d * d).sum(axis=0) / len(d))
        linf = np.abs(d).max(axis=0)
        for k, name in enumerate(("rho", "jx", "jy", "jz")):
            assert record[f"l2_{name}"] == pytest.approx(float(l2[k]), rel=1e-10)
            assert record[f"linf_{name}"] == pytest.approx(float(linf[k]), rel=1e-10)
    finally:
        solver.close()


@pytest.mark.gpu
def test_run_stops_on_steady_residuals_and_max_steps(tmp_path):
    from aerokinetic_gb300.solver import Solver
    solver = Solver(*_parts())
    try:
        steady = StopCriteria(mode="steady", mass_tolerance=1e9, momentum_x_tolerance=1e9, momentum_y_tolerance=1e9,
                              momentum_z_tolerance=1e9, minimum_t_star=0.0, consecutive_checks=3)
        summary = solver.run(200 * solver.plan.dt_convective, tmp_path / "steady", sample_every=5, check_every=10,
                             frame_every=100, checkpoint_every=0, termination=steady)
        assert summary["termination_reason"] == "residual_targets_met" and summary["steps"] == 30
        assert summary["steady_residual_criterion_met"] and summary["status"] == "completed"
        with (tmp_path / "steady" / "residuals.csv").open(newline="") as handle:
            rows = list(csv.DictReader(handle))
        assert [int(r["step"]) for r in rows] == [10, 20, 30] and rows[-1]["streak"] == "3"
        assert all(math.isfinite(float(r["l2_jx"])) and float(r["l2_jx"]) > 0 for r in rows)
    finally:
        solver.close()
    solver = Solver(*_parts())
    try:
        summary = solver.run(200 * solver.plan.dt_convective, tmp_path / "limit", sample_every=5, check_every=10,
                             frame_every=100, checkpoint_every=0, termination=StopCriteria(max_steps=23))
        assert summary["termination_reason"] == "max_steps_reached" and summary["steps"] == 23
    finally:
        solver.close()
