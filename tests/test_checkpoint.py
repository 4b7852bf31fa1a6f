"""Checkpoints continue the same timeline bit for bit; resume_run finishes an
interrupted run with the history an uninterrupted run writes."""
import csv
import json

import numpy as np
import pytest

from aerokinetic_gb300 import Flow, Grid, Section, naca4


def _parts(farfield, chord=16):
    section = Section((naca4("0012", 41),))
    flow = Flow(reynolds=2e4, alpha_deg=6.0, lattice_speed=0.05, seed=11)
    grid = Grid(cells_per_chord=chord, upstream_chords=2.0, downstream_chords=3.0, transverse_chords=1.5,
                span_chords=0.25, farfield=farfield, memory_limit_gib=8)
    return section, flow, grid


def test_checkpoint_files_are_validated(tmp_path):
    from aerokinetic_gb300.checkpoint import FORMAT, restore_checkpoint
    path = tmp_path / "bad.npz"
    np.savez(path, metadata=np.asarray(json.dumps({"format": "other"})))
    with pytest.raises(ValueError, match="checkpoint"):
        restore_checkpoint(object, path)
    meta = {"format": FORMAT, "schema_version": 1, "kind": "uniform", "steps": 3,
            "array_sha256": {"pdf": "0" * 64}}
    np.savez(path, metadata=np.asarray(json.dumps(meta)), pdf=np.zeros(3))
    with pytest.raises(ValueError, match="checksum"):
        restore_checkpoint(object, path)


@pytest.mark.gpu
@pytest.mark.parametrize("farfield,storage", [("characteristic_transport_v1", "f64"), ("legacy", "f64"),
                                              ("characteristic_transport_v1", "f16"),
                                              ("exterior_regularized_fd_v1", "f64"),
                                              ("exterior_regularized_fd_v1", "f16")])
def test_uniform_checkpoint_continues_bit_for_bit(tmp_path, farfield, storage):
    from aerokinetic_gb300.solver import Solver
    straight = Solver(*_parts(farfield), storage=storage)
    split = Solver(*_parts(farfield), storage=storage)
    try:
        ref = straight.advance(20, sample_last=True)
        split.advance(9)
        split.save_checkpoint(tmp_path / "c.npz", {"note": "mid-run"})
        restored = Solver.from_checkpoint(tmp_path / "c.npz")
        try:
            assert restored.steps == 9 and restored._checkpoint_context == {"note": "mid-run"}
            got = restored.advance(11, sample_last=True)
            assert (got["cl"], got["cd"], got["cm"], got["step"]) == (ref["cl"], ref["cd"], ref["cm"], ref["step"])
            # solid cells hold no state the fluid reads (every slot a fluid
            # cell pulls from a solid cell is rewritten by the walls first)
            fluid = ~straight._solid_xy
            assert np.array_equal(restored.pdf()[fluid], straight.pdf()[fluid])
            if farfield == "exterior_regularized_fd_v1":
                # the ring, its band state and the running sums continue too
                for k in ("wall_mass_exchange_accumulated", "exterior_source_mass_accumulated"):
                    assert got[k] == ref[k], k
                assert restored.boundary_diagnostics() == straight.boundary_diagnostics()
        finally:
            restored.close()
    finally:
        straight.close()
        split.close()


@pytest.mark.gpu
def test_refined_checkpoint_continues_bit_for_bit(golden, tmp_path):
    from aerokinetic_gb300.refined import RefinedSolver
    from aerokinetic_gb300.refined_plan import load_refined_project
    project, refinement = load_refined_project(golden["histories"]["refined_startup"]["project"])
    straight, split = RefinedSolver(project, refinement), RefinedSolver(project, refinement)
    try:
        for _ in range(6):
            straight.step()
        for _ in range(3):
            split.step()
        split.save_checkpoint(tmp_path / "r.npz")
        restored = RefinedSolver.from_checkpoint(tmp_path / "r.npz")
        try:
            assert restored.steps == 3 and restored.last_budget == split.last_budget
            for _ in range(3):
                got = restored.step()
            assert got == straight.last_loads
            (ca, fa), (cb, fb) = restored.states(), straight.states()
            assert np.array_equal(ca, cb)
            fluid = ~straight._fine_solid_xy()
            assert np.array_equal(fa[fluid], fb[fluid])
            assert restored.last_budget == straight.last_budget
            assert restored.cumulative_wall_mass_exchange == straight.cumulative_wall_mass_exchange
            assert np.array_equal(restored.cumulative_external_in, straight.cumulative_external_in)
        finally:
            restored.close()
    finally:
        straight.close()
        split.close()


@pytest.mark.gpu
def test_resume_run_finishes_the_same_history(tmp_path):
    from aerokinetic_gb300.solver import Solver
    kwargs = dict(sample_every=5, frame_every=40, check_every=10, checkpoint_every=20)
    whole = Solver(*_parts("characteristic_transport_v1"))
    duration = 60 * whole.plan.dt_convective
    try:
        summary = whole.run(duration, tmp_path / "whole", **kwargs)
        assert summary["status"] == "completed" and summary["steps"] == 60
    finally:
        whole.close()
    first = Solver(*_parts("characteristic_transport_v1"))
    try:
        # stopped after the sample at step 35 (checkpoints at 20 and at the stop)
        stopped = first.run(duration, tmp_path / "split", callback=lambda s, r: r["step"] < 35, **kwargs)
        assert stopped["status"] == "stopped"
    finally:
        first.close()
    resumed = Solver.resume_run(tmp_path / "split")
    assert resumed["status"] == "completed" and resumed["steps"] == 60

    def rows(path):
        with (path / "history.csv").open(newline="") as handle:
            return [{k: r[k] for k in ("step", "cl", "cd", "cm")} for r in csv.DictReader(handle)]
    assert rows(tmp_path / "split") == rows(tmp_path / "whole")
    meta = json.loads((tmp_path / "split" / "metadata.json").read_text())
    assert meta["status"] == "completed" and meta["start_step"] == 0
    with pytest.raises(ValueError, match="already completed"):
        Solver.resume_run(tmp_path / "split")
