"""Batches of independent uniform cases (ak_batch_*): same bits alone and in a mix."""
import numpy as np
import pytest

from aerokinetic_gb300 import Flow, Grid, Section, naca4


def _parts(chord, alpha, reynolds, seed, farfield="characteristic_transport_v1", sgs="none"):
    section = Section((naca4("0012", 41),))
    flow = Flow(reynolds=reynolds, alpha_deg=alpha, lattice_speed=0.05, seed=seed, sgs=sgs)
    grid = Grid(cells_per_chord=chord, upstream_chords=2.0, downstream_chords=3.0, transverse_chords=1.5,
                span_chords=0.25, farfield=farfield, memory_limit_gib=8)
    return section, flow, grid


CASES = [(16, 4.0, 2e4, 1), (24, -2.0, 5e4, 2), (16, 10.0, 1e4, 3), (20, 6.0, 3e4, 4)]
# the same with two cases on the legacy outer boundary (UBB + outflow)
MIXED_BOUNDARIES = [(16, 4.0, 2e4, 1, "legacy"), (24, -2.0, 5e4, 2), (16, 10.0, 1e4, 3, "legacy"), (20, 6.0, 3e4, 4)]


def _solvers(storage, cases=CASES):
    from aerokinetic_gb300.solver import Solver
    return [Solver(*_parts(*c), storage=storage) for c in cases]


@pytest.mark.gpu
@pytest.mark.parametrize("storage,cases", [("f64", CASES), ("f16", CASES), ("f32", MIXED_BOUNDARIES),
                                           ("f64", MIXED_BOUNDARIES), ("f16", MIXED_BOUNDARIES)])
def test_batch_matches_cases_stepped_alone(storage, cases):
    """Every case of a mixed-size batch (characteristic and legacy outer
    boundaries) ends bit-identical to the same case stepped alone, and its
    sampled loads are the same numbers."""
    from aerokinetic_gb300.batch import Batch
    alone, mixed = _solvers(storage, cases), _solvers(storage, cases)
    try:
        with Batch(mixed) as batch:
            for chunk in (7, 1, 12):
                records = batch.advance(chunk)
                for solver, record in zip(alone, records):
                    ref = solver.advance(chunk, sample_last=True)
                    for key in ("cl", "cd", "cm", "step"):
                        assert record[key] == ref[key], key
            batch.advance(5, sample_last=False)
            for solver in alone:
                solver.advance(5)
            assert batch.launches >= 4 * 25
        for a, b in zip(alone, mixed):
            assert a.steps == b.steps == 25
            assert np.array_equal(a.pdf(), b.pdf())
            assert a.diagnostics() == b.diagnostics()
    finally:
        for s in alone + mixed:
            s.close()


@pytest.mark.gpu
def test_batch_mixes_subgrid_and_molecular_cases():
    """Cases with sgs="smagorinsky" keep their own subgrid rate inside a batch
    beside molecular-viscosity cases: each ends bit-identical to itself alone."""
    from aerokinetic_gb300.batch import Batch
    from aerokinetic_gb300.solver import Solver
    specs = [(16, 4.0, 2e4, 1, "characteristic_transport_v1", "smagorinsky"), (20, 6.0, 3e4, 4),
             (24, -2.0, 5e4, 2, "characteristic_transport_v1", "smagorinsky")]
    alone = [Solver(*_parts(*c), storage="f32") for c in specs]
    mixed = [Solver(*_parts(*c), storage="f32") for c in specs]
    plain = Solver(*_parts(*specs[0][:4]), storage="f32")
    try:
        with Batch(mixed) as batch:
            records = batch.advance(12)
        for solver, record in zip(alone, records):
            assert solver.advance(12, sample_last=True)["cl"] == record["cl"]
        for a, b in zip(alone, mixed):
            assert np.array_equal(a.pdf(), b.pdf())
        plain.advance(12)
        assert not np.array_equal(plain.pdf(), alone[0].pdf())
    finally:
        for s in alone + mixed + [plain]:
            s.close()


@pytest.mark.gpu
def test_batch_tuning_leaves_the_state_unchanged():
    from aerokinetic_gb300.batch import Batch
    alone, mixed = _solvers("f32"), _solvers("f32")
    try:
        with Batch(mixed) as batch:
            batch.advance(3, sample_last=False)
            schedule = batch.tune(trials=2)
            assert schedule["block_width"] in (64, 128, 256) and schedule["ctas_per_sm"] >= 1
            batch.advance(4, sample_last=False)
        for solver in alone:
            solver.advance(7)
        for a, b in zip(alone, mixed):
            assert np.array_equal(a.pdf(), b.pdf())
    finally:
        for s in alone + mixed:
            s.close()


@pytest.mark.gpu
def test_batch_rejects_what_it_cannot_run():
    from aerokinetic_gb300 import _native
    from aerokinetic_gb300.batch import Batch
    from aerokinetic_gb300.solver import Solver
    exterior = Solver(*_parts(16, 4.0, 2e4, 1, farfield="exterior_regularized_fd_v1"))
    a, b = _solvers("f64", CASES[:1])[0], _solvers("f32", CASES[1:2])[0]
    try:
        with pytest.raises(ValueError, match="outer boundary"):
            Batch([exterior])
        with pytest.raises(ValueError, match="storage"):
            Batch([a, b])
        with pytest.raises(ValueError, match="twice"):
            Batch([a, a])
        with Batch([a]) as batch:
            batch.advance(2, sample_last=False)
            a.advance(1)  # stepped outside the batch
            with pytest.raises(ValueError, match="outside"):
                batch.advance(1)
        assert isinstance(_native.load().ak_batch_launches(None), int)
    finally:
        for s in (exterior, a, b):
            s.close()
