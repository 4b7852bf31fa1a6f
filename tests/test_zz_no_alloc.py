"""ak_step_loads_static: the loads path for callers that cannot allocate.

Some callers may not allocate device memory once they are running: a host
whose memory pool already holds the GPU's free memory, a control loop with a
fixed device budget, a plugin host that forbids allocation after start-up.
ak_step's loads path allocates its per-block partial sums on the first
sampled step; ak_step_loads_static keeps them in a static device array
instead.  These tests drive both entry points through the C ABI on two
identical cases, for each outer boundary, and check on two calls in a row
that the loads agree within the loads tolerance of the parity tests (2e-10)
and that the static path leaves the device's free memory unchanged; and that
a case needing more partial sums than the array holds is rejected before
anything runs, leaving its populations, boundary history and step count as
they were.  The file is collected last.
"""
import ctypes

import numpy as np
import pytest

from aerokinetic_gb300 import Contour, Flow, Grid, Section, naca0012

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

STATIC_DOUBLES = 131072  # the static array's capacity in doubles


def make_solver(farfield, section=None, grid=None, storage="f64"):
    from aerokinetic_gb300.solver import Solver
    section = section or Section((naca0012(81),), 1., (.25, 0))
    grid = grid or Grid(cells_per_chord=32, upstream_chords=1.5, downstream_chords=3, transverse_chords=1.5,
                        span_chords=.5, memory_limit_gib=2, farfield=farfield)
    return Solver(section, Flow(reynolds=30000, alpha_deg=4), grid, storage=storage)


@pytest.fixture(autouse=True)
def _needs_device():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.mark.parametrize("farfield", ["characteristic_transport_v1", "legacy", "exterior_regularized_fd_v1"])
def test_static_scratch_loads_match_the_allocating_path(farfield):
    from aerokinetic_gb300 import _native
    lib = _native.load()
    a, b = make_solver(farfield), make_solver(farfield)
    try:
        n = len(a.contours)
        for call in range(2):
            la, lb = np.zeros((n, 5)), np.zeros((n, 5))
            _native.check(lib.ak_step(a._case, 16, la.ctypes.data_as(ctypes.c_void_p)))
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
            _native.check(lib.ak_step_loads_static(b._case, 16, lb.ctypes.data_as(ctypes.c_void_p)))
            torch.cuda.synchronize()
            assert torch.cuda.mem_get_info()[0] == free_before, "the static path allocated device memory"
            assert np.all(np.isfinite(lb)) and np.abs(lb[:, :2]).max() > 0
            np.testing.assert_allclose(lb, la, rtol=0, atol=2e-10, err_msg=f"call {call}")
        assert lib.ak_steps_done(a._case) == lib.ak_steps_done(b._case) == 32
        assert lib.ak_step_loads_static(b._case, 1, None) == _native.AK_ERR_INVALID
    finally:
        a.close()
        b.close()


def test_over_capacity_case_is_rejected_before_any_launch():
    """Eight short NACA0012 elements over a long span: more wall links than
    the static array's partial sums cover.  The rejected call must not touch
    the case: same populations, same characteristic-farfield history, same
    step count; ak_step then continues it normally."""
    from aerokinetic_gb300 import _native
    from aerokinetic_gb300.checkpoint import boundary_state
    lib = _native.load()
    base = naca0012(41).xy
    section = Section(tuple(Contour(base + [0.0, 0.6 * k], f"e{k}") for k in range(8)), 1.0, (0.25, 2.1))
    grid = Grid(cells_per_chord=16, upstream_chords=0.5, downstream_chords=1.0, transverse_chords=0.5,
                span_chords=32.0, memory_limit_gib=8, farfield="characteristic_transport_v1")
    solver = make_solver(None, section, grid, storage="f32")
    try:
        n = len(solver.contours)
        needed = -(-solver.info["wall_links"] // 256) * 5 * n
        assert needed > STATIC_DOUBLES, "the case must exceed the static array"
        solver.advance(3)  # a boundary history that the rejected call must keep
        torch.cuda.synchronize()
        pdf0, (rows0, values0) = solver.pdf(), boundary_state(lib, solver._case)
        steps0 = lib.ak_steps_done(solver._case)
        loads = np.zeros((n, 5))
        code = lib.ak_step_loads_static(solver._case, 2, loads.ctypes.data_as(ctypes.c_void_p))
        assert code == _native.AK_ERR_INVALID
        assert b"static scratch" in lib.ak_last_error()
        torch.cuda.synchronize()
        assert lib.ak_steps_done(solver._case) == steps0
        rows1, values1 = boundary_state(lib, solver._case)
        assert np.array_equal(rows0, rows1) and np.array_equal(values0, values1)
        assert np.array_equal(solver.pdf(), pdf0)
        record = solver.advance(2, sample_last=True)
        assert np.isfinite(record["cl"]) and lib.ak_steps_done(solver._case) == steps0 + 2
    finally:
        solver.close()
