"""ak_step_loads_static: the loads path for callers that cannot allocate.

Some callers may not allocate device memory once they are running: a host
thread that is capturing a CUDA graph, a control loop with a fixed device
budget, a plugin host that forbids allocation after start-up.  ak_step's loads
path allocates its per-block partial sums on the first sampled step;
ak_step_loads_static keeps them in a static device array instead.  This test
drives both entry points through the C ABI on two identical cases and checks,
on two calls in a row, that the loads agree within the loads tolerance of the
parity tests (2e-10) and that the static path leaves the device's free memory
unchanged.  It lives in its own file, collected last.
"""
import ctypes

import numpy as np
import pytest

from aerokinetic_gb300 import Flow, Grid, Section, naca0012

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def make_solver():
    from aerokinetic_gb300.solver import Solver
    return Solver(Section((naca0012(81),), 1., (.25, 0)), Flow(reynolds=30000, alpha_deg=4),
                  Grid(cells_per_chord=32, upstream_chords=1.5, downstream_chords=3, transverse_chords=1.5,
                       span_chords=.5, memory_limit_gib=2, farfield="characteristic_transport_v1"))


def test_static_scratch_loads_match_the_allocating_path():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from aerokinetic_gb300 import _native
    lib = _native.load()
    a, b = make_solver(), make_solver()
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
        code = lib.ak_step_loads_static(b._case, 1, None)
        assert code == _native.AK_ERR_INVALID
    finally:
        a.close()
        b.close()
