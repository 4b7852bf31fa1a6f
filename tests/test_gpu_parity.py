"""Parity of the sm_103a engine with the CPU oracle and the reference's records.

Bars (the reference's own implementation gates, tools/research_tests/
study_protocol.json:37-40): populations within 2e-12 per step and loads within
2e-10 over tens of steps; flags, cut links and Bouzidi fractions bit-exact.
The reduced-precision forms are compared with the FP64 engine and their
errors bounded explicitly.
"""
import numpy as np
import pytest

from aerokinetic_gb300.config import Flow, Grid, Plan
from aerokinetic_gb300.geometry import Contour, Section, naca0012
from aerokinetic_gb300.project import Project
from tests.conftest import oracle_threads

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

O = pytest.importorskip("oracle.oracle")


@pytest.fixture(scope="module", autouse=True)
def _needs_device():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def solver_for(project, storage="f64"):
    from aerokinetic_gb300.solver import Solver
    return Solver(project.section, project.flow, project.grid, storage=storage)


def oracle_for(project):
    plan = Plan.create(project.section, project.flow, project.grid)
    contours = [c.xy for c in project.section.normalized(project.flow.alpha_deg)]
    lead = O.leading_edge([e.xy for e in project.section.elements], project.section.moment_reference,
                          project.section.chord, project.flow.alpha_deg)
    smagorinsky = project.flow.smagorinsky_constant if project.flow.sgs == "smagorinsky" else 0.0
    return O.AirfoilCase(contours, plan.shape, plan.origin, plan.dx, plan.span, plan.relaxation_rate,
                         project.flow.lattice_speed, project.grid.cells_per_chord, project.grid.farfield,
                         project.flow.perturbation, project.flow.seed, lead, oracle_threads(),
                         smagorinsky=smagorinsky)


def kat_project(farfield="legacy"):
    return Project(Section((naca0012(81),), 1., (.25, 0)), Flow(reynolds=30000, alpha_deg=4, physical_chord_m=.15),
                   Grid(cells_per_chord=32, upstream_chords=1.5, downstream_chords=3, transverse_chords=1.5,
                        span_chords=.5, memory_limit_gib=2, farfield=farfield))


def geometry_project(fixture):
    s = fixture["section"]
    elements = tuple(Contour(np.array(xy), name) for xy, name in zip(s["elements"], s["names"]))
    return Project(Section(elements, s["chord"], tuple(s["moment_reference"])), Flow(**fixture["flow"]),
                   Grid(**fixture["grid"]))


@pytest.mark.parametrize("name", ["kat272", "uniform_c1", "failure_capture_n16", "two_element"])
def test_flags_links_and_fractions_bit_exact(golden, name):
    fixture = golden["geometry"][name]
    solver = solver_for(geometry_project(fixture))
    try:
        assert list(solver.plan.shape) == fixture["plan"]["shape"]
        flags = solver._solid_xy.astype(int)
        ref = (np.array(fixture["solid_xy"]) != 0).astype(int)
        assert np.array_equal(flags, ref)
        rows, q = solver.wall_links()
        c = O.stencil()[0]
        mine = {(int(e), int(x), int(y), int(c[d][0]), int(c[d][1])): qq for (e, x, y, d), qq in zip(rows, q)}
        theirs = {tuple(r[:5]): r[5] for r in fixture["wall_links_2d"]}
        assert mine.keys() == theirs.keys()
        assert all(mine[k] == theirs[k] for k in theirs)  # exact equality of doubles
        assert solver.wall_fallback_links == 3 * solver.plan.shape[2] * fixture["wall_fallback_links_2d"]
    finally:
        solver.close()


def compare_run(project, steps, sample_every, pdf_tol=2e-12, load_tol=2e-10, storage="f64"):
    solver, oracle = solver_for(project, storage), oracle_for(project)
    try:
        # df64 storage holds 48 bits: ~2^-48 of a population near its rest weight
        np.testing.assert_allclose(solver.pdf(), oracle.lattice.interior(), rtol=0,
                                   atol=1e-15 if storage == "f64" else 5e-15)
        fluid = oracle.lattice.fluid
        worst = 0.0
        for s in range(1, steps + 1):
            sample = s % sample_every == 0
            mine = solver.step(sample)
            theirs = oracle.step(sample)
            if sample:
                for k in ("cl", "cd", "cm"):
                    assert mine[k] == pytest.approx(theirs[k], abs=load_tol), (s, k)
                np.testing.assert_allclose(mine["element_lattice_loads"], theirs["element_lattice_loads"][:, :4],
                                           rtol=0, atol=load_tol)
            if s % max(1, steps // 4) == 0 or s == steps:
                diff = np.abs(solver.pdf() - oracle.lattice.interior())[fluid].max()
                worst = max(worst, diff)
                assert diff <= pdf_tol * s, (s, diff)
        return worst
    finally:
        solver.close()


@pytest.mark.parametrize("farfield,storage", [("characteristic_transport_v1", "f64"), ("legacy", "f16"),
                                              ("characteristic_transport_v1", "f32")])
def test_graph_replayed_steps_equal_eager_steps(farfield, storage):
    """ak_step replays captured graphs (walls beside the outer boundary);
    ak_step_timed runs the same kernels eagerly in one stream: same bits,
    including after the loads' partial sums move (diagnostics in between)."""
    import ctypes
    project = kat_project(farfield)
    graphed, eager = solver_for(project, storage), solver_for(project, storage)
    try:
        ms = np.zeros(4)
        for chunk in (1, 5, 3):
            loads = graphed.advance(chunk, sample_last=True)
            graphed.diagnostics()
            for _ in range(chunk):
                assert eager._lib.ak_step_timed(eager._case, 1, ms.ctypes.data_as(ctypes.c_void_p)) == 0
            eager.steps += chunk
        assert np.array_equal(graphed.pdf(), eager.pdf())
        ref = eager.step(sample=True)
        got = graphed.step(sample=True)
        assert (got["cl"], got["cd"], got["cm"]) == (ref["cl"], ref["cd"], ref["cm"])
        assert loads["step"] == 9
    finally:
        graphed.close()
        eager.close()


def test_legacy_case_matches_oracle():
    compare_run(kat_project("legacy"), steps=40, sample_every=8)


def test_characteristic_case_matches_oracle():
    compare_run(kat_project("characteristic_transport_v1"), steps=40, sample_every=8)


@pytest.mark.parametrize("farfield", ["legacy", "characteristic_transport_v1"])
def test_df64_form_meets_the_plain_tolerances(farfield):
    """The df64 form (FP64-sized storage, double-float collision, FP64
    boundaries) against the FP64 oracle at the plain form's own bars:
    2e-12 per population per step and 2e-10 on the loads."""
    compare_run(kat_project(farfield), steps=40, sample_every=8, storage="df64")


def test_df64_known_answer_272_steps(golden):
    kat = golden["kat272"]
    solver = solver_for(kat_project("legacy"), "df64")
    try:
        solver.advance(kat["steps"] - 1)
        loads = solver.step(sample=True)
        for k, v in kat["last_sample"].items():
            assert loads[k] == pytest.approx(v, rel=1e-10)
    finally:
        solver.close()


def test_known_answer_272_steps_on_gpu(golden):
    kat = golden["kat272"]
    solver = solver_for(kat_project("legacy"))
    try:
        solver.advance(kat["steps"] - 1)
        loads = solver.step(sample=True)
        for k, v in kat["last_sample"].items():
            assert loads[k] == pytest.approx(v, rel=2e-12)
    finally:
        solver.close()


def test_characteristic_history_on_gpu(golden):
    record = golden["histories"]["characteristic_down3"]
    solver = solver_for(Project.from_dict(record["project"]))
    try:
        for row in record["history"][:40]:
            loads = solver.advance(row["step"] - solver.steps, sample_last=True)
            for k in ("cl", "cd", "cm"):
                assert loads[k] == pytest.approx(row[k], abs=2e-12)
            diag = solver.diagnostics()
            assert diag["local_mach_max"] == pytest.approx(row["local_mach_max"], rel=1e-12)
            assert diag["density_error_max"] == pytest.approx(row["density_error_max"], rel=1e-12)
    finally:
        solver.close()


def test_failure_capture_guard_and_loads(golden):
    """docs/verification_failure_capture_20261107: colliding density pulses; the
    engine reproduces loads and guards, then raises like the reference."""
    from aerokinetic_gb300.solver import NumericalFailure
    record = golden["histories"]["failure_capture_n16"]
    solver = solver_for(Project.from_dict(record["project"]))
    try:
        nx, ny, nz = solver.plan.shape
        y = np.arange(ny) + 0.5
        a = .085 * np.exp(-.5 * ((y - 5.5) / 1.5) ** 2)
        b = .085 * np.exp(-.5 * ((y - 12.5) / 1.5) ** 2)
        u = np.zeros((nx, ny, nz, 3))
        u[..., 0] = solver.flow.lattice_speed
        u[..., 1] = (np.sqrt(1 / 3) * (a - b))[None, :, None]
        u[solver._solid_xy] = 0.0
        solver.set_fields(np.broadcast_to((1 + a + b)[None, :, None], solver.plan.shape), u)
        for row in record["history"]:
            loads = solver.step(sample=True)
            diag = solver.diagnostics()
            for k in ("cl", "cd", "cm"):
                assert loads[k] == pytest.approx(row[k], rel=1e-12, abs=1e-13)
            assert diag["local_mach_max"] == pytest.approx(row["local_mach_max"], rel=1e-12)
        with pytest.raises(NumericalFailure):
            for _ in range(20):
                solver.step()
                solver.diagnostics()
    finally:
        solver.close()


def test_full_size_uniform_case_matches_oracle(golden):
    """384x256x8 characteristic-farfield case at lattice Mach 0.1 (the uniform
    bench workload) over 64 steps, loads every 8."""
    compare_run(geometry_project(golden["geometry"]["uniform_c1"]), steps=64, sample_every=8)


def test_non_finite_state_is_reported(golden):
    """A host-made fault: NaN populations written through the ABI."""
    from aerokinetic_gb300.solver import NumericalFailure
    solver = solver_for(kat_project("legacy"))
    try:
        pdf = solver.pdf()
        pdf[40, 40, 3, 5] = np.nan
        solver.set_pdf(pdf)
        with pytest.raises(NumericalFailure):
            solver.diagnostics()
    finally:
        solver.close()


@pytest.mark.parametrize("storage,inst_tol,mean_tol", [("f32", 5e-4, 5e-4), ("f16", 5e-3, 5e-3)])
def test_precision_forms_track_fp64(storage, inst_tol, mean_tol):
    """FP32 arithmetic with FP32 / FP16 shifted storage against the FP64 form on
    the impulsive start (steps 20..200, every 20): the largest instantaneous
    Cl/Cd/Cm difference relative to max|C| stays below inst_tol, the
    difference of the sample means below mean_tol."""
    project = kat_project("characteristic_transport_v1")
    ref, low = solver_for(project, "f64"), solver_for(project, storage)
    try:
        a, b = [], []
        for _ in range(10):
            ra = ref.advance(20, sample_last=True)
            rb = low.advance(20, sample_last=True)
            a.append([ra["cl"], ra["cd"], ra["cm"]])
            b.append([rb["cl"], rb["cd"], rb["cm"]])
        a, b = np.array(a), np.array(b)
        scale = np.abs(a).max()
        assert np.abs(a - b).max() <= inst_tol * scale, np.abs(a - b).max() / scale
        assert np.abs(a.mean(axis=0) - b.mean(axis=0)).max() <= mean_tol * scale
        rho_a, _ = ref.macros()
        rho_b, _ = low.macros()
        fluid = ~ref._solid_xy
        assert np.abs(rho_a - rho_b)[fluid].max() < 2e-2 * np.abs(rho_a - 1)[fluid].max()
    finally:
        ref.close()
        low.close()


# ---------------------------------------------------------------- two levels
def refined_pair(record, steps_needed=0, storage="f64"):
    from aerokinetic_gb300.refined import RefinedSolver
    from aerokinetic_gb300.refined_plan import load_refined_project
    from oracle.refined import RefinedCase
    project, refinement = load_refined_project(record["project"])
    solver = RefinedSolver(project, refinement, storage=storage)
    plan = solver.plan
    sec, flow = project.section, project.flow
    lead = O.leading_edge([e.xy for e in sec.elements], sec.moment_reference, sec.chord, flow.alpha_deg)
    oracle = RefinedCase([c.xy for c in sec.normalized(flow.alpha_deg)], plan.shape, plan.origin,
                         plan.coarse_level.dx, plan.coarse_level.dt, plan.coarse_level.tau_shear,
                         plan.coarse_level.tau_bulk, plan.box.lower, plan.box.upper, flow.lattice_speed,
                         flow.perturbation, flow.seed, lead, plan.span, oracle_threads())
    return solver, oracle


@pytest.mark.parametrize("storage", ["f64", "df64"])
def test_refined_levels_match_oracle(golden, storage):
    """Both levels' populations and the loads after each of 3 coarse steps, in
    the plain form and the df64 form, at the plain form's tolerances."""
    solver, oracle = refined_pair(golden["histories"]["refined_startup"], storage=storage)
    try:
        compare_refined(solver, oracle, steps=3)
    finally:
        solver.close()


def compare_refined(solver, oracle, steps, pdf_tol=2e-12, load_tol=2e-10):
    """states() (the pre-collision populations of both levels, the reference's
    contract) against the oracle's state on every coarse cell and every fine
    fluid cell after each coarse step, the loads of each step, and the held
    representation (post-collision in the fused columns) against the oracle's
    state collided once more."""
    post = solver.coarse_post_collision()
    assert post.any() and not post.all()
    fluid = (oracle.fine.flags[1:-1, 1:-1, 1:-1] == 0)[oracle.fine_slices]
    coarse, fine = solver.states()
    np.testing.assert_allclose(coarse, oracle.coarse.interior(), rtol=0, atol=1e-14)
    np.testing.assert_allclose(fine, oracle.fine.interior()[oracle.fine_slices], rtol=0, atol=1e-14)
    for s in range(1, steps + 1):
        mine, theirs = solver.step(), oracle.step()
        for k in ("cl", "cd", "cm"):
            assert mine[k] == pytest.approx(theirs[k], abs=load_tol), (s, k)
        coarse, fine = solver.states()
        assert np.abs(coarse - oracle.coarse.interior()).max() <= pdf_tol * s
        # solid cells hold no state the fluid reads (the engine leaves them unstreamed)
        assert np.abs(fine - oracle.fine.interior()[oracle.fine_slices])[fluid].max() <= pdf_tol * s
    held, _ = solver.held_states()
    expected = oracle.coarse.interior().copy()
    expected[post] = O.collide(expected[post], oracle.coarse.omega_s, oracle.coarse.omega_b)
    assert np.abs(held - expected).max() <= pdf_tol * steps


def test_headline_two_level_case_matches_oracle():
    """The benchmark's two-level case itself (coarse 512 x 384 x 8 at chord 32,
    fine 160 x 76 x 16, AoA 8): states of both levels and loads against the
    oracle for 3 coarse steps at the plain form's bars."""
    import bench
    from aerokinetic_gb300.refined import RefinedSolver
    from aerokinetic_gb300.refined_plan import refined_project_dict
    project, refinement = bench.refined_parts()
    solver, oracle = refined_pair({"project": refined_project_dict(project, refinement)})
    try:
        assert tuple(solver.plan.shape) == (512, 384, 8)
        compare_refined(solver, oracle, steps=3)
    finally:
        solver.close()


def test_states_need_a_step_after_an_external_write(golden):
    """After ak_set_pdf on the coarse level the pre-collision state is not
    known until the next step; states() says so instead of returning the
    held representation."""
    solver, _ = refined_pair(golden["histories"]["refined_startup"])
    try:
        solver.step()
        held, _ = solver.held_states()
        from aerokinetic_gb300 import _native
        import ctypes
        _native.check(solver._lib.ak_set_pdf(solver._coarse, held.ctypes.data_as(ctypes.c_void_p)))
        with pytest.raises(ValueError, match="next step"):
            solver.states()
        solver.step()
        coarse, fine = solver.states()
        assert np.isfinite(coarse).all() and np.isfinite(fine).all()
    finally:
        solver.close()


def test_refined_startup_history_on_gpu(golden):
    from aerokinetic_gb300.refined import RefinedSolver
    from aerokinetic_gb300.refined_plan import load_refined_project
    record = golden["histories"]["refined_startup"]
    project, refinement = load_refined_project(record["project"])
    solver = RefinedSolver(project, refinement)
    try:
        for row in record["history"]:
            loads = solver.advance(row["step"] - solver.steps)
            for k in ("cl", "cd", "cm"):
                assert loads[k] == pytest.approx(row[k], abs=1e-11), (row["step"], k)
    finally:
        solver.close()


def test_refined_graph_replay_matches_eager_steps(golden):
    """ak_refined_step replays a captured coarse step (one graph per buffer
    parity); ak_refined_step_timed issues the same kernels one by one: the
    states agree bit for bit over an odd number of steps."""
    import ctypes
    from aerokinetic_gb300 import _native
    from aerokinetic_gb300.refined import RefinedSolver
    from aerokinetic_gb300.refined_plan import load_refined_project
    project, refinement = load_refined_project(golden["histories"]["refined_startup"]["project"])
    replay, eager = RefinedSolver(project, refinement), RefinedSolver(project, refinement)
    try:
        replay.advance(5)
        ms = np.zeros(6)
        _native.check(eager._lib.ak_refined_step_timed(eager._handle, 5, ms.ctypes.data_as(ctypes.c_void_p)))
        assert ms[0] > 0
        for a, b in zip(replay.states(), eager.states()):
            assert np.array_equal(a, b)
    finally:
        replay.close()
        eager.close()


def test_refined_two_step_graphs_match_single_steps():
    """Budget steps replayed two per graph (the second step's first fine step
    and donor moments overlapping the first step's far pass) against the same
    steps replayed one per graph and issued eagerly: states, loads, outer
    flux and integrals agree bit for bit on the benchmark's two-level case."""
    import ctypes
    import bench
    from aerokinetic_gb300 import _native
    from aerokinetic_gb300.refined import RefinedSolver
    project, refinement = bench.refined_parts()
    pairs, single, eager = (RefinedSolver(project, refinement, storage="f64") for _ in range(3))
    try:
        lib = pairs._lib
        n = len(pairs.contours)
        out = {}
        for name, solver in (("pairs", pairs), ("single", single)):
            loads, outer, stats = np.zeros((n, 5)), np.zeros(8), np.zeros(16)
            ptrs = [a.ctypes.data_as(ctypes.c_void_p) for a in (loads, outer, stats)]
            if name == "pairs":
                _native.check(lib.ak_refined_step_budget(solver._handle, 6, *ptrs))
            else:
                for _ in range(6):
                    _native.check(lib.ak_refined_step_budget(solver._handle, 1, *ptrs))
            out[name] = (loads, outer, stats)
        ms = np.zeros(6)
        _native.check(lib.ak_refined_step_timed(eager._handle, 6, ms.ctypes.data_as(ctypes.c_void_p)))
        for a, b in zip(out["pairs"], out["single"]):
            assert np.array_equal(a, b)
        assert lib.ak_refined_steps_done(pairs._handle) == lib.ak_refined_steps_done(eager._handle) == 6
        for a, b, c in zip(pairs.states(), single.states(), eager.states()):
            assert np.array_equal(a, b) and np.array_equal(a, c)
    finally:
        for solver in (pairs, single, eager):
            solver.close()


def test_budget_step_integrals_match_the_region_statistics():
    """The budget step's integrals (exact fixed-point sums: the fused coarse
    pass's warp rows, the transfer block's band and the fine block) against
    the FP64 region statistics of the same state (ak_refined_integrals), on
    the benchmark's two-level case after budget steps replayed several per
    graph."""
    import ctypes
    import bench
    from aerokinetic_gb300 import _native
    from aerokinetic_gb300.refined import RefinedSolver
    project, refinement = bench.refined_parts()
    solver = RefinedSolver(project, refinement, storage="f64")
    try:
        lib = solver._lib
        n = len(solver.contours)
        loads, outer, stats = np.zeros((n, 5)), np.zeros(8), np.zeros(16)
        ptrs = [a.ctypes.data_as(ctypes.c_void_p) for a in (loads, outer, stats)]
        _native.check(lib.ak_refined_step_budget(solver._handle, 6, *ptrs))
        ref = np.zeros(16)
        _native.check(lib.ak_refined_integrals(solver._handle, ref.ctypes.data_as(ctypes.c_void_p)))
        for lo in (0, 8):  # coarse cells outside the box, fine physical block
            assert stats[lo + 6] == ref[lo + 6] > 0 and stats[lo + 7] == ref[lo + 7] == 0
            assert stats[lo + 2] + stats[lo + 6] == pytest.approx(ref[lo + 2] + ref[lo + 6], rel=1e-15)
            np.testing.assert_allclose(stats[lo + 3:lo + 6], ref[lo + 3:lo + 6], rtol=1e-12, atol=1e-11)
    finally:
        solver.close()


def test_refined_budget_integrals_and_diagnostics_match_oracle(golden):
    """conserved_integrals, the per-step budget (last_budget) and diagnostics
    (refined_solver.py:291-361) against the oracle sampling the outer faces in
    the engine's z-wrapped layout; residuals within the reference's gates."""
    solver, oracle = refined_pair(golden["histories"]["refined_startup"])
    oracle.outer_convention = "wrapped"
    try:
        mine, theirs = solver.conserved_integrals(), oracle.conserved_integrals()
        assert mine["mass"] == pytest.approx(theirs["mass"], rel=1e-14)
        # the reference's momentum integral (pdf @ stencil, then a sum over
        # axis 0) carries ~3.5e-12 relative rounding on this case against an
        # exactly rounded sum (math.fsum); the engine's tree sum is closer to it
        np.testing.assert_allclose(mine["momentum"], theirs["momentum"], rtol=1e-10, atol=1e-16)
        wall_mass = 0.0
        for s in range(1, 4):
            solver.step()
            ref = oracle.step_with_budget()["budget"]
            got = solver.last_budget
            assert abs(got["mass_residual_per_volume"]) <= 5e-11
            assert max(map(abs, got["momentum_residual_per_volume"])) <= 2e-12
            for key in ("wall_mass_exchange", "external_mass_in"):
                assert got[key] == pytest.approx(ref[key], rel=1e-9, abs=1e-14), (s, key)
            for key in ("wall_impulse", "external_impulse_in"):
                np.testing.assert_allclose(got[key], ref[key], rtol=1e-9, atol=1e-14)
            np.testing.assert_allclose(got["momentum_residual_per_volume"], ref["momentum_residual_per_volume"],
                                       rtol=0, atol=1e-12)
            wall_mass += ref["wall_mass_exchange"]
        assert solver.cumulative_wall_mass_exchange == pytest.approx(wall_mass, rel=1e-9, abs=1e-14)
        ours, ref = solver.diagnostics(), oracle.diagnostics()
        assert ours["local_mach_max"] == pytest.approx(ref["local_mach_max"], rel=1e-12)
        assert ours["density_error_max"] == pytest.approx(ref["density_error_max"], rel=1e-10)
        assert ours["fine_boundary_calls"] == 6 and ours["last_budget"] is solver.last_budget
    finally:
        solver.close()


def test_refined_run_writes_history_frames_and_summary(golden, tmp_path):
    """RefinedSolver.run (refined_run.py:19-156) for a new run: history rows at
    sample_every, frames, metadata and summary with the guards' diagnostics."""
    import csv
    import dataclasses
    import json
    from aerokinetic_gb300.project import RunSettings
    from aerokinetic_gb300.refined import RefinedSolver
    from aerokinetic_gb300.refined_plan import load_refined_project
    project, refinement = load_refined_project(golden["histories"]["refined_startup"]["project"])
    settings = RunSettings(duration_convective=0.1, sample_every=4, frame_every=16, check_every=4, average_after=0.0)
    project = dataclasses.replace(project, run=settings)
    solver = RefinedSolver(project, refinement)
    try:
        steps = int(np.ceil(0.1 / solver.coarse_level.dt - 1e-9))
        summary = solver.run(tmp_path / "out")
        assert summary["status"] == "completed" and summary["steps"] == steps
        rows = list(csv.DictReader((tmp_path / "out" / "history.csv").open()))
        assert [int(r["step"]) for r in rows] == list(range(4, steps + 1, 4))
        assert summary["samples"] == len(rows) and summary["mean"] is not None
        assert summary["diagnostics"]["local_mach_max"] < 0.3
        meta = json.loads((tmp_path / "out" / "metadata.json").read_text())
        assert meta["status"] == "completed" and meta["case_fingerprint"] == solver.case_fingerprint
        frames = sorted((tmp_path / "out" / "frames").glob("frame_*.npz"))
        assert len(frames) >= 2
        with np.load(frames[-1]) as frame:
            assert frame["coarse_speed"].shape == tuple(solver.plan.shape[:2])
            assert frame["fine_speed"].shape == tuple(solver.fine_shape[:2])
            assert np.isnan(frame["fine_cp"][frame["fine_mask"]]).all()
        with pytest.raises(FileExistsError):
            solver.run(tmp_path / "out")
    finally:
        solver.close()


@pytest.mark.gpu
@pytest.mark.parametrize("storage,tol", [("f32", 5e-3), ("f16", 5e-3)])
def test_refined_precision_forms_track_fp64(golden, storage, tol):
    """The two-level case in the FP32-compute forms (FP32 storage; FP16
    storage with the walls' fine level in FP32; FP32 transfer arithmetic)
    stays within 0.5 % of the FP64 form on Cl, Cd and Cm (relative, floor
    0.05) over 60 coarse steps."""
    from aerokinetic_gb300.refined import RefinedSolver
    from aerokinetic_gb300.refined_plan import load_refined_project
    project, refinement = load_refined_project(golden["histories"]["refined_startup"]["project"])
    plain, low = RefinedSolver(project, refinement), RefinedSolver(project, refinement, storage=storage)
    assert low.fine_storage == "f32"
    try:
        for _ in range(6):
            a, b = plain.advance(10), low.advance(10)
            for k in ("cl", "cd", "cm"):
                assert abs(a[k] - b[k]) <= tol * max(abs(a[k]), 0.05), (a["step"], k, a[k], b[k])
    finally:
        plain.close()
        low.close()


@pytest.mark.gpu
@pytest.mark.parametrize("storage", ["f64", "f32", "df64"])
def test_population_tensor_views_the_engine_state(storage):
    """Solver.population_tensor is a torch view of the engine's current copy:
    its interior equals ak_get_pdf without any copy by the engine."""
    import torch
    solver = solver_for(kat_project("characteristic_transport_v1"), storage)
    try:
        solver.advance(3)
        view = solver.population_tensor()
        assert view.is_cuda and view.shape[:3] == (27, solver.plan.shape[2], solver.plan.shape[1] + 2)
        nx, ny, nz = solver.plan.shape
        interior = view[:, :, 1:ny + 1, 1:nx + 1].double()
        if storage == "df64":
            interior = interior[..., 0] + interior[..., 1]
        got = interior.permute(3, 2, 1, 0).cpu().numpy()
        assert np.array_equal(got, solver.pdf())
        before = view.clone()
        solver.advance(1)
        assert not torch.equal(solver.population_tensor(), before)
    finally:
        solver.close()
