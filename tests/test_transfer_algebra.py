"""Unit parity of the two-level transfer algebra and plans with the reference.

The fixtures (tests/golden/transfer.json, refined_plans.json) hold outputs of
the reference's own NumPy code on seeded inputs, written by
tests/golden/make_golden.py: D3Q27Transfer.moments / populations /
_rescale_stress, prolong_cell_averages, restrict_cell_averages
(refinement.py:78-254), StreamingFaceFlux (interface.py:44-104) and
RefinedPlan.create (refined_solver.py:42-99).  The oracle's restatement
(oracle/refined.py) must reproduce them; the engine's kernels are compared
with the oracle on the GPU (tests/test_gpu_transfer.py).
"""
import numpy as np
import pytest

from oracle.refined import FaceFlux, Level, Transfer, prolong_cell_averages, restrict_cell_averages

TOL = 1e-15  # absolute, on O(1) densities and O(1e-2) populations


@pytest.fixture(scope="module")
def fx(golden):
    return golden["transfer"]


@pytest.fixture(scope="module")
def transfer(fx):
    L = fx["coarse_level"]
    return Transfer(Level(L["dx"], L["dt"], L["tau_shear"], L["tau_bulk"]))


def test_moments_and_populations(fx, transfer):
    np.testing.assert_allclose(transfer.moments(np.array(fx["cells"])), fx["moments"], rtol=0, atol=TOL)
    np.testing.assert_allclose(transfer.populations(np.array(fx["fields"])), fx["populations"], rtol=0, atol=TOL)


def test_stress_rescale_both_ways(fx, transfer):
    fields = np.array(fx["fields"])
    np.testing.assert_allclose(Transfer.rescale_stress(fields, transfer.coarse, transfer.fine),
                               fx["rescale_to_fine"], rtol=0, atol=TOL)
    np.testing.assert_allclose(Transfer.rescale_stress(fields, transfer.fine, transfer.coarse),
                               fx["rescale_to_coarse"], rtol=0, atol=TOL)


def test_prolongation_and_time_interpolation(fx, transfer):
    block = np.array(fx["block"])
    np.testing.assert_allclose(prolong_cell_averages(transfer.moments(block)), fx["prolonged_moments"], rtol=0,
                               atol=TOL)
    mixed = 0.5 * transfer.moments(block) + 0.5 * transfer.moments(block[::-1])
    fine = transfer.populations(Transfer.rescale_stress(prolong_cell_averages(mixed), transfer.coarse,
                                                        transfer.fine))
    np.testing.assert_allclose(fine, fx["prolonged_in_time"], rtol=0, atol=TOL)


def test_restriction(fx, transfer):
    fine = np.array(fx["fine"])
    np.testing.assert_allclose(restrict_cell_averages(transfer.moments(fine)), fx["restricted_moments"], rtol=0,
                               atol=TOL)
    np.testing.assert_allclose(transfer.restrict(fine), fx["restricted"], rtol=0, atol=TOL)


def test_face_fluxes(fx):
    lattice = np.array(fx["lattice"])
    for face in fx["face_fluxes"]:
        flux = FaceFlux(lattice.shape[:3], face["axis"], face["index"], face["ranges"], periodic=True)
        np.testing.assert_allclose(flux(lattice), face["flux"], rtol=0, atol=TOL)


@pytest.mark.parametrize("name", ["two_level_512x384x8", "two_element_large"])
def test_refined_plan_matches_the_reference(golden, name):
    """Box placement, levels and span of the two-level benchmark cases equal
    the reference's RefinedPlan.create bit for bit."""
    from aerokinetic_gb300 import Flow, Grid, Project, Section, naca0012
    from aerokinetic_gb300.refined_plan import RefinedPlan, RefinementSettings
    from aerokinetic_gb300.serve import flapped_section
    ref = golden["refined_plans"][name]
    spec = ref["spec"]
    section = Section((naca0012(161),)) if spec["flap"] is None else flapped_section(**spec["flap"])
    project = Project(section, Flow(**spec["flow"]), Grid(**spec["grid"]))
    plan = RefinedPlan.create(project, RefinementSettings(**spec["refinement"]))
    assert list(plan.shape) == ref["shape"]
    assert list(plan.origin) == ref["origin"]
    assert list(plan.box.lower) == ref["box_lower"] and list(plan.box.upper) == ref["box_upper"]
    for key in ("coarse_level", "fine_level"):
        level = getattr(plan, key)
        assert {k: getattr(level, k) for k in ref[key]} == ref[key]
    assert plan.span == ref["span"]
    assert plan.minimum_wall_interface_distance_coarse_cells == ref["minimum_wall_interface_distance_coarse_cells"]


def test_benchmark_cases_use_the_pinned_parameters(golden):
    """bench.py builds its two-level cases from the same parameters."""
    import bench
    project, refinement = bench.refined_parts()
    spec = golden["refined_plans"]["two_level_512x384x8"]["spec"]
    assert project.flow.alpha_deg == spec["flow"]["alpha_deg"] and project.grid.cells_per_chord == 32
    assert refinement.upstream_chords == spec["refinement"]["upstream_chords"]
    project, refinement = bench.large_parts()
    spec = golden["refined_plans"]["two_element_large"]["spec"]
    assert project.grid.cells_per_chord == spec["grid"]["cells_per_chord"]
    assert refinement.downstream_chords == spec["refinement"]["downstream_chords"]
