"""Serving loop (continuous batching): admission by memory, retirement on
convergence, and results independent of the mix."""
import math

import numpy as np
import pytest

from aerokinetic_gb300 import Flow, Grid, Section, naca4_parametric
from aerokinetic_gb300.serve import (Server, SolveRequest, flapped_section, poisson_arrivals, random_requests)


def _request(name, chord, alpha, reynolds, seed, flap=None, max_steps=300, tolerance=2e-3):
    section = flapped_section(0.02, 0.4, 0.12, flap, n_side=41) if flap is not None else Section(
        (naca4_parametric(0.0, 0.0, 0.12, 41, name="main"),))
    flow = Flow(reynolds=reynolds, alpha_deg=alpha, lattice_speed=0.05, seed=seed)
    grid = Grid(cells_per_chord=chord, upstream_chords=2.0, downstream_chords=3.0, transverse_chords=1.5,
                span_chords=0.25, farfield="characteristic_transport_v1", memory_limit_gib=8)
    return SolveRequest(section, flow, grid, max_steps=max_steps, window=100, cl_tolerance=tolerance, name=name)


def test_request_generators_are_seeded_and_in_range():
    a, b = random_requests(12, seed=5), random_requests(12, seed=5)
    assert [r.name for r in a] == [r.name for r in b]
    for r, s in zip(a, b):
        assert r.flow == s.flow and r.grid == s.grid and r.max_steps == s.max_steps
        assert 24 <= r.grid.cells_per_chord <= 96 and -4 <= r.flow.alpha_deg <= 14
        assert 1e4 <= r.flow.reynolds <= 1e5 and r.max_steps % r.window == 0
        assert len(r.section.elements) in (1, 2)
    times = poisson_arrivals(4.0, 2000, seed=3)
    assert np.all(np.diff(times) > 0) and abs(np.mean(np.diff(times)) - 0.25) < 0.02
    section = flapped_section(0.02, 0.4, 0.12, 20.0)
    assert section.chord == 1.0 and [e.name for e in section.elements] == ["main", "flap"]
    with pytest.raises(ValueError):
        SolveRequest(section, Flow(), Grid(), max_steps=0)


def test_server_rejects_bad_settings():
    req = _request("a", 16, 4.0, 2e4, 1)
    with pytest.raises(ValueError, match="multiple of the chunk"):
        Server(chunk=30).run([req])
    with pytest.raises(MemoryError):
        Server(memory_budget_gib=1e-4, chunk=50).run([req])


@pytest.mark.gpu
def test_served_results_match_solves_alone():
    """Four requests (one with a flap) arriving while others run, under a
    memory budget that fits two at a time: every result equals the same
    request served alone, bit for bit, and residency never exceeds the budget."""
    requests = [_request("a", 16, 4.0, 2e4, 1), _request("b", 20, 8.0, 3e4, 2, flap=15.0),
                _request("c", 16, -2.0, 1e4, 3, max_steps=200), _request("d", 24, 2.0, 5e4, 4)]
    probe = Server(chunk=50, storage="f32")
    need = sorted(probe.footprint(r) for r in requests)
    budget = (need[-1] + need[-2]) / 2**30 * 1.01
    server = Server(memory_budget_gib=budget, chunk=50, storage="f32")
    mixed = {r.name: r for r in server.run(requests, arrivals=[0.0, 0.0, 0.01, 0.02])}
    stats = server.stats
    assert stats["completed"] == 4 and stats["peak_resident_cases"] <= 2
    assert stats["peak_resident_gib"] <= budget and stats["batch_rebuilds"] >= 2
    assert stats["latency_p50_s"] <= stats["latency_p99_s"]
    for request in requests:
        alone = Server(chunk=50, storage="f32").run([request])[0]
        got = mixed[request.name]
        assert (got.cl, got.cd, got.cm, got.steps, got.status) == (alone.cl, alone.cd, alone.cm, alone.steps,
                                                                    alone.status)
        assert got.steps <= request.max_steps and math.isfinite(got.cl)
        assert got.finished_s >= got.admitted_s >= got.arrival_s
