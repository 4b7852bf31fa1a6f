"""Checkpoints of GPU cases: populations plus every history-dependent boundary.

Same contract as the reference's checkpoint.py:32-135 (uniform) and
refined_checkpoint.py (two levels): one uncompressed .npz replaced atomically,
JSON metadata with the project, its fingerprint, the clocks, the fallback-link
count and the caller's context, and the arrays that continue the same timeline
bit for bit.  The arrays are the engine's: populations in lbmpy's zero-centred
D3Q27 order as (nx, ny, nz, 27) doubles (exact for every storage form), and the
outer boundary's history keyed by its link geometry (ak_get_boundary_state).
The reference stores lbmpy's own field and index arrays instead, which cannot
be produced without lbmpy, so the format is named "aerokinetic_gb300_checkpoint".
"""
import ctypes
import hashlib
import json
import os
from pathlib import Path

import numpy as np

from ._native import check
from .convergence import restore_control, save_control
from .project import Project

FORMAT = "aerokinetic_gb300_checkpoint"
SCHEMA = 1


def _ptr(array):
    return array.ctypes.data_as(ctypes.c_void_p)


def boundary_state(lib, handle):
    n_links, n_values = ctypes.c_int64(), ctypes.c_int64()
    check(lib.ak_boundary_state_size(handle, ctypes.byref(n_links), ctypes.byref(n_values)))
    rows = np.zeros((n_links.value, 4), dtype=np.int32)
    values = np.zeros(n_values.value)
    check(lib.ak_get_boundary_state(handle, _ptr(rows), _ptr(values)))
    return rows, values


def set_boundary_state(lib, handle, rows, values):
    n_links, n_values = ctypes.c_int64(), ctypes.c_int64()
    check(lib.ak_boundary_state_size(handle, ctypes.byref(n_links), ctypes.byref(n_values)))
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    values = np.ascontiguousarray(values, dtype=np.float64)
    if rows.shape != (n_links.value, 4) or values.shape != (n_values.value,):
        raise ValueError("Checkpoint boundary arrays do not match the rebuilt case")
    if not np.isfinite(values).all():
        raise ValueError("Checkpoint boundary history is not finite")
    check(lib.ak_set_boundary_state(handle, _ptr(rows), _ptr(values)))


def _digest(array):
    return hashlib.sha256(np.ascontiguousarray(array).tobytes(order="C")).hexdigest()


def _write(path, arrays, metadata):
    """Uncompressed npz through a temporary file in the same directory: an
    interrupted write leaves the previous checkpoint usable."""
    metadata = dict(metadata, array_sha256={k: _digest(v) for k, v in arrays.items()})
    arrays = dict(arrays, metadata=np.asarray(json.dumps(metadata, ensure_ascii=False, allow_nan=False)))
    path = Path(path)
    tmp = path.with_name(path.name + ".tmp")
    with open(tmp, "wb") as handle:
        np.savez(handle, **arrays)
        handle.flush()
        os.fsync(handle.fileno())
    tmp.replace(path)
    return path


def _read(path, kind):
    saved = np.load(path, allow_pickle=False)
    meta = json.loads(str(saved["metadata"]))
    if meta.get("format") != FORMAT or meta.get("schema_version") != SCHEMA or meta.get("kind") != kind:
        saved.close()
        raise ValueError(f"Not an {FORMAT} ({kind}) checkpoint of schema {SCHEMA}")
    if set(saved.files) != set(meta["array_sha256"]) | {"metadata"}:
        saved.close()
        raise ValueError("Checkpoint array manifest differs")
    for name, expected in meta["array_sha256"].items():
        if _digest(saved[name]) != expected:
            saved.close()
            raise ValueError(f"Checkpoint array checksum failed: {name}")
    if type(meta.get("steps")) is not int or meta["steps"] < 0:
        saved.close()
        raise ValueError("Invalid checkpoint step count")
    return saved, meta


# ---------------------------------------------------------------- uniform
def save_checkpoint(solver, path, context=None):
    project = Project(solver.section, solver.flow, solver.grid)
    rows, values = boundary_state(solver._lib, solver._case)
    metadata = {"format": FORMAT, "schema_version": SCHEMA, "kind": "uniform", "project": project.as_dict(),
                "case_fingerprint": project.case_fingerprint, "steps": solver.steps, "storage": solver.storage,
                "wall_fallback_links": solver.wall_fallback_links, "context": context or {}}
    arrays = {"pdf": solver.pdf(), "boundary_rows": rows, "boundary_values": values}
    save_control(solver, arrays, metadata)
    return _write(path, arrays, metadata)


def restore_checkpoint(solver_type, path, progress=None):
    saved, meta = _read(path, "uniform")
    with saved:
        project = Project.from_dict(meta["project"])
        if project.case_fingerprint != meta["case_fingerprint"]:
            raise ValueError("Checkpoint physical/numerical case is inconsistent")
        solver = solver_type(project.section, project.flow, project.grid, progress=progress, storage=meta["storage"])
        try:
            pdf = saved["pdf"]
            if pdf.shape != tuple(solver.plan.shape) + (27,) or pdf.dtype != np.float64 or not np.isfinite(pdf).all():
                raise ValueError("Checkpoint populations do not match the rebuilt case")
            solver.set_pdf(pdf)
            set_boundary_state(solver._lib, solver._case, saved["boundary_rows"], saved["boundary_values"])
            if meta["wall_fallback_links"] != solver.wall_fallback_links:
                raise ValueError("Checkpoint wall links differ from the rebuilt case")
            solver.steps = meta["steps"]
            check(solver._lib.ak_set_steps_done(solver._case, solver.steps))
            solver._checkpoint_context = meta["context"]
            restore_control(solver, saved, meta)
            solver.diagnostics()
        except Exception:
            solver.close()
            raise
    return solver


# ---------------------------------------------------------------- two levels
def save_refined_checkpoint(solver, path, context=None):
    if not solver.initialized:
        raise ValueError("Checkpoint requires a valid synchronized state")
    arrays = {}
    for label, handle, shape in (("coarse", solver._coarse, tuple(solver.plan.shape)),
                                 ("fine", solver._fine, solver._padded_shape())):
        pdf = np.empty(shape + (27,))
        check(solver._lib.ak_get_pdf(handle, _ptr(pdf)))
        arrays[f"{label}_pdf"] = pdf
    arrays["coarse_boundary_rows"], arrays["coarse_boundary_values"] = boundary_state(solver._lib, solver._coarse)
    arrays["cumulative_loads"] = solver._cumulative_loads()
    flux = np.zeros(8)
    check(solver._lib.ak_refined_outer_flux(solver._handle, _ptr(flux)))
    arrays["cumulative_outer"] = flux[4:].copy()
    metadata = {"format": FORMAT, "schema_version": SCHEMA, "kind": "refined",
                "project": solver.project.as_dict(), "refinement": dict(solver.refinement.__dict__),
                "case_fingerprint": solver.case_fingerprint, "steps": solver.steps, "fine_steps": solver.fine_steps,
                "storage": solver.storage, "fine_storage": solver.fine_storage, "budget": solver.budget,
                "last_loads": solver.last_loads, "last_budget": solver.last_budget,
                "initial_integrals": solver._initial_integrals, "wall_fallback_links": solver.wall_fallback_links,
                "context": context or {}}
    save_control(solver, arrays, metadata)
    return _write(path, arrays, metadata)


def restore_refined_checkpoint(solver_type, path, progress=None):
    from .refined_plan import RefinementSettings
    saved, meta = _read(path, "refined")
    with saved:
        if meta.get("fine_steps") != 2 * meta["steps"]:
            raise ValueError("Invalid refined checkpoint clocks")
        project = Project.from_dict(meta["project"])
        refinement = RefinementSettings(**meta["refinement"])
        solver = solver_type(project, refinement, progress=progress, storage=meta["storage"], budget=meta["budget"],
                             fine_storage=meta.get("fine_storage"))
        try:
            if solver.case_fingerprint != meta["case_fingerprint"]:
                raise ValueError("Refined checkpoint case fingerprint differs")
            for label, handle, shape in (("coarse", solver._coarse, tuple(solver.plan.shape)),
                                         ("fine", solver._fine, solver._padded_shape())):
                pdf = saved[f"{label}_pdf"]
                if pdf.shape != shape + (27,) or pdf.dtype != np.float64 or not np.isfinite(pdf).all():
                    raise ValueError(f"Checkpoint {label} populations do not match the rebuilt case")
                check(solver._lib.ak_set_pdf(handle, _ptr(np.ascontiguousarray(pdf))))
            set_boundary_state(solver._lib, solver._coarse, saved["coarse_boundary_rows"],
                               saved["coarse_boundary_values"])
            if meta["wall_fallback_links"] != solver.wall_fallback_links:
                raise ValueError("Checkpoint wall links differ from the rebuilt case")
            cumulative = np.ascontiguousarray(saved["cumulative_loads"], dtype=np.float64)
            outer = np.ascontiguousarray(saved["cumulative_outer"], dtype=np.float64)
            if cumulative.shape != (len(solver.contours), 5) or outer.shape != (4,):
                raise ValueError("Checkpoint running sums do not match the rebuilt case")
            check(solver._lib.ak_refined_restore_counters(solver._handle, meta["steps"], _ptr(cumulative),
                                                          _ptr(outer)))
            solver.steps = meta["steps"]
            solver.last_loads, solver.last_budget = meta["last_loads"], meta["last_budget"]
            solver._initial_integrals = meta["initial_integrals"]
            solver._integrals = None
            solver._checkpoint_context = meta["context"]
            restore_control(solver, saved, meta)
            solver.diagnostics()
        except Exception:
            solver.close()
            raise
    return solver
