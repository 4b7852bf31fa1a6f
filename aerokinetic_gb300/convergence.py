"""Stationarity residuals and explicit stop criteria of the run loops.

Mirrors the reference's convergence.py:20-176: the four residuals are the
volume-weighted L2 and the L-infinity of d(rho, j / U)/dt* over the owned
fluid cells between two checks, written to residuals.csv with the budget's
balance defects, and a steady-mode streak ends the run when every L2 residual
stays under its tolerance for consecutive_checks checks after minimum_t_star.
The reductions run on the device against a snapshot kept there
(ak_residuals), so a check moves nine numbers per level, not the lattice.
"""
from dataclasses import asdict
import csv
import ctypes
import os
from pathlib import Path
import shutil
import time
import uuid

import numpy as np

from ._native import check

CHANNELS = ("rho", "jx", "jy", "jz")
RESIDUAL_COLUMNS = ("step", "t_star", *(f"l2_{c}" for c in CHANNELS), *(f"linf_{c}" for c in CHANNELS),
                    *(f"balance_{c}" for c in CHANNELS), "streak")


def _levels(solver):
    """(case handle, cell volume) of the owned levels."""
    if hasattr(solver, "coarse_level"):
        return ((solver._coarse, solver.coarse_level.dx ** 3), (solver._fine, solver.fine_level.dx ** 3))
    return ((solver._case, solver.plan.dx ** 3),)


def _file_hash(path, limit=None):
    from .solver import _file_hash as digest
    return digest(path, limit)


def validate_history(output, context):
    if "residuals_bytes" in context:
        path = Path(output) / "residuals.csv"
        if _file_hash(path, context["residuals_bytes"]) != context["residuals_sha256"]:
            raise ValueError("Residual history before checkpoint changed")


class RunControl:
    def __init__(self, solver, settings, output, *, resume=False, callback=None, start_step=None):
        self.solver, self.criteria, self.callback = solver, settings.termination, callback
        self.path = Path(output) / "residuals.csv"
        self.started = time.monotonic()
        self.dt = solver.coarse_level.dt if hasattr(solver, "coarse_level") else solver.plan.dt_convective
        self.run_start_step = solver.steps if start_step is None else start_step
        self.levels = _levels(solver)
        self._lib = solver._lib
        self.inv_speed = 1.0 / solver.flow.lattice_speed
        self.previous_step, self.streak, self.last_record = solver.steps, 0, None
        restored = getattr(solver, "_restored_control", None) if resume else None
        if restored is not None:
            meta, arrays = restored
            for (handle, _), data in zip(self.levels, arrays):
                count = ctypes.c_int64()
                check(self._lib.ak_residual_snapshot(handle, 0, None, ctypes.byref(count)))
                data = np.ascontiguousarray(data, dtype=np.float64)
                if data.shape != (count.value,) or len(arrays) != len(self.levels):
                    raise ValueError("Residual checkpoint ownership differs")
                check(self._lib.ak_residual_snapshot(handle, 1, data.ctypes.data_as(ctypes.c_void_p),
                                                     ctypes.byref(count)))
            if (type(meta["previous_step"]) is not int or not 0 <= meta["previous_step"] <= solver.steps
                    or type(meta["streak"]) is not int or meta["streak"] < 0):
                raise ValueError("Invalid residual checkpoint clock/streak")
            self.previous_step, self.streak = meta["previous_step"], meta["streak"]
            self.last_record, self.run_start_step = meta["last_record"], meta["run_start_step"]
        else:
            self._measure(reset=True)
        context = getattr(solver, "_checkpoint_context", {}) if resume else {}
        validate_history(output, context)
        if resume and self.path.exists():
            prefix = context.get("residuals_bytes", 0)
            if self.path.stat().st_size > prefix:
                recovery = Path(output) / "recovery" / uuid.uuid4().hex
                recovery.mkdir(parents=True)
                shutil.copy2(self.path, recovery / "residuals_before_resume.csv")
                with self.path.open("r+b") as handle:
                    handle.truncate(prefix)
        append = resume and "residuals_bytes" in context
        self.handle = self.path.open("a" if append else "w", newline="", encoding="utf-8")
        self.writer = csv.DictWriter(self.handle, RESIDUAL_COLUMNS)
        if not append:
            self.writer.writeheader()
            self.handle.flush()
        solver._run_control = self

    def _measure(self, reset, interval=1.0):
        square, infinity, volume = np.zeros(4), np.zeros(4), 0.0
        for handle, cell_volume in self.levels:
            out = np.zeros(9)
            check(self._lib.ak_residuals(handle, self.inv_speed, 1.0 / interval, 1 if reset else 0,
                                         out.ctypes.data_as(ctypes.c_void_p)))
            square += cell_volume * out[:4]
            infinity = np.maximum(infinity, out[4:8])
            volume += cell_volume * out[8]
        if volume <= 0:
            raise ValueError("Residual domain has no owned fluid volume")
        return np.sqrt(square / volume), infinity

    def observe(self):
        step = self.solver.steps
        if step <= self.previous_step:
            return None
        l2, linf = self._measure(False, (step - self.previous_step) * self.dt)
        if not (np.isfinite(l2).all() and np.isfinite(linf).all()):
            raise ValueError("Non-finite residual state")
        record = {"step": step, "t_star": step * self.dt}
        record.update(zip((f"l2_{c}" for c in CHANNELS), map(float, l2)))
        record.update(zip((f"linf_{c}" for c in CHANNELS), map(float, linf)))
        budget = getattr(self.solver, "last_budget", None)
        if budget:
            defects = [budget["mass_residual_per_volume"], *budget["momentum_residual_per_volume"]]
            record.update(zip((f"balance_{c}" for c in CHANNELS), (abs(float(v)) / self.dt for v in defects)))
        eligible = (self.criteria.mode == "steady" and record["t_star"] >= self.criteria.minimum_t_star
                    and all(value <= limit for value, limit in zip(l2, self.criteria.thresholds)))
        self.streak = self.streak + 1 if eligible else 0
        record["streak"] = self.streak
        self.previous_step, self.last_record = step, record
        self.writer.writerow(record)
        self.handle.flush()
        if self.callback:
            self.callback(self.solver, dict(record))
        return record

    def stop_reason(self):
        if self.criteria.mode == "steady" and self.streak >= self.criteria.consecutive_checks:
            return "residual_targets_met"
        if self.criteria.max_steps and self.solver.steps - self.run_start_step >= self.criteria.max_steps:
            return "max_steps_reached"
        if self.criteria.wall_time_limit_s and time.monotonic() - self.started >= self.criteria.wall_time_limit_s:
            return "wall_time_limit"
        return None

    def checkpoint_context(self):
        self.handle.flush()
        os.fsync(self.handle.fileno())
        return {"residuals_bytes": self.path.stat().st_size, "residuals_sha256": _file_hash(self.path)}

    def summary(self, reason):
        return {"termination_reason": reason, "termination": asdict(self.criteria), "last_residuals": self.last_record,
                "steady_residual_criterion_met": reason == "residual_targets_met",
                "statistical_convergence": "not_established"}

    def close(self):
        self.handle.close()


def save_control(solver, arrays, metadata):
    """The control's snapshot and clocks in a checkpoint (convergence.py save_control)."""
    control = getattr(solver, "_run_control", None)
    if control is None:
        return
    for i, (handle, _) in enumerate(control.levels):
        count = ctypes.c_int64()
        check(control._lib.ak_residual_snapshot(handle, 0, None, ctypes.byref(count)))
        data = np.empty(count.value)
        check(control._lib.ak_residual_snapshot(handle, 0, data.ctypes.data_as(ctypes.c_void_p),
                                                ctypes.byref(count)))
        arrays[f"control_snapshot_{i}"] = data
    metadata["control"] = {"previous_step": control.previous_step, "streak": control.streak,
                           "last_record": control.last_record, "run_start_step": control.run_start_step,
                           "levels": len(control.levels)}


def restore_control(solver, saved, metadata):
    meta = metadata.get("control")
    if meta is None:
        return
    solver._restored_control = (meta, [saved[f"control_snapshot_{i}"] for i in range(meta["levels"])])
