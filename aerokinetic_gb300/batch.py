"""Batch: independent uniform cases advanced together on one GPU.

The reference runs one case per process (src/aerokinetic/cli.py:121-139); a
polar sweep is many such runs.  Here a Batch borrows several Solver objects
(uniform grid, characteristic or legacy outer boundary, one storage form) and
steps them with one set of launches per step over packed work tables (include/
aerokinetic_gb300.h, ak_batch_*).  Every case computes the same bits as it
would alone, so each Solver's state, diagnostics and frames stay valid.
"""
import ctypes

import numpy as np

from . import _native
from ._native import check

__all__ = ["Batch"]

MAX_ELEMENTS = 8


class Batch:
    def __init__(self, solvers, tune_trials=0):
        self.solvers = list(solvers)
        if not self.solvers:
            raise ValueError("A batch needs at least one solver")
        if len({id(s) for s in self.solvers}) != len(self.solvers):
            raise ValueError("A solver appears twice in the batch")
        self._lib = _native.load()
        handles = (ctypes.c_void_p * len(self.solvers))(*[s._case.value for s in self.solvers])
        handle = ctypes.c_void_p()
        check(self._lib.ak_batch_create(handles, len(self.solvers), ctypes.byref(handle)))
        self._handle = handle
        self.schedule = None
        if tune_trials:
            self.tune(tune_trials)

    def tune(self, trials=3):
        """Pick the stream-collide block width, persistent grid (FP64 and df64
        forms) and table order."""
        report = np.zeros(5)
        check(self._lib.ak_batch_tune(self._handle, int(trials), report.ctypes.data_as(ctypes.c_void_p)))
        self.schedule = {"block_width": int(report[0]), "ctas_per_sm": int(report[1]),
                         "order": ("case-major", "interleaved")[int(report[2])],
                         "ms_per_launch": float(report[3]), "previous_ms_per_launch": float(report[4])}
        return self.schedule

    def advance(self, nsteps, sample_last=True):
        """nsteps steps of every case; with sample_last each solver's record of
        the last step (Solver.step(sample=True)'s keys) in batch order."""
        nsteps = int(nsteps)
        if nsteps < 1:
            raise ValueError("nsteps must be >= 1")
        raw = np.zeros((len(self.solvers), MAX_ELEMENTS, 5)) if sample_last else None
        check(self._lib.ak_batch_step(self._handle, nsteps,
                                      raw.ctypes.data_as(ctypes.c_void_p) if sample_last else None))
        records = []
        for i, solver in enumerate(self.solvers):
            solver.steps += nsteps
            if sample_last:
                solver.last_loads = solver._record(np.ascontiguousarray(raw[i, :len(solver.contours)]))
                records.append(solver.last_loads)
        return records if sample_last else None

    @property
    def launches(self):
        return int(self._lib.ak_batch_launches(self._handle))

    @property
    def stream(self):
        return self._lib.ak_batch_stream(self._handle)

    @property
    def cells(self):
        return sum(int(np.prod(s.plan.shape)) for s in self.solvers)

    def close(self):
        if getattr(self, "_handle", None):
            self._lib.ak_batch_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
