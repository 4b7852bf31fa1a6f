"""Build and load the engine's shared library (C ABI: include/aerokinetic_gb300.h).

The library is compiled in-tree for sm_103a with nvcc and loaded with ctypes.
There is no fallback: if it cannot be built or loaded, or no CUDA device is
present, every entry point raises.
"""
import ctypes
import os
import shutil
import subprocess
import threading
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
ROOT = PACKAGE.parent
SOURCES = [PACKAGE / "csrc" / "ak_engine.cu"]
HEADERS = sorted((PACKAGE / "csrc").glob("*.cuh")) + [ROOT / "include" / "aerokinetic_gb300.h"]
LIBRARY = PACKAGE / "_build" / "libaerokinetic_gb300.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

AK_OK, AK_ERR_INVALID, AK_ERR_CUDA, AK_ERR_NOMEM, AK_ERR_NONFINITE, AK_ERR_GUARD, AK_ERR_GEOMETRY = range(7)
FARFIELD = {"legacy": 0, "characteristic_transport_v1": 1, "exterior_regularized_fd_v1": 2}
STORAGE = {"f64": 0, "f32": 1, "f16": 2, "df64": 3}


class EngineError(RuntimeError):
    """A CUDA-side failure reported by the engine."""


class NumericalFailure(RuntimeError):
    """Non-finite state or a violated low-Mach guard (solver.py:23)."""


def nvcc():
    for candidate in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if candidate and Path(candidate).exists():
            return candidate
    raise EngineError("nvcc not found; the CUDA toolkit is required to build the engine")


def build(force=False, verbose=False):
    """Compile the engine for sm_103a unless an up-to-date build exists."""
    newest = max(p.stat().st_mtime for p in SOURCES + HEADERS)
    if LIBRARY.exists() and not force and LIBRARY.stat().st_mtime >= newest:
        return LIBRARY
    LIBRARY.parent.mkdir(exist_ok=True)
    tmp = LIBRARY.with_name(f"{LIBRARY.name}.{os.getpid()}.tmp")
    cmd = [nvcc(), ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
           "-o", str(tmp), *map(str, SOURCES)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise EngineError("engine build failed:\n" + " ".join(cmd) + "\n" + proc.stderr[-4000:])
    os.replace(tmp, LIBRARY)
    return LIBRARY


class CaseDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
                ("origin_x", ctypes.c_double), ("origin_y", ctypes.c_double), ("dx", ctypes.c_double),
                ("omega_shear", ctypes.c_double), ("omega_bulk", ctypes.c_double), ("speed", ctypes.c_double),
                ("farfield", ctypes.c_int32), ("storage", ctypes.c_int32), ("n_elements", ctypes.c_int32),
                ("element_sizes", ctypes.POINTER(ctypes.c_int32)), ("polygon_xy", ctypes.POINTER(ctypes.c_double)),
                ("smagorinsky", ctypes.c_double)]


class RefinedDesc(ctypes.Structure):
    _fields_ = [("coarse", CaseDesc), ("tau_shear", ctypes.c_double), ("tau_bulk", ctypes.c_double),
                ("dt_coarse", ctypes.c_double), ("span", ctypes.c_double),
                ("box_lower", ctypes.c_int32 * 3), ("box_upper", ctypes.c_int32 * 3),
                ("fine_storage", ctypes.c_int32)]


class CaseInfo(ctypes.Structure):
    _fields_ = [("cells", ctypes.c_int64), ("fluid_cells", ctypes.c_int64), ("wall_keys", ctypes.c_int64),
                ("wall_links", ctypes.c_int64), ("outer_links", ctypes.c_int64),
                ("fallback_links", ctypes.c_int64), ("device_bytes", ctypes.c_int64),
                ("row_pitch", ctypes.c_int32), ("storage", ctypes.c_int32)]


_P = ctypes.c_void_p
_D = ctypes.c_double
SIGNATURES = {
    "ak_case_create": ([ctypes.POINTER(CaseDesc), ctypes.POINTER(_P)], ctypes.c_int),
    "ak_case_destroy": ([_P], ctypes.c_int),
    "ak_case_get_info": ([_P, ctypes.POINTER(CaseInfo)], ctypes.c_int),
    "ak_init_perturbed": ([_P, _D, _D, _D, _D, _D, _D], ctypes.c_int),
    "ak_init_fields": ([_P, _P, _P], ctypes.c_int),
    "ak_step": ([_P, ctypes.c_int32, _P], ctypes.c_int),
    "ak_step_loads_static": ([_P, ctypes.c_int32, _P], ctypes.c_int),
    "ak_steps_done": ([_P], ctypes.c_int64),
    "ak_kernel_launches": ([_P], ctypes.c_int64),
    "ak_case_stream": ([_P], _P),
    "ak_step_timed": ([_P, ctypes.c_int32, _P], ctypes.c_int),
    "ak_diagnostics": ([_P, _P], ctypes.c_int),
    "ak_macros": ([_P, _P, _P], ctypes.c_int),
    "ak_get_pdf": ([_P, _P], ctypes.c_int),
    "ak_set_pdf": ([_P, _P], ctypes.c_int),
    "ak_get_flags": ([_P, _P], ctypes.c_int),
    "ak_get_wall_links": ([_P, _P, _P], ctypes.c_int),
    "ak_refined_create": ([ctypes.POINTER(RefinedDesc), ctypes.POINTER(_P)], ctypes.c_int),
    "ak_refined_destroy": ([_P], ctypes.c_int),
    "ak_refined_init_perturbed": ([_P, _D, _D, _D, _D, _D], ctypes.c_int),
    "ak_refined_step": ([_P, ctypes.c_int32, _P], ctypes.c_int),
    "ak_refined_step_budget": ([_P, ctypes.c_int32, _P, _P, _P], ctypes.c_int),
    "ak_refined_steps_done": ([_P], ctypes.c_int64),
    "ak_refined_track_budget": ([_P, ctypes.c_int32], ctypes.c_int),
    "ak_refined_outer_flux": ([_P, _P], ctypes.c_int),
    "ak_refined_integrals": ([_P, _P], ctypes.c_int),
    "ak_refined_cumulative_loads": ([_P, _P], ctypes.c_int),
    "ak_boundary_state_size": ([_P, _P, _P], ctypes.c_int),
    "ak_get_boundary_state": ([_P, _P, _P], ctypes.c_int),
    "ak_set_boundary_state": ([_P, _P, _P], ctypes.c_int),
    "ak_set_steps_done": ([_P, ctypes.c_int64], ctypes.c_int),
    "ak_case_buffers": ([_P, _P, _P, _P, _P], ctypes.c_int),
    "ak_exterior_report": ([_P, _P], ctypes.c_int),
    "ak_residuals": ([_P, _D, _D, ctypes.c_int32, _P], ctypes.c_int),
    "ak_residual_snapshot": ([_P, ctypes.c_int32, _P, _P], ctypes.c_int),
    "ak_refined_restore_counters": ([_P, ctypes.c_int64, _P, _P], ctypes.c_int),
    "ak_batch_create": ([_P, ctypes.c_int32, _P], ctypes.c_int),
    "ak_batch_destroy": ([_P], ctypes.c_int),
    "ak_batch_step": ([_P, ctypes.c_int32, _P], ctypes.c_int),
    "ak_batch_tune": ([_P, ctypes.c_int32, _P], ctypes.c_int),
    "ak_batch_launches": ([_P], ctypes.c_int64),
    "ak_batch_steps_done": ([_P], ctypes.c_int64),
    "ak_batch_stream": ([_P], _P),
    "ak_refined_step_timed": ([_P, ctypes.c_int32, _P], ctypes.c_int),
    "ak_refined_level": ([_P, ctypes.c_int32], _P),
    "ak_refined_probe": ([_P, ctypes.c_int32, _P, _P], ctypes.c_int),
    "ak_refined_states": ([_P, _P, _P], ctypes.c_int),
    "ak_fma_peak": ([ctypes.c_int32, _P], ctypes.c_int),
    "ak_collision_flops": ([ctypes.c_int32, _P], ctypes.c_int),
    "ak_last_error": ([], ctypes.c_char_p),
    "ak_version": ([], ctypes.c_char_p),
}

_lib = None
_lock = threading.Lock()


def load(build_if_needed=True):
    """The loaded library (ctypes.CDLL) with every C-ABI signature declared."""
    global _lib
    with _lock:
        if _lib is None:
            path = build() if build_if_needed else LIBRARY
            lib = ctypes.CDLL(str(path))
            for name, (argtypes, restype) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.argtypes = argtypes
                fn.restype = restype
            _lib = lib
    return _lib


def check(code):
    if code == AK_OK:
        return
    message = load().ak_last_error().decode(errors="replace")
    if code == AK_ERR_INVALID or code == AK_ERR_GEOMETRY:
        raise ValueError(message)
    if code == AK_ERR_NOMEM:
        raise MemoryError(message)
    if code in (AK_ERR_NONFINITE, AK_ERR_GUARD):
        raise NumericalFailure(message)
    raise EngineError(message)
