"""ctypes binding of libgbattract (include/gbattract.h).

This is the reference-facing boundary as Python sees it: every call goes
through the C ABI.  The library must have been built (build.py); importing
this module on a machine without it raises, there is no fallback path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .model import MODES_MAX

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libgbattract.so"

GBA_OK = 0
ERRORS = {1: "invalid argument", 2: "unknown id", 3: "CUDA error", 4: "out of memory",
          5: "timeout", 6: "no device", 7: "device check"}


class IntrplDescC(C.Structure):
    _fields_ = [("numGrids", C.c_uint32), ("dimN", C.c_uint32 * 3),
                ("gridSpacing", C.c_float), ("posMin", C.c_float * 3)]


class NLDescC(C.Structure):
    _fields_ = [("dimN", C.c_uint32 * 3), ("gridSpacing", C.c_float), ("dPlateau", C.c_float),
                ("posMin", C.c_float * 3), ("numEl", C.c_uint32)]


class GridBuildOptsC(C.Structure):
    _fields_ = [("spacing", C.c_float), ("plateau", C.c_float), ("nl_cutoff", C.c_float),
                ("margin", C.c_float), ("outer_ext", C.c_uint32), ("n_alphabet", C.c_uint32),
                ("alphabet", C.c_uint32 * 99)]


class PairJobC(C.Structure):
    _fields_ = [("rec", C.c_uint32), ("lig", C.c_uint32), ("grid", C.c_uint32),
                ("params", C.c_uint32), ("start", C.c_void_p), ("n", C.c_size_t),
                ("out_state", C.c_void_p), ("out_result", C.c_void_p),
                ("out_nevals", C.c_void_p), ("out_done_ns", C.c_void_p)]


class TuneResultC(C.Structure):
    _fields_ = [("energy_threads", C.c_int), ("energy_blocks_per_sm", C.c_int),
                ("minimize_threads", C.c_int), ("minimize_chunk", C.c_int),
                ("energy_ms", C.c_float), ("minimize_ms", C.c_float), ("from_cache", C.c_int),
                ("minimize_team", C.c_int)]


class GbaError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gbattract error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


_lib = None


def load() -> C.CDLL:
    """Loads libgbattract.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"libgbattract.so not built ({LIB_PATH}); run build()")
    lib = C.CDLL(str(LIB_PATH))
    P, U32, SZ, I = C.c_void_p, C.c_uint32, C.c_size_t, C.c_int
    sig = {
        "gba_version": ([], C.c_char_p),
        "gba_create": ([I, C.POINTER(P)], I),
        "gba_destroy": ([P], I),
        "gba_last_error": ([P], C.c_char_p),
        "gba_upload_protein": ([P, U32, P, P, P, P, U32, P, P, C.POINTER(U32)], I),
        "gba_upload_grid": ([P, C.POINTER(IntrplDescC), P, C.POINTER(IntrplDescC), P,
                             C.POINTER(NLDescC), P, P, C.POINTER(U32)], I),
        "gba_upload_params": ([P, U32, P, I, I, C.c_float, C.POINTER(U32)], I),
        "gba_release": ([P, U32], I),
        "gba_energy_6d": ([P, U32, U32, U32, U32, P, SZ, P, P], I),
    }
    optional = {
        "gba_energy_6d_modes": ([P, U32, U32, U32, U32, U32, P, SZ, P, P], I),
        "gba_build_grid": ([P, U32, U32, C.POINTER(GridBuildOptsC), C.POINTER(U32)], I),
        "gba_grid_info": ([P, U32, C.POINTER(IntrplDescC), C.POINTER(IntrplDescC),
                           C.POINTER(NLDescC)], I),
        "gba_download_grid": ([P, U32, P, P, P, P], I),
        "gba_census_6d": ([P, U32, U32, U32, U32, P, SZ, P, P], I),
        "gba_minimize_6d": ([P, U32, U32, U32, U32, P, SZ, I, P, P, P, P], I),
        "gba_minimize_6d_plain": ([P, U32, U32, U32, U32, P, SZ, I, SZ, P, P, P, P], I),
        "gba_batch_minimize_6d": ([P, C.POINTER(PairJobC), SZ, I, P], I),
        "gba_batch_energy_6d": ([P, C.POINTER(PairJobC), SZ, P], I),
        "gba_set_deadline": ([P, U32], I),
        "gba_set_minimize_team": ([P, I], I),
        "gba_set_pose_order": ([P, I], I),
        "gba_kernel_timing": ([P, C.c_int32], I),
        "gba_set_kernel_options": ([P, C.c_uint32], I),
        "gba_set_host_sincos": ([P, C.c_float], I),
        "gba_energy_6d_noalloc": ([P, U32, U32, U32, U32, P, SZ, P, P], I),
        "gba_allocation_count": ([C.POINTER(C.c_uint64)], I),
        "gba_kernel_time": ([P, C.POINTER(C.c_double), C.POINTER(C.c_uint64), C.c_int32], I),
        "gba_grid_octets": ([P, U32, I], I),
        "gba_autotune": ([P, U32, U32, U32, U32, P, SZ, I, C.c_char_p, C.POINTER(TuneResultC)], I),
        "gba_set_pair_shape": ([P, U32, U32, U32, U32, C.POINTER(TuneResultC)], I),
        "gba_minimize_6d_modes": ([P, U32, U32, U32, U32, U32, P, SZ, I, P, P, P, P], I),
        "gba_minimize_6d_modes_plain": ([P, U32, U32, U32, U32, U32, P, SZ, I, SZ, P, P, P, P], I),
    }
    for name, (args, res) in {**sig, **optional}.items():
        try:
            f = getattr(lib, name)
        except AttributeError:
            if name in sig:
                raise
            continue
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


def exported_symbols() -> list:
    """Names declared in include/*.h that the loaded library exports."""
    lib = load()
    return [n for n in declared_symbols() if hasattr(lib, n)]


def declared_symbols() -> list:
    """Function names declared in the C headers under include/."""
    import re
    names = set()
    for hdr in sorted((Path(__file__).resolve().parent.parent / "include").glob("*.h")):
        names.update(re.findall(r"\b(gba_[a-z0-9_]+)\s*\(", hdr.read_text()))
    return sorted(names)


def ptr(a) -> int | None:
    """Address of a numpy array, torch tensor (host or device) or None."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    raise TypeError(f"cannot take the address of {type(a)}")


def check(ctx, rc: int) -> None:
    if rc != GBA_OK:
        msg = load().gba_last_error(ctx)
        raise GbaError(rc, msg.decode() if msg else "")


MODES_WIDTH = 6 + 2 * MODES_MAX
