"""ctypes binding of libsofigpu.so (include/sofigpu.h).

There is no fallback: if the native library is missing or cannot load, every
entry point raises. Build it with ``gpi_project_gb300.build.build()``.
"""
from __future__ import annotations

import ctypes
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build")
HEADER = os.path.join(REPO, "include", "sofigpu.h")

SOFI_OK, SOFI_E_ARG, SOFI_E_CUDA, SOFI_E_STATE, SOFI_E_NOMEM, SOFI_E_UNSTABLE, SOFI_E_NODEV = range(7)


class SofiError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[sofi error {code}] {msg}")
        self.code = code


class UnstableError(SofiError):
    pass


class SofiConfig(ctypes.Structure):
    """sofi_config of include/sofigpu.h (the GlobVar fields time_loop reads)."""
    _fields_ = [(n, t) for n, t in [
        ("weq", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("fdorder", ctypes.c_int),
        ("maxrelerror", ctypes.c_int), ("L", ctypes.c_int), ("dt", ctypes.c_float), ("dh", ctypes.c_float),
        ("nt", ctypes.c_int), ("fw", ctypes.c_int), ("abs_type", ctypes.c_int), ("free_surf", ctypes.c_int),
        ("boundary", ctypes.c_int), ("seismo", ctypes.c_int), ("ndt", ctypes.c_int), ("snap", ctypes.c_int),
        ("snap_first", ctypes.c_int), ("snap_inc", ctypes.c_int), ("snap_last", ctypes.c_int),
        ("idx", ctypes.c_int), ("idy", ctypes.c_int), ("nshots", ctypes.c_int), ("shared_model", ctypes.c_int),
        ("fdorder_time", ctypes.c_int)]]


class TtiStressArgs(ctypes.Structure):
    """sofi_tti_stress_args of include/sofigpu.h (device pointers as integers)."""
    _fields_ = ([(k, ctypes.c_void_p) for k in
                 ["vx", "vy", "sxx", "syy", "sxy", "r", "p", "q", "psi_vxx", "psi_vyx", "psi_vyy", "psi_vxy",
                  "c11", "c13", "c33", "c15", "c35", "c55ipjp", "c15ipjp", "c35ipjp", "c11d_base", "c13d_base",
                  "c33d_base", "c15d_base", "c35d_base", "c55ipjpd_base", "c15ipjpd_base", "c35ipjpd_base",
                  "absorb", "K_x", "a_x", "b_x", "K_x_half", "a_x_half", "b_x_half", "K_y", "a_y", "b_y",
                  "K_y_half", "a_y_half", "b_y_half"]]
                + [("bip", ctypes.c_float * 8), ("cip", ctypes.c_float * 8), ("peta", ctypes.c_float * 8),
                   ("hc", ctypes.c_float * 7)])


NOALLOC_MAX_CELLS = 1 << 20
_LIB = None


def padded_shape(nx: int, ny: int) -> tuple:
    """(rows, pitch) of one 2-D field in the library's device layout."""
    return ny + 16, ((nx + 16 + 31) // 32) * 32


def lib_path() -> str:
    return os.path.join(BUILD, "libsofigpu.so")


def load():
    """Load libsofigpu.so (raises if absent: the CUDA path is the only path)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build the CUDA extension first "
                           "(python -c 'import gpi_project_gb300.build as b; b.build()')")
    L = ctypes.CDLL(path)
    P = ctypes.POINTER
    fp, ip, vp = P(ctypes.c_float), P(ctypes.c_int), ctypes.c_void_p
    sig = {
        "sofi_create": ([P(SofiConfig), ctypes.c_int, P(vp)], ctypes.c_int),
        "sofi_destroy": ([vp], ctypes.c_int),
        "sofi_last_error": ([], ctypes.c_char_p),
        "sofi_abi_version": ([], ctypes.c_int),
        "sofi_device_bytes": ([P(SofiConfig), P(ctypes.c_longlong)], ctypes.c_int),
        "sofi_set_hc": ([vp, fp], ctypes.c_int),
        "sofi_set_model_field": ([vp, ctypes.c_int, ctypes.c_char_p, fp, ctypes.c_long, ctypes.c_long], ctypes.c_int),
        "sofi_set_model_vector": ([vp, ctypes.c_char_p, fp, ctypes.c_int], ctypes.c_int),
        "sofi_set_sources": ([vp, ctypes.c_int, ctypes.c_int, fp, fp], ctypes.c_int),
        "sofi_set_receivers": ([vp, ctypes.c_int, ctypes.c_int, ip, ip], ctypes.c_int),
        "sofi_reset": ([vp, ctypes.c_int], ctypes.c_int),
        "sofi_run": ([vp, ctypes.c_int], ctypes.c_int),
        "sofi_synchronize": ([vp], ctypes.c_int),
        "sofi_current_step": ([vp, ip], ctypes.c_int),
        "sofi_get_section": ([vp, ctypes.c_int, ctypes.c_int, fp], ctypes.c_int),
        "sofi_num_samples": ([vp, ip], ctypes.c_int),
        "sofi_get_field": ([vp, ctypes.c_int, ctypes.c_char_p, fp], ctypes.c_int),
        "sofi_set_field": ([vp, ctypes.c_int, ctypes.c_char_p, fp], ctypes.c_int),
        "sofi_num_snapshots": ([vp, ip, ip], ctypes.c_int),
        "sofi_get_snapshot": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, fp], ctypes.c_int),
        "sofi_last_run_ms": ([vp, fp], ctypes.c_int),
        "sofi_set_kernel_timing": ([vp, ctypes.c_int], ctypes.c_int),
        "sofi_kernel_time": ([vp, ctypes.c_char_p, P(ctypes.c_double), P(ctypes.c_longlong)], ctypes.c_int),
        "sofi_launch_count": ([vp, P(ctypes.c_longlong)], ctypes.c_int),
        "sofi_velocity_variant": ([vp, P(ctypes.c_int), P(ctypes.c_int)], ctypes.c_int),
        "sofi_stress_variant": ([vp, P(ctypes.c_int)], ctypes.c_int),
        "sofi_pdl": ([vp, P(ctypes.c_int)], ctypes.c_int),
        "sofi_block_threads_x": ([vp, P(ctypes.c_int), P(ctypes.c_int)], ctypes.c_int),
        "sofi_post_fused": ([vp, P(ctypes.c_int)], ctypes.c_int),
        "sofi_set_pdl": ([vp, ctypes.c_int], ctypes.c_int),
        "sofi_fwi_begin": ([vp, ctypes.c_int, ctypes.c_int, P(ctypes.c_float), P(ctypes.c_float),
                            P(ctypes.c_float)], ctypes.c_int),
        "sofi_fwi_backward": ([vp, P(ctypes.c_float), P(ctypes.c_float)], ctypes.c_int),
        "sofi_fwi_gradients": ([vp, P(ctypes.c_float), P(ctypes.c_float), P(ctypes.c_float)], ctypes.c_int),
        "sofi_fwi_checkpoints": ([vp, P(ctypes.c_int), P(ctypes.c_int)], ctypes.c_int),
        "sofi_get_stream": ([vp, P(vp)], ctypes.c_int),
        "sofi_tti_stress_noalloc": ([P(SofiConfig), P(TtiStressArgs), vp], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _LIB = L
    return L


def check(rc: int):
    if rc != SOFI_OK:
        msg = load().sofi_last_error().decode(errors="replace")
        if rc == SOFI_E_UNSTABLE:
            raise UnstableError(rc, msg)
        raise SofiError(rc, msg)


def declared_symbols(header: str = HEADER) -> list:
    """Function names declared in a public header of include/."""
    txt = open(header).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_]+\s*\*?\s*(sofi_[a-z0-9_]+)\s*\(", txt, re.M)))
