"""ctypes binding of libsofiserve.so (include/sofiserve.h): the continuous-
batching request loop that keeps many forward-modelling solves resident on one
GPU and advances them chunk by chunk on their own priority streams."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import host as H
from ._native import BUILD

REQ_WAITING, REQ_PREPARING, REQ_READY, REQ_RESIDENT, REQ_DONE, REQ_FAILED = range(6)

_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int)


class SofiRequest(ctypes.Structure):
    _fields_ = [("par", H.SofihPar), ("vp", _fp), ("vs", _fp), ("rho", _fp), ("qp", _fp), ("qs", _fp),
                ("eps", _fp), ("del_", _fp), ("theta", _fp), ("nsrc", ctypes.c_int), ("srcpos", _fp),
                ("ntr", ctypes.c_int), ("rec_ix", _ip), ("rec_iy", _ip), ("arrival", ctypes.c_double)]


class SofiRequestInfo(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int), ("status", ctypes.c_int), ("error", ctypes.c_char * 256),
                ("arrival", ctypes.c_double), ("ready", ctypes.c_double), ("admitted", ctypes.c_double),
                ("finished", ctypes.c_double), ("device_bytes", ctypes.c_longlong), ("priority", ctypes.c_int),
                ("ntr", ctypes.c_int), ("ns", ctypes.c_int), ("cell_updates", ctypes.c_double),
                ("launches", ctypes.c_longlong)]


class SofiServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int), ("completed", ctypes.c_int), ("failed", ctypes.c_int),
                ("p50_s", ctypes.c_double), ("p99_s", ctypes.c_double), ("mean_s", ctypes.c_double),
                ("max_s", ctypes.c_double), ("first_arrival", ctypes.c_double), ("last_finish", ctypes.c_double),
                ("shots_per_s", ctypes.c_double), ("gcell_per_s", ctypes.c_double),
                ("peak_bytes", ctypes.c_longlong), ("peak_resident", ctypes.c_int), ("launches", ctypes.c_longlong)]


class SofiServerOptions(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("hbm_budget", ctypes.c_longlong), ("max_resident", ctypes.c_int),
                ("chunk_steps", ctypes.c_int), ("depth", ctypes.c_int), ("prep_threads", ctypes.c_int),
                ("prep_omp_threads", ctypes.c_int), ("use_priorities", ctypes.c_int),
                ("largest_first", ctypes.c_int)]


DECLARED = ["sofi_server_last_error", "sofi_server_default_options", "sofi_server_create", "sofi_server_destroy",
            "sofi_server_clock", "sofi_server_submit", "sofi_server_poll", "sofi_server_drain",
            "sofi_server_info", "sofi_server_section", "sofi_server_stats_get", "sofi_server_plan",
            "sofi_server_priority", "sofi_server_percentile"]

_LIB = None


def load():
    """libsofiserve.so with argument types; raises if it was not built."""
    global _LIB
    if _LIB is None:
        path = os.path.join(BUILD, "libsofiserve.so")
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build gpi_project_gb300 first")
        L = ctypes.CDLL(path)
        P, vp = ctypes.POINTER, ctypes.c_void_p
        L.sofi_server_last_error.restype = ctypes.c_char_p
        L.sofi_server_default_options.argtypes = [P(SofiServerOptions)]
        L.sofi_server_create.argtypes = [P(SofiServerOptions), P(vp)]
        L.sofi_server_destroy.argtypes = [vp]
        L.sofi_server_clock.argtypes = [vp]
        L.sofi_server_clock.restype = ctypes.c_double
        L.sofi_server_submit.argtypes = [vp, P(SofiRequest), _ip]
        L.sofi_server_poll.argtypes = [vp, _ip]
        L.sofi_server_drain.argtypes = [vp]
        L.sofi_server_info.argtypes = [vp, ctypes.c_int, P(SofiRequestInfo)]
        L.sofi_server_section.argtypes = [vp, ctypes.c_int, ctypes.c_int, _fp]
        L.sofi_server_stats_get.argtypes = [vp, P(SofiServerStats)]
        L.sofi_server_plan.argtypes = [P(ctypes.c_longlong), ctypes.c_int, ctypes.c_longlong, ctypes.c_longlong,
                                       ctypes.c_int, ctypes.c_int, _ip]
        L.sofi_server_priority.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_int]
        L.sofi_server_percentile.argtypes = [P(ctypes.c_double), ctypes.c_int, ctypes.c_double]
        L.sofi_server_percentile.restype = ctypes.c_double
        _LIB = L
    return _LIB


def _check(rc: int):
    if rc:
        raise RuntimeError(f"[sofi serve error {rc}] {load().sofi_server_last_error().decode()}")


def plan(bytes_, in_use: int, budget: int, resident: int, max_resident: int) -> list[int]:
    """Admission decision of the loop for ready requests in arrival order."""
    b = np.ascontiguousarray(bytes_, dtype=np.int64)
    out = np.zeros(max(len(b), 1), np.int32)
    load().sofi_server_plan(b.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)), len(b), in_use, budget, resident,
                            max_resident, out.ctypes.data_as(_ip))
    return out[:len(b)].tolist()


def priority(cell_updates: float, least: int, greatest: int) -> int:
    return load().sofi_server_priority(float(cell_updates), least, greatest)


def percentile(x, q: float) -> float:
    a = np.ascontiguousarray(x, dtype=np.float64)
    return load().sofi_server_percentile(a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(a), q)


class Server:
    """One request loop on one device. ``submit`` keeps the request's arrays
    alive until the server is closed."""

    def __init__(self, device: int = 0, hbm_budget: int = 0, max_resident: int = 64, chunk_steps: int = 32,
                 depth: int = 2, prep_threads: int = 2, prep_omp_threads: int = 0, use_priorities: bool = True,
                 largest_first: bool = False):
        self.lib = load()
        o = SofiServerOptions()
        self.lib.sofi_server_default_options(ctypes.byref(o))
        o.device, o.hbm_budget, o.max_resident, o.chunk_steps = device, hbm_budget, max_resident, chunk_steps
        o.depth, o.prep_threads, o.prep_omp_threads = depth, prep_threads, prep_omp_threads
        o.use_priorities = 1 if use_priorities else 0
        o.largest_first = 1 if largest_first else 0
        self.h = ctypes.c_void_p()
        _check(self.lib.sofi_server_create(ctypes.byref(o), ctypes.byref(self.h)))
        self._keep = []

    def clock(self) -> float:
        return self.lib.sofi_server_clock(self.h)

    def submit(self, par: H.SofihPar, mats: dict, srcpos, rec_ix, rec_iy, arrival: float = -1.0) -> int:
        """Queue one solve: material arrays [NX][NY] (vp vs rho [qp qs] ...),
        srcpos [12][nsrc] in grid indices, receiver grid indices."""
        keep = {k: np.ascontiguousarray(v, dtype=np.float32) for k, v in mats.items() if v is not None}
        sp = np.ascontiguousarray(srcpos, dtype=np.float32)
        ix = np.ascontiguousarray(rec_ix, dtype=np.int32)
        iy = np.ascontiguousarray(rec_iy, dtype=np.int32)
        r = SofiRequest()
        r.par = par

        def f(name):
            a = keep.get(name)
            return None if a is None else a.ctypes.data_as(_fp)

        r.vp, r.vs, r.rho, r.qp, r.qs = f("vp"), f("vs"), f("rho"), f("qp"), f("qs")
        r.eps, r.del_, r.theta = f("epsilon"), f("delta"), f("theta")
        r.nsrc, r.srcpos = sp.shape[1], sp.ctypes.data_as(_fp)
        r.ntr, r.rec_ix, r.rec_iy = len(ix), ix.ctypes.data_as(_ip), iy.ctypes.data_as(_ip)
        r.arrival = arrival
        rid = ctypes.c_int()
        _check(self.lib.sofi_server_submit(self.h, ctypes.byref(r), ctypes.byref(rid)))
        self._keep.append((keep, sp, ix, iy))
        return rid.value

    def poll(self) -> int:
        a = ctypes.c_int()
        _check(self.lib.sofi_server_poll(self.h, ctypes.byref(a)))
        return a.value

    def drain(self):
        _check(self.lib.sofi_server_drain(self.h))

    def info(self, rid: int) -> dict:
        i = SofiRequestInfo()
        _check(self.lib.sofi_server_info(self.h, rid, ctypes.byref(i)))
        return {k: (getattr(i, k).decode() if k == "error" else getattr(i, k)) for k, _ in i._fields_}

    def section(self, rid: int, comp: int) -> np.ndarray:
        i = self.info(rid)
        out = np.empty((i["ntr"], i["ns"]), np.float32)
        _check(self.lib.sofi_server_section(self.h, rid, comp, out.ctypes.data_as(_fp)))
        return out

    def stats(self) -> dict:
        s = SofiServerStats()
        _check(self.lib.sofi_server_stats_get(self.h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.sofi_server_destroy(self.h)
            self.h = ctypes.c_void_p()
        self._keep = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
