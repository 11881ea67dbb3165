"""ctypes binding of libsofihost.so (include/sofihost.h): parameter files,
model preparation, acquisition and outputs on the host."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from ._native import BUILD

MAX_L = 8


class SofihPar(ctypes.Structure):
    _fields_ = [("weq", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("dh", ctypes.c_float),
                ("dt", ctypes.c_float), ("time", ctypes.c_float), ("nt", ctypes.c_int),
                ("fdorder", ctypes.c_int), ("maxrelerror", ctypes.c_int), ("L", ctypes.c_int),
                ("f_ref", ctypes.c_float), ("fl", ctypes.c_float * MAX_L), ("fw", ctypes.c_int),
                ("abs_type", ctypes.c_int), ("free_surf", ctypes.c_int), ("boundary", ctypes.c_int),
                ("npower", ctypes.c_float), ("k_max_cpml", ctypes.c_float), ("vppml", ctypes.c_float),
                ("fpml", ctypes.c_float), ("damping", ctypes.c_float), ("source_shape", ctypes.c_int),
                ("source_type", ctypes.c_int), ("run_multiple_shots", ctypes.c_int),
                ("source_file", ctypes.c_char * 256), ("seismo", ctypes.c_int), ("ndt", ctypes.c_int),
                ("readrec", ctypes.c_int), ("seis_format", ctypes.c_int), ("rec_file", ctypes.c_char * 256),
                ("seis_file", ctypes.c_char * 256), ("refrec", ctypes.c_float * 2), ("xrec1", ctypes.c_float),
                ("yrec1", ctypes.c_float), ("xrec2", ctypes.c_float), ("yrec2", ctypes.c_float),
                ("ngeoph", ctypes.c_int), ("snap", ctypes.c_int), ("snap_format", ctypes.c_int),
                ("tsnap1", ctypes.c_float), ("tsnap2", ctypes.c_float), ("tsnapinc", ctypes.c_float),
                ("idx", ctypes.c_int), ("idy", ctypes.c_int), ("snap_file", ctypes.c_char * 256),
                ("mfile", ctypes.c_char * 256), ("sigout", ctypes.c_int), ("sigout_format", ctypes.c_int),
                ("sigout_file", ctypes.c_char * 256), ("fdorder_time", ctypes.c_int),
                ("mode_fwi", ctypes.c_int), ("fwi_itermax", ctypes.c_int), ("fwi_velocity", ctypes.c_int),
                ("fwi_adjoint", ctypes.c_int), ("fwi_lnorm", ctypes.c_int), ("fwi_dtinv", ctypes.c_int),
                ("data_dir", ctypes.c_char * 256), ("gradient", ctypes.c_char * 256), ("readmod", ctypes.c_int),
                ("tau", ctypes.c_float), ("signal_file", ctypes.c_char * 256), ("rec_array", ctypes.c_int),
                ("drx", ctypes.c_int), ("rec_array_depth", ctypes.c_float), ("rec_array_dist", ctypes.c_float),
                ("rec_topo", ctypes.c_int), ("source_topo", ctypes.c_int), ("srcrec", ctypes.c_int),
                ("plane_wave_depth", ctypes.c_float), ("plane_wave_angle", ctypes.c_float), ("ts", ctypes.c_float),
                ("snapshot_start", ctypes.c_int), ("snapshot_end", ctypes.c_int), ("snapshot_incr", ctypes.c_int)]


_LIB = None


def load():
    global _LIB
    if _LIB is None:
        path = os.path.join(BUILD, "libsofihost.so")
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build gpi_project_gb300 first")
        L = ctypes.CDLL(path)
        P, vp, fp, ip = ctypes.POINTER, ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int)
        L.sofih_last_error.restype = ctypes.c_char_p
        L.sofih_read_par.argtypes = [ctypes.c_char_p, P(SofihPar)]
        L.sofih_prepare.argtypes = [P(SofihPar)] + [fp] * 8 + [ctypes.c_int, P(vp)]
        L.sofih_prep_free.argtypes = [vp]
        L.sofih_prep_num_fields.argtypes = [vp]
        L.sofih_prep_field_name.argtypes = [vp, ctypes.c_int]
        L.sofih_prep_field_name.restype = ctypes.c_char_p
        L.sofih_prep_field.argtypes = [vp, ctypes.c_int]
        L.sofih_prep_field.restype = fp
        L.sofih_prep_vector.argtypes = [vp, ctypes.c_char_p, P(fp)]
        L.sofih_holberg.argtypes = [ctypes.c_int, ctypes.c_int, fp]
        L.sofih_check_cfl.argtypes = [P(SofihPar), vp, fp]
        L.sofih_wavelet.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_int, fp, fp]
        L.sofih_wavelet_file.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_float, ctypes.c_int, fp, fp]
        L.sofih_read_signal.argtypes = [ctypes.c_char_p, ctypes.c_float, P(fp), ip]
        L.sofih_read_sources.argtypes = [P(SofihPar), ctypes.c_char_p, P(fp), P(fp), ip]
        L.sofih_read_receivers.argtypes = [P(SofihPar), ctypes.c_char_p, P(ip), P(ip), ip]
        L.sofih_write_signal.argtypes = [P(SofihPar), ctypes.c_int, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_float, ctypes.c_float, ctypes.c_char_p, ctypes.c_int]
        L.sofih_read_model.argtypes = [P(SofihPar), ctypes.c_char_p, P(fp), ctypes.c_int]
        L.sofih_model_suffixes.argtypes = [ctypes.c_int, P(ctypes.c_char_p), ctypes.c_int]
        L.sofih_write_su.argtypes = [ctypes.c_char_p, fp, ctypes.c_int, ctypes.c_int, ip, ip, ctypes.c_float,
                                     ctypes.c_float, P(SofihPar), ctypes.c_int, ctypes.c_int]
        L.sofih_write_su_traces.argtypes = [ctypes.c_char_p, fp, ctypes.c_int, ctypes.c_int, ip, ip, ip,
                                            ctypes.c_float, ctypes.c_float, P(SofihPar), ctypes.c_int, ctypes.c_int]
        L.sofih_read_receiver_traces.argtypes = [P(SofihPar), ctypes.c_char_p, P(ip), P(ip), P(ip), ip]
        L.sofih_scan_topo.argtypes = [P(SofihPar), ctypes.c_char_p, ip]
        L.sofih_snapshot_shots.argtypes = [P(SofihPar), ctypes.c_int, ip]
        L.sofih_write_snap_format.argtypes = [ctypes.c_char_p, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.sofih_seis_ext.argtypes = [ctypes.c_int]
        L.sofih_seis_ext.restype = ctypes.c_char_p
        L.sofih_write_seis.argtypes = [ctypes.c_char_p, fp, ctypes.c_int, ctypes.c_int, ip, ip, ip, ctypes.c_float,
                                       ctypes.c_float, P(SofihPar), ctypes.c_int, ctypes.c_int]
        L.sofih_fwi_read_data.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, fp]
        L.sofih_fwi_residual.argtypes = [fp, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, fp,
                                         P(ctypes.c_double)]
        L.sofih_fwi_model_gradients.argtypes = [ctypes.c_size_t] + [fp] * 9
        L.sofih_fwi_model_gradients.restype = None
        L.sofih_write_gradient.argtypes = [ctypes.c_char_p, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        _LIB = L
    return _LIB


def _err():
    return RuntimeError(load().sofih_last_error().decode())


def _fp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def read_par(path: str) -> SofihPar:
    p = SofihPar()
    if load().sofih_read_par(path.encode(), ctypes.byref(p)):
        raise _err()
    return p


def make_par(**kw) -> SofihPar:
    p = SofihPar()
    p.npower, p.k_max_cpml, p.damping, p.ndt, p.idx, p.idy, p.readrec = 2.0, 1.0, 8.0, 1, 1, 1, 1
    p.fdorder_time = 2
    p.readmod, p.tau = 1, 0.0001
    p.srcrec, p.snapshot_start, p.snapshot_end, p.snapshot_incr, p.snap_format, p.seis_format = 1, 1, -9999, 1, 3, 1
    for k, v in kw.items():
        if k == "fl":
            for i, f in enumerate(v):
                p.fl[i] = f
        elif k == "refrec":
            p.refrec[0], p.refrec[1] = v
        else:
            setattr(p, k, v)
    return p


def prepare(p: SofihPar, mats: dict, nthreads: int = 0):
    """Prepared model: (fields {name: [NY][NX]}, vectors {name: array})."""
    L = load()
    order = ["vp", "vs", "rho", "qp", "qs", "epsilon", "delta", "theta"]
    arrs = [None if mats.get(k) is None else np.ascontiguousarray(mats[k], dtype=np.float32).reshape(-1)
            for k in order]
    h = ctypes.c_void_p()
    if L.sofih_prepare(ctypes.byref(p), *[_fp(a) for a in arrs], nthreads, ctypes.byref(h)):
        raise _err()
    try:
        fields = {}
        for k in range(L.sofih_prep_num_fields(h)):
            name = L.sofih_prep_field_name(h, k).decode()
            ptr = L.sofih_prep_field(h, k)
            fields[name] = np.ctypeslib.as_array(ptr, shape=(p.ny, p.nx)).copy()
        vecs = {}
        for name in ["K_x", "a_x", "b_x", "K_x_half", "a_x_half", "b_x_half", "K_y", "a_y", "b_y", "K_y_half",
                     "a_y_half", "b_y_half", "bip", "cip", "peta"]:
            d = ctypes.POINTER(ctypes.c_float)()
            n = L.sofih_prep_vector(h, name.encode(), ctypes.byref(d))
            if n:
                vecs[name] = np.ctypeslib.as_array(d, shape=(n,)).copy()
        dtmax = ctypes.c_float()
        stable = L.sofih_check_cfl(ctypes.byref(p), h, ctypes.byref(dtmax)) == 0
        vecs["_dt_max"] = np.array([dtmax.value], np.float32)
        vecs["_stable"] = np.array([stable], np.int32)
    finally:
        L.sofih_prep_free(h)
    return fields, vecs


def holberg(fdorder: int, maxrelerror: int) -> np.ndarray:
    hc = np.zeros(7, np.float32)
    if load().sofih_holberg(fdorder, maxrelerror, _fp(hc)):
        raise _err()
    return hc


def wavelet(shape: int, nt: int, dt: float, srcpos: np.ndarray, signal_file: str | None = None) -> np.ndarray:
    """Source signals [nsrc][nt] (wavelet.c); SOURCE_SHAPE 3 reads `signal_file`."""
    sp = np.ascontiguousarray(srcpos, dtype=np.float32)
    out = np.empty((sp.shape[1], nt), np.float32)
    if shape == 3:
        rc = load().sofih_wavelet_file((signal_file or "").encode(), nt, dt, sp.shape[1], _fp(sp), _fp(out))
    else:
        rc = load().sofih_wavelet(shape, nt, dt, sp.shape[1], _fp(sp), _fp(out))
    if rc:
        raise _err()
    return out


def read_signal(path: str, dt: float) -> np.ndarray:
    """Samples of a SOURCE_SHAPE 3 signal file (read_srcsig.c)."""
    smp, n = ctypes.POINTER(ctypes.c_float)(), ctypes.c_int()
    L = load()
    if L.sofih_read_signal(path.encode(), dt, ctypes.byref(smp), ctypes.byref(n)):
        raise _err()
    out = np.ctypeslib.as_array(smp, shape=(n.value,)).copy()
    ctypes.CDLL(None).free(smp)
    return out


def read_sources(p: SofihPar, path: str):
    L = load()
    sp, xy, n = ctypes.POINTER(ctypes.c_float)(), ctypes.POINTER(ctypes.c_float)(), ctypes.c_int()
    if L.sofih_read_sources(ctypes.byref(p), path.encode(), ctypes.byref(sp), ctypes.byref(xy), ctypes.byref(n)):
        raise _err()
    n = n.value
    return (np.ctypeslib.as_array(sp, shape=(12, n)).copy(), np.ctypeslib.as_array(xy, shape=(2, n)).copy())


def read_receivers(p: SofihPar, path: str):
    L = load()
    ix, iy, n = ctypes.POINTER(ctypes.c_int)(), ctypes.POINTER(ctypes.c_int)(), ctypes.c_int()
    if L.sofih_read_receivers(ctypes.byref(p), path.encode(), ctypes.byref(ix), ctypes.byref(iy), ctypes.byref(n)):
        raise _err()
    n = n.value
    return (np.ctypeslib.as_array(ix, shape=(n,)).copy(), np.ctypeslib.as_array(iy, shape=(n,)).copy())


def read_receiver_traces(p: SofihPar, path: str):
    """(ix, iy, trace numbers) as sofih_read_receiver_traces gives them."""
    L = load()
    ipp = ctypes.POINTER(ctypes.c_int)
    ix, iy, tr, n = ipp(), ipp(), ipp(), ctypes.c_int()
    if L.sofih_read_receiver_traces(ctypes.byref(p), path.encode(), ctypes.byref(ix), ctypes.byref(iy),
                                    ctypes.byref(tr), ctypes.byref(n)):
        raise _err()
    n = n.value
    return tuple(np.ctypeslib.as_array(a, shape=(n,)).copy() for a in (ix, iy, tr))


def scan_topo(p: SofihPar, mfile: str) -> np.ndarray:
    """The topography row of every column (sofih_scan_topo)."""
    topo = np.zeros(p.nx, dtype=np.int32)
    if load().sofih_scan_topo(ctypes.byref(p), mfile.encode(), topo.ctypes.data_as(ctypes.POINTER(ctypes.c_int))):
        raise _err()
    return topo


def write_seis(path: str, section, ix, iy, xs: float, ys: float, p: SofihPar, ishot: int = 1, comp: int = 1,
               trace=None):
    """One seismogram file in p.seis_format (sofih_write_seis)."""
    sec = np.ascontiguousarray(section, dtype=np.float32)
    ix = np.ascontiguousarray(ix, dtype=np.int32)
    iy = np.ascontiguousarray(iy, dtype=np.int32)
    ipp = ctypes.POINTER(ctypes.c_int)
    tr = None if trace is None else np.ascontiguousarray(trace, dtype=np.int32)
    if load().sofih_write_seis(path.encode(), _fp(sec), sec.shape[0], sec.shape[1], ix.ctypes.data_as(ipp),
                               iy.ctypes.data_as(ipp), None if tr is None else tr.ctypes.data_as(ipp), xs, ys,
                               ctypes.byref(p), ishot, comp):
        raise _err()


def write_snap(path: str, frame, append: bool = False, fmt: int = 3):
    """Append (or start) a snapshot file in SNAP_FORMAT fmt (sofih_write_snap_format)."""
    f = np.ascontiguousarray(frame, dtype=np.float32).reshape(-1)
    if load().sofih_write_snap_format(path.encode(), _fp(f), f.size, int(append), fmt):
        raise _err()


def seis_ext(fmt: int):
    v = load().sofih_seis_ext(fmt)
    return v.decode() if v is not None else None


def snapshot_shots(p: SofihPar, nshots: int) -> list:
    """The 1-based shots whose snapshots the files hold, in order, after nshots shots."""
    out = np.zeros(max(nshots, 1), dtype=np.int32)
    n = load().sofih_snapshot_shots(ctypes.byref(p), nshots, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return [int(v) for v in out[:n]]


def write_su(path: str, section, ix, iy, xs: float, ys: float, p: SofihPar, ishot: int = 1, comp: int = 1,
             trace=None):
    """One SU file; trace: the traces' numbers (None: 1..ntr)."""
    sec = np.ascontiguousarray(section, dtype=np.float32)
    ix = np.ascontiguousarray(ix, dtype=np.int32)
    iy = np.ascontiguousarray(iy, dtype=np.int32)
    ipp = ctypes.POINTER(ctypes.c_int)
    tr = None if trace is None else np.ascontiguousarray(trace, dtype=np.int32)
    if load().sofih_write_su_traces(path.encode(), _fp(sec), sec.shape[0], sec.shape[1], ix.ctypes.data_as(ipp),
                                    iy.ctypes.data_as(ipp), None if tr is None else tr.ctypes.data_as(ipp), xs, ys,
                                    ctypes.byref(p), ishot, comp):
        raise _err()


def write_signal(p: SofihPar, ishot: int, signal, ix: int, iy: int, xs: float, ys: float) -> str:
    """Source wavelet file <SIGOUT_FILE>.shot<ishot>.<ext> (initsrc.c:64-93); returns its path."""
    sig = np.ascontiguousarray(signal, dtype=np.float32).reshape(-1)
    buf = ctypes.create_string_buffer(600)
    if load().sofih_write_signal(ctypes.byref(p), ishot, _fp(sig), sig.size, ix, iy, xs, ys, buf, 600):
        raise _err()
    return buf.value.decode()


def read_model(p: SofihPar, mfile: str) -> dict:
    """Material arrays [NX][NY] of MFILE.<suffix> (binary) or MFILE.<suffix>.su."""
    L = load()
    names = (ctypes.c_char_p * 8)()
    n = L.sofih_model_suffixes(p.weq, names, 8)
    out = (ctypes.POINTER(ctypes.c_float) * 8)()
    if L.sofih_read_model(ctypes.byref(p), mfile.encode(), out, 8):
        raise _err()
    libc = ctypes.CDLL(None)
    res = {}
    for k in range(n):
        res[names[k].decode()] = np.ctypeslib.as_array(out[k], shape=(p.nx, p.ny)).copy()
        libc.free(ctypes.cast(out[k], ctypes.c_void_p))
    return res


# ---- FWI gradient pass (host side)
def fwi_read_data(path: str, ntr: int, ns: int) -> np.ndarray:
    """The first ntr traces of ns samples of an observed SU file (inseis.c)."""
    out = np.empty((ntr, ns), dtype=np.float32)
    if load().sofih_fwi_read_data(path.encode(), ntr, ns, _fp(out)):
        raise _err()
    return out


def fwi_residual(calc, data, velocity: int, dt: float) -> tuple:
    """calc_res.c (LNORM 2): the time-reversed residual [ntr][ns] and its L2."""
    c = np.ascontiguousarray(calc, dtype=np.float32)
    d = np.ascontiguousarray(data, dtype=np.float32)
    assert c.shape == d.shape
    out = np.empty_like(c)
    l2 = ctypes.c_double()
    if load().sofih_fwi_residual(_fp(c), _fp(d), c.shape[0], c.shape[1], velocity, dt, _fp(out), ctypes.byref(l2)):
        raise _err()
    return out, l2.value


def fwi_model_gradients(lam, mu, rhos, vp, vs, rho) -> tuple:
    """inversion.c:225-240: (vp, vs, rho') gradients, any common layout."""
    a = [np.ascontiguousarray(x, dtype=np.float32) for x in (lam, mu, rhos, vp, vs, rho)]
    out = [np.empty_like(a[0]) for _ in range(3)]
    load().sofih_fwi_model_gradients(a[0].size, *[_fp(x) for x in a + out])
    return tuple(out)


def write_gradient(path: str, g, idx: int = 1, idy: int = 1):
    """A [ny][nx] gradient file as the reference writes it (writemod.c, format 3)."""
    a = np.ascontiguousarray(g, dtype=np.float32)
    if load().sofih_write_gradient(path.encode(), _fp(a), a.shape[1], a.shape[0], idx, idy):
        raise _err()
