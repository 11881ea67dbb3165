"""Python binding of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg and
reference arm may import this module; the product (``gpi_project_gb300``)
never does. It wraps ``liboracle_f32.so`` / ``liboracle_f64.so`` (the C
restatement in sofi_oracle.c) and restates the reference's file readers so a
reference example (JSON + model + source + receiver files) can be run end to
end:

* ``read_par_json``  -- reference src/json_parser.c:52-140 (line-oriented
  ``"KEY" : "VALUE"`` pairs, comma-joined multi-keys, lines mentioning
  "comment" skipped) and the derived values of src/read_par_json.c
  (NT = iround(TIME/DT) at :505, NS = NT/NDT at :516).
* ``read_model``     -- binary model files, NX traces of NY float32 samples
  (src/readmod_elastic.c:103-111).
* ``read_sources``   -- src/sources.c:60-118 (SOURCE_SHAPE <= 4 layout) and
  src/splitsrc.c:34-36 (grid index = floor(x/DH) + 1).
* ``read_receivers`` -- src/receiver.c:48-80 (file), :118-160 (line).
* ``read_su``        -- 240-byte native-endian trace header + float32 samples
  (src/write_su.c:31-67, src/su_struct.h).
"""
from __future__ import annotations

import ctypes
import math
import os
import re
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")

WEQ_CODES = {"AC_ISO": 0, "VAC_ISO": 1, "EL_ISO": 2, "VEL_ISO": 3, "EL_VTI": 4, "VEL_VTI": 5,
             "EL_TTI": 6, "VEL_TTI": 7}
WEQ_NAMES = {v: k for k, v in WEQ_CODES.items()}
COMPONENTS = {"vx": 1, "vy": 2, "p": 3, "div": 4, "curl": 5}


def build():
    """Compile liboracle_f32.so / liboracle_f64.so with the oracle Makefile."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


class OrcParams(ctypes.Structure):
    _fields_ = [("weq", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int),
                ("fdorder", ctypes.c_int), ("maxrelerror", ctypes.c_int), ("L", ctypes.c_int),
                ("dt", ctypes.c_float), ("dh", ctypes.c_float), ("nt", ctypes.c_int),
                ("fw", ctypes.c_int), ("abs_type", ctypes.c_int), ("free_surf", ctypes.c_int),
                ("boundary", ctypes.c_int), ("npower", ctypes.c_float), ("k_max_cpml", ctypes.c_float),
                ("vppml", ctypes.c_float), ("fpml", ctypes.c_float), ("damping", ctypes.c_float),
                ("f_ref", ctypes.c_float), ("fl", ctypes.c_float * 8), ("seismo", ctypes.c_int),
                ("ndt", ctypes.c_int), ("snap", ctypes.c_int), ("tsnap1", ctypes.c_float),
                ("tsnap2", ctypes.c_float), ("tsnapinc", ctypes.c_float), ("idx", ctypes.c_int),
                ("idy", ctypes.c_int), ("nthreads", ctypes.c_int), ("fdorder_time", ctypes.c_int),
                ("readmod", ctypes.c_int), ("tau", ctypes.c_float)]


_LIBS: dict = {}


def _lib(precision: str = "f32"):
    if precision not in _LIBS:
        path = os.path.join(BUILD, f"liboracle_{precision}.so")
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        P = ctypes.POINTER
        fp = P(ctypes.c_float)
        ip = P(ctypes.c_int)
        lib.orc_create.restype = ctypes.c_void_p
        lib.orc_create.argtypes = [P(OrcParams)]
        lib.orc_destroy.argtypes = [ctypes.c_void_p]
        lib.orc_error.restype = ctypes.c_char_p
        lib.orc_error.argtypes = [ctypes.c_void_p]
        lib.orc_set_material.argtypes = [ctypes.c_void_p, ctypes.c_char_p, fp]
        lib.orc_prepare.argtypes = [ctypes.c_void_p]
        lib.orc_set_sources.argtypes = [ctypes.c_void_p, ctypes.c_int, fp, fp]
        lib.orc_set_receivers.argtypes = [ctypes.c_void_p, ctypes.c_int, ip, ip]
        lib.orc_wavelet.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_int, fp, fp]
        lib.orc_wavelet_samples.argtypes = [ctypes.c_int, ctypes.c_float, ctypes.c_int, fp, fp, ctypes.c_int, fp]
        lib.orc_reset.argtypes = [ctypes.c_void_p]
        lib.orc_run.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.orc_current_step.argtypes = [ctypes.c_void_p]
        lib.orc_get_field.argtypes = [ctypes.c_void_p, ctypes.c_char_p, fp]
        lib.orc_set_field.argtypes = [ctypes.c_void_p, ctypes.c_char_p, fp]
        lib.orc_get_vector.argtypes = [ctypes.c_void_p, ctypes.c_char_p, fp, ctypes.c_int]
        lib.orc_get_section.argtypes = [ctypes.c_void_p, ctypes.c_int, fp]
        lib.orc_num_samples.argtypes = [ctypes.c_void_p]
        lib.orc_num_snapshots.argtypes = [ctypes.c_void_p]
        lib.orc_snapshot_size.argtypes = [ctypes.c_void_p]
        lib.orc_get_snapshot.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, fp]
        lib.orc_timings.argtypes = [ctypes.c_void_p, P(ctypes.c_double)]
        lib.orc_fwi_begin.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        lib.orc_fwi_backward.argtypes = [ctypes.c_void_p, fp, fp]
        lib.orc_fwi_gradients.argtypes = [ctypes.c_void_p, fp, fp, fp]
        _LIBS[precision] = lib
    return _LIBS[precision]


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


# ----------------------------------------------------------------- config


@dataclass
class SofiConfig:
    """The forward-modelling parameters of one reference JSON file."""
    weq: int = 2
    nx: int = 100
    ny: int = 100
    dh: float = 1.0
    dt: float = 1e-4
    time: float = 0.1
    nt: int = 1000
    fdorder: int = 4
    fdorder_time: int = 2
    maxrelerror: int = 0
    L: int = 0
    f_ref: float = 0.0
    fl: list = field(default_factory=list)
    fw: int = 0
    abs_type: int = 0
    free_surf: int = 0
    boundary: int = 0
    npower: float = 2.0
    k_max_cpml: float = 1.0
    vppml: float = 3500.0
    fpml: float = 30.0
    damping: float = 8.0
    source_shape: int = 1
    source_type: int = 1
    source_file: str = ""
    seismo: int = 1
    ndt: int = 1
    readrec: int = 1
    rec_file: str = ""
    refrec: tuple = (0.0, 0.0)
    xrec1: float = 0.0
    yrec1: float = 0.0
    xrec2: float = 0.0
    yrec2: float = 0.0
    ngeoph: int = 1
    snap: int = 0
    tsnap1: float = 0.0
    tsnap2: float = 0.0
    tsnapinc: float = 0.0
    idx: int = 1
    idy: int = 1
    mfile: str = ""
    readmod: int = 1
    tau: float = 0.0001
    seis_file: str = ""
    snap_file: str = ""

    def to_ctypes(self, nthreads: int = 0) -> OrcParams:
        p = OrcParams()
        p.weq, p.nx, p.ny, p.fdorder, p.maxrelerror = self.weq, self.nx, self.ny, self.fdorder, self.maxrelerror
        p.L = self.L
        p.dt, p.dh, p.nt = self.dt, self.dh, self.nt
        p.fw, p.abs_type, p.free_surf, p.boundary = self.fw, self.abs_type, self.free_surf, self.boundary
        p.npower, p.k_max_cpml, p.vppml, p.fpml, p.damping = (self.npower, self.k_max_cpml, self.vppml,
                                                              self.fpml, self.damping)
        p.f_ref = self.f_ref
        for k, f in enumerate(self.fl[:8]):
            p.fl[k] = f
        p.seismo, p.ndt = self.seismo, self.ndt
        p.snap, p.tsnap1, p.tsnap2, p.tsnapinc = self.snap, self.tsnap1, self.tsnap2, self.tsnapinc
        p.idx, p.idy = self.idx, self.idy
        p.nthreads = nthreads
        p.fdorder_time = self.fdorder_time
        p.readmod, p.tau = self.readmod, self.tau
        return p


def iround(x: float) -> int:
    return int(math.floor(x + 0.5))


def read_par_json(path: str) -> dict:
    """Key/value strings of a reference parameter file (json_parser.c:52-140)."""
    out: dict = {}
    with open(path) as fh:
        for line in fh:
            if ":" not in line or '"' not in line or "comment" in line or "Comment" in line:
                continue
            m = re.match(r'\s*"([^"]*)"\s*:\s*"([^"]*)"', line)
            if not m:
                continue
            keys = [k.strip() for k in m.group(1).split(",")]
            vals = [v.strip() for v in m.group(2).split(",")]
            if len(keys) != len(vals):
                raise ValueError(f"{path}: mismatched multi-key line: {line!r}")
            for k, v in zip(keys, vals):
                out[k] = v
    return out


def config_from_json(path: str) -> SofiConfig:
    """Typed forward-modelling configuration (read_par_json.c:150-520)."""
    d = read_par_json(path)
    f32 = lambda k, default=0.0: float(np.float32(float(d.get(k, default))))  # noqa: E731
    i = lambda k, default=0: int(d.get(k, default))  # noqa: E731
    c = SofiConfig()
    c.weq = WEQ_CODES[d.get("WEQ", "EL_ISO")]
    c.nx, c.ny = i("NX"), i("NY")
    c.dh, c.dt, c.time = f32("DH"), f32("DT"), f32("TIME")
    c.nt = iround(float(np.float32(c.time) / np.float32(c.dt)))
    c.fdorder, c.maxrelerror = i("FDORDER", 4), i("MAXRELERROR", 0)
    c.fdorder_time = i("FDORDER_TIME", 2)
    c.L = i("L", 0)
    if c.weq in (2, 4, 6):
        c.L = 0
    if c.L:
        c.f_ref = f32("F_REF")
        c.fl = [f32(f"FL{k + 1}") for k in range(c.L)]
    c.free_surf, c.boundary, c.fw, c.abs_type = i("FREE_SURF"), i("BOUNDARY"), i("FW"), i("ABS_TYPE")
    if c.abs_type == 1:
        c.npower, c.k_max_cpml, c.fpml, c.vppml = f32("NPOWER"), f32("K_MAX_CPML"), f32("FPML"), f32("VPPML")
    if c.abs_type == 2:
        c.damping = f32("DAMPING")
    c.source_shape, c.source_type = i("SOURCE_SHAPE", 1), i("SOURCE_TYPE", 1)
    c.source_file = d.get("SOURCE_FILE", "")
    c.seismo = i("SEISMO")
    if c.seismo:
        c.ndt = i("NDT", 1)
        c.readrec = i("READREC", 1)
        c.rec_file = d.get("REC_FILE", "")
        c.refrec = (f32("REFRECX"), f32("REFRECY"))
        c.xrec1, c.yrec1, c.xrec2, c.yrec2 = f32("XREC1"), f32("YREC1"), f32("XREC2"), f32("YREC2")
        c.ngeoph = i("NGEOPH", 1)
        c.seis_file = d.get("SEIS_FILE", "")
    c.snap = i("SNAP")
    if c.snap:
        c.tsnap1, c.tsnap2, c.tsnapinc = f32("TSNAP1"), f32("TSNAP2"), f32("TSNAPINC")
        c.snap_file = d.get("SNAP_FILE", "")
    c.idx, c.idy = i("IDX", 1), i("IDY", 1)
    c.mfile = d.get("MFILE", "")
    return c


MODEL_SUFFIXES = {2: ["vp", "vs", "rho"], 3: ["vp", "vs", "rho", "qp", "qs"],
                  4: ["vp", "vs", "rho", "epsilon", "delta"],
                  5: ["vp", "vs", "rho", "epsilon", "delta", "qp", "qs"],
                  6: ["vp", "vs", "rho", "epsilon", "delta", "theta"],
                  7: ["vp", "vs", "rho", "epsilon", "delta", "theta", "qp", "qs"]}


def read_model(mfile: str, weq: int, nx: int, ny: int) -> dict:
    """Binary model files, NX traces of NY float32 samples each."""
    out = {}
    for s in MODEL_SUFFIXES[weq]:
        a = np.fromfile(f"{mfile}.{s}", dtype=np.float32)
        if a.size < nx * ny:
            raise ValueError(f"{mfile}.{s}: {a.size} values < NX*NY")
        out[s] = a[: nx * ny].copy()
    return out


def read_sources(path: str, cfg: SofiConfig) -> np.ndarray:
    """srcpos matrix [12][nsrc] in grid indices (sources.c + splitsrc.c)."""
    rows = []
    with open(path) as fh:
        for line in fh:
            if "#" in line or not line.split():
                continue
            vals = [float(np.float32(float(t))) for t in line.split()[:7]]
            if len(vals) < 5:
                raise ValueError(f"{path}: missing source parameter in {line!r}")
            xsrc, ysrc, tshift, fc, amp = vals[:5]
            azi = vals[5] if len(vals) > 5 else 0.0
            stype = vals[6] if len(vals) > 6 else float(cfg.source_type)
            rows.append((xsrc, ysrc, tshift, fc, amp, azi, stype))
    n = len(rows)
    sp = np.zeros((12, n), dtype=np.float32)
    for k, (x, y, ts, fc, amp, azi, st) in enumerate(rows):
        sp[0, k] = math.floor(np.float32(x) / np.float32(cfg.dh)) + 1
        sp[1, k] = math.floor(np.float32(y) / np.float32(cfg.dh)) + 1
        sp[3, k], sp[4, k], sp[5, k], sp[6, k], sp[7, k] = ts, fc, amp, azi, st
    return sp


def source_coords(path: str) -> np.ndarray:
    """Physical (x, y) [m] of the sources, for SU header fields."""
    out = []
    with open(path) as fh:
        for line in fh:
            if "#" in line or not line.split():
                continue
            t = line.split()
            out.append((float(np.float32(float(t[0]))), float(np.float32(float(t[1])))))
    return np.array(out, dtype=np.float32)


def read_receivers(cfg: SofiConfig) -> tuple:
    """Receiver grid indices (ix, iy), duplicates removed (receiver.c:48-110)."""
    pts = []
    if cfg.readrec:
        with open(cfg.rec_file) as fh:
            for line in fh:
                if "#" in line or "%" in line or not line.split():
                    continue
                x, y = (float(np.float32(float(t))) for t in line.split()[:2])
                ix = math.floor((np.float32(x) + np.float32(cfg.refrec[0])) / np.float32(cfg.dh)) + 1
                iy = math.floor((np.float32(y) + np.float32(cfg.refrec[1])) / np.float32(cfg.dh)) + 1
                pts.append((ix, iy))
    else:
        dh = np.float32(cfg.dh)
        x1, y1 = math.floor(np.float32(cfg.xrec1) / dh) + 1, math.floor(np.float32(cfg.yrec1) / dh) + 1
        x2, y2 = math.floor(np.float32(cfg.xrec2) / dh) + 1, math.floor(np.float32(cfg.yrec2) / dh) + 1
        if x1 == x2 and y1 == y2:
            pts = [(x1, y1)]
        elif y1 == y2:
            pts = [(x, y1) for x in range(x1, x2 + 1, cfg.ngeoph)]
        elif x1 == x2:
            pts = [(x1, y) for y in range(y1, y2 + 1, cfg.ngeoph)]
        else:
            raise NotImplementedError("oblique receiver lines")
    seen, keep = set(), []
    for p in pts:
        if p not in seen:
            seen.add(p)
            keep.append(p)
    ix = np.array([p[0] for p in keep], dtype=np.int32)
    iy = np.array([p[1] for p in keep], dtype=np.int32)
    return ix, iy


def read_su(path: str) -> tuple:
    """(headers as raw 240-byte rows, data [ntr][ns]) of an SU file."""
    b = np.fromfile(path, dtype=np.uint8)
    ns = int(b[114:116].view(np.uint16)[0])
    rec = 240 + 4 * ns
    ntr = b.size // rec
    b = b[: ntr * rec].reshape(ntr, rec)
    data = b[:, 240:].copy().view(np.float32).reshape(ntr, ns)
    return b[:, :240].copy(), data


# ------------------------------------------------------------------ solve


class Oracle:
    """One oracle context: configure, prepare a model, run, read outputs."""

    def __init__(self, cfg: SofiConfig, precision: str = "f32", nthreads: int = 0):
        self.cfg = cfg
        self.lib = _lib(precision)
        self._p = cfg.to_ctypes(nthreads)
        self.h = self.lib.orc_create(ctypes.byref(self._p))
        if not self.h:
            raise ValueError("oracle rejected the configuration")

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, rc):
        if rc:
            raise RuntimeError(self.lib.orc_error(self.h).decode())

    def set_material(self, mats: dict):
        for k, v in mats.items():
            a = np.ascontiguousarray(v, dtype=np.float32).reshape(-1)
            assert a.size == self.cfg.nx * self.cfg.ny, k
            self._check(self.lib.orc_set_material(self.h, k.encode(), _fptr(a)))
        self._check(self.lib.orc_prepare(self.h))

    def set_sources(self, srcpos: np.ndarray, signals: np.ndarray):
        sp = np.ascontiguousarray(srcpos, dtype=np.float32)
        sig = np.ascontiguousarray(signals, dtype=np.float32)
        assert sp.shape[0] == 12 and sig.shape == (sp.shape[1], self.cfg.nt)
        self._check(self.lib.orc_set_sources(self.h, sp.shape[1], _fptr(sp), _fptr(sig)))

    def set_receivers(self, ix, iy):
        ix = np.ascontiguousarray(ix, dtype=np.int32)
        iy = np.ascontiguousarray(iy, dtype=np.int32)
        self._check(self.lib.orc_set_receivers(self.h, ix.size, _iptr(ix), _iptr(iy)))
        self.ntr = ix.size

    def reset(self):
        self._check(self.lib.orc_reset(self.h))

    def run(self, nsteps: int | None = None):
        n = self.cfg.nt - self.lib.orc_current_step(self.h) if nsteps is None else nsteps
        self._check(self.lib.orc_run(self.h, n))

    def field(self, name: str) -> np.ndarray:
        out = np.empty((self.cfg.ny, self.cfg.nx), dtype=np.float32)
        self._check(self.lib.orc_get_field(self.h, name.encode(), _fptr(out)))
        return out

    def set_field(self, name: str, a: np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.float32)
        self._check(self.lib.orc_set_field(self.h, name.encode(), _fptr(a)))

    def vector(self, name: str, n: int) -> np.ndarray:
        out = np.zeros(n, dtype=np.float32)
        self._check(self.lib.orc_get_vector(self.h, name.encode(), _fptr(out), n))
        return out

    def section(self, comp) -> np.ndarray:
        comp = COMPONENTS.get(comp, comp)
        ns = self.lib.orc_num_samples(self.h)
        out = np.empty((self.ntr, ns), dtype=np.float32)
        self._check(self.lib.orc_get_section(self.h, comp, _fptr(out)))
        return out

    def snapshots(self, comp) -> np.ndarray:
        comp = COMPONENTS.get(comp, comp)
        n, sz = self.lib.orc_num_snapshots(self.h), self.lib.orc_snapshot_size(self.h)
        out = np.empty((n, sz), dtype=np.float32)
        for k in range(n):
            self._check(self.lib.orc_get_snapshot(self.h, k, comp, _fptr(out[k])))
        return out

    def timings(self) -> np.ndarray:
        out = (ctypes.c_double * 4)()
        self.lib.orc_timings(self.h, out)
        return np.array(list(out))

    # ---- MODE = FWI (EL_ISO): one gradient pass of inversion.c
    def fwi_begin(self, velocity: int = 1, adjoint_type: int = 1):
        self._check(self.lib.orc_fwi_begin(self.h, velocity, adjoint_type))

    def fwi_backward(self, adj_x: np.ndarray, adj_y: np.ndarray):
        ax = np.ascontiguousarray(adj_x, dtype=np.float32)
        ay = np.ascontiguousarray(adj_y, dtype=np.float32)
        assert ax.shape == ay.shape == (self.ntr, self.cfg.nt)
        self._check(self.lib.orc_fwi_backward(self.h, _fptr(ax), _fptr(ay)))

    def fwi_gradients(self) -> tuple:
        """(gradLam_shot, gradMu_shot, gradRhos_shot) as [NY][NX] float32."""
        out = [np.empty((self.cfg.ny, self.cfg.nx), dtype=np.float32) for _ in range(3)]
        self._check(self.lib.orc_fwi_gradients(self.h, *[_fptr(a) for a in out]))
        return tuple(out)


# ------------------------------------------------------------------ FWI


def fwi_residual(calc: np.ndarray, data: np.ndarray, velocity: int, dt: float) -> tuple:
    """calc_res.c:136-160 and :216-262 for LNORM = 2 (no trace kill, time
    window or normalisation): with VELOCITY = 0 both sections are integrated
    (running float sum times DT), the residual is synthetic minus observed,
    stored time-reversed (sample j at NS - j + 1), and L2 sums its squares.
    Returns (residual [ntr][ns], L2)."""
    calc = np.asarray(calc, dtype=np.float32)
    data = np.asarray(data, dtype=np.float32)
    if velocity == 0:
        dt32 = np.float32(dt)
        ic = np.empty_like(calc)
        idata = np.empty_like(data)
        for a, out in ((calc, ic), (data, idata)):
            acc = np.zeros(a.shape[0], dtype=np.float32)
            for j in range(a.shape[1]):
                acc = (acc + a[:, j]).astype(np.float32)
                out[:, j] = acc * dt32
        calc, data = ic, idata
    diff = (calc - data).astype(np.float32)[:, ::-1].copy()
    l2 = float(np.sum(diff.astype(np.float64) ** 2))
    return diff, l2


def fwi_model_gradients(lam, mu, rhos, vp, vs, rho) -> tuple:
    """inversion.c:225-240: the vp / vs / rho' gradients of one shot from the
    Lame / density sums ([NY][NX]) and the model ([NY][NX]), with the
    reference's types (double constants, float arrays); its vs gradient takes
    Vp0 in the mu term."""
    f8 = np.float64
    lam, mu, rhos = (np.asarray(a, dtype=np.float32) for a in (lam, mu, rhos))
    vp, vs, rho = (np.asarray(a, dtype=np.float32) for a in (vp, vs, rho))
    gvp = (2.0 * rho.astype(f8) * vp * lam).astype(np.float32)
    gvs = ((-4.0 * vs.astype(f8) * rho * lam) + 2.0 * rho.astype(f8) * vp * mu).astype(np.float32)
    grho = ((((vp * vp).astype(f8) - (2.0 * vs.astype(f8) * vs)) * lam) + (vs * vs * mu).astype(f8)
            + rhos).astype(np.float32)
    return gvp, gvs, grho


def wavelet(shape: int, nt: int, dt: float, srcpos: np.ndarray, precision: str = "f32",
            samples: np.ndarray | None = None) -> np.ndarray:
    """Source signals [nsrc][nt] (wavelet.c); SOURCE_SHAPE 3 takes the signal
    file's samples (``read_srcsig``)."""
    sp = np.ascontiguousarray(srcpos, dtype=np.float32)
    out = np.empty((sp.shape[1], nt), dtype=np.float32)
    if shape == 3:
        smp = np.ascontiguousarray(samples, dtype=np.float32)
        rc = _lib(precision).orc_wavelet_samples(nt, dt, sp.shape[1], _fptr(sp), _fptr(smp), smp.size, _fptr(out))
    else:
        rc = _lib(precision).orc_wavelet(shape, nt, dt, sp.shape[1], _fptr(sp), _fptr(out))
    if rc == 2:
        raise ValueError("source signal contains only zeros")
    if rc:
        raise ValueError(f"unsupported SOURCE_SHAPE {shape} or wavelet parameters")
    return out


def read_srcsig(path: str, dt: float) -> np.ndarray:
    """Samples of a SOURCE_SHAPE 3 signal file (reference src/read_srcsig.c:38-184):
    SU when the name holds ".su" (any case; first trace, ns and dt from its
    header, delrt must be 0), else ASCII: one value per line, '#' comment
    lines, of which one holding "DT" and "=" states the interval. A stated
    interval must equal DT (as float32)."""
    dt32, sdt = np.float32(dt), None
    if ".su" in path.lower():
        b = np.fromfile(path, dtype=np.uint8)
        ns = int(b[114:116].view(np.uint16)[0])
        sudt = int(b[116:118].view(np.uint16)[0])
        if ns < 1 or int(b[108:110].view(np.int16)[0]) != 0:
            raise ValueError("SU signal file without samples or with a delay recording time")
        samples = b[240:240 + 4 * ns].view(np.float32).copy()
        if sudt > 0:
            sdt = np.float32(sudt * 1e-6)
    else:
        vals = []
        with open(path) as fh:
            for line in fh:
                q = line.lstrip()
                if not q:
                    continue
                if q.startswith("#"):
                    body = q[1:]
                    if "dt" in body.lower() and "=" in body:
                        try:
                            sdt = np.float32(float(body.split("=", 1)[1].split()[0]))
                        except (ValueError, IndexError):
                            pass
                    continue
                try:
                    vals.append(np.float32(float(q.split()[0])))
                except ValueError:
                    vals.append(np.float32(0.0))
        samples = np.array(vals, dtype=np.float32)
    if sdt is not None and sdt != dt32:
        raise ValueError(f"signal file interval {sdt} differs from DT {dt32}")
    return samples


def run_example(json_path: str, workdir: str, precision: str = "f32", nthreads: int = 0,
                overrides: dict | None = None) -> dict:
    """Run a reference example file through the oracle; paths resolve from workdir."""
    cfg = config_from_json(json_path)
    for k, v in (overrides or {}).items():
        setattr(cfg, k, v)

    def rel(p):
        return p if os.path.isabs(p) else os.path.join(workdir, p)

    cfg.rec_file = rel(cfg.rec_file)
    mats = read_model(rel(cfg.mfile), cfg.weq, cfg.nx, cfg.ny)
    srcpos = read_sources(rel(cfg.source_file), cfg)
    sig = wavelet(cfg.source_shape, cfg.nt, cfg.dt, srcpos)
    ix, iy = read_receivers(cfg)
    o = Oracle(cfg, precision, nthreads)
    o.set_material(mats)
    o.set_sources(srcpos, sig)
    o.set_receivers(ix, iy)
    o.run()
    comps = {1: ["vx", "vy"], 2: ["p"], 3: ["div", "curl"], 4: ["vx", "vy", "p", "div", "curl"]}
    out = {"cfg": cfg, "sections": {k: o.section(k) for k in comps.get(cfg.seismo, [])}}
    if cfg.snap:
        scomps = {1: ["vx", "vy"], 2: ["p"], 3: ["div", "curl"], 4: ["vx", "vy", "p", "div", "curl"]}
        out["snapshots"] = {k: o.snapshots(k) for k in scomps[cfg.snap]}
    out["timings"] = o.timings()
    o.close()
    return out
