"""Shared test helpers: run a synthetic case (tests/golden/cases.py) through the oracle."""
from __future__ import annotations

import math
import os

import numpy as np

from tests.golden.cases import receivers, synthetic_model

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
COMPS = ["vx", "vy", "p", "div", "curl"]


def case_config(case):
    from oracle import oracle as O
    c = O.SofiConfig()
    c.weq, c.nx, c.ny = case["weq"], case["nx"], case["ny"]
    c.dh, c.dt = float(np.float32(case["dh"])), float(np.float32(case["dt"]))
    c.nt = O.iround(float(np.float32(case["nt"] * case["dt"]) / np.float32(case["dt"])))
    c.fdorder, c.maxrelerror, c.L = case["fdorder"], case["maxrelerror"], case["L"]
    c.fdorder_time = case.get("fdorder_time", 2)
    c.fl, c.f_ref = [float(np.float32(f)) for f in case["fl"]], float(np.float32(case["f_ref"]))
    c.fw, c.abs_type, c.free_surf, c.boundary = case["fw"], case["abs_type"], case["free_surf"], case["boundary"]
    c.npower, c.k_max_cpml = float(np.float32(case["npower"])), float(np.float32(case["k_max_cpml"]))
    c.vppml, c.fpml, c.damping = (float(np.float32(case["vppml"])), float(np.float32(case["fpml"])),
                                  float(np.float32(case["damping"])))
    c.seismo, c.ndt = case["seismo"], case["ndt"]
    c.snap, c.idx, c.idy = case["snap"], case["idx"], case["idy"]
    c.tsnap1 = c.tsnap2 = float(np.float32(case["tsnap"]))
    c.tsnapinc = 1.0
    c.source_type = case["source_type"]
    c.readmod, c.tau = case.get("readmod", 1), float(np.float32(case.get("tau", 1e-4)))
    return c


def case_sources(case, cfg):
    n = len(case["sources"])
    sp = np.zeros((12, n), dtype=np.float32)
    dh = np.float32(cfg.dh)
    for k, s in enumerate(case["sources"]):
        s = [float(np.float32(t)) for t in s]
        sp[0, k] = math.floor(np.float32(s[0]) / dh) + 1
        sp[1, k] = math.floor(np.float32(s[1]) / dh) + 1
        sp[3, k], sp[4, k], sp[5, k] = s[2], s[3], s[4]
        sp[6, k] = s[5] if len(s) > 5 else 0.0
        sp[7, k] = s[6] if len(s) > 6 else case["source_type"]
    return sp


def case_receivers(case, cfg):
    dh = np.float32(cfg.dh)
    pts, seen = [], set()
    for x, y in receivers(case):
        p = (math.floor(np.float32(x) / dh) + 1, math.floor(np.float32(y) / dh) + 1)
        if p not in seen:
            seen.add(p)
            pts.append(p)
    return (np.array([p[0] for p in pts], dtype=np.int32), np.array([p[1] for p in pts], dtype=np.int32))


def run_oracle_case(case, precision="f32", nthreads=0, nsteps=None):
    from oracle import oracle as O
    cfg = case_config(case)
    o = O.Oracle(cfg, precision, nthreads)
    o.set_material(synthetic_model(case))
    sp = case_sources(case, cfg)
    o.set_sources(sp, O.wavelet(1, cfg.nt, cfg.dt, sp))
    o.set_receivers(*case_receivers(case, cfg))
    o.run(nsteps)
    return o


def rel_l2(a, b, floor=None):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b) if floor is None else max(np.linalg.norm(b), floor)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))


def rel_max(a, b, floor=None):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.abs(b).max() if floor is None else max(np.abs(b).max(), floor)
    return float(np.abs(a - b).max() / den) if den > 0 else float(np.abs(a - b).max())


# --- the reference's examples/weqN.json runs (all share weq3.json's settings) ---
EXAMPLE_WEQ = {"weq3": (2, 0, 1), "weq4": (3, 1, 1), "weq5": (4, 0, 1), "weq6": (5, 1, 1), "weq7": (6, 0, 1),
               "weq8": (7, 1, 1), "weq3_fy": (2, 0, 3), "weq8_fy": (7, 1, 3), "weq3_fdt4": (2, 0, 1),
               "weq4_fdt4": (3, 1, 1)}
# homogeneous examples/model/TTI_Thomsen_1.* (every cell holds these values)
EXAMPLE_MODEL = {"vp": 3369.0, "vs": 1643.0, "rho": 2000.0, "qp": 20.0, "qs": 10.0, "epsilon": 0.26,
                 "delta": -0.05, "theta": 30.0}
# examples/receiver/receiver.dat (metres) and examples/sources/source.dat
EXAMPLE_RECEIVERS = [(198.0, 198.0), (198.0, 398.0), (198.0, 598.0), (398.0, 198.0), (398.0, 598.0),
                     (598.0, 198.0), (598.0, 398.0), (598.0, 598.0)]
EXAMPLE_SOURCE = (398.0, 398.0, 0.0, 50.0, 1.0)


def example_config(name):
    """weqN.json of the reference examples with NPROCX = NPROCY = 1."""
    from oracle import oracle as O
    weq, L, stype = EXAMPLE_WEQ[name]
    c = O.SofiConfig()
    c.weq, c.nx, c.ny, c.dh, c.dt = weq, 400, 400, 2.0, float(np.float32(1e-4))
    c.nt = 2000
    c.fdorder, c.maxrelerror, c.L = 4, 0, L
    c.f_ref, c.fl = 50.0, [50.0] * L
    c.fw, c.abs_type, c.damping, c.free_surf, c.boundary = 20, 2, 8.0, 0, 0
    c.npower, c.k_max_cpml, c.vppml, c.fpml = 4.0, 1.0, 3500.0, 5.0
    c.seismo, c.ndt = 4, 10
    c.snap, c.idx, c.idy = 4, 2, 2
    c.tsnap1, c.tsnap2, c.tsnapinc = (float(np.float32(0.06)), float(np.float32(0.18)), float(np.float32(0.04)))
    c.source_type = stype
    c.fdorder_time = 4 if name.endswith("_fdt4") else 2  # weqN_fdt4.json: FDORDER_TIME = 4
    return c


def example_inputs(name, cfg):
    from oracle import oracle as O
    n = cfg.nx * cfg.ny
    mats = {k: np.full(n, v, dtype=np.float32) for k, v in EXAMPLE_MODEL.items()
            if k in O.MODEL_SUFFIXES[cfg.weq]}
    sp = np.zeros((12, 1), dtype=np.float32)
    x, y, ts, fc, amp = EXAMPLE_SOURCE
    sp[0, 0] = math.floor(np.float32(x) / np.float32(cfg.dh)) + 1
    sp[1, 0] = math.floor(np.float32(y) / np.float32(cfg.dh)) + 1
    sp[3, 0], sp[4, 0], sp[5, 0], sp[7, 0] = ts, fc, amp, cfg.source_type
    ix = np.array([math.floor(np.float32(x) / np.float32(cfg.dh)) + 1 for x, _ in EXAMPLE_RECEIVERS], np.int32)
    iy = np.array([math.floor(np.float32(y) / np.float32(cfg.dh)) + 1 for _, y in EXAMPLE_RECEIVERS], np.int32)
    return mats, sp, ix, iy


def run_oracle_example(name, precision="f32", nthreads=0, snap=True):
    from oracle import oracle as O
    cfg = example_config(name)
    if not snap:
        cfg.snap = 0
    mats, sp, ix, iy = example_inputs(name, cfg)
    o = O.Oracle(cfg, precision, nthreads)
    o.set_material(mats)
    o.set_sources(sp, O.wavelet(1, cfg.nt, cfg.dt, sp))
    o.set_receivers(ix, iy)
    o.run()
    return o


# --- feeding oracle-prepared inputs to the GPU time loop ---------------------

ISO_FIELDS = ["prip", "prjp", "ppi", "pu"]


def gpu_config_from(cfg, nshots=1, shared_model=1, snap_override=None):
    """sofi_config of include/sofigpu.h for an oracle SofiConfig."""
    from gpi_project_gb300 import make_config
    from oracle.oracle import iround
    snap = cfg.snap if snap_override is None else snap_override
    first = iround(cfg.tsnap1 / cfg.dt) if snap else 0
    inc = iround(cfg.tsnapinc / cfg.dt) if snap else 0
    last = iround(cfg.tsnap2 / cfg.dt) if snap else 0
    return make_config(weq=cfg.weq, nx=cfg.nx, ny=cfg.ny, fdorder=cfg.fdorder, maxrelerror=cfg.maxrelerror,
                       L=cfg.L, dt=cfg.dt, dh=cfg.dh, nt=cfg.nt, fw=cfg.fw, abs_type=cfg.abs_type,
                       free_surf=cfg.free_surf, boundary=cfg.boundary, seismo=cfg.seismo, ndt=cfg.ndt,
                       snap=snap, snap_first=first, snap_inc=inc, snap_last=last, idx=cfg.idx, idy=cfg.idy,
                       nshots=nshots, shared_model=shared_model, fdorder_time=getattr(cfg, "fdorder_time", 2))


def prepared_model(o, cfg):
    """The prepared arrays the GPU kernels read, taken from an oracle context."""
    weq, L = cfg.weq, cfg.L
    if weq == 0:  # acoustic: no mu
        f = {k: o.field(k) for k in ["prip", "prjp", "g"]}
    else:
        f = {k: o.field(k) for k in ISO_FIELDS}
    if weq in (2, 3):
        for k in ["g", "f", "fipjp"]:
            f[k] = o.field(k)
        if weq == 3:
            f["d_base"] = o.field("pu") * o.field("taus")
            f["e_base"] = o.field("ppi") * o.field("taup")
            f["dip_base"] = o.field("puipjp") * o.field("tausipjp")
            if cfg.free_surf:
                f["taus"], f["taup"] = o.field("taus"), o.field("taup")
    elif weq != 0:
        names = ["c11", "c13", "c33", "c55ipjp"] + (["c15", "c35", "c15ipjp", "c35ipjp"] if weq in (6, 7) else [])
        visco = weq in (5, 7)
        for k in names:
            f[k + ("u" if visco else "")] = o.field(k + "u" if visco else k)
        if visco:
            taus = {"c11": "tau11", "c13": "tau13", "c33": "tau33", "c55ipjp": "tau55ipjp", "c15": "tau15",
                    "c35": "tau35", "c15ipjp": "tau15ipjp", "c35ipjp": "tau35ipjp"}
            for k in names:
                f[k + "d_base"] = o.field(k) * o.field(taus[k])
    if cfg.fw > 0 and cfg.abs_type == 2:
        f["absorb"] = o.field("absorb")
    vec = {}
    if cfg.fw > 0 and cfg.abs_type == 1:
        for k in ["K_x", "a_x", "b_x", "K_x_half", "a_x_half", "b_x_half", "K_y", "a_y", "b_y", "K_y_half",
                  "a_y_half", "b_y_half"]:
            vec[k] = o.vector(k, 2 * cfg.fw)
    if L:
        for k in ["bip", "cip", "peta"]:
            vec[k] = o.vector(k, L)
    return f, vec
