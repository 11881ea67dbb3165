"""Seeded synthetic parity cases shared by the fixture generator and the tests.

Each case is a small forward-modelling run (a few hundred time steps on a
ragged grid) chosen to exercise one corner of the reference's time loop.
``synthetic_model`` builds the material deterministically from the seed;
``write_case`` writes the reference's own input files (parameter JSON, binary
model files as NX traces of NY float32 samples, source and receiver files) so
the compiled reference can run the case.
"""
from __future__ import annotations

import json
import os

import numpy as np

WEQ_NAMES = {0: "AC_ISO", 2: "EL_ISO", 3: "VEL_ISO", 4: "EL_VTI", 5: "VEL_VTI", 6: "EL_TTI", 7: "VEL_TTI"}


def _case(name, **kw):
    base = dict(name=name, weq=2, nx=123, ny=101, dh=2.0, dt=2.0e-4, nt=400, fdorder=4, maxrelerror=0, L=0,
                fl=[], f_ref=30.0, fw=10, abs_type=1, free_surf=0, boundary=0, npower=2.0, k_max_cpml=1.0,
                vppml=3500.0, fpml=30.0, damping=8.0, seismo=4, ndt=2, snap=4, tsnap=0.06, idx=2, idy=2,
                sources=[[121.0, 99.0, 0.0, 40.0, 1.0]], source_type=1, receivers=None, seed=1, fdorder_time=2,
                compiled_ref=True)
    base.update(kw)
    return base


CASES = [
    _case("el_cpml_fd8", fdorder=8, maxrelerror=1, seed=11),
    _case("el_abs_fd2", fdorder=2, abs_type=2, fw=8, seed=12, nx=97, ny=75),
    _case("el_abs_fd10", fdorder=10, maxrelerror=3, abs_type=2, fw=12, seed=13),
    _case("el_cpml_fd12", fdorder=12, maxrelerror=4, seed=14, nx=64, ny=48, fw=8,
          sources=[[61.0, 45.0, 0.0, 40.0, 1.0]]),
    _case("el_fs_cpml", free_surf=1, fdorder=6, maxrelerror=2, seed=15,
          sources=[[121.0, 11.0, 0.0, 40.0, 1.0]]),
    _case("el_fs_abs_force", free_surf=1, abs_type=2, fw=10, source_type=3, seed=16,
          sources=[[121.0, 7.0, 0.0, 40.0, 1.0]]),
    _case("visc_cpml_fs_l3", weq=3, L=3, fl=[5.0, 15.0, 50.0], f_ref=15.0, free_surf=1, fdorder=8,
          source_type=3, seed=17, sources=[[121.0, 21.0, 0.0, 40.0, 1.0]]),
    _case("visc_abs_l1", weq=3, L=1, fl=[40.0], f_ref=40.0, abs_type=2, seed=18),
    _case("vti_cpml", dt=1.5e-4, nt=500, weq=4, fdorder=6, seed=19),
    _case("vvti_cpml_l2", dt=1.5e-4, nt=500, weq=5, L=2, fl=[10.0, 50.0], f_ref=25.0, fdorder=4, seed=20),
    _case("tti_cpml", dt=1.5e-4, nt=500, weq=6, fdorder=6, seed=21),
    _case("tti_abs", dt=1.5e-4, nt=500, weq=6, fdorder=4, abs_type=2, seed=22),
    _case("vtti_cpml_l1", dt=1.5e-4, nt=500, weq=7, L=1, fl=[30.0], f_ref=30.0, fdorder=4, seed=23),
    _case("el_periodic_cpml", boundary=1, fdorder=4, seed=24),
    _case("el_mixed_sources", fdorder=4, seed=25, source_type=2,
          sources=[[101.0, 81.0, 0.0, 40.0, 1.0, 30.0, 4.0], [141.0, 111.0, 0.005, 35.0, 2.0, 0.0, 2.0],
                   [121.0, 99.0, 0.0, 40.0, 1.5, 0.0, 1.0]]),
    _case("el_moment_tensor", fdorder=4, seed=26, source_type=1,
          sources=[[121.0, 99.0, 0.0, 40.0, 1.0, 35.0, 5.0]]),
    # acoustic (WEQ = AC_ISO): one pressure field; no free surface and no
    # div/curl output (the reference has no mu and no sxy for it)
    _case("ac_cpml_fd8", weq=0, fdorder=8, maxrelerror=1, seismo=2, snap=1, seed=31),
    _case("ac_abs_fd4", weq=0, fdorder=4, abs_type=2, seismo=1, snap=2, seed=32),
    _case("ac_periodic_force", weq=0, fdorder=6, boundary=1, seismo=1, snap=0, seed=33, source_type=2,
          sources=[[121.0, 99.0, 0.0, 40.0, 1.0, 0.0, 2.0], [141.0, 111.0, 0.0, 35.0, 1.0, 0.0, 3.0]]),
    # 4th-order Adams-Bashforth time stepping (FDORDER_TIME = 4): EL_ISO and
    # VEL_ISO only; CPML exercises update_v_PML_4.c, which leaves the velocity of
    # the left frame and the corners un-updated. The reference as it compiles
    # today never fills g/f/fipjp for elastic FDORDER_TIME = 4
    # (prepare_update_s_el_4.c computes them into locals) and outputs zeros, so
    # the elastic case is pinned by the shipped weq3_fdt4 golden files instead.
    _case("visc_fdt4_cpml", weq=3, L=2, fl=[10.0, 40.0], f_ref=25.0, fdorder=4, fdorder_time=4, dt=1.0e-4,
          nt=600, seed=41),
    _case("visc_fdt4_abs", weq=3, L=1, fl=[30.0], f_ref=30.0, fdorder=8, maxrelerror=1, abs_type=2, fdorder_time=4,
          dt=1.0e-4, nt=600, seed=42),
    _case("el_fdt4_cpml", fdorder=6, fdorder_time=4, dt=1.0e-4, nt=600, seed=43, compiled_ref=False),
    # the reference's built-in models (READMOD = 0, hh_*.c): a half space below
    # 100 m under a vp = 0 layer (isotropic), or a homogeneous VTI / TTI medium
    _case("hh_el", readmod=0, nx=90, ny=80, fdorder=4, seed=51, sources=[[91.0, 131.0, 0.0, 40.0, 1.0]]),
    _case("hh_visc_l2", readmod=0, weq=3, L=2, fl=[10.0, 50.0], f_ref=25.0, nx=90, ny=80, fdorder=6, seed=52,
          sources=[[91.0, 131.0, 0.0, 40.0, 1.0]]),
    _case("hh_vti", readmod=0, weq=4, dt=1.5e-4, nt=500, nx=90, ny=80, seed=53),
    _case("hh_vvti_l1", readmod=0, weq=5, L=1, fl=[30.0], f_ref=30.0, tau=0.05, dt=1.5e-4, nt=500, nx=90, ny=80,
          seed=54),
    _case("hh_tti", readmod=0, weq=6, dt=1.5e-4, nt=500, fdorder=6, nx=90, ny=80, seed=55),
    _case("hh_vtti_l2", readmod=0, weq=7, L=2, fl=[10.0, 50.0], f_ref=25.0, tau=0.05, dt=1.5e-4, nt=500, nx=90,
          ny=80, seed=56),
]

# Source wavelets (wavelet.c, read_srcsig.c) on a 40 x 40 grid, NT 600, DT
# 1e-4 s: the source-file line (x y tshift, then the shape's columns), and for
# SOURCE_SHAPE 3 the signal file. The reference writes the first source's
# signal with SIGOUT = 1 (initsrc.c:64-93), as float32 (SIGOUT_FORMAT 3).
WAVELET_NT, WAVELET_DT = 600, 1.0e-4


def _signal_samples(n, seed):
    rng = np.random.default_rng(seed)
    t = np.arange(n) * WAVELET_DT
    return (np.sin(2 * np.pi * 35.0 * t) * np.exp(-((t - 0.01) / 0.006) ** 2)
            + 0.01 * rng.standard_normal(n)).astype(np.float32)


WAVELET_CASES = [
    dict(name="ricker", shape=1, line="41.0 41.0 0.002 40.0 1.5"),
    dict(name="fuchs_mueller", shape=2, line="41.0 41.0 0.01 35.0 0.75"),
    dict(name="sin3", shape=4, line="41.0 41.0 0.005 25.0 2.0 0.0 3"),
    dict(name="berlage", shape=5, line="41.0 41.0 0.005 30.0 2.0 2.0 150.0 -90.0"),
    dict(name="berlage_typed", shape=5, line="41.0 41.0 0.0 45.0 0.5 0.5 60.0 30.0 0.0 2"),
    dict(name="klauder", shape=6, line="41.0 41.0 0.0 10.0 60.0 1.0 0.5 3.0"),
    dict(name="klauder_late", shape=6, line="41.0 41.0 0.004 20.0 80.0 2.5 1.0 2.0 0.0 1"),
    dict(name="file_ascii", shape=3, line="41.0 41.0 0.0 30.0 1.25", signal_file="signal.dat",
         signal=_signal_samples(450, 5), signal_dt_line="# DT = 1.0e-04"),
    dict(name="file_su", shape=3, line="41.0 41.0 0.0 30.0 0.8", signal_file="signal.su",
         signal=_signal_samples(700, 6)),
]


def write_signal_file(case, work):
    """The SOURCE_SHAPE 3 signal file of a wavelet case: ASCII one value per
    line (repr, exact in float32) after a DT comment, or an SU trace whose
    header states ns and dt [us] (su_struct.h offsets 114 and 116)."""
    path = os.path.join(work, case["signal_file"])
    sig = case["signal"]
    if path.endswith(".su"):
        hdr = np.zeros(240, np.uint8)
        hdr[114:116] = np.array([sig.size], np.uint16).view(np.uint8)
        hdr[116:118] = np.array([int(round(WAVELET_DT * 1e6))], np.uint16).view(np.uint8)
        with open(path, "wb") as fh:
            fh.write(hdr.tobytes() + sig.astype(np.float32).tobytes())
    else:
        with open(path, "w") as fh:
            fh.write(case["signal_dt_line"] + "\n")
            for v in sig:
                fh.write(f"{float(v)!r}\n")
    return path


# MODE = FWI (one gradient pass, ITERMAX 1, DTINV 1, LNORM 2): EL_ISO only,
# NDT = 1 and full-grid gradients (IDX = IDY = 1). The observed data come from
# the same acquisition on `true_model` (a faster, denser blob).
FWI_CASES = [
    _case("fwi_el_cpml", fdorder=8, maxrelerror=1, seed=51, nt=300, source_type=3, seismo=1, snap=0, ndt=1,
          idx=1, idy=1, velocity=1, adjoint_type=1),
    _case("fwi_el_abs_v0", fdorder=4, abs_type=2, fw=10, seed=52, nt=300, source_type=1, seismo=1, snap=0, ndt=1,
          idx=1, idy=1, velocity=0, adjoint_type=2),
    # with a free surface the receivers near it see surface waves ~1e6 times a
    # deep blob's echo, below float32 resolution: a shallow, stronger blob here
    _case("fwi_el_fs", fdorder=6, maxrelerror=2, free_surf=1, seed=53, nt=300, source_type=2, seismo=1, snap=0,
          ndt=1, idx=1, idy=1, velocity=1, adjoint_type=3, sources=[[121.0, 11.0, 0.0, 40.0, 1.0]],
          blob=(0.3, 0.7, 0.08, 0.3, 1.15, 1.08)),
]


# Acquisition set-ups of receiver.c / sources.c beyond a receiver file and a
# source file: receivers and sources placed below the topography (REC_TOPO,
# SOURCE_TOPO) with co-located receivers in the file and REFRECX; receiver
# planes (REC_ARRAY, the first at depth 0 whose row 0 becomes 1) with a plane
# wave of sources (SRCREC 2). `par` sets or adds parameter-file keys.
_LINE = [[3.0 + 5.0 * k, 4.0] for k in range(10)]
ACQ_CASES = [
    _case("acq_topo", nx=60, ny=50, nt=250, fw=10, seismo=1, ndt=1, snap=0, seed=41, topo=True,
          sources=[[61.0, 6.0, 0.0, 60.0, 1.0]], receivers=[[30.2, 4.0]] + _LINE[:5] + [[30.9, 4.0]] + _LINE[5:],
          par={"REC_TOPO": "1", "SOURCE_TOPO": "1", "REFRECX": "1.0"}),
    _case("acq_planes", nx=60, ny=50, nt=250, fw=10, seismo=1, ndt=1, snap=0, seed=42,
          sources=[[61.0, 61.0, 0.0, 60.0, 1.0]],
          par={"READREC": "0", "XREC1": "10.0", "XREC2": "100.0", "YREC1": "10.0", "YREC2": "10.0",
               "REC_ARRAY": "3", "DRX": "7", "REC_ARRAY_DEPTH": "0.0", "REC_ARRAY_DIST": "9.0"}),
    # the receiver line of the parameter file, its keys in the combined form of
    # the reference's examples ("XREC1,YREC1" : "x , y"), every NGEOPH-th point
    _case("acq_line", nx=60, ny=50, nt=250, fw=10, seismo=1, ndt=1, snap=0, seed=46,
          sources=[[61.0, 61.0, 0.0, 60.0, 1.0]],
          par={"READREC": "0", "XREC1,YREC1": "10.0 , 12.0", "XREC2,YREC2": "100.0 , 12.0", "NGEOPH": "3"}),
    _case("acq_vline", nx=60, ny=50, nt=250, fw=10, seismo=1, ndt=1, snap=0, seed=47,
          sources=[[61.0, 61.0, 0.0, 60.0, 1.0]],
          par={"READREC": "0", "XREC1,YREC1": "80.0 , 8.0", "XREC2,YREC2": "80.0 , 90.0", "NGEOPH": "4"}),
]
# Three shots (RUN_MULTIPLE_SHOTS 1) of which shots 1 and 2 write snapshots
# (SNAPSHOT_START 2): the files hold shot 1's frames, then shot 2's.
SNAP_SHOTS_CASE = _case("snap_shots", nx=60, ny=50, nt=250, fw=10, seismo=1, ndt=1, snap=1, tsnap=0.03, idx=1, idy=1,
                        seed=44, sources=[[31.0, 31.0, 0.0, 60.0, 1.0], [61.0, 41.0, 0.0, 60.0, 1.0],
                                          [91.0, 61.0, 0.0, 60.0, 1.0]],
                        par={"RUN_MULTIPLE_SHOTS": "1", "SNAPSHOT_START": "2", "SNAPSHOT_INCR": "1"})
# Seismograms and snapshots in the binary and ASCII formats (SEIS_FORMAT and
# SNAP_FORMAT 3, then 2), written by the reference for the same run.
FORMAT_CASE = _case("fmt_out", nx=40, ny=40, nt=60, fw=5, seismo=1, ndt=2, snap=1, tsnap=0.006, idx=1, idy=1,
                    seed=45, sources=[[41.0, 41.0, 0.0, 60.0, 1.0]],
                    receivers=[[20.0, 20.0], [50.0, 30.0], [60.0, 60.0]])
# A plane wave of sources (SRCREC 2). The compiled reference builds it
# (sources.c:337-367) into a source matrix of 8 rows and then reads rows 9-11
# of it in splitsrc.c:50-51, past the allocation, and crashes there; its log's
# source table (sources.c:386-404, printed before the crash, two decimals) is
# what pins the positions.
PLANE_WAVE_CASE = _case("acq_plane_wave", nx=60, ny=50, nt=250, fw=10, seismo=1, ndt=1, snap=0, seed=43,
                        par={"SRCREC": "2", "PLANE_WAVE_DEPTH": "20.0", "PLANE_WAVE_ANGLE": "12.0", "TS": "0.025",
                             "LOG_VERBOSITY": "INFO"})


def topo_rows(case):
    """Rows of the constant low-velocity cover over each column of a case
    with topography (the scan finds the row below them)."""
    return 5 + (np.arange(case["nx"]) * 3) % 9


def _smooth(a, w=7):
    """Separable moving average over w cells (edges replicated), as float32."""
    k = np.ones(w) / w
    p = np.pad(a, w // 2, mode="edge")
    p = np.apply_along_axis(lambda r: np.convolve(r, k, mode="valid"), 0, p)
    p = np.apply_along_axis(lambda r: np.convolve(r, k, mode="valid"), 1, p)
    return p.astype(np.float32)


def synthetic_model(case) -> dict:
    """Layered + 2% perturbed isotropic model (plus anisotropy / Q), [NX][NY] x-major."""
    rng = np.random.default_rng(case["seed"])
    nx, ny = case["nx"], case["ny"]
    y = np.arange(ny)
    layer = np.where(y < ny // 3, 0, np.where(y < 2 * ny // 3, 1, 2))
    vp1 = np.array([2000.0, 2800.0, 3500.0])[layer]
    rho1 = np.array([1800.0, 2100.0, 2400.0])[layer]
    pert = 1.0 + 0.02 * rng.standard_normal((nx, ny))
    vp = (vp1[None, :] * pert).astype(np.float32)
    vs = (vp / 1.73).astype(np.float32)
    rho = (rho1[None, :] * (1.0 + 0.02 * rng.standard_normal((nx, ny)))).astype(np.float32)
    if case.get("topo"):
        cover = np.arange(ny)[None, :] < topo_rows(case)[:, None]
        vp[cover], vs[cover], rho[cover] = 1600.0, 925.0, 1800.0
    mats = {"vp": vp, "vs": vs, "rho": rho}
    weq = case["weq"]
    if weq in (4, 5, 6, 7):
        mats["epsilon"] = _smooth(rng.uniform(0.0, 0.25, (nx, ny)))
        mats["delta"] = _smooth(rng.uniform(-0.1, 0.15, (nx, ny)))
    if weq in (6, 7):
        mats["theta"] = _smooth(rng.uniform(0.0, 45.0, (nx, ny)))
    if weq in (3, 5, 7):
        mats["qp"] = _smooth(rng.uniform(20.0, 100.0, (nx, ny)))
        mats["qs"] = (mats["qp"] * 0.7).astype(np.float32)
    return {k: np.ascontiguousarray(v).reshape(-1) for k, v in mats.items()}


def true_model(case, mats) -> dict:
    """The FWI cases' true model: vp, vs x 1.05 and rho x 1.03 in a central
    blob, or as the case's blob = (x0, x1, y0, y1 as grid fractions, velocity
    factor, density factor) gives."""
    nx, ny = case["nx"], case["ny"]
    x0, x1, y0, y1, fv, fr = case.get("blob", (0.4, 0.6, 0.4, 0.6, 1.05, 1.03))
    out = {k: v.copy() for k, v in mats.items()}
    for k, f in (("vp", fv), ("vs", fv), ("rho", fr)):
        a = out[k].reshape(nx, ny)
        a[int(nx * x0): int(nx * x1), int(ny * y0): int(ny * y1)] *= np.float32(f)
    return out


def receivers(case):
    if case["receivers"] is not None:
        return case["receivers"]
    nx, ny, dh = case["nx"], case["ny"], case["dh"]
    out = []
    for k in range(12):
        x = (case["fw"] + 2 + k * (nx - 2 * case["fw"] - 4) / 11.0) * dh
        out.append([round(x, 1), (3 if case["free_surf"] else case["fw"] + 5) * dh])
    out.append([nx * dh / 2.0, ny * dh / 2.0])
    out.append([(nx - 3) * dh, (ny - 3) * dh])  # inside the absorbing frame
    return out


def json_text(case) -> str:
    weq = WEQ_NAMES[case["weq"]]
    kv = {
        "NPROCX": "1", "NPROCY": "1", "MODE": "FW", "FDORDER": str(case["fdorder"]), "FDORDER_TIME": str(case["fdorder_time"]),
        "MAXRELERROR": str(case["maxrelerror"]), "NX": str(case["nx"]), "NY": str(case["ny"]),
        "DH": repr(case["dh"]), "TIME": repr(case["nt"] * case["dt"]), "DT": repr(case["dt"]), "WEQ": weq,
        "SOURCE_SHAPE": "1", "SIGNAL_FILE": "none", "SIGOUT": "0", "SOURCE_TYPE": str(case["source_type"]),
        "SRCREC": "1", "SOURCE_FILE": "./source.dat", "RUN_MULTIPLE_SHOTS": "0", "PLANE_WAVE_DEPTH": "0.0",
        "PLANE_WAVE_ANGLE": "0.0", "TS": "0.2", "READMOD": str(case.get("readmod", 1)), "TAU": repr(case.get("tau", 1e-4)),
        "MFILE": "./model/m", "WRITE_MODELFILES": "0",
        "L": str(case["L"]), "F_REF": repr(case["f_ref"]), "FREE_SURF": str(case["free_surf"]),
        "BOUNDARY": str(case["boundary"]), "FW": str(case["fw"]), "ABS_TYPE": str(case["abs_type"]),
        "NPOWER": repr(case["npower"]), "K_MAX_CPML": repr(case["k_max_cpml"]), "VPPML": repr(case["vppml"]),
        "FPML": repr(case["fpml"]), "DAMPING": repr(case["damping"]), "SNAP": str(case["snap"]),
        "TSNAP1": repr(case["tsnap"]), "TSNAP2": repr(case["tsnap"]), "TSNAPINC": "1.0",
        "IDX": str(case["idx"]), "IDY": str(case["idy"]), "SNAP_FORMAT": "3", "SNAP_FILE": "./out/snap",
        "SEISMO": str(case["seismo"]), "READREC": "1", "REC_FILE": "./receiver.dat", "REFRECX": "0.0",
        "REFRECY": "0.0", "NGEOPH": "1", "REC_ARRAY": "0", "NDT": str(case["ndt"]), "SEIS_FORMAT": "1",
        "SEIS_FILE": "./out/seis", "LOG_FILE": "./log/test.log", "LOG": "0", "LOG_VERBOSITY": "WARN",
        "OUT_TIMESTEP_INFO": "100000",
    }
    for k, f in enumerate(case["fl"]):
        kv[f"FL{k + 1}"] = repr(f)
    lines = ["{"] + [f'"{k}" : "{v}",' for k, v in kv.items()]
    lines[-1] = lines[-1].rstrip(",")
    return "\n".join(lines + ["}"]) + "\n"


def acq_json_text(case) -> str:
    """json_text with the keys of case['par'] set, or added where json_text has none."""
    lines = json_text(case).rstrip().splitlines()
    par = dict(case.get("par", {}))
    out = []
    for ln in lines[1:-1]:
        key = ln.split('"')[1]
        if key in par:
            ln = f'"{key}" : "{par.pop(key)}",'
        out.append(ln.rstrip(",") + ",")
    out[-1] = out[-1].rstrip(",")
    # added keys go first: the reference's parser wants an odd number of
    # commas on a line of combined keys ("XREC1,YREC1" : "x , y",)
    return "\n".join(["{"] + [f'"{k}" : "{v}",' for k, v in par.items()] + out + ["}"]) + "\n"


def write_case(case, work):
    os.makedirs(os.path.join(work, "model"), exist_ok=True)
    os.makedirs(os.path.join(work, "out"), exist_ok=True)
    os.makedirs(os.path.join(work, "log"), exist_ok=True)
    mats = synthetic_model(case)
    for k, v in mats.items():
        v.astype(np.float32).tofile(os.path.join(work, "model", f"m.{k}"))
    with open(os.path.join(work, "source.dat"), "w") as fh:
        for s in case["sources"]:
            fh.write(" ".join(repr(float(t)) for t in s) + "\n")
    with open(os.path.join(work, "receiver.dat"), "w") as fh:
        for r in receivers(case):
            fh.write(f"{r[0]!r} {r[1]!r}\n")
    jpath = os.path.join(work, "case.json")
    with open(jpath, "w") as fh:
        fh.write(acq_json_text(case) if case.get("par") else json_text(case))
    return jpath, mats


def fwi_json_text(case) -> str:
    """The case's parameter file in MODE = FWI (read_par_json_fwi.c keys):
    observed data under ./obs/seis, gradients under ./grad/g."""
    kv = {"MODE": "FWI", "RUN_MULTIPLE_SHOTS": "1", "ITERMAX": "1", "DATA_DIR": "./obs/seis",
          "PARAMETERIZATION": "1", "ADJOINT_TYPE": str(case["adjoint_type"]), "VELOCITY": str(case["velocity"]),
          "INV_VP_ITER": "1", "INV_VS_ITER": "1", "INV_RHO_ITER": "1", "TIME_FILT": "0", "USE_WORKFLOW": "0",
          "INV_MODELFILE": "./inv/model", "NFSTART": "1", "NF": "1", "GRADIENT": "./grad/g", "NFSTART_GRAD": "1",
          "NF_GRAD": "1", "GRAD_METHOD": "2", "LNORM": "2", "NORMALIZE": "0", "DTINV": "1", "WRITE_DIFF": "0",
          "EPS_SCALE": "0.01", "STEPMAX": "4", "SCALEFAC": "4.0", "TESTSHOT_START": "1", "TESTSHOT_END": "1",
          "TESTSHOT_INCR": "1", "PRO": "0.01", "MISFIT_LOG_FILE": "./log/L2.dat"}
    lines = json_text(case).rstrip().splitlines()
    body = [ln for ln in lines[1:-1] if not any(f'"{k}" :' in ln for k in kv)]
    body[-1] = body[-1].rstrip(",") + ","
    extra = [f'"{k}" : "{v}",' for k, v in kv.items()]
    extra[-1] = extra[-1].rstrip(",")
    return "\n".join(["{"] + body + extra + ["}"]) + "\n"


def fwi_case_by_name(name):
    for c in FWI_CASES:
        if c["name"] == name:
            return c
    raise KeyError(name)


def case_by_name(name):
    for c in CASES:
        if c["name"] == name:
            return c
    raise KeyError(name)


if __name__ == "__main__":
    print(json.dumps([c["name"] for c in CASES]))
