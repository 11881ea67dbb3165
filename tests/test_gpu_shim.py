"""The drop-in time_loop() (gpi_project_gb300/csrc/shim/time_loop_gb300.c)
executed on the GPU.

The shim is compiled with a caller shaped like the reference's
(tests/shim_harness/harness.c) against stand-ins of the reference's headers
that declare only the members it touches (tests/shim_harness/fd.h); linking it
into the reference itself is tests/test_shim_link.py. The harness fills the
reference's structures with the oracle-prepared model (MemModel), sources,
receivers and, for MODE = FWI, the model as read (MemInv) and the adjoint
signals, and calls time_loop() as sofi2D.c:369-370 (MODE = FW) and
inversion.c:130,222 (sw = 0, then sw = 1) do. The shim's outputs (the
SECTION arrays, the final MemWavefield, the shot's gradients in MemInv) equal
those of the C ABI driven directly (same kernel variants, fixed by
SOFI_VROWS / SOFI_SW) bit for bit, and lie within the parity bar of the
oracle; Perform counts the sampled steps as time_loop.c:93-116,312 does.
"""
import os
import subprocess

import numpy as np
import pytest

from tests.golden.cases import FWI_CASES, case_by_name, synthetic_model
from tests.helpers import COMPS, case_config, case_receivers, case_sources, gpu_config_from, prepared_model
from tests.test_gpu_parity import compare_sections

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HARNESS = os.path.join(REPO, "tests", "shim_harness")
# oracle field -> MemModel member
MEMBERS = {"prip": "prip", "prjp": "prjp", "ppi": "ppi", "pu": "pu", "g": "g", "f": "f", "fipjp": "fipjp",
           "taus": "ptaus", "taup": "ptaup", "puipjp": "puipjp", "tausipjp": "ptausipjp", "absorb": "absorb_coeff"}
FIXED = {"SOFI_VROWS": "w4", "SOFI_SW": "4"}
OUT_INFO = 100


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    from gpi_project_gb300 import build as B
    lib = os.path.dirname(B.build()["gpu"])
    exe = str(tmp_path_factory.mktemp("shim") / "harness")
    subprocess.run(["gcc", "-O2", "-std=c99", "-D_GNU_SOURCE", "-Wall", "-I", HARNESS, "-I",
                    os.path.join(REPO, "include"), "-o", exe, os.path.join(HARNESS, "harness.c"),
                    os.path.join(REPO, "gpi_project_gb300", "csrc", "shim", "time_loop_gb300.c"), "-L", lib,
                    "-lsofigpu", f"-Wl,-rpath,{lib}", "-lm"], check=True)
    return exe


def _inputs(case):
    from oracle import oracle as O
    cfg = case_config(case)
    o = O.Oracle(cfg, "f32", os.cpu_count() or 1)
    mats = synthetic_model(case)
    o.set_material(mats)
    sp = case_sources(case, cfg)
    sig, rec = O.wavelet(1, cfg.nt, cfg.dt, sp), case_receivers(case, cfg)
    o.set_sources(sp, sig)
    o.set_receivers(*rec)
    return o, cfg, mats, sp, sig, rec


def _write(d, o, cfg, sp, sig, rec, mode, velocity=1, adjoint=1):
    """The harness's input directory (tests/shim_harness/harness.c)."""
    f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)  # noqa: E731
    names = ["prip", "prjp", "ppi", "pu", "g", "f", "fipjp"]
    if cfg.weq == 3:
        names += ["taus", "taup", "puipjp", "tausipjp"]
    if cfg.fw > 0 and cfg.abs_type == 2:
        names.append("absorb")
    for n in names:
        f32(o.field(n)).tofile(os.path.join(d, f"f_{MEMBERS[n]}.bin"))
    _, vecs = prepared_model(o, cfg)
    for k, v in vecs.items():
        f32(v).tofile(os.path.join(d, f"v_{k}.bin"))
    f32(o.vector("hc", 7)).tofile(os.path.join(d, "hc.bin"))
    f32(sp).tofile(os.path.join(d, "srcpos.bin"))
    f32(sig).tofile(os.path.join(d, "signals.bin"))
    np.ascontiguousarray(np.stack(rec), dtype=np.int32).tofile(os.path.join(d, "rec.bin"))
    ns = cfg.nt // cfg.ndt
    kv = dict(NX=cfg.nx, NY=cfg.ny, ND=cfg.fdorder // 2, NT=cfg.nt, DT=repr(cfg.dt), DH=repr(cfg.dh),
              FDORDER=cfg.fdorder, MAXRELERROR=cfg.maxrelerror, L=cfg.L, FW=cfg.fw, ABS_TYPE=cfg.abs_type,
              FREE_SURF=cfg.free_surf, BOUNDARY=cfg.boundary, SEISMO=cfg.seismo, NDT=cfg.ndt, WEQ=cfg.weq,
              MODE=mode, OUTNTIMESTEPINFO=OUT_INFO, NSRC=sp.shape[1], NTR=len(rec[0]), NS=ns,
              VELOCITY=velocity, ADJOINT_TYPE=adjoint)
    with open(os.path.join(d, "params.txt"), "w") as fh:
        fh.write("".join(f"{k} {v}\n" for k, v in kv.items()))
    return ns


def _run(exe, d):
    r = subprocess.run([exe, d], capture_output=True, text=True, timeout=600, env={**os.environ, **FIXED})
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    perf = {}
    for ln in open(os.path.join(d, "perf.txt")):
        k, v = ln.split()
        perf[k] = float(v)
    return perf


def _load(d, name, shape):
    return np.fromfile(os.path.join(d, name), dtype=np.float32).reshape(shape)


@pytest.mark.parametrize("name", ["el_cpml_fd8", "visc_cpml_fs_l3", "el_abs_fd10"])
def test_shim_forward_equals_abi_and_oracle(harness, name, tmp_path, monkeypatch):
    from gpi_project_gb300 import TimeLoop
    for k, v in FIXED.items():
        monkeypatch.setenv(k, v)
    case = dict(case_by_name(name), snap=0)
    o, cfg, _, sp, sig, rec = _inputs(case)
    d = str(tmp_path)
    ns = _write(d, o, cfg, sp, sig, rec, mode=1)
    perf = _run(harness, d)
    o.run()
    fields, vecs = prepared_model(o, cfg)
    t = TimeLoop(gpu_config_from(cfg, snap_override=0))
    t.set_model(fields)
    t.set_vectors(vecs)
    t.set_sources(sp, sig)
    t.set_receivers(*rec)
    t.reset()
    t.run()
    ntr = len(rec[0])
    for c in COMPS:
        got = _load(d, f"sec_{c}.bin", (ntr, ns))
        np.testing.assert_array_equal(got, t.section(c), err_msg=f"{name} {c}")
    compare_sections(t, o, case["seismo"], name)  # the same sections, against the oracle
    for f in ("vx", "vy", "sxx", "syy", "sxy"):
        np.testing.assert_array_equal(_load(d, f"fld_{f}.bin", (cfg.ny, cfg.nx)), t.field(f), err_msg=f"{name} {f}")
    # time_loop.c:93-116,312: steps 1, 1 + OUT, ... are sampled
    assert perf["infocounter"] == (cfg.nt - 1) // OUT_INFO + 1
    assert perf["time_av_timestep"] > 0 and perf["time_av_v_update"] > 0 and perf["time_av_s_update"] > 0
    t.close()
    o.close()


@pytest.mark.parametrize("case", FWI_CASES[:2], ids=[c["name"] for c in FWI_CASES[:2]])
def test_shim_fwi_passes_equal_abi(harness, case, tmp_path, monkeypatch):
    """MODE = FWI through the shim: the forward call (sw = 0) keeps the
    gradient quantities on the GPU, the backward call (sw = 1) takes the
    adjoint signals at the receivers and adds the shot's gradients to
    MemInv; both equal the C ABI's gradient pass on the same inputs."""
    from gpi_project_gb300 import TimeLoop
    from gpi_project_gb300 import host as H
    for k, v in FIXED.items():
        monkeypatch.setenv(k, v)
    g = np.load(os.path.join(REPO, "tests", "golden", f"ref_{case['name']}.npz"))
    o, cfg, mats, sp, sig, rec = _inputs(case)
    fields, vecs = prepared_model(o, cfg)
    model = [mats[k].reshape(cfg.nx, cfg.ny).T.copy() for k in ("vp", "vs", "rho")]
    t = TimeLoop(gpu_config_from(cfg))
    t.set_model(fields)
    if vecs:
        t.set_vectors(vecs)
    t.set_sources(sp, sig)
    t.set_receivers(*rec)
    t.fwi_begin(*model, velocity=case["velocity"], adjoint_type=case["adjoint_type"])
    t.reset()
    t.run()
    fwd = {c: t.section(c) for c in ("vx", "vy")}
    rx, _ = H.fwi_residual(fwd["vx"], g["obs_vx"], case["velocity"], cfg.dt)
    ry, _ = H.fwi_residual(fwd["vy"], g["obs_vy"], case["velocity"], cfg.dt)
    t.fwi_backward(rx, ry)
    lam, mu, rhos = t.fwi_gradients()
    t.close()
    d = str(tmp_path)
    ns = _write(d, o, cfg, sp, sig, rec, mode=0, velocity=case["velocity"], adjoint=case["adjoint_type"])
    for k, a in zip(("vp0", "vs0", "rho0"), model):
        np.ascontiguousarray(a, dtype=np.float32).tofile(os.path.join(d, f"{k}.bin"))
    np.ascontiguousarray(rx, dtype=np.float32).tofile(os.path.join(d, "adj_x.bin"))
    np.ascontiguousarray(ry, dtype=np.float32).tofile(os.path.join(d, "adj_y.bin"))
    perf = _run(harness, d)
    ntr = len(rec[0])
    for c in ("vx", "vy"):
        np.testing.assert_array_equal(_load(d, f"sec_{c}.bin", (ntr, ns)), fwd[c], err_msg=c)
    for k, a in (("lam", lam), ("mu", mu), ("rhos", rhos)):
        got = _load(d, f"grad_{k}.bin", (cfg.ny, cfg.nx))
        np.testing.assert_array_equal(got, a, err_msg=f"{case['name']} gradient {k}")
        assert np.abs(a).max() > 0
    assert perf["infocounter"] == 2 * ((cfg.nt - 1) // OUT_INFO + 1)
    o.close()


@pytest.mark.parametrize("fmt", [3, 2])
def test_shim_snapshots_equal_abi(harness, fmt, tmp_path, monkeypatch):
    """snap() through the shim, two shots: the snapshot files (SNAP_FORMAT 3
    float32, 2 ASCII "%e", named as snap_ssg.c:53-68 names them) hold both
    shots' frames one after the other (time_loop.c:36 numbers snapshots
    across shots), each frame equal to the C ABI's snapshot of the same run."""
    from gpi_project_gb300 import TimeLoop
    for k, v in FIXED.items():
        monkeypatch.setenv(k, v)
    case = dict(case_by_name("el_cpml_fd8"), snap=1, idx=1, idy=1, tsnap=0.04)
    o, cfg, _, sp, sig, rec = _inputs(case)
    d = str(tmp_path)
    _write(d, o, cfg, sp, sig, rec, mode=1)
    with open(os.path.join(d, "params.txt"), "a") as fh:
        fh.write(f"SNAP 1\nSNAP_FORMAT {fmt}\nTSNAP1 {cfg.tsnap1!r}\nTSNAP2 {cfg.tsnap2!r}\nTSNAPINC 1.0\nSHOTS 2\n")
    _run(harness, d)
    fields, vecs = prepared_model(o, cfg)
    t = TimeLoop(gpu_config_from(cfg))
    t.set_model(fields)
    t.set_vectors(vecs)
    t.set_sources(sp, sig)
    t.set_receivers(*rec)
    t.reset()
    t.run()
    ext = "bin" if fmt == 3 else "asc"
    for c in ("vx", "vy"):
        frames = t.snapshots(c)
        assert frames.shape[0] == 1 and np.abs(frames).max() > 0
        want = np.concatenate([frames.reshape(-1)] * 2)
        path = os.path.join(d, f"snap.{ext}.{c}.0.0")
        if fmt == 3:
            np.testing.assert_array_equal(np.fromfile(path, np.float32), want, err_msg=c)
        else:
            with open(path) as fh:
                assert fh.read() == "".join("%e\n" % v for v in want), c
    t.close()
    o.close()
