"""FWI gradient pass on the GPU (sofi_fwi_* through the C ABI, residuals and
gradient conversion by the host library) against the compiled reference's
per-shot gradients and forward seismograms (tests/golden/ref_fwi_*.npz):
seismograms within the parity bar, the vp / vs / rho' gradients within
GRAD_L2 relative L2 and GRAD_MAX relative max-norm. The gradients correlate
two float32 wave fields over every step, so they carry the fields' rounding
differences (the GPU contracts products into fused multiply-adds) twice."""
import os

import numpy as np
import pytest

from tests.golden.cases import FWI_CASES, synthetic_model
from tests.helpers import case_config, case_receivers, case_sources, gpu_config_from, prepared_model, rel_l2, rel_max

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
L2_TOL, MAX_TOL = 1e-4, 1e-3
GRAD_L2, GRAD_MAX = 1e-3, 1e-2


def gpu_fwi(case, obs_vx, obs_vy, variants=None, backward_sections=None):
    from oracle import oracle as O
    from gpi_project_gb300 import TimeLoop
    from gpi_project_gb300 import host as H
    cfg = case_config(case)
    o = O.Oracle(cfg, "f32", os.cpu_count() or 1)
    mats = synthetic_model(case)
    o.set_material(mats)
    fields, vecs = prepared_model(o, cfg)
    sp = case_sources(case, cfg)
    t = TimeLoop(gpu_config_from(cfg))
    t.set_model(fields)
    if vecs:
        t.set_vectors(vecs)
    t.set_sources(sp, O.wavelet(1, cfg.nt, cfg.dt, sp))
    t.set_receivers(*case_receivers(case, cfg))
    model = [mats[k].reshape(cfg.nx, cfg.ny).T for k in ("vp", "vs", "rho")]
    t.fwi_begin(*model, velocity=case["velocity"], adjoint_type=case["adjoint_type"])
    t.reset()
    t.run()
    if variants is not None:  # what the forward steps ran
        variants.append((t.velocity_variant(), t.stress_variant()))
    fwd = {"vx": t.section("vx"), "vy": t.section("vy")}
    rx, _ = H.fwi_residual(fwd["vx"], obs_vx, case["velocity"], cfg.dt)
    ry, _ = H.fwi_residual(fwd["vy"], obs_vy, case["velocity"], cfg.dt)
    t.fwi_backward(rx, ry)
    if backward_sections is not None:  # what the backward run recorded at the receivers
        backward_sections.update(vx=t.section("vx"), vy=t.section("vy"))
    lam, mu, rhos = t.fwi_gradients()
    grads = dict(zip(("vp", "vs", "rho"), H.fwi_model_gradients(lam, mu, rhos, *model)))
    t.close()
    o.close()
    return fwd, grads


@pytest.mark.parametrize("case", FWI_CASES, ids=[c["name"] for c in FWI_CASES])
def test_gpu_fwi_gradient_matches_compiled_reference(case):
    g = np.load(os.path.join(HERE, "golden", f"ref_{case['name']}.npz"))
    fwd, grads = gpu_fwi(case, g["obs_vx"], g["obs_vy"])
    for c in ("vx", "vy"):
        ref = g[f"fwd_{c}"]
        assert rel_l2(fwd[c], ref) <= L2_TOL and rel_max(fwd[c], ref) <= MAX_TOL, (case["name"], c)
    for k in ("vp", "vs", "rho"):
        ref = g[f"grad_{k}"]
        e2, em = rel_l2(grads[k], ref), rel_max(grads[k], ref)
        print(case["name"], k, "rel L2", e2, "rel max", em)
        assert e2 <= GRAD_L2 and em <= GRAD_MAX, (case["name"], k, e2, em)


FWD_VARIANTS = [("w4", "4", (4, 1), 4), ("w2", "2", (2, 1), 2), ("1", "0", (1, 1), 1), ("2", "4", (1, 1), 4)]


@pytest.mark.parametrize("vrows,sw,v_used,s_used", FWD_VARIANTS, ids=[f"v{v[0]}-s{v[1]}" for v in FWD_VARIANTS])
@pytest.mark.parametrize("case", FWI_CASES, ids=[c["name"] for c in FWI_CASES])
def test_gpu_fwi_forward_variants_match_compiled_reference(case, vrows, sw, v_used, s_used, monkeypatch):
    """The forward steps run the FWI instantiations of the variant the
    autotuner picks for plain steps of the grid: four, two or one cell per
    thread in each update (rows per thread of the one-cell velocity kernel
    become one). Each, fixed by SOFI_VROWS / SOFI_SW, gives seismograms and
    gradients within the bar of the compiled reference's."""
    monkeypatch.setenv("SOFI_VROWS", vrows)
    monkeypatch.setenv("SOFI_SW", sw)
    g = np.load(os.path.join(HERE, "golden", f"ref_{case['name']}.npz"))
    used = []
    fwd, grads = gpu_fwi(case, g["obs_vx"], g["obs_vy"], used)
    assert used[0] == (v_used, s_used), used
    for c in ("vx", "vy"):
        ref = g[f"fwd_{c}"]
        assert rel_l2(fwd[c], ref) <= L2_TOL and rel_max(fwd[c], ref) <= MAX_TOL, (case["name"], c)
    for k in ("vp", "vs", "rho"):
        ref = g[f"grad_{k}"]
        e2, em = rel_l2(grads[k], ref), rel_max(grads[k], ref)
        assert e2 <= GRAD_L2 and em <= GRAD_MAX, (case["name"], vrows, sw, k, e2, em)


def test_gpu_fwi_rejects_unsupported(monkeypatch):
    from gpi_project_gb300 import TimeLoop
    from gpi_project_gb300 import timeloop as T
    z = np.ones((40, 50), dtype=np.float32)
    for kw in (dict(weq=3, L=1), dict(weq=2, ndt=2), dict(weq=2, nshots=2)):
        cfg = T.make_config(**{**dict(nx=50, ny=40, fdorder=4, maxrelerror=0, dt=1e-4, dh=1.0, nt=20, fw=5,
                                      abs_type=1, seismo=1, ndt=1, nshots=1, shared_model=1), **kw})
        t = TimeLoop(cfg)
        with pytest.raises(Exception):
            t.fwi_begin(z, z, z, velocity=1, adjoint_type=1)
        t.close()


@pytest.mark.parametrize("name", ["fwi_el_cpml", "fwi_el_abs_v0"])
def test_cli_fwi_writes_the_reference_gradient_files(name, tmp_path):
    """sofi2d_gb300 on the reference's own MODE = FWI parameter file: the
    forward seismograms and the gradient files (per shot and summed) it
    writes match the compiled reference's."""
    import subprocess
    from gpi_project_gb300 import build as B
    from gpi_project_gb300 import host as H
    from tests.golden.cases import fwi_case_by_name, fwi_json_text, write_case
    case = fwi_case_by_name(name)
    g = np.load(os.path.join(HERE, "golden", f"ref_{name}.npz"))
    work = str(tmp_path)
    write_case(case, work)
    for d in ("obs", "grad"):
        os.makedirs(os.path.join(work, d), exist_ok=True)
    with open(os.path.join(work, "fwi.json"), "w") as fh:
        fh.write(fwi_json_text(case))
    p = H.read_par(os.path.join(work, "fwi.json"))
    assert p.mode_fwi == 1 and p.fwi_velocity == case["velocity"] and p.fwi_adjoint == case["adjoint_type"]
    ntr = g["obs_vx"].shape[0]
    ix = np.arange(1, ntr + 1, dtype=np.int32)
    for comp, k in (("vx", 1), ("vy", 2)):
        H.write_su(os.path.join(work, "obs", f"seis_{comp}.su.shot1"), g[f"obs_{comp}"], ix, ix, 0.0, 0.0, p, 1, k)
    cli = B.build()["cli"]
    r = subprocess.run([cli, "fwi.json"], cwd=work, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    nx, ny = case["nx"], case["ny"]
    from oracle.oracle import read_su
    for comp in ("vx", "vy"):
        _, sec = read_su(os.path.join(work, "out", f"seis_{comp}.su.shot1"))
        assert rel_l2(sec, g[f"fwd_{comp}"]) <= L2_TOL and rel_max(sec, g[f"fwd_{comp}"]) <= MAX_TOL
    for k in ("vp", "vs", "rho"):
        for suffix in (".shot1", ""):
            a = np.fromfile(os.path.join(work, "grad", f"g_gradient.{k}{suffix}"), dtype=np.float32)
            a = a.reshape(nx, ny).T
            ref = g[f"grad_{k}"]
            assert rel_l2(a, ref) <= GRAD_L2 and rel_max(a, ref) <= GRAD_MAX, (name, k, suffix, rel_l2(a, ref))


@pytest.mark.parametrize("case", FWI_CASES, ids=[c["name"] for c in FWI_CASES])
def test_gpu_fwi_checkpointed_equals_whole_store(case, monkeypatch):
    """With checkpoints every K steps (the whole forward run does not fit the
    store), each segment's forward steps are recomputed from its checkpoint
    before the backward steps that read them: the same kernels on the same
    state, so the gradients equal the whole-store pass bit for bit, for
    segment lengths that divide NT and that do not. The recomputed segments
    record no seismograms: the sections after the pass hold the backward
    run's samples, as after the whole-store pass (a drop-in time_loop()
    hands them back to the caller after sw = 1)."""
    g = np.load(os.path.join(HERE, "golden", f"ref_{case['name']}.npz"))
    monkeypatch.delenv("SOFI_FWI_CHECKPOINT", raising=False)
    bw_whole = {}
    _, whole = gpu_fwi(case, g["obs_vx"], g["obs_vy"], backward_sections=bw_whole)
    assert np.abs(bw_whole["vx"]).max() + np.abs(bw_whole["vy"]).max() > 0
    for k in ("7", "64", str(case["nt"])):
        monkeypatch.setenv("SOFI_FWI_CHECKPOINT", k)
        bw = {}
        fwd, ck = gpu_fwi(case, g["obs_vx"], g["obs_vy"], backward_sections=bw)
        for name in ("vp", "vs", "rho"):
            np.testing.assert_array_equal(ck[name], whole[name], err_msg=f"{case['name']} K={k} {name}")
        for c in ("vx", "vy"):
            np.testing.assert_array_equal(bw[c], bw_whole[c], err_msg=f"{case['name']} K={k} backward {c}")


@pytest.mark.parametrize("case", FWI_CASES, ids=[c["name"] for c in FWI_CASES])
def test_gpu_fwi_pdl_equals_ordinary_launches(case, monkeypatch):
    """The pass's per-step kernels launched as programmatic dependents give the
    same seismograms and gradients as ordinary launches, bit for bit."""
    g = np.load(os.path.join(HERE, "golden", f"ref_{case['name']}.npz"))
    monkeypatch.delenv("SOFI_FWI_CHECKPOINT", raising=False)
    monkeypatch.setenv("SOFI_PDL", "0")
    fwd0, ref = gpu_fwi(case, g["obs_vx"], g["obs_vy"])
    monkeypatch.setenv("SOFI_PDL", "1")
    fwd1, got = gpu_fwi(case, g["obs_vx"], g["obs_vy"])
    for name in ("vp", "vs", "rho"):
        np.testing.assert_array_equal(got[name], ref[name], err_msg=f"{case['name']} {name}")
    for k in fwd0:
        np.testing.assert_array_equal(fwd1[k], fwd0[k], err_msg=f"{case['name']} forward {k}")
