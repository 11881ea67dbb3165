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


def gpu_fwi(case, obs_vx, obs_vy):
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
    fwd = {"vx": t.section("vx"), "vy": t.section("vy")}
    rx, _ = H.fwi_residual(fwd["vx"], obs_vx, case["velocity"], cfg.dt)
    ry, _ = H.fwi_residual(fwd["vy"], obs_vy, case["velocity"], cfg.dt)
    t.fwi_backward(rx, ry)
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
