"""FWI gradient pass (MODE = FWI, EL_ISO, one iteration) of the oracle pinned
to the compiled reference: for seeded cases (CPML, damping frame, free
surface; VELOCITY 0 and 1; ADJOINT_TYPE 1-3; explosive and force sources)
the forward sections, and the per-shot vp / vs / rho' gradients the
reference writes (output_gradient.c), are reproduced bit for bit from the
same observed data (tests/golden/ref_fwi_*.npz, made by make_fixtures.py)."""
import os

import numpy as np
import pytest

from tests.golden.cases import FWI_CASES, synthetic_model
from tests.helpers import case_config, case_receivers, case_sources

HERE = os.path.dirname(os.path.abspath(__file__))


def oracle_fwi(case, obs_vx, obs_vy):
    from oracle import oracle as O
    cfg = case_config(case)
    o = O.Oracle(cfg, "f32", os.cpu_count() or 1)
    mats = synthetic_model(case)
    o.set_material(mats)
    sp = case_sources(case, cfg)
    o.set_sources(sp, O.wavelet(1, cfg.nt, cfg.dt, sp))
    o.set_receivers(*case_receivers(case, cfg))
    o.reset()
    o.fwi_begin(case["velocity"], case["adjoint_type"])
    o.run()
    fwd = {"vx": o.section("vx"), "vy": o.section("vy")}
    rx, l2x = O.fwi_residual(fwd["vx"], obs_vx, case["velocity"], cfg.dt)
    ry, l2y = O.fwi_residual(fwd["vy"], obs_vy, case["velocity"], cfg.dt)
    o.fwi_backward(rx, ry)
    lam, mu, rhos = o.fwi_gradients()
    nx, ny = cfg.nx, cfg.ny
    model = [mats[k].reshape(nx, ny).T for k in ("vp", "vs", "rho")]
    grads = O.fwi_model_gradients(lam, mu, rhos, *model)
    o.close()
    return fwd, (rx, ry), dict(zip(("vp", "vs", "rho"), grads))


@pytest.mark.parametrize("case", FWI_CASES, ids=[c["name"] for c in FWI_CASES])
def test_oracle_fwi_gradient_equals_compiled_reference(case):
    g = np.load(os.path.join(HERE, "golden", f"ref_{case['name']}.npz"))
    fwd, res, grads = oracle_fwi(case, g["obs_vx"], g["obs_vy"])
    for c in ("vx", "vy"):
        np.testing.assert_array_equal(fwd[c], g[f"fwd_{c}"], err_msg=f"{case['name']} forward {c}")
    assert max(np.abs(r).max() for r in res) > 0  # the data differ from the synthetics
    for k in ("vp", "vs", "rho"):
        assert np.abs(g[f"grad_{k}"]).max() > 0, (case["name"], k)
        np.testing.assert_array_equal(grads[k], g[f"grad_{k}"], err_msg=f"{case['name']} gradient {k}")


def test_fwi_residual_reverses_time_and_integrates():
    from oracle import oracle as O
    calc = np.arange(12, dtype=np.float32).reshape(2, 6)
    data = np.ones((2, 6), dtype=np.float32)
    d1, l2 = O.fwi_residual(calc, data, 1, 0.5)
    np.testing.assert_array_equal(d1, (calc - data)[:, ::-1])
    assert l2 == pytest.approx(float(np.sum((calc - data) ** 2)))
    d0, _ = O.fwi_residual(calc, data, 0, 0.5)
    np.testing.assert_allclose(d0[:, ::-1], (np.cumsum(calc, 1) - np.cumsum(data, 1)) * 0.5)
