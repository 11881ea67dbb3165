"""Batched shots: S resident shots advanced by one sofi_run give, shot for shot,
the sections a single-shot context gives (same kernels, same arithmetic), for a
shared model and for one model per shot, with the four-cell kernels on wide
and on narrow blocks, and with the TTI stress kernel's interior and frame
tiles."""
import os

import numpy as np
import pytest

from tests.golden.cases import case_by_name, synthetic_model
from tests.helpers import case_config, case_receivers, gpu_config_from, prepared_model, rel_l2

pytestmark = pytest.mark.gpu


def _inputs(name, nshift, **over):
    from oracle import oracle as O
    case = dict(case_by_name(name), **over)
    cfg = case_config(case)
    o = O.Oracle(cfg)
    o.set_material(synthetic_model(case))
    fields, vecs = prepared_model(o, cfg)
    shots = []
    for k in range(nshift):
        sp = np.zeros((12, 1), np.float32)
        sp[0, 0] = 20 + 23 * k
        sp[1, 0] = 30 + 7 * k
        sp[4, 0], sp[5, 0], sp[7, 0] = 40.0, 1.0, 1 + (k % 3)
        shots.append((sp, O.wavelet(1, cfg.nt, cfg.dt, sp)))
    return o, cfg, fields, vecs, shots


def _run(cfg, fields_per_model, vecs, shots, rec, shared):
    from gpi_project_gb300 import TimeLoop
    t = TimeLoop(gpu_config_from(cfg, nshots=len(shots), shared_model=int(shared), snap_override=0))
    for m, f in enumerate(fields_per_model):
        t.set_model(f, model=m)
    t.set_vectors(vecs)
    for s, (sp, sig) in enumerate(shots):
        t.set_sources(sp, sig, shot=s)
        t.set_receivers(*rec, shot=s)
    t.reset()
    t.run()
    out = [{c: t.section(c, shot=s) for c in ["vx", "vy", "p", "div"]} for s in range(len(shots))]
    t.close()
    return out


@pytest.mark.parametrize("vrows", ["w4", "n4"])
@pytest.mark.parametrize("name", ["el_cpml_fd8", "visc_cpml_fs_l3", "tti_cpml"])
def test_batch_equals_single_shots(name, vrows, monkeypatch):
    monkeypatch.setenv("SOFI_VROWS", vrows)
    monkeypatch.setenv("SOFI_SW", "n4" if vrows == "n4" else "4")
    o, cfg, fields, vecs, shots = _inputs(name, 5)
    rec = case_receivers(case_by_name(name), cfg)
    batched = _run(cfg, [fields], vecs, shots, rec, shared=True)
    for s, shot in enumerate(shots):
        alone = _run(cfg, [fields], vecs, [shot], rec, shared=True)[0]
        for c in alone:
            np.testing.assert_array_equal(batched[s][c], alone[c], err_msg=f"{name} shot {s} {c}")
    o.close()


@pytest.mark.parametrize("vrows", ["w4", "n4"])
def test_batch_with_a_model_per_shot(vrows, monkeypatch):
    monkeypatch.setenv("SOFI_VROWS", vrows)
    monkeypatch.setenv("SOFI_SW", "n4" if vrows == "n4" else "4")
    o, cfg, fields, vecs, shots = _inputs("el_abs_fd10", 3)
    rec = case_receivers(case_by_name("el_abs_fd10"), cfg)
    models = [fields, {k: v * 1.01 if k in ("prip", "prjp") else v for k, v in fields.items()},
              {k: v * 0.99 if k in ("g", "f", "fipjp") else v for k, v in fields.items()}]
    batched = _run(cfg, models, vecs, shots[:3], rec, shared=False)
    for s in range(3):
        alone = _run(cfg, [models[s]], vecs, [shots[s]], rec, shared=True)[0]
        for c in alone:
            np.testing.assert_array_equal(batched[s][c], alone[c], err_msg=f"model-per-shot {s} {c}")
    assert rel_l2(batched[0]["vx"], batched[1]["vx"]) > 1e-6  # the models differ
    o.close()


@pytest.mark.parametrize("shared", [True, False], ids=["shared-model", "model-per-shot"])
def test_tti_batch_interior_tiles(shared):
    """TTI on 300 x 120: six 64 x 32 interior tiles per shot beside the frame's
    32 x 8 tiles; the shot is the fastest block index with a shared model and
    the slowest with a model per shot."""
    over = {"nx": 300, "ny": 120}
    o, cfg, fields, vecs, shots = _inputs("tti_cpml", 3, **over)
    rec = case_receivers(dict(case_by_name("tti_cpml"), **over), cfg)
    models = [fields] if shared else [fields, {k: v * 1.01 if k.startswith("c1") else v for k, v in fields.items()},
                                      {k: v * 0.99 if k.startswith("c3") else v for k, v in fields.items()}]
    batched = _run(cfg, models, vecs, shots, rec, shared=shared)
    for s in range(3):
        alone = _run(cfg, [models[0 if shared else s]], vecs, [shots[s]], rec, shared=True)[0]
        for c in alone:
            np.testing.assert_array_equal(batched[s][c], alone[c], err_msg=f"tti shot {s} {c}")
    o.close()
