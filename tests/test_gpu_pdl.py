"""Programmatic dependent launch of the step kernels (on by default): every
kernel launched that way waits in hardware for its predecessor before it
touches memory, so the results equal ordinary launches of the same kernels
bit for bit, for each kernel family that uses it (four-, two- and one-cell
velocity and stress kernels, acoustic, TTI in one pass, the post kernel with a
free surface and force sources), from the captured step graphs and from direct
launches, and when the switch changes between two parts of a run."""
import os

import numpy as np
import pytest

from tests.golden.cases import case_by_name
from tests.helpers import COMPS, case_receivers, case_sources, gpu_config_from, prepared_model, run_oracle_case

pytestmark = pytest.mark.gpu

CASES = [("el_cpml_fd8", "w4", "4"), ("el_abs_fd10", "w2", "2"), ("el_fs_abs_force", "1", "0"),
         ("visc_cpml_fs_l3", "w4", "4"), ("vvti_cpml_l2", "2", "0"), ("tti_cpml", "w4", "4"),
         ("ac_cpml_fd8", "w4", "4"), ("el_periodic_cpml", "w4", "4"), ("el_moment_tensor", "w4", "4")]


def _run(o, cfg, case, pdl, monkeypatch, vrows, sw, graph=True, switch_at=None):
    from oracle import oracle as O
    from gpi_project_gb300 import TimeLoop
    monkeypatch.setenv("SOFI_VROWS", vrows)
    monkeypatch.setenv("SOFI_SW", sw)
    monkeypatch.setenv("SOFI_PDL", "1" if pdl else "0")
    monkeypatch.setenv("SOFI_GRAPH", "1" if graph else "0")
    sp = case_sources(case, cfg)
    sig = O.wavelet(1, cfg.nt, cfg.dt, sp)
    fields, vecs = prepared_model(o, cfg)
    t = TimeLoop(gpu_config_from(cfg))
    assert t.pdl() == pdl
    t.set_model(fields)
    if vecs:
        t.set_vectors(vecs)
    t.set_sources(sp, sig)
    t.set_receivers(*case_receivers(case, cfg))
    t.reset()
    if switch_at:
        t.run(switch_at)
        t.set_pdl(not pdl)
        assert t.pdl() == (not pdl)
    t.run()
    out = {k: t.field(k) for k in ["vx", "vy", "sxx", "syy", "sxy"]}
    comps = {1: ["vx", "vy"], 2: ["p"], 3: ["div", "curl"], 4: COMPS}[cfg.seismo]
    out.update({f"section {c}": t.section(c) for c in comps})
    if cfg.snap:
        out["snapshots"] = t.snapshots({1: "vx", 2: "p", 3: "div", 4: "vx"}[cfg.snap])
    t.close()
    return out


@pytest.mark.parametrize("name,vrows,sw", CASES, ids=[c[0] for c in CASES])
def test_pdl_equals_ordinary_launches(name, vrows, sw, monkeypatch):
    case = case_by_name(name)
    o = run_oracle_case(case, nthreads=os.cpu_count() or 1, nsteps=1)
    ref = _run(o, o.cfg, case, False, monkeypatch, vrows, sw)
    for graph in (True, False):
        got = _run(o, o.cfg, case, True, monkeypatch, vrows, sw, graph=graph)
        for k in ref:
            np.testing.assert_array_equal(got[k], ref[k], err_msg=f"{name} graph={graph} {k}")
            if not (name.startswith("ac_") and k == "sxy"):  # no shear stress in acoustic media
                assert np.abs(ref[k]).max() > 0, (name, k)
    o.close()


def test_pdl_switched_during_a_run(monkeypatch):
    case = case_by_name("visc_cpml_fs_l3")
    o = run_oracle_case(case, nthreads=os.cpu_count() or 1, nsteps=1)
    ref = _run(o, o.cfg, case, True, monkeypatch, "w4", "4")
    for pdl in (True, False):
        got = _run(o, o.cfg, case, pdl, monkeypatch, "w4", "4", switch_at=77)
        for k in ref:
            np.testing.assert_array_equal(got[k], ref[k], err_msg=f"switched from {pdl} {k}")
    o.close()
