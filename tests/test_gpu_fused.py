"""The fused velocity + stress step (opt-in: one kernel per step, v / s /
velocity CPML memory in two buffer sets swapped every step) against the
separate four-cell kernels it is built from: the same device functions compute every cell, so
fields, seismograms and snapshots agree bit for bit, with graphs and without,
for batched shots, and after an odd number of steps (the state then lives in
the second buffer set). One case is also held to the oracle bar directly."""
import os

import numpy as np
import pytest

from tests.golden.cases import case_by_name
from tests.helpers import COMPS, case_receivers, case_sources, gpu_config_from, prepared_model, run_oracle_case

pytestmark = pytest.mark.gpu

CASES = ["el_cpml_fd8", "el_abs_fd2", "el_cpml_fd12", "el_fs_cpml", "el_fs_abs_force", "visc_cpml_fs_l3",
         "visc_abs_l1", "vti_cpml", "vvti_cpml_l2", "el_mixed_sources", "el_moment_tensor"]


def _run(o, cfg, case, fused, monkeypatch, nsteps=None, graph=True, nshots=1):
    from oracle import oracle as O
    from gpi_project_gb300 import TimeLoop
    monkeypatch.setenv("SOFI_VROWS", "w4")
    monkeypatch.setenv("SOFI_SW", "4")
    monkeypatch.setenv("SOFI_FUSED", "1" if fused else "0")
    monkeypatch.setenv("SOFI_GRAPH", "1" if graph else "0")
    sp = case_sources(case, cfg)
    sig = O.wavelet(1, cfg.nt, cfg.dt, sp)
    fields, vecs = prepared_model(o, cfg)
    t = TimeLoop(gpu_config_from(cfg, nshots=nshots, shared_model=1))
    assert t.fused() == fused
    t.set_model(fields)
    if vecs:
        t.set_vectors(vecs)
    for s in range(nshots):
        spk = sp.copy()
        spk[0] += 4 * s  # shots at different x
        t.set_sources(spk, sig, shot=s)
        t.set_receivers(*case_receivers(case, cfg), shot=s)
    t.reset()
    t.run(nsteps)
    out = {}
    for s in range(nshots):
        out.update({f"{s} field {k}": t.field(k, shot=s) for k in ["vx", "vy", "sxx", "syy", "sxy"]})
        comps = {1: ["vx", "vy"], 2: ["p"], 3: ["div", "curl"], 4: COMPS}[cfg.seismo]
        out.update({f"{s} section {c}": t.section(c, shot=s) for c in comps})
    if cfg.snap and nshots == 1:
        out["snapshots"] = t.snapshots({1: "vx", 2: "p", 3: "div", 4: "vx"}[cfg.snap])
    t.close()
    return out


@pytest.mark.parametrize("name", CASES)
def test_fused_step_equals_separate_kernels(name, monkeypatch):
    case = case_by_name(name)
    o = run_oracle_case(case, nthreads=os.cpu_count() or 1, nsteps=1)
    sep = _run(o, o.cfg, case, False, monkeypatch)
    fus = _run(o, o.cfg, case, True, monkeypatch)
    for k in sep:
        np.testing.assert_array_equal(fus[k], sep[k], err_msg=f"{name} {k}")
        assert np.abs(sep[k]).max() > 0, (name, k)
    o.close()


@pytest.mark.parametrize("name", ["visc_cpml_fs_l3", "el_abs_fd2"])
def test_fused_odd_steps_direct_launches_and_batches(name, monkeypatch):
    case = case_by_name(name)
    o = run_oracle_case(case, nthreads=os.cpu_count() or 1, nsteps=1)
    sep = _run(o, o.cfg, case, False, monkeypatch, nsteps=333)
    for graph in (True, False):
        fus = _run(o, o.cfg, case, True, monkeypatch, nsteps=333, graph=graph)
        for k in sep:
            np.testing.assert_array_equal(fus[k], sep[k], err_msg=f"{name} graph={graph} {k}")
    sep = _run(o, o.cfg, case, False, monkeypatch, nshots=3)
    fus = _run(o, o.cfg, case, True, monkeypatch, nshots=3)
    for k in sep:
        np.testing.assert_array_equal(fus[k], sep[k], err_msg=f"{name} batched {k}")
    o.close()


def test_fused_availability(monkeypatch):
    from gpi_project_gb300 import TimeLoop
    from gpi_project_gb300 import timeloop as T
    monkeypatch.setenv("SOFI_FUSED", "1")
    base = dict(nx=100, ny=80, fdorder=4, maxrelerror=0, dt=1e-4, dh=1.0, nt=10, fw=10, abs_type=1, seismo=1, ndt=1,
                nshots=1, shared_model=1)
    for kw, ok in ((dict(weq=2), True), (dict(weq=5, L=2), True), (dict(weq=6), False), (dict(weq=0), False),
                   (dict(weq=2, boundary=1), False), (dict(weq=3, L=1, fdorder_time=4), False)):
        t = TimeLoop(T.make_config(**{**base, **kw}))
        assert t.fused() == ok, kw
        if not ok:
            with pytest.raises(Exception):
                t.set_fused(True)
        t.close()


def test_fused_matches_oracle(monkeypatch):
    from tests.test_gpu_parity import compare_sections, gpu_run_like
    from oracle import oracle as O
    monkeypatch.setenv("SOFI_FUSED", "1")
    case = case_by_name("vvti_cpml_l2")
    o = run_oracle_case(case, nthreads=os.cpu_count() or 1)
    sp = case_sources(case, o.cfg)
    t = gpu_run_like(o, o.cfg, sp, O.wavelet(1, o.cfg.nt, o.cfg.dt, sp), *case_receivers(case, o.cfg))
    assert t.fused()
    compare_sections(t, o, o.cfg.seismo, case["name"])
    t.close()
    o.close()
