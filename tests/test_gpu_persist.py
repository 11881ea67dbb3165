"""The persistent step kernel (chunks of steps in one cooperative launch, a
grid barrier between the velocity, stress and post phases) against the plain
four-cell kernels: the same bodies run in both, so fields and sections are
bit-identical, also where snapshot and timed steps interleave plain launches
with persistent chunks. One case is also held to the oracle bar directly."""
import os

import numpy as np
import pytest

from tests.golden.cases import case_by_name
from tests.helpers import COMPS, case_receivers, case_sources, gpu_config_from, prepared_model, run_oracle_case

pytestmark = pytest.mark.gpu

CASES = ["el_cpml_fd8", "el_abs_fd2", "el_cpml_fd12", "el_fs_cpml", "el_fs_abs_force", "visc_cpml_fs_l3",
         "visc_abs_l1", "vti_cpml", "vvti_cpml_l2", "el_mixed_sources", "el_moment_tensor", "ac_cpml_fd8",
         "ac_abs_fd4"]


def _run(o, cfg, case, persist, monkeypatch, timing=0):
    from oracle import oracle as O
    from gpi_project_gb300 import TimeLoop
    monkeypatch.setenv("SOFI_VROWS", "w4")
    monkeypatch.setenv("SOFI_SW", "4")
    monkeypatch.setenv("SOFI_PERSIST", "1" if persist else "0")
    sp = case_sources(case, cfg)
    sig = O.wavelet(1, cfg.nt, cfg.dt, sp)
    fields, vecs = prepared_model(o, cfg)
    t = TimeLoop(gpu_config_from(cfg))
    assert t.persistent()[0] == persist and t.velocity_variant() == (4, 1)
    t.set_model(fields)
    if vecs:
        t.set_vectors(vecs)
    t.set_sources(sp, sig)
    t.set_receivers(*case_receivers(case, cfg))
    if timing:
        t.set_kernel_timing(timing)
    t.reset()
    t.run()
    out = {"field " + k: t.field(k) for k in (["vx", "vy", "sxx"] if cfg.weq == 0 else ["vx", "vy", "sxx", "syy", "sxy"])}
    comps = {1: ["vx", "vy"], 2: ["p"], 3: ["div", "curl"], 4: COMPS}[cfg.seismo]
    out.update({"section " + c: t.section(c) for c in comps})
    if cfg.snap:
        out["snapshots"] = t.snapshots({1: "vx", 2: "p", 3: "div", 4: "vx"}[cfg.snap])
    launches = t.launch_count()
    t.close()
    return out, launches


@pytest.mark.parametrize("name", CASES)
def test_persistent_equals_plain_kernels(name, monkeypatch):
    case = case_by_name(name)
    o = run_oracle_case(case, nthreads=os.cpu_count() or 1, nsteps=1)
    cfg = o.cfg
    plain, n_plain = _run(o, cfg, case, False, monkeypatch)
    pers, n_pers = _run(o, cfg, case, True, monkeypatch)
    assert n_pers < n_plain / 4, (n_pers, n_plain)  # chunks of steps per launch
    for k in plain:
        np.testing.assert_array_equal(pers[k], plain[k], err_msg=f"{name} {k}")
        assert np.abs(plain[k]).max() > 0, (name, k)
    o.close()


def test_persistent_with_timed_steps(monkeypatch):
    """Every 7th step timed (a plain launch between persistent chunks)."""
    case = case_by_name("visc_cpml_fs_l3")
    o = run_oracle_case(case, nthreads=os.cpu_count() or 1, nsteps=1)
    plain, _ = _run(o, o.cfg, case, False, monkeypatch)
    pers, _ = _run(o, o.cfg, case, True, monkeypatch, timing=7)
    for k in plain:
        np.testing.assert_array_equal(pers[k], plain[k], err_msg=k)
    o.close()


def test_persistent_default_and_availability(monkeypatch):
    from gpi_project_gb300 import TimeLoop
    from gpi_project_gb300 import timeloop as T
    for k in ("SOFI_VROWS", "SOFI_SW", "SOFI_PERSIST", "SOFI_KERNELS"):
        monkeypatch.delenv(k, raising=False)
    small = T.make_config(weq=3, nx=400, ny=400, fdorder=8, maxrelerror=1, L=2, dt=1e-4, dh=1.0, nt=10, fw=20,
                          abs_type=1, seismo=1, ndt=1, nshots=1, shared_model=1)
    t = TimeLoop(small)
    on, blocks = t.persistent()
    assert not on and blocks > 0  # available, off by default
    t.set_persistent(True)
    assert t.persistent()[0] is True
    t.set_persistent(False)
    t.close()
    monkeypatch.setenv("SOFI_PERSIST", "1")
    t = TimeLoop(small)
    assert t.persistent()[0] is True
    t.close()
    monkeypatch.delenv("SOFI_PERSIST")
    for kw in (dict(weq=6), dict(weq=2, boundary=1), dict(weq=2, fdorder_time=4)):
        cfg = T.make_config(**{**dict(nx=200, ny=200, fdorder=4, maxrelerror=0, dt=1e-4, dh=1.0, nt=10, fw=10,
                                      abs_type=1, seismo=1, ndt=1, nshots=1, shared_model=1), **kw})
        t = TimeLoop(cfg)
        assert t.persistent() == (False, 0), kw
        with pytest.raises(Exception):
            t.set_persistent(True)
        t.close()


def test_persistent_matches_oracle(monkeypatch):
    from tests.test_gpu_parity import compare_sections, gpu_run_like
    from oracle import oracle as O
    monkeypatch.setenv("SOFI_PERSIST", "1")
    case = case_by_name("visc_cpml_fs_l3")
    o = run_oracle_case(case, nthreads=os.cpu_count() or 1)
    sp = case_sources(case, o.cfg)
    t = gpu_run_like(o, o.cfg, sp, O.wavelet(1, o.cfg.nt, o.cfg.dt, sp), *case_receivers(case, o.cfg))
    assert t.persistent()[0] is True
    compare_sections(t, o, o.cfg.seismo, case["name"])
    t.close()
    o.close()
