"""The post-stress work inside the one-cell stress kernel (k_update_s_post).

Where a step has no free surface and no moment-tensor source (and at most 8
sources per shot), the one-cell ISO / VTI stress kernel injects the explosive
sources, samples the seismograms and probes for NaN itself, and the step
launches no k_post. A run that way equals, bit for bit, a run with the
separate post kernel (SOFI_POSTF=0) for isotropic media: every seismogram
component, the snapshots, the final wavefield; for VTI media the two stress
kernels' products of moduli and derivatives may be contracted into fused
multiply-adds differently by the code generator, and they agree to float32
rounding grown over the run (relative L2 2e-5). Both lie within the parity
bar of the oracle. Cases: elastic and viscoelastic ISO, elastic
and viscoelastic VTI, CPML and damping frames, FDORDER 2-12, SEISMO 1-4,
several sources with a force source before the last explosive one, periodic
x, batched shots; configurations outside its scope keep the post kernel.
"""
import os

import numpy as np
import pytest

from tests.golden.cases import case_by_name
from tests.helpers import COMPS, case_receivers, case_sources, rel_l2, run_oracle_case
from tests.test_gpu_parity import compare_sections, gpu_run_like

pytestmark = pytest.mark.gpu

CASES = [("el_cpml_fd8", {}), ("el_abs_fd2", {}), ("el_cpml_fd12", {}), ("visc_abs_l1", {}), ("vti_cpml", {}),
         ("vvti_cpml_l2", {}), ("hh_el", {}), ("el_mixed_sources", {}), ("el_periodic_cpml", {}),
         ("el_abs_fd10", {"seismo": 1}), ("el_cpml_fd8", {"seismo": 2}), ("visc_abs_l1", {"seismo": 3}),
         ("el_cpml_fd8", {"ndt": 3})]
NOT_FUSED = ["el_fs_cpml", "el_moment_tensor", "tti_cpml"]


def _run(case, o, postf, monkeypatch):
    from oracle import oracle as O
    monkeypatch.setenv("SOFI_SW", "0")
    monkeypatch.setenv("SOFI_POSTF", postf)
    cfg = o.cfg
    sp = case_sources(case, cfg)
    t = gpu_run_like(o, cfg, sp, O.wavelet(1, cfg.nt, cfg.dt, sp), *case_receivers(case, cfg))
    out = {k: t.field(k) for k in ["vx", "vy", "sxx", "syy", "sxy"]}
    comps = {1: ["vx", "vy"], 2: ["p"], 3: ["div", "curl"], 4: COMPS}[case["seismo"]]
    out.update({c: t.section(c) for c in comps})
    if cfg.snap:
        out["snap_vx"] = t.snapshots("vx")
    return t, out


@pytest.mark.parametrize("name,over", CASES, ids=[n + "".join(f"-{k}{v}" for k, v in o.items()) for n, o in CASES])
def test_fused_post_equals_post_kernel(name, over, monkeypatch):
    case = dict(case_by_name(name), **over)
    o = run_oracle_case(case, nthreads=os.cpu_count() or 1)
    tf, fused = _run(case, o, "1", monkeypatch)
    assert tf.post_fused()
    compare_sections(tf, o, case["seismo"], name)
    tf.close()
    tp, plain = _run(case, o, "0", monkeypatch)
    assert not tp.post_fused()
    tp.close()
    for k in fused:
        if case["weq"] in (4, 5):  # VTI
            assert rel_l2(fused[k], plain[k]) <= 2e-5, (name, over, k, rel_l2(fused[k], plain[k]))
        else:
            np.testing.assert_array_equal(fused[k], plain[k], err_msg=f"{name} {over} {k}")
    o.close()


@pytest.mark.parametrize("name", NOT_FUSED)
def test_post_kernel_kept_outside_scope(name, monkeypatch):
    case = case_by_name(name)
    o = run_oracle_case(case, nthreads=os.cpu_count() or 1)
    t, _ = _run(case, o, "1", monkeypatch)
    assert not t.post_fused()
    compare_sections(t, o, case["seismo"], name)
    t.close()
    o.close()


def test_fused_post_batched_shots(monkeypatch):
    """Three shots (explosive and force sources) in one batched solve, fused
    against the post kernel."""
    from tests.test_gpu_batch import _inputs, _run as batch_run
    monkeypatch.setenv("SOFI_SW", "0")
    o, cfg, fields, vecs, shots = _inputs("el_cpml_fd8", 3)
    rec = case_receivers(case_by_name("el_cpml_fd8"), cfg)
    out = {}
    for postf in ("1", "0"):
        monkeypatch.setenv("SOFI_POSTF", postf)
        out[postf] = batch_run(cfg, [fields], vecs, shots, rec, shared=True)
    for s in range(3):
        for c in out["0"][s]:
            np.testing.assert_array_equal(out["1"][s][c], out["0"][s][c], err_msg=f"shot {s} {c}")
    o.close()


@pytest.mark.parametrize("seismo", [1, 4])
def test_fused_post_receivers_sharing_columns(seismo, monkeypatch):
    """Receivers down two columns (a cell's receiver found after others of its
    column in the column's list), two receivers on one cell, and a source on a
    receiver's cell: the fused post work equals the post kernel bit for bit."""
    from oracle import oracle as O
    case = dict(case_by_name("el_cpml_fd8"), seismo=seismo)
    o = run_oracle_case(case, nthreads=os.cpu_count() or 1, nsteps=1)
    cfg = o.cfg
    sp = case_sources(case, cfg)
    si, sj = int(sp[0, 0]), int(sp[1, 0])  # the source's cell
    col = cfg.nx // 3
    ix = [col] * 8 + [col + 5] * 4 + [col, si, 30, 31, 32]
    iy = [25 + 6 * k for k in range(8)] + [60 - 9 * k for k in range(4)] + [25 + 6 * 3, sj, 40, 40, 40]
    ix, iy = np.array(ix, np.int32), np.array(iy, np.int32)
    sig = O.wavelet(1, cfg.nt, cfg.dt, sp)
    out = {}
    for postf in ("1", "0"):
        monkeypatch.setenv("SOFI_SW", "0")
        monkeypatch.setenv("SOFI_POSTF", postf)
        t = gpu_run_like(o, cfg, sp, sig, ix, iy)
        assert t.post_fused() == (postf == "1")
        out[postf] = {c: t.section(c) for c in COMPS}
        out[postf]["sxx"] = t.field("sxx")
        t.close()
    for c in out["0"]:
        np.testing.assert_array_equal(out["1"][c], out["0"][c], err_msg=f"seismo {seismo} {c}")
    assert np.abs(out["1"]["vx"][8]).max() > 0  # the column's receivers recorded the wave
    np.testing.assert_array_equal(out["1"]["vx"][3], out["1"]["vx"][12])  # one cell, two receivers
    o.close()
