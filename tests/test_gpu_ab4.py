"""4th-order time stepping (FDORDER_TIME = 4): the four-cells-per-thread
kernels (the default) against the one-cell kernels, which the oracle parity
tests pinned first. Per cell the arithmetic is the same, so fields, sections
and snapshots agree bit for bit: CPML (with the reference's skipped update in
the left frame and the corners) and damping frames, elastic and viscoelastic,
a grid width that leaves a ragged last vector (NX = 123), batched shots."""
import os

import numpy as np
import pytest

from tests.golden.cases import case_by_name
from tests.helpers import COMPS, case_receivers, case_sources, gpu_config_from, prepared_model, run_oracle_case

pytestmark = pytest.mark.gpu


def _run(o, cfg, case, wide, monkeypatch, nshots=1):
    from oracle import oracle as O
    from gpi_project_gb300 import TimeLoop
    monkeypatch.setenv("SOFI_VROWS", "w4" if wide else "1")
    monkeypatch.setenv("SOFI_SW", "4" if wide else "0")
    sp = case_sources(case, cfg)
    sig = O.wavelet(1, cfg.nt, cfg.dt, sp)
    fields, vecs = prepared_model(o, cfg)
    t = TimeLoop(gpu_config_from(cfg, nshots=nshots, shared_model=1))
    assert t.velocity_variant()[0] == (4 if wide else 1) and t.stress_variant() == (4 if wide else 1)
    t.set_model(fields)
    if vecs:
        t.set_vectors(vecs)
    for s in range(nshots):
        spk = sp.copy()
        spk[0] += 5 * s  # shots at different x
        t.set_sources(spk, sig, shot=s)
        t.set_receivers(*case_receivers(case, cfg), shot=s)
    t.reset()
    t.run()
    out = {}
    for s in range(nshots):
        out.update({f"{s} field {k}": t.field(k, shot=s) for k in ["vx", "vy", "sxx", "syy", "sxy"]})
        comps = {1: ["vx", "vy"], 2: ["p"], 3: ["div", "curl"], 4: COMPS}[cfg.seismo]
        out.update({f"{s} section {c}": t.section(c, shot=s) for c in comps})
    if cfg.snap and nshots == 1:
        out["snapshots"] = t.snapshots({1: "vx", 2: "p", 3: "div", 4: "vx"}[cfg.snap])
    t.close()
    return out


@pytest.mark.parametrize("name", ["visc_fdt4_cpml", "visc_fdt4_abs", "el_fdt4_cpml"])
def test_ab4_four_cells_equal_one_cell(name, monkeypatch):
    case = case_by_name(name)
    assert case["fdorder_time"] == 4 and case["nx"] % 4 != 0
    o = run_oracle_case(case, nthreads=os.cpu_count() or 1, nsteps=1)
    one = _run(o, o.cfg, case, False, monkeypatch)
    four = _run(o, o.cfg, case, True, monkeypatch)
    for k in one:
        np.testing.assert_array_equal(four[k], one[k], err_msg=f"{name} {k}")
        assert np.abs(one[k]).max() > 0, (name, k)
    one = _run(o, o.cfg, case, False, monkeypatch, nshots=3)
    four = _run(o, o.cfg, case, True, monkeypatch, nshots=3)
    for k in one:
        np.testing.assert_array_equal(four[k], one[k], err_msg=f"{name} batched {k}")
    o.close()
