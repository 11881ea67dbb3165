"""Pin the oracle (CPU restatement) against the reference's own outputs.

* shipped golden seismograms/snapshots of examples/weqN_ref (2x2 ranks in the
  reference; the oracle runs one domain, so agreement is to float round-off,
  except the TTI files whose 2x2 decomposition leaves a seam artefact);
* fixtures made by the reference compiled here (oracle/_ref, one rank) on the
  synthetic cases of tests/golden/cases.py -- bit-identical on x86-64.
"""
import os

import numpy as np
import pytest

from tests.golden.cases import CASES, synthetic_model
from tests.helpers import COMPS, GOLDEN, rel_l2, rel_max, run_oracle_case, run_oracle_example

# Shipped examples run by the reference on 2x2 ranks: the one-domain oracle
# agrees to float round-off (relative L2 bound per example; measured values
# are 2e-6..2.3e-5). The TTI examples' shipped files carry the 2x2 seam
# artefact and are pinned against the one-rank compiled reference instead.
SHIPPED_TOL = {"weq3": 5e-5, "weq4": 5e-5, "weq5": 5e-5, "weq6": 5e-5, "weq3_fy": 5e-5, "weq3_fdt4": 5e-5,
               "weq4_fdt4": 5e-5}


@pytest.mark.parametrize("name", sorted(SHIPPED_TOL))
def test_oracle_vs_shipped_golden(name, oracle_mod):
    g = np.load(os.path.join(GOLDEN, f"shipped_{name}.npz"))
    o = run_oracle_example(name, nthreads=os.cpu_count() or 1)
    tol = SHIPPED_TOL[name]
    for comp in ["vx", "vy", "p", "div"]:
        a, b = o.section(comp), g[f"seis_{comp}"]
        if not np.isfinite(b).all():
            assert np.array_equal(np.isfinite(a), np.isfinite(b))
            continue
        assert rel_l2(a, b) < tol, (name, comp, rel_l2(a, b))
    for comp in ["vx", "vy", "p", "div"]:
        a = o.snapshots(comp).reshape(-1, 200, 200)
        assert a.shape[0] == 4
        assert np.allclose(np.sqrt((a.astype(np.float64) ** 2).sum(axis=(1, 2))), g[f"snapnorm_{comp}"],
                           rtol=5e-5)
        assert rel_l2(a[:, ::8, ::8], g[f"snapsub_{comp}"]) < tol
    o.close()


@pytest.mark.parametrize("name", ["weq7", "weq8", "weq8_fy"])
def test_oracle_vs_compiled_reference_tti_examples(name, oracle_mod):
    g = np.load(os.path.join(GOLDEN, f"ref1x1_{name}.npz"))
    o = run_oracle_example(name, nthreads=os.cpu_count() or 1, snap=False)
    for comp in ["vx", "vy", "p", "div", "curl"]:
        a, b = o.section(comp), g[f"seis_{comp}"]
        assert np.array_equal(np.isfinite(a), np.isfinite(b)), comp
        fin = np.isfinite(b)
        assert rel_max(a[fin], b[fin], floor=1e-30) < 1e-5, (name, comp)
    o.close()


def test_tti_shipped_files_carry_decomposition_seam():
    """The shipped 2x2 TTI seismograms differ from the one-rank reference by ~1%."""
    for name in ["weq7", "weq8"]:
        g = np.load(os.path.join(GOLDEN, f"shipped_{name}.npz"))
        r = np.load(os.path.join(GOLDEN, f"ref1x1_{name}.npz"))
        assert 1e-3 < rel_l2(g["seis_vx"], r["seis_vx"]) < 0.1


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_oracle_vs_compiled_reference(case):
    """Bit-level agreement with the reference compiled from its sources (x86-64 here)."""
    if not case.get("compiled_ref", True):
        pytest.skip("the compiled reference has no working output for this case (see tests/golden/cases.py)")
    g = np.load(os.path.join(GOLDEN, f"ref_{case['name']}.npz"))
    import zlib
    crc = 0
    mats = synthetic_model(case)
    for k in sorted(mats):
        crc = zlib.crc32(mats[k].tobytes(), crc)
    assert crc == int(g["model_crc"][0]), "synthetic model generator drifted"
    o = run_oracle_case(case, nthreads=os.cpu_count() or 1)
    for comp in COMPS:
        key = f"seis_{comp}"
        if key not in g:
            continue
        a, b = o.section(comp), g[key]
        fin = np.isfinite(b)
        assert (np.isfinite(a) == fin).all(), (comp, "non-finite pattern differs")
        # identical on x86-64 (same compiler, no contraction); a few ulp elsewhere
        assert rel_max(a[fin], b[fin], floor=1e-30) < 1e-5, (case["name"], comp, rel_max(a[fin], b[fin]))
    for comp in COMPS:
        key = f"snap_{comp}"
        if key in g:
            a = o.snapshots(comp).reshape(-1)
            b = g[key]
            fin = np.isfinite(b)
            assert rel_max(a[fin], b[fin], floor=1e-30) < 1e-5, (case["name"], "snap", comp)
    o.close()
