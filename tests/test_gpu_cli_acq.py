"""sofi2d_gb300 on the GPU with the acquisition set-ups and the several-shot
snapshots of tests/golden/cases.py (ACQ_CASES, SNAP_SHOTS_CASE), against the
reference compiled here on the same parameter files:

  * receivers and a source below the topography of the P-wave model, a
    co-located receiver of the file dropped (its trace number left out of the
    SU headers), REFRECX; receiver planes whose first row 0 becomes 1: SU
    trace headers byte for byte, samples within relative L2 1e-4 and
    relative max 1e-3 of the reference's;
  * three shots of which two write snapshots: the snapshot files hold both
    shots' frames in shot order, within the same bar.
"""
import os
import subprocess

import numpy as np
import pytest

from tests.golden.cases import ACQ_CASES, SNAP_SHOTS_CASE, write_case
from tests.helpers import GOLDEN, rel_l2, rel_max

pytestmark = pytest.mark.gpu

L2_TOL, MAX_TOL = 1e-4, 1e-3
CASES = {c["name"]: c for c in ACQ_CASES + [SNAP_SHOTS_CASE]}


@pytest.mark.parametrize("name", sorted(CASES))
def test_cli_matches_compiled_reference(name, tmp_path):
    from gpi_project_gb300 import build as B
    from oracle.oracle import read_su
    case = CASES[name]
    g = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    work = str(tmp_path)
    write_case(case, work)
    r = subprocess.run([B.build()["cli"], "case.json"], cwd=work, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    checked = 0
    for comp in ("vx", "vy"):
        if f"seis_{comp}" not in g:
            continue
        path = os.path.join(work, "out", f"seis_{comp}.su")
        raw = np.fromfile(path, np.uint8)
        _, sec = read_su(path)
        ref = g[f"seis_{comp}"]
        np.testing.assert_array_equal(raw.reshape(ref.shape[0], -1)[:, :240], g[f"hdr_{comp}"])
        assert rel_l2(sec, ref) <= L2_TOL and rel_max(sec, ref) <= MAX_TOL, (name, comp, rel_l2(sec, ref))
        checked += 1
    for comp in ("vx", "vy"):
        if f"snap_{comp}" not in g:
            continue
        got = np.fromfile(os.path.join(work, "out", f"snap.bin.{comp}"), np.float32)
        ref = g[f"snap_{comp}"]
        assert got.shape == ref.shape, (name, comp, got.shape, ref.shape)
        assert rel_l2(got, ref) <= L2_TOL and rel_max(got, ref) <= MAX_TOL, (name, comp, rel_l2(got, ref))
        checked += 1
    assert checked >= 2
