"""The four-cell velocity and stress kernels on narrow blocks (8 x 32 threads,
32 columns by 32 rows) against the same kernels on the usual 32 x 8-thread
blocks: only the tiling differs, so fields, sections and snapshots agree bit
for bit (CPML, damping, free surface, periodic x, elastic, viscoelastic L = 1
to 3, VTI, FD orders 4 to 12, grid widths that leave ragged blocks)."""
import os

import numpy as np
import pytest

from tests.golden.cases import case_by_name
from tests.helpers import run_oracle_case
from tests.test_gpu_pdl import _run

pytestmark = pytest.mark.gpu

# tti_cpml: narrow velocity blocks beside the one-pass TTI stress kernel;
# ac_cpml_fd8: no narrow form for acoustic media, n4 runs the wide kernels
CASES = ["el_cpml_fd8", "el_abs_fd10", "el_cpml_fd12", "el_fs_abs_force", "el_fs_cpml", "visc_cpml_fs_l3",
         "visc_abs_l1", "vti_cpml", "vvti_cpml_l2", "el_periodic_cpml", "el_mixed_sources", "tti_cpml",
         "ac_cpml_fd8"]


@pytest.mark.parametrize("name", CASES)
def test_narrow_blocks_equal_wide_blocks(name, monkeypatch):
    case = case_by_name(name)
    o = run_oracle_case(case, nthreads=os.cpu_count() or 1, nsteps=1)
    wide = _run(o, o.cfg, case, True, monkeypatch, "w4", "4")
    narrow = _run(o, o.cfg, case, True, monkeypatch, "n4", "n4")
    for k in wide:
        np.testing.assert_array_equal(narrow[k], wide[k], err_msg=f"{name} {k}")
    o.close()


def test_block_threads_reported(monkeypatch):
    from gpi_project_gb300 import TimeLoop
    from tests.helpers import gpu_config_from
    case = case_by_name("el_cpml_fd8")
    o = run_oracle_case(case, nthreads=os.cpu_count() or 1, nsteps=1)
    for vr, sw, want in (("n4", "n4", (8, 8)), ("w4", "4", (32, 32)), ("n4", "4", (8, 32))):
        monkeypatch.setenv("SOFI_VROWS", vr)
        monkeypatch.setenv("SOFI_SW", sw)
        with TimeLoop(gpu_config_from(o.cfg)) as t:
            assert t.block_threads_x() == want, (vr, sw)
    o.close()
