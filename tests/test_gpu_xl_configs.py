"""GPU path against the float32 oracle and the float64 arbiter at the full
benchmark configurations (full grids and full NT), through the product path:
host preparation by libsofihost and the autotuned kernel variants.

  c1  elastic 400 x 400, FD8, CPML 20, NT 2000, one explosive shot
  c2  viscoelastic L = 3, 4000 x 2000, FD8, CPML 30, free surface, NT 6000, force source
  c3  TTI elastic 2048 x 2048, FD6, CPML 20, NT 4000, explosive source
  c4  64 viscoelastic shots on 2000 x 1000 in one batched solve, NT 4000; shots 0, 21, 42, 63 checked

Bar: relative L2 <= 1e-4 and relative max <= 1e-3 per component of the
seismogram sections (time_loop.c:282-285, seismo_ssg.c:28-67) and of the
final wavefield, against both oracle builds; denominators floored at 1 % of
the shot's largest component. The oracle runs take minutes on the host's
cores (c2: two 48 G cell-update runs), so these tests come after the others.
Set SOFI_PARITY_RECORD=<path> to write the error tables to a JSON file.
"""
import os

import pytest

from tests.config_parity import L2_TOL, MAX_TOL, config_parity, save_record

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

CONFIGS = [("c1", None), ("c2", None), ("c3", None), ("c4", (0, 21, 42, 63))]


@pytest.mark.parametrize("name,shots", CONFIGS, ids=[c[0] for c in CONFIGS])
def test_full_config_matches_f32_oracle_and_f64_arbiter(name, shots):
    rec = config_parity(name, check_shots=shots, nthreads=os.cpu_count() or 1)
    path = os.environ.get("SOFI_PARITY_RECORD")
    if path:
        save_record(rec, path)
    assert rec["full_nt"]
    for comp, e in rec["errors"].items():
        for pair in ("gpu_f32", "gpu_f64"):
            l2, mx = e[pair]
            assert l2 <= L2_TOL and mx <= MAX_TOL, (name, comp, pair, l2, mx, rec["nt"])
