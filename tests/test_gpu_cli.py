"""The command-line driver sofi2d_gb300 end to end on the GPU in MODE = FW.

It reads a parameter file in the reference's format with the settings of its
examples/weq3.json (EL_ISO, 400 x 400, DH 2 m, DT 1e-4 s, TIME 0.2 s, FDORDER 4,
damping frame 20, Ricker 50 Hz explosive source at (398 m, 398 m), eight
receivers, SEISMO 4 every NDT 10 steps, snapshots SNAP 4 at 0.06 / 0.10 / 0.14
/ 0.18 s with IDX = IDY = 2, SIGOUT in SU) with one domain, the homogeneous
model files examples/model/TTI_Thomsen_1.{vp,vs,rho} (vp 3369, vs 1643, rho
2000 in every cell), and writes the seismogram, snapshot and wavelet files.
They are compared with the files the reference ships for that example
(tests/golden/shipped_weq3.npz, written by the reference on 2 x 2 ranks) and
with the reference compiled here on one rank (tests/golden/ref1x1_weq3.npz):

  * SU trace headers byte for byte with the compiled reference's
    (saveseis_glob.c:29-148, outseis_glob.c:30-104; the shipped files come
    from an older version that placed receivers at index * DH, not
    (index - 1) * DH, so their position fields differ),
  * samples within relative L2 1e-4 and relative max 1e-3 per component of
    both. An explosion in a homogeneous medium has no curl but rounding
    noise: 3e-6 of div's norm in both reference files, whose curls differ by
    1.4 times curl's own norm. So curl's difference is measured against
    div's norm and maximum, as for the snapshots,
  * snapshot frames (snap_ssg.c:28-209, merged as snapmerge writes them) on the
    shipped 25 x 25 subsample and by frame norm, within the same bar,
  * the wavelet file's samples equal the reference's shipped signal_out file.
"""
import os
import subprocess

import numpy as np
import pytest

from tests.helpers import EXAMPLE_MODEL, EXAMPLE_RECEIVERS, EXAMPLE_SOURCE, GOLDEN, rel_l2, rel_max

pytestmark = pytest.mark.gpu

L2_TOL, MAX_TOL = 1e-4, 1e-3

WEQ3_KEYS = {
    "NPROCX": "1", "NPROCY": "1", "MODE": "FW", "FDORDER": "4", "FDORDER_TIME": "2", "MAXRELERROR": "0",
    "NX": "400", "NY": "400", "DH": "2.0", "TIME": "0.2", "DT": "1.0e-4", "WEQ": "EL_ISO", "SOURCE_SHAPE": "1",
    "SIGNAL_FILE": "signal_mseis.tz", "SIGOUT": "1", "SIGOUT_FILE": "./weq3/signal_out", "SIGOUT_FORMAT": "1",
    "SOURCE_TYPE": "1", "SRCREC": "1", "SOURCE_FILE": "./sources/source.dat", "RUN_MULTIPLE_SHOTS": "0",
    "PLANE_WAVE_DEPTH": "2106.0", "PLANE_WAVE_ANGLE": "0.0", "TS": "0.2", "READMOD": "1",
    "MFILE": "./model/TTI_Thomsen_1", "WRITE_MODELFILES": "0", "L": "0", "F_REF": "50.0", "FL1": "50.0",
    "FREE_SURF": "0", "BOUNDARY": "0", "FW": "20", "ABS_TYPE": "2", "NPOWER": "4.0", "K_MAX_CPML": "1.0",
    "VPPML": "3500.0", "FPML": "5.0", "DAMPING": "8.0", "SNAP": "4", "TSNAP1": "0.06", "TSNAP2": "0.18",
    "TSNAPINC": "0.04", "IDX": "2", "IDY": "2", "SNAP_FORMAT": "3", "SNAP_FILE": "./weq3/snap", "SEISMO": "4",
    "READREC": "1", "REC_FILE": "./receiver/receiver.dat", "REFRECX, REFRECY": "0.0 , 0.0",
    "XREC1,YREC1": "50.0 , 1.0", "XREC2,YREC2": "350.0 , 1.0", "NGEOPH": "5", "REC_ARRAY": "0", "NDT": "10",
    "SEIS_FORMAT": "1", "SEIS_FILE": "./weq3/seis", "LOG_FILE": "./log/test.log", "LOG": "0",
    "OUT_TIMESTEP_INFO": "100",
}


def _write_inputs(work):
    for d in ("model", "sources", "receiver", "weq3", "log"):
        os.makedirs(os.path.join(work, d), exist_ok=True)
    for k in ("vp", "vs", "rho"):
        np.full(400 * 400, EXAMPLE_MODEL[k], np.float32).tofile(os.path.join(work, "model", f"TTI_Thomsen_1.{k}"))
    with open(os.path.join(work, "sources", "source.dat"), "w") as fh:
        fh.write(" ".join(repr(float(v)) for v in EXAMPLE_SOURCE) + "\n")
    with open(os.path.join(work, "receiver", "receiver.dat"), "w") as fh:
        for x, y in EXAMPLE_RECEIVERS:
            fh.write(f"{x!r} {y!r}\n")
    lines = ["{"] + [f'"{k}" : "{v}",' for k, v in WEQ3_KEYS.items()]
    lines[-1] = lines[-1].rstrip(",")
    with open(os.path.join(work, "weq3.json"), "w") as fh:
        fh.write("\n".join(lines + ["}"]) + "\n")


def test_cli_mode_fw_writes_the_reference_files(tmp_path):
    from gpi_project_gb300 import build as B
    from oracle.oracle import read_su
    work = str(tmp_path)
    _write_inputs(work)
    cli = B.build()["cli"]
    r = subprocess.run([cli, "weq3.json"], cwd=work, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    g = np.load(os.path.join(GOLDEN, "shipped_weq3.npz"))
    r1 = np.load(os.path.join(GOLDEN, "ref1x1_weq3.npz"))
    secs = {}
    for comp in ("vx", "vy", "p", "div", "curl"):
        hdr, data = read_su(os.path.join(work, "weq3", f"seis_{comp}.su"))
        np.testing.assert_array_equal(hdr, r1[f"hdr_{comp}"], err_msg=f"SU headers of {comp}")
        secs[comp] = data
    for ref_set in (g, r1):
        floor2 = np.linalg.norm(ref_set["seis_div"].astype(np.float64))
        floorm = float(np.abs(ref_set["seis_div"]).max())
        for comp, data in secs.items():
            ref = ref_set[f"seis_{comp}"]
            f2, fm = (floor2, floorm) if comp == "curl" else (None, None)
            e2, em = rel_l2(data, ref, f2), rel_max(data, ref, fm)
            assert e2 <= L2_TOL and em <= MAX_TOL, (comp, e2, em)
    for comp in ("vx", "vy", "p", "div", "curl"):
        a = np.fromfile(os.path.join(work, "weq3", f"snap.bin.{comp}"), dtype=np.float32).reshape(4, 200, 200)
        sub, norms = a[:, ::8, ::8], np.sqrt((a.astype(np.float64) ** 2).sum(axis=(1, 2)))
        ref_sub, ref_norm = g[f"snapsub_{comp}"], g[f"snapnorm_{comp}"]
        for k in range(4):
            if comp == "curl":  # noise: compare against div's scale
                scale = np.abs(g["snapsub_div"][k]).max()
                assert np.abs(sub[k] - ref_sub[k]).max() <= MAX_TOL * scale, (comp, k)
                continue
            assert rel_l2(sub[k], ref_sub[k]) <= L2_TOL and rel_max(sub[k], ref_sub[k]) <= MAX_TOL, (comp, k)
            assert abs(norms[k] - ref_norm[k]) <= L2_TOL * ref_norm[k], (comp, k, norms[k], ref_norm[k])
    raw = np.fromfile(os.path.join(work, "weq3", "signal_out.shot1.su"), dtype=np.uint8)
    ref_raw = np.load(os.path.join(GOLDEN, "shipped_sigout_weq3.npz"))["raw"]
    assert raw.size == ref_raw.size
    np.testing.assert_array_equal(raw[240:].view(np.float32), ref_raw[240:].view(np.float32))
