"""Generate the golden fixtures in tests/golden/ (run here, where the reference exists).

Two kinds of fixture, both small enough to commit:

* ``shipped_<weq>.npz`` -- the seismograms the reference ships in
  examples/weqN_ref (produced by the reference itself on 2x2 ranks) plus a
  subsample of its snapshot files, copied as numbers.
* ``ref_<case>.npz``   -- outputs of the reference compiled from its own
  sources by oracle/ref/Makefile (oracle/_ref/sofi2D, one rank) on seeded
  synthetic cases that the shipped files do not cover: CPML, FDORDER 2-12,
  MAXRELERROR 1-4, free surface (elastic and viscoelastic), L = 3, VTI/TTI with
  CPML, periodic x, force / custom-force / moment-tensor sources and ragged
  grid sizes; and the acquisition set-ups of ACQ_CASES (receiver planes,
  receivers and sources below the topography, co-located receivers) and the
  plane wave's source table (``ref_acq_plane_wave.npz``). Models are regenerated from the seed by ``synthetic_model`` (a
  CRC of the model bytes is stored to catch a drift).

    python tests/golden/make_fixtures.py [--reference <reference source tree>]
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import tempfile
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
from tests.golden.cases import (ACQ_CASES, CASES, FORMAT_CASE, FWI_CASES, PLANE_WAVE_CASE,  # noqa: E402
                                SNAP_SHOTS_CASE, WAVELET_CASES, WAVELET_DT, WAVELET_NT, _case, fwi_json_text,
                                json_text, synthetic_model, true_model, write_case, write_signal_file)

SHIPPED = {"weq3": "EL_ISO", "weq4": "VEL_ISO", "weq5": "EL_VTI", "weq6": "VEL_VTI", "weq7": "EL_TTI",
           "weq8": "VEL_TTI", "weq3_fy": "EL_ISO", "weq8_fy": "VEL_TTI", "weq3_fdt4": "EL_ISO",
           "weq4_fdt4": "VEL_ISO"}


def read_su(path):
    b = np.fromfile(path, dtype=np.uint8)
    ns = int(b[114:116].view(np.uint16)[0])
    rec = 240 + 4 * ns
    ntr = b.size // rec
    b = b[: ntr * rec].reshape(ntr, rec)
    return b[:, :240].copy(), b[:, 240:].copy().view(np.float32).reshape(ntr, ns)


def shipped(reference):
    ex = os.path.join(reference, "examples")
    for name in SHIPPED:
        base = name.split("_")[0]
        suffix = name[len(base):]  # "", "_fy" or "_fdt4"
        out = {}
        for comp in ["vx", "vy", "p", "div", "curl"]:
            f = os.path.join(ex, f"{base}_ref", f"seis{suffix}_{comp}.su")
            hdr, data = read_su(f)
            out[f"seis_{comp}"] = data
            out[f"hdr_{comp}"] = hdr
            s = os.path.join(ex, f"{base}_ref", f"snap{suffix}.bin.{comp}")
            if os.path.exists(s):
                a = np.fromfile(s, dtype=np.float32).reshape(4, 200, 200)
                out[f"snapnorm_{comp}"] = np.sqrt((a.astype(np.float64) ** 2).sum(axis=(1, 2)))
                out[f"snapsub_{comp}"] = a[:, ::8, ::8].copy()
        np.savez_compressed(os.path.join(HERE, f"shipped_{name}.npz"), **out)
        print("wrote shipped", name)


def shipped_sigout(reference):
    """The source wavelet file the reference writes with SIGOUT = 1 (SU) for
    examples/weq3.json, byte for byte."""
    f = os.path.join(reference, "examples", "weq3_ref", "signal_out.shot1.su")
    raw = np.fromfile(f, dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "shipped_sigout_weq3.npz"), raw=raw)
    print("wrote shipped sigout", raw.size, "bytes")


def run_reference(case, exe):
    work = tempfile.mkdtemp(prefix="sofi_fix_")
    try:
        jpath, mats = write_case(case, work)
        r = subprocess.run([exe, jpath], cwd=work, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"{case['name']}: reference failed\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
        out = {}
        for comp in ["vx", "vy", "p", "div", "curl"]:
            f = os.path.join(work, "out", f"seis_{comp}.su")
            if os.path.exists(f):
                hdr, data = read_su(f)
                out[f"seis_{comp}"] = data
                out[f"hdr_{comp}"] = hdr
            s = os.path.join(work, "out", f"snap.bin.{comp}.0.0")
            if os.path.exists(s):
                out[f"snap_{comp}"] = np.fromfile(s, dtype=np.float32)
        crc = 0
        for k in sorted(mats):
            crc = zlib.crc32(mats[k].tobytes(), crc)
        out["model_crc"] = np.array([crc], dtype=np.uint64)
        out["case"] = np.frombuffer(json.dumps(case, sort_keys=True).encode(), dtype=np.uint8)
        return out
    finally:
        shutil.rmtree(work, ignore_errors=True)


def ref_examples(reference, exe):
    """One-rank compiled-reference runs of the TTI examples and of weq3
    (seismograms and their SU headers; the shipped weq3 files were written by
    an older version whose headers place receivers at index * DH)."""
    ex = os.path.join(reference, "examples")
    for name in ["weq3", "weq7", "weq8", "weq8_fy"]:
        work = tempfile.mkdtemp(prefix="sofi_ex_")
        try:
            for d in ["model", "sources", "receiver"]:
                os.symlink(os.path.join(ex, d), os.path.join(work, d))
            base = name.split("_")[0]
            os.makedirs(os.path.join(work, base), exist_ok=True)
            os.makedirs(os.path.join(work, "log"), exist_ok=True)
            txt = open(os.path.join(ex, f"{name}.json")).read()
            txt = txt.replace('"NPROCX" : "2"', '"NPROCX" : "1"').replace('"NPROCY" : "2"', '"NPROCY" : "1"')
            txt = txt.replace('"SNAP" : "4"', '"SNAP" : "0"')
            with open(os.path.join(work, "run.json"), "w") as fh:
                fh.write(txt)
            r = subprocess.run([exe, "run.json"], cwd=work, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(r.stdout[-2000:])
            suffix = "_fy" if name.endswith("_fy") else ""
            out = {}
            for comp in ["vx", "vy", "p", "div", "curl"]:
                out[f"hdr_{comp}"], out[f"seis_{comp}"] = read_su(os.path.join(work, base, f"seis{suffix}_{comp}.su"))
            np.savez_compressed(os.path.join(HERE, f"ref1x1_{name}.npz"), **out)
            print("wrote ref1x1", name)
        finally:
            shutil.rmtree(work, ignore_errors=True)


def ref_wavelets(exe):
    """The first source's signal as the compiled reference computes it
    (wavelet.c) for every SOURCE_SHAPE, written by its SIGOUT output in
    float32: ref_wavelets.npz holds, per case, the signal and the inputs."""
    out = {}
    for wc in WAVELET_CASES:
        work = tempfile.mkdtemp(prefix="sofi_wav_")
        try:
            case = _case("wav_" + wc["name"], nx=40, ny=40, dh=2.0, dt=WAVELET_DT, nt=WAVELET_NT, fw=0, abs_type=0,
                         seismo=1, ndt=1, snap=0, seed=3)
            jpath, _ = write_case(case, work)
            with open(os.path.join(work, "source.dat"), "w") as fh:
                fh.write(wc["line"] + "\n")
            txt = open(jpath).read()
            sigfile = "none"
            if wc["shape"] == 3:
                write_signal_file(wc, work)
                sigfile = "./" + wc["signal_file"]
            txt = txt.replace('"SOURCE_SHAPE" : "1"', f'"SOURCE_SHAPE" : "{wc["shape"]}"')
            txt = txt.replace('"SIGNAL_FILE" : "none"', f'"SIGNAL_FILE" : "{sigfile}"')
            txt = txt.replace('"SIGOUT" : "0",', '"SIGOUT" : "1",\n"SIGOUT_FORMAT" : "3",\n"SIGOUT_FILE" : "./out/sig",')
            with open(jpath, "w") as fh:
                fh.write(txt)
            r = subprocess.run([exe, jpath], cwd=work, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"{wc['name']}: reference failed\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
            sig = np.fromfile(os.path.join(work, "out", "sig.shot1.bin"), dtype=np.float32)
            assert sig.size == WAVELET_NT, (wc["name"], sig.size)
            out[f"{wc['name']}_signal"] = sig
            print("wrote wavelet", wc["name"], float(np.abs(sig).max()))
        finally:
            shutil.rmtree(work, ignore_errors=True)
    np.savez_compressed(os.path.join(HERE, "ref_wavelets.npz"), **out)


def ref_formats(exe):
    """The same run written with SEIS_FORMAT / SNAP_FORMAT 3 (float32) and 2
    (ASCII): ref_fmt_out.npz holds every file's bytes."""
    out = {}
    for fmt, ext, sext in ((3, "bin", "bin"), (2, "txt", "asc")):
        case = dict(FORMAT_CASE, par={"SEIS_FORMAT": str(fmt), "SNAP_FORMAT": str(fmt)})
        work = tempfile.mkdtemp(prefix="sofi_fmt_")
        try:
            jpath, _ = write_case(case, work)
            r = subprocess.run([exe, jpath], cwd=work, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"formats {fmt}: reference failed\n{r.stdout[-2000:]}")
            for comp in ("vx", "vy"):
                out[f"seis{fmt}_{comp}"] = np.fromfile(os.path.join(work, "out", f"seis_{comp}.{ext}"), np.uint8)
                out[f"snap{fmt}_{comp}"] = np.fromfile(os.path.join(work, "out", f"snap.{sext}.{comp}.0.0"),
                                                       np.uint8)
        finally:
            shutil.rmtree(work, ignore_errors=True)
    np.savez_compressed(os.path.join(HERE, "ref_fmt_out.npz"), **out)
    print("wrote fmt_out", {k: v.size for k, v in out.items()})


def ref_plane_wave(exe):
    """The plane-wave sources as the compiled reference logs them: it builds
    them and prints its source table, then crashes reading past its 8-row
    source matrix (splitsrc.c:50-51). ref_acq_plane_wave.npz holds the table
    (shot, x, y, tshift, fc, amp, azimuth, type) of the first 50 sources."""
    case = PLANE_WAVE_CASE
    work = tempfile.mkdtemp(prefix="sofi_pw_")
    try:
        jpath, _ = write_case(case, work)
        r = subprocess.run([exe, jpath], cwd=work, capture_output=True, text=True)
        assert r.returncode != 0, "the reference's plane-wave path ran through: read its seismograms instead"
        rows = []
        for ln in r.stdout.splitlines():
            t = ln.split("]", 1)[-1].split()
            if ln.startswith("INFO") and len(t) == 8 and t[0].isdigit():
                rows.append([float(v) for v in t])
        assert len(rows) == 50, len(rows)
        np.savez_compressed(os.path.join(HERE, "ref_acq_plane_wave.npz"), table=np.array(rows),
                            case=np.frombuffer(json.dumps(case, sort_keys=True).encode(), dtype=np.uint8))
        print("wrote acq_plane_wave", len(rows), "sources; the reference exited with", r.returncode)
    finally:
        shutil.rmtree(work, ignore_errors=True)


def run_reference_fwi(case, exe):
    """Observed data from a forward run on the case's true model, then one
    FWI gradient pass on its model (MODE = FWI), both with the compiled
    reference: the observed sections, the FWI forward sections and the
    per-shot vp / vs / rho' gradients ([NY][NX])."""
    work = tempfile.mkdtemp(prefix="sofi_fwi_")
    try:
        jpath, mats = write_case(case, work)
        nx, ny = case["nx"], case["ny"]
        true = true_model(case, mats)
        os.makedirs(os.path.join(work, "true"), exist_ok=True)
        for k, v in true.items():
            v.astype(np.float32).tofile(os.path.join(work, "true", f"m.{k}"))
        for d in ("obs", "grad", "inv"):
            os.makedirs(os.path.join(work, d), exist_ok=True)
        txt = json_text(case).replace('"MFILE" : "./model/m"', '"MFILE" : "./true/m"')
        txt = txt.replace('"SEIS_FILE" : "./out/seis"', '"SEIS_FILE" : "./obs/seis"')
        with open(os.path.join(work, "true.json"), "w") as fh:
            fh.write(txt)
        with open(os.path.join(work, "fwi.json"), "w") as fh:
            fh.write(fwi_json_text(case))
        for run in ("true.json", "fwi.json"):
            r = subprocess.run([exe, run], cwd=work, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"{case['name']} {run}: reference failed\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
            if run == "true.json":
                for comp in ("vx", "vy"):
                    shutil.copy(os.path.join(work, "obs", f"seis_{comp}.su"),
                                os.path.join(work, "obs", f"seis_{comp}.su.shot1"))
        out = {}
        for comp in ("vx", "vy"):
            _, out[f"obs_{comp}"] = read_su(os.path.join(work, "obs", f"seis_{comp}.su"))
            _, out[f"fwd_{comp}"] = read_su(os.path.join(work, "out", f"seis_{comp}.su.shot1"))
        for g in ("vp", "vs", "rho"):
            a = np.fromfile(os.path.join(work, "grad", f"g_gradient.{g}.shot1"), dtype=np.float32)
            out[f"grad_{g}"] = a.reshape(nx, ny).T.copy()  # writemod.c: x outer, y inner
        out["case"] = np.frombuffer(json.dumps(case, sort_keys=True).encode(), dtype=np.uint8)
        return out
    finally:
        shutil.rmtree(work, ignore_errors=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None,
                    help="reference source tree (default: the one oracle/_ref was built from)")
    ap.add_argument("--only", default="")
    a = ap.parse_args()
    if a.reference is None:
        with open(os.path.join(REPO, "oracle", "_ref", "source_dir.txt")) as fh:
            a.reference = fh.read().strip()
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle", "ref"), f"REFERENCE={a.reference}"],
                   check=True)
    exe = os.path.join(REPO, "oracle", "_ref", "sofi2D")
    if not a.only:
        shipped(a.reference)
    if not a.only or a.only == "examples":
        ref_examples(a.reference, exe)
        if a.only:
            return
    if not a.only or a.only == "sigout":
        shipped_sigout(a.reference)
        if a.only:
            return
    if not a.only or a.only == "wavelets":
        ref_wavelets(exe)
        if a.only:
            return
    if not a.only or a.only == "fmt_out":
        ref_formats(exe)
        if a.only:
            return
    if not a.only or a.only == "acq_plane_wave":
        ref_plane_wave(exe)
        if a.only:
            return
    if not a.only or a.only == SNAP_SHOTS_CASE["name"]:  # which shot's snapshots the files keep
        out = run_reference(SNAP_SHOTS_CASE, exe)
        np.savez_compressed(os.path.join(HERE, f"ref_{SNAP_SHOTS_CASE['name']}.npz"), **out)
        print("wrote", SNAP_SHOTS_CASE["name"], sorted(k for k in out if k.startswith("snap")))
        if a.only:
            return
    for case in ACQ_CASES:  # receiver planes, topography, co-located receivers
        if a.only and case["name"] != a.only:
            continue
        out = run_reference(case, exe)
        np.savez_compressed(os.path.join(HERE, f"ref_{case['name']}.npz"), **out)
        print("wrote", case["name"], out["hdr_vx"].shape)
    for case in FWI_CASES:
        if a.only and case["name"] != a.only:
            continue
        out = run_reference_fwi(case, exe)
        np.savez_compressed(os.path.join(HERE, f"ref_{case['name']}.npz"), **out)
        print("wrote", case["name"], "gradients", [float(np.abs(out[f"grad_{g}"]).max()) for g in ("vp", "vs", "rho")])
    for case in CASES:
        if (a.only and case["name"] != a.only) or not case.get("compiled_ref", True):
            continue
        out = run_reference(case, exe)
        np.savez_compressed(os.path.join(HERE, f"ref_{case['name']}.npz"), **out)
        print("wrote", case["name"], sorted(k for k in out if k.startswith("seis")))


if __name__ == "__main__":
    main()
