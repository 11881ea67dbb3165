"""The drop-in time_loop() shim compiles against the reference's headers and
links with the reference's objects in place of src/time_loop.c (CPU only:
building and linking, no GPU call). Skipped where the reference tree is absent."""
import glob
import os
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference_tree():
    """The reference source tree oracle/_ref was built from (build() records it)."""
    try:
        with open(os.path.join(REPO, "oracle", "_ref", "source_dir.txt")) as fh:
            return fh.read().strip()
    except OSError:
        return ""


REF = _reference_tree()


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")), reason="reference sources not present")
def test_shim_links_into_reference(tmp_path):
    from gpi_project_gb300 import build
    out = build.build()
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle", "ref"), f"REFERENCE={REF}"], check=True)
    objs = [o for o in glob.glob(os.path.join(REPO, "oracle", "_ref", "obj", "*.o"))
            if not o.endswith("fd_time_loop.o")]
    shim_o = str(tmp_path / "time_loop_gb300.o")
    subprocess.run(["gcc", "-O2", "-std=c99", "-D_GNU_SOURCE", "-DUSE_MPI", "-c",
                    "-I", os.path.join(REPO, "oracle", "ref", "mpi_stub"), "-I", os.path.join(REF, "src"),
                    "-I", os.path.join(REF, "libkissfft"), "-I", os.path.join(REPO, "include"),
                    os.path.join(REPO, "gpi_project_gb300", "csrc", "shim", "time_loop_gb300.c"), "-o", shim_o],
                   check=True)
    exe = str(tmp_path / "sofi2D_gb300_timeloop")
    subprocess.run(["gcc", "-o", exe, shim_o, *objs, "-L", os.path.dirname(out["gpu"]), "-lsofigpu",
                    f"-Wl,-rpath,{os.path.dirname(out['gpu'])}", "-lm"], check=True)
    assert os.path.exists(exe)
    nm = subprocess.run(["nm", shim_o], capture_output=True, text=True).stdout
    assert " T time_loop" in nm and "U sofi_run" in nm
