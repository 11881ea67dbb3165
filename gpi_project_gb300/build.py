"""Build the native libraries of gpi_project_gb300 in-tree (gpi_project_gb300/_build/).

* libsofigpu.so  -- CUDA kernels + C ABI (include/sofigpu.h), sm_103a only.
* libsofihost.so -- C host: parameter/model/acquisition readers, model
                    preparation, SU/snapshot writers (include/sofihost.h).
* libsofiserve.so -- continuous-batching request loop over the two above
                    (include/sofiserve.h).
* sofi2d_gb300   -- command-line driver (reads a SOFI2D parameter file).

Sources compile in parallel; nvcc cross-compiles without a GPU.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
INC = os.path.join(REPO, "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("build failed: " + " ".join(cmd))
    return r


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def cuda_objects():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith(".cu")]


def host_sources():
    d = os.path.join(CSRC, "host")
    return [os.path.join(d, f) for f in sorted(os.listdir(d)) if f.endswith(".c") and f != "sofi2d_main.c"]


def _deps(exts):
    out = []
    for root in (CSRC, INC):
        for dp, _, fs in os.walk(root):
            out += [os.path.join(dp, f) for f in fs if f.endswith(exts)]
    return out


def build(verbose: bool = False) -> dict:
    os.makedirs(OUT, exist_ok=True)
    gpu_lib = os.path.join(OUT, "libsofigpu.so")
    host_lib = os.path.join(OUT, "libsofihost.so")
    cli = os.path.join(OUT, "sofi2d_gb300")
    serve_lib = os.path.join(OUT, "libsofiserve.so")
    serve_src = os.path.join(CSRC, "serve", "sofiserve.c")
    jobs = []
    cu = cuda_objects()
    deps_cu = _deps((".cu", ".cuh", ".h"))
    if _newer(gpu_lib, deps_cu):
        objs = []
        for src in cu:
            obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
            objs.append(obj)
            jobs.append([NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INC,
                         "-I", CSRC, "-c", src, "-o", obj])
    else:
        objs = None
    hs = host_sources()
    deps_h = _deps((".c", ".h"))
    host_build = _newer(host_lib, deps_h) or _newer(cli, deps_h)
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        list(ex.map(_run, jobs))
    if objs is not None:
        _run([NVCC, *ARCH, "-shared", "-o", gpu_lib, *objs, "-lcudart"])
    if host_build and hs:
        _run(["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-fPIC", "-shared", "-fopenmp", "-Wall", "-I", INC,
              "-o", host_lib, *hs, "-lm"])
        main = os.path.join(CSRC, "host", "sofi2d_main.c")
        if os.path.exists(main):
            _run(["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-fopenmp", "-Wall", "-I", INC, "-o", cli, main, *hs,
                  "-L", OUT, "-lsofigpu", "-Wl,-rpath,$ORIGIN", "-lm"])
    if _newer(serve_lib, [serve_src, gpu_lib, host_lib] + _deps((".h",))):
        _run(["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-fPIC", "-shared", "-Wall", "-I", INC, "-o", serve_lib,
              serve_src, "-L", OUT, "-lsofigpu", "-lsofihost", "-Wl,-rpath,$ORIGIN", "-lpthread", "-lm"])
    return {"gpu": gpu_lib, "host": host_lib, "cli": cli, "serve": serve_lib}


if __name__ == "__main__":
    print(build(verbose=True))
