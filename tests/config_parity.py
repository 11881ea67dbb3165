"""Parity of the GPU path with the oracle at the benchmark configurations.

One workload of ``gpi_project_gb300.workloads`` (c1-c4: the plain elastic
400 x 400 solve, the viscoelastic 4000 x 2000 solve with free surface, the TTI
2048 x 2048 solve, 64 batched viscoelastic shots on 2000 x 1000) runs

  * on the GPU through the product path: host preparation by libsofihost,
    the autotuned kernel variants, every shot of the workload in one context;
  * through the float32 oracle (bit-identical to the reference's own float
    build, reference src/time_loop.c:27-326) and the float64 oracle (the same
    stencil in double, the arbiter), one context per checked shot.

The compared outputs are what time_loop() hands back after NT steps: the
seismogram sections that seismo_ssg.c:28-67 fills at time_loop.c:282-285 and
the final wavefield (a snapshot of vx, vy, sxx, syy, sxy at step NT). For each
component the relative L2 error ||a - b|| / ||b|| and the relative max error
max|a - b| / max|b| are stated for the three pairs GPU-f32, GPU-f64 and
f32-f64. Denominators are floored at 1 % of the largest component of the same
shot and physical unit (a near-silent component would otherwise dominate);
over several shots the largest error counts.
"""
from __future__ import annotations

import json
import os
import time

import numpy as np

SECTION_COMPS = {1: ["vx", "vy"], 2: ["p"], 3: ["div", "curl"], 4: ["vx", "vy", "p", "div", "curl"]}
FIELDS = ["vx", "vy", "sxx", "syy", "sxy"]
PAIRS = ("gpu_f32", "gpu_f64", "f32_f64")
L2_TOL, MAX_TOL = 1e-4, 1e-3


def _oracle_config(par):
    from oracle import oracle as O
    cfg = O.SofiConfig()
    for k in ["weq", "nx", "ny", "dh", "dt", "fdorder", "maxrelerror", "L", "fw", "abs_type", "free_surf",
              "npower", "k_max_cpml", "vppml", "fpml", "seismo", "ndt", "fdorder_time"]:
        if k in par:
            setattr(cfg, k, par[k])
    cfg.f_ref, cfg.fl = par.get("f_ref", 0.0), list(par.get("fl", []))
    cfg.nt = par["nt"]
    return cfg


def oracle_outputs(W, shot, precision, nthreads=0):
    """Sections and final wavefield of one shot through the oracle."""
    from oracle import oracle as O
    par = W["par"]
    cfg = _oracle_config(par)
    o = O.Oracle(cfg, precision, nthreads)
    try:
        o.set_material({k: v.reshape(-1) for k, v in W["mats"].items()})
        srcs = W["src"] if isinstance(W["src"], list) else [W["src"]]
        src = srcs[shot % len(srcs)]
        # identical float32 signals for both builds: the arbiter measures the stencil arithmetic
        o.set_sources(src, O.wavelet(1, cfg.nt, cfg.dt, src))
        o.set_receivers(*W["rec"])
        o.run()
        return ({c: o.section(c) for c in SECTION_COMPS[par["seismo"]]}, {f: o.field(f) for f in FIELDS})
    finally:
        o.close()


def gpu_outputs(W, shots, device=0):
    """Sections and final wavefield of the given shots through the GPU path."""
    from gpi_project_gb300 import workloads
    t, *_ = workloads.gpu_loop(W, device=device)
    try:
        t.reset()
        t0 = time.perf_counter()
        t.run()
        secs = time.perf_counter() - t0
        variant = {"velocity": list(t.velocity_variant()), "stress": t.stress_variant(),
                   "block_threads_x": list(t.block_threads_x())}
        out = {s: ({c: t.section(c, shot=s) for c in SECTION_COMPS[W["par"]["seismo"]]},
                   {f: t.field(f, shot=s) for f in FIELDS}) for s in shots}
        return out, variant, secs
    finally:
        t.close()


def _errs(a, b, floor_l2, floor_max):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = a - b
    return (float(np.linalg.norm(d) / max(np.linalg.norm(b), floor_l2)),
            float(np.abs(d).max() / max(np.abs(b).max(), floor_max)))


# components of one physical quantity share a floor: velocities, stresses, velocity derivatives
UNIT_GROUP = {"vx": "v", "vy": "v", "sxx": "s", "syy": "s", "sxy": "s", "p": "s", "div": "d", "curl": "d"}


def _floors(group, comp):
    """1 % of the largest L2 norm and max among the components of ``group``
    that share ``comp``'s physical unit."""
    same = [np.asarray(v, np.float64) for c, v in group.items() if UNIT_GROUP[c] == UNIT_GROUP[comp]]
    return 0.01 * max(np.linalg.norm(v) for v in same), 0.01 * max(float(np.abs(v).max()) for v in same)


def compare(gpu, f32, f64):
    """Per component, the (relL2, relMax) of the three pairs for one shot."""
    res = {}
    for gi, kind in ((0, "sections"), (1, "fields")):
        g, a, b = gpu[gi], f32[gi], f64[gi]
        for c in g:
            fl32, fl64 = _floors(a, c), _floors(b, c)
            res[f"{kind}.{c}"] = {"gpu_f32": _errs(g[c], a[c], *fl32), "gpu_f64": _errs(g[c], b[c], *fl64),
                                  "f32_f64": _errs(a[c], b[c], *fl64)}
    return res


def merge_max(per_shot):
    out = {}
    for r in per_shot:
        for c, pairs in r.items():
            o = out.setdefault(c, {p: [0.0, 0.0] for p in PAIRS})
            for p in PAIRS:
                o[p] = [max(o[p][0], pairs[p][0]), max(o[p][1], pairs[p][1])]
    return out


def config_parity(name, nt=None, check_shots=None, nthreads=0, device=0):
    """GPU, float32 oracle and float64 oracle on workload ``name``; the error table."""
    from gpi_project_gb300 import workloads
    W = workloads.workload(name)
    if nt:
        W["par"]["nt"] = int(nt)
    shots = list(check_shots) if check_shots else [0]
    gpu, variant, gpu_s = gpu_outputs(W, shots, device)
    per_shot, ts = [], {"f32": 0.0, "f64": 0.0}
    for s in shots:
        outs = {}
        for prec in ("f32", "f64"):
            t0 = time.perf_counter()
            outs[prec] = oracle_outputs(W, s, prec, nthreads)
            ts[prec] += time.perf_counter() - t0
        per_shot.append(compare(gpu[s], outs["f32"], outs["f64"]))
    par = W["par"]
    return {"workload": name, "nx": par["nx"], "ny": par["ny"], "nt": par["nt"], "full_nt": nt is None,
            "weq": par["weq"], "fdorder": par["fdorder"], "L": par.get("L", 0), "shots": W["nshots"],
            "shots_checked": shots, "variant": variant, "gpu_run_s": round(gpu_s, 2),
            "oracle_s": {k: round(v, 1) for k, v in ts.items()}, "errors": merge_max(per_shot)}


def within_bar(rec, pair="gpu_f32"):
    return all(e[pair][0] <= L2_TOL and e[pair][1] <= MAX_TOL for e in rec["errors"].values())


def save_record(rec, path):
    """Add one workload's table to the JSON record at ``path``."""
    data = {}
    if os.path.exists(path):
        with open(path) as f:
            data = json.load(f)
    data[rec["workload"]] = rec
    with open(path, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
