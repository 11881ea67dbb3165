#!/usr/bin/env python3
"""Benchmark of the SOFI2D time loop on GB300: Gcell-updates/s and % of the HBM roofline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c2] [--impl gb300|reference]

A step is one complete forward solve of the workload (reset + NT time steps,
what one time_loop() call of the reference does for one shot). Default
workload: c2 (viscoelastic 4000 x 2000, L = 3, FD8, CPML 30, free surface,
NT 6000; see gpi_project_gb300/workloads.py), seeded synthetic inputs.

value      NX*NY*NT*shots / device time of the K timed steps (inputs resident in
           HBM; CUDA events on the library's stream), in Gcell-updates/s
e2e        the same through the C ABI from pinned host buffers: model upload,
           sources/receivers, run, section download inside the timed region
roofline   dominant kernel (the stress update): algorithmic bytes per launch /
           its mean event-timed duration, against the measured HBM copy peak
cpu_baseline  the oracle (CPU restatement of the reference, all host threads)
           on a bounded sample of the same grid
--impl reference  times that CPU implementation as the reference arm.
Multi-GPU: replicas only (independent solves, no collective); rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="c2")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=0, help="time steps of the CPU sample (0 = auto)")
    ap.add_argument("--served-requests", type=int, default=24,
                    help="requests of the served (c5) leg added to the line; 0 = none")
    ap.add_argument("--batched-leg", default="c4",
                    help="batched workload timed after the main line and added to it ('' = none)")
    ap.add_argument("--nt", type=int, default=0,
                    help="time steps per solve (default: the workload's NT; a small value keeps profiler captures short)")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float, device: str = "cuda") -> float:
    """The largest of every rank's x (a duration: the job ends with its slowest
    replica); x itself when there is one rank."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Whole-job throughput of `world` replicas that each processed
    units_per_rank, in the slowest one's `seconds` (weak scaling)."""
    return units_per_rank * world / seconds


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def traffic_from_profiles(kernel: str, workload: str):
    """DRAM bytes per cell of `kernel` from the committed ncu summary, if any."""
    p = os.path.join(REPO, "profiles", "traffic.json")
    try:
        with open(p) as fh:
            d = json.load(fh)
        return d[workload][kernel]["dram_bytes_per_cell"]
    except (OSError, KeyError, ValueError):
        return None


def host_par(W):
    from gpi_project_gb300 import host
    return host.make_par(**W["par"])


def working_set_bytes(W) -> float:
    """Device bytes the workload's solves keep resident: the state arrays of
    every shot and the per-cell coefficient arrays (CPML frames and
    receivers not counted)."""
    from gpi_project_gb300 import workloads
    par = W["par"]
    L = par.get("L", 0)
    state = 5 + 3 * L
    bpc = workloads.bytes_per_cell(par["weq"], L, par.get("fdorder_time", 2))["step"]
    coeff = max(0, (bpc - 8 * state) // 4)
    return 4.0 * par["nx"] * par["ny"] * (state * W["nshots"] + coeff)


def config_of(W, world: int) -> dict:
    """The `config` object of the line, the same for both arms."""
    par = W["par"]
    ws = working_set_bytes(W)
    l2 = (f"inputs larger than L2 (resident working set ~{ws / 1e9:.2f} GB)" if ws > 129e6 else
          f"working set ~{ws / 1e6:.0f} MB stays in L2 between steps (part of this workload)")
    return {"workload": W["name"], "nx": par["nx"], "ny": par["ny"], "nt": par["nt"], "weq": par["weq"],
            "fdorder": par["fdorder"], "L": par.get("L", 0), "fw": par["fw"], "shots": W["nshots"],
            "free_surf": par.get("free_surf", 0), "receivers": len(W["rec"][0]), "l2": l2,
            "parallelism": f"replicas x{world}"}


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return "unknown"


def cpu_leg(args, workload: str) -> dict:
    """cpu_baseline of the main line: the reference arm's own measurement
    (`--impl reference`, all host threads), run as a fresh process before
    this one loads CUDA or torch, so both readings come from the same code in
    the same process state."""
    cmd = [sys.executable, os.path.abspath(__file__), "--impl", "reference", "--workload", workload,
           "--steps", "3", "--warmup", "1"]
    if args.nt:
        cmd += ["--nt", str(args.nt)]
    if args.cpu_steps:
        cmd += ["--cpu-steps", str(args.cpu_steps)]
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "LOCAL_WORLD_SIZE")}
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=900)
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    if r.returncode or not lines:
        raise SystemExit(f"CPU baseline leg failed (rc {r.returncode}): {r.stderr[-2000:]}")
    return json.loads(lines[-1])["cpu_baseline"]


def parity_record(workload: str):
    """The error table of the GPU path against the float32 oracle and the
    float64 arbiter at this workload's full size, as the config-parity GPU
    test recorded it (profiles/parity_configs.json), or None."""
    p = os.path.join(REPO, "profiles", "parity_configs.json")
    try:
        with open(p) as fh:
            d = json.load(fh)[workload]
    except (OSError, KeyError, ValueError):
        return None
    return {"source": "tests/test_gpu_xl_configs.py on GB300, recorded in profiles/parity_configs.json",
            "nt": d["nt"], "full_nt": d["full_nt"], "shots_checked": d["shots_checked"],
            "bar": {"rel_l2": 1e-4, "rel_max": 1e-3},
            "errors_rel_l2_rel_max": {c: {p: [float(f"{x:.3g}") for x in v] for p, v in e.items()}
                                      for c, e in d["errors"].items()}}


def cpu_sample(W, nsteps, nthreads):
    """Gcell-updates/s of the oracle on `nsteps` time steps of the workload grid,
    timed after a few warm-up steps (the first touch of the freshly allocated
    fields and the thread pool's start stay out of the sample, as the GPU's
    warm-up steps do)."""
    from oracle import oracle as O
    par = W["par"]
    cfg = O.SofiConfig()
    for k in ["weq", "nx", "ny", "dh", "dt", "fdorder", "maxrelerror", "L", "fw", "abs_type", "free_surf",
              "npower", "k_max_cpml", "vppml", "fpml", "seismo", "ndt", "fdorder_time"]:
        if k in par:
            setattr(cfg, k, par[k])
    cfg.f_ref, cfg.fl = par.get("f_ref", 0.0), list(par.get("fl", []))
    cfg.nt = par["nt"]
    o = O.Oracle(cfg, "f32", nthreads)
    o.set_material({k: v.reshape(-1) for k, v in W["mats"].items()})
    src = W["src"] if isinstance(W["src"], np.ndarray) else W["src"][0]
    o.set_sources(src, O.wavelet(1, cfg.nt, cfg.dt, src))
    o.set_receivers(*W["rec"])
    warm = min(max(2, nsteps // 10), cfg.nt - nsteps)
    if warm > 0:
        o.run(warm)
    t0 = time.perf_counter()
    o.run(nsteps)
    dt = time.perf_counter() - t0
    o.close()
    return cfg.nx * cfg.ny * nsteps / dt / 1e9, dt


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def auto_cpu_steps(W, target_s=12.0, rate_per_core=10e6):
    cells = W["par"]["nx"] * W["par"]["ny"]
    n = int(target_s * rate_per_core * cpu_threads() / cells)
    return max(5, min(n, W["par"]["nt"]))


def run_reference(args, W):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    n = args.cpu_steps or auto_cpu_steps(W, target_s=6.0)
    nth = cpu_threads()
    for _ in range(args.warmup):
        cpu_sample(W, max(1, n // 4), nth)
    rates, secs = [], 0.0
    for _ in range(args.steps):
        r, s = cpu_sample(W, n, nth)
        rates.append(r)
        secs += s
    val = float(np.mean(rates))
    par = W["par"]
    line = {
        "impl": "reference", "metric": "Gcell-updates/s", "value": round(val, 4), "unit": "Gcell-updates/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * secs / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded; gpi_project_gb300/workloads.py)",
        "config": config_of(W, world),
        "cpu_baseline": {"value": round(val, 4), "unit": "Gcell-updates/s", "cores": nth, "kind": "port",
                         "cpu_model": cpu_model(), "spread": [round(min(rates), 4), round(max(rates), 4)],
                         "sample": f"{n} time steps of the {par['nx']}x{par['ny']} grid per step, after "
                                   f"{args.warmup} warm-up samples; first shot only"},
        "e2e": {"value": round(val, 4), "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def served_leg(n_req: int, device: int, passes: int = 1, seed: int = 1005) -> dict:
    """c5: a seeded stream of uneven solves through the request loop.

    Three runs of the same stream: the plain loop (one solve resident at a
    time, the reference's one-shot-after-another order), the loop with every
    request arriving at once (throughput, HBM roofline), and Poisson arrivals at
    70 % of that throughput (latency). Host arrays in, sections out: every run
    is end to end, model preparation included.
    """
    from gpi_project_gb300 import host, serve, workloads
    reqs = workloads.request_stream(n_req, seed=seed)
    cells = sum(r["cell_updates"] for r in reqs)
    alg = sum(r["cell_updates"] * workloads.bytes_per_cell(r["par"]["weq"], r["par"]["L"])["step"] for r in reqs)
    h2d = sum(sum(a.nbytes for a in r["mats"].values()) for r in reqs)

    def run(max_resident, arrivals, stream=reqs):
        with serve.Server(device=device, max_resident=max_resident) as srv:
            t0 = srv.clock() + 0.01
            ids = [srv.submit(host.make_par(**r["par"]), r["mats"], r["src"], *r["rec"], arrival=t0 + a)
                   for r, a in zip(stream, arrivals)]
            srv.drain()
            st = srv.stats()
            d2h = 0
            for rid in ids:
                i = srv.info(rid)
                if i["state"] != serve.REQ_DONE:
                    raise SystemExit(f"served request {rid} failed: {i['error']}")
                d2h += i["ntr"] * i["ns"] * 4 * 2
            st["d2h"] = d2h
            st["makespan"] = st["last_finish"] - t0
        return st

    warm = workloads.request_stream(3, seed=seed + 100, nt_range=(64, 64), nx_range=(256, 512),
                                    ny_range=(256, 512))
    run(8, [0.0] * len(warm), warm)
    zero = [0.0] * n_req
    plain = run(1, zero)
    sats = [run(64, zero) for _ in range(passes)]
    sat = min(sats, key=lambda x: x["makespan"])
    rate = 0.7 * n_req / sat["makespan"]
    rng = __import__("numpy").random.default_rng(seed + 1)
    arr = list(__import__("numpy").cumsum(rng.exponential(1.0 / rate, n_req)))
    lat = run(64, arr)
    peak, peak_kind = measured_peaks()
    ach = alg / sat["makespan"] / 1e9
    return {
        "requests": n_req, "cell_updates": cells, "makespan_s": round(sat["makespan"], 4),
        "grid": "NX 256-4096, NY 256-2048 log-uniform; NT 1000-6000; FDORDER 4/8; elastic or viscoelastic L=3",
        "gcell_per_s": round(cells / sat["makespan"] / 1e9, 3),
        "shots_per_s": round(n_req / sat["makespan"], 3),
        "plain_gcell_per_s": round(cells / plain["makespan"] / 1e9, 3),
        "plain_shots_per_s": round(n_req / plain["makespan"], 3),
        "speedup_vs_plain": round(plain["makespan"] / sat["makespan"], 3),
        "hbm_roofline": {"achieved": round(ach, 1), "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": round(ach / peak, 4), "algorithmic_bytes": int(alg)},
        "all_at_once": {"p50_s": round(sat["p50_s"], 3), "p99_s": round(sat["p99_s"], 3),
                        "plain_p50_s": round(plain["p50_s"], 3), "plain_p99_s": round(plain["p99_s"], 3),
                        "peak_resident": sat["peak_resident"], "peak_bytes": sat["peak_bytes"]},
        "poisson": {"rate_per_s": round(rate, 3), "p50_s": round(lat["p50_s"], 3), "p99_s": round(lat["p99_s"], 3),
                    "mean_s": round(lat["mean_s"], 3), "peak_resident": lat["peak_resident"]},
        "h2d_bytes": int(h2d), "d2h_bytes": int(sat["d2h"]), "gpu_launches": int(sat["launches"]),
    }


def main_served(args):
    """--workload c5: the request stream through the serving loop is the line."""
    rank, world, local = dist_info()
    from gpi_project_gb300 import workloads
    n_req = args.served_requests or 24
    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import oracle as O
        O.build()
        r = workloads.request_stream(1)[0]
        W = dict(name="c5", par=r["par"], mats=r["mats"], src=r["src"], rec=r["rec"], nshots=1)
        run_reference(args, W)
        return
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    with ClockSampler(local) as clk:
        leg = served_leg(n_req, local, passes=max(1, args.steps))
    # every replica serves the same stream: the job ends with the slowest
    # replica's makespan, and counts every replica's cell updates
    makespan = max_over_ranks(leg["makespan_s"])
    job_gcell = job_rate(leg["cell_updates"], world, makespan) / 1e9
    if rank != 0:
        return
    cps = makespan / leg["requests"]
    out = {
        "metric": "Gcell-updates/s", "value": round(job_gcell, 3), "unit": "Gcell-updates/s", "n_gpus": world,
        "steps": max(1, args.steps), "warmup": 1, "ms_per_step": round(1e3 * cps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded request stream; gpi_project_gb300/workloads.py request_stream)",
        "config": {"workload": "c5", "requests": n_req, "grid": leg["grid"],
                   "l2": "inputs larger than L2 (the stream holds ~0.5 GB of models)",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": round(job_gcell, 3), "unit": "Gcell-updates/s", "h2d_bytes_per_step": leg["h2d_bytes"],
                "d2h_bytes_per_step": leg["d2h_bytes"]},
        "roofline": {"kernel": "whole step of every resident solve", "bound": "hbm", **leg["hbm_roofline"],
                     "traffic": None},
        "gpu_launches": leg["gpu_launches"], "served": leg, "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        O.build()
        r = workloads.request_stream(1)[0]
        W = dict(name="c5", par=r["par"], mats=r["mats"], src=r["src"], rec=r["rec"], nshots=1)
        n = args.cpu_steps or auto_cpu_steps(W)
        v, sec = cpu_sample(W, n, cpu_threads())
        out["cpu_baseline"] = {"value": round(v, 4), "unit": "Gcell-updates/s", "cores": cpu_threads(),
                               "kind": "port", "sample": f"{n} time steps of the first request "
                                                         f"({r['par']['nx']}x{r['par']['ny']}, {sec:.1f} s)"}
    print(json.dumps(out), flush=True)


def main_fwi(args):
    """--workload fwi / fwi2: a step is one FWI gradient pass of one shot
    (forward run keeping every step's gradient quantities, or checkpoints when
    they do not fit, residuals against the observed data, backward run with
    the correlation) through the C ABI; value counts every run's cell updates
    (three runs for a checkpointed pass)."""
    rank, world, local = dist_info()
    from gpi_project_gb300 import workloads
    W = workloads.workload(args.workload)
    par = W["par"]
    if args.nt:
        par["nt"] = args.nt
    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps({"impl": "reference", "unavailable": "the FWI workload has no CPU reference arm here; "
                          "its cpu_baseline is the oracle's gradient pass"}))
        return
    import torch
    from gpi_project_gb300 import TimeLoop, host, make_config
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    nx, ny, nt = par["nx"], par["ny"], par["nt"]
    cfg = make_config(weq=2, nx=nx, ny=ny, fdorder=par["fdorder"], maxrelerror=par["maxrelerror"], dt=par["dt"],
                      dh=par["dh"], nt=nt, fw=par["fw"], abs_type=par["abs_type"], seismo=1, ndt=1, nshots=1,
                      shared_model=1)
    p = host_par(W)
    sig = host.wavelet(1, nt, par["dt"], W["src"])

    def context(mats):
        fields, vecs = host.prepare(p, mats)
        vecs.pop("_dt_max"), vecs.pop("_stable")
        t = TimeLoop(cfg, device=local)
        t.set_model(fields)
        t.set_vectors(vecs)
        t.set_sources(W["src"], sig)
        t.set_receivers(*W["rec"])
        return t

    tt = context(W["true_mats"])  # the observed data (not timed)
    tt.reset()
    tt.run()
    obs = [tt.section("vx"), tt.section("vy")]
    tt.close()
    t = context(W["mats"])
    model = [W["mats"][k].T.copy() for k in ("vp", "vs", "rho")]
    l2, ck = [0.0], [(0, 1)]

    def gradient_pass():
        t.fwi_begin(*model, velocity=1, adjoint_type=1)
        t.reset()
        t.run()
        rx, lx = host.fwi_residual(t.section("vx"), obs[0], 1, par["dt"])
        ry, ly = host.fwi_residual(t.section("vy"), obs[1], 1, par["dt"])
        t.fwi_backward(rx, ry)
        g = t.fwi_gradients()
        l2[0] = lx + ly
        ck[0] = t.fwi_checkpoints()
        return g

    for _ in range(max(1, args.warmup)):
        gradient_pass()
    torch.cuda.synchronize()
    launches0 = t.launch_count()
    with ClockSampler(local) as clk:
        w0 = time.perf_counter()
        for _ in range(args.steps):
            g = gradient_pass()
        torch.cuda.synchronize()
        sec = (time.perf_counter() - w0) / args.steps
    launches = t.launch_count() - launches0
    sec = max_over_ranks(sec)
    # algorithmic work: the forward and the backward run; a checkpointed pass
    # also recomputes the forward steps, counted apart (recomputed_gcell_per_s)
    updates = 2.0 * nx * ny * nt
    value = job_rate(updates, world, sec) / 1e9
    peak, peak_kind = measured_peaks()
    # algorithmic bytes per cell update: the EL_ISO step (60 B) plus, on a stored forward step, the five
    # gradient quantities written to the store once (20 B); backward, the density term (v, store 2 x 4 B,
    # sum read + written: 24 B) and the lambda / mu terms (store 3 x 4, stresses 12, model 4 x 4, two sums
    # read + written: 56 B); a checkpointed pass runs the forward steps twice (the first time storing
    # nothing) and counts the recompute as work. The velocity terms' trip through two scratch fields (16 B)
    # is not credited.
    bpc = (60 + 20 + 60 + 24 + 56) / 2.0
    with_recompute = None
    if ck[0][0]:
        with_recompute = job_rate(3.0 * nx * ny * nt, world, sec) / 1e9
        bpc = (60 + 60 + 20 + 60 + 24 + 56) / 2.0  # the recompute's bytes, per algorithmic cell update
    store_gb = 5.0 * nx * ny * nt * 4 / 1e9
    t.close()
    if rank != 0:
        return
    out = {
        "metric": "Gcell-updates/s", "value": round(value, 4), "unit": "Gcell-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(1, args.warmup), "ms_per_step": round(1e3 * sec, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": f"synthetic (seeded; gpi_project_gb300/workloads.py '{W['name']}', observed data from a perturbed model)",
        "config": {"workload": W["name"], "nx": nx, "ny": ny, "nt": nt, "weq": 2, "fdorder": par["fdorder"],
                   "fw": par["fw"], "velocity": 1, "adjoint_type": 1, "receivers": len(W["rec"][0]),
                   "forward_store_gb": round(store_gb, 2), "checkpoint_interval": ck[0][0],
                   "segments": ck[0][1],
                   "l2": "inputs larger than L2 (forward store %.1f GB)" % store_gb, "parallelism": f"replicas x{world}"},
        "e2e": {"value": round(value, 4), "unit": "Gcell-updates/s",
                "h2d_bytes_per_step": int(2 * len(W["rec"][0]) * nt * 4 + 3 * nx * ny * 4),
                "d2h_bytes_per_step": int(2 * len(W["rec"][0]) * nt * 4 + 3 * nx * ny * 4)},
        "step_roofline": {"bytes_per_cell": bpc, "achieved": round(bpc * value, 1),
                          "frac": round(bpc * value / peak, 4), "peak": peak, "peak_kind": peak_kind, "unit": "GB/s"},
        "gpu_launches": int(launches), "misfit_l2": l2[0], "clocks": clk.summary(),
        **({"recomputed_gcell_per_s": round(with_recompute, 4)} if with_recompute else {}),
    }
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        O.build()
        ocfg = O.SofiConfig()
        for k in ["weq", "nx", "ny", "dh", "dt", "fdorder", "maxrelerror", "fw", "abs_type", "npower", "k_max_cpml",
                  "vppml", "fpml", "seismo", "ndt"]:
            setattr(ocfg, k, par[k])
        # the oracle keeps every step's forward quantities in host memory: at most ~4 GB of them
        ns = args.cpu_steps or max(10, min(nt, auto_cpu_steps(W) // 2, int(4e9 / (20.0 * nx * ny))))
        ocfg.nt = ns
        o = O.Oracle(ocfg, "f32", cpu_threads())
        o.set_material({k: v.reshape(-1) for k, v in W["mats"].items()})
        o.set_sources(W["src"], O.wavelet(1, ns, ocfg.dt, W["src"]))
        o.set_receivers(*W["rec"])
        w0 = time.perf_counter()
        o.reset()
        o.fwi_begin(1, 1)
        o.run()
        cx, cy = o.section("vx"), o.section("vy")
        o.fwi_backward(*[np.ascontiguousarray(O.fwi_residual(c, c * 0.99, 1, ocfg.dt)[0]) for c in (cx, cy)])
        csec = time.perf_counter() - w0
        o.close()
        out["cpu_baseline"] = {"value": round(2.0 * nx * ny * ns / csec / 1e9, 4), "unit": "Gcell-updates/s",
                               "cores": cpu_threads(), "kind": "port",
                               "sample": f"the oracle's gradient pass with NT = {ns} on the same grid ({csec:.1f} s)"}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    rank, world, local = dist_info()
    if args.workload == "c5":
        return main_served(args)
    if args.workload in ("fwi", "fwi2"):
        return main_fwi(args)
    from gpi_project_gb300 import workloads
    W = workloads.workload(args.workload)
    if args.nt:
        W["par"]["nt"] = args.nt
    if args.impl == "reference":
        if world > 1 and rank != 0:
            return
        from oracle import oracle as O
        O.build()
        run_reference(args, W)
        return

    cpu_base = None
    if not args.no_cpu_baseline and rank == 0:
        cpu_base = cpu_leg(args, W["name"])

    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    par = W["par"]
    nshots = W["nshots"]
    t, fields, vecs, srcs, sigs = workloads.gpu_loop(W, device=local)

    # pinned host copies of every input, for the end-to-end leg
    def pinned(a):
        buf = torch.empty(a.shape, dtype=torch.float32, pin_memory=True)
        buf.numpy()[...] = a
        return buf

    pin_fields = {k: pinned(v) for k, v in fields.items()}
    h2d_bytes = sum(v.numel() * 4 for v in pin_fields.values())

    def upload_all():
        t.set_model({k: v.numpy() for k, v in pin_fields.items()})
        t.set_vectors(vecs)
        for s in range(nshots):
            t.set_sources(srcs[s % len(srcs)], sigs[s % len(sigs)], shot=s)
            t.set_receivers(*W["rec"], shot=s)

    stream = torch.cuda.ExternalStream(t.stream_handle())
    cells = par["nx"] * par["ny"] * par["nt"] * nshots

    def solve():
        t.reset()
        t.run(sync=False)

    for _ in range(args.warmup):
        solve()
    t.synchronize()

    # ---- device-timed region: inputs resident in HBM ----
    peak, peak_kind = measured_peaks()
    bpc = workloads.bytes_per_cell(par["weq"], par.get("L", 0), par.get("fdorder_time", 2))
    t.set_kernel_timing(33)  # graph chunks of 32 steps run between the timed direct steps
    launches0 = t.launch_count()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        with torch.cuda.stream(stream):
            ev0.record()
        for _ in range(args.steps):
            solve()
        with torch.cuda.stream(stream):
            ev1.record()
        t.synchronize()
        torch.cuda.synchronize()
    dev_ms = ev0.elapsed_time(ev1)
    launches = t.launch_count() - launches0
    ms_s, n_s = t.kernel_time("update_s")
    ms_v, n_v = t.kernel_time("update_v")
    t.set_kernel_timing(0)
    dev_ms = max_over_ranks(dev_ms)
    value = job_rate(cells * args.steps, world, dev_ms * 1e-3) / 1e9

    # ---- end to end through the C ABI: host buffers in, sections out ----
    ntr = len(W["rec"][0])
    d2h_bytes = 0
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    for _ in range(args.steps):
        upload_all()
        solve()
        comps = {1: ["vx", "vy"], 2: ["p"], 3: ["div", "curl"], 4: ["vx", "vy", "p", "div", "curl"]}[par["seismo"]]
        for s in range(nshots):
            for c in comps:
                sec = t.section(c, shot=s)
                d2h_bytes += sec.nbytes
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - w0)
    e2e_val = job_rate(cells * args.steps, world, e2e_s) / 1e9
    d2h_bytes //= max(args.steps, 1)

    # ---- roofline of the dominant kernel ----
    ncell = par["nx"] * par["ny"] * nshots
    ach_s = bpc["update_s"] * ncell / (ms_s * 1e-3) / 1e9 if ms_s else None
    traffic = traffic_from_profiles("update_s", W["name"])
    kname = {0: "k_update_s_ac (pressure)", 6: "k_tti_tiles (TTI stress)", 7: "k_tti_tiles (TTI stress + memory variables)"}
    if par.get("fdorder_time", 2) == 4:
        kname = {par["weq"]: "k_update_s_ab4w (Adams-Bashforth stress, histories, memory variables)"}
    roof = {"kernel": kname.get(par["weq"], "k_update_sw / k_update_s (stress + memory variables)"), "bound": "hbm",
            "achieved": round(ach_s, 1) if ach_s else None, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
            "frac": round(ach_s / peak, 4) if ach_s else None,
            "traffic": round(traffic * ncell) if traffic else None,
            "algorithmic_bytes_per_launch": bpc["update_s"] * ncell,
            "mean_launch_ms": round(ms_s, 4), "timed_launches": n_s}
    step_roof = {"bytes_per_cell": bpc["step"], "achieved": round(bpc["step"] * value / world, 1),
                 "frac": round(bpc["step"] * value / world / peak, 4), "unit": "GB/s",
                 "update_v_mean_ms": round(ms_v, 4), "update_s_mean_ms": round(ms_s, 4)}
    batched = None
    if nshots > 1:
        batched = plain_vs_batched(W, local, fields, vecs, srcs, dev_ms / args.steps)
        batched["shots_per_s"] = round(nshots * args.steps * world / (dev_ms * 1e-3), 3)
    if rank != 0:
        return
    out = {
        "metric": "Gcell-updates/s", "value": round(value, 4), "unit": "Gcell-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dev_ms / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded; gpi_project_gb300/workloads.py)",
        "config": config_of(W, world),
        "e2e": {"value": round(e2e_val, 4), "unit": "Gcell-updates/s", "h2d_bytes_per_step": int(h2d_bytes),
                "d2h_bytes_per_step": int(d2h_bytes)},
        "roofline": roof, "step_roofline": step_roof, "gpu_launches": int(launches),
        "autotune": {**dict(zip(["velocity_cells_per_thread", "velocity_rows_per_thread"], t.velocity_variant())),
                     "stress_cells_per_thread": t.stress_variant(),
                     **dict(zip(["velocity_block_threads_x", "stress_block_threads_x"], t.block_threads_x()))},
        **({"batched": batched} if batched else {}),
        "clocks": clk.summary(),
    }
    par_rec = parity_record(W["name"])
    if par_rec:
        out["parity"] = par_rec
    t.close()
    if args.served_requests > 0 and world == 1:
        with ClockSampler(local) as clk2:
            out["served"] = served_leg(args.served_requests, local)
        out["served"]["clocks"] = clk2.summary()
    if args.batched_leg and args.batched_leg != W["name"] and world == 1:
        with ClockSampler(local) as clk3:
            out["batched_" + args.batched_leg] = batched_leg(args.batched_leg, local)
        out["batched_" + args.batched_leg]["clocks"] = clk3.summary()
    if cpu_base:
        out["cpu_baseline"] = cpu_base
    print(json.dumps(out), flush=True)


def plain_vs_batched(W, device, fields, vecs, srcs, batched_ms):
    """Shots/s of W's batched solve (one launch per kernel per step covers
    every shot) against the same shots run one after another as plain
    single-shot solves on the same GPU (the first shot's solve, timed twice
    with CUDA events after one warm-up solve that also tunes)."""
    import torch
    from gpi_project_gb300 import workloads
    W1 = dict(W, nshots=1, src=srcs[0])
    t1, *_ = workloads.gpu_loop(W1, device=device, fields=fields, vecs=vecs)
    stream = torch.cuda.ExternalStream(t1.stream_handle())
    t1.reset()
    t1.run()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nplain = 2
    with torch.cuda.stream(stream):
        ev0.record()
    for _ in range(nplain):
        t1.reset()
        t1.run(sync=False)
    with torch.cuda.stream(stream):
        ev1.record()
    t1.synchronize()
    plain_ms = ev0.elapsed_time(ev1) / nplain
    t1.close()
    n = W["nshots"]
    return {"shots": n, "shots_per_s": round(n / (batched_ms * 1e-3), 3),
            "plain_shots_per_s": round(1.0 / (plain_ms * 1e-3), 3),
            "speedup_vs_plain": round(n * plain_ms / batched_ms, 3),
            "batched_ms_per_solve": round(batched_ms, 2), "plain_ms_per_shot": round(plain_ms, 2)}


def batched_leg(name: str, device: int, warmup: int = 1, steps: int = 1) -> dict:
    """Workload `name` (c4: 64 viscoelastic shots on 2000 x 1000, NT 4000) as a
    batched solve: Gcell-updates/s and shots/s with inputs resident, the HBM
    roofline of the whole step, and the gain over plain single-shot solves."""
    import torch
    from gpi_project_gb300 import workloads
    W = workloads.workload(name)
    par = W["par"]
    t, fields, vecs, srcs, _ = workloads.gpu_loop(W, device=device)
    stream = torch.cuda.ExternalStream(t.stream_handle())
    for _ in range(warmup):
        t.reset()
        t.run(sync=False)
    t.synchronize()
    launches0 = t.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        ev0.record()
    for _ in range(steps):
        t.reset()
        t.run(sync=False)
    with torch.cuda.stream(stream):
        ev1.record()
    t.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    launches = t.launch_count() - launches0
    variant = {"velocity_cells_per_thread": t.velocity_variant()[0], "stress_cells_per_thread": t.stress_variant(),
               "block_threads_x": list(t.block_threads_x())}
    t.close()
    cells = float(par["nx"]) * par["ny"] * par["nt"] * W["nshots"]
    value = cells / (ms * 1e-3) / 1e9
    bpc = workloads.bytes_per_cell(par["weq"], par.get("L", 0))["step"]
    peak, peak_kind = measured_peaks()
    out = {"config": config_of(W, 1), "gcell_per_s": round(value, 4), "steps": steps, "warmup": warmup,
           "step_roofline": {"bytes_per_cell": bpc, "achieved": round(bpc * value, 1),
                             "frac": round(bpc * value / peak, 4), "peak": peak, "peak_kind": peak_kind,
                             "unit": "GB/s"},
           "gpu_launches": int(launches), "autotune": variant}
    out.update(plain_vs_batched(W, device, fields, vecs, srcs, ms))
    return out


if __name__ == "__main__":
    main()
