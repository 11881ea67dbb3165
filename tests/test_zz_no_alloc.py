"""Allocation-free TTI stress update (sofi_tti_stress_noalloc) against sofi_run.

Some callers cannot allocate device memory once they are running -- a process
held to a fixed memory budget, or code inside a stream capture -- so the
library offers the TTI stress update on buffers the caller owns, with its
derivative scratch in a fixed array of the library. This test (collected
last, so a failure here leaves every other test already run) checks that two
calls in a row reproduce what a context's sofi_run computes for the same two
steps, within the GPU parity tolerance (relative L2 <= 1e-4, relative max <=
1e-3). The test itself allocates its buffers with torch; the entry point
does not allocate.
"""
import ctypes

import numpy as np
import pytest

from tests.golden.cases import case_by_name
from tests.helpers import case_config, gpu_config_from, prepared_model, rel_l2, rel_max

pytestmark = pytest.mark.gpu

L2_TOL, MAX_TOL = 1e-4, 1e-3


def _pad(torch, a, nx, ny, periodic=False):
    """[NY][NX] into the padded device layout; periodic: the 8 ghost columns on
    either side hold the opposite edge's columns (what exchange_v leaves)."""
    from gpi_project_gb300 import _native as N
    rows, pitch = N.padded_shape(nx, ny)
    t = torch.zeros((rows, pitch), dtype=torch.float32)
    a = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32))
    t[8:8 + ny, 8:8 + nx] = a
    if periodic:
        t[8:8 + ny, 0:8] = a[:, nx - 8:nx]
        t[8:8 + ny, 8 + nx:16 + nx] = a[:, 0:8]
    return t.cuda()


def _unpad(t, nx, ny):
    return t[8:8 + ny, 8:8 + nx].cpu().numpy()


CASES = [("tti_cpml", {}), ("vtti_cpml_l1", {}), ("tti_abs", {}), ("tti_cpml", {"boundary": 1})]


@pytest.mark.parametrize("name,over", CASES, ids=[n + "".join(f"-{k}{v}" for k, v in o.items()) for n, o in CASES])
def test_noalloc_tti_stress_matches_context(name, over):
    """CPML (elastic, viscoelastic), the damping frame, and periodic x with the
    caller filling the velocity ghost columns."""
    torch = pytest.importorskip("torch")
    from oracle import oracle as O
    from gpi_project_gb300 import TimeLoop, _native as N
    case = dict(case_by_name(name), **over)
    cfg = case_config(case)
    cfg.seismo, cfg.snap = 0, 0
    o = O.Oracle(cfg)
    from tests.golden.cases import synthetic_model
    o.set_material(synthetic_model(case))
    fields, vecs = prepared_model(o, cfg)
    gcfg = gpu_config_from(cfg, snap_override=0)
    t = TimeLoop(gcfg)
    t.set_model(fields)
    t.set_vectors(vecs)
    t.set_sources(np.zeros((12, 0), np.float32), np.zeros((0, cfg.nt), np.float32))
    t.reset()
    rng = np.random.default_rng(7)
    nx, ny = cfg.nx, cfg.ny
    init = {k: (rng.standard_normal((ny, nx)) * s).astype(np.float32)
            for k, s in [("vx", 1e-3), ("vy", 1e-3), ("sxx", 1e3), ("syy", 1e3), ("sxy", 1e3)]}
    for k, v in init.items():
        t.set_field(k, v)
    visco = cfg.weq == 7
    L = cfg.L

    # caller-owned device buffers in the library's padded layout
    dev = {k: _pad(torch, init[k], nx, ny) for k in ["sxx", "syy", "sxy"]}
    rows, pitch = N.padded_shape(nx, ny)
    if visco:
        for k in "rpq":
            dev[k] = torch.zeros((L, rows, pitch), dtype=torch.float32, device="cuda")
    fw2 = 2 * cfg.fw
    cpml, periodic = cfg.abs_type == 1, bool(cfg.boundary)
    if cfg.abs_type == 2:
        dev["absorb"] = _pad(torch, fields["absorb"], nx, ny)
    for k in ["psi_vxx", "psi_vyx"]:
        dev[k] = torch.zeros((ny, fw2), dtype=torch.float32, device="cuda")
    for k in ["psi_vyy", "psi_vxy"]:
        dev[k] = torch.zeros((fw2, nx), dtype=torch.float32, device="cuda")
    suffix = "u" if visco else ""
    mods = ["c11", "c13", "c33", "c15", "c35", "c55ipjp", "c15ipjp", "c35ipjp"]
    for m in mods:
        dev[m] = _pad(torch, fields[m + suffix], nx, ny)
        if visco:
            dev[m + "d_base"] = _pad(torch, fields[m + "d_base"], nx, ny)
    for k in ["K_x", "a_x", "b_x", "K_x_half", "a_x_half", "b_x_half", "K_y", "a_y", "b_y", "K_y_half",
              "a_y_half", "b_y_half"]:
        if cpml:
            dev[k] = torch.from_numpy(np.ascontiguousarray(vecs[k], dtype=np.float32)).cuda()

    args = N.TtiStressArgs()
    for k, v in dev.items():
        setattr(args, k, v.data_ptr())
    hc = o.vector("hc", 7)
    for k in range(7):
        args.hc[k] = float(hc[k])
    if visco:
        for l in range(L):
            args.bip[l], args.cip[l], args.peta[l] = float(vecs["bip"][l]), float(vecs["cip"][l]), float(
                vecs["peta"][l])
    lib = N.load()
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        t.run(1)  # velocity + stress update of one step through the context
        dev["vx"] = _pad(torch, t.field("vx"), nx, ny, periodic)
        dev["vy"] = _pad(torch, t.field("vy"), nx, ny, periodic)
        args.vx, args.vy = dev["vx"].data_ptr(), dev["vy"].data_ptr()
        torch.cuda.synchronize()
        N.check(lib.sofi_tti_stress_noalloc(ctypes.byref(gcfg), ctypes.byref(args), ctypes.c_void_p(stream)))
        torch.cuda.synchronize()
        for k in ["sxx", "syy", "sxy"]:
            got, ref = _unpad(dev[k], nx, ny), t.field(k)
            assert rel_l2(got, ref) <= L2_TOL and rel_max(got, ref) <= MAX_TOL, (name, over, call, k)
        if visco:
            for k in "rpq":
                for l in range(L):
                    got, ref = _unpad(dev[k][l], nx, ny), t.field(f"{k}{l + 1}")
                    assert rel_l2(got, ref, floor=1e-30) <= L2_TOL, (name, call, k, l)
    t.close()
    o.close()


def test_noalloc_rejects_oversized_grid():
    pytest.importorskip("torch")
    from gpi_project_gb300 import make_config, _native as N
    cfg = make_config(weq=6, nx=2048, ny=2048, fdorder=6, dt=1e-4, dh=1.0, nt=10, fw=10, abs_type=1)
    args = N.TtiStressArgs()
    rc = N.load().sofi_tti_stress_noalloc(ctypes.byref(cfg), ctypes.byref(args), None)
    assert rc == N.SOFI_E_ARG
    assert b"exceeds the fixed scratch" in N.load().sofi_last_error()
