"""Seeded synthetic forward-modelling workloads.

The reference publishes no benchmark suite; these stand in for the five
benchmark configurations with their shapes, sizes and value distributions:

  c1  isotropic elastic, 400 x 400, DH 1 m, DT 1e-4 s, NT 2000, FD8 Holberg,
      CPML 20; three layers (Vp 2000/2800/3500, rho 1800/2100/2400, Vs = Vp/1.73)
      with 2 % Gaussian perturbation; explosive Ricker 25 Hz at the top centre;
      100 receivers at 10 m depth recording vx, vy
  c2  viscoelastic, 4000 x 2000, DH 2 m, DT 2e-4 s, NT 6000, FD8, L = 3
      (5/15/50 Hz, F_REF 15 Hz), CPML 30, free surface; smooth random Vp
      1500-4500, Vs = Vp/1.8, Gardner density, smooth Q 20-100 (Qp = Qs);
      Ricker 15 Hz vertical force; 1000 receivers
  c3  TTI elastic, 2048 x 2048, DH 2.5 m, DT 2.0e-4 s, NT 4000, FD6, CPML 20;
      Vp 2000-4000, Vs = Vp/1.8, rho 2000-2600, eps 0-0.25, delta -0.1-0.15,
      tilt 0-45 deg, each field smoothed by a Gaussian of sigma 20 cells; explosive Ricker 20 Hz; 512 receivers
  c4  64 shots on the c1 layered model enlarged to 2000 x 1000 with c2's Q field
      and L = 3, NT 4000, explosive sources spread across the surface
  fdt4  c2's viscoelastic model and grid with 4th-order Adams-Bashforth time
      stepping (FDORDER_TIME 4): no free surface (the reference has none for
      it), DT 1e-4 s (the smaller stability region of the scheme), NT 6000
  ac  acoustic (AC_ISO) on c2's geometry: 4000 x 2000, DH 2 m, DT 2e-4 s, NT 6000,
      FD8, CPML 30; c2's smooth Vp field and Gardner density; explosive Ricker
      15 Hz; 1000 receivers recording pressure
Values are drawn from numpy's PCG64 with seed 1000 + config number.
"""
from __future__ import annotations

import math

import numpy as np


def smooth_field(rng, nx, ny, corr_cells, lo, hi, sigma=None):
    """Gaussian-correlated random field scaled to [lo, hi], shape [NX][NY].

    The white noise is convolved with a Gaussian of standard deviation
    ``sigma`` cells, or corr_cells / 2 pi cells when ``sigma`` is None.
    """
    w = rng.standard_normal((nx, ny))
    kx = np.fft.fftfreq(nx)[:, None]
    ky = np.fft.rfftfreq(ny)[None, :]
    s = corr_cells / (2.0 * math.pi) if sigma is None else float(sigma)
    g = np.exp(-0.5 * ((kx * 2 * math.pi * s) ** 2 + (ky * 2 * math.pi * s) ** 2))
    f = np.fft.irfft2(np.fft.rfft2(w) * g, s=(nx, ny))
    f = (f - f.min()) / max(f.max() - f.min(), 1e-30)
    return (lo + (hi - lo) * f).astype(np.float32)


def layered(rng, nx, ny):
    y = np.arange(ny)
    layer = np.where(y < ny // 3, 0, np.where(y < 2 * ny // 3, 1, 2))
    vp = np.array([2000.0, 2800.0, 3500.0])[layer][None, :] * (1.0 + 0.02 * rng.standard_normal((nx, ny)))
    rho = np.array([1800.0, 2100.0, 2400.0])[layer][None, :] * (1.0 + 0.02 * rng.standard_normal((nx, ny)))
    vp = vp.astype(np.float32)
    return vp, (vp / 1.73).astype(np.float32), rho.astype(np.float32)


def _srcpos(points, dh, fc, stype, tshift=0.0, amp=1.0):
    """srcpos [12][n] in grid indices (reference srcpos_loc layout)."""
    n = len(points)
    sp = np.zeros((12, n), np.float32)
    for k, (x, y) in enumerate(points):
        sp[0, k] = math.floor(np.float32(x) / np.float32(dh)) + 1
        sp[1, k] = math.floor(np.float32(y) / np.float32(dh)) + 1
        sp[3, k], sp[4, k], sp[5, k], sp[7, k] = tshift, fc, amp, stype
    return sp


def workload(name: str) -> dict:
    """Parameters (sofihost field names), material arrays, sources, receivers."""
    if name == "c1":
        rng = np.random.default_rng(1001)
        nx = ny = 400
        vp, vs, rho = layered(rng, nx, ny)
        par = dict(weq=2, nx=nx, ny=ny, dh=1.0, dt=1e-4, nt=2000, fdorder=8, maxrelerror=1, fw=20, abs_type=1,
                   npower=4.0, k_max_cpml=1.0, vppml=float(vp.max()), fpml=25.0, seismo=1, ndt=1)
        mats = dict(vp=vp, vs=vs, rho=rho)
        src = _srcpos([(200.0, 5.0)], 1.0, 25.0, 1)
        xs = np.linspace(21.0, 378.0, 100)
        rec = (np.floor(xs / 1.0).astype(np.int32) + 1, np.full(100, 11, np.int32))
        nshots = 1
    elif name == "c1b":
        # the 400 x 400 elastic solve above, 64 shots (sources along the top) batched on one model
        rng = np.random.default_rng(1001)
        nx = ny = 400
        vp, vs, rho = layered(rng, nx, ny)
        par = dict(weq=2, nx=nx, ny=ny, dh=1.0, dt=1e-4, nt=2000, fdorder=8, maxrelerror=1, fw=20, abs_type=1,
                   npower=4.0, k_max_cpml=1.0, vppml=float(vp.max()), fpml=25.0, seismo=1, ndt=1)
        mats = dict(vp=vp, vs=vs, rho=rho)
        src = [_srcpos([(x, 5.0)], 1.0, 25.0, 1) for x in np.linspace(30.0, 370.0, 64)]
        xs = np.linspace(21.0, 378.0, 100)
        rec = (np.floor(xs / 1.0).astype(np.int32) + 1, np.full(100, 11, np.int32))
        nshots = 64
    elif name == "fwi":
        # one FWI gradient pass (MODE = FWI, EL_ISO, VELOCITY 1, ADJOINT_TYPE 1) on the 400 x 400 grid above,
        # force-y source; the observed data come from `true_mats` (a 5 % faster, 3 % denser blob)
        rng = np.random.default_rng(1006)
        nx = ny = 400
        vp, vs, rho = layered(rng, nx, ny)
        par = dict(weq=2, nx=nx, ny=ny, dh=1.0, dt=1e-4, nt=2000, fdorder=8, maxrelerror=1, fw=20, abs_type=1,
                   npower=4.0, k_max_cpml=1.0, vppml=float(vp.max()), fpml=25.0, seismo=1, ndt=1)
        mats = dict(vp=vp, vs=vs, rho=rho)
        true = {k: v.copy() for k, v in mats.items()}
        for k, f in (("vp", 1.05), ("vs", 1.05), ("rho", 1.03)):
            true[k][160:240, 180:260] *= np.float32(f)
        src = _srcpos([(200.0, 5.0)], 1.0, 25.0, 3)
        xs = np.linspace(21.0, 378.0, 100)
        rec = (np.floor(xs / 1.0).astype(np.int32) + 1, np.full(100, 11, np.int32))
        nshots = 1
        return dict(name=name, par=dict(par, L=0), mats=mats, true_mats=true, src=src, rec=rec, nshots=nshots)
    elif name == "fwi2":
        # the gradient pass on a 4000 x 2000 EL_ISO grid, NT 4000: 640 GB of forward quantities, so the pass
        # checkpoints (about 63 states of the wavefield and CPML memory) and recomputes each segment once
        rng = np.random.default_rng(1007)
        nx, ny = 4000, 2000
        vp, vs, rho = layered(rng, nx, ny)
        par = dict(weq=2, nx=nx, ny=ny, dh=1.0, dt=1e-4, nt=4000, fdorder=8, maxrelerror=1, fw=30, abs_type=1,
                   npower=4.0, k_max_cpml=1.0, vppml=float(vp.max()), fpml=25.0, seismo=1, ndt=1)
        mats = dict(vp=vp, vs=vs, rho=rho)
        true = {k: v.copy() for k, v in mats.items()}
        for k, f in (("vp", 1.05), ("vs", 1.05), ("rho", 1.03)):
            true[k][1800:2200, 600:1000] *= np.float32(f)
        src = _srcpos([(2000.0, 5.0)], 1.0, 25.0, 3)
        xs = np.linspace(31.0, nx - 32.0, 1000)
        rec = (np.floor(xs).astype(np.int32) + 1, np.full(1000, 11, np.int32))
        return dict(name=name, par=dict(par, L=0), mats=mats, true_mats=true, src=src, rec=rec, nshots=1)
    elif name == "c2":
        rng = np.random.default_rng(1002)
        nx, ny = 4000, 2000
        vp = smooth_field(rng, nx, ny, 60, 1500.0, 4500.0)
        vs = (vp / 1.8).astype(np.float32)
        rho = (310.0 * vp.astype(np.float64) ** 0.25).astype(np.float32)
        q = smooth_field(rng, nx, ny, 60, 20.0, 100.0)
        par = dict(weq=3, nx=nx, ny=ny, dh=2.0, dt=2e-4, nt=6000, fdorder=8, maxrelerror=1, L=3, f_ref=15.0,
                   fl=[5.0, 15.0, 50.0], fw=30, abs_type=1, free_surf=1, npower=4.0, k_max_cpml=1.0,
                   vppml=4500.0, fpml=15.0, seismo=1, ndt=1)
        mats = dict(vp=vp, vs=vs, rho=rho, qp=q, qs=q)
        src = _srcpos([(4000.0, 10.0)], 2.0, 15.0, 3)
        xs = np.linspace(31 * 2.0, (nx - 32) * 2.0, 1000)
        rec = (np.floor(xs / 2.0).astype(np.int32) + 1, np.full(1000, 6, np.int32))
        nshots = 1
    elif name == "c3":
        rng = np.random.default_rng(1003)
        nx = ny = 2048
        # every field is white noise smoothed by a Gaussian of sigma 20 cells
        vp = smooth_field(rng, nx, ny, 0, 2000.0, 4000.0, sigma=20)
        vs = (vp / 1.8).astype(np.float32)
        rho = smooth_field(rng, nx, ny, 0, 2000.0, 2600.0, sigma=20)
        mats = dict(vp=vp, vs=vs, rho=rho, epsilon=smooth_field(rng, nx, ny, 0, 0.0, 0.25, sigma=20),
                    delta=smooth_field(rng, nx, ny, 0, -0.1, 0.15, sigma=20),
                    theta=smooth_field(rng, nx, ny, 0, 0.0, 45.0, sigma=20))
        par = dict(weq=6, nx=nx, ny=ny, dh=2.5, dt=2.0e-4, nt=4000, fdorder=6, maxrelerror=1, fw=20, abs_type=1,
                   npower=4.0, k_max_cpml=1.0, vppml=5000.0, fpml=20.0, seismo=1, ndt=1)
        src = _srcpos([(2560.0, 30.0)], 2.5, 20.0, 1)
        xs = np.linspace(21 * 2.5, (nx - 22) * 2.5, 512)
        rec = (np.floor(xs / 2.5).astype(np.int32) + 1, np.full(512, 25, np.int32))
        nshots = 1
    elif name == "fdt4":
        W = workload("c2")
        W["name"] = "fdt4"
        W["par"].update(free_surf=0, dt=1e-4, fdorder_time=4)
        W["src"] = _srcpos([(4000.0, 100.0)], 2.0, 15.0, 3)
        W["rec"] = (W["rec"][0], np.full(1000, 40, np.int32))
        return W
    elif name == "ac":
        rng = np.random.default_rng(1002)
        nx, ny = 4000, 2000
        vp = smooth_field(rng, nx, ny, 60, 1500.0, 4500.0)
        rho = (310.0 * vp.astype(np.float64) ** 0.25).astype(np.float32)
        par = dict(weq=0, nx=nx, ny=ny, dh=2.0, dt=2e-4, nt=6000, fdorder=8, maxrelerror=1, fw=30, abs_type=1,
                   npower=4.0, k_max_cpml=1.0, vppml=4500.0, fpml=15.0, seismo=2, ndt=1)
        mats = dict(vp=vp, rho=rho)
        src = _srcpos([(4000.0, 100.0)], 2.0, 15.0, 1)
        xs = np.linspace(31 * 2.0, (nx - 32) * 2.0, 1000)
        rec = (np.floor(xs / 2.0).astype(np.int32) + 1, np.full(1000, 40, np.int32))
        nshots = 1
    elif name == "c4":
        rng = np.random.default_rng(1004)
        nx, ny = 2000, 1000
        vp, vs, rho = layered(rng, nx, ny)
        q = smooth_field(rng, nx, ny, 30, 20.0, 100.0)
        par = dict(weq=3, nx=nx, ny=ny, dh=1.0, dt=1e-4, nt=4000, fdorder=8, maxrelerror=1, L=3, f_ref=15.0,
                   fl=[5.0, 15.0, 50.0], fw=20, abs_type=1, npower=4.0, k_max_cpml=1.0, vppml=3600.0,
                   fpml=25.0, seismo=1, ndt=1)
        mats = dict(vp=vp, vs=vs, rho=rho, qp=q, qs=q)
        xsrc = np.linspace(30.0, nx - 31.0, 64)
        src = [_srcpos([(x, 5.0)], 1.0, 25.0, 1) for x in xsrc]
        xs = np.linspace(21.0, nx - 22.0, 200)
        rec = (np.floor(xs).astype(np.int32) + 1, np.full(200, 11, np.int32))
        nshots = 64
    else:
        raise KeyError(name)
    par.setdefault("L", 0)
    return dict(name=name, par=par, mats=mats, src=src, rec=rec, nshots=nshots)


def gpu_loop(W: dict, device: int = 0, fields=None, vecs=None):
    """A TimeLoop holding workload W through the product path.

    The model is prepared on the host by libsofihost (``sofih_prepare``, the
    reference's prepmod / av_* / prepare_update_s_* / PML_pro set-up), the
    wavelets by ``sofih_wavelet``; every shot gets its source and the common
    receiver line. Variants are left to the autotuner. Returns the loop, the
    prepared fields and vectors (for re-upload) and the per-shot sources and
    signals."""
    from . import host
    from .timeloop import TimeLoop, make_config
    par = W["par"]
    if fields is None:
        fields, vecs = host.prepare(host.make_par(**par), W["mats"])
    vecs = dict(vecs)
    dt_max = float(vecs.pop("_dt_max", [0.0])[0])
    if not int(vecs.pop("_stable", [1])[0]):
        raise ValueError(f"workload {W['name']} violates the stability bound (DT_max {dt_max})")
    nshots = W["nshots"]
    cfg = make_config(weq=par["weq"], nx=par["nx"], ny=par["ny"], fdorder=par["fdorder"],
                      fdorder_time=par.get("fdorder_time", 2), maxrelerror=par["maxrelerror"], L=par.get("L", 0),
                      dt=par["dt"], dh=par["dh"], nt=par["nt"], fw=par["fw"], abs_type=par["abs_type"],
                      free_surf=par.get("free_surf", 0), seismo=par["seismo"], ndt=par["ndt"], nshots=nshots,
                      shared_model=1)
    t = TimeLoop(cfg, device=device)
    srcs = W["src"] if isinstance(W["src"], list) else [W["src"]]
    sigs = [host.wavelet(1, par["nt"], par["dt"], s) for s in srcs]
    t.set_model(fields)
    t.set_vectors(vecs)
    for s in range(nshots):
        t.set_sources(srcs[s % len(srcs)], sigs[s % len(sigs)], shot=s)
        t.set_receivers(*W["rec"], shot=s)
    return t, fields, vecs, srcs, sigs


# Algorithmic bytes per cell-update (each evolving state array read and written
# once, each per-cell coefficient array read once; CPML frame memory, sources
# and receivers not credited).
def bytes_per_cell(weq: int, L: int, fdorder_time: int = 2) -> dict:
    """Per-kernel and whole-step algorithmic bytes of one cell-update.

    FDORDER_TIME 4 (EL_ISO / VEL_ISO): each history (svx, svy; vxx, vyy, vxy,
    vyx) reads three levels and writes one (16 B), each memory variable reads
    four levels and writes one (20 B)."""
    if fdorder_time == 4:
        v = 36 + 2 * 16
        s = 8 + 24 + 4 * 16 + (12 + 60 * L + 12 if weq == 3 else 12)
        return {"update_v": v, "update_s": s, "step": 40 + 2 * 16 + 4 * 16 + 60 * L + (32 if weq == 3 else 20)}
    if weq == 0:  # acoustic: vx, vy, p; rip, rjp, g
        return {"update_v": 28, "update_s": 20, "step": 36}
    if weq == 2:
        return {"update_v": 36, "update_s": 44, "step": 60}
    if weq == 3:
        return {"update_v": 36, "update_s": 8 + 24 + 24 * L + 24, "step": 8 * (5 + 3 * L) + 4 * 8}
    if weq == 4:
        return {"update_v": 36, "update_s": 8 + 24 + 16, "step": 64}
    if weq == 6:
        return {"update_v": 36, "update_s": 8 + 24 + 32, "step": 80}
    if weq == 5:
        return {"update_v": 36, "update_s": 8 + 24 + 24 * L + 32, "step": 8 * (5 + 3 * L) + 4 * 10}
    return {"update_v": 36, "update_s": 8 + 24 + 24 * L + 64, "step": 8 * (5 + 3 * L) + 4 * 18}


def request_stream(n: int, seed: int = 1005, rate: float | None = None, max_cells: int = 4096 * 2048,
                   nt_range=(1000, 6000), nx_range=(256, 4096), ny_range=(256, 2048)) -> list[dict]:
    """c5: a seeded stream of independent forward-modelling requests.

    Grid sizes log-uniform from 256 x 256 to 4096 x 2048 (NX and NY drawn
    separately, multiples of 16, capped at ``max_cells``), NT uniform in
    ``nt_range``, FDORDER 4 or 8, elastic or viscoelastic (L = 3, Q 20-100 per
    layer), three layers with 2 % perturbation, Ricker 10-40 Hz explosive
    source 5 cells below the CPML frame and up to 128 receivers on that row.
    DT is half the stability bound of the Holberg stencil for the largest
    velocity. Arrival offsets are Poisson with ``rate`` per second, or all 0.
    The ranges can be narrowed (tests use small grids and few steps).
    """
    from . import host as H

    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    for k in range(n):
        nx = int(round(2.0 ** rng.uniform(math.log2(nx_range[0]), math.log2(nx_range[1])) / 16)) * 16
        ny = int(round(2.0 ** rng.uniform(math.log2(ny_range[0]), math.log2(ny_range[1])) / 16)) * 16
        while nx * ny > max_cells:
            nx, ny = nx // 2, ny
        nt = int(rng.integers(nt_range[0], nt_range[1] + 1))
        fd = int(rng.choice([4, 8]))
        visco = bool(rng.integers(0, 2))
        fc = float(rng.uniform(10.0, 40.0))
        dh = 2.0
        vlay = np.sort(rng.uniform(1500.0, 4500.0, 3))
        b1, b2 = sorted(rng.integers(ny // 5, 4 * ny // 5, 2).tolist())
        y = np.arange(ny)
        layer = np.where(y < b1, 0, np.where(y < b2, 1, 2))
        vp = (vlay[layer][None, :] * (1.0 + 0.02 * rng.standard_normal((nx, ny)))).astype(np.float32)
        vs = (vp / 1.73).astype(np.float32)
        rho = (310.0 * vp.astype(np.float64) ** 0.25).astype(np.float32)
        mats = dict(vp=vp, vs=vs, rho=rho)
        fw = 20
        hc = H.holberg(fd, 1)
        vmax = float(vp.max()) * (1.1 if visco else 1.0)  # unrelaxed velocities exceed vp
        dt = float(np.float32(0.5 * dh / (math.sqrt(2.0) * float(np.abs(hc).sum()) * vmax)))
        par = dict(weq=3 if visco else 2, nx=nx, ny=ny, dh=dh, dt=dt, nt=nt, time=nt * dt, fdorder=fd,
                   maxrelerror=1, fw=fw, abs_type=1, npower=4.0, k_max_cpml=1.0, vppml=float(vp.max()), fpml=fc,
                   source_shape=1, seismo=1, ndt=1, L=0)
        if visco:
            q = np.array(rng.uniform(20.0, 100.0, 3))[layer][None, :].repeat(nx, 0).astype(np.float32)
            mats.update(qp=q, qs=q)
            par.update(L=3, f_ref=fc, fl=[fc / 3.0, fc, 3.0 * fc])
        src = _srcpos([((nx // 2) * dh, (fw + 5) * dh)], dh, fc, 1)
        ntr = max(1, min(128, nx - 2 * fw))
        rix = np.linspace(fw + 1, nx - fw, ntr).astype(np.int32)
        riy = np.full(ntr, fw + 6, np.int32)
        if rate:
            t += float(rng.exponential(1.0 / rate))
        out.append(dict(par=par, mats=mats, src=src, rec=(rix, riy), arrival=t if rate else 0.0,
                        cells=nx * ny, cell_updates=float(nx) * ny * nt))
    return out
