"""Python face of the GPU time loop (reference src/time_loop.c:27-326).

``TimeLoop`` drives one libsofigpu context: the GlobVar settings of the loop
(``SofiConfig``), the prepared MemModel arrays, the shot's sources and
receivers, then ``run()`` and the outputs (sections, snapshots, wavefield).
Argument meaning follows the reference; errors raise ``SofiError``
(``UnstableError`` where the reference stops with "Simulation is unstable!").
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N

WEQ = {"AC_ISO": 0, "EL_ISO": 2, "VEL_ISO": 3, "EL_VTI": 4, "VEL_VTI": 5, "EL_TTI": 6, "VEL_TTI": 7}
COMP = {"vx": 1, "vy": 2, "p": 3, "div": 4, "curl": 5}


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _fp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def make_config(**kw) -> N.SofiConfig:
    c = N.SofiConfig()
    defaults = dict(weq=2, fdorder=4, maxrelerror=0, L=0, fw=0, abs_type=0, free_surf=0, boundary=0, seismo=0,
                    ndt=1, snap=0, snap_first=0, snap_inc=0, snap_last=0, idx=1, idy=1, nshots=1, shared_model=1,
                    fdorder_time=2)
    defaults.update(kw)
    for k, v in defaults.items():
        if isinstance(v, str) and k == "weq":
            v = WEQ[v]
        setattr(c, k, v)
    return c


class TimeLoop:
    def __init__(self, cfg: N.SofiConfig, device: int = 0):
        self.lib = N.load()
        self.cfg = cfg
        h = ctypes.c_void_p()
        N.check(self.lib.sofi_create(ctypes.byref(cfg), device, ctypes.byref(h)))
        self.h = h
        self.ntr = [0] * cfg.nshots

    # -------------------------------------------------------------- set-up
    def set_hc(self, hc):
        a = _f32(hc)
        N.check(self.lib.sofi_set_hc(self.h, _fp(a)))

    def set_model(self, fields: dict, model: int = 0):
        """Prepared model arrays, each [NY][NX] (row j-1, column i-1)."""
        for name, arr in fields.items():
            a = _f32(arr)
            assert a.shape == (self.cfg.ny, self.cfg.nx), (name, a.shape)
            N.check(self.lib.sofi_set_model_field(self.h, model, name.encode(), _fp(a), self.cfg.nx, 1))

    def set_vectors(self, vectors: dict):
        for name, v in vectors.items():
            a = _f32(v).reshape(-1)
            N.check(self.lib.sofi_set_model_vector(self.h, name.encode(), _fp(a), a.size))

    def set_sources(self, srcpos, signals, shot: int = 0):
        sp = _f32(srcpos)
        sig = _f32(signals)
        n = sp.shape[1] if sp.ndim == 2 else 0
        assert sp.shape[0] == 12 and sig.shape == (n, self.cfg.nt)
        N.check(self.lib.sofi_set_sources(self.h, shot, n, _fp(sp), _fp(sig)))

    def set_receivers(self, ix, iy, shot: int = 0):
        ix = np.ascontiguousarray(ix, dtype=np.int32)
        iy = np.ascontiguousarray(iy, dtype=np.int32)
        N.check(self.lib.sofi_set_receivers(self.h, shot, ix.size, _ip(ix), _ip(iy)))
        self.ntr[shot] = ix.size

    # ------------------------------------------------------------- stepping
    def reset(self, shot: int = -1):
        N.check(self.lib.sofi_reset(self.h, shot))

    def run(self, nsteps: int | None = None, sync: bool = True):
        step = ctypes.c_int()
        N.check(self.lib.sofi_current_step(self.h, ctypes.byref(step)))
        n = self.cfg.nt - step.value if nsteps is None else nsteps
        N.check(self.lib.sofi_run(self.h, n))
        if sync:
            self.synchronize()

    def synchronize(self):
        N.check(self.lib.sofi_synchronize(self.h))

    def last_run_ms(self) -> float:
        ms = ctypes.c_float()
        N.check(self.lib.sofi_last_run_ms(self.h, ctypes.byref(ms)))
        return ms.value

    def set_kernel_timing(self, every: int):
        N.check(self.lib.sofi_set_kernel_timing(self.h, every))

    def kernel_time(self, name: str):
        ms, n = ctypes.c_double(), ctypes.c_longlong()
        N.check(self.lib.sofi_kernel_time(self.h, name.encode(), ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def stream_handle(self) -> int:
        s = ctypes.c_void_p()
        N.check(self.lib.sofi_get_stream(self.h, ctypes.byref(s)))
        return s.value or 0

    def velocity_variant(self) -> tuple:
        """(cells per thread in x, rows per thread) of the velocity kernel."""
        a, b = ctypes.c_int(), ctypes.c_int()
        N.check(self.lib.sofi_velocity_variant(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    # ---- FWI gradient pass (EL_ISO, one shot)
    def fwi_begin(self, vp, vs, rho, velocity: int = 1, adjoint_type: int = 1):
        """vp / vs / rho as [NY][NX]; the next reset + run is the forward run."""
        m = [_f32(a).reshape(self.cfg.ny, self.cfg.nx) for a in (vp, vs, rho)]
        self._fwi_model = m
        N.check(self.lib.sofi_fwi_begin(self.h, velocity, adjoint_type, *[_fp(a) for a in m]))

    def fwi_backward(self, adj_x, adj_y):
        ax, ay = _f32(adj_x), _f32(adj_y)
        assert ax.shape == ay.shape == (self.ntr[0], self.cfg.nt)
        N.check(self.lib.sofi_fwi_backward(self.h, _fp(ax), _fp(ay)))

    def fwi_checkpoints(self) -> tuple:
        """(interval K, segments) of the pass's checkpoints (K = 0: whole store)."""
        a, b = ctypes.c_int(), ctypes.c_int()
        N.check(self.lib.sofi_fwi_checkpoints(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def fwi_gradients(self) -> tuple:
        """(gradLam_shot, gradMu_shot, gradRhos_shot), [NY][NX] float32."""
        out = [np.empty((self.cfg.ny, self.cfg.nx), dtype=np.float32) for _ in range(3)]
        N.check(self.lib.sofi_fwi_gradients(self.h, *[_fp(a) for a in out]))
        return tuple(out)

    def pdl(self) -> bool:
        """Whether the step kernels use programmatic dependent launch."""
        a = ctypes.c_int()
        N.check(self.lib.sofi_pdl(self.h, ctypes.byref(a)))
        return bool(a.value)

    def set_pdl(self, on: bool) -> None:
        N.check(self.lib.sofi_set_pdl(self.h, int(bool(on))))

    def post_fused(self) -> bool:
        """Whether the stress kernel also does the post-stress kernel's work
        (sources, seismograms, NaN probe) on the current settings."""
        n = ctypes.c_int()
        N.check(self.lib.sofi_post_fused(self.h, ctypes.byref(n)))
        return bool(n.value)

    def block_threads_x(self) -> tuple:
        """Threads per block along x of the four-cell (velocity, stress) kernels: 32, or 8 for narrow blocks."""
        a, b = ctypes.c_int(), ctypes.c_int()
        N.check(self.lib.sofi_block_threads_x(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def stress_variant(self) -> int:
        """Cells per thread in x of the stress kernel."""
        a = ctypes.c_int()
        N.check(self.lib.sofi_stress_variant(self.h, ctypes.byref(a)))
        return a.value

    def launch_count(self) -> int:
        n = ctypes.c_longlong()
        N.check(self.lib.sofi_launch_count(self.h, ctypes.byref(n)))
        return n.value

    # -------------------------------------------------------------- outputs
    def section(self, comp, shot: int = 0) -> np.ndarray:
        ns = ctypes.c_int()
        N.check(self.lib.sofi_num_samples(self.h, ctypes.byref(ns)))
        out = np.zeros((self.ntr[shot], ns.value), dtype=np.float32)
        N.check(self.lib.sofi_get_section(self.h, shot, COMP.get(comp, comp), _fp(out)))
        return out

    def field(self, name: str, shot: int = 0) -> np.ndarray:
        out = np.empty((self.cfg.ny, self.cfg.nx), dtype=np.float32)
        N.check(self.lib.sofi_get_field(self.h, shot, name.encode(), _fp(out)))
        return out

    def set_field(self, name: str, a, shot: int = 0):
        a = _f32(a)
        N.check(self.lib.sofi_set_field(self.h, shot, name.encode(), _fp(a)))

    def snapshots(self, comp, shot: int = 0) -> np.ndarray:
        n, sz = ctypes.c_int(), ctypes.c_int()
        N.check(self.lib.sofi_num_snapshots(self.h, ctypes.byref(n), ctypes.byref(sz)))
        out = np.empty((n.value, sz.value), dtype=np.float32)
        for k in range(n.value):
            N.check(self.lib.sofi_get_snapshot(self.h, shot, k, COMP.get(comp, comp), _fp(out[k])))
        return out

    def close(self):
        if getattr(self, "h", None):
            self.lib.sofi_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def device_bytes(cfg: N.SofiConfig) -> int:
    b = ctypes.c_longlong()
    N.check(N.load().sofi_device_bytes(ctypes.byref(cfg), ctypes.byref(b)))
    return b.value
