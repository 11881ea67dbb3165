"""CPU-side checks of the C ABI: the library loads and exports every symbol
include/*.h declares; configuration errors are reported, not fatal."""
import ctypes
import glob
import os

import pytest

from gpi_project_gb300 import _native as N

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def built():
    from gpi_project_gb300 import build
    return build.build()


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(built["gpu"])
    names = N.declared_symbols(os.path.join(REPO, "include", "sofigpu.h"))
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n


def test_abi_version(built):
    assert N.load().sofi_abi_version() == 2  # 2: sofi_config gained fdorder_time
    import ctypes
    assert ctypes.sizeof(N.SofiConfig) == 24 * 4  # the C struct: 22 ints and 2 floats


def test_bad_config_reports_error_without_gpu(built):
    from gpi_project_gb300 import make_config
    lib = N.load()
    b = ctypes.c_longlong()
    cfg = make_config(weq=2, nx=100, ny=100, fdorder=7, dt=1e-4, dh=1.0, nt=10)
    assert lib.sofi_device_bytes(ctypes.byref(cfg), ctypes.byref(b)) == N.SOFI_E_ARG
    assert b"FDORDER" in lib.sofi_last_error()
    cfg = make_config(weq=3, nx=100, ny=100, fdorder=8, L=0, dt=1e-4, dh=1.0, nt=10)
    assert lib.sofi_device_bytes(ctypes.byref(cfg), ctypes.byref(b)) == N.SOFI_E_ARG
    cfg = make_config(weq=3, nx=4000, ny=2000, fdorder=8, L=3, dt=2e-4, dh=2.0, nt=6000, fw=30, abs_type=1,
                      free_surf=1)
    assert lib.sofi_device_bytes(ctypes.byref(cfg), ctypes.byref(b)) == 0
    # 14 state + 12 model fields of a padded 2016 x 4032 grid: ~0.85 GB
    assert 0.6e9 < b.value < 1.2e9


def test_create_without_device_fails_cleanly(built):
    from gpi_project_gb300 import SofiError, TimeLoop, make_config
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(SofiError):
        TimeLoop(make_config(weq=2, nx=64, ny=64, fdorder=4, dt=1e-4, dh=1.0, nt=10))
