"""Request-loop policy and library surface on the CPU (no GPU calls)."""
import os
import re
import subprocess

import numpy as np
import pytest

from gpi_project_gb300 import serve as S
from gpi_project_gb300 import workloads as W

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_header_declares_every_export():
    text = open(os.path.join(REPO, "include", "sofiserve.h")).read()
    declared = set(re.findall(r"\b(sofi_server_\w+)\s*\(", text))
    assert declared == set(S.DECLARED)
    lib = os.path.join(REPO, "gpi_project_gb300", "_build", "libsofiserve.so")
    syms = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    for name in S.DECLARED:
        assert re.search(rf"\bT {name}\b", syms), name


def test_plan_first_fit_in_arrival_order():
    gb = 1 << 30
    # 10 GB budget, 2 GB in use: 5 fits, 4 no longer fits, 1 and 2 still fit
    assert S.plan([5 * gb, 4 * gb, 1 * gb, 2 * gb], 2 * gb, 10 * gb, 0, 64) == [1, 0, 1, 1]
    # slot limit: one slot left
    assert S.plan([gb, gb, gb], 0, 100 * gb, 7, 8) == [1, 0, 0]
    # nothing fits an exhausted budget
    assert S.plan([1], 10, 10, 0, 8) == [0]
    assert S.plan([], 0, 10, 0, 8) == []


def test_priority_prefers_small_solves():
    least, greatest = 0, -5
    small = S.priority(256 * 256 * 1000, least, greatest)
    mid = S.priority(2048 * 1024 * 3000, least, greatest)
    big = S.priority(4096 * 2048 * 6000, least, greatest)
    assert small == greatest
    assert greatest <= small < mid <= big <= least
    assert S.priority(1e30, least, greatest) == least


def test_percentile_nearest_rank():
    x = np.arange(1, 101, dtype=np.float64)[::-1].copy()
    assert S.percentile(x, 0.5) == 50.0
    assert S.percentile(x, 0.99) == 99.0
    assert S.percentile(x, 1.0) == 100.0
    assert S.percentile([3.0], 0.99) == 3.0
    assert S.percentile([], 0.5) == 0.0


def test_create_without_device_reports_nodev():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError, match="error 6"):
        S.Server()


def test_request_stream_shapes_and_arrivals():
    rs = W.request_stream(12, rate=4.0)
    arr = [r["arrival"] for r in rs]
    assert arr == sorted(arr) and arr[0] > 0
    for r in rs:
        p = r["par"]
        assert 256 <= p["nx"] <= 4096 and 256 <= p["ny"] <= 2048 and p["nx"] * p["ny"] <= 4096 * 2048
        assert 1000 <= p["nt"] <= 6000 and p["fdorder"] in (4, 8) and p["weq"] in (2, 3)
        assert r["mats"]["vp"].shape == (p["nx"], p["ny"])
    # seeded: the same stream twice
    again = W.request_stream(12, rate=4.0)
    assert all(np.array_equal(a["mats"]["vp"], b["mats"]["vp"]) for a, b in zip(rs, again))
