"""The continuous-batching request loop on the GPU: every served solve equals
the same solve run alone, matches the oracle, and admission respects the HBM
budget and the slot count."""
import os

import numpy as np
import pytest

from gpi_project_gb300 import host as H
from gpi_project_gb300 import serve as S
from gpi_project_gb300 import timeloop as T
from gpi_project_gb300 import workloads as W
from tests.helpers import rel_l2, rel_max

pytestmark = pytest.mark.gpu

L2_TOL, MAX_TOL = 1e-4, 1e-3


def small_stream(n, seed, nt=(120, 260)):
    # uneven small grids, both orders, elastic and viscoelastic
    return W.request_stream(n, seed=seed, nt_range=nt, nx_range=(96, 320), ny_range=(96, 256))


def device_bytes(r):
    p = r["par"]
    cfg = T.make_config(weq=p["weq"], nx=p["nx"], ny=p["ny"], fdorder=p["fdorder"], maxrelerror=1, L=p["L"],
                        dt=p["dt"], dh=p["dh"], nt=p["nt"], fw=p["fw"], abs_type=1, seismo=1, ndt=1, nshots=1,
                        shared_model=1)
    return T.device_bytes(cfg)


def submit_all(srv, reqs, arrivals=None):
    ids = []
    for k, r in enumerate(reqs):
        a = -1.0 if arrivals is None else arrivals[k]
        ids.append(srv.submit(H.make_par(**r["par"]), r["mats"], r["src"], *r["rec"], arrival=a))
    return ids


def sections(srv, rid):
    return {c: srv.section(rid, c) for c in (1, 2)}


def test_each_request_same_alone_and_in_the_mix():
    """Bit-identical sections: a context's kernels touch only its own arrays,
    so sharing the GPU with other solves changes no arithmetic."""
    reqs = small_stream(6, seed=11)
    assert {r["par"]["weq"] for r in reqs} == {2, 3} and {r["par"]["fdorder"] for r in reqs} == {4, 8}
    alone = []
    with S.Server(max_resident=1) as srv:
        for r in reqs:
            (rid,) = submit_all(srv, [r])
            srv.drain()
            assert srv.info(rid)["state"] == S.REQ_DONE, srv.info(rid)["error"]
            alone.append(sections(srv, rid))
    with S.Server(max_resident=16, chunk_steps=32, depth=2) as srv:
        # staggered arrivals: later requests join while earlier ones run
        ids = submit_all(srv, reqs, arrivals=[0.002 * k for k in range(len(reqs))])
        srv.drain()
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["failed"] == 0
        assert st["peak_resident"] >= 2
        for k, rid in enumerate(ids):
            mixed = sections(srv, rid)
            for c in (1, 2):
                np.testing.assert_array_equal(mixed[c], alone[k][c], err_msg=f"request {k} comp {c}")
                assert np.abs(mixed[c]).max() > 0


def test_served_request_matches_oracle():
    from oracle import oracle as O
    reqs = small_stream(3, seed=3, nt=(200, 200))
    with S.Server() as srv:
        ids = submit_all(srv, reqs)
        srv.drain()
        for r, rid in zip(reqs, ids):
            assert srv.info(rid)["state"] == S.REQ_DONE, srv.info(rid)["error"]
            keys = {f for f in O.SofiConfig.__dataclass_fields__}
            cfg = O.SofiConfig(**{k: v for k, v in r["par"].items() if k in keys})
            o = O.Oracle(cfg, "f32", os.cpu_count() or 1)
            o.set_material(r["mats"])
            o.set_sources(r["src"], O.wavelet(1, cfg.nt, cfg.dt, r["src"]))
            o.set_receivers(*r["rec"])
            o.run()
            for c, name in ((1, "vx"), (2, "vy")):
                a, b = srv.section(rid, c), o.section(name)
                assert rel_l2(a, b) <= L2_TOL and rel_max(a, b) <= MAX_TOL, (rid, name, rel_l2(a, b))
            o.close()


def test_admission_by_budget_and_slots():
    reqs = small_stream(8, seed=3, nt=(150, 150))
    sizes = sorted(device_bytes(r) for r in reqs)
    budget = sizes[-1] + sizes[-2] + sizes[0] // 2  # never the three largest together
    with S.Server(hbm_budget=budget, max_resident=3) as srv:
        ids = submit_all(srv, reqs)
        srv.drain()
        st = srv.stats()
        assert st["completed"] == len(reqs)
        assert st["peak_bytes"] <= budget
        assert st["peak_resident"] <= 3
        for rid, r in zip(ids, reqs):
            i = srv.info(rid)
            assert i["device_bytes"] == device_bytes(r)
            assert i["arrival"] <= i["ready"] <= i["admitted"] <= i["finished"]


def test_request_larger_than_budget_fails_alone():
    reqs = small_stream(3, seed=8, nt=(100, 100))
    big = W.request_stream(1, seed=9, nt_range=(100, 100), nx_range=(1024, 1024), ny_range=(1024, 1024))[0]
    assert device_bytes(big) > 64 << 20 > sum(device_bytes(r) for r in reqs)
    with S.Server(hbm_budget=64 << 20) as srv:
        ids = submit_all(srv, reqs + [big])
        srv.drain()
        infos = [srv.info(i) for i in ids]
        assert [i["state"] for i in infos[:3]] == [S.REQ_DONE] * 3
        assert infos[3]["state"] == S.REQ_FAILED and "budget" in infos[3]["error"]
