"""The product's C host (libsofihost) against the oracle and the reference's files.

Model preparation must equal the oracle's (itself bit-identical to the
compiled reference) exactly: both evaluate the reference's float/double
expressions in the same order on the same libm.
"""
import os

import numpy as np
import pytest

from tests.golden.cases import CASES, WAVELET_CASES, WAVELET_DT, WAVELET_NT, synthetic_model, write_signal_file
from tests.helpers import case_config, prepared_model, rel_max, GOLDEN


@pytest.fixture(scope="module")
def H():
    from gpi_project_gb300 import build, host
    build.build()
    return host


def par_from_case(H, case, cfg):
    return H.make_par(weq=cfg.weq, nx=cfg.nx, ny=cfg.ny, dh=cfg.dh, dt=cfg.dt, nt=cfg.nt, fdorder=cfg.fdorder,
                      maxrelerror=cfg.maxrelerror, L=cfg.L, f_ref=cfg.f_ref, fl=cfg.fl, fw=cfg.fw,
                      abs_type=cfg.abs_type, free_surf=cfg.free_surf, boundary=cfg.boundary, npower=cfg.npower,
                      k_max_cpml=cfg.k_max_cpml, vppml=cfg.vppml, fpml=cfg.fpml, damping=cfg.damping,
                      fdorder_time=cfg.fdorder_time, readmod=cfg.readmod, tau=cfg.tau)


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_host_prepare_equals_oracle(H, case, oracle_mod):
    O = oracle_mod
    cfg = case_config(case)
    mats = synthetic_model(case)
    o = O.Oracle(cfg, "f32", 1)
    o.set_material(mats)
    ref_f, ref_v = prepared_model(o, cfg)
    got_f, got_v = H.prepare(par_from_case(H, case, cfg), mats if case.get("readmod", 1) else {}, nthreads=4)
    for k, a in ref_f.items():
        assert k in got_f, k
        np.testing.assert_array_equal(got_f[k], a, err_msg=f"{case['name']} {k}")
    for k, a in ref_v.items():
        np.testing.assert_array_equal(got_v[k], a, err_msg=f"{case['name']} {k}")
    o.close()


def test_host_wavelet_equals_oracle(H, oracle_mod):
    sp = np.zeros((12, 3), np.float32)
    sp[3] = [0.0, 0.01, 0.002]
    sp[4] = [25.0, 10.0, 40.0]
    sp[5] = [1.0, 2.0, 0.5]
    for shape in (1, 2, 4):
        np.testing.assert_array_equal(H.wavelet(shape, 500, 1e-4, sp), oracle_mod.wavelet(shape, 500, 1e-4, sp))


@pytest.mark.parametrize("wc", WAVELET_CASES, ids=[w["name"] for w in WAVELET_CASES])
def test_wavelets_equal_compiled_reference(H, oracle_mod, wc, tmp_path):
    """Every SOURCE_SHAPE: the source-file columns read by the host library,
    the signal file (SOURCE_SHAPE 3, ASCII and SU), and the signal of the
    host library and of the oracle equal the compiled reference's SIGOUT
    output bit for bit (tests/golden/ref_wavelets.npz, wavelet.c,
    read_srcsig.c, sources.c)."""
    ref = np.load(os.path.join(GOLDEN, "ref_wavelets.npz"))[f"{wc['name']}_signal"]
    src = tmp_path / "source.dat"
    src.write_text("# a comment line\n" + wc["line"] + "\n")
    p = H.make_par(weq=2, nx=40, ny=40, dh=2.0, dt=WAVELET_DT, nt=WAVELET_NT, source_shape=wc["shape"],
                   source_type=1)
    sp, xy = H.read_sources(p, str(src))
    assert sp.shape == (12, 1) and xy[0, 0] == 41.0
    sigfile = write_signal_file(wc, str(tmp_path)) if wc["shape"] == 3 else None
    got = H.wavelet(wc["shape"], WAVELET_NT, WAVELET_DT, sp, signal_file=sigfile)[0]
    np.testing.assert_array_equal(got, ref, err_msg=wc["name"])
    samples = oracle_mod.read_srcsig(sigfile, WAVELET_DT) if sigfile else None
    if sigfile:
        np.testing.assert_array_equal(H.read_signal(sigfile, WAVELET_DT), samples)
    orc = oracle_mod.wavelet(wc["shape"], WAVELET_NT, WAVELET_DT, sp, samples=samples)[0]
    np.testing.assert_array_equal(orc, ref, err_msg=wc["name"])


def test_wavelet_errors(H, tmp_path):
    """A Berlage exponent <= 0, an all-zero signal and a signal file whose DT
    differs are errors (wavelet.c:88-89,135-136, read_srcsig.c:172-175)."""
    sp = np.zeros((12, 1), np.float32)
    sp[4], sp[5], sp[8] = 30.0, 1.0, 0.0
    with pytest.raises(RuntimeError, match="exponent"):
        H.wavelet(5, 100, 1e-4, sp)
    sp[3] = 1.0  # sin^3 starting after the last step: all zero
    with pytest.raises(RuntimeError, match="zeros"):
        H.wavelet(4, 100, 1e-4, sp)
    f = tmp_path / "s.txt"
    f.write_text("# DT = 2.0e-04\n0.5\n1.0\n")
    with pytest.raises(RuntimeError, match="interval"):
        H.read_signal(str(f), 1e-4)


def test_builtin_model_takes_no_material_arrays(H):
    """READMOD = 0 selects the reference's built-in model: material arrays
    given with it are an error (a zeroed parameter struct would otherwise
    drop them silently), and acoustic media have no built-in model."""
    n = 30 * 80
    mats = {"vp": np.full(n, 3000.0, np.float32), "vs": np.full(n, 1700.0, np.float32),
            "rho": np.full(n, 2000.0, np.float32)}
    p = H.make_par(weq=2, nx=30, ny=80, dh=2.0, dt=1e-4, nt=10, fdorder=4, readmod=0)
    with pytest.raises(RuntimeError, match="READMOD"):
        H.prepare(p, mats)
    f, _ = H.prepare(p, {})
    # mu of the layer above 100 m and of the half space below
    assert f["pu"].min() == 1.0 and f["pu"].max() == np.float32(2000.0) * np.float32(2000.0) * np.float32(2000.0)
    with pytest.raises(RuntimeError, match="built-in"):
        H.prepare(H.make_par(weq=0, nx=30, ny=20, dh=2.0, dt=1e-4, nt=10, fdorder=4, readmod=0), {})


def test_host_holberg_table(H, oracle_mod):
    for fd in (2, 4, 6, 8, 10, 12):
        for me in range(5):
            cfg = oracle_mod.SofiConfig(weq=2, nx=40, ny=40, fdorder=fd, maxrelerror=me, nt=2)
            o = oracle_mod.Oracle(cfg)
            np.testing.assert_array_equal(H.holberg(fd, me), o.vector("hc", 7))
            o.close()


def test_parameter_file_and_acquisition(H, tmp_path):
    from tests.golden.cases import case_by_name, write_case
    from tests.helpers import case_receivers, case_sources
    case = case_by_name("el_mixed_sources")
    jpath, _ = write_case(case, str(tmp_path))
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        p = H.read_par(jpath)
        assert (p.nx, p.ny, p.fdorder, p.fw, p.abs_type, p.nt) == (case["nx"], case["ny"], 4, 10, 1, case["nt"])
        assert np.float32(p.dt) == np.float32(case["dt"]) and p.seismo == 4 and p.ndt == 2
        sp, xy = H.read_sources(p, "source.dat")
        cfg = case_config(case)
        np.testing.assert_array_equal(sp, case_sources(case, cfg))
        ix, iy = H.read_receivers(p, "receiver.dat")
        rx, ry = case_receivers(case, cfg)
        np.testing.assert_array_equal(ix, rx)
        np.testing.assert_array_equal(iy, ry)
    finally:
        os.chdir(cwd)


def test_su_writer_matches_reference_headers(H, tmp_path):
    """Trace headers as the reference writes them (compared with its own SU files)."""
    from tests.golden.cases import case_by_name
    from tests.helpers import case_receivers
    case = case_by_name("el_cpml_fd8")
    g = np.load(os.path.join(GOLDEN, f"ref_{case['name']}.npz"))
    cfg = case_config(case)
    p = par_from_case(H, case, cfg)
    p.ndt = case["ndt"]
    ix, iy = case_receivers(case, cfg)
    data = g["seis_vx"]
    out = str(tmp_path / "x.su")
    H.write_su(out, data, ix, iy, case["sources"][0][0], case["sources"][0][1], p, 1, 1)
    b = np.fromfile(out, np.uint8)
    rec = 240 + 4 * data.shape[1]
    hdr = b.reshape(-1, rec)[:, :240]
    np.testing.assert_array_equal(hdr, g["hdr_vx"])
    np.testing.assert_array_equal(b.reshape(-1, rec)[:, 240:].copy().view(np.float32), data)


def test_sigout_su_file_equals_reference(tmp_path):
    """SIGOUT = 1, SU: the wavelet file the reference ships for
    examples/weq3.json (Ricker 50 Hz, DT 1e-4, NT 2000, NDT 10), byte for byte.
    Its headers place the source at (200 m, 200 m), grid (101, 101), whereas
    the example's source file (and the seismograms shipped beside it) use
    (398 m, 398 m); the samples do not depend on the position, so the file is
    reproduced with the position it records."""
    from gpi_project_gb300 import host
    from tests.helpers import EXAMPLE_SOURCE
    dt = float(np.float32(1e-4))
    p = host.make_par(weq=2, nx=400, ny=400, dh=2.0, dt=dt, nt=2000, ndt=10, refrec=(0.0, 0.0), sigout=1,
                      sigout_format=1, sigout_file=str(tmp_path / "signal_out").encode())
    _, _, ts, fc, amp = EXAMPLE_SOURCE
    x = y = 200.0
    sp = np.zeros((12, 1), np.float32)
    sp[0, 0], sp[1, 0] = np.floor(np.float32(x) / np.float32(2.0)) + 1, np.floor(np.float32(y) / np.float32(2.0)) + 1
    sp[3, 0], sp[4, 0], sp[5, 0], sp[7, 0] = ts, fc, amp, 1
    sig = host.wavelet(1, 2000, dt, sp)[0]
    path = host.write_signal(p, 1, sig, int(sp[0, 0]), int(sp[1, 0]), x, y)
    assert path.endswith("signal_out.shot1.su")
    ref = np.load(os.path.join(GOLDEN, "shipped_sigout_weq3.npz"))["raw"]
    got = np.fromfile(path, dtype=np.uint8)
    assert got.size == ref.size
    np.testing.assert_array_equal(got, ref)


def test_sigout_ascii_and_binary(tmp_path):
    from gpi_project_gb300 import host
    sig = np.linspace(-1.0, 1.0, 37, dtype=np.float32) ** 3
    for fmt, ext in ((2, "txt"), (3, "bin")):
        p = host.make_par(weq=2, nx=10, ny=10, dh=1.0, dt=1e-3, nt=37, sigout=1, sigout_format=fmt,
                          sigout_file=str(tmp_path / "w").encode())
        path = host.write_signal(p, 3, sig, 5, 5, 4.0, 4.0)
        assert path.endswith(f"w.shot3.{ext}")
        back = np.loadtxt(path, dtype=np.float64) if fmt == 2 else np.fromfile(path, dtype=np.float32)
        np.testing.assert_allclose(back, sig, rtol=1e-6, atol=1e-30)
    p = host.make_par(weq=2, nx=10, ny=10, dh=1.0, dt=1e-3, nt=37, sigout=1, sigout_format=4,
                      sigout_file=str(tmp_path / "w").encode())
    with pytest.raises(RuntimeError, match="SIGOUT_FORMAT"):
        host.write_signal(p, 1, sig, 5, 5, 4.0, 4.0)


def test_su_model_files_read_like_binary(tmp_path):
    """MFILE.vp.su present: every model comes from MFILE.<suffix>.su, one trace
    per x column; extra traces and samples are ignored (readmod_elastic.c)."""
    from gpi_project_gb300 import host
    nx, ny = 23, 17
    rng = np.random.default_rng(5)
    mats = {k: rng.uniform(1.0, 3.0, (nx, ny)).astype(np.float32) for k in ("vp", "vs", "rho")}
    p = host.make_par(weq=2, nx=nx, ny=ny, dh=1.0, dt=1e-4, nt=10)
    for k, a in mats.items():
        a.tofile(tmp_path / f"bin.{k}")
        big = np.concatenate([a, rng.uniform(0, 1, (nx, 5)).astype(np.float32)], axis=1)  # ns = NY + 5
        big = np.concatenate([big, rng.uniform(0, 1, (3, ny + 5)).astype(np.float32)], axis=0)  # NX + 3 traces
        ix = np.arange(1, big.shape[0] + 1, dtype=np.int32)
        host.write_su(str(tmp_path / f"su.{k}.su"), big, ix, np.ones_like(ix), 0.0, 0.0, p)
    a = host.read_model(p, str(tmp_path / "bin"))
    b = host.read_model(p, str(tmp_path / "su"))
    for k in mats:
        np.testing.assert_array_equal(a[k], mats[k])
        np.testing.assert_array_equal(b[k], mats[k])
    short = host.make_par(weq=2, nx=nx, ny=ny + 6, dh=1.0, dt=1e-4, nt=10)
    with pytest.raises(RuntimeError, match="samples"):
        host.read_model(short, str(tmp_path / "su"))


def test_parameter_file_fdorder_time_and_fwi_keys(tmp_path):
    """FDORDER_TIME 4 is read (2 and 4 only, read_par_json.c); MODE = FWI and
    the keys of one gradient pass (read_par_json_fwi.c) are read."""
    from gpi_project_gb300 import host as H
    from tests.golden.cases import FWI_CASES, fwi_json_text
    base = '{\n"NX" : "10",\n"NY" : "12",\n"DH" : "1.0",\n"DT" : "1e-4",\n"TIME" : "0.01",\n"WEQ" : "VEL_ISO",\n'
    path = str(tmp_path / "p.json")
    with open(path, "w") as fh:
        fh.write(base + '"FDORDER_TIME" : "4"\n}\n')
    p = H.read_par(path)
    assert p.fdorder_time == 4 and p.mode_fwi == 0
    with open(path, "w") as fh:
        fh.write(base + '"FDORDER_TIME" : "3"\n}\n')
    with pytest.raises(RuntimeError):
        H.read_par(path)
    case = FWI_CASES[1]
    with open(path, "w") as fh:
        fh.write(fwi_json_text(case))
    p = H.read_par(path)
    assert (p.mode_fwi, p.fwi_velocity, p.fwi_adjoint, p.fwi_lnorm, p.fwi_dtinv) == (
        1, case["velocity"], case["adjoint_type"], 2, 1)
    assert p.data_dir.decode() == "./obs/seis" and p.gradient.decode() == "./grad/g"


@pytest.mark.parametrize("name", ["acq_topo", "acq_planes", "acq_line", "acq_vline"])
def test_acquisition_matches_compiled_reference(H, name, tmp_path, oracle_mod):
    """Receivers and sources as the compiled reference's receiver.c / sources.c
    place them: below the topography of the P-wave model (REC_TOPO,
    SOURCE_TOPO), with a co-located receiver of the file dropped and its trace
    number left out, with REFRECX, as receiver planes (REC_ARRAY) whose
    first row 0 becomes 1, and on the parameter file's line (combined
    "XREC1,YREC1" keys, NGEOPH). The oracle run on the host library's acquisition
    reproduces the reference's seismograms, and the SU file written with the
    host's receivers, trace numbers and source position carries the
    reference's trace headers byte for byte."""
    from tests.golden.cases import ACQ_CASES, write_case
    O = oracle_mod
    case = next(c for c in ACQ_CASES if c["name"] == name)
    g = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    write_case(case, str(tmp_path))
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        p = H.read_par("case.json")
        sp, xy = H.read_sources(p, p.source_file.decode())
        ix, iy, tr = H.read_receiver_traces(p, p.rec_file.decode())
        np.testing.assert_array_equal(H.read_receivers(p, p.rec_file.decode())[0], ix)
    finally:
        os.chdir(cwd)
    assert len(ix) == g["hdr_vx"].shape[0]
    cfg = case_config(case)
    o = O.Oracle(cfg, "f32", os.cpu_count() or 1)
    o.set_material(synthetic_model(case))
    o.set_sources(sp, H.wavelet(p.source_shape, cfg.nt, cfg.dt, sp))
    o.set_receivers(ix, iy)
    o.run()
    for comp in ("vx", "vy"):
        a, b = o.section(comp), g[f"seis_{comp}"]
        assert np.abs(b).max() > 0
        assert rel_max(a, b, floor=1e-30) < 1e-5, (name, comp, rel_max(a, b, floor=1e-30))
    out = str(tmp_path / "x.su")
    H.write_su(out, o.section("vx"), ix, iy, xy[0, 0], xy[1, 0], p, 1, 1, trace=tr)
    rec = 240 + 4 * g["seis_vx"].shape[1]
    np.testing.assert_array_equal(np.fromfile(out, np.uint8).reshape(-1, rec)[:, :240], g["hdr_vx"])
    o.close()


def test_topography_scan(H, tmp_path):
    """sofih_scan_topo: the first row whose P velocity differs from the top
    row's, per column, from the binary model and from the SU model."""
    from tests.golden.cases import ACQ_CASES, topo_rows, write_case
    case = ACQ_CASES[0]
    write_case(case, str(tmp_path))
    p = H.read_par(str(tmp_path / "case.json"))
    want = topo_rows(case) + 1
    np.testing.assert_array_equal(H.scan_topo(p, str(tmp_path / "model" / "m")), want)
    vp = np.fromfile(tmp_path / "model" / "m.vp", np.float32).reshape(case["nx"], case["ny"])
    H.write_su(str(tmp_path / "model" / "s.vp.su"), vp, np.arange(1, case["nx"] + 1), np.ones(case["nx"]), 0.0,
               0.0, p)
    np.testing.assert_array_equal(H.scan_topo(p, str(tmp_path / "model" / "s")), want)


def test_plane_wave_sources_match_reference_log(H, tmp_path):
    """SRCREC 2: one source per column at PLANE_WAVE_DEPTH + x tan(angle),
    no time shift, centre frequency 1 / TS, unit amplitude (sources.c:337-367).
    The compiled reference logs its source table (two decimals) before it
    crashes reading past its 8-row source matrix; the host's sources equal
    that table."""
    from tests.golden.cases import PLANE_WAVE_CASE, write_case
    g = np.load(os.path.join(GOLDEN, "ref_acq_plane_wave.npz"))["table"]
    write_case(PLANE_WAVE_CASE, str(tmp_path))
    p = H.read_par(str(tmp_path / "case.json"))
    assert p.srcrec == 2
    sp, xy = H.read_sources(p, "unused")
    assert sp.shape == (12, PLANE_WAVE_CASE["nx"])
    n = g.shape[0]
    np.testing.assert_allclose(xy[0, :n], g[:, 1], atol=0.006)
    np.testing.assert_allclose(xy[1, :n], g[:, 2], atol=0.006)
    for row, col in ((3, 3), (4, 4), (5, 5), (6, 6), (7, 7)):  # tshift, fc, amp, azimuth, type
        np.testing.assert_allclose(sp[row, :n], g[:, col], atol=0.006)
    dh = np.float32(p.dh)
    np.testing.assert_array_equal(sp[1], np.floor(xy[1] / dh) + 1)


@pytest.mark.parametrize("par,msg", [({"REC_TOPO": "1", "FREE_SURF": "1"}, "FREE_SURF"),
                                     ({"SOURCE_TOPO": "2"}, "SOURCE_TOPO"),
                                     ({"READREC": "0", "REC_ARRAY": "2"}, "DRX"),
                                     ({"SRCREC": "2", "PLANE_WAVE_DEPTH": "0.0"}, "PLANE_WAVE_DEPTH"),
                                     ({"SRCREC": "2", "PLANE_WAVE_DEPTH": "5.0", "SOURCE_SHAPE": "5"},
                                      "SOURCE_SHAPE")])
def test_acquisition_settings_the_reference_rejects(H, tmp_path, par, msg):
    """The combinations read_par_json.c / sources.c stop on are errors here too."""
    from tests.golden.cases import _case, write_case
    case = _case("bad", nx=40, ny=40, nt=10, fw=5, seismo=1, ndt=1, snap=0, seed=5, par=par)
    write_case(case, str(tmp_path))
    with pytest.raises(Exception, match=msg):
        H.read_par(str(tmp_path / "case.json"))


def test_snapshot_files_hold_every_snapshotting_shot(H, tmp_path, oracle_mod):
    """Several shots (RUN_MULTIPLE_SHOTS 1): the reference numbers snapshots
    across shots (time_loop.c:36), so the files hold the frames of every shot
    that initsrc.c lets write them, one shot after the other (shots 1 and 2 of
    3 with SNAPSHOT_START 2). The compiled reference's files equal the
    oracle's snapshots of those shots run alone, concatenated, and
    sofih_snapshot_shots names them; the rule's other cases follow
    initsrc.c:96 as written."""
    from tests.golden.cases import SNAP_SHOTS_CASE, write_case
    from tests.helpers import case_receivers, case_sources
    O = oracle_mod
    case = SNAP_SHOTS_CASE
    g = np.load(os.path.join(GOLDEN, f"ref_{case['name']}.npz"))
    write_case(case, str(tmp_path))
    p = H.read_par(str(tmp_path / "case.json"))
    shots = H.snapshot_shots(p, 3)
    assert shots == [1, 2]
    cfg = case_config(case)
    frames = {"vx": [], "vy": []}
    for s in shots:
        one = dict(case, sources=[case["sources"][s - 1]])
        o = O.Oracle(cfg, "f32", os.cpu_count() or 1)
        o.set_material(synthetic_model(case))
        sp = case_sources(one, cfg)
        o.set_sources(sp, O.wavelet(1, cfg.nt, cfg.dt, sp))
        o.set_receivers(*case_receivers(one, cfg))
        o.run()
        for c in frames:
            frames[c].append(o.snapshots(c).reshape(-1))
        o.close()
    for c, f in frames.items():
        a = np.concatenate(f)
        assert a.shape == g[f"snap_{c}"].shape
        assert rel_max(a, g[f"snap_{c}"], floor=1e-30) < 1e-5, c
    for start, incr, n, want in [(1, 1, 3, [1]), (3, 1, 2, [1, 2]), (3, 2, 3, [1, 3]), (2, 2, 3, [2]),
                                 (4, 2, 3, [2]), (2, 3, 1, [])]:
        p.snapshot_start, p.snapshot_incr = start, incr
        assert H.snapshot_shots(p, n) == want, (start, incr, n)
    p.snap = 0
    assert H.snapshot_shots(p, 3) == []


def test_seismogram_and_snapshot_formats_match_reference(H, tmp_path):
    """SEIS_FORMAT 2 / 3 and SNAP_FORMAT 2 / 3 (outseis_glob.c:85-97,
    writedsk.c:36-52): written from the same samples, the ASCII and float32
    files equal the compiled reference's byte for byte; the file-name
    extensions follow saveseis_glob.c:39-57, and SNAP_FORMAT 1 is refused as
    the reference refuses it."""
    from tests.golden.cases import FORMAT_CASE, write_case
    g = np.load(os.path.join(GOLDEN, "ref_fmt_out.npz"))
    write_case(FORMAT_CASE, str(tmp_path))
    p = H.read_par(str(tmp_path / "case.json"))
    ntr = len(FORMAT_CASE["receivers"])
    ix = iy = np.ones(ntr, np.int32)
    for comp in ("vx", "vy"):
        sec = g[f"seis3_{comp}"].view(np.float32).reshape(ntr, -1)
        for fmt in (2, 3):
            p.seis_format = fmt
            out = str(tmp_path / f"s{fmt}.{comp}")
            H.write_seis(out, sec, ix, iy, 0.0, 0.0, p)
            np.testing.assert_array_equal(np.fromfile(out, np.uint8), g[f"seis{fmt}_{comp}"], err_msg=f"{fmt} {comp}")
        frame = g[f"snap3_{comp}"].view(np.float32)
        for fmt in (2, 3):
            out = str(tmp_path / f"n{fmt}.{comp}")
            H.write_snap(out, frame[: frame.size // 2], False, fmt)
            H.write_snap(out, frame[frame.size // 2:], True, fmt)
            np.testing.assert_array_equal(np.fromfile(out, np.uint8), g[f"snap{fmt}_{comp}"], err_msg=f"{fmt} {comp}")
    assert [H.seis_ext(f) for f in range(7)] == ["sgy", "su", "txt", "bin", "sgy", "sgy", None]
    with pytest.raises(Exception, match="SU format"):
        H.write_snap(str(tmp_path / "x"), frame, False, 1)
    p.seis_format = 4
    H.write_seis(str(tmp_path / "e.sgy"), sec, ix, iy, 0.0, 0.0, p)
    assert os.path.getsize(tmp_path / "e.sgy") == 0
    p.seis_format = 1  # checkfd.c:119-122: SU traces hold at most 65535 samples
    with pytest.raises(Exception, match="65535"):
        H.write_seis(str(tmp_path / "long.su"), np.zeros((1, 65536), np.float32), ix[:1], iy[:1], 0.0, 0.0, p)
