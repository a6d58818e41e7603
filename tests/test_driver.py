"""gpat_run, the C++ replay driver: it drives the C ABI in the order of
solve_transport_equation (stochastic-mhd.f90:312-567) from the reference's
on-disk inputs (conf.dat, mhd_config.dat, mhd_data_XXXX) and writes quick.dat
and fdists_XXXX.dat.  On a GPU its f(p) must equal the same sequence driven
from Python, bit for bit (FP64 path)."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from gpat import build, configs, fields
from gpat.engine import Engine, make_mhd_config, make_params, read_particle_dump

SEED = 0x1234567


def _dataset(tmp_path: Path):
    w = configs.planar_shock(scale=0.02, t_end=0.3, dt_out=0.1, dt_min=1e-3)
    data = tmp_path / "data"
    data.mkdir()
    (tmp_path / "config").mkdir()
    out = tmp_path / "out"
    out.mkdir()
    fields.write_mhd_config(data / "mhd_config.dat", w.mhd_config)
    for t in range(4):
        fields.write_mhd_data(data / f"mhd_data_{t:04d}", w.frame)
    p = w.params
    keys = ("b0", "p0", "pmin", "pmax", "momentum_dependency", "gamma_turb", "mag_dependency",
            "kpara0", "kret", "dt_min_rel", "dt_max_rel")
    vals = dict(b0=1.0, **p)
    lines = ["!< conf.dat written by the test"] + [f"{k} = {vals[k]!r}" for k in keys]
    lines += ["acc_region_flag = 0", "npp_global = 64", "nmu_global = 4",
              f"pbcx = {p['pbcx']}", f"pbcy = {p['pbcy']}", f"pbcz = {p['pbcz']}"]
    (tmp_path / "config" / "conf.dat").write_text("\n".join(lines) + "\n")
    return w, data, out


def _run_driver(tmp_path, data, out, precision="fp64", ft=False, nlgc=False, extra=(),
                shock_plane=True):
    exe = build.build_driver()
    plane = ["--shock_xpos", "0.5"] if shock_plane else []
    cmd = [str(exe), "-dm", str(data) + "/", "-cf", "conf.dat", "-dd", str(out) + "/",
           "-ts", "0", "-te", "3", "-np", "2000", "-nm", "40000", "-is", "1", *plane, "-df", "1", "-pv", "1.0", "-dt", "1e-7", "-sf", "1", "-nd", "2",
           "--precision", precision, "--seed", str(SEED), "-ug", "1",
           "-ft", ".true." if ft else ".false.",
           "-nl", ".true." if nlgc else ".false.", "-kk", "0.05", "-du", "3.0", "-pd", "1",
           "-ded", ".true.", "-de", ".true.", *extra]
    return subprocess.run(cmd, cwd=tmp_path, capture_output=True, text=True, timeout=600)


def _read_fdists(path: Path):
    raw = path.read_bytes()
    npp = int(np.frombuffer(raw[:4], np.int32)[0])
    off = 4
    edges = np.frombuffer(raw[off:off + 8 * (npp + 1)], np.float64); off += 8 * (npp + 1)
    f = np.frombuffer(raw[off:off + 8 * npp], np.float64); off += 8 * npp
    c = np.frombuffer(raw[off:off + 8 * npp], np.uint64)
    return edges, f, c


def test_driver_usage_without_gpu(engine_lib):
    exe = build.build_driver()
    r = subprocess.run([str(exe), "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "usage" in r.stderr
    r = subprocess.run([str(exe), "--no_such_switch", "1"], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 2
    r = subprocess.run([str(exe), "-dm", "/nonexistent/"], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 1 and "gpat_load_mhd_config" in r.stderr
    r = subprocess.run([str(exe), "-sm", "2"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "-sm must be 1" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("ft,nlgc", [(False, False), (True, True)])
def test_driver_matches_python_sequence(tmp_path, ft, nlgc):
    w, data, out = _dataset(tmp_path)
    r = _run_driver(tmp_path, data, out, ft=ft, nlgc=nlgc)
    assert r.returncode == 0, r.stderr
    quick = (out / "quick.dat").read_text().splitlines()
    assert len(quick) == 5 and quick[0].split()[0] == "iframe"
    edges, f_drv, c_drv = _read_fdists(out / "fdists_0003.dat")

    # The same calls from Python.
    prm = make_params(**dict(w.params, npp_global=64, nptl_max=40000, seed=SEED, precision=0,
                             b0=1.0, drift1=4e7, drift2=2e8, charge=-1, duu0=3.0))
    eng = Engine(prm, w.mhd_config, 0)
    eng.calc_tstamps_mhd(0, 3)
    eng.read_field_data(data / "mhd_data_0000", 0)
    eng.calc_fields_gradients(0)
    for tf in range(1, 4):
        eng.read_field_data(data / f"mhd_data_{tf:04d}", 0)
        eng.calc_fields_gradients(0)
        eng.inject_particles_at_x(2000, 0.5, 1e-7, 1, 1.0, tf)
        eng.particle_mover(nsteps_interval=10, mhd_tframe=tf, num_fine_steps=1,
                           focused_transport=ft, nlgc=nlgc, kperp_kpara=0.05,
                           dump_escaped_dist=True)
        eng.split_particle(2.72, 2.0, 10)
        if tf == 3:
            fe, ce = eng.calc_escaped_distributions()
            esc = eng.get_escaped_particles()
            fem, cem = eng.escaped_distributions_mu(4)
        eng.reset_escaped_particles()
    # escaped distributions and particles of the last frame (-ded, -de)
    raw = (out / "fescaped_0003.dat").read_bytes()
    npp, ncol = np.frombuffer(raw[:8], np.int32)
    off = 8 + 8 * (npp + 1)
    assert np.array_equal(np.frombuffer(raw[off:off + 8 * npp * ncol], np.float64), fe.ravel())
    off += 8 * npp * ncol
    assert np.array_equal(np.frombuffer(raw[off:off + 8 * npp * ncol], np.uint64), ce.ravel())
    d = read_particle_dump(out / "escaped_particles_0003.dat")
    assert len(d["x"]) == len(esc)
    for k in d:
        assert np.array_equal(d[k], esc[k]), k
    f, c = eng.calc_particle_distributions()
    assert np.array_equal(c, c_drv) and np.array_equal(f, f_drv)
    np.testing.assert_allclose(edges, eng.pbins_edges(), rtol=0)
    # focused transport: nmu_global = 4 pitch-angle bins (Parker keeps 1)
    assert (out / "fglobal_mu_0003.dat").exists() == ft
    if ft:
        for name, (fr, cr) in (("fglobal_mu_0003.dat", eng.particle_distributions_mu(4)),
                               ("fescaped_mu_0003.dat", (fem, cem))):
            raw = (out / name).read_bytes()
            nmu, npp_, nface = np.frombuffer(raw[:12], np.int32)
            nb = int(nmu * npp_ * nface)
            off = 12 + 8 * (nmu + 1) + 8 * (npp_ + 1)
            assert nmu == 4 and npp_ == 64
            assert np.array_equal(np.frombuffer(raw[off:off + 8 * nb], np.float64), fr.ravel())
            assert np.array_equal(np.frombuffer(raw[off + 8 * nb:], np.uint64), cr.ravel())
            assert cr.sum() > 0 or name.startswith("fescaped")   # frame 3 may have no escapes
    q = eng.quick_check()
    last = quick[-1].split()
    assert int(last[0]) == 3 and float(last[1]) == q["nptl_current"]
    # particle dumps (-pd 1) per frame, and the restart dump at t_end
    assert all((out / f"particles_{t:04d}.dat").exists() for t in range(4))
    got = eng.get_particles()
    for path in (out / "particles_0003.dat", out / "restart" / "particles_0003.dat"):
        d = read_particle_dump(path)
        assert len(d["x"]) == len(got)
        for k in d:
            assert np.array_equal(d[k], got[k]), k
    eng.close()


def _read_tracked(path: Path) -> dict:
    """particles_tracked_XXXX.dat: int64 nsteps_tracking_max, int64
    nptl_tracking, then each dataset in Fortran order."""
    raw = path.read_bytes()
    nsteps, ntrk = np.frombuffer(raw[:16], np.int64)
    m = int(nsteps * ntrk)
    out, off = {}, 16
    names = [("x", "f8"), ("y", "f8"), ("z", "f8"), ("p", "f8"), ("v", "f8"), ("mu", "f8"),
             ("weight", "f8"), ("t", "f8"), ("dt", "f8"), ("split_times", "i1"),
             ("count_flag", "i1"), ("origin", "i4"), ("nsteps_tracked", "i4"),
             ("nsteps_pushed", "i4"), ("tag_injected", "i4"), ("tag_splitted", "i4")]
    for k, t in names:
        size = np.dtype(t).itemsize * m
        out[k] = np.frombuffer(raw[off:off + size], t).reshape(int(ntrk), int(nsteps))
        off += size
    assert off == len(raw)
    return out


@pytest.mark.gpu
def test_driver_particle_tracking(tmp_path):
    """-tf .true. -ptf -ni: the tags table is read from
    particle_tracking/, the mover runs with one fine step, and
    particles_tracked_XXXX.dat per frame equals the records of the same
    calls made from Python; the distributions are not written."""
    w, data, out = _dataset(tmp_path)
    (out / "particle_tracking").mkdir()
    table = np.array([(0, t, a, b) for t in (3, 50, 777, 2100)
                      for a, b in ((1, 1), (1, 3), (2, 2), (2, 4))], np.int32)
    tags_file = out / "particle_tracking" / "tags.dat"
    with open(tags_file, "wb") as f:
        np.array([table.shape[1], table.shape[0]], np.int32).tofile(f)
        table.tofile(f)
    r = _run_driver(tmp_path, data, out, extra=("-tf", ".true.", "-ptf", "tags.dat",
                                                "-ni", "5", "-nf", "4"))
    assert r.returncode == 0, r.stderr
    assert not (out / "fdists_0001.dat").exists()
    assert len((out / "quick.dat").read_text().splitlines()) == 1

    prm = make_params(**dict(w.params, npp_global=64, nptl_max=40000, seed=SEED, precision=0,
                             b0=1.0, drift1=4e7, drift2=2e8, charge=-1, duu0=3.0))
    eng = Engine(prm, w.mhd_config, 0)
    eng.calc_tstamps_mhd(0, 3)
    eng.read_particle_tracking(tags_file, 5)
    eng.read_field_data(data / "mhd_data_0000", 0)
    eng.calc_fields_gradients(0)
    for tf in range(1, 4):
        eng.read_field_data(data / f"mhd_data_{tf:04d}", 0)
        eng.calc_fields_gradients(0)
        eng.inject_particles_at_x(2000, 0.5, 1e-7, 1, 1.0, tf)
        eng.particle_mover(nsteps_interval=5, mhd_tframe=tf, num_fine_steps=1)
        rec = eng.get_tracked_particles()
        d = _read_tracked(out / "particle_tracking" / f"particles_tracked_{tf:04d}.dat")
        for k in d:
            assert np.array_equal(d[k], rec[k]), (tf, k)
        assert (d["tag_splitted"] < 0).sum() > 0
        eng.split_particle(2.72, 2.0, 5)
    got = eng.get_particles()
    d = read_particle_dump(out / "restart" / "particles_0003.dat")
    for k in d:
        assert np.array_equal(d[k], got[k]), k
    eng.close()


def _read_flocal(path: Path):
    """flocalK_XXXX.dat: int32 dims {nmu, npbins, nrx, nry, nrz}, p edges,
    mu edges, flocal and counts in Fortran order."""
    raw = path.read_bytes()
    dims = np.frombuffer(raw[:20], np.int32)
    nb = int(np.prod(dims))
    off = 20
    pe = np.frombuffer(raw[off:off + 8 * (dims[1] + 1)], np.float64); off += 8 * (dims[1] + 1)
    me = np.frombuffer(raw[off:off + 8 * (dims[0] + 1)], np.float64); off += 8 * (dims[0] + 1)
    f = np.frombuffer(raw[off:off + 8 * nb], np.float64); off += 8 * nb
    c = np.frombuffer(raw[off:off + 8 * nb], np.uint64); off += 8 * nb
    assert off == len(raw)
    return dims, pe, me, f, c


@pytest.mark.gpu
def test_driver_restart_quota_local_dist(tmp_path):
    """A run stopped by -qh after its first frame and resumed with -rf ends
    with the particles, f(p), local distributions (-ld), quick.dat and
    pmax_global.dat of an uninterrupted run, bit for bit; -vdt reads the
    frame time stamps from time_stamps.dat."""
    w, data, out = _dataset(tmp_path)
    conf = tmp_path / "config" / "conf.dat"
    conf.write_text(conf.read_text() + "\n".join([
        "dump_interval1 = 1", "pmin1 = 0.1", "pmax1 = 100.0", "npbins1 = 16", "nmu1 = 4",
        "rx1 = 8", "ry1 = 4", "rz1 = 1",
        "dump_interval2 = 100", "pmin2 = 0.1", "pmax2 = 10.0", "npbins2 = 8", "nmu2 = 1",
        "rx2 = 1", "ry2 = 1", "rz2 = 1", "dump_interval3 = 100", "dump_interval4 = 100"])
        + "\n")
    with open(data / "time_stamps.dat", "wb") as f:
        np.array([0, 3], np.int64).tofile(f)
        (np.arange(4) * w.mhd_config.dt_out).tofile(f)
    extra = ("-ld", ".true.", "-vdt", ".true.", "-tm", "3")
    r = _run_driver(tmp_path, data, out, extra=extra)
    assert r.returncode == 0, r.stderr
    out2 = tmp_path / "out2"
    out2.mkdir()
    r = _run_driver(tmp_path, data, out2, extra=extra + ("-qh", "0.5"))
    assert r.returncode == 0, r.stderr
    assert "reached the quota time at frame 1" in r.stdout
    assert np.fromfile(out2 / "restart" / "latest_restart", np.int32)[0] == 1
    assert (out2 / "restart" / "particles_0001.dat").exists()
    assert not (out2 / "fdists_0002.dat").exists()
    r = _run_driver(tmp_path, data, out2, extra=extra + ("-rf", ".true."))
    assert r.returncode == 0, r.stderr
    assert np.fromfile(out2 / "restart" / "latest_restart", np.int32)[0] == 3
    a = read_particle_dump(out / "restart" / "particles_0003.dat")
    b = read_particle_dump(out2 / "restart" / "particles_0003.dat")
    assert len(a["x"]) == len(b["x"]) > 0
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    for name in ("fdists_0003.dat", "flocal1_0003.dat", "pmax_global.dat", "quick.dat",
                 "restart/particle_module_state_0003.dat", "restart/prng_state_0003.dat"):
        assert (out / name).read_bytes() == (out2 / name).read_bytes(), name
    dims, pe, me, f, c = _read_flocal(out / "flocal1_0003.dat")
    nx, ny = w.mhd_config.nx, w.mhd_config.ny
    assert list(dims) == [1, 16, (nx + 7) // 8, (ny + 3) // 4, 1] and c.sum() > 0 and f.sum() > 0
    assert pe[0] == pytest.approx(0.1) and pe[-1] == pytest.approx(100.0)
    assert list(me) == [-1.0, 1.0]
    assert not (out / "flocal2_0003.dat").exists()
    # local escaped distributions of set 1 (-ld with -ded): x and y faces
    raw = (out / "fescaped1_0003.dat").read_bytes()
    assert np.array_equal(np.frombuffer(raw[:20], np.int32), dims)
    assert len(raw) == 20 + 16 * 2 * 16 * (dims[3] + dims[2])
    assert raw == (out2 / "fescaped1_0003.dat").read_bytes()
    assert len((out / "pmax_global.dat").read_text().splitlines()) == 4


@pytest.mark.gpu
def test_load_tstamps_mhd(tmp_path):
    """load_tstamps_mhd: stamps from time_stamps.dat, frames past tmax_mhd
    continued with the last interval (injection times show them)."""
    w, data, _ = _dataset(tmp_path)
    with open(data / "time_stamps.dat", "wb") as f:
        np.array([0, 5], np.int64).tofile(f)
        np.array([0.0, 0.1, 0.25, 0.3, 0.5, 0.9]).tofile(f)
    prm = make_params(**dict(w.params, nptl_max=1000, precision=0))
    eng = Engine(prm, w.mhd_config, 0)
    eng.load_tstamps_mhd(1, 4, 2, data)          # frames 1..4: 0.1, 0.25, then +0.15
    eng.read_field_data(data / "mhd_data_0000", 0)
    eng.calc_fields_gradients(0)
    eng.inject_particles_spatial_uniform(200, 1e-6, 1, 1.0, 3, (0, 0, 0, 1, 0.125, 1))
    t = eng.get_particles()["t"]
    assert t.min() >= 0.4 - 1e-12 and t.max() < 0.55 + 1e-12 and t.max() > 0.5
    assert eng.get_pmax_global() == pytest.approx(w.params["p0"])
    with pytest.raises(Exception):
        eng.load_tstamps_mhd(1, 4, 2, tmp_path / "nowhere")
    eng.close()


@pytest.mark.gpu
def test_driver_injects_at_the_located_shock(tmp_path):
    """-is without --shock_xpos locates the shock each frame
    (locate_shock_xpos + inject_particles_at_shock): the restart dump equals
    the same calls made from Python, and the particles start on the shock."""
    w, data, out = _dataset(tmp_path)
    r = _run_driver(tmp_path, data, out, shock_plane=False)
    assert r.returncode == 0, r.stderr
    prm = make_params(**dict(w.params, npp_global=64, nptl_max=40000, seed=SEED, precision=0,
                             b0=1.0, drift1=4e7, drift2=2e8, charge=-1, duu0=3.0))
    eng = Engine(prm, w.mhd_config, 0)
    eng.calc_tstamps_mhd(0, 3)
    eng.read_field_data(data / "mhd_data_0000", 0)
    eng.calc_fields_gradients(0)
    for tf in range(1, 4):
        eng.read_field_data(data / f"mhd_data_{tf:04d}", 0)
        eng.calc_fields_gradients(0)
        eng.inject_particles_at_shock(2000, 1e-7, 1, 1.0, tf)
        if tf == 1:
            x0 = eng.get_particles()["x"]
            assert np.all(np.abs(x0 - 0.5) <= w.mhd_config.dx)   # the planar shock at 0.5
        eng.particle_mover(nsteps_interval=10, mhd_tframe=tf, num_fine_steps=1,
                           dump_escaped_dist=True)
        eng.split_particle(2.72, 2.0, 10)
        eng.reset_escaped_particles()
    got = eng.get_particles()
    d = read_particle_dump(out / "restart" / "particles_0003.dat")
    assert len(d["x"]) == len(got)
    for k in d:
        assert np.array_equal(d[k], got[k]), k
    eng.close()


@pytest.mark.gpu
def test_driver_1d_run(tmp_path):
    """-nd 1 runs on the FP64 mover by default and ends with the particles
    and f(p) of the same calls made from Python."""
    n = 128
    cfg = make_mhd_config(n, 1, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.05, ndim=1)
    x = fields.node_coords(n, 0.0, 1.0 / n)[None, None, :]
    z = np.zeros_like(x)
    vx = 1.0 - 0.75 * (1.0 + np.tanh((x - 0.5) / 0.01)) / 2.0
    frame = fields.assemble_frame(vx, z, z, 1.0 + z, 1.0 + z, 0.2 + z, z).astype(np.float32)
    data, out = tmp_path / "data", tmp_path / "out"
    data.mkdir()
    out.mkdir()
    (tmp_path / "config").mkdir()
    fields.write_mhd_config(data / "mhd_config.dat", cfg)
    for t in range(3):
        fields.write_mhd_data(data / f"mhd_data_{t:04d}", frame)
    vals = dict(b0=1.0, p0=0.1, pmin=0.1, pmax=100.0, momentum_dependency=0, gamma_turb=5 / 3,
                mag_dependency=0, kpara0=1e-3, kret=0.1, dt_min_rel=1e-3, dt_max_rel=1e-2)
    lines = [f"{k} = {v!r}" for k, v in vals.items()]
    lines += ["acc_region_flag = 0", "npp_global = 32", "nmu_global = 1", "pbcx = 1",
              "pbcy = 0", "pbcz = 0"]
    (tmp_path / "config" / "conf.dat").write_text("\n".join(lines) + "\n")
    exe = build.build_driver()
    cmd = [str(exe), "-dm", str(data) + "/", "-cf", "conf.dat", "-dd", str(out) + "/", "-ts", "0",
           "-te", "2", "-np", "500", "-nm", "5000", "-is", "1", "--shock_xpos", "0.5", "-df", "1",
           "-pv", "1.0", "-dt", "1e-7", "-sf", "0", "-nd", "1", "-ug", "1", "-nl", ".false.",
           "--seed", str(SEED)]
    r = subprocess.run(cmd, cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    prm = make_params(**dict(vals, ndim=1, npp_global=32, nptl_max=5000, seed=SEED, precision=0,
                             pbcx=1, drift1=4e7, drift2=2e8, charge=-1))
    eng = Engine(prm, cfg, 0)
    eng.calc_tstamps_mhd(0, 2)
    for tf in range(1, 3):
        eng.read_field_data(data / f"mhd_data_{tf:04d}", 0)
        eng.calc_fields_gradients(0)
        eng.inject_particles_at_x(500, 0.5, 1e-7, 1, 1.0, tf)
        eng.particle_mover(nsteps_interval=10, mhd_tframe=tf, num_fine_steps=1)
    got = eng.get_particles()
    d = read_particle_dump(out / "restart" / "particles_0002.dat")
    assert len(d["x"]) == len(got) > 0
    for k in d:
        assert np.array_equal(d[k], got[k]), k
    _, f_drv, c_drv = _read_fdists(out / "fdists_0002.dat")
    f, c = eng.calc_particle_distributions()
    assert np.array_equal(c, c_drv) and np.array_equal(f, f_drv) and c.sum() > 0
    eng.close()


def _bump(shape, seed, lo, hi):
    """Smooth positive per-node array over the ghost-padded grid."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    Y, X = np.meshgrid(np.linspace(0, 1, ny), np.linspace(0, 1, nx), indexing="ij")
    f = np.zeros_like(X)
    for _ in range(3):
        kx, ky = rng.integers(1, 4, size=2)
        f += np.sin(2 * np.pi * (kx * X + ky * Y) + rng.uniform(0, 2 * np.pi))
    f = (f - f.min()) / (f.max() - f.min())
    return np.broadcast_to(lo + (hi - lo) * f, shape).astype(np.float32)


@pytest.mark.gpu
def test_driver_turbulence_and_db2_injection(tmp_path):
    """-db 1 -co 1: deltab_XXXX / lc_XXXX read with every frame
    (stochastic-mhd.f90:337-346, :417-424); -ib 1 injects where db2_slab
    exceeds -db2, normalised by -nb (:466-469)."""
    w, data, out = _dataset(tmp_path)
    shape = w.frame.shape[:3]
    for t in range(4):
        db = np.concatenate([_bump(shape, 10 + t, 0.5, 2.0).ravel(),
                             _bump(shape, 20 + t, 0.3, 1.0).ravel()])
        lc = np.concatenate([_bump(shape, 30 + t, 0.5, 1.5).ravel(),
                             _bump(shape, 40 + t, 0.5, 1.5).ravel()])
        db.tofile(data / f"deltab_{t:04d}")
        lc.tofile(data / f"lc_{t:04d}")
    exe = build.build_driver()
    cmd = [str(exe), "-dm", str(data) + "/", "-cf", "conf.dat", "-dd", str(out) + "/",
           "-ts", "0", "-te", "3", "-np", "300", "-nm", "40000", "-is", "0", "-in", "1",
           "-df", "1", "-pv", "1.0", "-dt", "1e-7", "-sf", "1", "-nd", "2", "--seed", str(SEED),
           "-db", "1", "-co", "1", "-ib", ".true.", "-db2", "1.4", "-nb", "2000", "-ug", "1"]
    r = subprocess.run(cmd, cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    edges, f_drv, c_drv = _read_fdists(out / "fdists_0003.dat")

    prm = make_params(**dict(w.params, npp_global=64, nptl_max=40000, seed=SEED, precision=0,
                             b0=1.0, drift1=4e7, drift2=2e8, charge=-1, deltab_flag=1,
                             correlation_flag=1))
    eng = Engine(prm, w.mhd_config, 0)
    eng.calc_tstamps_mhd(0, 3)
    cfg = w.mhd_config
    box = (cfg.xmin, cfg.ymin, cfg.zmin, cfg.xmin + cfg.nx * cfg.dx, cfg.ymin + cfg.ny * cfg.dy,
           cfg.zmax)
    injected = 0
    for tf in range(4):
        eng.read_field_data(data / f"mhd_data_{tf:04d}", 0)
        eng.read_magnetic_fluctuation(data / f"deltab_{tf:04d}", 0)
        eng.read_correlation_length(data / f"lc_{tf:04d}", 0)
        eng.calc_fields_gradients(0)
        if tf == 0:
            continue
        injected += eng.inject_particles_at_large(4, 300, 1e-7, 1, 1.0, tf, False, 1.4, 2000,
                                                  box)
        eng.particle_mover(nsteps_interval=10, mhd_tframe=tf, num_fine_steps=1, nlgc=True,
                           kperp_kpara=0.01)
        eng.split_particle(2.72, 2.0, 10)
    assert injected > 0
    f, c = eng.calc_particle_distributions()
    assert np.array_equal(c, c_drv) and np.array_equal(f, f_drv)
    eng.close()


@pytest.mark.gpu
def test_driver_spherical_nonuniform_grid(tmp_path):
    """-sc 1 with the reference's default -ug 0: node positions from
    xpos.dat / ypos.dat in the data directory (set_local_grid_positions,
    stochastic-mhd.f90:186), the FP64 mover in spherical coordinates; f(p)
    equals the same calls made from Python, bit for bit."""
    from gpat.engine import make_mhd_config
    nx, ny = 64, 32
    rng = np.random.default_rng(4)
    pos = []
    for n, lo, hi in ((nx, 0.5, 1.5), (ny, 0.6, np.pi - 0.6)):
        h = rng.uniform(0.7, 1.3, n + 3)
        x = np.concatenate([[0.0], np.cumsum(h)])
        pos.append(lo + (x - x[2]) * (hi - lo) / (x[n + 2] - x[2]))
    cfg = make_mhd_config(nx, ny, 1, 0.5, 1.5, 0.6, np.pi - 0.6, dt_out=0.05)
    data = tmp_path / "data"
    data.mkdir()
    (tmp_path / "config").mkdir()
    out = tmp_path / "out"
    out.mkdir()
    fields.write_mhd_config(data / "mhd_config.dat", cfg)
    frame = fields.planar_shock_2d(nx, ny, 0.5, 1.5, 0.6, np.pi - 0.6, r=3.0, w=0.02, x0=1.0,
                                   db=fields.kolmogorov_az_2d(nx, ny, 1.0, 1.0, 0.5, 2 * np.pi,
                                                              16 * np.pi, 2))
    for t in range(3):
        fields.write_mhd_data(data / f"mhd_data_{t:04d}", frame)
    pos[0].tofile(data / "xpos.dat")
    pos[1].tofile(data / "ypos.dat")
    keys = dict(b0=1.0, p0=0.1, pmin=0.05, pmax=100.0, momentum_dependency=0, gamma_turb=5 / 3,
                mag_dependency=0, kpara0=2e-3, kret=0.1, dt_min_rel=2e-3, dt_max_rel=5e-2)
    lines = ["!< conf.dat written by the test"] + [f"{k} = {v!r}" for k, v in keys.items()]
    lines += ["acc_region_flag = 0", "npp_global = 64", "nmu_global = 1", "pbcx = 1", "pbcy = 1",
              "pbcz = 0"]
    (tmp_path / "config" / "conf.dat").write_text("\n".join(lines) + "\n")
    exe = build.build_driver()
    cmd = [str(exe), "-dm", str(data) + "/", "-cf", "conf.dat", "-dd", str(out) + "/",
           "-ts", "0", "-te", "2", "-np", "1500", "-nm", "20000", "-is", "0", "-df", "1",
           "-pv", "1.0", "-dt", "1e-7", "-sf", "1", "-nd", "2", "--seed", str(SEED), "-sc", "1",
           "-nl", ".false."]
    r = subprocess.run(cmd, cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    edges, f_drv, c_drv = _read_fdists(out / "fdists_0002.dat")

    prm = make_params(ndim=2, npp_global=64, nptl_max=20000, seed=SEED, precision=0, b0=1.0,
                      drift1=4e7, drift2=2e8, charge=-1, pbcx=1, pbcy=1, spherical_coord=1,
                      nonuniform_grid=1, **{k: v for k, v in keys.items() if k != "b0"})
    eng = Engine(prm, cfg, 0)
    eng.calc_tstamps_mhd(0, 2)
    eng.read_grid_positions(data)
    box = (0.5, 0.6, cfg.zmin, 0.5 + nx * cfg.dx, 0.6 + ny * cfg.dy, cfg.zmax)
    for tf in range(3):
        eng.read_field_data(data / f"mhd_data_{tf:04d}", 0)
        eng.calc_fields_gradients(0)
        if tf == 0:
            continue
        if tf == 1:
            eng.inject_particles_spatial_uniform(1500, 1e-7, 1, 1.0, tf, box)
        eng.particle_mover(nsteps_interval=10, mhd_tframe=tf, num_fine_steps=1)
        eng.split_particle(2.72, 2.0, 10)
    f, c = eng.calc_particle_distributions()
    assert np.array_equal(c, c_drv) and np.array_equal(f, f_drv) and c.sum() > 0
    eng.close()


@pytest.mark.gpu
def test_driver_acceleration_surfaces_3d(tmp_path):
    """-as 1 with two surfaces read from <dir><name>_XXXX.dat with every
    frame (stochastic-mhd.f90:196-203, :324-333, :406-415); f(p) equals the
    same calls made from Python, bit for bit."""
    from gpat.engine import make_mhd_config
    n = 16
    g = n + 4
    cfg = make_mhd_config(n, n, n, 0.0, 1.0, 0.0, 1.0, zmin=0.0, zmax=1.0, dt_out=0.05, ndim=3)
    data = tmp_path / "data"
    data.mkdir()
    (tmp_path / "config").mkdir()
    out = tmp_path / "out"
    out.mkdir()
    fields.write_mhd_config(data / "mhd_config.dat", cfg)
    frame = fields.turbulence_3d(n, seed=5)
    rng = np.random.default_rng(6)
    for t in range(3):
        fields.write_mhd_data(data / f"mhd_data_{t:04d}", frame)
        (0.5 + 0.1 * rng.standard_normal((g, g))).tofile(data / f"top_{t:04d}.dat")
        (0.3 + 0.1 * rng.standard_normal((g, g))).tofile(data / f"side_{t:04d}.dat")
    keys = dict(b0=1.0, p0=0.1, pmin=0.05, pmax=100.0, momentum_dependency=0, gamma_turb=5 / 3,
                mag_dependency=0, kpara0=2e-3, kret=0.1, dt_min_rel=2e-3, dt_max_rel=5e-2)
    lines = ["!< conf.dat written by the test"] + [f"{k} = {v!r}" for k, v in keys.items()]
    lines += ["acc_region_flag = 1", "acc_xmin = 0.0", "acc_xmax = 1.0", "acc_ymin = 0.0",
              "acc_ymax = 1.0", "acc_zmin = 0.0", "acc_zmax = 1.0", "npp_global = 64",
              "nmu_global = 1", "pbcx = 0", "pbcy = 0", "pbcz = 0"]
    (tmp_path / "config" / "conf.dat").write_text("\n".join(lines) + "\n")
    exe = build.build_driver()
    cmd = [str(exe), "-dm", str(data) + "/", "-cf", "conf.dat", "-dd", str(out) + "/",
           "-ts", "0", "-te", "2", "-np", "2000", "-nm", "20000", "-is", "0", "-df", "1",
           "-pv", "1.0", "-dt", "1e-7", "-sf", "0", "-nd", "3", "--seed", str(SEED), "-ug", "1",
           "-nl", ".false.", "-ti", "1", "-as", "1", "-sf1", "top", "-sn1", "+z", "-s2e", "T",
           "-sf2", "side", "-sn2", "-x", "-ii", "F"]
    r = subprocess.run(cmd, cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    edges, f_drv, c_drv = _read_fdists(out / "fdists_0002.dat")

    prm = make_params(ndim=3, npp_global=64, nptl_max=20000, seed=SEED, precision=0, b0=1.0,
                      drift1=4e7, drift2=2e8, charge=-1, pbcx=0, pbcy=0, pbcz=0, time_interp=1,
                      acc_region_flag=1, acc_region=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0),
                      **{k: v for k, v in keys.items() if k != "b0"})
    eng = Engine(prm, cfg, 0)
    eng.calc_tstamps_mhd(0, 2)
    eng.init_acc_surface("+z", "-x", False)
    eng.read_field_data(data / "mhd_data_0000", 0)
    eng.read_acc_surface(0, data / "top_0000.dat", data / "side_0000.dat")
    eng.calc_fields_gradients(0)
    for tf in (1, 2):
        eng.read_field_data(data / f"mhd_data_{tf:04d}", 1)
        eng.read_acc_surface(1, data / f"top_{tf:04d}.dat", data / f"side_{tf:04d}.dat")
        eng.calc_fields_gradients(1)
        if tf == 1:
            eng.inject_particles_spatial_uniform(2000, 1e-7, 1, 1.0, tf,
                                                 (0.0, 0.0, 0.0, 1.0, 1.0, 1.0))
        eng.particle_mover(nsteps_interval=10, mhd_tframe=tf, num_fine_steps=1)
        eng.copy_fields()
    f, c = eng.calc_particle_distributions()
    assert np.array_equal(c, c_drv) and np.array_equal(f, f_drv) and c.sum() > 0
    eng.close()
