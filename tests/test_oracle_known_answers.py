"""Known-answer checks that pin the CPU oracle (no GPU).

The reference ships no tests or golden vectors, so the oracle is pinned by
published vectors (Philox) and by cases whose answer follows exactly from
the reference's own update rules (particle_module.f90): discrete drift with
a linear velocity field, diffusion covariance 2*kappa*t, the half-cell
periodic wrap, remove_particles' swap order, split_particle's weights and
tags, and the log-p binning of calc_particle_distributions.
"""
import ctypes as C
import math

import numpy as np
import pytest

import oracle
from gpat.engine import make_mhd_config, make_params
from gpat import fields


def test_philox_published_vectors():
    # Random123 known-answer vectors for philox4x32-10.
    assert oracle.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert oracle.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == \
        [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert oracle.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344],
                         [0xA4093822, 0x299F31D0]) == [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_u01_range_and_resolution():
    lib = oracle.load()
    assert lib.orc_u01(0, 0) == 0.0
    top = lib.orc_u01(0xFFFFFFFF, 0xFFFFFFFF)
    assert top < 1.0 and top == 1.0 - 2.0 ** -53


def _linear_frame(nx, ny, a, b, c):
    """vx = a + b x + c y on the nodes (others zero, B = x)."""
    dx, dy = 1.0 / nx, 1.0 / ny
    x = fields.node_coords(nx, 0.0, dx)
    y = fields.node_coords(ny, 0.0, dy)
    X, Y = np.meshgrid(x, y)
    vx = a + b * X + c * Y
    z = np.zeros_like(X)
    return fields.assemble_frame(vx, z, z, z + 1.0, z + 1.0, z, z)[None]


def test_gradients_linear_field_exact():
    nx, ny = 32, 16
    cfg = make_mhd_config(nx, ny, 1, 0.0, 1.0, 0.0, 1.0)
    frame = _linear_frame(nx, ny, 0.25, 0.5, -0.75)
    full = oracle.full_fields(frame, 2, cfg)
    # d vx/dx = 0.5 and d vx/dy = -0.75 everywhere, ends included (the
    # one-sided 2nd-order formula is exact for linear data).
    np.testing.assert_allclose(full[0, :, :, 8], 0.5, rtol=0, atol=2e-5)
    np.testing.assert_allclose(full[0, :, :, 9], -0.75, rtol=0, atol=2e-5)
    assert np.all(full[0, :, :, 10] == 0.0)   # no z-gradient in 2D


def test_interp_reproduces_linear_field():
    nx, ny = 32, 16
    cfg = make_mhd_config(nx, ny, 1, 0.0, 1.0, 0.0, 1.0)
    frame = _linear_frame(nx, ny, 0.25, 0.5, -0.75)
    full = oracle.full_fields(frame, 2, cfg)
    lib = oracle.load()
    rng = np.random.default_rng(0)
    for _ in range(50):
        x, y = rng.uniform(-0.5 / nx, 1 + 0.5 / nx), rng.uniform(-0.5 / ny, 1 + 0.5 / ny)
        pos = (C.c_int32 * 3)()
        w = (C.c_double * 8)()
        lib.orc_get_interp_paramters(2, x * nx, y * ny, 0.0, pos, w)
        assert abs(sum(w) - 1.0) < 1e-15
        f = (C.c_double * 32)()
        lib.orc_interp_fields(full.ctypes.data_as(C.POINTER(C.c_float)), None, 0, 2, nx + 4,
                              ny + 4, pos, w, 0.0, f)
        assert abs(f[0] - (0.25 + 0.5 * x - 0.75 * y)) < 1e-6


def _kappa(params, bx, by, bz, p=0.1, ndim=3, mu=0.5):
    prm = oracle.params_from(params)
    f = (C.c_double * 32)()
    f[4], f[5], f[6] = bx, by, bz
    k = (C.c_double * 22)()
    oracle.load().orc_calc_spatial_diffusion_coefficients(C.byref(prm), p, mu, f, None, k)
    return list(k)


def test_kappa_tensor_is_projection_of_b():
    prm = make_params(ndim=3, kpara0=0.02, kret=0.1, momentum_dependency=0)
    bx, by, bz = 0.3, -0.4, 1.2
    k = _kappa(prm, bx, by, bz)
    kpara, kperp = k[2], k[3]
    assert kpara == pytest.approx(0.02) and kperp == pytest.approx(0.002)
    b = np.array([bx, by, bz]) / math.sqrt(bx * bx + by * by + bz * bz)
    K = kperp * np.eye(3) + (kpara - kperp) * np.outer(b, b)
    got = np.array([[k[7], k[10], k[11]], [k[10], k[8], k[12]], [k[11], k[12], k[9]]])
    np.testing.assert_allclose(got, K, rtol=1e-14, atol=1e-18)
    assert k[4] == pytest.approx(math.sqrt(2 * kpara))
    assert k[6] == pytest.approx(math.sqrt(2 * (kpara - kperp)))


def _single_run(params_kw, frame, cfg, parts_init, t0, dtf, ndim=2, fine=1):
    prm = oracle.params_from(make_params(**params_kw))
    ocfg = oracle.config_from(cfg)
    full = oracle.full_fields(frame, ndim, cfg)
    parts = oracle.Particles(len(parts_init["x"]) * 2 + 8, parts_init)
    cnt = oracle.mover(prm, ocfg, full, parts, t0, dtf, num_fine_steps=fine)
    return parts, cnt


def _parts(n, **vals):
    a = {k: np.zeros(n, dtype=t) for k, t in oracle.FIELDS}
    a["weight"][:] = 1.0
    a["count_flag"][:] = 1
    a["tag_splitted"][:] = 1
    a["tag_injected"][:] = np.arange(n, dtype=np.int32)
    for k, v in vals.items():
        a[k][:] = v
    return a


def test_drift_only_compression_matches_discrete_solution():
    """vx = -a x, kappa = 0: dy_dt == 0 forces dt = dt_min, so every push is
    x <- x (1 - a dt), p <- p (1 + a dt / 3) (push_particle_2d)."""
    nx, ny, a = 64, 8, 0.5
    cfg = make_mhd_config(nx, ny, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.1)
    frame = _linear_frame(nx, ny, 0.0, -a, 0.0)
    dt_min = 1.0e-3
    kw = dict(ndim=2, kpara0=0.0, kret=0.05, momentum_dependency=0, dt_min_rel=dt_min / 0.1,
              pbcx=0, pbcy=0, p0=0.1)
    x0 = np.linspace(0.3, 0.7, 9)
    parts, cnt = _single_run(kw, frame, cfg, _parts(9, x=x0, y=0.5, p=0.1), 0.0, 0.1)
    out = parts.view()
    order = np.argsort(out["tag_injected"])
    nsteps = 100
    np.testing.assert_allclose(out["x"][order], x0 * (1 - a * dt_min) ** nsteps, rtol=5e-7)
    np.testing.assert_allclose(out["p"][order], 0.1 * (1 + a * dt_min / 3) ** nsteps, rtol=1e-12)
    np.testing.assert_allclose(out["t"], 0.1, rtol=1e-13)
    # Pushes: the clock sums dt_min in double; an overshoot of the target is
    # undone and redone with the remainder (one extra push).
    t, pushes = 0.0, 0
    while t - 0.0 < 0.1:
        t += dt_min
        pushes += 1
    if t > 0.1 and 0.1 - (t - dt_min) > 0:
        pushes += 1
    assert cnt.steps == 9 * pushes


def test_diffusion_covariance_matches_two_kappa_t():
    """V = 0, uniform in-plane B at 30 degrees: <dx dx^T> = 2 kappa t."""
    nx = ny = 32
    cfg = make_mhd_config(nx, ny, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.05)
    th = math.radians(30.0)
    shape = (ny + 4, nx + 4)
    z = np.zeros(shape)
    frame = fields.assemble_frame(z, z, z, z + 1, z + math.cos(th), z + math.sin(th), z)[None]
    kpara, kret, T = 1.0e-3, 0.2, 0.05
    kw = dict(ndim=2, kpara0=kpara, kret=kret, momentum_dependency=0, dt_min_rel=0.01,
              pbcx=0, pbcy=0, p0=0.1, seed=7)
    n = 20000
    parts, _ = _single_run(kw, frame, cfg, _parts(n, x=0.5, y=0.5, p=0.1), 0.0, T)
    out = parts.view()
    d = np.stack([out["x"] - 0.5, out["y"] - 0.5])
    cov = d @ d.T / n
    b = np.array([math.cos(th), math.sin(th)])
    K = kpara * kret * np.eye(2) + kpara * (1 - kret) * np.outer(b, b)
    expect = 2 * K * T
    # sampling error of a variance ~ sqrt(2/n)
    np.testing.assert_allclose(cov, expect, atol=4 * math.sqrt(2.0 / n) * expect.max())
    assert abs(d.mean(axis=1)).max() < 4 * math.sqrt(expect.max() / n)


def test_periodic_wrap_uses_half_cell_extended_box():
    """particle_boundary_condition inside the mover wraps with the box
    extended by half a cell (particle_module.f90:1524-1529, 1607-1608)."""
    nx = ny = 16
    cfg = make_mhd_config(nx, ny, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.1)
    z = np.zeros((ny + 4, nx + 4))
    frame = fields.assemble_frame(z + 1.0, z, z, z + 1, z + 1, z, z)[None]  # vx = 1
    kw = dict(ndim=2, kpara0=0.0, momentum_dependency=0, dt_min_rel=0.01, pbcx=0, pbcy=0)
    x_start = 1.0 + 0.5 / nx + 1e-9       # just outside the extended box
    parts, _ = _single_run(kw, frame, cfg, _parts(1, x=x_start, y=0.5, p=0.1, t=0.2), 0.1, 0.1)
    # t already at the interval end: no push, only the boundary passes.  The
    # first pass wraps by the extended period 1 + dx to x < 0; the exact-box
    # pass (:1959-1973) wraps it back by 1: a net shift of one cell.
    out = parts.view()
    assert out["x"][0] == pytest.approx(x_start - 1.0 / nx, abs=1e-15)


def test_open_boundary_leak_and_escape_count():
    nx = ny = 16
    cfg = make_mhd_config(nx, ny, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.1)
    z = np.zeros((ny + 4, nx + 4))
    frame = fields.assemble_frame(z + 1.0, z, z, z + 1, z + 1, z, z)[None]
    kw = dict(ndim=2, kpara0=0.0, momentum_dependency=0, dt_min_rel=0.01, pbcx=1, pbcy=0)
    w = np.array([1.0, 0.5, 0.25, 1.0])
    x = np.array([0.97, 0.98, 0.5, 0.1])   # vx = 1 for t = 0.1: first two leave
    parts, cnt = _single_run(kw, frame, cfg, _parts(4, x=x, y=0.5, p=0.1, weight=w), 0.0, 0.1)
    assert parts.n == 2
    assert cnt.nptl_escaped == 2
    assert cnt.leak() == 1.5


def test_remove_particles_swap_order():
    """remove_particles (particle_module.f90:5365-5403) on flags [1,0,1,-1,1]
    keeps particles 1,5,3 in that order."""
    a = _parts(5)
    a["count_flag"][:] = [1, 0, 1, -1, 1]
    parts = oracle.Particles(5, a)
    cnt = oracle.OrcCounters()
    n = oracle.load().orc_remove_particles(C.byref(parts.c), 5, C.byref(cnt))
    assert n == 3
    assert list(parts.a["tag_injected"][:3]) == [0, 4, 2]
    assert cnt.nptl_escaped == 1


def test_split_particle_weights_tags_and_cap():
    prm = oracle.params_from(make_params(p0=0.1, pmax=10.0))
    a = _parts(4, p=[0.05, 0.25, 0.9, 20.0])
    parts = oracle.Particles(6, a)
    cnt = oracle.OrcCounters()
    oracle.split(prm, parts, 2.72, 2.0, cnt)       # threshold 0.2; p <= pmax
    assert parts.n == 6
    v = parts.view()
    assert list(v["weight"]) == [1.0, 0.5, 0.5, 1.0, 0.5, 0.5]
    assert list(v["split_times"]) == [0, 1, 1, 0, 1, 1]
    assert list(v["tag_splitted"]) == [1, 1, 1, 1, 2, 2]
    assert list(v["tag_injected"][4:]) == [1, 2]
    # second round: threshold 0.2 * 2.72 for split_times 1; cap stops it.
    parts2 = oracle.Particles(7, v)
    oracle.split(prm, parts2, 2.72, 2.0, cnt)
    v2 = parts2.view()
    assert parts2.n == 7                               # one more fits
    assert v2["weight"][2] == 0.25 and v2["tag_splitted"][6] == 1 + 2
    assert cnt.nptl_split == 3


def test_histogram_bins_and_strict_lower_edge():
    prm = oracle.params_from(make_params(pmin=0.1, pmax=1000.0, npp_global=4))
    edges = (C.c_double * 5)()
    oracle.load().orc_pbins_edges(C.byref(prm), edges)
    np.testing.assert_allclose(list(edges), [0.1, 1.0, 10.0, 100.0, 1000.0], rtol=1e-14)
    a = _parts(6, p=[0.1, 0.5, 5.0, 50.0, 999.0, 1000.0], weight=[1, 0.5, 0.25, 1, 1, 0.125])
    f, c = oracle.histogram(prm, oracle.Particles(6, a))
    # p == pmin is excluded (p > pmin).  p == pmax passes the range test but
    # its index is npp + 1, one past fglobal's last bin (diagnostics.f90:
    # 775-780 writes out of bounds there); it is dropped here.
    assert list(c) == [1, 1, 1, 1]
    assert list(f) == [0.5, 0.25, 1.0, 1.0]


def _long_push_case():
    """kappa 1000 at a fixed dt of dt_out / 20 on the unit periodic box:
    the diffusion steps are about 1.4 box lengths (rms per axis), so most
    pushes land more than one period away."""
    n = 32
    cfg = make_mhd_config(n, n, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.02)
    prm = make_params(ndim=2, p0=0.1, pmin=0.1, pmax=100.0, kpara0=1000.0, kret=0.1,
                      dt_min_rel=0.05, dt_max_rel=0.05, pbcx=0, pbcy=0, momentum_dependency=0,
                      nptl_max=2000, seed=3)
    frame = fields.planar_shock_2d(n, n, 0.0, 1.0, 0.0, 1.0, u1=1.0, r=3.0, w=0.05)
    return prm, cfg, frame


def test_pushes_longer_than_a_period_stay_in_the_box():
    """particle_boundary_condition wraps by one period; a longer push then
    leaves the particle outside, where the reference indexes outside its
    arrays.  The oracle (and the engine) wrap by whole periods more: every
    particle stays in the periodic box with its flag, and each moved its 20
    pushes (one interval at dt = dt_out / 20)."""
    prm, cfg, frame = _long_push_case()
    oprm = oracle.params_from(prm)
    parts = oracle.Particles(2000)
    cnt = oracle.OrcCounters()
    oracle.inject_spatial_uniform(oprm, parts, 1000, 1e-3, 1, 1.0, 0.0, 0.0,
                                  (0.0, 0.0, 0.0, 1.0, 1.0, 1.0), cnt)
    oracle.mover(oprm, oracle.config_from(cfg), oracle.full_fields(frame, 2, cfg), parts, 0.0,
                 0.02, counters=cnt)
    v = parts.view()
    assert parts.n == 1000 and (v["count_flag"] == 1).all()
    assert v["x"].min() >= 0.0 and v["x"].max() <= 1.0
    assert v["y"].min() >= 0.0 and v["y"].max() <= 1.0
    assert 20 * 1000 <= cnt.steps <= 21 * 1000


def test_pushes_longer_than_a_period_stay_in_the_box_3d():
    """The same in 3D, where the wrap acts on z too: κ 1000 at dt = dt_out / 20
    on a periodic unit cube with a turbulent frame."""
    n = 16
    cfg = make_mhd_config(n, n, n, 0.0, 1.0, 0.0, 1.0, zmin=0.0, zmax=1.0, dt_out=0.02, ndim=3)
    prm = make_params(ndim=3, p0=0.1, pmin=0.1, pmax=100.0, kpara0=1000.0, kret=0.1,
                      dt_min_rel=0.05, dt_max_rel=0.05, pbcx=0, pbcy=0, pbcz=0,
                      momentum_dependency=0, nptl_max=1000, seed=5)
    frame = fields.turbulence_3d(n, seed=7)
    oprm = oracle.params_from(prm)
    parts = oracle.Particles(1000)
    cnt = oracle.OrcCounters()
    oracle.inject_spatial_uniform(oprm, parts, 500, 1e-3, 1, 1.0, 0.0, 0.0,
                                  (0.0, 0.0, 0.0, 1.0, 1.0, 1.0), cnt)
    oracle.mover(oprm, oracle.config_from(cfg), oracle.full_fields(frame, 3, cfg), parts, 0.0,
                 0.02, counters=cnt)
    v = parts.view()
    assert parts.n == 500 and (v["count_flag"] == 1).all()
    for k in ("x", "y", "z"):
        assert v[k].min() >= 0.0 and v[k].max() <= 1.0, k
    assert 20 * 500 <= cnt.steps <= 21 * 500
