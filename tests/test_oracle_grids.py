"""Spherical and non-uniform grids in the CPU oracle (no GPU).

Known answers that follow from the reference's own rules
(particle_module.f90, mhd_data_parallel.f90): binarySearch_R's cell count,
idxh_grid gradients that are exact for linear data on a stretched grid,
interpolation weights that reproduce the functions they are linear in
(x, y on a Cartesian grid; r^3 and cos(theta) in spherical coordinates),
the one-step covariance 2 S K S dt of the spherical position noise, mean
square displacement 6 kappa t of isotropic diffusion in 3D spherical
coordinates, and 2 kappa t on a stretched Cartesian grid.
"""
import ctypes as C
import math

import numpy as np
import pytest

import oracle
from gpat import fields
from gpat.engine import make_mhd_config, make_params


def _stretched(n, lo, hi, seed):
    """n + 4 increasing node positions, the interior spanning [lo, hi]
    with uneven spacing and two ghost nodes per side."""
    rng = np.random.default_rng(seed)
    h = rng.uniform(0.5, 1.5, n + 3)
    x = np.concatenate([[0.0], np.cumsum(h)])
    x = lo + (x - x[2]) * (hi - lo) / (x[n + 2] - x[2])
    return x


def test_binary_search_counts_nodes_at_or_below():
    a = np.array([0.0, 0.5, 1.0, 2.0, 4.0])
    assert oracle.binary_search(a, -1.0) == 0
    assert oracle.binary_search(a, 0.0) == 1
    assert oracle.binary_search(a, 0.7) == 2
    assert oracle.binary_search(a, 2.0) == 4
    assert oracle.binary_search(a, 9.0) == 5
    rng = np.random.default_rng(1)
    x = np.sort(rng.uniform(0, 1, 37))
    for v in rng.uniform(-0.1, 1.1, 200):
        assert oracle.binary_search(x, v) == int(np.sum(x <= v))


def test_uniform_positions_formula():
    x = oracle.uniform_grid_positions(9, 0.25, -1.0)
    assert np.array_equal(x, 0.25 * (np.arange(9) - 2.0) - 1.0)


def test_nonuniform_gradients_exact_for_linear_data():
    nx, ny = 24, 12
    X = _stretched(nx, 0.0, 1.0, 3)
    Y = _stretched(ny, 0.0, 0.5, 4)
    oracle.set_grid_positions(X, Y)
    XX, YY = np.meshgrid(X, Y)
    vx = 0.25 + 0.5 * XX - 0.75 * YY
    z = np.zeros_like(XX)
    frame = fields.assemble_frame(vx, z, z, z + 1.0, z + 1.0, z, z)[None]
    cfg = make_mhd_config(nx, ny, 1, 0.0, 1.0, 0.0, 0.5)
    full = oracle.full_fields(frame.astype(np.float32), 2, cfg, nonuniform=True)
    np.testing.assert_allclose(full[0, :, :, 8], 0.5, rtol=0, atol=1e-4)
    np.testing.assert_allclose(full[0, :, :, 9], -0.75, rtol=0, atol=1e-4)
    assert np.all(full[0, :, :, 10] == 0.0)
    # On uniform positions it agrees with the uniform routine to FP32 rounding.
    U = oracle.uniform_grid_positions(nx + 4, 1.0 / nx, 0.0)
    V = oracle.uniform_grid_positions(ny + 4, 0.5 / ny, 0.0)
    oracle.set_grid_positions(U, V)
    rng = np.random.default_rng(5)
    f8 = rng.normal(size=(1, ny + 4, nx + 4, 8)).astype(np.float32)
    a = oracle.full_fields(f8, 2, cfg, nonuniform=True)
    b = oracle.full_fields(f8, 2, cfg)
    np.testing.assert_allclose(a, b, rtol=1e-6, atol=1e-5)
    oracle.set_grid_positions(None)


def _params(**kw):
    base = dict(ndim=2, p0=0.1, pmin=0.05, pmax=10.0, kpara0=1e-3, kret=0.3,
                momentum_dependency=0, pbcx=1, pbcy=1, pbcz=1)
    base.update(kw)
    return oracle.params_from(make_params(**base))


def test_nonuniform_interp_finds_cell_and_is_bilinear():
    nx, ny = 20, 10
    X = _stretched(nx, 0.0, 1.0, 7)
    Y = _stretched(ny, 0.0, 1.0, 8)
    oracle.set_grid_positions(X, Y)
    prm = _params(nonuniform_grid=1)
    cfg = oracle.config_from(make_mhd_config(nx, ny, 1, 0.0, 1.0, 0.0, 1.0))
    XX, YY = np.meshgrid(X, Y)
    full = np.zeros((1, ny + 4, nx + 4, 32), np.float32)
    full[0, :, :, 0] = 1.0 + 2.0 * XX - 3.0 * YY + 0.5 * XX * YY
    rng = np.random.default_rng(9)
    lib = oracle.load()
    for _ in range(100):
        x, y = rng.uniform(X[1], X[-1]), rng.uniform(Y[1], Y[-1])
        pos, w = oracle.grid_interp_paramters(prm, cfg, x, y, 0.0)
        # the corner is the searched cell (Fortran index = memory - 1)
        assert X[pos[0] + 1] <= x <= X[pos[0] + 2] and Y[pos[1] + 1] <= y <= Y[pos[1] + 2]
        assert abs(w.sum() - 1.0) < 1e-14
        f = (C.c_double * 32)()
        lib.orc_interp_fields(full.ctypes.data_as(C.POINTER(C.c_float)), None, 0, 2, nx + 4,
                              ny + 4, (C.c_int32 * 3)(*pos), (C.c_double * 8)(*w), 0.0, f)
        assert abs(f[0] - (1.0 + 2.0 * x - 3.0 * y + 0.5 * x * y)) < 2e-5
    oracle.set_grid_positions(None)


@pytest.mark.parametrize("ndim", [2, 3])
def test_spherical_weights_linear_in_r3_and_cos_theta(ndim):
    n = 12
    R = _stretched(n, 0.5, 2.0, 11)
    T = _stretched(n, 0.3, math.pi - 0.3, 12)
    Pp = _stretched(n, 0.0, 1.5, 13) if ndim == 3 else None
    oracle.set_grid_positions(R, T, Pp)
    prm = _params(ndim=ndim, spherical_coord=1, nonuniform_grid=1)
    cfg = oracle.config_from(make_mhd_config(n, n, n if ndim == 3 else 1, 0.5, 2.0, 0.3,
                                             math.pi - 0.3, zmin=0.0, zmax=1.5, ndim=ndim))
    nz = n + 4 if ndim == 3 else 1
    PH = Pp if ndim == 3 else np.zeros(1)
    ZZ, YY, XX = np.meshgrid(PH, T, R, indexing="ij")

    def fn(r, t, ph):
        return 1.0 + 0.3 * r ** 3 - 0.7 * np.cos(t) + 0.2 * r ** 3 * np.cos(t) + 0.4 * ph

    full = np.zeros((nz, n + 4, n + 4, 32), np.float32)
    full[..., 0] = fn(XX, YY, ZZ if ndim == 3 else 0.0)
    rng = np.random.default_rng(14)
    lib = oracle.load()
    for _ in range(100):
        r, t = rng.uniform(R[1], R[-1]), rng.uniform(T[1], T[-1])
        ph = rng.uniform(Pp[1], Pp[-1]) if ndim == 3 else 0.0
        pos, w = oracle.grid_interp_paramters(prm, cfg, r, t, ph)
        assert abs(w.sum() - 1.0) < 1e-12
        f = (C.c_double * 32)()
        lib.orc_interp_fields(full.ctypes.data_as(C.POINTER(C.c_float)), None, 0, ndim,
                              n + 4, n + 4, (C.c_int32 * 3)(*pos), (C.c_double * 8)(*w), 0.0, f)
        assert abs(f[0] - fn(r, t, ph)) < 2e-5 * (1 + abs(fn(r, t, ph)))
    oracle.set_grid_positions(None)


def _uniform_b_frame(nx, ny, nz, b):
    shape = (nz, ny + 4, nx + 4)
    z = np.zeros(shape)
    return fields.assemble_frame(z, z, z, z + 1.0, z + b[0], z + b[1], z + b[2]).astype(np.float32)


def _start(n, x, y, z, p=0.1):
    a = {k: np.zeros(n, dtype=t) for k, t in oracle.FIELDS}
    a["weight"][:] = 1.0
    a["count_flag"][:] = 1
    a["tag_splitted"][:] = 1
    a["tag_injected"][:] = np.arange(n, dtype=np.int32)
    a["x"][:], a["y"][:], a["z"][:], a["p"][:] = x, y, z, p
    return a


def _kappa(prm, b):
    f = (C.c_double * 32)()
    f[4], f[5], f[6] = b
    f[7] = math.sqrt(sum(c * c for c in b))
    k = (C.c_double * 22)()
    oracle.load().orc_calc_spatial_diffusion_coefficients(C.byref(prm), 0.1, 0.0, f, None, k)
    return np.array([[k[7], k[10], k[11]], [k[10], k[8], k[12]], [k[11], k[12], k[9]]])


@pytest.mark.parametrize("ndim", [2, 3])
def test_spherical_one_step_covariance(ndim):
    """One push of fixed dt from a common start: the increments have mean
    (drift) dt and covariance 2 S K S dt, S = diag(1, 1/r, 1/(r sin theta))
    (push_particle_2d :3559-3580, push_particle_3d :4852-4870)."""
    n = 16
    R = oracle.uniform_grid_positions(n + 4, 1.0 / n, 0.5)
    T = oracle.uniform_grid_positions(n + 4, 1.0 / n, 1.0)
    Pp = oracle.uniform_grid_positions(n + 4, 1.0 / n, 0.0) if ndim == 3 else None
    oracle.set_grid_positions(R, T, Pp)
    b = (0.6, 0.8, 0.0) if ndim == 2 else (0.6, 0.5, 0.62)
    dtf = 1e-4
    prm = _params(ndim=ndim, spherical_coord=1, kpara0=1e-3, kret=0.2, dt_min_rel=1.0,
                  dt_max_rel=1.0)
    cfg = make_mhd_config(n, n, n if ndim == 3 else 1, 0.5, 1.5, 1.0, 2.0, zmin=0.0, zmax=1.0,
                          dt_out=dtf, ndim=ndim)
    frame = _uniform_b_frame(n, n, n + 4 if ndim == 3 else 1, b)
    full = oracle.full_fields(frame, ndim, cfg)
    r0, t0, p0 = 1.0, 1.5, 0.5
    N = 200000
    parts = oracle.Particles(N, _start(N, r0, t0, p0 if ndim == 3 else 0.0))
    oracle.mover(prm, oracle.config_from(cfg), full, parts, 0.0, dtf)
    out = parts.view()
    assert len(out["x"]) == N and np.all(out["t"] == dtf)
    D = np.stack([out["x"] - r0, out["y"] - t0] + ([out["z"] - p0] if ndim == 3 else []))
    K = _kappa(prm, b)
    ir, ist = 1.0 / r0, 1.0 / math.sin(t0)
    S = np.diag([1.0, ir, ir * ist])[:ndim, :ndim]
    cov_expect = 2.0 * S @ K[:ndim, :ndim] @ S * dtf
    cov = np.cov(D)
    scale = np.sqrt(np.outer(np.diag(cov_expect), np.diag(cov_expect)))
    assert np.all(np.abs(cov - cov_expect) < 6.0 * scale * math.sqrt(2.0 / N)), (cov, cov_expect)
    # Drift: (2 kxx + kxy cot)/r, (kxy + kyy cot)/r^2 (+ the phi terms in 3D).
    cot = math.cos(t0) / math.sin(t0)
    if ndim == 2:
        drift = [(2 * K[0, 0] + K[0, 1] * cot) * ir, (K[0, 1] + K[1, 1] * cot) * ir * ir]
    else:
        drift = [(2 * K[0, 0] + K[0, 1] * cot) * ir, (K[0, 1] + K[1, 1] * cot) * ir * ir,
                 K[0, 2] * ist * ir * ir]
    mean = D.mean(axis=1)
    for i in range(ndim):
        err = math.sqrt(cov_expect[i, i] / N)
        assert abs(mean[i] - drift[i] * dtf) < 6 * err + 1e-3 * abs(drift[i] * dtf), i
    oracle.set_grid_positions(None)


def test_spherical_3d_isotropic_msd():
    """Isotropic kappa in 3D spherical coordinates: <r^2> - r0^2 = 6 kappa t
    and the mean Cartesian position stays at the start (pure Brownian motion
    written in r, theta, phi)."""
    n = 16
    R = oracle.uniform_grid_positions(n + 4, 1.0 / n, 0.5)
    T = oracle.uniform_grid_positions(n + 4, 1.6 / n, 0.8)
    Pp = oracle.uniform_grid_positions(n + 4, 1.0 / n, 0.0)
    oracle.set_grid_positions(R, T, Pp)
    kap, t_end = 2e-3, 0.5
    prm = _params(ndim=3, spherical_coord=1, kpara0=kap, kret=1.0, dt_min_rel=1e-3,
                  dt_max_rel=2e-2)
    cfg = make_mhd_config(n, n, n, 0.5, 1.5, 0.8, 2.4, zmin=0.0, zmax=1.0, dt_out=t_end, ndim=3)
    frame = _uniform_b_frame(n, n, n + 4, (0.6, 0.0, 0.8))
    full = oracle.full_fields(frame, 3, cfg)
    r0, th0, ph0 = 1.0, 1.6, 0.5
    N = 40000
    parts = oracle.Particles(N, _start(N, r0, th0, ph0))
    oracle.mover(prm, oracle.config_from(cfg), full, parts, 0.0, t_end)
    out = parts.view()
    assert len(out["x"]) == N
    r, th, ph = out["x"], out["y"], out["z"]
    msd = np.mean(r * r) - r0 * r0
    se = np.std(r * r) / math.sqrt(N)
    assert abs(msd - 6 * kap * t_end) < 5 * se + 0.03 * 6 * kap * t_end, (msd, 6 * kap * t_end)
    cart = np.stack([r * np.sin(th) * np.cos(ph), r * np.sin(th) * np.sin(ph), r * np.cos(th)])
    c0 = np.array([math.sin(th0) * math.cos(ph0), math.sin(th0) * math.sin(ph0), math.cos(th0)])
    err = math.sqrt(2 * kap * t_end / N)
    assert np.all(np.abs(cart.mean(axis=1) - c0 * r0) < 6 * err)
    oracle.set_grid_positions(None)


def test_stretched_grid_diffusion_covariance():
    """Uniform oblique B on a non-uniform Cartesian grid: the grid only sets
    the time-step limits, so the covariance after t is 2 K t."""
    nx, ny = 32, 32
    X = _stretched(nx, 0.0, 1.0, 21)
    Y = _stretched(ny, 0.0, 1.0, 22)
    oracle.set_grid_positions(X, Y)
    b = (0.8, 0.6, 0.0)
    prm = _params(nonuniform_grid=1, kpara0=2e-4, kret=0.25, dt_min_rel=1e-3, dt_max_rel=0.05)
    cfg = make_mhd_config(nx, ny, 1, 0.0, 1.0, 0.0, 1.0, dt_out=1.0)
    frame = _uniform_b_frame(nx, ny, 1, b)
    oracle.set_grid_positions(X, Y)
    full = oracle.full_fields(frame, 2, cfg, nonuniform=True)
    N = 40000
    parts = oracle.Particles(N, _start(N, 0.5, 0.5, 0.0))
    oracle.mover(prm, oracle.config_from(cfg), full, parts, 0.0, 1.0)
    out = parts.view()
    D = np.stack([out["x"] - 0.5, out["y"] - 0.5])
    K = _kappa(prm, b)[:2, :2]
    cov = np.cov(D)
    expect = 2 * K * 1.0
    scale = np.sqrt(np.outer(np.diag(expect), np.diag(expect)))
    assert np.all(np.abs(cov - expect) < 6 * scale * math.sqrt(2.0 / N)), (cov, expect)
    oracle.set_grid_positions(None)


def test_spherical_local_distribution_weights():
    n = 8
    cfg = make_mhd_config(n, n, 1, 0.5, 1.5, 0.5, 2.5, dt_out=0.1)
    ocfg = oracle.config_from(cfg)
    rng = np.random.default_rng(31)
    N = 500
    a = _start(N, rng.uniform(0.5, 1.5, N), rng.uniform(0.5, 2.5, N), 0.0,
               p=np.exp(rng.uniform(np.log(0.1), np.log(5.0), N)))
    a["weight"][:] = 0.5 ** rng.integers(0, 4, N)
    parts = oracle.Particles(N, a)
    f, c = oracle.local_distribution(ocfg, 2, parts, 0.1, 10.0, 8, spherical=True)
    g, c2 = oracle.local_distribution(ocfg, 2, parts, 0.1, 10.0, 8)
    assert np.array_equal(c, c2)
    # the same bins, each particle's weight divided by r^2 sin(theta)
    w = a["weight"] / (a["x"] * a["x"]) / np.sin(a["y"])
    ix = np.floor((a["x"] - 0.5) / (1.0 / n)).astype(int)
    iy = np.floor((a["y"] - 0.5) / (2.0 / n)).astype(int)
    ip = np.floor((np.log10(a["p"]) - np.log10(0.1)) / (2.0 / 8)).astype(int) + 1
    ok = (ip > 0) & (ip < 8)
    expect = np.zeros((n, n, 8))
    np.add.at(expect, (iy[ok], ix[ok], ip[ok] - 1), w[ok])
    np.testing.assert_allclose(f.reshape(n, n, 8), expect, rtol=1e-12, atol=1e-15)
