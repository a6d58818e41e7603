"""1D runs in the CPU oracle (no GPU), pinned by answers that follow from
push_particle_1d / push_particle_1d_ft (particle_module.f90:2993-3357):
discrete compression with no diffusion, the variance 2 kpara t of pure
diffusion, <r^2> - r0^2 = 6 kappa t of radial diffusion in spherical
coordinates, and streaming at v mu in focused transport."""
import math

import numpy as np

import oracle
from gpat import fields
from gpat.engine import make_mhd_config, make_params

N = 64


def _frame(vx, bx=1.0):
    shape = (1, 1, N + 4)
    z = np.zeros(shape)
    return fields.assemble_frame(np.broadcast_to(vx, shape), z, z, z + 1.0, z + bx, z,
                                 z).astype(np.float32)


def _start(n, x, p=0.1, v=0.0, mu=0.0):
    a = {k: np.zeros(n, dtype=t) for k, t in oracle.FIELDS}
    a["weight"][:] = 1.0
    a["count_flag"][:] = 1
    a["tag_splitted"][:] = 1
    a["tag_injected"][:] = np.arange(n, dtype=np.int32)
    a["x"][:], a["y"][:], a["p"][:], a["v"][:], a["mu"][:] = x, 0.5, p, v, mu
    return a


def _run(prm, cfg, frame, a, dtf, **kw):
    full = oracle.full_fields(frame, 1, cfg)
    parts = oracle.Particles(len(a["x"]), a)
    oracle.mover(oracle.params_from(prm), oracle.config_from(cfg), full, parts, 0.0, dtf, **kw)
    out = parts.view()
    order = np.argsort(out["tag_injected"])
    return {k: v[order] for k, v in out.items()}


def test_1d_gradients_and_interpolation_layout():
    cfg = make_mhd_config(N, 1, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.1, ndim=1)
    x = fields.node_coords(N, 0.0, 1.0 / N)
    full = oracle.full_fields(_frame(0.5 - 0.25 * x), 1, cfg)
    assert full.shape == (1, 1, N + 4, 32)
    np.testing.assert_allclose(full[0, 0, :, 8], -0.25, atol=1e-6)
    assert np.all(full[0, 0, :, 9] == 0.0) and np.all(full[0, 0, :, 10] == 0.0)


def test_1d_compression_discrete_solution():
    cfg = make_mhd_config(N, 1, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.1, ndim=1)
    x = fields.node_coords(N, 0.0, 1.0 / N)
    a_ = 0.5
    prm = make_params(ndim=1, p0=0.1, pmin=0.05, pmax=10.0, kpara0=0.0, kret=0.1,
                      momentum_dependency=0, dt_min_rel=1e-2, dt_max_rel=1e-2, pbcx=1)
    x0 = np.linspace(0.3, 0.7, 9)
    out = _run(prm, cfg, _frame(-a_ * x), _start(9, x0), 0.1)
    np.testing.assert_allclose(out["x"], x0 * (1 - a_ * 1e-3) ** 100, rtol=1e-6)
    np.testing.assert_allclose(out["p"], 0.1 * (1 + a_ * 1e-3 / 3) ** 100, rtol=1e-12)


def test_1d_pure_diffusion_variance():
    cfg = make_mhd_config(N, 1, 1, 0.0, 1.0, 0.0, 1.0, dt_out=1.0, ndim=1)
    kpara = 2e-4
    prm = make_params(ndim=1, p0=0.1, pmin=0.05, pmax=10.0, kpara0=kpara, kret=0.1,
                      momentum_dependency=0, dt_min_rel=1e-3, dt_max_rel=0.05, pbcx=1)
    M = 40000
    out = _run(prm, cfg, _frame(0.0), _start(M, 0.5), 1.0)
    d = out["x"] - 0.5
    assert abs(np.mean(d)) < 6 * math.sqrt(2 * kpara / M)
    assert abs(np.var(d) - 2 * kpara) < 6 * 2 * kpara * math.sqrt(2.0 / M)


def test_1d_spherical_radial_diffusion():
    cfg = make_mhd_config(N, 1, 1, 0.5, 1.5, 0.0, 1.0, dt_out=0.5, ndim=1)
    oracle.set_grid_positions(oracle.uniform_grid_positions(N + 4, 1.0 / N, 0.5))
    kap = 2e-3
    prm = make_params(ndim=1, p0=0.1, pmin=0.05, pmax=10.0, kpara0=kap, kret=0.1,
                      momentum_dependency=0, dt_min_rel=1e-3, dt_max_rel=2e-2, pbcx=1,
                      spherical_coord=1)
    M = 40000
    out = _run(prm, cfg, _frame(0.0), _start(M, 1.0), 0.5)
    oracle.set_grid_positions(None)
    r = out["x"]
    msd = np.mean(r * r) - 1.0
    se = np.std(r * r) / math.sqrt(M)
    assert abs(msd - 6 * kap * 0.5) < 5 * se + 0.03 * 6 * kap * 0.5, msd


def test_1d_focused_transport_streaming():
    cfg = make_mhd_config(N, 1, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.1, ndim=1)
    prm = make_params(ndim=1, p0=0.1, pmin=0.05, pmax=10.0, kpara0=0.0, kret=0.1,
                      momentum_dependency=0, dt_min_rel=1e-2, dt_max_rel=1e-2, pbcx=1,
                      duu0=0.0)
    mu = np.linspace(-0.9, 0.9, 7)
    a = _start(7, 0.5, v=1.5, mu=mu)
    out = _run(prm, cfg, _frame(0.0), a, 0.1, focused_transport=True)
    np.testing.assert_allclose(out["x"], 0.5 + 1.5 * mu * 0.1, rtol=1e-12, atol=1e-13)
    assert np.array_equal(out["mu"], mu) and np.all(out["p"] == 0.1)
