"""Focused transport, NLGC and the 2D out-of-plane drift: CUDA FP64 mover
against the oracle, through the C ABI.

Bit-exact where the path calls no library pow(): NLGC and focused transport
with momentum- and |B|-independent coefficients and duu0 = 0 (D_mumu's
pow() terms are then multiplied by 0).  With pitch-angle scattering on,
calc_duu evaluates |mu|^(gamma-1) and |mu|^(gamma-2) every push, whose
last bit may differ between libm and CUDA: those cases use a per-particle
relative tolerance of 1e-9 on >= 99.5 % of the particles.
"""
import numpy as np
import pytest

from gpat import fields
from gpat.engine import Engine, GPATError, make_mhd_config, make_params
from test_gpu_parity import STATE, run_pair, shock_case, turbulent_frame_2d

pytestmark = pytest.mark.gpu

FT_STATE = STATE + ("v", "mu")


def _same(gpu, ref, keys, exact=True, rtol=1e-9, frac=0.995):
    g, r = gpu.order_by_tags(), ref.order_by_tags()
    assert len(g) == len(r)
    for k in ("tag_injected", "tag_splitted"):
        assert np.array_equal(g[k], r[k]), k
    if exact:
        for k in keys:
            assert np.array_equal(g[k], r[k]), f"{k} differs"
        return
    ok = np.ones(len(g), bool)
    for k in ("x", "y", "z", "p", "v", "mu", "t"):
        ok &= np.isclose(g[k], r[k], rtol=rtol, atol=rtol * 1e-3)
    assert ok.mean() >= frac, f"only {ok.mean():.5f} of particles within {rtol}"
    assert (g["count_flag"] == r["count_flag"]).mean() >= frac


def _inject_shock(n, v0=2.0):
    return lambda e: e.inject_particles_at_x(n, 0.5, 1e-6, 1, v0, 1)


def _cube(n=24, seed=8):
    cfg = make_mhd_config(n, n, n, 0.0, 1.0, 0.0, 1.0, zmin=0.0, zmax=1.0, dt_out=0.02, ndim=3)
    params = dict(ndim=3, p0=0.1, pmin=0.1, pmax=100.0, kpara0=2e-3, kret=0.05, dt_min_rel=5e-3,
                  dt_max_rel=5e-2, pbcx=0, pbcy=0, pbcz=1, momentum_dependency=0, nptl_max=3000,
                  seed=21)
    return cfg, fields.turbulence_3d(n, seed=seed), params


BOX = (0.0, 0.0, 0.0, 1.0, 1.0, 1.0)


def test_focused_transport_2d_without_scattering_bit_exact():
    params, cfg = shock_case(duu0=0.0, pbcx=0, pbcy=0)
    ts = np.arange(4) * 0.02
    eng, gpu, ref, cnt, _ = run_pair(params, cfg, turbulent_frame_2d(), ts, _inject_shock(2000),
                                     intervals=3, fine=2, mover_kw=dict(focused_transport=True))
    _same(gpu, ref, FT_STATE)
    assert eng.counters().steps == cnt.steps
    assert np.any(gpu["mu"] != 0.0) and np.any(gpu["v"] != 2.0)


def test_focused_transport_2d_scattering():
    params, cfg = shock_case(duu0=10.0, pbcx=0, pbcy=0)
    ts = np.arange(3) * 0.02
    eng, gpu, ref, cnt, _ = run_pair(params, cfg, turbulent_frame_2d(), ts, _inject_shock(2000),
                                     intervals=2, mover_kw=dict(focused_transport=True))
    _same(gpu, ref, FT_STATE, exact=False)


def test_focused_transport_2d_check_drift_and_acceleration_region():
    params, cfg = shock_case(duu0=0.0, check_drift_2d=1, acc_region_flag=1,
                             acc_region=(0.0, 0.55, 0.0, 1.0, 0.0, 1.0))
    ts = np.arange(3) * 0.02
    eng, gpu, ref, cnt, _ = run_pair(params, cfg, turbulent_frame_2d(), ts, _inject_shock(1500),
                                     intervals=2, fine=3, mover_kw=dict(focused_transport=True))
    _same(gpu, ref, FT_STATE)
    assert np.any(gpu["z"] != 0.0)


def test_focused_transport_3d_without_scattering_bit_exact():
    cfg, frame, params = _cube()
    params["duu0"] = 0.0
    ts = np.arange(3) * 0.02
    eng, gpu, ref, cnt, _ = run_pair(
        params, cfg, frame, ts, lambda e: e.inject_particles_spatial_uniform(1500, 1e-6, 1, 1.0,
                                                                             1, BOX),
        intervals=2, fine=2, mover_kw=dict(focused_transport=True))
    _same(gpu, ref, FT_STATE)
    c = eng.counters()
    assert (c.leak_hi, c.leak_lo) == (cnt.leak_hi, cnt.leak_lo)


def test_focused_transport_3d_scattering():
    cfg, frame, params = _cube()
    params["duu0"] = 10.0
    ts = np.arange(2) * 0.02
    eng, gpu, ref, cnt, _ = run_pair(
        params, cfg, frame, ts, lambda e: e.inject_particles_spatial_uniform(1500, 1e-6, 1, 1.0,
                                                                             1, BOX),
        mover_kw=dict(focused_transport=True))
    _same(gpu, ref, FT_STATE, exact=False)


def test_nlgc_parker_2d_bit_exact():
    params, cfg = shock_case(pbcx=0)
    ts = np.arange(4) * 0.02
    eng, gpu, ref, cnt, _ = run_pair(
        params, cfg, turbulent_frame_2d(), ts,
        lambda e: e.inject_particles_spatial_uniform(2000, 1e-6, 1, 1.0, 1, BOX), intervals=3,
        fine=2, mover_kw=dict(nlgc=True, kperp_kpara=0.05))
    _same(gpu, ref, STATE)
    assert eng.counters().steps == cnt.steps


def test_nlgc_parker_3d_bit_exact():
    cfg, frame, params = _cube()
    ts = np.arange(3) * 0.02
    eng, gpu, ref, cnt, _ = run_pair(
        params, cfg, frame, ts, lambda e: e.inject_particles_spatial_uniform(1500, 1e-6, 1, 1.0,
                                                                             1, BOX),
        intervals=2, mover_kw=dict(nlgc=True, kperp_kpara=0.05))
    _same(gpu, ref, STATE)


def test_nlgc_focused_transport_momentum_dependent():
    params, cfg = shock_case(duu0=5.0, momentum_dependency=1, mag_dependency=1, kpara0=1e-3)
    ts = np.arange(2) * 0.02
    eng, gpu, ref, cnt, _ = run_pair(params, cfg, turbulent_frame_2d(), ts, _inject_shock(1500),
                                     mover_kw=dict(focused_transport=True, nlgc=True,
                                                   kperp_kpara=0.02))
    _same(gpu, ref, FT_STATE, exact=False)


def test_parker_2d_out_of_plane_drift_bit_exact():
    """push_particle_2d's deltaz is local: an undone landing push keeps its
    out-of-plane drift in z."""
    params, cfg = shock_case(check_drift_2d=1, pbcx=0)
    ts = np.arange(3) * 0.02
    eng, gpu, ref, cnt, _ = run_pair(
        params, cfg, turbulent_frame_2d(), ts,
        lambda e: e.inject_particles_spatial_uniform(2000, 1e-6, 1, 1.0, 1, BOX), intervals=2,
        fine=4)
    _same(gpu, ref, STATE)
    assert np.any(gpu["z"] != 0.0)


def test_focused_transport_needs_fp64():
    params, cfg = shock_case(precision=1)
    eng = Engine(make_params(**params), cfg, 0)
    eng.set_tstamps([0.0, 0.02])
    eng.set_fields(turbulent_frame_2d(), 0)
    eng.calc_fields_gradients(0)
    eng.inject_particles_at_x(100, 0.5, 1e-6, 1, 1.0, 1)
    with pytest.raises(GPATError, match="UNSUPPORTED"):
        eng.particle_mover(focused_transport=True)
    eng.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_nlgc_diffusion_covariance(precision):
    """NLGC kperp = kpara0 kperp_kpara mu^2: two groups of particles with
    different mu spread with covariance 2 K(mu) t in a uniform oblique B."""
    import math
    n = 64
    cfg = make_mhd_config(n, n, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.05)
    th = math.radians(35.0)
    z = np.zeros((n + 4, n + 4))
    frame = fields.assemble_frame(z, z, z, z + 1, z + math.cos(th), z + math.sin(th), z)[None]
    kpara, kk, T = 1e-3, 0.3, 0.05
    N = 100000 if precision else 20000
    prm = make_params(ndim=2, kpara0=kpara, momentum_dependency=0, dt_min_rel=0.01, pbcx=0,
                      pbcy=0, p0=0.1, precision=precision, nptl_max=N, seed=3)
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps([0.0, T])
    eng.set_fields(frame, 0)
    eng.calc_fields_gradients(0)
    from gpat.engine import ParticleSet
    ps = ParticleSet.empty(N)
    a = ps.arrays
    a["x"][:] = 0.5
    a["y"][:] = 0.5
    a["p"][:] = 0.1
    a["weight"][:] = 1.0
    a["count_flag"][:] = 1
    a["tag_splitted"][:] = 1
    a["tag_injected"][:] = np.arange(N, dtype=np.int32)
    a["mu"][:] = np.where(np.arange(N) % 2 == 0, 0.25, 0.9)
    eng.put_particles(ps)
    eng.particle_mover(mhd_tframe=1, nlgc=True, kperp_kpara=kk)
    out = eng.get_particles()
    b = np.array([math.cos(th), math.sin(th)])
    for mu in (0.25, 0.9):
        sel = out["mu"] == mu
        m = int(sel.sum())
        d = np.stack([out["x"][sel] - 0.5, out["y"][sel] - 0.5])
        cov = d @ d.T / m
        kperp = kpara * kk * mu * mu
        K = kperp * np.eye(2) + (kpara - kperp) * np.outer(b, b)
        np.testing.assert_allclose(cov, 2 * K * T, atol=5 * math.sqrt(2.0 / m) * 2 * K.max() * T)
    eng.close()
