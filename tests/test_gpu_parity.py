"""Parity of the CUDA engine with the CPU oracle, through the C ABI.

Bit-exact for the FP64 mover wherever the path has no library transcendental
(fields, gradients, drift, noise, landing, boundaries, removal, splitting,
histograms, fixed-point sums).  With momentum-dependent kappa the path calls
pow(), whose last bit may differ between libm and CUDA: those cases use a
per-particle relative tolerance of 1e-12 on >= 99.9 % of the particles.
The split-precision mover is checked statistically against the FP64 mover.
"""
import math

import numpy as np
import pytest

import oracle
from gpat import configs, fields
from gpat.engine import (Engine, GPATCapacityError, GPATError, ParticleSet, make_mhd_config,
                         make_params)

pytestmark = pytest.mark.gpu

STATE = ("x", "y", "z", "p", "t", "dt", "weight", "count_flag", "split_times", "nsteps_pushed",
         "tag_injected", "tag_splitted", "rng_ctr")


def turbulent_frame_2d(n=64, seed=5, r=3.0, w=0.02):
    db = fields.kolmogorov_az_2d(n, n, 1.0, 1.0, 0.5, 2 * np.pi, 16 * np.pi, seed)
    return fields.planar_shock_2d(n, n, 0.0, 1.0, 0.0, 1.0, u1=1.0, r=r, w=w, x0=0.5, db=db)


def run_pair(params_kw, cfg, frame, tstamps, inject, intervals=1, fine=1, frame2=None,
             split=None, nthreads=0, mover_kw=None):
    """Runs the engine and the oracle from the same injected particles;
    mover_kw holds particle_mover's focused_transport / nlgc / kperp_kpara."""
    mover_kw = mover_kw or {}
    prm = make_params(**params_kw)
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps(tstamps)
    eng.set_fields(frame, 0)
    eng.calc_fields_gradients(0)
    if frame2 is not None:
        eng.set_fields(frame2, 1)
        eng.calc_fields_gradients(1)
    inject(eng)
    start = eng.get_particles()
    oprm = oracle.params_from(prm)
    ocfg = oracle.config_from(cfg)
    f1 = oracle.full_fields(frame, prm.ndim, cfg)
    f2 = oracle.full_fields(frame2, prm.ndim, cfg) if frame2 is not None else None
    parts = oracle.Particles(prm.nptl_max, start.arrays)
    cnt = oracle.OrcCounters()
    for k in range(intervals):
        eng.particle_mover(nsteps_interval=10, mhd_tframe=k + 1, num_fine_steps=fine, **mover_kw)
        oracle.mover(oprm, ocfg, f1, parts, float(tstamps[k]), float(tstamps[k + 1] - tstamps[k]),
                     num_fine_steps=fine, counters=cnt, f2=f2, nthreads=nthreads, **mover_kw)
        if split:
            eng.split_particle(*split)
            oracle.split(oprm, parts, split[0], split[1], cnt)
    gpu = eng.get_particles()
    ref = ParticleSet(parts.view())
    return eng, gpu, ref, cnt, oprm


def assert_same_set(gpu, ref, exact=True, rtol=1e-12, frac=0.999):
    g, r = gpu.order_by_tags(), ref.order_by_tags()
    assert len(g) == len(r)
    for k in ("tag_injected", "tag_splitted", "count_flag", "split_times"):
        assert np.array_equal(g[k], r[k]), k
    if exact:
        for k in STATE:
            assert np.array_equal(g[k], r[k]), f"{k} differs"
    else:
        ok = np.ones(len(g), bool)
        for k in ("x", "y", "z", "p", "t"):
            ok &= np.isclose(g[k], r[k], rtol=rtol, atol=rtol * 1e-3)
        assert ok.mean() >= frac, f"only {ok.mean():.5f} of particles within {rtol}"


def shock_case(n=64, ndim=2, **kw):
    cfg = make_mhd_config(n, n, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.02)
    base = dict(ndim=2, p0=0.1, pmin=0.1, pmax=100.0, kpara0=3e-3, kret=0.1, dt_min_rel=2e-3,
                dt_max_rel=5e-2, pbcx=1, pbcy=0, momentum_dependency=0, nptl_max=4000, seed=11)
    base.update(kw)
    return base, cfg


def test_gradients_bit_exact_2d():
    params, cfg = shock_case()
    frame = turbulent_frame_2d()
    eng = Engine(make_params(**params), cfg, 0)
    eng.set_fields(frame, 0)
    eng.calc_fields_gradients(0)
    got = eng.get_fields(0)
    ref = oracle.full_fields(frame, 2, cfg)
    assert np.array_equal(got, ref)


def test_gradients_bit_exact_3d():
    n = 24
    cfg = make_mhd_config(n, n, n, 0.0, 1.0, 0.0, 1.0, zmin=0.0, zmax=1.0, ndim=3)
    frame = fields.turbulence_3d(n, seed=4)
    eng = Engine(make_params(ndim=3, nptl_max=16), cfg, 0)
    eng.set_fields(frame, 0)
    eng.calc_fields_gradients(0)
    assert np.array_equal(eng.get_fields(0), oracle.full_fields(frame, 3, cfg))


def test_injection_bit_exact():
    params, cfg = shock_case(pmax=10.0)
    eng = Engine(make_params(**params), cfg, 0)
    eng.set_tstamps([0.0, 0.02, 0.04])
    eng.inject_particles_at_x(500, 0.5, 1e-6, 1, 2.0, 1)
    eng.inject_particles_at_x(300, 0.25, 1e-6, 2, 2.0, 2, power_index=3.5)
    box = (0.1, 0.2, 0.0, 0.9, 0.8, 1.0)
    eng.inject_particles_spatial_uniform(400, 1e-6, 2, 2.0, 1, box, power_index=1.0)
    eng.inject_particles_spatial_uniform(200, 1e-6, 1, 2.0, 2, box)
    got = eng.get_particles()
    prm = oracle.params_from(eng.params)
    parts = oracle.Particles(4000)
    cnt = oracle.OrcCounters()
    ocfg = oracle.config_from(cfg)
    oracle.inject_at_x(prm, ocfg, parts, 500, 0.5, 1e-6, 1, 2.0, 0.0, cnt)
    oracle.inject_at_x(prm, ocfg, parts, 300, 0.25, 1e-6, 2, 2.0, 0.02, cnt, power_index=3.5)
    oracle.inject_spatial_uniform(prm, parts, 400, 1e-6, 2, 2.0, 0.0, 0.02, box, cnt,
                                  power_index=1.0)
    oracle.inject_spatial_uniform(prm, parts, 200, 1e-6, 1, 2.0, 0.02, 0.02, box, cnt)
    ref = parts.view()
    assert len(got) == parts.n == 1400
    for k in ("x", "y", "z", "mu", "t", "dt", "weight", "tag_injected", "tag_splitted"):
        assert np.array_equal(got[k], ref[k]), k
    # power-law momenta go through pow(): allow the last bit
    np.testing.assert_allclose(got["p"], ref["p"], rtol=2e-15)
    np.testing.assert_allclose(got["v"], ref["v"], rtol=2e-15)


def test_mover_fp64_drift_only_bit_exact():
    params, cfg = shock_case(kpara0=0.0)
    frame = turbulent_frame_2d()
    ts = np.arange(4) * 0.02
    eng, gpu, ref, cnt, _ = run_pair(params, cfg, frame, ts,
                                     lambda e: e.inject_particles_at_x(1000, 0.5, 1e-6, 1, 1.0, 1),
                                     intervals=3)
    assert_same_set(gpu, ref)
    assert eng.counters().steps == cnt.steps


def test_mover_fp64_diffusion_bit_exact_2d():
    params, cfg = shock_case()
    frame = turbulent_frame_2d()
    ts = np.arange(4) * 0.02
    eng, gpu, ref, cnt, _ = run_pair(params, cfg, frame, ts,
                                     lambda e: e.inject_particles_at_x(2000, 0.5, 1e-6, 1, 1.0, 1),
                                     intervals=3, fine=4)
    assert_same_set(gpu, ref)
    c = eng.counters()
    assert c.steps == cnt.steps
    assert (c.leak_hi, c.leak_lo) == (cnt.leak_hi, cnt.leak_lo)
    assert c.nptl_escaped == cnt.nptl_escaped


def test_mover_fp64_random_start_times_and_landing():
    params, cfg = shock_case(pbcx=0)
    frame = turbulent_frame_2d()
    ts = np.arange(3) * 0.02
    box = (0.0, 0.0, 0.0, 1.0, 1.0, 1.0)
    eng, gpu, ref, cnt, _ = run_pair(
        params, cfg, frame, ts,
        lambda e: e.inject_particles_spatial_uniform(2000, 1e-6, 1, 1.0, 1, box), intervals=2,
        fine=5)
    assert_same_set(gpu, ref)


def test_mover_fp64_momentum_dependent_kappa():
    params, cfg = shock_case(momentum_dependency=1, kpara0=1e-3)
    frame = turbulent_frame_2d()
    ts = np.arange(3) * 0.02
    eng, gpu, ref, cnt, _ = run_pair(params, cfg, frame, ts,
                                     lambda e: e.inject_particles_at_x(2000, 0.5, 1e-6, 1, 1.0, 1),
                                     intervals=2)
    assert_same_set(gpu, ref, exact=False, rtol=1e-12, frac=0.999)


def test_mover_fp64_time_interpolation():
    params, cfg = shock_case(time_interp=1)
    f1 = turbulent_frame_2d(seed=5)
    f2 = turbulent_frame_2d(seed=6)
    ts = np.arange(2) * 0.02
    eng, gpu, ref, cnt, _ = run_pair(params, cfg, f1, ts,
                                     lambda e: e.inject_particles_at_x(1000, 0.5, 1e-6, 1, 1.0, 1),
                                     frame2=f2)
    assert_same_set(gpu, ref)


def test_mover_fp64_acceleration_region():
    params, cfg = shock_case(acc_region_flag=1, acc_region=(0.0, 0.5, 0.0, 0.5, 0.0, 1.0))
    frame = turbulent_frame_2d()
    ts = np.arange(2) * 0.02
    eng, gpu, ref, cnt, _ = run_pair(params, cfg, frame, ts,
                                     lambda e: e.inject_particles_at_x(1000, 0.5, 1e-6, 1, 1.0, 1))
    assert_same_set(gpu, ref)


def test_mover_fp64_3d_bit_exact():
    n = 24
    cfg = make_mhd_config(n, n, n, 0.0, 1.0, 0.0, 1.0, zmin=0.0, zmax=1.0, dt_out=0.02, ndim=3)
    frame = fields.turbulence_3d(n, seed=8)
    params = dict(ndim=3, p0=0.1, pmin=0.1, pmax=100.0, kpara0=2e-3, kret=0.05, dt_min_rel=5e-3,
                  dt_max_rel=5e-2, pbcx=0, pbcy=0, pbcz=1, momentum_dependency=0, nptl_max=3000,
                  seed=21)
    box = (0.0, 0.0, 0.0, 1.0, 1.0, 1.0)
    ts = np.arange(3) * 0.02
    eng, gpu, ref, cnt, _ = run_pair(
        params, cfg, frame, ts,
        lambda e: e.inject_particles_spatial_uniform(1500, 1e-6, 1, 1.0, 1, box), intervals=2,
        fine=2)
    assert_same_set(gpu, ref)
    c = eng.counters()
    assert (c.leak_hi, c.leak_lo) == (cnt.leak_hi, cnt.leak_lo)


def test_split_and_histogram_exact():
    params, cfg = shock_case(kpara0=5e-3, pmax=1.0, npp_global=64, nptl_max=200000)
    frame = turbulent_frame_2d(r=4.0)
    ts = np.arange(5) * 0.02
    eng, gpu, ref, cnt, oprm = run_pair(
        params, cfg, frame, ts, lambda e: e.inject_particles_at_x(3000, 0.5, 1e-6, 1, 1.0, 1),
        intervals=4, split=(1.2, 1.05, 10))
    assert_same_set(gpu, ref)
    assert eng.counters().nptl_split == cnt.nptl_split > 0
    f_gpu, c_gpu = eng.calc_particle_distributions()
    parts = oracle.Particles(len(gpu) + 1, gpu.arrays)
    f_ref, c_ref = oracle.histogram(oprm, parts)
    assert np.array_equal(c_gpu, c_ref)
    assert np.array_equal(f_gpu, f_ref)
    np.testing.assert_allclose(eng.pbins_edges(), np.logspace(-1, 0, 65), rtol=1e-13)
    qc = eng.quick_check()
    s = oracle.quick_check(parts)
    assert qc["ntot"] == s[0] and qc["pdt_min"] == s[1] and qc["pdt_max"] == s[2]
    assert qc["pdt_avg"] == pytest.approx(s[3] / len(gpu), rel=1e-12)


def test_split_capacity_matches_reference_stop():
    params, cfg = shock_case(kpara0=5e-3, pmax=1.0, nptl_max=1100)
    frame = turbulent_frame_2d(r=4.0)
    prm = make_params(**params)
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps([0.0, 0.02])
    eng.set_fields(frame, 0)
    eng.calc_fields_gradients(0)
    eng.inject_particles_at_x(1000, 0.5, 1e-6, 1, 1.0, 1)
    ps = eng.get_particles()
    ps.arrays["p"][:] = np.linspace(0.05, 0.5, 1000)      # 700+ candidates
    eng.put_particles(ps)
    with pytest.raises(GPATCapacityError):
        eng.split_particle(1.5, 1.5, 10)
    parts = oracle.Particles(1100, ps.arrays)
    cnt = oracle.OrcCounters()
    oracle.split(oracle.params_from(prm), parts, 1.5, 1.5, cnt)
    got = eng.get_particles()
    assert len(got) == parts.n == 1100
    for k in STATE:
        assert np.array_equal(got[k], parts.view()[k]), k


def test_mixed_precision_diffusion_statistics():
    """Split-precision mover: covariance 2 kappa t in a uniform oblique B."""
    n = 64
    cfg = make_mhd_config(n, n, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.05)
    th = math.radians(35.0)
    z = np.zeros((n + 4, n + 4))
    frame = fields.assemble_frame(z, z, z, z + 1, z + math.cos(th), z + math.sin(th), z)[None]
    kpara, kret, T = 1e-3, 0.1, 0.05
    prm = make_params(ndim=2, kpara0=kpara, kret=kret, momentum_dependency=0, dt_min_rel=0.01,
                      pbcx=0, pbcy=0, p0=0.1, precision=1, nptl_max=200000, seed=3)
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps([0.0, T])
    eng.set_fields(frame, 0)
    eng.calc_fields_gradients(0)
    N = 200000
    ps = ParticleSet.empty(N)
    ps.arrays["x"][:] = 0.5
    ps.arrays["y"][:] = 0.5
    ps.arrays["p"][:] = 0.1
    ps.arrays["weight"][:] = 1.0
    ps.arrays["count_flag"][:] = 1
    ps.arrays["tag_splitted"][:] = 1
    ps.arrays["tag_injected"][:] = np.arange(N, dtype=np.int32)
    eng.put_particles(ps)
    eng.particle_mover(mhd_tframe=1)
    out = eng.get_particles()
    d = np.stack([out["x"] - 0.5, out["y"] - 0.5])
    cov = d @ d.T / N
    b = np.array([math.cos(th), math.sin(th)])
    K = kpara * kret * np.eye(2) + kpara * (1 - kret) * np.outer(b, b)
    np.testing.assert_allclose(cov, 2 * K * T, atol=5 * math.sqrt(2.0 / N) * 2 * K.max() * T)
    np.testing.assert_allclose(out["t"], T, rtol=1e-12)


def test_mixed_vs_fp64_spectrum_shock():
    """f(p) of the split-precision mover agrees with the FP64 mover on a
    small planar shock (same injection, independent noise) within Monte
    Carlo error bin by bin (chi-square at 99.9 % confidence)."""
    w = configs.planar_shock(scale=0.2, dt_out=0.1, dt_min=2e-4)
    hists = {}
    for prec in (0, 1):
        eng = configs.build_engine(w, precision=prec, nptl_max=w.nptl * 4, npp_global=32)
        configs.inject(eng, w)
        for k in range(5):
            eng.particle_mover(mhd_tframe=k + 1)
        f, c = eng.calc_particle_distributions()
        hists[prec] = c.astype(float)
        eng.close()
    a, b = hists[0], hists[1]
    m = (a + b) > 20
    chi2 = float(np.sum((a[m] - b[m]) ** 2 / (a[m] + b[m])))
    dof = int(m.sum())
    # 99.9 % quantile of chi2 ~ dof + 3.1 sqrt(2 dof) for moderate dof
    assert chi2 < dof + 3.1 * math.sqrt(2 * dof) + 10, (chi2, dof)


def test_status_and_errors():
    params, cfg = shock_case()
    eng = Engine(make_params(**params), cfg, 0)
    eng.set_tstamps([0.0, 0.02])
    with pytest.raises(GPATError):            # no fields yet
        eng.particle_mover(mhd_tframe=1)
    with pytest.raises(GPATError):            # focused transport is out of scope
        eng.particle_mover(focused_transport=True, mhd_tframe=1)
    with pytest.raises(GPATCapacityError):
        eng.inject_particles_at_x(params["nptl_max"] + 5, 0.5, 1e-6, 1, 1.0, 1)
    assert eng.counters().nptl_current == params["nptl_max"]


def test_pushes_longer_than_a_period_match_oracle():
    """kappa 1000 at a fixed dt of dt_out / 20 on the unit periodic box: most
    pushes land more than one period away, and the one-period wrap of
    particle_boundary_condition is followed by whole periods more (where the
    reference would index outside its arrays).  The FP64 mover matches the
    oracle bit for bit; the split-precision mover keeps every particle in
    the box too."""
    n = 32
    cfg = make_mhd_config(n, n, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.02)
    kw = dict(ndim=2, p0=0.1, pmin=0.1, pmax=100.0, kpara0=1000.0, kret=0.1, dt_min_rel=0.05,
              dt_max_rel=0.05, pbcx=0, pbcy=0, momentum_dependency=0, nptl_max=2000, seed=3)
    frame = fields.planar_shock_2d(n, n, 0.0, 1.0, 0.0, 1.0, u1=1.0, r=3.0, w=0.05)
    box = (0.0, 0.0, 0.0, 1.0, 1.0, 1.0)

    def inject(e):
        e.inject_particles_spatial_uniform(1000, 1e-3, 1, 1.0, 1, box)

    eng, gpu, ref, cnt, _ = run_pair(kw, cfg, frame, [0.0, 0.02, 0.04], inject, intervals=2)
    assert_same_set(gpu, ref)
    assert len(gpu) == 1000 and (gpu["count_flag"] == 1).all()
    eng.close()
    mixed = Engine(make_params(**dict(kw, precision=1)), cfg, 0)
    mixed.set_tstamps([0.0, 0.02, 0.04])
    mixed.set_fields(frame, 0)
    mixed.calc_fields_gradients(0)
    inject(mixed)
    for k in range(2):
        mixed.particle_mover(nsteps_interval=10, mhd_tframe=k + 1)
    ps = mixed.get_particles()
    assert len(ps) == 1000 and (ps["count_flag"] == 1).all()
    assert 0.0 <= ps["x"].min() and ps["x"].max() <= 1.0
    assert 0.0 <= ps["y"].min() and ps["y"].max() <= 1.0
    mixed.close()
