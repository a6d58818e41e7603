"""Spatially dependent turbulence variance and correlation length
(deltab_flag, correlation_flag): the CUDA FP64 mover and db2 injection
against the oracle, through the C ABI.  Variance alone divides kappa (no
pow()) and is bit-exact; the correlation length enters through pow() and is
checked at 1e-9 relative on >= 99.5 % of the particles."""
import numpy as np
import pytest

import oracle
from gpat import fields
from gpat.engine import Engine, make_mhd_config, make_params
from test_gpu_focused import FT_STATE, _same
from test_gpu_parity import STATE, shock_case, turbulent_frame_2d

pytestmark = pytest.mark.gpu

BOX = (0.0, 0.0, 0.0, 1.0, 1.0, 1.0)


def _smooth(n, seed, lo, hi):
    rng = np.random.default_rng(seed)
    x = fields.node_coords(n, 0.0, 1.0 / n)
    X, Y = np.meshgrid(x, x)
    f = np.zeros_like(X)
    for _ in range(4):
        kx, ky = rng.integers(1, 4, size=2)
        f += np.sin(2 * np.pi * (kx * X + ky * Y) + rng.uniform(0, 2 * np.pi))
    f = (f - f.min()) / (f.max() - f.min())
    return (lo + (hi - lo) * f)[None].astype(np.float32)


def _run(params, frame, arrays, intervals=2, mover_kw=None, inject=None):
    mover_kw = mover_kw or {}
    n = 64
    cfg = make_mhd_config(n, n, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.02)
    prm = make_params(**params)
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps(np.arange(intervals + 1) * 0.02)
    eng.set_fields(frame, 0)
    eng.calc_fields_gradients(0)
    eng.set_fluctuations(0, *arrays)
    (inject or (lambda e: e.inject_particles_spatial_uniform(2000, 1e-6, 1, 1.0, 1, BOX)))(eng)
    start = eng.get_particles()
    aux = oracle.aux_fields(*arrays, 2, cfg)
    assert np.array_equal(eng.get_fluctuations(0), aux)
    oprm = oracle.params_from(prm)
    parts = oracle.Particles(prm.nptl_max, start.arrays)
    cnt = oracle.OrcCounters()
    full = oracle.full_fields(frame, 2, cfg)
    for k in range(intervals):
        eng.particle_mover(mhd_tframe=k + 1, **mover_kw)
        oracle.mover(oprm, oracle.config_from(cfg), full, parts, 0.02 * k, 0.02, counters=cnt,
                     aux1=aux, **mover_kw)
    from gpat.engine import ParticleSet
    return eng, eng.get_particles(), ParticleSet(parts.view())


def test_variance_bit_exact():
    params, _ = shock_case(deltab_flag=1, pbcx=0)
    arrays = (_smooth(64, 1, 0.5, 2.0), None, None, None)
    eng, gpu, ref = _run(params, turbulent_frame_2d(), arrays)
    _same(gpu, ref, STATE)
    eng.close()


def test_variance_and_correlation_length_nlgc():
    params, _ = shock_case(deltab_flag=1, correlation_flag=1, pbcx=0)
    arrays = (_smooth(64, 1, 0.5, 2.0), _smooth(64, 2, 0.3, 1.0), _smooth(64, 3, 0.5, 1.5),
              _smooth(64, 4, 0.5, 1.5))
    for kw in ({}, dict(nlgc=True, kperp_kpara=0.05)):
        eng, gpu, ref = _run(params, turbulent_frame_2d(), arrays, mover_kw=kw)
        _same(gpu, ref, STATE, exact=False)
        eng.close()


def test_variance_with_focused_transport_bit_exact():
    params, _ = shock_case(deltab_flag=1, duu0=0.0, pbcx=0, pbcy=0)
    arrays = (_smooth(64, 5, 0.5, 2.0), None, None, None)
    eng, gpu, ref = _run(params, turbulent_frame_2d(), arrays,
                         mover_kw=dict(focused_transport=True),
                         inject=lambda e: e.inject_particles_at_x(1500, 0.5, 1e-6, 1, 2.0, 1))
    _same(gpu, ref, FT_STATE)
    eng.close()


def test_db2_injection_bit_exact(tmp_path):
    n = 64
    cfg = make_mhd_config(n, n, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.1)
    prm = make_params(ndim=2, p0=0.1, pmin=0.01, pmax=10.0, nptl_max=20000, seed=23,
                      deltab_flag=1)
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps([0.0, 0.1, 0.2])
    frame = turbulent_frame_2d()
    eng.set_fields(frame, 0)
    eng.calc_fields_gradients(0)
    db2, db2d = _smooth(64, 7, 0.1, 1.0), _smooth(64, 8, 0.2, 0.6)
    path = tmp_path / "deltab_0000"
    with open(path, "wb") as f:
        f.write(db2.tobytes())
        f.write(db2d.tobytes())
    eng.read_magnetic_fluctuation(path, 0)
    aux = oracle.aux_fields(db2, db2d, None, None, 2, cfg)
    assert np.array_equal(eng.get_fluctuations(0), aux)
    full = oracle.full_fields(frame, 2, cfg)
    oprm, ocfg = oracle.params_from(prm), oracle.config_from(cfg)
    box = (0.1, 0.2, 0.0, 0.9, 0.8, 1.0)
    for thr in (0.5, 0.8):
        assert eng.count_cells_large(4, thr, box) == \
            oracle.count_cells_large(oprm, ocfg, full, 4, thr, box, aux=aux)
    n_inj = eng.inject_particles_at_large(4, 3000, 1e-6, 1, 1.0, 1, False, 0.6, 800, box)
    parts = oracle.Particles(20000)
    cnt = oracle.OrcCounters()
    oracle.inject_at_large(oprm, ocfg, full, parts, n_inj, 1e-6, 1, 1.0, 0.0, 0.1, 4, 0.6, box,
                           cnt, aux=aux)
    got, ref = eng.get_particles(), parts.view()
    assert len(got) == parts.n == n_inj > 0
    for k in ("x", "y", "z", "p", "mu", "t", "tag_injected"):
        assert np.array_equal(got[k], ref[k]), k
    eng.close()
