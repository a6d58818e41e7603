"""1D runs: the CUDA FP64 mover against the oracle through the C ABI.
Without pow() the trajectories are bit-exact (Cartesian, non-uniform, focused
transport without scattering); spherical runs are checked at 1e-9 relative
on >= 99.5 % of particles."""
import numpy as np
import pytest

import oracle
from gpat import fields
from gpat.engine import Engine, ParticleSet, make_mhd_config, make_params
from test_gpu_focused import FT_STATE, _same
from test_gpu_parity import STATE

pytestmark = pytest.mark.gpu

N = 256


def _stretched(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    h = rng.uniform(0.6, 1.4, n + 3)
    x = np.concatenate([[0.0], np.cumsum(h)])
    return lo + (x - x[2]) * (hi - lo) / (x[n + 2] - x[2])


def _frame(lo, hi):
    x = np.linspace(lo, hi, N + 4)[None, None, :]
    z = np.zeros((1, 1, N + 4))
    vx = 1.0 - 0.6 * (1 + np.tanh((x - 0.5 * (lo + hi)) / 0.02)) / 2
    by = 0.5 + 0.2 * np.sin(2 * np.pi * (x - lo) / (hi - lo))
    return fields.assemble_frame(vx + z, 0.1 * by + z, z, 1.0 + z, 1.0 + z, by + z,
                                 0.3 + z).astype(np.float32)


def _run(spherical=False, nonuniform=False, mover_kw=None, **kw):
    lo, hi = (0.5, 1.5) if spherical else (0.0, 1.0)
    cfg = make_mhd_config(N, 1, 1, lo, hi, 0.0, 1.0, dt_out=0.02, ndim=1)
    frame = _frame(lo, hi)
    base = dict(ndim=1, p0=0.1, pmin=0.05, pmax=100.0, kpara0=2e-3, kret=0.1, dt_min_rel=2e-3,
                dt_max_rel=5e-2, pbcx=1, momentum_dependency=0, nptl_max=6000, seed=61,
                precision=0, spherical_coord=int(spherical), nonuniform_grid=int(nonuniform))
    base.update(kw)
    prm = make_params(**base)
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps(np.arange(4) * 0.02)
    pos = _stretched(N, lo, hi, 7) if nonuniform else \
        oracle.uniform_grid_positions(N + 4, cfg.dx, lo)
    if nonuniform:
        eng.set_grid_positions(pos)
    eng.set_fields(frame, 0)
    eng.calc_fields_gradients(0)
    box = (lo + 0.1 * (hi - lo), 0.0, 0.0, hi - 0.1 * (hi - lo), 1.0, 1.0)
    eng.inject_particles_spatial_uniform(3000, 1e-6, 1, 2.0, 1, box)
    start = eng.get_particles()
    oracle.set_grid_positions(pos)
    full = oracle.full_fields(frame, 1, cfg, nonuniform=nonuniform)
    assert np.array_equal(eng.get_fields(0), full)
    oprm, ocfg = oracle.params_from(prm), oracle.config_from(cfg)
    parts = oracle.Particles(prm.nptl_max, start.arrays)
    cnt = oracle.OrcCounters()
    mover_kw = mover_kw or {}
    for k in range(2):
        eng.particle_mover(mhd_tframe=k + 1, **mover_kw)
        oracle.mover(oprm, ocfg, full, parts, 0.02 * k, 0.02, counters=cnt, **mover_kw)
    oracle.set_grid_positions(None)
    return eng, eng.get_particles(), ParticleSet(parts.view()), cnt


def test_1d_parker_bit_exact():
    eng, gpu, ref, cnt = _run()
    _same(gpu, ref, STATE)
    assert eng.counters().steps == cnt.steps
    assert np.all(gpu["y"] == ref["y"])
    eng.close()


def test_1d_nlgc_dpp_nonuniform_bit_exact():
    eng, gpu, ref, _ = _run(nonuniform=True, mover_kw=dict(nlgc=True, kperp_kpara=0.05),
                            dpp_wave=1)
    _same(gpu, ref, STATE)
    # local distributions bin x by the node search, y uniformly (1D keeps
    # no y positions)
    f, c = eng.local_distribution(pmin=0.05, pmax=10.0, npbins=16, rx=8)
    oracle.set_grid_positions(_stretched(N, 0.0, 1.0, 7))
    parts = oracle.Particles(len(gpu) + 8, gpu.arrays)
    cfg = make_mhd_config(N, 1, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.02, ndim=1)
    fo, co = oracle.local_distribution(oracle.config_from(cfg), 1, parts, 0.05, 10.0, 16, 1, 8,
                                       1, 1, nonuniform=True)
    oracle.set_grid_positions(None)
    assert np.array_equal(c.ravel(), co) and c.sum() > 0
    assert np.array_equal(f.ravel(), fo)
    eng.close()


def test_1d_focused_transport_bit_exact():
    eng, gpu, ref, _ = _run(mover_kw=dict(focused_transport=True), duu0=0.0)
    _same(gpu, ref, FT_STATE)
    eng.close()


def test_1d_spherical_and_scattering():
    eng, gpu, ref, _ = _run(spherical=True)
    _same(gpu, ref, STATE, exact=False)
    eng.close()
    eng, gpu, ref, _ = _run(mover_kw=dict(focused_transport=True), duu0=3.0)
    _same(gpu, ref, FT_STATE, exact=False)
    eng.close()
