"""Acceleration-region surfaces of 3D runs (acc_by_surface): the CUDA FP64
mover against the oracle through the C ABI, bit-exact (no pow() on the
path), with one and two surfaces, time-interpolated between frames."""
import numpy as np
import pytest

import oracle
from gpat import fields
from gpat.engine import Engine, GPATError, ParticleSet, make_mhd_config, make_params
from test_gpu_focused import FT_STATE, _same
from test_gpu_parity import STATE

pytestmark = pytest.mark.gpu

N = 20
G = N + 4


def _height(seed, base, amp):
    rng = np.random.default_rng(seed)
    u = np.linspace(0.0, 1.0, G)
    A, B = np.meshgrid(u, u)
    kx, ky = rng.integers(1, 3, size=2)
    return base + amp * np.sin(2 * np.pi * (kx * A + ky * B) + rng.uniform(0, 6.28))


def _run(norm2=None, intersection=True, mover_kw=None, **kw):
    cfg = make_mhd_config(N, N, N, 0.0, 1.0, 0.0, 1.0, zmin=0.0, zmax=1.0, dt_out=0.02,
                          ndim=3)
    f1 = fields.turbulence_3d(N, seed=3)
    f2 = fields.turbulence_3d(N, seed=4)
    base = dict(ndim=3, p0=0.1, pmin=0.05, pmax=100.0, kpara0=2e-3, kret=0.1, dt_min_rel=2e-3,
                dt_max_rel=5e-2, pbcx=0, pbcy=0, pbcz=0, momentum_dependency=0, nptl_max=6000,
                seed=51, precision=0, time_interp=1, acc_region_flag=1,
                acc_region=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0))
    base.update(kw)
    prm = make_params(**base)
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps(np.arange(4) * 0.02)
    for slot, f in ((0, f1), (1, f2)):
        eng.set_fields(f, slot)
        eng.calc_fields_gradients(slot)
    s11, s12 = _height(1, 0.5, 0.2), _height(2, 0.45, 0.2)
    s21, s22 = (_height(3, 0.4, 0.15), _height(4, 0.6, 0.15)) if norm2 else (None, None)
    eng.init_acc_surface("+z", norm2, intersection)
    eng.set_acc_surface(0, s11, s21)
    eng.set_acc_surface(1, s12, s22)
    eng.inject_particles_spatial_uniform(3000, 1e-6, 1, 2.0, 1, (0, 0, 0, 1, 1, 1))
    start = eng.get_particles()
    oracle.set_acc_surface("+z", s11, s12, norm2=norm2, s21=s21, s22=s22,
                           intersection=intersection, shape=(G, G, G))
    full1, full2 = oracle.full_fields(f1, 3, cfg), oracle.full_fields(f2, 3, cfg)
    oprm, ocfg = oracle.params_from(prm), oracle.config_from(cfg)
    parts = oracle.Particles(prm.nptl_max, start.arrays)
    cnt = oracle.OrcCounters()
    mover_kw = mover_kw or {}
    eng.particle_mover(mhd_tframe=1, **mover_kw)
    oracle.mover(oprm, ocfg, full1, parts, 0.0, 0.02, counters=cnt, f2=full2, **mover_kw)
    oracle.set_acc_surface(None)
    return eng, eng.get_particles(), ParticleSet(parts.view())


@pytest.mark.parametrize("norm2,intersection", [(None, True), ("-x", True), ("+y", False)])
def test_surfaces_bit_exact(norm2, intersection):
    eng, gpu, ref = _run(norm2, intersection)
    _same(gpu, ref, STATE)
    moved = gpu["p"] != 0.1
    assert 0 < moved.sum() < len(gpu)   # the surfaces split the particles
    eng.close()


def test_surfaces_focused_transport_bit_exact():
    eng, gpu, ref = _run("-x", True, mover_kw=dict(focused_transport=True), duu0=0.0)
    _same(gpu, ref, FT_STATE)
    eng.close()


def test_surface_entry_points_check_arguments():
    cfg = make_mhd_config(N, N, N, 0.0, 1.0, 0.0, 1.0, zmin=0.0, zmax=1.0, ndim=3)
    eng = Engine(make_params(ndim=3, precision=0, nptl_max=100), cfg, 0)
    with pytest.raises(GPATError):
        eng.set_acc_surface(0, np.zeros((G, G)))           # before init
    with pytest.raises(GPATError):
        eng.init_acc_surface("+w")
    eng.init_acc_surface("-y", "+x")
    with pytest.raises(GPATError):
        eng.set_acc_surface(0, np.zeros((G, G)))           # surface 2 missing
    eng.close()
    eng = Engine(make_params(ndim=3, precision=1, nptl_max=100), cfg, 0)
    with pytest.raises(GPATError):
        eng.init_acc_surface("+z")                          # FP64 only
    eng.close()
