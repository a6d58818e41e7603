"""Edge cases through the C ABI: an empty particle set goes through every
entry point of a frame (mover, split, distributions, quick_check, pmax,
escaped store) in both precisions; injection past nptl_max stops at the cap
with the oracle's particles and reports GPAT_ERR_CAPACITY; a single particle
(a ragged launch of one thread) moves bit-exactly; particles that start
outside an open box all leave, with their weight in leak."""
import numpy as np
import pytest

import oracle
from gpat import _abi
from gpat.engine import Engine, GPATError, ParticleSet, make_params
from test_gpu_parity import STATE, shock_case, turbulent_frame_2d

pytestmark = pytest.mark.gpu


def _engine(precision, **kw):
    params, cfg = shock_case(precision=precision, **kw)
    prm = make_params(**params)
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps(np.arange(4) * 0.02)
    frame = turbulent_frame_2d()
    eng.set_fields(frame, 0)
    eng.calc_fields_gradients(0)
    return eng, prm, cfg, frame


@pytest.mark.parametrize("precision", [0, 1])
def test_empty_set_through_a_frame(precision):
    eng, prm, cfg, _ = _engine(precision)
    # a split of an empty set right after a split of a full one
    eng.inject_particles_spatial_uniform(10, 1e-6, 1, 1.0, 1, (0, 0, 0, 1, 1, 1))
    eng.split_particle(1.0, 0.5, 10)
    eng.put_particles(ParticleSet.empty(0))
    eng.split_particle(1.0, 0.5, 10)
    eng.inject_particles_spatial_uniform(0, 1e-6, 1, 1.0, 1, (0, 0, 0, 1, 1, 1))
    eng.particle_mover(mhd_tframe=1, dump_escaped_dist=True)
    eng.split_particle(2.72, 2.0, 10)
    f, c = eng.calc_particle_distributions()
    assert not f.any() and not c.any()
    fl, cl = eng.local_distribution(pmin=0.05, pmax=10.0, npbins=8, rx=8, ry=8)
    assert not fl.any() and not cl.any()
    fm, cm = eng.particle_distributions_mu(4)
    assert not cm.any()
    q = eng.quick_check()
    assert q["nptl_current"] == 0 and q["leak"] == 0.0
    assert eng.get_pmax_global() == 0.0
    assert len(eng.get_particles()) == 0 and len(eng.get_escaped_particles()) == 0
    assert eng.counters().steps == 0
    eng.close()


def test_injection_past_capacity_matches_oracle():
    eng, prm, cfg, _ = _engine(0, nptl_max=100)
    with pytest.raises(GPATError) as err:
        eng.inject_particles_spatial_uniform(150, 1e-6, 1, 1.0, 1, (0, 0, 0, 1, 1, 1))
    assert err.value.code == _abi.GPAT_ERR_CAPACITY
    got = eng.get_particles()
    parts = oracle.Particles(100)
    oracle.inject_spatial_uniform(oracle.params_from(prm), parts, 150, 1e-6, 1, 1.0, 0.0, 0.02,
                                  (0, 0, 0, 1, 1, 1), oracle.OrcCounters())
    ref = ParticleSet(parts.view())
    assert len(got) == len(ref) == 100
    for k in STATE + ("tag_injected",):
        assert np.array_equal(got[k], ref[k]), k
    eng.close()


def test_single_particle_bit_exact():
    eng, prm, cfg, frame = _engine(0)
    eng.inject_particles_spatial_uniform(1, 1e-6, 1, 1.0, 1, (0.4, 0.4, 0, 0.6, 0.6, 1))
    start = eng.get_particles()
    eng.particle_mover(mhd_tframe=1)
    parts = oracle.Particles(4, start.arrays)
    oracle.mover(oracle.params_from(prm), oracle.config_from(cfg), oracle.full_fields(frame, 2, cfg),
                 parts, 0.0, 0.02)
    got, ref = eng.get_particles(), ParticleSet(parts.view())
    assert len(got) == len(ref) == 1
    for k in STATE:
        assert np.array_equal(got[k], ref[k]), k
    eng.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_particles_outside_an_open_box_all_leave(precision):
    eng, prm, cfg, _ = _engine(precision, pbcx=1, pbcy=1)
    ps = ParticleSet.empty(64)
    ps["x"][:] = np.where(np.arange(64) % 2 == 0, -0.3, 1.3)
    ps["y"][:] = 0.5
    ps["p"][:] = 0.1
    ps["weight"][:] = 0.25
    ps["count_flag"][:] = 1
    ps["tag_injected"][:] = np.arange(64)
    ps["tag_splitted"][:] = 1
    eng.put_particles(ps)
    eng.particle_mover(mhd_tframe=1)
    q = eng.quick_check()
    assert q["nptl_current"] == 0 and q["leak"] == 64 * 0.25
    assert eng.counters().steps == 0
    eng.close()
