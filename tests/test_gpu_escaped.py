"""Escaped particles (escaped_ptls, kept while the mover runs with
dump_escaped_dist): the CUDA engine against the oracle's remove_particles
through the C ABI.  FP64: the escaped set and each particle's state at
escape are bit-exact; split precision: every escape counted in
nptl_escaped is stored, with an open-boundary face in count_flag."""
import numpy as np
import pytest

import oracle
from gpat.engine import Engine, ParticleSet, make_params
from test_gpu_parity import STATE, shock_case, turbulent_frame_2d

pytestmark = pytest.mark.gpu


def _engine(precision):
    params, cfg = shock_case(pbcx=1, pbcy=1, kpara0=2e-2, precision=precision, nptl_max=8000)
    prm = make_params(**params)
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps(np.arange(4) * 0.02)
    frame = turbulent_frame_2d()
    eng.set_fields(frame, 0)
    eng.calc_fields_gradients(0)
    eng.inject_particles_spatial_uniform(4000, 1e-6, 1, 1.0, 1, (0, 0, 0, 1, 1, 1))
    return eng, prm, cfg, frame


def test_escaped_particles_match_oracle_fp64():
    eng, prm, cfg, frame = _engine(0)
    start = eng.get_particles()
    parts = oracle.Particles(prm.nptl_max, start.arrays)
    store = oracle.EscapedStore(prm.nptl_max)
    cnt = oracle.OrcCounters()
    full = oracle.full_fields(frame, 2, cfg)
    oprm, ocfg = oracle.params_from(prm), oracle.config_from(cfg)
    for k in range(2):
        eng.particle_mover(mhd_tframe=k + 1, dump_escaped_dist=True)
        oracle.mover(oprm, ocfg, full, parts, 0.02 * k, 0.02, counters=cnt)
    store.detach()
    got = eng.get_escaped_particles().order_by_tags()
    ref = ParticleSet(store.view()).order_by_tags()
    assert len(got) == len(ref) == eng.counters().nptl_escaped > 100
    for k in STATE:
        assert np.array_equal(got[k], ref[k]), k
    assert np.all(got["count_flag"] < 0)
    # reset_escaped_particles empties the store; a call without
    # dump_escaped_dist stores nothing
    eng.reset_escaped_particles()
    assert len(eng.get_escaped_particles()) == 0
    eng.particle_mover(mhd_tframe=3)
    assert len(eng.get_escaped_particles()) == 0
    eng.close()


def test_escaped_particles_split_precision():
    eng, prm, cfg, frame = _engine(1)
    before = eng.counters().nptl_escaped
    tags_in = set(eng.get_particles()["tag_injected"].tolist())
    for k in range(2):
        eng.particle_mover(mhd_tframe=k + 1, dump_escaped_dist=True)
    esc = eng.get_escaped_particles()
    assert len(esc) == eng.counters().nptl_escaped - before > 100
    assert np.all((esc["count_flag"] <= -1) & (esc["count_flag"] >= -4))
    remaining = set(eng.get_particles()["tag_injected"].tolist())
    assert set(esc["tag_injected"].tolist()) == tags_in - remaining
    eng.close()
