"""Particle tracking: the CUDA engine against the oracle through the C ABI.
The FP64 mover is bit-exact on this case (no pow()), so the tracked
particles' tags and counts and every record of particles_tracked must match
exactly: selection at injection, a record every nsteps_interval pushes with
the landing rule, split_particle's tracking branch over two frames (one
lineage listed only in part, so some halves stop being tracked) and the
compaction of sync_tracked_particles."""
import numpy as np
import pytest

import oracle
from gpat.engine import Engine, GPATError, ParticleSet, make_params
from test_gpu_parity import shock_case, turbulent_frame_2d

pytestmark = pytest.mark.gpu

KEYS = ("x", "y", "z", "p", "v", "mu", "weight", "t", "dt", "split_times", "count_flag",
        "origin", "nsteps_tracked", "nsteps_pushed", "tag_injected", "tag_splitted", "rng_ctr")
TRACKED = (5, 17, 40, 41, 99, 200, 777, 1500)


def _table():
    """tags_tracking rows (origin, tag_injected, tag after split 1, after
    split 2), sorted; every third lineage lists only the first half."""
    cols = []
    for k, t in enumerate(TRACKED):
        leaves = [(1, 1), (1, 3), (2, 2), (2, 4)]
        if k % 3 == 2:
            leaves = leaves[:2]
        cols += [(0, t, a, b) for a, b in leaves]
    return np.array(cols, np.int32)


def _equal(gpu: ParticleSet, parts):
    """Same particles; removal keeps order on the GPU and swaps in the
    reference, so both sides are put in tag order."""
    gpu, ref = gpu.order_by_tags(), ParticleSet(parts.view()).order_by_tags()
    assert len(gpu) == len(ref)
    for k in KEYS:
        assert np.array_equal(gpu[k], ref[k]), k


def _records_equal(got: dict, ref: dict):
    for k in KEYS:
        assert np.array_equal(got[k], ref[k]), k


@pytest.mark.parametrize("nsteps_interval,num_fine_steps", [(1, 1), (3, 2)])
def test_tracking_matches_oracle(nsteps_interval, num_fine_steps):
    params, cfg = shock_case(precision=0, nptl_max=20000, kpara0=1e-2)
    prm = make_params(**params)
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps(np.arange(4) * 0.02)
    frame = turbulent_frame_2d()
    eng.set_fields(frame, 0)
    eng.calc_fields_gradients(0)
    table = _table()
    eng.init_particle_tracking(table, nsteps_interval)
    trk = oracle.Tracking(table, prm.dt_min_rel, nsteps_interval)
    try:
        nsteps, ntrk, _ = eng.tracking_dims()
        assert (nsteps, ntrk) == (trk.nsteps_max, len(table))
        box = (0.0, 0.0, 0.0, 1.0, 1.0, 1.0)
        eng.inject_particles_spatial_uniform(2000, 1e-6, 1, 2.0, 1, box)
        oprm, ocfg = oracle.params_from(prm), oracle.config_from(cfg)
        parts = oracle.Particles(prm.nptl_max)
        cnt = oracle.OrcCounters()
        oracle.inject_spatial_uniform(oprm, parts, 2000, 1e-6, 1, 2.0, 0.0, 0.02, box, cnt)
        gpu = eng.get_particles()
        _equal(gpu, parts)
        assert (gpu["tag_splitted"] < 0).sum() == len(TRACKED)
        _records_equal(eng.get_tracked_particles(), trk.sync())
        full = oracle.full_fields(frame, 2, cfg)
        for k in range(2):
            eng.particle_mover(mhd_tframe=k + 1, nsteps_interval=nsteps_interval,
                               num_fine_steps=num_fine_steps)
            oracle.mover(oprm, ocfg, full, parts, 0.02 * k, 0.02, counters=cnt,
                         nsteps_interval=nsteps_interval, num_fine_steps=num_fine_steps)
            _equal(eng.get_particles(), parts)
            _records_equal(eng.get_tracked_particles(), trk.sync())
            # ratio 1: every particle above 0.9 p0 splits in both frames
            eng.split_particle(1.0, 0.9, nsteps_interval)
            oracle.split(oprm, parts, 1.0, 0.9, cnt)
            gpu = eng.get_particles()
            _equal(gpu, parts)
        rec = eng.get_tracked_particles()
        _records_equal(rec, trk.sync())
        # tracked halves after two splits, and halves that left the table
        tracked = gpu["tag_splitted"] < 0
        assert np.any(tracked & (gpu["split_times"] == 2))
        assert np.any(~tracked & (gpu["tag_injected"] < 0))
        assert (rec["tag_splitted"] < 0).sum() > 10 * len(TRACKED)
        assert eng.tracking_dims()[2] == trk.dropped()
    finally:
        trk.detach()
    eng.free_particle_tracking()
    with pytest.raises(GPATError):
        eng.tracking_dims()
    eng.close()


def test_tracking_entry_points_check_arguments():
    params, cfg = shock_case(precision=1)
    eng = Engine(make_params(**params), cfg, 0)
    with pytest.raises(GPATError):
        eng.init_particle_tracking(_table(), 10)             # FP64 only
    eng.close()
    params, cfg = shock_case(precision=0)
    eng = Engine(make_params(**params), cfg, 0)
    with pytest.raises(GPATError):
        eng.init_particle_tracking(np.zeros((4, 1), np.int32), 10)   # < 2 rows
    with pytest.raises(GPATError):
        eng.get_tracked_particles()                          # not initialised
    with pytest.raises(GPATError):
        eng.init_particle_tracking(np.zeros((1, 200), np.int32), 10)  # > int8 split levels
    eng.init_particle_tracking(_table(), 10)
    nsteps, ntrk, dropped = eng.tracking_dims()
    assert nsteps == int(np.ceil((1.0 / params["dt_min_rel"]) / 10)) + 1 and dropped == 0
    rec = eng.get_tracked_particles()
    assert rec["x"].shape == (ntrk, nsteps) and not rec["tag_splitted"].any()
    eng.close()
    # records for 1e9 steps x 32 particles (~3 TB) fail cleanly
    params, cfg = shock_case(precision=0, dt_min_rel=1e-9)
    eng = Engine(make_params(**params), cfg, 0)
    with pytest.raises(GPATError):
        eng.init_particle_tracking(_table(), 1)
    eng.init_particle_tracking(_table()[:2], 10 ** 6)   # still usable afterwards
    assert eng.tracking_dims()[1] == 2
    eng.close()
