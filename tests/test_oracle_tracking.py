"""Particle tracking in the CPU oracle (no GPU), pinned by answers that follow
from particle_module.f90: nsteps_tracking_max of init_particle_tracking
(:5874), is_particle_selected at injection (:434-440, :5923-5963), one
record every nsteps_interval pushes of a drift-only run whose time steps
are exact binary fractions (:1697-1703), the landing rule that takes a
record back and leaves the undone push's record in place (:1716-1722,
:1806-1812), split_particle's tracking branch (:5452-5474) and the
compaction of sync_tracked_particles (:5994-6030)."""
import numpy as np

import oracle
from gpat.engine import make_mhd_config, make_params
from test_oracle_1d import N, _frame, _start

DT_REL = 2.0 ** -7     # dt = dt_min_rel * dtf = 2^-10 with dtf = 2^-3
DTF = 2.0 ** -3


def _case(**kw):
    cfg = make_mhd_config(N, 1, 1, 0.0, 1.0, 0.0, 1.0, dt_out=DTF, ndim=1)
    base = dict(ndim=1, p0=0.1, pmin=0.05, pmax=10.0, kpara0=0.0, kret=0.1,
                momentum_dependency=0, dt_min_rel=DT_REL, dt_max_rel=DT_REL, pbcx=1)
    base.update(kw)
    prm = make_params(**base)
    x = (np.arange(N + 4) - 2) / N
    return prm, cfg, oracle.full_fields(_frame(-0.5 * x), 1, cfg)


def _tracked_start(n, t, tags_inj, tag_spl=-1, x=0.5):
    a = _start(n, x)
    a["t"][:] = t
    a["tag_injected"][:] = tags_inj
    a["tag_splitted"][:] = tag_spl
    return a


def test_nsteps_tracking_max():
    lib = oracle.load()
    assert lib.orc_nsteps_tracking_max(DT_REL, 16) == 9
    assert lib.orc_nsteps_tracking_max(1e-3, 10) == 101
    assert lib.orc_nsteps_tracking_max(0.03, 7) == 6


def test_injection_selects_listed_particles():
    prm, cfg, _ = _case()
    tags = np.array([[0, 3], [0, 3], [0, 5], [1, 4]], np.int32)
    trk = oracle.Tracking(tags, DT_REL, 16)
    try:
        parts = oracle.Particles(64)
        cnt = oracle.OrcCounters()
        cnt.tag_max = 1
        oracle.inject_at_x(oracle.params_from(prm), oracle.config_from(cfg), parts, 8, 0.5,
                           1e-6, 1, 2.0, 0.0, cnt)
        a = parts.view()
        for tag in range(1, 9):
            i = int(np.flatnonzero(np.abs(a["tag_injected"]) == tag)[0])
            tracked = tag in (3, 5)
            assert (a["tag_injected"][i] < 0) == tracked
            assert a["tag_splitted"][i] == (-1 if tracked else 1)
            assert a["nsteps_tracked"][i] == (1 if tracked else 0)
        rec = trk.sync()
        assert np.all(rec["tag_injected"][:2, 0] == -3) and rec["tag_injected"][2, 0] == -5
        assert np.all(rec["nsteps_tracked"][:3, 0] == 1)
        assert np.all(rec["x"][:3, 0] == 0.5)
        assert not rec["tag_splitted"][3].any() and not rec["tag_splitted"][:, 1:].any()
    finally:
        trk.detach()


def test_records_every_nsteps_interval_pushes():
    prm, cfg, full = _case()
    tags = np.array([[0, 3]], np.int32)
    trk = oracle.Tracking(tags, DT_REL, 16)
    try:
        parts = oracle.Particles(4, _tracked_start(1, 0.0, -3))
        oracle.mover(oracle.params_from(prm), oracle.config_from(cfg), full, parts, 0.0, DTF,
                     nsteps_interval=16)
        a = parts.view()
        assert a["t"][0] == DTF and a["nsteps_tracked"][0] == 9 and a["nsteps_pushed"][0] == 0
        # rows 2..9 hold the records; with row 1 (the injection record) empty
        # here, sync moves them up by one
        rec = trk.sync()
        k = np.arange(1, 9)
        np.testing.assert_array_equal(rec["t"][0, :8], 16 * k * 2.0 ** -10)
        np.testing.assert_array_equal(rec["nsteps_tracked"][0, :8], k + 1)
        assert not rec["nsteps_pushed"][0].any() and rec["tag_splitted"][0, 8] == 0
        np.testing.assert_allclose(rec["x"][0, :8], 0.5 * (1 - 0.5 * 2.0 ** -10) ** (16 * k),
                                   rtol=1e-6)
        assert trk.dropped() == 0
    finally:
        trk.detach()


def test_landing_takes_a_record_back():
    prm, cfg, full = _case()
    tags = np.array([[0, 3]], np.int32)
    half = 2.0 ** -11
    # nsteps_interval 16: push 128 overshoots and was recorded in row 9; the
    # landing takes the count back to 8 and sets the push count to 14, so
    # the redo push is not recorded and row 9 keeps the undone state
    trk = oracle.Tracking(tags, DT_REL, 16)
    try:
        parts = oracle.Particles(4, _tracked_start(1, half, -3))
        oracle.mover(oracle.params_from(prm), oracle.config_from(cfg), full, parts, 0.0, DTF,
                     nsteps_interval=16)
        a = parts.view()
        assert a["t"][0] == DTF
        assert a["nsteps_tracked"][0] == 8 and a["nsteps_pushed"][0] == 15
        rec = trk.sync()
        k = np.arange(1, 9)
        np.testing.assert_array_equal(rec["t"][0, :8], half + 16 * k * 2.0 ** -10)
        assert rec["t"][0, 7] > DTF and rec["nsteps_tracked"][0, 7] == 9
    finally:
        trk.detach()
    # nsteps_interval 1: the redo push is recorded in the row taken back
    trk = oracle.Tracking(tags, DT_REL, 1)
    try:
        assert trk.nsteps_max == 129
        parts = oracle.Particles(4, _tracked_start(1, half, -3))
        oracle.mover(oracle.params_from(prm), oracle.config_from(cfg), full, parts, 0.0, DTF,
                     nsteps_interval=1)
        a = parts.view()
        assert a["nsteps_tracked"][0] == 129 and a["nsteps_pushed"][0] == 0
        rec = trk.sync()
        np.testing.assert_array_equal(rec["t"][0, :127], half + np.arange(1, 128) * 2.0 ** -10)
        assert rec["t"][0, 127] == DTF and rec["dt"][0, 127] == half
        assert rec["nsteps_tracked"][0, 127] == 129 and rec["tag_splitted"][0, 128] == 0
        assert trk.dropped() == 0
    finally:
        trk.detach()


def test_split_follows_the_table():
    prm, _, _ = _case()
    # A: both halves listed; B: child missing; C: parent missing; D untracked
    tags = np.array([[0, 3, 1], [0, 3, 2], [0, 4, 1], [0, 6, 2]], np.int32)
    trk = oracle.Tracking(tags, DT_REL, 4)
    try:
        a = _tracked_start(4, 0.0, [-3, -4, -6, 7], [-1, -1, -1, 1])
        a["p"][:] = 0.3
        a["nsteps_tracked"][:] = 5
        a["nsteps_pushed"][:] = [0, 2, 0, 0]
        parts = oracle.Particles(16, a)
        cnt = oracle.OrcCounters()
        oracle.split(oracle.params_from(prm), parts, 2.0, 1.0, cnt)
        out = parts.view()
        assert parts.n == 8 and cnt.nptl_split == 4
        assert np.all(out["weight"] == 0.5) and np.all(out["split_times"] == 1)
        np.testing.assert_array_equal(out["tag_splitted"][:4], [-1, -1, 1, 1])
        np.testing.assert_array_equal(out["tag_splitted"][4:], [-2, 2, -2, 2])
        np.testing.assert_array_equal(out["nsteps_tracked"][:4], [6, 5, 5, 5])
        np.testing.assert_array_equal(out["nsteps_tracked"][4:], [6, 5, 6, 5])
        rec = trk.sync()
        # records in row 6: A's parent in column 1, A's child in column 2,
        # C's child in column 4; B (push count 2) records nothing
        np.testing.assert_array_equal(rec["tag_splitted"][:, 0], [-1, -2, 0, -2])
        np.testing.assert_array_equal(rec["nsteps_tracked"][:, 0], [6, 6, 0, 6])
        np.testing.assert_array_equal(rec["tag_injected"][:, 0], [-3, -3, 0, -6])
        assert np.all(rec["weight"][[0, 1, 3], 0] == 0.5)
    finally:
        trk.detach()


def test_split_past_the_last_row_is_dropped():
    prm, _, _ = _case()
    tags = np.array([[0, 3, 1], [0, 3, 2]], np.int32)
    trk = oracle.Tracking(tags, DT_REL, 1)
    try:
        a = _tracked_start(1, 0.0, -3)
        a["p"][:] = 0.3
        a["nsteps_tracked"][:] = trk.nsteps_max
        parts = oracle.Particles(4, a)
        oracle.split(oracle.params_from(prm), parts, 2.0, 1.0, oracle.OrcCounters())
        assert trk.dropped() == 2
        np.testing.assert_array_equal(parts.view()["nsteps_tracked"], [trk.nsteps_max + 1] * 2)
    finally:
        trk.detach()


def test_sync_compacts_each_column():
    trk = oracle.Tracking(np.array([[0, 1], [0, 2]], np.int32), 0.25, 1)
    try:
        assert trk.nsteps_max == 5
        r = trk.rec.a
        r["tag_splitted"][:5] = [-1, 0, -1, 5, -1]
        r["x"][:5] = [1.0, 2.0, 3.0, 4.0, 5.0]
        r["tag_splitted"][5:10] = [0, 0, 0, 0, -3]
        r["x"][5:10] = [0.0, 0.0, 0.0, 9.0, 7.0]
        out = trk.sync()
        np.testing.assert_array_equal(out["x"][0], [1.0, 3.0, 5.0, 0.0, 0.0])
        np.testing.assert_array_equal(out["tag_splitted"][0], [-1, -1, -1, 0, 0])
        np.testing.assert_array_equal(out["x"][1], [7.0, 0.0, 0.0, 0.0, 0.0])
        np.testing.assert_array_equal(out["tag_splitted"][1], [-3, 0, 0, 0, 0])
    finally:
        trk.detach()
