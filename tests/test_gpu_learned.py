"""Learned splitting: the network's GPU forward and gradient against the CPU
oracle (oracle/mlp_oracle.py), training, and weighted splitting / roulette
driven by the trained network on a 3D run (unbiased tail, more effective
samples, unique lineage tags, bounded weights: the importance is floored at
a tenth of its weighted mean, so the total weight stays within Monte Carlo
error of the injected weight)."""
import math

import numpy as np
import pytest

import mlp_oracle as mo
from gpat import configs
from gpat.engine import Mlp, tail_by_ancestor, tail_weights, weighted_split, window_params

# defensive fraction of the weighted mean importance added to every particle's
DEFENSIVE = 0.1

pytestmark = pytest.mark.gpu


def test_forward_and_gradient_match_oracle():
    rng = np.random.default_rng(2)
    m = Mlp(seed=3)
    params = mo.init_params(7)
    norm = np.concatenate([rng.normal(size=8) * 0.1, 1.0 + rng.random(8)]).astype(np.float32)
    m.set_params(params, norm)
    x = rng.normal(size=(5000, 8)).astype(np.float32)
    z = m.forward(x)
    # the tensor-core kernels round inputs, activations and deltas to BF16
    # (FP32 accumulation); the oracle restates that rounding in float64
    zr = mo.forward(params, norm.astype(np.float64), x, round_act=True)
    np.testing.assert_allclose(z, zr, rtol=2e-3, atol=2e-3)
    # and against the unrounded network: BF16 operand error only
    z64 = mo.forward(params, norm.astype(np.float64), x)
    assert np.abs(z - z64).max() < 0.05 * max(1.0, np.abs(z64).max())
    y = (rng.random(5000) < 0.2).astype(np.float32)
    loss, g = m.loss_grad(x, y)
    lr, gr = mo.loss_grad(params, norm.astype(np.float64), x, y, round_act=True)
    assert abs(loss - lr) < 1e-3 * max(1.0, abs(lr))
    np.testing.assert_allclose(g, gr, rtol=1e-2, atol=5e-3 * np.abs(gr).max())
    lr64, gr64 = mo.loss_grad(params, norm.astype(np.float64), x, y)
    cos = float(g @ gr64 / (np.linalg.norm(g) * np.linalg.norm(gr64)))
    assert cos > 0.999, cos
    p2, n2 = m.get_params()
    assert np.array_equal(p2, params) and np.array_equal(n2, norm)
    m.close()


def test_training_learns_a_rule():
    rng = np.random.default_rng(4)
    n = 200_000
    x = rng.normal(size=(n, 8)).astype(np.float32)
    logit = 2.0 * x[:, 0] - 1.5 * x[:, 3] * x[:, 3] + 1.0
    y = (rng.random(n) < 1.0 / (1.0 + np.exp(-logit))).astype(np.float32)
    m = Mlp(seed=5, record_capacity=n)
    m.set_records(x, y)
    l0, _ = m.loss_grad(x[:20000], y[:20000])
    m.train(epochs=4, batch=4096, lr=3e-3, seed=2)
    l1, _ = m.loss_grad(x[:20000], y[:20000])
    # the Bayes loss of this rule is about 0.43; an untrained net sits near 0.7+
    assert l1 < 0.5 and l1 < l0 - 0.1
    m.close()


def check_total_weight(eng, nptl, target):
    """The live particles' total weight is the injected nptl within Monte
    Carlo error, and no weight exceeds the floor's bound.  A roulette survivor
    weighs at most (1 + a) / a * W / target (a = DEFENSIVE, W the total
    weight at the judgement), 5.5 here; every roulette adds at most
    w * 5.5 to the variance of the total, so after 8 judgements of at most
    40000 particles of weight <= 1 its standard deviation is below
    sqrt(8 * 20000 * 5.5) ~ 940, 4.7 % of nptl: 15 % is over 3 sigma."""
    c, wsum, _ = tail_weights(eng, 0.0)
    bound = (1.0 + DEFENSIVE) / DEFENSIVE * nptl / target
    assert abs(wsum - nptl) < 0.15 * nptl, (wsum, nptl)
    ps = eng.get_particles()
    live = ps["count_flag"] == 1
    assert ps["weight"][live].max() < 2.0 * bound, (ps["weight"][live].max(), bound)


def check_tail_and_samples(plain, pushes_plain, eng, pushes, nptl):
    """Tails of a plain and a learned-splitting run, one sample per injected
    particle (split copies share their parent's history): above the plain
    run's 98th and 99.5th percentiles the fractions agree within four
    combined standard errors, and above the 99.5th the learned run has more
    effective samples per push (measured 2.4x to 2.8x over two networks,
    fused and separate; 1.3x at the 98th, 6x at the 99.9th)."""
    pend = plain.get_particles()["p"]
    for q in (0.98, 0.995):
        thr = float(np.quantile(pend, q))
        a0, a1 = tail_by_ancestor(plain, thr, nptl), tail_by_ancestor(eng, thr, nptl)
        assert abs(a1["fraction"] - a0["fraction"]) < 4.0 * math.hypot(a0["sigma"], a1["sigma"]), \
            (q, a0, a1)
    gain = (a1["ess"] / pushes) / (a0["ess"] / pushes_plain)
    assert gain > 1.5, (gain, a0, a1, pushes_plain, pushes)


def test_learned_splitting_3d_unbiased_and_more_samples():
    n_grid, nptl, nint = 32, 20000, 8
    w = configs.turbulence_3d(scale=nptl / 1e8, n=n_grid, nframes=nint)

    def run(recorder=None, learned=None, target=None):
        eng = configs.build_engine(w, nptl_max=nptl * 40)
        configs.inject(eng, w)
        pushes = 0
        for k in range(nint):
            if learned is not None:
                # importance-weighted population of about `target` particles
                _, lse, lsw = learned.score(eng, k / nint)
                z_ref, z_floor = window_params(lse, lsw, target, DEFENSIVE)
                weighted_split(eng, learned, k / nint, 1.0, z_ref, window_ratio=4.0, max_level=3,
                               z_floor=z_floor)
            if recorder is not None:
                recorder.record(eng, k / nint)
            eng.particle_mover(mhd_tframe=k + 1)
            pushes += eng.counters().last_mover_steps
        return eng, pushes

    net = Mlp(seed=9, record_capacity=nptl * nint)
    plain, pushes_plain = run(recorder=net)
    # threshold: the top 2 % of the plain run's final momenta
    pthr = float(np.quantile(plain.get_particles()["p"], 0.98))
    npos, nrec = net.label(plain, pthr)
    assert nrec > 0 and 0 < npos < nrec
    net.train(epochs=4, batch=4096, lr=3e-3, seed=3)
    eng_l, pushes_l = run(learned=net, target=2 * nptl)
    ps = eng_l.get_particles()
    check_tail_and_samples(plain, pushes_plain, eng_l, pushes_l, nptl)
    # lineage tags stay unique
    key = (ps["tag_injected"].astype(np.int64) << 32) | (ps["tag_splitted"].astype(np.int64) &
                                                         0xFFFFFFFF)
    assert len(np.unique(key)) == len(key)
    check_total_weight(eng_l, nptl, 2 * nptl)
    for e in (plain, eng_l):
        e.close()
    net.close()


def test_learned_splitting_fused_in_the_mover():
    """The same method with the network evaluated inside the mover launch as
    particles finish each interval (gpat_set_mover_learned): the tail weight
    agrees with a plain run within Monte Carlo error, every finished particle
    is judged, the tail gets more effective samples per push, and lineage
    tags stay unique."""
    from gpat.engine import FusedWindow, mover_learned_stats, set_mover_learned
    n_grid, nptl, nint = 32, 20000, 8
    w = configs.turbulence_3d(scale=nptl / 1e8, n=n_grid, nframes=nint)
    net = Mlp(seed=9, record_capacity=nptl * nint)
    plain = configs.build_engine(w, nptl_max=nptl * 40)
    configs.inject(plain, w)
    pushes_plain = 0
    for k in range(nint):
        net.record(plain, k / nint)
        plain.particle_mover(mhd_tframe=k + 1)
        pushes_plain += plain.counters().last_mover_steps
    pthr = float(np.quantile(plain.get_particles()["p"], 0.98))
    net.label(plain, pthr)
    net.train(epochs=4, batch=4096, lr=3e-3, seed=3)

    target = 2 * nptl
    eng = configs.build_engine(w, nptl_max=nptl * 40)
    configs.inject(eng, w)
    win = FusedWindow(target, DEFENSIVE)
    win.start(*net.score(eng, 0.0)[1:])
    pushes = 0
    for k in range(nint):
        z_ref, z_floor = win.params()
        set_mover_learned(eng, net, (k + 1) / nint, 1.0, z_ref, 4.0, 3, z_floor=z_floor)
        n_before = eng.nptl_current
        eng.particle_mover(mhd_tframe=k + 1)
        pushes += eng.counters().last_mover_steps
        st = mover_learned_stats(eng)
        # a periodic box: every particle finishes the interval and is judged once
        assert st["judged"] == n_before, (st, n_before)
        assert eng.nptl_current == n_before + st["nsplit"] - st["nkilled"]
        win.update(st)
    set_mover_learned(eng, None)
    # the lagged, extrapolated normalisation keeps the population near target
    assert 0.7 * target < eng.nptl_current < 1.3 * target, eng.nptl_current
    check_tail_and_samples(plain, pushes_plain, eng, pushes, nptl)
    ps = eng.get_particles()
    key = (ps["tag_injected"].astype(np.int64) << 32) | (ps["tag_splitted"].astype(np.int64) &
                                                         0xFFFFFFFF)
    assert len(np.unique(key)) == len(key)
    check_total_weight(eng, nptl, target)
    for e in (plain, eng):
        e.close()
    net.close()


@pytest.mark.parametrize("fused", [False, True])
def test_splits_past_thirty_levels_take_fresh_lineage_ids(fused):
    """Copies split past the int32 tag's 30 binary levels take fresh negative
    tag_splitted ids: every (tag_injected, tag_splitted) pair stays unique
    (so every copy keeps its own Philox stream), the total weight is kept in
    expectation, and an engine that receives such a set hands out ids past
    the ones it holds."""
    from gpat.engine import FusedWindow, mover_learned_stats, set_mover_learned
    n_grid, nptl, nint = 32, 20000, 2
    w = configs.turbulence_3d(scale=nptl / 1e8, n=n_grid, nframes=4)
    net = Mlp(seed=11)   # an untrained network: z varies a little with the features

    def split_run(eng, target):
        if fused:
            win = FusedWindow(target, DEFENSIVE)
            win.start(*net.score(eng, 0.0)[1:])
        for k in range(nint):
            if fused:
                z_ref, z_floor = win.params()
                set_mover_learned(eng, net, (k + 1) / 4, 1.0, z_ref, 4.0, 3, z_floor=z_floor)
                eng.particle_mover(mhd_tframe=k + 1)
                win.update(mover_learned_stats(eng))
            else:
                _, lse, lsw = net.score(eng, k / 4)
                z_ref, z_floor = window_params(lse, lsw, target, DEFENSIVE)
                weighted_split(eng, net, k / 4, 1.0, z_ref, 4.0, 3, z_floor=z_floor)
                eng.particle_mover(mhd_tframe=k + 1)
        set_mover_learned(eng, None)
        return eng.get_particles()

    def unique_keys(ps):
        key = (ps["tag_injected"].astype(np.int64) << 32) | \
              (ps["tag_splitted"].astype(np.int64) & 0xFFFFFFFF)
        return len(np.unique(key)) == len(key)

    eng = configs.build_engine(w, nptl_max=nptl * 40)
    configs.inject(eng, w)
    ps = eng.get_particles()
    ps.arrays["split_times"][:] = 30   # every split is past the 30 levels
    eng.put_particles(ps)
    out = split_run(eng, 4 * nptl)   # w / w_t ~ 4: particles above the window split once
    neg = out["tag_splitted"] < 0
    assert neg.sum() > nptl // 4, neg.sum()
    assert len(np.unique(out["tag_splitted"][neg])) == neg.sum()
    assert unique_keys(out)
    assert abs(out["weight"].sum() - nptl) < 0.15 * nptl
    # a second engine receiving the set continues past its ids
    eng2 = configs.build_engine(w, nptl_max=nptl * 40)
    eng2.put_particles(out)
    lowest = int(out["tag_splitted"].min())
    out2 = split_run(eng2, 16 * nptl)   # the received weights (~0.5) split again
    new = out2["tag_splitted"] < lowest
    assert new.sum() > 0 and unique_keys(out2)
    for e in (eng, eng2):
        e.close()
    net.close()
