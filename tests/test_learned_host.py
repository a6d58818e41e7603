"""Host logic of learned splitting, without a GPU: the weight-window
parameters with a defensive floor, the one-interval extrapolation of the
sums the mover judges with, and the tail statistics of split runs with one
sample per injected particle."""
import math

import numpy as np
import pytest

from gpat.engine import FusedWindow, ParticleSet, tail_by_ancestor, window_params


def _target_weights(z, w, target, defensive):
    """w_t of every particle from window_params, as the device computes it
    (floored log-importance log(exp(z) + exp(z_floor)))."""
    lse = math.log(float(np.sum(w * np.exp(z))))
    lsw = math.log(float(np.sum(w)))
    z_ref, z_floor = window_params(lse, lsw, target, defensive)
    zp = np.logaddexp(z, z_floor) if math.isfinite(z_floor) else z
    return np.exp(z_ref - zp)


@pytest.mark.parametrize("defensive", [0.0, 0.1, 0.5])
def test_window_aims_the_population_at_the_target(defensive):
    rng = np.random.default_rng(3)
    z = rng.normal(-10.0, 4.0, 50_000)
    w = rng.uniform(0.5, 2.0, z.size)
    target = 80_000
    wt = _target_weights(z, w, target, defensive)
    assert np.sum(w / wt) == pytest.approx(target, rel=1e-9)


def test_defensive_floor_bounds_the_target_weight():
    rng = np.random.default_rng(4)
    z = np.concatenate([rng.normal(-30.0, 3.0, 49_000), rng.normal(0.0, 1.0, 1_000)])
    w = np.ones(z.size)
    target, a = 100_000, 0.1
    bare = _target_weights(z, w, target, 0.0)
    floored = _target_weights(z, w, target, a)
    # without the floor hopeless particles get astronomical target weights
    assert bare.max() > 1e6
    # with it no target weight exceeds (1 + a) / a * W / target
    assert floored.max() <= (1.0 + a) / a * w.sum() / target * (1.0 + 1e-12)


def test_no_floor_is_the_bare_importance():
    z_ref, z_floor = window_params(2.0, 5.0, 100, 0.0)
    assert z_floor == -math.inf and z_ref == pytest.approx(2.0 - math.log(100))


def test_fused_window_carries_the_sums_forward():
    win = FusedWindow(target=1000, defensive=0.1, max_step=2.0)
    win.start(10.0, 7.0)
    # no history yet: the sums themselves
    assert win.params() == window_params(10.0, 7.0, 1000, 0.1)
    win.update(dict(judged=50, log_sum_wexpz=10.5, log_sum_w=7.0))
    # the last change (+0.5) carried one interval ahead
    assert win.params() == window_params(11.0, 7.0, 1000, 0.1)
    win.update(dict(judged=50, log_sum_wexpz=20.5, log_sum_w=7.0))
    # a jump of 10 is carried forward by at most max_step
    assert win.params() == window_params(22.5, 7.0, 1000, 0.1)
    # an interval with nobody judged keeps the sums
    win.update(dict(judged=0, log_sum_wexpz=-math.inf, log_sum_w=-math.inf))
    assert win.params() == window_params(22.5, 7.0, 1000, 0.1)


class _FakeEngine:
    def __init__(self, ps):
        self.ps = ps

    def get_particles(self):
        return self.ps


def _set(tags, p, w, flag=None):
    n = len(tags)
    ps = ParticleSet.empty(n)
    ps.arrays["tag_injected"][:] = tags
    ps.arrays["p"][:] = p
    ps.arrays["weight"][:] = w
    ps.arrays["count_flag"][:] = 1 if flag is None else flag
    return ps


def test_tail_by_ancestor_groups_lineages():
    # ancestor 0: two copies in the tail; ancestor 1: one of two copies;
    # ancestor 2: none; ancestor 3: a tail copy that was removed
    eng = _FakeEngine(_set(tags=[0, 0, 1, 1, 2, 3], p=[5.0, 6.0, 7.0, 0.5, 0.5, 9.0],
                           w=[0.5, 0.5, 0.25, 0.25, 1.0, 1.0], flag=[1, 1, 1, 1, 1, 0]))
    a = tail_by_ancestor(eng, 1.0, n_injected=4)
    assert a["particles"] == 3 and a["ancestors"] == 2
    assert a["fraction"] == pytest.approx((1.0 + 0.25) / 4)
    assert a["sigma"] == pytest.approx(math.sqrt(1.0 + 0.0625) / 4)
    assert a["ess"] == pytest.approx(1.25 ** 2 / 1.0625)


def test_tail_by_ancestor_equals_per_particle_without_splitting():
    rng = np.random.default_rng(5)
    n = 10_000
    p = rng.exponential(1.0, n)
    eng = _FakeEngine(_set(tags=np.arange(n), p=p, w=np.ones(n)))
    a = tail_by_ancestor(eng, 3.0, n)
    c = int(np.sum(p > 3.0))
    assert a["particles"] == a["ancestors"] == c
    assert a["ess"] == pytest.approx(c) and a["fraction"] == pytest.approx(c / n)


def test_tail_by_ancestor_empty_tail():
    eng = _FakeEngine(_set(tags=[0, 1], p=[0.1, 0.2], w=[1.0, 1.0]))
    assert tail_by_ancestor(eng, 1.0, 2) == dict(fraction=0.0, sigma=0.0, ess=0.0,
                                                   particles=0, ancestors=0)
