"""Distributions with pitch-angle bins and the local escaped distributions
in the CPU oracle (no GPU), pinned by hand-counted bins that follow
diagnostics.f90: the global and escaped f(p, mu) (:773-779, :949-957) with
the strict lower p bound, the single-precision mu step 2.0 / nmu (:206) and
the bins p == pmax and mu == 1 would index past the end; and the per-face
local escaped distributions (:958-1230)."""
import numpy as np

import oracle
from gpat.engine import make_mhd_config, make_params


def _parts(rows):
    """rows of (x, y, z, p, mu, weight, count_flag)."""
    n = len(rows)
    a = {k: np.zeros(n, dtype=t) for k, t in oracle.FIELDS}
    for k, col in zip(("x", "y", "z", "p", "mu", "weight", "count_flag"), zip(*rows)):
        a[k][:] = col
    return oracle.Particles(n + 1, a)


def test_global_distribution_with_mu_bins():
    prm = oracle.params_from(make_params(p0=1.0, pmin=1.0, pmax=100.0, npp_global=2))
    third = -1.0 + 2.0 / 3.0      # (mu + 1) / dmu is just below 1 with dmu = 2/3 in single
    parts = _parts([
        (0, 0, 0, 5.0, -0.9, 1.0, 1),      # ip 1, imu 1
        (0, 0, 0, 50.0, 0.9, 2.0, 1),      # ip 2, imu 3
        (0, 0, 0, 50.0, third, 4.0, 1),    # ip 2, imu 1 (2 with a double-precision step)
        (0, 0, 0, 1.0, 0.0, 8.0, 1),       # p == pmin: outside
        (0, 0, 0, 100.0, 0.0, 16.0, 1),    # p == pmax: ip 3, dropped
        (0, 0, 0, 5.0, 1.0, 32.0, 1),      # mu == 1: 2 / dmu rounds below 3, imu 3
        (0, 0, 0, 5.0, 0.2, 64.0, 1),      # ip 1, imu 2
    ])
    f, c = oracle.distribution_mu(prm, parts, 3)
    np.testing.assert_array_equal(c, [1, 1, 1, 1, 0, 1])
    np.testing.assert_array_equal(f, [1.0, 64.0, 32.0, 4.0, 0.0, 2.0])
    # with an exact step (nmu 2) mu == 1 indexes bin 3 and is dropped
    f, c = oracle.distribution_mu(prm, parts, 2)
    np.testing.assert_array_equal(c, [1, 1, 1, 1])
    np.testing.assert_array_equal(f, [1.0, 64.0, 4.0, 2.0])


def test_escaped_distribution_by_face():
    prm = oracle.params_from(make_params(p0=1.0, pmin=1.0, pmax=100.0, npp_global=2))
    parts = _parts([
        (0, 0, 0, 5.0, 0.5, 1.0, -1),
        (0, 0, 0, 50.0, -0.5, 2.0, -4),
        (0, 0, 0, 50.0, -0.5, 4.0, -4),
        (0, 0, 0, 50.0, -0.5, 8.0, 1),     # not escaped
        (0, 0, 0, 50.0, -0.5, 16.0, -5),   # face 5 of a 2D run: no column
    ])
    f, c = oracle.distribution_mu(prm, parts, 2, by_face=True, nfaces=4)
    f = f.reshape(4, 2, 2)                 # (face, ip, imu)
    assert f[0, 0, 1] == 1.0 and f[3, 1, 0] == 6.0 and f.sum() == 7.0
    assert c.sum() == 3


def test_local_escaped_distribution_faces():
    cfg = oracle.config_from(make_mhd_config(8, 4, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.1))
    # rx 2: nrx 4, nry 4; p bins over [1, 100] in 2, so only ip 1 counts
    rows = [
        (-0.01, 0.6, 0.0, 5.0, 0.0, 1.0, -1),   # low x face, iy 3
        (1.01, 0.1, 0.0, 5.0, 0.0, 2.0, -2),    # high x face, iy 1
        (0.3, 1.02, 0.0, 5.0, 0.0, 4.0, -4),    # high y face, ix 2
        (0.3, 1.30, 0.0, 5.0, 0.0, 8.0, -1),    # x face but y outside: skipped
        (0.3, 0.5, 0.0, 50.0, 0.0, 16.0, -3),   # ip 2 = npbins: skipped
        (0.3, 0.5, 0.0, 5.0, 0.0, 32.0, -5),    # z face of a 2D run: skipped
    ]
    out = oracle.local_escaped_distribution(cfg, 2, _parts(rows), 1.0, 100.0, 2, 1, 2, 1, 1)
    (fx, cx), (fy, cy), fz = out
    assert fz is None
    fx = fx.reshape(2, 1, 4, 2)                # (side, iz, iy, ip) with nmu 1
    fy = fy.reshape(2, 1, 4, 2)                # (side, iz, ix, ip)
    assert fx[0, 0, 2, 0] == 1.0 and fx[1, 0, 0, 0] == 2.0 and fx.sum() == 3.0
    assert fy[1, 0, 1, 0] == 4.0 and fy.sum() == 4.0
    assert cx.sum() == 2 and cy.sum() == 1
