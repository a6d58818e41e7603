"""Injection where a field quantity is large (inject_particles_at_large_*,
particle_module.f90:785-1468; get_ncells_large_*, mhd_data_parallel.f90:
2211-2498) in the CPU oracle, against independent numpy evaluations (no
GPU)."""
import numpy as np
import pytest

import oracle
from gpat import fields
from gpat.engine import make_mhd_config, make_params

N = 48
BOX = (0.1, 0.2, 0.0, 0.9, 0.8, 1.0)


def _setup():
    cfg = make_mhd_config(N, N, 1, 0.0, 1.0, 0.0, 1.0)
    db = fields.kolmogorov_az_2d(N, N, 1.0, 1.0, 0.5, 2 * np.pi, 16 * np.pi, 3)
    frame = fields.planar_shock_2d(N, N, 0.0, 1.0, 0.0, 1.0, r=3.0, w=0.03, db=db)
    prm = make_params(ndim=2, p0=0.1, pmin=0.01, pmax=10.0, nptl_max=5000, seed=17)
    return cfg, oracle.full_fields(frame, 2, cfg), oracle.params_from(prm)


def _node_quantity(full, quantity):
    """Per-node quantity on nodes 1..N (C index 2..N+1), float32 as the
    reference's real(sp) arrays; divv from the node two lower per axis."""
    f = full[0]
    core = f[2:N + 2, 2:N + 2]
    if quantity == 0:
        return np.abs(core[..., 23] - core[..., 21]).astype(np.float64)
    if quantity == 1:
        t1, t2, t3 = core[..., 25] - core[..., 27], core[..., 26] - core[..., 22], \
            core[..., 21] - core[..., 23]
        return np.sqrt(t1 * t1 + t2 * t2 + t3 * t3).astype(np.float64)
    if quantity == 2:
        sh = f[0:N, 0:N]
        return -(sh[..., 8].astype(np.float64) + sh[..., 12].astype(np.float64))
    return core[..., 3].astype(np.float64)


def _interp(full, x, y, var):
    f = full[0].astype(np.float64)
    px, py = x * N, y * N
    ix, iy = np.floor(px).astype(int), np.floor(py).astype(int)
    rx, ry = px - ix, py - iy
    cx, cy = ix + 2, iy + 2
    return (f[cy, cx, var] * (1 - rx) * (1 - ry) + f[cy, cx + 1, var] * rx * (1 - ry) +
            f[cy + 1, cx, var] * (1 - rx) * ry + f[cy + 1, cx + 1, var] * rx * ry)


@pytest.mark.parametrize("quantity", [0, 1, 2, 3])
def test_cell_counts_match_numpy(quantity):
    cfg, full, prm = _setup()
    q = _node_quantity(full, quantity)
    xs = np.arange(N) / N
    inbox = ((xs[None, :] > BOX[0]) & (xs[None, :] < BOX[3]) &
             (xs[:, None] > BOX[1]) & (xs[:, None] < BOX[4]))
    for qmin in np.quantile(q[inbox], [0.0, 0.5, 0.9]):
        want = int(np.sum(inbox & (q > qmin)))
        got = oracle.count_cells_large(prm, oracle.config_from(cfg), full, quantity, qmin, BOX)
        assert got == want


@pytest.mark.parametrize("quantity,var", [(0, None), (2, None), (3, 3)])
def test_injected_particles_satisfy_criterion(quantity, var):
    cfg, full, prm = _setup()
    q = _node_quantity(full, quantity)
    qmin = float(np.quantile(q, 0.8))
    parts = oracle.Particles(3000)
    cnt = oracle.OrcCounters()
    oracle.inject_at_large(prm, oracle.config_from(cfg), full, parts, 2000, 1e-6, 1, 1.0, 0.0,
                           0.1, quantity, qmin, BOX, cnt)
    a = parts.view()
    assert parts.n == 2000
    x, y = a["x"], a["y"]
    assert np.all((x >= BOX[0]) & (x <= BOX[3]) & (y >= BOX[1]) & (y <= BOX[4]))
    if quantity == 0:
        val = np.abs(_interp(full, x, y, 23) - _interp(full, x, y, 21))
    elif quantity == 2:
        val = -(_interp(full, x, y, 8) + _interp(full, x, y, 12))
    else:
        val = _interp(full, x, y, var)
    assert np.all(val >= qmin * (1 - 1e-12) - 1e-12)
    assert np.all(a["p"] == 0.1) and np.all((a["t"] >= 0.0) & (a["t"] <= 0.1))
    assert np.all(np.abs(a["mu"]) <= np.float32(0.99))


def test_threshold_below_start_value_keeps_part_box_corner():
    """With qmin <= -2 (jz, absj, -divv) the reference never enters its
    rejection loop and every particle sits at the part_box corner."""
    cfg, full, prm = _setup()
    parts = oracle.Particles(100)
    cnt = oracle.OrcCounters()
    oracle.inject_at_large(prm, oracle.config_from(cfg), full, parts, 50, 1e-6, 1, 1.0, 0.0, 0.1,
                           0, -5.0, BOX, cnt)
    a = parts.view()
    assert np.all(a["x"] == BOX[0]) and np.all(a["y"] == BOX[1]) and np.all(a["z"] == BOX[2])
