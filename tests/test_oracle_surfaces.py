"""Acceleration-region surfaces of 3D runs (acc_by_surface) in the CPU
oracle (no GPU).  With a uniform compression along y and no diffusion,
x and z stay fixed, so whether a particle gains momentum is decided by the
surfaces alone (check_above_acc_surface, acc_region_surface.f90:343-383,
applied in push_particle_3d :4886-4900)."""
import numpy as np
import pytest

import oracle
from gpat import fields
from gpat.engine import make_mhd_config, make_params

N = 16


def _setup(a=0.5):
    cfg = make_mhd_config(N, N, N, 0.0, 1.0, 0.0, 1.0, zmin=0.0, zmax=1.0, dt_out=1.0, ndim=3)
    y = fields.node_coords(N, 0.0, 1.0 / N)
    shape = (N + 4, N + 4, N + 4)
    vy = np.broadcast_to(-a * (y[None, :, None] - 0.5), shape)
    z = np.zeros(shape)
    frame = fields.assemble_frame(z, vy, z, z + 1.0, z + 1.0, z, z).astype(np.float32)
    full = oracle.full_fields(frame, 3, cfg)
    prm = oracle.params_from(make_params(ndim=3, p0=0.1, pmin=0.05, pmax=10.0, kpara0=0.0,
                                         kret=0.1, momentum_dependency=0, dt_min_rel=0.01,
                                         dt_max_rel=0.01, acc_region_flag=1,
                                         acc_region=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)))
    return cfg, full, prm


def _grid(xs, zs):
    """Particles on a lattice of (x, z) at y = 0.45."""
    X, Z = np.meshgrid(xs, zs)
    n = X.size
    a = {k: np.zeros(n, dtype=t) for k, t in oracle.FIELDS}
    a["weight"][:] = 1.0
    a["count_flag"][:] = 1
    a["tag_splitted"][:] = 1
    a["tag_injected"][:] = np.arange(n, dtype=np.int32)
    a["x"][:], a["y"][:], a["z"][:], a["p"][:] = X.ravel(), 0.45, Z.ravel(), 0.1
    return a


def _move(cfg, full, prm, a, f2=None):
    parts = oracle.Particles(len(a["x"]), a)
    oracle.mover(prm, oracle.config_from(cfg), full, parts, 0.0, 1.0, f2=f2)
    out = parts.view()
    order = np.argsort(out["tag_injected"])
    return {k: v[order] for k, v in out.items()}


def _flat(h, axis_len=(N + 4, N + 4)):
    return np.full(axis_len, h)


@pytest.fixture(autouse=True)
def _off():
    yield
    oracle.set_acc_surface(None)


def test_one_surface_splits_the_region():
    cfg, full, prm = _setup()
    a = _grid(np.linspace(0.1, 0.9, 5), np.linspace(0.1, 0.9, 8))
    oracle.set_acc_surface("+z", _flat(0.5), shape=(N + 4, N + 4, N + 4))
    out = _move(cfg, full, prm, a)
    above = a["z"] > 0.5
    assert np.all(out["p"][above] > 0.1) and np.all(out["p"][~above] == 0.1)
    assert np.array_equal(out["z"], a["z"]) and np.array_equal(out["x"], a["x"])
    oracle.set_acc_surface("-z", _flat(0.5), shape=(N + 4, N + 4, N + 4))
    out = _move(cfg, full, prm, a)
    assert np.all(out["p"][~above] > 0.1) and np.all(out["p"][above] == 0.1)


@pytest.mark.parametrize("intersection", [True, False])
def test_two_surfaces_intersection_and_union(intersection):
    cfg, full, prm = _setup()
    a = _grid(np.linspace(0.1, 0.9, 9), np.linspace(0.1, 0.9, 8))
    # surface 2 normal to x: heights over (y, z) -> (nyg, nzg) array
    oracle.set_acc_surface("+z", _flat(0.5), norm2="-x", s21=_flat(0.35),
                           intersection=intersection, shape=(N + 4, N + 4, N + 4))
    out = _move(cfg, full, prm, a)
    r1, r2 = a["z"] > 0.5, a["x"] < 0.35
    inside = (r1 & r2) if intersection else (r1 | r2)
    assert np.all(out["p"][inside] > 0.1) and np.all(out["p"][~inside] == 0.1)


def test_surface_varies_in_space_and_time():
    cfg, full, prm = _setup()
    x = fields.node_coords(N, 0.0, 1.0 / N)
    # height h(x) = 0.2 + 0.5 x over the (x, y) plane, the first index x
    h = np.broadcast_to((0.2 + 0.5 * x)[None, :], (N + 4, N + 4))
    a = _grid(np.linspace(0.1, 0.9, 9), np.linspace(0.1, 0.9, 8))
    oracle.set_acc_surface("+z", h, shape=(N + 4, N + 4, N + 4))
    out = _move(cfg, full, prm, a)
    above = a["z"] > 0.2 + 0.5 * a["x"]
    assert np.all(out["p"][above] > 0.1) and np.all(out["p"][~above] == 0.1)
    # a surface rising from 0.3 to 0.7 over the interval: a particle at
    # z = 0.45 is above it for the first 37.5 % of the steps only
    oracle.set_acc_surface("+z", _flat(0.3), s12=_flat(0.7), shape=(N + 4, N + 4, N + 4))
    b = _grid([0.5], [0.45])
    out = _move(cfg, full, prm, b, f2=full)
    gain = 1.0 + 0.5 * 0.01 / 3.0
    assert 0.1 * gain ** 36 < out["p"][0] < 0.1 * gain ** 40
