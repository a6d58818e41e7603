"""The shock locator and injection at the shock in the CPU oracle (no GPU):
locate_shock_xpos (mhd_data_parallel.f90:1988-2006) finds, per row, the
node of steepest dvx/dx, and inject_particles_at_shock
(particle_module.f90:542-633), with the row interpolation its comments
describe, puts particles on a planar shock at its x and on a curved shock
x_s(y) = 0.5 + 0.08 sin(2 pi y) within a cell or two of x_s(y)."""
import numpy as np

import oracle
from gpat import fields
from gpat.engine import make_mhd_config, make_params

NX, NY = 256, 64


def shock_frame(xs, u1=1.0, r=4.0, w=0.004):
    """vx = u1 [1 - (1 - 1/r)(1 + tanh((x - xs(y)) / w)) / 2] on the nodes."""
    x = fields.node_coords(NX, 0.0, 1.0 / NX)[None, None, :]
    y = fields.node_coords(NY, 0.0, 1.0 / NY)[None, :, None]
    vx = u1 * (1.0 - (1.0 - 1.0 / r) * (1.0 + np.tanh((x - xs(y)) / w)) / 2.0)
    z = np.zeros_like(vx)
    one = np.ones_like(vx)
    return fields.assemble_frame(vx, z, z, one, one, z, z).astype(np.float32)


def _inject(xs):
    cfg = make_mhd_config(NX, NY, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.1)
    prm = make_params(ndim=2, p0=0.1, pmin=0.05, pmax=10.0)
    full = oracle.full_fields(shock_frame(xs), 2, cfg)
    parts = oracle.Particles(600)
    cnt = oracle.OrcCounters()
    oracle.inject_at_shock(oracle.params_from(prm), oracle.config_from(cfg), full, parts, 500,
                           1e-6, 1, 1.0, 0.3, cnt)
    return full, parts.view()


def test_locate_shock_planar():
    full, a = _inject(lambda y: 0.5 + 0.0 * y)
    S = oracle.locate_shock_xpos(full)
    assert S.shape == (1, NY + 4)
    x_of = (S[0] - 3) / NX
    assert np.all(np.abs(x_of - 0.5) <= 1.0 / NX)
    assert len(a["x"]) == 500 and np.all(a["t"] == 0.3)
    assert np.all(np.abs(a["x"] - 0.5) <= 1.0 / NX)
    assert a["y"].min() >= 0.0 and a["y"].max() < 1.0


def test_injection_follows_a_curved_shock():
    xs = lambda y: 0.5 + 0.08 * np.sin(2 * np.pi * y)
    _, a = _inject(xs)
    err = np.abs(a["x"] - xs(a["y"]))
    assert err.max() <= 2.0 / NX, err.max()
    assert np.corrcoef(a["x"], xs(a["y"]))[0, 1] > 0.99
