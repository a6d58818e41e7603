"""Momentum diffusion (set_dpp_params) in the CPU oracle: known answers (no
GPU).

With no compression, calc_dpp_wave_scattering (particle_module.f90:
2918-2931, momentum-independent kappa) gives dp/dt = 4 p va^2 / (9 kpara)
and Dpp = p^2 va^2 / (9 kpara); calc_dpp_flow_shear (:2946-2979) with
pindex = 2 gives dp/dt = 4 G tau0 p and Dpp = G tau0 p^2, with
G = 2 sigma:sigma / 15 (strong scattering) or (b.sigma.b)^2 / 5 (weak).
Both are geometric Brownian motions dp = 4 D p dt + sqrt(2 D) p dW, so
ln p is Gaussian with mean ln p0 + 3 D t and variance 2 D t.
"""
import math

import numpy as np
import pytest

import oracle
from gpat import fields
from gpat.engine import make_mhd_config, make_params


def _frame(n, vx_of_y=None, b=(1.0, 0.0, 0.0), rho=1.0):
    dx = 1.0 / n
    x = fields.node_coords(n, 0.0, dx)
    y = fields.node_coords(n, 0.0, dx)
    X, Y = np.meshgrid(x, y)
    z = np.zeros_like(X)
    vx = vx_of_y(Y) if vx_of_y is not None else z
    return fields.assemble_frame(vx, z, z, z + rho, z + b[0], z + b[1], z + b[2])[None]


def _run(prm, frame, cfg, n, t, box):
    oprm = oracle.params_from(prm)
    parts = oracle.Particles(n)
    cnt = oracle.OrcCounters()
    oracle.inject_spatial_uniform(oprm, parts, n, 1e-6, 1, 1.0, 0.0, 0.0, box, cnt)
    oracle.mover(oprm, oracle.config_from(cfg), oracle.full_fields(frame, 2, cfg), parts, 0.0, t,
                 counters=cnt)
    return parts.view()


def _check_gbm(lnp, d, t):
    n = len(lnp)
    mean, var = 3.0 * d * t, 2.0 * d * t
    assert abs(lnp.mean() - mean) < 4.0 * math.sqrt(var / n) + 0.02 * mean
    assert abs(lnp.var() - var) < 4.0 * var * math.sqrt(2.0 / n) + 0.02 * var


def test_wave_scattering_is_geometric_brownian_motion():
    n_grid, n, t = 32, 4000, 0.2
    cfg = make_mhd_config(n_grid, n_grid, 1, 0.0, 1.0, 0.0, 1.0)
    kpara = 1.0 / 9.0 / 0.25                     # D = va^2 / (9 kpara) = 0.25
    prm = make_params(ndim=2, p0=0.1, pmin=0.01, pmax=10.0, kpara0=kpara, kret=0.0,
                      momentum_dependency=0, dpp_wave=1, dt_min_rel=1e-3, dt_max_rel=1e-2,
                      nptl_max=n, seed=7)
    out = _run(prm, _frame(n_grid), cfg, n, t, (0.0, 0.0, 0.0, 1.0, 1.0, 1.0))
    _check_gbm(np.log(out["p"] / 0.1), 0.25, t)


@pytest.mark.parametrize("weak", [0, 1])
def test_flow_shear_is_geometric_brownian_motion(weak):
    n_grid, n, t, shear = 32, 4000, 0.2, 5.0
    cfg = make_mhd_config(n_grid, n_grid, 1, 0.0, 1.0, 0.0, 1.0)
    s2 = 1.0 / math.sqrt(2.0)
    b = (s2, s2, 0.0) if weak else (1.0, 0.0, 0.0)
    # sigma_xy = S/2: strong G = 4 sigma_xy^2 / 15, weak (b.sigma.b)^2 / 5 with
    # b.sigma.b = 2 sigma_xy bx by = S/2.
    g = (shear * shear / 20.0) if weak else (shear * shear / 15.0)
    tau0 = 0.25 / g                              # D = G tau0 = 0.25
    prm = make_params(ndim=2, p0=0.1, pmin=0.01, pmax=10.0, kpara0=1e-4, kret=0.0,
                      momentum_dependency=0, pindex=2.0, dpp_shear=1, weak_scattering=weak,
                      tau0=tau0, dt_min_rel=1e-3, dt_max_rel=1e-2, nptl_max=n, seed=9)
    frame = _frame(n_grid, vx_of_y=lambda y: shear * y, b=b)
    out = _run(prm, frame, cfg, n, t, (0.0, 0.35, 0.0, 1.0, 0.65, 1.0))
    _check_gbm(np.log(out["p"] / 0.1), 0.25, t)
