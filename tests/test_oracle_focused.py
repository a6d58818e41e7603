"""Focused transport and NLGC in the CPU oracle: known answers (no GPU).

Cases whose answer follows from the reference's update rules
(particle_module.f90): streaming along a uniform B at v*mu with no
scattering (push_particle_2d_ft :3626-3964, push_particle_3d_ft
:4930-5324), the stationary pitch-angle distribution that the drift and
D_mumu of calc_duu (:3116-3155) produce, and the mu^2 law of
calc_spatial_diffusion_coefficients_nlgc (:2464-2771).
"""
import ctypes as C
import math

import numpy as np
import pytest

import oracle
from gpat import fields
from gpat.engine import make_mhd_config, make_params


def _uniform_b_frame(nx, ny, b=(1.0, 0.0, 0.0)):
    dx, dy = 1.0 / nx, 1.0 / ny
    x = fields.node_coords(nx, 0.0, dx)
    y = fields.node_coords(ny, 0.0, dy)
    X, _ = np.meshgrid(x, y)
    z = np.zeros_like(X)
    return fields.assemble_frame(z, z, z, z + 1.0, z + b[0], z + b[1], z + b[2])[None]


def _uniform_b_frame_3d(n, b=(1.0, 0.0, 0.0)):
    z = np.zeros((n + 4, n + 4, n + 4))
    return fields.assemble_frame(z, z, z, z + 1.0, z + b[0], z + b[1], z + b[2])


def _kappa(prm, bx, by, bz, p, mu):
    f = (C.c_double * 32)()
    f[4], f[5], f[6] = bx, by, bz
    k = (C.c_double * 22)()
    oracle.load().orc_calc_spatial_diffusion_coefficients(C.byref(prm), p, mu, f, None, k)
    return list(k)


def _inject(prm, n, box, v0, mu=None, dt=1e-6):
    parts = oracle.Particles(n)
    cnt = oracle.OrcCounters()
    oracle.inject_spatial_uniform(prm, parts, n, dt, 1, v0, 0.0, 0.0, box, cnt)
    if mu is not None:
        parts.a["mu"][:n] = mu
    return parts, cnt


def test_nlgc_kperp_scales_with_mu_squared():
    prm = oracle.params_from(make_params(ndim=3, kpara0=0.02, momentum_dependency=0))
    prm.nlgc = 1
    prm.kperp_kpara = 0.01
    for mu in (0.0, 0.3, -0.7):
        k = _kappa(prm, 0.3, -0.4, 1.2, 0.1, mu)
        assert k[2] == pytest.approx(0.02, rel=1e-15)
        assert k[3] == pytest.approx(0.02 * 0.01 * mu * mu, rel=1e-15, abs=0)
    # momentum dependence: kpara ~ p^pindex, kperp ~ p^((5 - gamma)/3)
    prm.momentum_dependency = 1
    g = prm.gamma_turb
    k1 = _kappa(prm, 1.0, 0.0, 0.0, 0.1, 0.5)
    k2 = _kappa(prm, 1.0, 0.0, 0.0, 0.4, 0.5)
    assert k2[2] / k1[2] == pytest.approx(4.0 ** prm.pindex, rel=1e-13)
    assert k2[3] / k1[3] == pytest.approx(4.0 ** ((5.0 - g) / 3.0), rel=1e-13)


def test_focused_transport_kappa_is_perpendicular_projector():
    prm = oracle.params_from(make_params(ndim=3, kpara0=0.02, kret=0.1, momentum_dependency=0))
    prm.focused_transport = 1
    bx, by, bz = 0.3, -0.4, 1.2
    k = _kappa(prm, bx, by, bz, 0.1, 0.5)
    kperp = k[3]
    b = np.array([bx, by, bz]) / math.sqrt(bx * bx + by * by + bz * bz)
    want = kperp * (np.eye(3) - np.outer(b, b))
    got = np.array([[k[7], k[10], k[11]], [k[10], k[8], k[12]], [k[11], k[12], k[9]]])
    np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-19)


@pytest.mark.parametrize("ndim", [2, 3])
def test_focused_streaming_along_uniform_b(ndim):
    """No scattering (duu0 = 0), no kperp, no flow: each particle moves
    along B by v*mu*dtf, keeping p, v and mu."""
    n = 16 if ndim == 3 else 32
    cfg = make_mhd_config(n, n, n if ndim == 3 else 1, 0.0, 1.0, 0.0, 1.0, zmin=0.0, zmax=1.0,
                          ndim=ndim)
    frame = _uniform_b_frame_3d(n) if ndim == 3 else _uniform_b_frame(n, n)
    prm = make_params(ndim=ndim, p0=0.1, pmin=0.01, pmax=10.0, kpara0=1e-3, kret=0.0,
                      momentum_dependency=0, duu0=0.0, dt_min_rel=1e-3, dt_max_rel=1e-2,
                      nptl_max=200)
    oprm = oracle.params_from(prm)
    box = (0.3, 0.3, 0.3, 0.7, 0.7, 0.7) if ndim == 3 else (0.3, 0.3, 0.0, 0.7, 0.7, 1.0)
    parts, cnt = _inject(oprm, 200, box, 1.0)
    start = parts.view()
    dtf = 0.2
    oracle.mover(oprm, oracle.config_from(cfg), oracle.full_fields(frame, ndim, cfg), parts,
                 0.0, dtf, counters=cnt, focused_transport=True)
    end = parts.view()
    assert parts.n == 200
    np.testing.assert_allclose(end["x"] - start["x"], start["v"] * start["mu"] * dtf,
                               rtol=0, atol=1e-12)   # 10^3 rounded additions
    assert np.array_equal(end["y"], start["y"]) and np.array_equal(end["z"], start["z"])
    for k in ("p", "v", "mu"):
        assert np.array_equal(end[k], start[k]), k
    np.testing.assert_allclose(end["t"], dtf, rtol=1e-14)


def test_pitch_angle_scattering_stationary_law():
    """calc_duu's drift is duu0 [-2 mu dtmp + (1 - mu^2) |mu|^(gamma-2)]
    (mu > 0), which differs from dD_mumu/dmu by the factor (gamma - 1) on the
    second term.  The zero-flux solution of the Fokker-Planck equation of
    that Ito SDE is f(mu) ~ (|mu|^(gamma-1) + h0)^((2-gamma)/(gamma-1)), not
    the uniform law: for gamma = 5/3, <mu^2> = 0.3731 instead of 0.3267."""
    from scipy.integrate import quad
    n = 4000
    cfg = make_mhd_config(32, 32, 1, 0.0, 1.0, 0.0, 1.0)
    frame = _uniform_b_frame(32, 32)
    prm = make_params(ndim=2, p0=0.1, pmin=0.01, pmax=10.0, kpara0=1e-3, kret=0.0,
                      momentum_dependency=0, duu0=10.0, dt_min_rel=1e-4, dt_max_rel=1e-2,
                      nptl_max=n, seed=21)
    oprm = oracle.params_from(prm)
    parts, cnt = _inject(oprm, n, (0.0, 0.0, 0.0, 1.0, 1.0, 1.0), 1.0, mu=0.8)
    full = oracle.full_fields(frame, 2, cfg)
    for k in range(2):
        oracle.mover(oprm, oracle.config_from(cfg), full, parts, 0.5 * k, 0.5, counters=cnt,
                     focused_transport=True)
    mu = parts.view()["mu"]
    g, h0 = prm.gamma_turb, float(np.float32(0.2))
    mu_max = float(np.float32(0.99))
    law = lambda u: (u ** (g - 1.0) + h0) ** ((2.0 - g) / (g - 1.0))
    z = quad(law, 0.0, mu_max)[0]
    m2 = quad(lambda u: u * u * law(u), 0.0, mu_max)[0] / z
    m4 = quad(lambda u: u ** 4 * law(u), 0.0, mu_max)[0] / z
    sigma = math.sqrt((m4 - m2 * m2) / n)
    assert np.all(np.abs(mu) <= mu_max)
    assert abs(mu.mean()) < 4.0 * math.sqrt(m2 / n)
    assert abs((mu * mu).mean() - m2) < 4.0 * sigma
    assert abs((mu * mu).mean() - mu_max ** 2 / 3.0) > 4.0 * sigma   # not uniform
