"""Spatially dependent turbulence variance and correlation length
(deltab_flag, correlation_flag) in the CPU oracle: known answers (no GPU).

calc_grad_sigma2_* / calc_grad_lc_* (mhd_data_parallel.f90:771-1604) are
exact on linear data and leave the z component of 2D records at its
initial 1; calc_spatial_diffusion_coefficients (particle_module.f90:
2208-2450) divides kappa_par by dB^2 and multiplies it by Lc^(gamma-1),
which a uniform field shows in the diffusion covariance.
"""
import ctypes as C
import math

import numpy as np
import pytest

import oracle
from gpat import fields
from gpat.engine import make_mhd_config, make_params


def test_aux_gradients_linear_and_2d_z_component():
    nx, ny = 24, 16
    cfg = make_mhd_config(nx, ny, 1, 0.0, 1.0, 0.0, 1.0)
    x = fields.node_coords(nx, 0.0, 1.0 / nx)
    y = fields.node_coords(ny, 0.0, 1.0 / ny)
    X, Y = np.meshgrid(x, y)
    db2 = (0.5 + 0.25 * X - 0.75 * Y)[None].astype(np.float32)
    lc = (2.0 + X)[None].astype(np.float32)
    aux = oracle.aux_fields(db2, None, lc, None, 2, cfg)
    np.testing.assert_allclose(aux[..., 1], 0.25, atol=2e-5)
    np.testing.assert_allclose(aux[..., 2], -0.75, atol=2e-5)
    np.testing.assert_allclose(aux[..., 9], 1.0, atol=2e-5)
    assert np.all(aux[..., 3] == 1.0)            # 2D: d/dz keeps the initial 1
    assert np.all(aux[..., 4] == 1.0) and np.all(aux[..., 5] == 0.0)   # db2_2d left at 1


def _kappa(prm, aux16, p=0.1, mu=0.5):
    f = (C.c_double * 32)()
    f[4] = 1.0
    k = (C.c_double * 22)()
    a = (C.c_double * 16)(*aux16)
    oracle.load().orc_calc_spatial_diffusion_coefficients(C.byref(prm), p, mu, f, a, k)
    return list(k)


def test_kappa_scales_with_variance_and_correlation_length():
    prm = oracle.params_from(make_params(ndim=2, kpara0=0.02, kret=0.1, momentum_dependency=0))
    aux = [1.0] * 16
    aux[0], aux[8] = 4.0, 2.0
    g = prm.gamma_turb
    prm.deltab_flag, prm.correlation_flag = 1, 0
    assert _kappa(prm, aux)[2] == pytest.approx(0.02 / 4.0, rel=1e-15)
    prm.deltab_flag, prm.correlation_flag = 0, 1
    assert _kappa(prm, aux)[2] == pytest.approx(0.02 * 2.0 ** (g - 1.0), rel=1e-14)
    prm.deltab_flag = 1
    assert _kappa(prm, aux)[2] == pytest.approx(0.02 / 4.0 * 2.0 ** (g - 1.0), rel=1e-14)
    # NLGC: kperp ~ db2_slab^(-1/3) db2_2d^(2/3) lc_slab^((g-1)/3) lc_2d^(2/3)
    prm.nlgc, prm.kperp_kpara = 1, 0.01
    aux[4], aux[12] = 9.0, 3.0
    want = 0.02 * 0.01 * 0.25 * 4.0 ** (-1 / 3) * 9.0 ** (2 / 3) * 2.0 ** ((g - 1) / 3) * 3.0 ** (2 / 3)
    assert _kappa(prm, aux, mu=0.5)[3] == pytest.approx(want, rel=1e-13)


def test_uniform_variance_reduces_the_diffusion_covariance():
    n = 48
    cfg = make_mhd_config(n, n, 1, 0.0, 1.0, 0.0, 1.0)
    z = np.zeros((n + 4, n + 4))
    frame = fields.assemble_frame(z, z, z, z + 1, z + 1.0, z, z)[None]
    kpara, T, N = 4e-3, 0.05, 4000
    prm = make_params(ndim=2, kpara0=kpara, kret=0.0, momentum_dependency=0, dt_min_rel=0.01,
                      pbcx=0, pbcy=0, p0=0.1, deltab_flag=1, nptl_max=N, seed=3)
    oprm = oracle.params_from(prm)
    aux = oracle.aux_fields(np.full((1, n + 4, n + 4), 4.0, np.float32), None, None, None, 2, cfg)
    parts = oracle.Particles(N)
    a = parts.a
    a["x"][:] = 0.5; a["y"][:] = 0.5; a["p"][:] = 0.1; a["weight"][:] = 1.0
    a["count_flag"][:] = 1; a["tag_splitted"][:] = 1; a["tag_injected"][:N] = np.arange(N)
    parts.n = N
    oracle.mover(oprm, oracle.config_from(cfg), oracle.full_fields(frame, 2, cfg), parts, 0.0, T,
                 aux1=aux)
    dx = parts.view()["x"] - 0.5
    var = np.mean(dx * dx)
    want = 2.0 * (kpara / 4.0) * T
    assert abs(var - want) < 5.0 * math.sqrt(2.0 / N) * want
