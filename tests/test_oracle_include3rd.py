"""2D runs with transport along the third dimension (include_3rd_dim) in the
CPU oracle (no GPU): with uniform fields the particles diffuse with the full
3D tensor K = kperp I + (kpara - kperp) b b, so the covariance of (x, y, z)
after t is 2 K t, and a uniform vz carries them along z
(push_particle_2d_include_3rd, particle_module.f90:3979-4266)."""
import math

import numpy as np

import oracle
from gpat import fields
from gpat.engine import make_mhd_config, make_params


def _start(n, x, y, z):
    a = {k: np.zeros(n, dtype=t) for k, t in oracle.FIELDS}
    a["weight"][:] = 1.0
    a["count_flag"][:] = 1
    a["tag_splitted"][:] = 1
    a["tag_injected"][:] = np.arange(n, dtype=np.int32)
    a["x"][:], a["y"][:], a["z"][:], a["p"][:] = x, y, z, 0.1
    return a


def _uniform(nx, ny, v, b):
    shape = (1, ny + 4, nx + 4)
    z = np.zeros(shape)
    return fields.assemble_frame(z + v[0], z + v[1], z + v[2], z + 1.0, z + b[0], z + b[1],
                                 z + b[2]).astype(np.float32)


def test_include_3rd_dim_covariance_and_drift():
    n = 32
    cfg = make_mhd_config(n, n, 1, 0.0, 1.0, 0.0, 1.0, zmin=0.0, zmax=1.0, dt_out=1.0)
    b = (0.5, 0.4, 0.7)
    vz = 0.05
    prm = oracle.params_from(make_params(ndim=2, p0=0.1, pmin=0.05, pmax=10.0, kpara0=2e-4,
                                         kret=0.2, momentum_dependency=0, pbcx=0, pbcy=0,
                                         pbcz=0, dt_min_rel=1e-3, dt_max_rel=0.05,
                                         include_3rd_dim=1))
    full = oracle.full_fields(_uniform(n, n, (0.0, 0.0, vz), b), 2, cfg)
    N = 40000
    parts = oracle.Particles(N, _start(N, 0.5, 0.5, 0.3))
    oracle.mover(prm, oracle.config_from(cfg), full, parts, 0.0, 1.0)
    out = parts.view()
    assert len(out["x"]) == N
    D = np.stack([out["x"] - 0.5, out["y"] - 0.5, out["z"] - 0.3 - vz])
    kpara, kperp = 2e-4, 4e-5
    bn = np.array(b) / np.linalg.norm(b)
    K = kperp * np.eye(3) + (kpara - kperp) * np.outer(bn, bn)
    cov = np.cov(D)
    scale = np.sqrt(np.outer(np.diag(2 * K), np.diag(2 * K)))
    assert np.all(np.abs(cov - 2 * K) < 6 * scale * math.sqrt(2.0 / N)), (cov, 2 * K)
    err = np.sqrt(np.diag(2 * K) / N)
    assert np.all(np.abs(D.mean(axis=1)) < 6 * err)


def test_without_include_3rd_dim_z_stays():
    n = 32
    cfg = make_mhd_config(n, n, 1, 0.0, 1.0, 0.0, 1.0, zmin=0.0, zmax=1.0, dt_out=1.0)
    prm = oracle.params_from(make_params(ndim=2, p0=0.1, pmin=0.05, pmax=10.0, kpara0=2e-4,
                                         kret=0.2, momentum_dependency=0, pbcx=0, pbcy=0,
                                         dt_min_rel=1e-3, dt_max_rel=0.05))
    full = oracle.full_fields(_uniform(n, n, (0.0, 0.0, 0.05), (0.5, 0.4, 0.7)), 2, cfg)
    parts = oracle.Particles(1000, _start(1000, 0.5, 0.5, 0.3))
    oracle.mover(prm, oracle.config_from(cfg), full, parts, 0.0, 1.0)
    assert np.all(parts.view()["z"] == 0.3)
