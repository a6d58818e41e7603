"""Split-precision mover in 3D: the noise decomposition P P^T = 2 kappa
(push_particle_3d, particle_module.f90:4870-4877) and f(p) agreement with
the FP64 mover on compressible turbulence."""
import math

import numpy as np
import pytest

from gpat import configs, fields
from gpat.engine import Engine, ParticleSet, make_mhd_config, make_params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
def test_diffusion_covariance_3d(precision):
    n = 32
    cfg = make_mhd_config(n, n, n, 0.0, 1.0, 0.0, 1.0, zmin=0.0, zmax=1.0, dt_out=0.04, ndim=3)
    b = np.array([0.4, -0.3, 0.866])
    b = b / np.linalg.norm(b)
    shape = (n + 4, n + 4, n + 4)
    z = np.zeros(shape)
    frame = fields.assemble_frame(z, z, z, z + 1, z + b[0], z + b[1], z + b[2])
    kpara, kret, T = 1e-3, 0.1, 0.04
    N = 200000 if precision else 40000
    eng = Engine(make_params(ndim=3, kpara0=kpara, kret=kret, momentum_dependency=0,
                             dt_min_rel=0.01, pbcx=0, pbcy=0, pbcz=0, p0=0.1,
                             precision=precision, nptl_max=N, seed=17), cfg, 0)
    eng.set_tstamps([0.0, T])
    eng.set_fields(frame, 0)
    eng.calc_fields_gradients(0)
    ps = ParticleSet.empty(N)
    for k in ("x", "y", "z"):
        ps.arrays[k][:] = 0.5
    ps.arrays["p"][:] = 0.1
    ps.arrays["weight"][:] = 1.0
    ps.arrays["count_flag"][:] = 1
    ps.arrays["tag_splitted"][:] = 1
    ps.arrays["tag_injected"][:] = np.arange(N, dtype=np.int32)
    eng.put_particles(ps)
    eng.particle_mover(mhd_tframe=1)
    out = eng.get_particles()
    d = np.stack([out["x"] - 0.5, out["y"] - 0.5, out["z"] - 0.5])
    cov = d @ d.T / N
    K = kpara * kret * np.eye(3) + kpara * (1 - kret) * np.outer(b, b)
    np.testing.assert_allclose(cov, 2 * K * T, atol=5 * math.sqrt(2.0 / N) * 2 * K.max() * T)
    eng.close()


def test_mixed_vs_fp64_spectrum_3d_turbulence():
    w = configs.turbulence_3d(scale=3e-4, n=32, nframes=4)
    hists = {}
    for prec in (0, 1):
        eng = configs.build_engine(w, precision=prec, nptl_max=w.nptl, npp_global=24)
        configs.inject(eng, w)
        for k in range(4):
            eng.particle_mover(mhd_tframe=k + 1)
        f, c = eng.calc_particle_distributions()
        hists[prec] = c.astype(float)
        assert eng.counters().nptl_current == w.nptl     # periodic box: nobody escapes
        eng.close()
    a, b = hists[0], hists[1]
    m = (a + b) > 20
    chi2 = float(np.sum((a[m] - b[m]) ** 2 / (a[m] + b[m])))
    dof = int(m.sum())
    assert chi2 < dof + 4 * math.sqrt(2 * dof) + 10, (chi2, dof)
