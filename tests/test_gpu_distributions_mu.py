"""Distributions with pitch-angle bins and local escaped distributions: the
CUDA engine against the oracle through the C ABI on FP64 runs with open
boundaries (2D and 3D, so every face is exercised).  Counts and the exact
fixed-point weight sums match bit for bit."""
import numpy as np
import pytest

import oracle
from gpat import fields
from gpat.engine import Engine, make_mhd_config, make_params
from test_gpu_parity import shock_case, turbulent_frame_2d

pytestmark = pytest.mark.gpu


def _run_2d():
    params, cfg = shock_case(pbcx=1, pbcy=1, kpara0=2e-2, precision=0, nptl_max=8000)
    prm = make_params(**params)
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps(np.arange(4) * 0.02)
    eng.set_fields(turbulent_frame_2d(), 0)
    eng.calc_fields_gradients(0)
    eng.inject_particles_spatial_uniform(4000, 1e-6, 1, 1.0, 1, (0, 0, 0, 1, 1, 1))
    for k in range(2):
        eng.particle_mover(mhd_tframe=k + 1, dump_escaped_dist=True)
    return eng, prm, cfg


def _run_3d():
    n = 20
    cfg = make_mhd_config(n, n, n, 0.0, 1.0, 0.0, 1.0, zmin=0.0, zmax=1.0, dt_out=0.02, ndim=3)
    prm = make_params(ndim=3, p0=0.1, pmin=0.05, pmax=100.0, kpara0=2e-2, kret=0.1,
                      dt_min_rel=2e-3, dt_max_rel=5e-2, pbcx=1, pbcy=1, pbcz=1,
                      momentum_dependency=0, nptl_max=6000, seed=17, precision=0)
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps(np.arange(4) * 0.02)
    eng.set_fields(fields.turbulence_3d(n, seed=6), 0)
    eng.calc_fields_gradients(0)
    eng.inject_particles_spatial_uniform(3000, 1e-6, 1, 1.0, 1, (0, 0, 0, 1, 1, 1))
    eng.particle_mover(mhd_tframe=1, dump_escaped_dist=True)
    return eng, prm, cfg


@pytest.mark.parametrize("ndim", [2, 3])
def test_mu_and_local_escaped_distributions_match_oracle(ndim):
    eng, prm, cfg = _run_2d() if ndim == 2 else _run_3d()
    oprm, ocfg = oracle.params_from(prm), oracle.config_from(cfg)
    live = eng.get_particles()
    esc = eng.get_escaped_particles()
    assert len(esc) > 50
    f, c = eng.particle_distributions_mu(5)
    fo, co = oracle.distribution_mu(oprm, oracle.Particles(len(live) + 1, live.arrays), 5)
    assert np.array_equal(c.ravel(), co) and c.sum() > 0
    assert np.array_equal(f.ravel(), fo)
    fe, ce = eng.escaped_distributions_mu(4)
    eparts = oracle.Particles(len(esc) + 1, esc.arrays)
    feo, ceo = oracle.distribution_mu(oprm, eparts, 4, by_face=True, nfaces=2 * ndim)
    assert np.array_equal(ce.ravel(), ceo) and ce.sum() > 0
    assert np.array_equal(fe.ravel(), feo)
    spec = dict(pmin=0.05, pmax=10.0, npbins=8, nmu=3, rx=4, ry=2, rz=5)
    (fx, fy, fz), (cx, cy, cz) = eng.local_escaped_distribution(**spec)
    ref = oracle.local_escaped_distribution(ocfg, ndim, eparts, 0.05, 10.0, 8, 3, 4, 2, 5)
    got = [(fx, cx), (fy, cy), (fz, cz)]
    for k in range(3):
        if k >= ndim:
            assert got[k][0] is None and ref[k] is None
            continue
        assert np.array_equal(got[k][1].ravel(), ref[k][1]), k
        assert np.array_equal(got[k][0].ravel(), ref[k][0]), k
    assert sum(int(g[1].sum()) for g in got[:ndim]) > 0
    eng.close()
