"""Local and escaped distributions (calc_particle_distributions' flocal and
calc_escaped_distributions, diagnostics.f90:782-960) against the oracle."""
import numpy as np
import pytest

import oracle
from gpat import fields
from gpat.engine import Engine, make_mhd_config, make_params

pytestmark = pytest.mark.gpu


def _shock(n=64):
    db = fields.kolmogorov_az_2d(n, n, 1.0, 1.0, 0.5, 2 * np.pi, 16 * np.pi, 9)
    return fields.planar_shock_2d(n, n, 0.0, 1.0, 0.0, 1.0, r=3.5, w=0.02, db=db)


def _params(**kw):
    base = dict(ndim=2, p0=0.1, pmin=0.1, pmax=100.0, kpara0=4e-3, kret=0.1, dt_min_rel=2e-3,
                dt_max_rel=5e-2, pbcx=1, pbcy=1, momentum_dependency=0, nptl_max=20000, seed=5,
                npp_global=48)
    base.update(kw)
    return base


def test_escaped_distribution_matches_oracle_fp64():
    n = 64
    cfg = make_mhd_config(n, n, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.02)
    frame = _shock(n)
    prm = make_params(**_params())
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps(np.arange(4) * 0.02)
    eng.set_fields(frame, 0)
    eng.calc_fields_gradients(0)
    box = (0.0, 0.0, 0.0, 1.0, 1.0, 1.0)
    eng.inject_particles_spatial_uniform(5000, 1e-6, 2, 1.0, 1, box, power_index=3.0)
    start = eng.get_particles()
    esc = oracle.EscapedHistogram(prm.npp_global, prm.pmin, prm.pmax)
    try:
        parts = oracle.Particles(prm.nptl_max, start.arrays)
        cnt = oracle.OrcCounters()
        full = oracle.full_fields(frame, 2, cfg)
        for k in range(3):
            eng.particle_mover(mhd_tframe=k + 1, dump_escaped_dist=True)
            oracle.mover(oracle.params_from(prm), oracle.config_from(cfg), full, parts,
                         k * 0.02, 0.02, counters=cnt)
    finally:
        esc.detach()
    f, c = eng.calc_escaped_distributions()
    assert c.sum() > 100 and c.sum() <= cnt.nptl_escaped
    ref_c = esc.counts.reshape(6, -1)[:4]
    ref_f = esc.weights().reshape(6, -1)[:4]
    assert np.array_equal(c, ref_c)
    assert np.array_equal(f, ref_f)
    eng.reset_escaped_particles()
    f0, c0 = eng.calc_escaped_distributions()
    assert c0.sum() == 0 and f0.sum() == 0.0
    eng.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_local_distribution_matches_oracle(precision):
    n = 64
    cfg = make_mhd_config(n, n, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.02)
    frame = _shock(n)
    prm = make_params(**_params(precision=precision, pbcx=0, pbcy=0))
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps(np.arange(3) * 0.02)
    eng.set_fields(frame, 0)
    eng.calc_fields_gradients(0)
    box = (0.0, 0.0, 0.0, 1.0, 1.0, 1.0)
    eng.inject_particles_spatial_uniform(8000, 1e-6, 2, 1.0, 1, box, power_index=2.0)
    for k in range(2):
        eng.particle_mover(mhd_tframe=k + 1)
    ps = eng.get_particles()
    parts = oracle.Particles(len(ps), ps.arrays)
    for spec in [dict(pmin=0.1, pmax=10.0, npbins=12, rx=4, ry=4, rz=1),
                 dict(pmin=0.05, pmax=5.0, npbins=7, rx=16, ry=8, rz=1)]:
        f, c = eng.local_distribution(**spec)
        nrx, nry = (n + spec["rx"] - 1) // spec["rx"], (n + spec["ry"] - 1) // spec["ry"]
        assert f.shape == (1, nry, nrx, spec["npbins"], 1)
        rf, rc = oracle.local_distribution(oracle.config_from(cfg), 2, parts, spec["pmin"],
                                           spec["pmax"], spec["npbins"], 1, spec["rx"],
                                           spec["ry"], spec["rz"])
        assert np.array_equal(c.ravel(), rc) and np.array_equal(f.ravel(), rf)
        assert c[..., -1, :].sum() == 0           # the last p bin stays empty (ip < npbins)
        assert 0 < c.sum() <= len(ps)
    eng.close()
