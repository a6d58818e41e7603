"""Injection where a field quantity is large: CUDA engine against the
oracle through the C ABI (cell counts and injected particles bit-exact)."""
import numpy as np
import pytest

import oracle
from gpat import fields
from gpat.engine import Engine, GPATError, make_mhd_config, make_params

pytestmark = pytest.mark.gpu

KEYS = ("x", "y", "z", "p", "v", "mu", "t", "dt", "weight", "tag_injected", "tag_splitted",
        "count_flag")


def _engine(ndim):
    if ndim == 2:
        n = 48
        cfg = make_mhd_config(n, n, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.1)
        db = fields.kolmogorov_az_2d(n, n, 1.0, 1.0, 0.5, 2 * np.pi, 16 * np.pi, 3)
        frame = fields.planar_shock_2d(n, n, 0.0, 1.0, 0.0, 1.0, r=3.0, w=0.03, db=db)
    else:
        n = 20
        cfg = make_mhd_config(n, n, n, 0.0, 1.0, 0.0, 1.0, zmin=0.0, zmax=1.0, dt_out=0.1,
                              ndim=3)
        frame = fields.turbulence_3d(n, seed=6)
    prm = make_params(ndim=ndim, p0=0.1, pmin=0.01, pmax=10.0, nptl_max=20000, seed=23)
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps([0.0, 0.1, 0.2])
    eng.set_fields(frame, 0)
    eng.calc_fields_gradients(0)
    return eng, cfg, oracle.full_fields(frame, ndim, cfg), oracle.params_from(prm)


@pytest.mark.parametrize("ndim", [2, 3])
@pytest.mark.parametrize("quantity", [0, 1, 2, 3])
def test_large_quantity_injection_bit_exact(ndim, quantity):
    eng, cfg, full, oprm = _engine(ndim)
    ocfg = oracle.config_from(cfg)
    box = (0.1, 0.2, 0.15, 0.9, 0.8, 0.85)
    # threshold with about 30 % of the box's nodes above it
    total = oracle.count_cells_large(oprm, ocfg, full, quantity, -1e30, box)
    lo, hi = -1e3, 1e3
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        if oracle.count_cells_large(oprm, ocfg, full, quantity, mid, box) >= 0.3 * total:
            lo = mid
        else:
            hi = mid
    qmin = lo
    for thr in (qmin, 0.5 * qmin):
        assert eng.count_cells_large(quantity, thr, box) == \
            oracle.count_cells_large(oprm, ocfg, full, quantity, thr, box)
    ncells = eng.count_cells_large(quantity, qmin, box)
    n = eng.inject_particles_at_large(quantity, 3000, 1e-6, 2, 1.5, 1, False, qmin, 400, box,
                                      power_index=3.0)
    assert n == int(3000 * (ncells / 400))
    n2 = eng.inject_particles_at_large(quantity, 700, 1e-6, 1, 1.5, 2, True, qmin, 1, box)
    assert n2 == (700 if ncells > 0 else 0)
    got = eng.get_particles()
    parts = oracle.Particles(20000)
    cnt = oracle.OrcCounters()
    oracle.inject_at_large(oprm, ocfg, full, parts, n, 1e-6, 2, 1.5, 0.0, 0.1, quantity, qmin,
                           box, cnt, power_index=3.0)
    oracle.inject_at_large(oprm, ocfg, full, parts, n2, 1e-6, 1, 1.5, 0.1, 0.1, quantity, qmin,
                           box, cnt)
    ref = parts.view()
    assert len(got) == parts.n == n + n2
    for k in KEYS:
        if k in ("p", "v"):   # power-law momenta go through pow()
            np.testing.assert_allclose(got[k], ref[k], rtol=2e-15)
        else:
            assert np.array_equal(got[k], ref[k]), k
    eng.close()


def test_large_quantity_rejects_bad_arguments():
    eng, cfg, full, oprm = _engine(2)
    with pytest.raises(GPATError):
        eng.count_cells_large(7, 0.0, (0, 0, 0, 1, 1, 1))
    with pytest.raises(GPATError):
        eng.inject_particles_at_large(0, 10, 1e-6, 1, 1.0, 1, False, 0.1, 0, (0, 0, 0, 1, 1, 1))
    eng.close()
