"""Golden vectors (tests/golden/*.npz, made by tests/golden/make_golden.py).

CPU: the oracle reproduces its committed outputs bit for bit.
GPU: the CUDA engine reproduces them through the C ABI.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle
from gpat.engine import Engine, ParticleSet, make_mhd_config, make_params

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = {
    "mover2d": dict(ndim=2, n=24, p0=0.1, pmin=0.1, pmax=100.0, kpara0=3e-3, kret=0.1,
                    dt_min_rel=5e-3, dt_max_rel=5e-2, pbcx=1, pbcy=0, momentum_dependency=0,
                    seed=99, nptl=256, fine=3, intervals=2, dt_out=0.02),
    "mover3d": dict(ndim=3, n=12, p0=0.1, pmin=0.1, pmax=100.0, kpara0=2e-3, kret=0.05,
                    dt_min_rel=1e-2, dt_max_rel=5e-2, pbcx=0, pbcy=1, pbcz=0,
                    momentum_dependency=0, seed=77, nptl=128, fine=2, intervals=1, dt_out=0.02),
}
FIELDS = [k for k, _ in oracle.FIELDS]


def _setup(name):
    case = CASES[name]
    g = np.load(GOLDEN / f"{name}.npz")
    ndim, n = case["ndim"], case["n"]
    cfg = make_mhd_config(n, n, n if ndim == 3 else 1, 0.0, 1.0, 0.0, 1.0, dt_out=case["dt_out"],
                          ndim=ndim)
    keys = ("p0", "pmin", "pmax", "kpara0", "kret", "dt_min_rel", "dt_max_rel", "pbcx", "pbcy",
            "pbcz", "momentum_dependency", "seed")
    prm = make_params(ndim=ndim, nptl_max=4 * case["nptl"],
                      **{k: case[k] for k in keys if k in case})
    return case, g, cfg, prm


def _by_tags(d):
    return ParticleSet(d).order_by_tags()


def test_philox_table():
    t = np.load(GOLDEN / "philox.npz")["table"]
    for row in t:
        assert oracle.philox(list(row[:4]), list(row[4:6])) == list(row[6:10])


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_golden(name):
    case, g, cfg, prm = _setup(name)
    full = oracle.full_fields(g["frame"], case["ndim"], cfg)
    assert np.array_equal(full, g["full"])
    start = {k: g[f"start_{k}"] for k in FIELDS}
    parts = oracle.Particles(4 * case["nptl"], start)
    cnt = oracle.OrcCounters()
    oprm, ocfg = oracle.params_from(prm), oracle.config_from(cfg)
    for k in range(case["intervals"]):
        oracle.mover(oprm, ocfg, full, parts, k * case["dt_out"], case["dt_out"],
                     num_fine_steps=case["fine"], counters=cnt, nthreads=3)
    got = parts.view()
    for k in FIELDS:
        assert np.array_equal(got[k], g[f"end_{k}"]), k
    assert list(g["counters"]) == [cnt.leak_hi, cnt.leak_lo, cnt.leak_negp_hi, cnt.leak_negp_lo,
                                   cnt.steps, cnt.nptl_escaped]
    f, c = oracle.histogram(oprm, parts)
    assert np.array_equal(f, g["fglobal"]) and np.array_equal(c, g["counts"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_engine_reproduces_golden(name):
    case, g, cfg, prm = _setup(name)
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps(np.arange(case["intervals"] + 1) * case["dt_out"])
    eng.set_fields(g["frame"], 0)
    eng.calc_fields_gradients(0)
    assert np.array_equal(eng.get_fields(0), g["full"])
    eng.put_particles(ParticleSet({k: np.ascontiguousarray(g[f"start_{k}"]) for k in FIELDS}))
    for k in range(case["intervals"]):
        eng.particle_mover(nsteps_interval=10, mhd_tframe=k + 1, num_fine_steps=case["fine"])
    got = eng.get_particles().order_by_tags()
    ref = _by_tags({k: g[f"end_{k}"] for k in FIELDS})
    for k in FIELDS:
        if k == "nsteps_tracked":
            continue   # set to 1 by every mover call, as the reference does
        assert np.array_equal(got[k], ref[k]), k
    c = eng.counters()
    cg = g["counters"]
    assert [c.leak_hi, c.leak_lo, c.leak_negp_hi, c.leak_negp_lo, c.steps, c.nptl_escaped] == \
        [int(v) for v in cg]
    f, counts = eng.calc_particle_distributions()
    assert np.array_equal(f, g["fglobal"]) and np.array_equal(counts, g["counts"])
    eng.close()
