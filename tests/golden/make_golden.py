"""Generates tests/golden/*.npz from the CPU oracle.

The reference has no tests or fixtures, so these vectors are the oracle's own
outputs on fixed inputs.  They pin the oracle against regressions and give the
GPU tests fixed expected values.  Inputs (frames, particles) are stored in the
files too, so nothing depends on numpy's FFT rounding on the machine that
reads them.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
for p in (str(REPO / "stochastic-parker_gb300"), str(REPO / "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

import oracle  # noqa: E402
from gpat import fields  # noqa: E402
from gpat.engine import make_mhd_config, make_params  # noqa: E402

CASES = {
    "mover2d": dict(ndim=2, n=24, p0=0.1, pmin=0.1, pmax=100.0, kpara0=3e-3, kret=0.1,
                    dt_min_rel=5e-3, dt_max_rel=5e-2, pbcx=1, pbcy=0, momentum_dependency=0,
                    seed=99, nptl=256, fine=3, intervals=2, dt_out=0.02),
    "mover3d": dict(ndim=3, n=12, p0=0.1, pmin=0.1, pmax=100.0, kpara0=2e-3, kret=0.05,
                    dt_min_rel=1e-2, dt_max_rel=5e-2, pbcx=0, pbcy=1, pbcz=0,
                    momentum_dependency=0, seed=77, nptl=128, fine=2, intervals=1, dt_out=0.02),
}


def philox_table():
    rows = []
    for c0 in (0, 1, 0xFFFFFFFF):
        for c1 in (0, 2):
            for key in ((0, 0), (0x5EED0001, 0), (0xDEADBEEF, 0x12345678)):
                ctr = [c0, c1, 7, 1]
                rows.append(ctr + list(key) + oracle.philox(ctr, list(key)))
    return np.array(rows, dtype=np.uint32)


def frame_for(case):
    n = case["n"]
    if case["ndim"] == 2:
        db = fields.kolmogorov_az_2d(n, n, 1.0, 1.0, 0.5, 2 * np.pi, 8 * np.pi, seed=5)
        return fields.planar_shock_2d(n, n, 0.0, 1.0, 0.0, 1.0, r=3.0, w=0.05, db=db)
    return fields.turbulence_3d(n, seed=11)


def run_case(name, case):
    ndim, n = case["ndim"], case["n"]
    cfg = make_mhd_config(n, n, n if ndim == 3 else 1, 0.0, 1.0, 0.0, 1.0, dt_out=case["dt_out"],
                          ndim=ndim)
    keys = ("p0", "pmin", "pmax", "kpara0", "kret", "dt_min_rel", "dt_max_rel", "pbcx", "pbcy",
            "pbcz", "momentum_dependency", "seed")
    prm = make_params(ndim=ndim, nptl_max=4 * case["nptl"],
                      **{k: case[k] for k in keys if k in case})
    oprm = oracle.params_from(prm)
    ocfg = oracle.config_from(cfg)
    frame = frame_for(case)
    full = oracle.full_fields(frame, ndim, cfg)
    parts = oracle.Particles(4 * case["nptl"])
    cnt = oracle.OrcCounters()
    box = (0.0, 0.0, 0.0, 1.0, 1.0, 1.0)
    oracle.inject_spatial_uniform(oprm, parts, case["nptl"], 1e-6, 1, 1.0, 0.0, case["dt_out"],
                                  box, cnt)
    start = parts.view()
    for k in range(case["intervals"]):
        oracle.mover(oprm, ocfg, full, parts, k * case["dt_out"], case["dt_out"],
                     num_fine_steps=case["fine"], counters=cnt, nthreads=1)
    end = parts.view()
    out = {"frame": frame, "full": full}
    out.update({f"start_{k}": v for k, v in start.items()})
    out.update({f"end_{k}": v for k, v in end.items()})
    out["counters"] = np.array([cnt.leak_hi, cnt.leak_lo, cnt.leak_negp_hi, cnt.leak_negp_lo,
                                cnt.steps, cnt.nptl_escaped], dtype=np.uint64)
    f, c = oracle.histogram(oprm, parts)
    out["fglobal"], out["counts"] = f, c
    np.savez_compressed(HERE / f"{name}.npz", **out)


def main():
    np.savez_compressed(HERE / "philox.npz", table=philox_table())
    for name, case in CASES.items():
        run_case(name, case)
    print("wrote", sorted(p.name for p in HERE.glob("*.npz")))


if __name__ == "__main__":
    main()
