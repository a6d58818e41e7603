"""f(p) agreement of the split-precision mover with the FP64 mover.

Both movers start from the same injected particles (injection is
deterministic) and run the same intervals with splitting; their noise streams
are independent, so the comparison carries Monte Carlo error.  The FP64 GPU
mover is bit-identical to the CPU oracle on these paths (tests/
test_gpu_parity.py), so it serves as the FP64 oracle at sizes the CPU would
take minutes for.

tail error: relative difference of the weighted counts summed over the top
decade of populated p of the FP64 run, with its standard error
sqrt(sum w^2 over both runs) / W_fp64.  Per-bin differences and a chi-square
over bins with enough particles are reported too.
"""
from __future__ import annotations

import math

import numpy as np

from . import configs


def _spectrum(eng, edges):
    ps = eng.get_particles()
    p, w = ps["p"], ps["weight"]
    npp = len(edges) - 1
    lo = math.log10(edges[0])
    d = (math.log10(edges[-1]) - lo) / npp
    ok = (p > edges[0]) & (p <= edges[-1])
    ib = np.floor((np.log10(p[ok]) - lo) / d).astype(np.int64)
    keep = (ib >= 0) & (ib < npp)
    ib, ww = ib[keep], w[ok][keep]
    f = np.bincount(ib, weights=ww, minlength=npp)
    f2 = np.bincount(ib, weights=ww * ww, minlength=npp)
    c = np.bincount(ib, minlength=npp)
    return f, f2, c


def compare(workload: configs.Workload, intervals: int, split=(2.72, 2.0),
            device: int = 0, tiles=None) -> dict:
    """Runs the workload in FP64 and split precision; returns the tail error.
    tiles: gpat_set_mover_tiles arguments for the split-precision run."""
    out = {}
    for prec in (0, 1):
        eng = configs.build_engine(workload, device=device, precision=prec,
                                   nptl_max=int(workload.nptl * 8))
        if prec == 1 and tiles:
            eng.set_mover_tiles(*tiles)
        configs.inject(eng, workload)
        for k in range(intervals):
            eng.particle_mover(nsteps_interval=10, mhd_tframe=k + 1, num_fine_steps=1)
            if split:
                eng.split_particle(split[0], split[1], 10)
        edges = eng.pbins_edges()
        f_dev, _ = eng.calc_particle_distributions()
        f, f2, c = _spectrum(eng, edges)
        out[prec] = dict(f=f, f2=f2, c=c, f_dev=f_dev, n=eng.nptl_current,
                         steps=eng.counters().steps)
        eng.close()
    return tail_stats(out[0], out[1], workload.params["pmin"], workload.params["pmax"])


def spectrum(eng) -> dict:
    """Weighted f(p), sum of w^2 and counts on the engine's bins."""
    edges = eng.pbins_edges()
    f_dev, _ = eng.calc_particle_distributions()
    f, f2, c = _spectrum(eng, edges)
    return dict(f=f, f2=f2, c=c, f_dev=f_dev, n=eng.nptl_current, steps=eng.counters().steps)


def subset_spectrum(eng, max_tag: int) -> dict:
    """f(p) of the particles injected with tag_injected <= max_tag (split
    children share their parent's injection tag); a tracked particle's tag
    is negated, hence the absolute value."""
    edges = eng.pbins_edges()
    ps = eng.get_particles()
    keep = np.abs(ps["tag_injected"].astype(np.int64)) <= max_tag
    p, w = ps["p"][keep], ps["weight"][keep]
    npp = len(edges) - 1
    lo = math.log10(edges[0])
    d = (math.log10(edges[-1]) - lo) / npp
    ok = (p > edges[0]) & (p <= edges[-1])
    ib = np.floor((np.log10(p[ok]) - lo) / d).astype(np.int64)
    sel = (ib >= 0) & (ib < npp)
    ib, ww = ib[sel], w[ok][sel]
    f = np.bincount(ib, weights=ww, minlength=npp)
    f2 = np.bincount(ib, weights=ww * ww, minlength=npp)
    c = np.bincount(ib, minlength=npp)
    return dict(f=f, f2=f2, c=c, f_dev=f, n=int(keep.sum()), steps=0)


def batched_runs_check(runs, engines, intervals: int, sample: int = 20000,
                       device: int = 0) -> list:
    """Per-run tail error of batched split-precision runs against FP64 runs
    of the same injected particles.  Injection draws are keyed by particle
    tag, so an FP64 run that injects the first `sample` particles starts
    from exactly the first `sample` particles of the batched run; each run's
    f(p) of those particles (children included) after `intervals` intervals
    with splitting is compared with the FP64 run's."""
    out = []
    for w, e in zip(runs, engines):
        s = min(sample, w.nptl)
        mixed = subset_spectrum(e, s)
        e64 = configs.build_engine(w, device=device, precision=0, nptl_max=16 * s + 64)
        configs.inject(e64, w, nptl=s)
        for k in range(intervals):
            e64.particle_mover(nsteps_interval=10, mhd_tframe=k + 1, num_fine_steps=1)
            if w.split:
                e64.split_particle(w.split["ratio"], w.split["pmin"], 10)
        ref = spectrum(e64)
        e64.close()
        try:
            t = tail_stats(ref, mixed, w.params["pmin"], w.params["pmax"])
        except RuntimeError:
            continue
        out.append({"run": w.name, "particles": w.nptl, "sample": s, "tail_err": t["tail_err"],
                    "tail_err_sigma": t["tail_err_sigma"], "top_decade_p": t["top_decade_p"],
                    "chi2": t["chi2"], "chi2_dof": t["chi2_dof"]})
    return out


def tail_stats(a: dict, b: dict, pmin: float, pmax: float) -> dict:
    """Tail error of spectrum b against the FP64 spectrum a."""
    populated = np.nonzero(a["c"])[0]
    if len(populated) == 0:
        raise RuntimeError("FP64 run has an empty spectrum")
    b_hi = int(populated[-1])
    edges = np.logspace(math.log10(pmin), math.log10(pmax), len(a["f"]) + 1)
    p_hi = edges[b_hi + 1]
    top = np.arange(len(a["f"])) [(edges[:-1] >= p_hi / 10.0) & (np.arange(len(a["f"])) <= b_hi)]
    w64, wmx = a["f"][top].sum(), b["f"][top].sum()
    sig = math.sqrt(a["f2"][top].sum() + b["f2"][top].sum()) / w64
    m = (a["c"] + b["c"]) >= 20
    chi2 = float(np.sum((a["f"][m] - b["f"][m]) ** 2 / (a["f2"][m] + b["f2"][m])))
    per_bin = np.where(a["f"] > 0, (b["f"] - a["f"]) / np.where(a["f"] > 0, a["f"], 1.0), 0.0)
    return {
        "tail_err": float((wmx - w64) / w64), "tail_err_sigma": sig,
        "top_decade_p": [float(p_hi / 10.0), float(p_hi)],
        "top_decade_particles_fp64": int(a["c"][top].sum()),
        "chi2": chi2, "chi2_dof": int(m.sum()),
        "per_bin_rel_err_top": [float(x) for x in per_bin[top]],
        "nptl_fp64": a["n"], "nptl_mixed": b["n"],
        "steps_fp64": int(a["steps"]), "steps_mixed": int(b["steps"]),
        # the device histogram against a host binning of the same particles
        "device_hist_matches": bool(np.array_equal(a["f_dev"], a["f"])),
    }


def planar_shock_check(scale: float = 1.0, t_end: float = 2.0, device: int = 0) -> dict:
    """The planar-shock workload (512x64, r = 4) to t_end with splitting."""
    w = configs.planar_shock(scale=scale, t_end=t_end)
    r = compare(w, w.nframes, split=(2.72, 2.0), device=device)
    r["workload"] = f"{w.name}, {w.nptl} particles injected, t = {t_end}, split 2.72 / 2.0"
    return r


def turbulent_shock_check(scale: float = 0.1, intervals: int = 25, device: int = 0,
                          tiles=None) -> dict:
    """The benchmarked 2048^2 turbulent shock (r = 3.5, dB/B0 = 0.5, 1000
    pushes per particle per interval) on a sample of scale x 1e7 particles,
    both precisions from the same injection, with splitting."""
    w = configs.turbulent_shock_2d(scale=scale, nframes=intervals + 1)
    r = compare(w, intervals, split=(w.split["ratio"], w.split["pmin"]), device=device,
                tiles=tiles)
    r["workload"] = (f"{w.name}, {w.nptl} particles injected, {intervals} intervals "
                     f"(t = {intervals * (w.tstamps[1] - w.tstamps[0]):g}), split "
                     f"{w.split['ratio']} / {w.split['pmin']}")
    return r
