"""The benchmark workloads as engine inputs.

planar_shock   2D planar shock, 512x64 over [0,1]x[0,0.125], r = 4, w = 0.002,
               uniform B = x, kappa_par = 0.01 (p/p0)^(4/3), kperp/kpar = 0.05,
               injection at x = 0.5, open in x, periodic in y, t in [0, 2],
               f(p) in 128 log bins over p0 .. 1e4 p0.
turbulent_shock_2d
               2048x2048 over [0,1]^2, r = 3.5, w = 0.001, B = x + random-phase
               Kolmogorov dB (dB/B0 = 0.5, k in [2 pi, 512 pi]) from Az,
               same kappa law along the local B, kperp/kpar = 0.05, 1e7
               particles on the shock at p0, 1e3 pushes per particle per
               interval (dt_min = dtf / 1000).
batched_shock_2d
               64 independent turbulent-shock runs (seeded): particles
               log-uniform in [1e4, 1e7], r uniform in [2, 4], kappa_0
               log-uniform in [1e-3, 1e-1], kperp/kpar uniform in [0.01, 0.2],
               grids 512^2, 1024^2 or 2048^2 with the turbulent_shock_2d
               fluctuation; moved together by the batched mover.
turbulence_3d  256^3 periodic box, v rms 0.3 (30 % compressive power),
               B = z + solenoidal dB (0.3), kperp/kpar = 0.02, 1e8 particles
               uniform in space, log-uniform p in [p0, 10 p0], adaptive dt
               between dt_out/5000 and dt_out/500.

Each builder takes ``scale`` (particle count multiplier) and grid overrides
so tests can run reduced cases with the same physics.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import fields
from .engine import make_mhd_config, make_params


@dataclass
class Workload:
    name: str
    params: dict
    mhd_config: object
    frame: np.ndarray
    nptl: int
    inject: dict                       # kind + arguments of the injector
    tstamps: np.ndarray
    nframes: int                       # mover intervals in the full run
    num_fine_steps: int = 1
    nsteps_interval: int = 10
    split: dict = field(default_factory=dict)


def planar_shock(scale: float = 1.0, nx: int = 512, ny: int = 64, t_end: float = 2.0,
                 dt_out: float = 0.1, dt_min: float = 1.0e-4, precision: int = 0,
                 seed: int = 1) -> Workload:
    p0 = 0.1
    params = dict(p0=p0, pmin=p0, pmax=1.0e4 * p0, momentum_dependency=1, gamma_turb=5.0 / 3.0,
                  mag_dependency=0, kpara0=0.01, kret=0.05, dt_min_rel=dt_min / dt_out,
                  dt_max_rel=1.0e-2, ndim=2, pbcx=1, pbcy=0, pbcz=0, npp_global=128,
                  precision=precision, seed=seed)
    cfg = make_mhd_config(nx, ny, 1, 0.0, 1.0, 0.0, 0.125, zmin=0.0, zmax=1.0, dt_out=dt_out)
    frame = fields.planar_shock_2d(nx, ny, 0.0, 1.0, 0.0, 0.125, u1=1.0, r=4.0, w=0.002, x0=0.5)
    nframes = int(round(t_end / dt_out))
    nptl = max(1, int(round(1.0e5 * scale)))
    params["nptl_max"] = nptl
    return Workload("planar_shock_512x64", params, cfg, frame, nptl,
                    dict(kind="at_x", xpos=0.5, dist_flag=1),
                    np.arange(nframes + 1) * dt_out, nframes,
                    split=dict(ratio=2.72, pmin=2.0))


def turbulent_shock_2d(scale: float = 1.0, n: int = 2048, dt_out: float = 0.01,
                       pushes: int = 1000, precision: int = 1, seed: int = 2,
                       nframes: int = 64) -> Workload:
    p0 = 0.1
    params = dict(p0=p0, pmin=p0, pmax=1.0e4 * p0, momentum_dependency=1, gamma_turb=5.0 / 3.0,
                  mag_dependency=0, kpara0=0.01, kret=0.05, dt_min_rel=1.0 / pushes,
                  dt_max_rel=1.0e-2, ndim=2, pbcx=1, pbcy=0, pbcz=0, npp_global=128,
                  precision=precision, seed=seed)
    cfg = make_mhd_config(n, n, 1, 0.0, 1.0, 0.0, 1.0, zmin=0.0, zmax=1.0, dt_out=dt_out)
    kmax = min(512.0 * np.pi, np.pi * n / 2)
    db = fields.kolmogorov_az_2d(n, n, 1.0, 1.0, db_rms=0.5, kmin=2.0 * np.pi, kmax=kmax,
                                 seed=1000 + seed)
    frame = fields.planar_shock_2d(n, n, 0.0, 1.0, 0.0, 1.0, u1=1.0, r=3.5, w=0.001, x0=0.5,
                                   db=db)
    nptl = max(1, int(round(1.0e7 * scale)))
    params["nptl_max"] = nptl
    return Workload(f"turbulent_shock_2d_{n}x{n}", params, cfg, frame, nptl,
                    dict(kind="at_x", xpos=0.5, dist_flag=1),
                    np.arange(nframes + 1) * dt_out, nframes,
                    split=dict(ratio=2.72, pmin=2.0))


def batched_shock_2d(nruns: int = 64, scale: float = 1.0, sizes=(512, 1024, 2048),
                     dt_out: float = 0.01, pushes: int = 1000, precision: int = 1,
                     seed: int = 11, nframes: int = 16, only: int | None = None) -> list:
    """The runs of the batched workload, each a turbulent_shock_2d variant.
    Fields of one size share the fluctuation (drawn once per size); the
    shock compression differs per run.  ``only`` builds that run alone (its
    parameters are the same as in the full list)."""
    rng = np.random.default_rng(seed)
    dbs = {}
    runs = []
    for r in range(nruns):
        nptl = int(round(10.0 ** rng.uniform(4.0, 7.0) * scale))
        comp = float(rng.uniform(2.0, 4.0))
        kappa0 = float(10.0 ** rng.uniform(-3.0, -1.0))
        kret = float(rng.uniform(0.01, 0.2))
        n = int(sizes[rng.integers(len(sizes))])
        if only is not None and r != only:
            continue
        if n not in dbs:
            kmax = min(512.0 * np.pi, np.pi * n / 2)
            dbs[n] = fields.kolmogorov_az_2d(n, n, 1.0, 1.0, db_rms=0.5, kmin=2.0 * np.pi,
                                             kmax=kmax, seed=2000 + n)
        p0 = 0.1
        params = dict(p0=p0, pmin=p0, pmax=1.0e4 * p0, momentum_dependency=1,
                      gamma_turb=5.0 / 3.0, mag_dependency=0, kpara0=kappa0, kret=kret,
                      dt_min_rel=1.0 / pushes, dt_max_rel=1.0e-2, ndim=2, pbcx=1, pbcy=0, pbcz=0,
                      npp_global=128, precision=precision, seed=seed * 1000 + r,
                      nptl_max=max(1, nptl))
        cfg = make_mhd_config(n, n, 1, 0.0, 1.0, 0.0, 1.0, zmin=0.0, zmax=1.0, dt_out=dt_out)
        frame = fields.planar_shock_2d(n, n, 0.0, 1.0, 0.0, 1.0, u1=1.0, r=comp, w=0.001,
                                       x0=0.5, db=dbs[n])
        runs.append(Workload(f"batched_shock_2d_run{r}_{n}x{n}_r{comp:.2f}", params, cfg, frame,
                             max(1, nptl), dict(kind="at_x", xpos=0.5, dist_flag=1),
                             np.arange(nframes + 1) * dt_out, nframes,
                             split=dict(ratio=2.72, pmin=2.0)))
    return runs


def turbulence_3d(scale: float = 1.0, n: int = 256, dt_out: float = 0.05, pushes: int = 500,
                  precision: int = 1, seed: int = 3, nframes: int = 16) -> Workload:
    """256^3 periodic box.  dt is adaptive between dt_out/5000 and
    dt_out/pushes (the reference's rule; compressive regions pick steps
    below dt_max, about 1800 pushes per interval on average).  Injection is log-uniform in [p0, 10 p0] (dist_flag 2 with power index 1
    draws p = (pmax/p0)^u p0), so pmax = 10 p0 also bounds f(p)."""
    p0 = 0.1
    params = dict(p0=p0, pmin=p0, pmax=10.0 * p0, momentum_dependency=1, gamma_turb=5.0 / 3.0,
                  mag_dependency=0, kpara0=0.01, kret=0.02, dt_min_rel=1.0 / (10 * pushes),
                  dt_max_rel=1.0 / pushes, ndim=3, pbcx=0, pbcy=0, pbcz=0, npp_global=128,
                  precision=precision, seed=seed)
    cfg = make_mhd_config(n, n, n, 0.0, 1.0, 0.0, 1.0, zmin=0.0, zmax=1.0, dt_out=dt_out, ndim=3)
    frame = fields.turbulence_3d(n, seed=3000 + seed)
    nptl = max(1, int(round(1.0e8 * scale)))
    params["nptl_max"] = nptl
    return Workload(f"turbulence_3d_{n}^3", params, cfg, frame, nptl,
                    dict(kind="uniform", dist_flag=2, power_index=1.0),
                    np.arange(nframes + 1) * dt_out, nframes)


def build_engine(w: Workload, device: int = 0, nptl_max: int | None = None, **overrides):
    """Creates an Engine for the workload with fields, gradients and time
    stamps set (the driver's set-up before its time loop)."""
    from .engine import Engine
    kw = dict(w.params)
    kw.update(overrides)
    if nptl_max is not None:
        kw["nptl_max"] = nptl_max
    eng = Engine(make_params(**kw), w.mhd_config, device)
    eng.set_tstamps(w.tstamps)
    eng.set_fields(w.frame, 0)
    eng.calc_fields_gradients(0)
    return eng


def inject(eng, w: Workload, nptl: int | None = None, ct_mhd: int = 1, dt: float = 1e-7):
    nptl = w.nptl if nptl is None else nptl
    spec = w.inject
    if spec["kind"] == "at_x":
        eng.inject_particles_at_x(nptl, spec["xpos"], dt, spec["dist_flag"], 1.0, ct_mhd)
    else:
        c = w.mhd_config
        box = (c.xmin, c.ymin, c.zmin, c.xmin + c.nx * c.dx, c.ymin + c.ny * c.dy,
               c.zmin + c.nz * c.dz)
        eng.inject_particles_spatial_uniform(nptl, dt, spec["dist_flag"], 1.0, ct_mhd, box,
                                             spec.get("power_index", 7.0))
