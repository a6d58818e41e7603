"""Statistical gates of the method on the GPU.

- Pure diffusion: with V = 0, a uniform oblique B and momentum-independent
  kappa, the displacement along b is N(0, 2 kappa_par t) and across it
  N(0, 2 kappa_perp t) (docs/source/theory/parker_1d2d.rst:17-24 for the
  Ito form; the increments of push_particle_2d / _3d, particle_module.f90:
  3546-3590, 4870-4877).  A Kolmogorov-Smirnov test against those normals
  must not reject at the 0.1 % level, for both movers and both increment
  kinds (the reference's uniform (2u-1) sqrt(3), and Box-Muller Gaussians).
- Spatial densities: the split-precision mover's x and y (and z) particle
  densities agree with the FP64 mover's, chi-square over bins with at least
  20 particles in each run, not rejected at the 0.1 % level.  Runs without
  splitting keep the particles independent, so the Poisson variances hold.
"""
import math

import numpy as np
import pytest

from gpat import configs, fields
from gpat.engine import Engine, ParticleSet, make_mhd_config, make_params

pytestmark = pytest.mark.gpu
stats = pytest.importorskip("scipy.stats")

NOISE = {"uniform": 0, "gauss": 1}


def _diffusion_run(ndim, precision, noise, n, kpara=1e-3, kret=0.1, T=0.5, pushes=200,
                   seed=31):
    g = 32 if ndim == 3 else 64
    if ndim == 2:
        b = np.array([0.8, 0.6, 0.0])
        cfg = make_mhd_config(g, g, 1, 0.0, 1.0, 0.0, 1.0, dt_out=T)
        shape = (1, g + 4, g + 4)
    else:
        b = np.array([0.4, -0.3, 0.866])
        b /= np.linalg.norm(b)
        cfg = make_mhd_config(g, g, g, 0.0, 1.0, 0.0, 1.0, zmin=0.0, zmax=1.0, dt_out=T, ndim=3)
        shape = (g + 4, g + 4, g + 4)
    z = np.zeros(shape)
    frame = fields.assemble_frame(z, z, z, z + 1, z + b[0], z + b[1], z + b[2])
    prm = make_params(ndim=ndim, kpara0=kpara, kret=kret, momentum_dependency=0,
                      dt_min_rel=1.0 / pushes, dt_max_rel=1.0 / pushes, pbcx=0, pbcy=0, pbcz=0,
                      p0=0.1, precision=precision, noise=NOISE[noise], nptl_max=n, seed=seed)
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps([0.0, T])
    eng.set_fields(frame, 0)
    eng.calc_fields_gradients(0)
    ps = ParticleSet.empty(n)
    for k in ("x", "y", "z"):
        ps.arrays[k][:] = 0.5
    ps.arrays["p"][:] = 0.1
    ps.arrays["weight"][:] = 1.0
    ps.arrays["count_flag"][:] = 1
    ps.arrays["tag_splitted"][:] = 1
    ps.arrays["tag_injected"][:] = np.arange(n, dtype=np.int32)
    eng.put_particles(ps)
    eng.particle_mover(mhd_tframe=1)
    out = eng.get_particles()
    steps = eng.counters().steps
    eng.close()
    d = np.stack([out["x"] - 0.5, out["y"] - 0.5, out["z"] - 0.5])[:ndim]
    return d, b[:ndim], steps


@pytest.mark.parametrize("ndim,precision,noise", [
    (2, 0, "uniform"), (2, 1, "uniform"), (2, 0, "gauss"), (2, 1, "gauss"),
    (3, 1, "uniform"), (3, 1, "gauss"), (3, 0, "gauss")])
def test_pure_diffusion_is_gaussian(ndim, precision, noise):
    n = 100_000 if precision else 40_000
    kpara, kret, T, pushes = 1e-3, 0.1, 0.5, 200
    d, b, steps = _diffusion_run(ndim, precision, noise, n, kpara, kret, T, pushes)
    # V = 0: every push at dt_min; in FP64 the 200 steps of dtf / 200 can sum
    # to just below dtf, and the landing adds one redo push
    assert n * pushes <= steps <= n * (pushes + 1)
    par = b @ d
    s_par = math.sqrt(2 * kpara * T)
    s_perp = math.sqrt(2 * kpara * kret * T)
    p_par = stats.kstest(par / s_par, "norm").pvalue
    assert p_par > 1e-3, (p_par, par.std() / s_par)
    if ndim == 2:
        perp = np.array([-b[1], b[0]]) @ d
        p_perp = stats.kstest(perp / s_perp, "norm").pvalue
        assert p_perp > 1e-3, (p_perp, perp.std() / s_perp)
    else:
        # two directions across b
        e1 = np.cross(b, [1.0, 0.0, 0.0])
        e1 /= np.linalg.norm(e1)
        e2 = np.cross(b, e1)
        for e in (e1, e2):
            pv = stats.kstest((e @ d) / s_perp, "norm").pvalue
            assert pv > 1e-3, (pv, (e @ d).std() / s_perp)


def _weighted_hist(ps, key, edges):
    v, w = ps[key], ps["weight"]
    return (np.histogram(v, edges, weights=w)[0], np.histogram(v, edges, weights=w * w)[0],
            np.histogram(v, edges)[0])


def _density_chi2(a, b, key, edges):
    fa, va, ca = _weighted_hist(a, key, edges)
    fb, vb, cb = _weighted_hist(b, key, edges)
    m = (ca >= 20) & (cb >= 20)
    chi2 = float(np.sum((fa[m] - fb[m]) ** 2 / (va[m] + vb[m])))
    dof = int(m.sum())
    return chi2, dof, stats.chi2.sf(chi2, dof)


def _both(w, intervals, nptl=None):
    out = {}
    for prec in (0, 1):
        eng = configs.build_engine(w, precision=prec, nptl_max=nptl or w.nptl)
        configs.inject(eng, w, nptl=nptl)
        for k in range(intervals):
            eng.particle_mover(nsteps_interval=10, mhd_tframe=k + 1, num_fine_steps=1)
        out[prec] = eng.get_particles()
        eng.close()
    return out


def test_planar_shock_densities_fp64_vs_split():
    w = configs.planar_shock(scale=1.0)
    runs = _both(w, 6)
    c = w.mhd_config
    for key, lo, hi, nb in (("x", c.xmin, c.xmin + c.nx * c.dx, 128),
                            ("y", c.ymin, c.ymin + c.ny * c.dy, 16)):
        chi2, dof, p = _density_chi2(runs[0], runs[1], key, np.linspace(lo, hi, nb + 1))
        assert dof >= 8 and p > 1e-3, (key, chi2, dof, p)


def test_turbulent_shock_densities_fp64_vs_split():
    w = configs.turbulent_shock_2d(scale=0.01, n=512, nframes=8)
    runs = _both(w, 4)
    for key, nb in (("x", 128), ("y", 32)):
        chi2, dof, p = _density_chi2(runs[0], runs[1], key, np.linspace(0.0, 1.0, nb + 1))
        assert dof >= 8 and p > 1e-3, (key, chi2, dof, p)


def test_turbulence_3d_densities_fp64_vs_split():
    w = configs.turbulence_3d(scale=2e-3, n=64, nframes=4)
    runs = _both(w, 2)
    for key in ("x", "y", "z"):
        chi2, dof, p = _density_chi2(runs[0], runs[1], key, np.linspace(0.0, 1.0, 33))
        assert dof >= 16 and p > 1e-3, (key, chi2, dof, p)
