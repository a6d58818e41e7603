"""Split-precision mover with field bricks staged in shared memory
(gpat_set_mover_tiles, csrc/mover_tile.cu) against the global-gather form
of the same mover (csrc/mover_mixed.cu).

Both draw the same Philox increments for the same push of the same particle,
so they follow the same trajectories; they differ only where a particle
pauses (a particle that walks out of the staged brick and halo finishes
its chunk in the global-gather overflow kernel), because a paused
particle's FP32 working state is rebuilt from its FP64 record.  The tolerance is therefore FP32 rounding
carried over the interval: positions within 1e-3 cells and momenta within
1e-4 relative on at least 99 % of the particles, the same particles kept,
and push counts within 0.5 %.
"""
import numpy as np
import pytest

from gpat import fields
from gpat.engine import Engine, GPATError, make_mhd_config, make_params

pytestmark = pytest.mark.gpu


def _engine_2d(nx, ny, nptl, seed, time_interp=0, bricks=None, bin_interval=64):
    cfg = make_mhd_config(nx, ny, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.02)
    db = fields.kolmogorov_az_2d(nx, ny, 1.0, 1.0, 0.5, 2 * np.pi, 16 * np.pi, seed)
    frame = fields.planar_shock_2d(nx, ny, 0.0, 1.0, 0.0, 1.0, r=3.0, w=0.02, db=db)
    prm = make_params(ndim=2, p0=0.1, pmin=0.1, pmax=100.0, kpara0=3e-3, kret=0.05,
                      dt_min_rel=2e-3, dt_max_rel=5e-2, pbcx=1, momentum_dependency=1,
                      precision=1, nptl_max=4 * nptl + 64, seed=100 + seed,
                      bin_interval=bin_interval, time_interp=time_interp)
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps(np.arange(6) * 0.02)
    eng.set_fields(frame, 0)
    eng.calc_fields_gradients(0)
    if time_interp:
        frame2 = fields.planar_shock_2d(nx, ny, 0.0, 1.0, 0.0, 1.0, r=2.5, w=0.03, db=db)
        eng.set_fields(frame2, 1)
        eng.calc_fields_gradients(1)
    if bricks:
        eng.set_mover_tiles(*bricks)
    eng.inject_particles_at_x(nptl, 0.5, 1e-6, 1, 1.0, 1)
    return eng


def _engine_3d(n, nptl, seed, bricks=None):
    cfg = make_mhd_config(n, n, n, 0.0, 1.0, 0.0, 1.0, zmin=0.0, zmax=1.0, dt_out=0.02, ndim=3)
    frame = fields.turbulence_3d(n, seed=seed)
    prm = make_params(ndim=3, p0=0.1, pmin=0.1, pmax=100.0, kpara0=2e-3, kret=0.05,
                      dt_min_rel=2e-3, dt_max_rel=5e-2, pbcx=0, pbcy=0, pbcz=0,
                      momentum_dependency=1, precision=1, nptl_max=2 * nptl, seed=200 + seed,
                      bin_interval=64)
    eng = Engine(prm, cfg, 0)
    eng.set_tstamps(np.arange(6) * 0.02)
    eng.set_fields(frame, 0)
    eng.calc_fields_gradients(0)
    if bricks:
        eng.set_mover_tiles(*bricks)
    eng.inject_particles_spatial_uniform(nptl, 1e-6, 1, 1.0, 1, (0, 0, 0, 1, 1, 1))
    return eng


def _agree(a, b, ndim):
    ga, gb = a.get_particles().order_by_tags(), b.get_particles().order_by_tags()
    ta = ga["tag_injected"].astype(np.int64) * (1 << 32) + ga["tag_splitted"]
    tb = gb["tag_injected"].astype(np.int64) * (1 << 32) + gb["tag_splitted"]
    common, ia, ib = np.intersect1d(ta, tb, return_indices=True)
    n = max(len(ta), len(tb))
    assert len(common) >= 0.995 * n, (len(ta), len(tb), len(common))
    cells = (a.cfg.dx, a.cfg.dy, a.cfg.dz)
    ok = np.ones(len(common), dtype=bool)
    for k, d in zip(("x", "y", "z")[:ndim], cells):
        ok &= np.abs(ga[k][ia] - gb[k][ib]) <= 1e-3 * d
    ok &= np.abs(ga["p"][ia] - gb["p"][ib]) <= 1e-4 * np.abs(gb["p"][ib])
    assert ok.mean() >= 0.99, ok.mean()
    sa, sb = a.counters().steps, b.counters().steps
    assert abs(sa - sb) <= 5e-3 * sb, (sa, sb)


@pytest.mark.parametrize("bricks", [(8, 8, 1), (16, 24, 1, 4, 4, 0, 256, 512)])
def test_tile_matches_global_gather_2d(bricks):
    glob = _engine_2d(64, 64, 4000, 1)
    tile = _engine_2d(64, 64, 4000, 1, bricks=bricks)
    for k in range(3):
        glob.particle_mover(mhd_tframe=k + 1)
        tile.particle_mover(mhd_tframe=k + 1)
        # particles that leave their bricks finish the chunk in the overflow
        # kernel: the launches per interval are the chunk rounds of the
        # global-gather mover
        lt, lg = tile.counters().last_mover_launches, glob.counters().last_mover_launches
        assert abs(lt - lg) <= 1, (lt, lg)
    _agree(tile, glob, 2)
    fa, na = tile.calc_escaped_distributions()
    fb, nb = glob.calc_escaped_distributions()
    assert abs(int(na.sum()) - int(nb.sum())) <= max(3, 0.01 * nb.sum())
    glob.close()
    tile.close()


def test_tile_matches_global_gather_time_interp_and_nlgc():
    glob = _engine_2d(48, 80, 3000, 2, time_interp=1)
    tile = _engine_2d(48, 80, 3000, 2, time_interp=1, bricks=(12, 10, 1, 2, 2, 0))
    for k in range(2):
        glob.particle_mover(mhd_tframe=k + 1, nlgc=True, kperp_kpara=0.05)
        tile.particle_mover(mhd_tframe=k + 1, nlgc=True, kperp_kpara=0.05)
    _agree(tile, glob, 2)
    glob.close()
    tile.close()


@pytest.mark.parametrize("bricks", [(6, 6, 6), (4, 8, 12, 1, 1, 3, 256)])
def test_tile_matches_global_gather_3d(bricks):
    glob = _engine_3d(24, 6000, 3)
    tile = _engine_3d(24, 6000, 3, bricks=bricks)
    for k in range(2):
        glob.particle_mover(mhd_tframe=k + 1)
        tile.particle_mover(mhd_tframe=k + 1)
    _agree(tile, glob, 3)
    glob.close()
    tile.close()


def test_tile_shapes_checked():
    eng = _engine_3d(24, 100, 4)
    with pytest.raises(GPATError):
        eng.set_mover_tiles(40, 40, 40)          # records exceed one CTA's shared memory
    with pytest.raises(GPATError):
        eng.set_mover_tiles(8, 8, 8, threads=384)   # threads per CTA: 256 or 512
    with pytest.raises(GPATError):
        eng.set_mover_tiles(1, 8, 8)
    with pytest.raises(GPATError):
        eng.set_mover_tiles(8, 8, 8, 6, 6, 6)    # the halo makes it too large
    eng.set_mover_tiles(6, 6, 6, 2, 2, 2)
    assert eng.mover_tiles() == dict(bx=6, by=6, bz=6, hx=2, hy=2, hz=2, threads=512,
                                     items=4096)
    eng.close()
    small = _engine_2d(16, 16, 300, 4)
    small.set_mover_tiles(100, 100, 1)           # larger than the grid: cut to it
    assert small.mover_tiles()["bx"] == 19 and small.mover_tiles()["by"] == 19
    small.particle_mover(mhd_tframe=1)           # one brick holds everything
    small.set_mover_tiles(0)
    assert small.mover_tiles()["bx"] == 0
    small.particle_mover(mhd_tframe=2)
    small.close()
    fp64 = Engine(make_params(ndim=2, precision=0, nptl_max=10),
                  make_mhd_config(16, 16, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.02), 0)
    with pytest.raises(GPATError):
        fp64.set_mover_tiles(8, 8, 1)
    fp64.close()
