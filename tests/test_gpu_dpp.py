"""Momentum diffusion (calc_dpp_wave_scattering, calc_dpp_flow_shear): CUDA
FP64 mover against the oracle, through the C ABI.

Wave scattering with momentum-independent kappa calls no pow() and is
bit-exact; flow shear evaluates p^(pindex-1), p^pindex and p0^(2-pindex),
whose last bit may differ between libm and CUDA, so it uses a per-particle
relative tolerance of 1e-9 on >= 99.5 % of the particles.
"""
import numpy as np
import pytest

from gpat.engine import Engine, GPATError, make_params
from test_gpu_focused import FT_STATE, _inject_shock, _same
from test_gpu_parity import STATE, run_pair, shock_case, turbulent_frame_2d

pytestmark = pytest.mark.gpu

BOX = (0.0, 0.0, 0.0, 1.0, 1.0, 1.0)


def test_wave_scattering_bit_exact():
    params, cfg = shock_case(dpp_wave=1, pbcx=0)
    ts = np.arange(3) * 0.02
    eng, gpu, ref, cnt, _ = run_pair(
        params, cfg, turbulent_frame_2d(), ts,
        lambda e: e.inject_particles_spatial_uniform(2000, 1e-6, 1, 1.0, 1, BOX), intervals=2,
        fine=2)
    _same(gpu, ref, STATE)
    assert eng.counters().steps == cnt.steps


@pytest.mark.parametrize("weak", [0, 1])
def test_flow_shear(weak):
    params, cfg = shock_case(dpp_shear=1, weak_scattering=weak, tau0=0.5, pbcx=0)
    ts = np.arange(3) * 0.02
    eng, gpu, ref, cnt, _ = run_pair(
        params, cfg, turbulent_frame_2d(), ts,
        lambda e: e.inject_particles_spatial_uniform(2000, 1e-6, 1, 1.0, 1, BOX), intervals=2)
    _same(gpu, ref, STATE, exact=False)
    g = gpu.order_by_tags()
    assert np.std(np.log(g["p"])) > 0.0


def test_wave_scattering_with_focused_transport_bit_exact():
    # kpara0 keeps the wave-scattering gain 4 va^2 / (9 kpara) moderate: the
    # speed v grows with p and a streaming particle must not cross more than
    # a cell per push.
    params, cfg = shock_case(dpp_wave=1, duu0=0.0, kpara0=3e-2, pbcx=0, pbcy=0)
    ts = np.arange(3) * 0.02
    eng, gpu, ref, cnt, _ = run_pair(params, cfg, turbulent_frame_2d(), ts, _inject_shock(1500),
                                     intervals=2, mover_kw=dict(focused_transport=True))
    _same(gpu, ref, FT_STATE)


def test_dpp_3d_momentum_dependent():
    from test_gpu_focused import _cube
    cfg, frame, params = _cube()
    params.update(dpp_wave=1, dpp_shear=1, momentum_dependency=1)
    ts = np.arange(2) * 0.02
    eng, gpu, ref, cnt, _ = run_pair(
        params, cfg, frame, ts,
        lambda e: e.inject_particles_spatial_uniform(1500, 1e-6, 1, 1.0, 1, BOX))
    _same(gpu, ref, STATE, exact=False)


def test_dpp_needs_fp64():
    params, cfg = shock_case(dpp_wave=1, precision=1)
    with pytest.raises(GPATError, match="UNSUPPORTED"):
        Engine(make_params(**params), cfg, 0)
