"""Physics and accuracy of the movers on the planar shock (r = 4).

- The FP64 mover recovers the diffusive-shock-acceleration spectrum: for
  r = 4 the weighted number per log-p bin falls as p^(3 - 3r/(r-1)) = p^-1
  above injection (a softer slope is expected where the diffusion step per
  push exceeds the shock width).
- The split-precision mover's f(p) tail agrees with the FP64 mover's within
  2 % plus three Monte Carlo standard errors.
"""
import math

import numpy as np
import pytest

from gpat import accuracy, configs

pytestmark = pytest.mark.gpu


def test_planar_shock_spectral_index_fp64():
    w = configs.planar_shock(scale=0.5, t_end=2.0)
    eng = configs.build_engine(w, precision=0, nptl_max=w.nptl * 8)
    configs.inject(eng, w)
    for k in range(w.nframes):
        eng.particle_mover(mhd_tframe=k + 1)
        eng.split_particle(2.72, 2.0, 10)
    f, c = eng.calc_particle_distributions()
    edges = eng.pbins_edges()
    centers = np.sqrt(edges[:-1] * edges[1:])
    # fit dN/dlnp over 1.5 p0 .. 6 p0 (p0 = 0.1): above injection, below the
    # escape-limited cut-off
    m = (centers > 0.15) & (centers < 0.6) & (c > 50)
    assert m.sum() >= 6
    slope = np.polyfit(np.log(centers[m]), np.log(f[m]), 1)[0]
    assert -1.6 < slope < -0.8, slope
    eng.close()


def test_mixed_tail_error_planar_shock():
    r = accuracy.planar_shock_check(scale=0.5)
    assert r["top_decade_particles_fp64"] > 1000
    assert abs(r["tail_err"]) <= 0.02 + 3 * r["tail_err_sigma"], r
    dof = max(1, r["chi2_dof"])
    assert r["chi2"] < dof + 4 * math.sqrt(2 * dof) + 10, r
