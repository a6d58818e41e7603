"""Synthetic MHD frames in the reference's on-disk layout.

A frame is the Fortran array ``farray(8, -1:nx+2, -1:ny+2, -1:nz+2)`` of
single-precision vx vy vz rho bx by bz |B| with two ghost cells per resolved
side (the layout examples/reconnection_2d/mhd_data/reorganize_fields.py
writes).  In numpy (C order) it is shape (nzg, nyg, nxg, 8).  Node
(i, j, k) of the Fortran array sits at x = xmin + (i - 1) dx, which is what
get_interp_paramters assumes (particle_module.f90:642-674).

The generators stand in for the reference's Athena/Athena++ inputs, which are
not available; every random field is seeded.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np


def node_coords(n: int, lo: float, d: float) -> np.ndarray:
    """Positions of the n + 4 nodes, ghosts included (Fortran -1 .. n+2)."""
    return lo + (np.arange(n + 4, dtype=np.float64) - 2.0) * d


def periodic_with_ghosts(a: np.ndarray, axes) -> np.ndarray:
    """Pads a periodic nodal array with two ghost nodes per side."""
    pad = [(0, 0)] * a.ndim
    for ax in axes:
        pad[ax] = (2, 2)
    return np.pad(a, pad, mode="wrap")


def tanh_shock_vx(x: np.ndarray, u1: float, r: float, w: float, x0: float) -> np.ndarray:
    """vx(x) = u1 [1 - (1 - 1/r)(1 + tanh((x - x0)/w))/2]."""
    return u1 * (1.0 - (1.0 - 1.0 / r) * 0.5 * (1.0 + np.tanh((x - x0) / w)))


def kolmogorov_az_2d(nx: int, ny: int, lx: float, ly: float, db_rms: float, kmin: float,
                     kmax: float, seed: int, slope: float = -5.0 / 3.0):
    """Random-phase 2D fluctuation dB = curl(Az z) with E(k) ~ k^slope.

    Returns (dbx, dby) on the nx*ny periodic nodes, normalised to the given
    rms of |dB|.  The field is divergence-free to round-off (spectral curl).
    """
    rng = np.random.default_rng(seed)
    kx = 2.0 * np.pi * np.fft.fftfreq(nx, d=lx / nx)
    ky = 2.0 * np.pi * np.fft.rfftfreq(ny, d=ly / ny)
    KX, KY = np.meshgrid(kx, ky, indexing="ij")
    k = np.sqrt(KX ** 2 + KY ** 2)
    band = (k >= kmin * (1 - 1e-9)) & (k <= kmax * (1 + 1e-9))
    amp = np.zeros_like(k)
    # |B_k|^2 ~ E(k)/k in 2D, |Az_k| = |B_k|/k.
    amp[band] = k[band] ** ((slope - 1.0) / 2.0) / k[band]
    phase = rng.uniform(0.0, 2.0 * np.pi, size=k.shape)
    az_hat = amp * np.exp(1j * phase)
    dbx = np.fft.irfft2(1j * KY * az_hat, s=(nx, ny))
    dby = np.fft.irfft2(-1j * KX * az_hat, s=(nx, ny))
    rms = np.sqrt(np.mean(dbx ** 2 + dby ** 2))
    scale = db_rms / rms if rms > 0 else 0.0
    return dbx * scale, dby * scale   # arrays indexed [ix, iy]


def random_field_3d(n: int, slope: float, seed: int, kind: str, kmin_mode: int = 1,
                    kmax_mode: int | None = None):
    """Gaussian random vector field on an n^3 periodic box (unit length).

    kind: 'solenoidal', 'compressive' or 'both' (returns the two parts
    separately, each with unit total power before scaling).  Spectrum
    E(k) ~ k^slope, i.e. |v_k|^2 ~ k^(slope-2).
    """
    rng = np.random.default_rng(seed)
    kmax_mode = kmax_mode or n // 2
    k1 = np.fft.fftfreq(n, d=1.0 / n)
    k3 = np.fft.rfftfreq(n, d=1.0 / n)
    KX, KY, KZ = np.meshgrid(k1, k1, k3, indexing="ij")
    k = np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2)
    band = (k >= kmin_mode) & (k <= kmax_mode)
    amp = np.zeros_like(k)
    amp[band] = k[band] ** ((slope - 2.0) / 2.0)
    shape = k.shape
    vh = [(rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) * amp for _ in range(3)]
    ks = np.where(k > 0, k, 1.0)
    kh = (KX / ks, KY / ks, KZ / ks)
    dot = vh[0] * kh[0] + vh[1] * kh[1] + vh[2] * kh[2]
    comp = [dot * kh[i] for i in range(3)]
    sol = [vh[i] - comp[i] for i in range(3)]

    def to_real(parts):
        return [np.fft.irfftn(p, s=(n, n, n), axes=(0, 1, 2)).astype(np.float64) for p in parts]

    if kind == "solenoidal":
        return to_real(sol)
    if kind == "compressive":
        return to_real(comp)
    return to_real(sol), to_real(comp)


def assemble_frame(vx, vy, vz, rho, bx, by, bz) -> np.ndarray:
    """Stacks the 8 variables (|B| computed) into (nzg, nyg, nxg, 8) float32."""
    b = np.sqrt(bx.astype(np.float64) ** 2 + by.astype(np.float64) ** 2 +
                bz.astype(np.float64) ** 2)
    return np.ascontiguousarray(np.stack([vx, vy, vz, rho, bx, by, bz, b], axis=-1),
                                dtype=np.float32)


def planar_shock_2d(nx, ny, xmin, xmax, ymin, ymax, u1=1.0, r=4.0, w=0.002, x0=0.5,
                    b0=(1.0, 0.0, 0.0), db=None) -> np.ndarray:
    """2D tanh shock along x, optional in-plane fluctuation db = (dbx, dby)
    on the nx*ny periodic nodes.  Returns (1, ny+4, nx+4, 8)."""
    dx, dy = (xmax - xmin) / nx, (ymax - ymin) / ny
    x = node_coords(nx, xmin, dx)
    vx1 = tanh_shock_vx(x, u1, r, w, x0)
    shape = (ny + 4, nx + 4)
    vx = np.broadcast_to(vx1[None, :], shape)
    zero = np.zeros(shape)
    rho = np.broadcast_to((u1 / vx1)[None, :], shape)
    bx = np.full(shape, b0[0])
    by = np.full(shape, b0[1])
    bz = np.full(shape, b0[2])
    if db is not None:
        dbx, dby = db
        bx = bx + periodic_with_ghosts(dbx, (0, 1)).T
        by = by + periodic_with_ghosts(dby, (0, 1)).T
    frame = assemble_frame(vx, zero, zero, rho, bx, by, bz)
    return frame[None]


def turbulence_3d(n: int, v_rms=0.3, comp_frac=0.3, db_rms=0.3, b0=1.0, seed=0,
                  slope=-5.0 / 3.0) -> np.ndarray:
    """Periodic n^3 box: v with the given compressive power fraction, B = b0 z
    + solenoidal dB.  Returns (n+4, n+4, n+4, 8)."""
    sol, comp = random_field_3d(n, slope, seed, "both")
    ps = sum(np.mean(c ** 2) for c in sol)
    pc = sum(np.mean(c ** 2) for c in comp)
    a_s = np.sqrt((1.0 - comp_frac) / ps) if ps > 0 else 0.0
    a_c = np.sqrt(comp_frac / pc) if pc > 0 else 0.0
    v = [a_s * s + a_c * c for s, c in zip(sol, comp)]
    vr = np.sqrt(np.mean(v[0] ** 2 + v[1] ** 2 + v[2] ** 2))
    v = [c * (v_rms / vr) for c in v]
    bsol = random_field_3d(n, slope, seed + 7919, "solenoidal")
    br = np.sqrt(np.mean(bsol[0] ** 2 + bsol[1] ** 2 + bsol[2] ** 2))
    bsol = [c * (db_rms * b0 / br) for c in bsol]
    # arrays are [ix, iy, iz]; the frame is [iz, iy, ix].
    def g(a):
        return periodic_with_ghosts(a, (0, 1, 2)).transpose(2, 1, 0)
    vx, vy, vz = (g(c) for c in v)
    bx, by, bz = g(bsol[0]), g(bsol[1]), g(bsol[2]) + b0
    rho = np.ones_like(vx)
    return assemble_frame(vx, vy, vz, rho, bx, by, bz)


def write_mhd_data(path: str | Path, frame: np.ndarray):
    """Raw single-precision stream file, variables fastest (mhd_data_XXXX)."""
    np.ascontiguousarray(frame, dtype=np.float32).tofile(path)


def write_mhd_config(path: str | Path, cfg):
    """156-byte mhd_config.dat record: 13 doubles then 13 int32."""
    d = [cfg.dx, cfg.dy, cfg.dz, cfg.xmin, cfg.ymin, cfg.zmin, cfg.xmax, cfg.ymax, cfg.zmax,
         cfg.lx, cfg.ly, cfg.lz, cfg.dt_out]
    i = [cfg.nx, cfg.ny, cfg.nz, cfg.nxs, cfg.nys, cfg.nzs, cfg.topox, cfg.topoy, cfg.topoz,
         cfg.nvar, cfg.bcx, cfg.bcy, cfg.bcz]
    with open(path, "wb") as f:
        f.write(np.asarray(d, dtype="<f8").tobytes())
        f.write(np.asarray(i, dtype="<i4").tobytes())
