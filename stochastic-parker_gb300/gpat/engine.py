"""Host-side mirror of the reference's particle/MHD-data module API.

``Engine`` wraps one handle of the C ABI (include/gpat_engine.h).  Its
methods carry the names and argument meanings of the Fortran procedures the
reference driver (src/programs/stochastic-mhd.f90:312-567) calls on the
mover path: read_particle_params, calc_fields_gradients, copy_fields,
inject_particles_spatial_uniform, particle_mover, split_particle,
calc_particle_distributions (global f(p)) and quick_check.  Errors raise
GPATError with the engine's code and message; nothing falls back to a host
implementation.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import _abi

REFERENCE_DEFAULTS = dict(
    # conf.dat sample values (config/conf.dat) and CLI defaults
    # (stochastic-mhd.f90:636-946) for the fields the mover reads.
    b0=1.0, p0=0.1, pmin=1.0e-2, pmax=1.0e1,
    momentum_dependency=1, gamma_turb=5.0 / 3.0, mag_dependency=0,
    kpara0=0.01, kret=0.05, dt_min_rel=1.0e-4, dt_max_rel=1.0e-2,
    acc_region_flag=0, acc_region=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0),
    drift1=4.0e7, drift2=2.0e8, charge=-1, check_drift_2d=0,
    ndim=2, pbcx=0, pbcy=0, pbcz=0, npp_global=128,
    seed=0x5EED0001, noise=_abi.NOISE_UNIFORM, precision=_abi.PREC_FP64,
    nptl_max=100_000, time_interp=0, duu0=10.0, tau0=1.0,
)


class GPATError(RuntimeError):
    def __init__(self, code: int, message: str):
        self.code = code
        super().__init__(f"{_abi.ERROR_NAMES.get(code, code)}: {message}")


class GPATCapacityError(GPATError):
    pass


def make_params(**kw) -> _abi.Params:
    """Builds a gpat_params_t from keyword values over REFERENCE_DEFAULTS.

    pindex defaults to 3 - gamma_turb as in read_particle_params
    (particle_module.f90:2798)."""
    vals = dict(REFERENCE_DEFAULTS)
    vals.update(kw)
    if "pindex" not in kw:
        vals["pindex"] = 3.0 - vals["gamma_turb"]
    p = _abi.Params()
    for name, _ in _abi.Params._fields_:
        if name == "acc_region":
            p.acc_region = (C.c_double * 6)(*vals["acc_region"])
        elif name in vals:
            setattr(p, name, vals[name])
    return p


def params_dict(p: _abi.Params) -> dict:
    out = {}
    for name, _ in _abi.Params._fields_:
        v = getattr(p, name)
        out[name] = tuple(v) if name == "acc_region" else v
    return out


def make_mhd_config(nx, ny, nz, xmin, xmax, ymin, ymax, zmin=0.0, zmax=1.0, dt_out=1.0,
                    ndim=2) -> _abi.MhdConfig:
    """mhd_config for a uniform grid of nx*ny(*nz) cells spanning the box."""
    c = _abi.MhdConfig()
    c.nx, c.ny, c.nz = nx, ny, nz
    c.dx = (xmax - xmin) / nx
    c.dy = (ymax - ymin) / ny
    c.dz = (zmax - zmin) / nz if ndim == 3 else (zmax - zmin)
    c.xmin, c.xmax, c.ymin, c.ymax, c.zmin, c.zmax = xmin, xmax, ymin, ymax, zmin, zmax
    c.lx, c.ly, c.lz = xmax - xmin, ymax - ymin, zmax - zmin
    c.dt_out = dt_out
    c.nxs, c.nys, c.nzs = nx, ny, nz
    c.topox = c.topoy = c.topoz = 1
    c.nvar = 8
    return c


@dataclass
class ParticleSet:
    """particle_type as numpy structure-of-arrays."""
    arrays: dict

    @classmethod
    def empty(cls, n: int) -> "ParticleSet":
        return cls({name: np.zeros(n, dtype=t) for name, t in _abi.PARTICLE_FIELDS})

    def __len__(self) -> int:
        return len(self.arrays["x"])

    def __getitem__(self, k):
        return self.arrays[k]

    def ctypes(self) -> _abi.Particles:
        s = _abi.Particles()
        for name, t in _abi.PARTICLE_FIELDS:
            a = self.arrays[name]
            assert a.flags["C_CONTIGUOUS"] and a.dtype == np.dtype(t), name
            setattr(s, name, a.ctypes.data_as(C.POINTER(_abi._CT[t])))
        return s

    def copy(self) -> "ParticleSet":
        return ParticleSet({k: v.copy() for k, v in self.arrays.items()})

    def take(self, idx) -> "ParticleSet":
        return ParticleSet({k: np.ascontiguousarray(v[idx]) for k, v in self.arrays.items()})

    def order_by_tags(self) -> "ParticleSet":
        """Canonical order (tag_injected, tag_splitted), for set comparisons."""
        key = (self.arrays["tag_injected"].astype(np.int64) << 32) | \
              (self.arrays["tag_splitted"].astype(np.int64) & 0xFFFFFFFF)
        return self.take(np.argsort(key, kind="stable"))


DUMP_FIELDS = [("x", "f8"), ("y", "f8"), ("z", "f8"), ("p", "f8"), ("v", "f8"), ("mu", "f8"),
               ("weight", "f8"), ("t", "f8"), ("dt", "f8"), ("split_times", "i1"),
               ("count_flag", "i1"), ("origin", "i4"), ("nsteps_tracked", "i4"),
               ("nsteps_pushed", "i4"), ("tag_injected", "i4"), ("tag_splitted", "i4")]


def read_particle_dump(path: str | Path) -> dict:
    """particles_XXXX.dat written by gpat_run (the datasets of the
    reference's particles_XXXX.h5, dump_particles diagnostics.f90:1810-1888)."""
    raw = Path(path).read_bytes()
    n = int(np.frombuffer(raw[:8], np.int64)[0])
    out, off = {}, 8
    for name, t in DUMP_FIELDS:
        size = np.dtype(t).itemsize * n
        out[name] = np.frombuffer(raw[off:off + size], t).copy()
        off += size
    if off != len(raw):
        raise ValueError(f"{path}: {len(raw)} bytes, expected {off} for {n} particles")
    return out


def read_particle_params(conf_path: str | Path, base: _abi.Params | None = None) -> _abi.Params:
    """read_particle_params (particle_module.f90:2778-2878) via the engine."""
    lib = _abi.load()
    p = base if base is not None else make_params()
    rc = lib.gpat_read_particle_params(str(conf_path).encode(), C.byref(p))
    if rc != _abi.GPAT_OK:
        raise GPATError(rc, f"cannot read {conf_path}")
    return p


def load_mhd_config(path: str | Path) -> _abi.MhdConfig:
    lib = _abi.load()
    c = _abi.MhdConfig()
    rc = lib.gpat_load_mhd_config(str(path).encode(), C.byref(c))
    if rc != _abi.GPAT_OK:
        raise GPATError(rc, f"cannot read {path}")
    return c


class Engine:
    """One GPAT rank's mover state on one GPU."""

    def __init__(self, params: _abi.Params, mhd_config: _abi.MhdConfig, device: int = 0):
        self.lib = _abi.load()
        self.params = params
        self.cfg = mhd_config
        self.device = device
        self.h = _abi.Handle()
        rc = self.lib.gpat_create(C.byref(params), C.byref(mhd_config), device, C.byref(self.h))
        if rc != _abi.GPAT_OK:
            raise GPATError(rc, "gpat_create failed")
        self.ndim = params.ndim
        self.nxg = mhd_config.nx + 4
        self.nyg = mhd_config.ny + 4 if params.ndim > 1 else 1
        self.nzg = mhd_config.nz + 4 if params.ndim == 3 else 1

    # -- plumbing ---------------------------------------------------------------
    def _check(self, rc: int):
        if rc == _abi.GPAT_OK:
            return
        msg = self.lib.gpat_last_error(self.h).decode()
        if rc == _abi.GPAT_ERR_CAPACITY:
            raise GPATCapacityError(rc, msg)
        raise GPATError(rc, msg)

    def close(self):
        if self.h:
            self.lib.gpat_destroy(self.h)
            self.h = _abi.Handle()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        """The engine's cudaStream_t as an integer handle."""
        return self.lib.gpat_stream(self.h) or 0

    # -- time stamps and fields --------------------------------------------------
    def set_tstamps(self, tstamps):
        ts = np.ascontiguousarray(tstamps, dtype=np.float64)
        self._check(self.lib.gpat_set_tstamps(self.h, ts.ctypes.data_as(C.POINTER(C.c_double)),
                                              len(ts)))

    def calc_tstamps_mhd(self, t_start: int, t_end: int):
        self._check(self.lib.gpat_calc_tstamps_mhd(self.h, t_start, t_end))

    def load_tstamps_mhd(self, t_start: int, t_end: int, tmax_mhd: int, dir_mhd_data):
        """load_tstamps_mhd: <dir_mhd_data>time_stamps.dat (varying dt_mhd)."""
        d = str(dir_mhd_data)
        d = d if d.endswith("/") else d + "/"
        self._check(self.lib.gpat_load_tstamps_mhd(self.h, t_start, t_end, tmax_mhd, d.encode()))

    def get_pmax_global(self) -> float:
        v = C.c_double()
        self._check(self.lib.gpat_get_pmax_global(self.h, C.byref(v)))
        return v.value

    def field_shape(self, nvar: int = 8):
        """numpy (C order) shape of a Fortran (nvar, nxg, nyg, nzg) array."""
        return (self.nzg, self.nyg, self.nxg, nvar)

    def set_fields(self, farray: np.ndarray, var_flag: int = 0):
        a = np.ascontiguousarray(farray, dtype=np.float32)
        nvar = a.shape[-1]
        if a.shape != self.field_shape(nvar):
            raise ValueError(f"field array shape {a.shape} != {self.field_shape(nvar)}")
        self._check(self.lib.gpat_set_fields(self.h, var_flag,
                                             a.ctypes.data_as(C.POINTER(C.c_float)), nvar))

    def read_field_data(self, filename: str | Path, var_flag: int = 0):
        self._check(self.lib.gpat_read_field_data(self.h, str(filename).encode(), var_flag))

    def calc_fields_gradients(self, var_flag: int = 0):
        self._check(self.lib.gpat_calc_fields_gradients(self.h, var_flag))

    def copy_fields(self):
        self._check(self.lib.gpat_copy_fields(self.h))

    def get_fields(self, var_flag: int = 0) -> np.ndarray:
        out = np.empty(self.field_shape(32), dtype=np.float32)
        self._check(self.lib.gpat_get_fields(self.h, var_flag,
                                             out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    # -- particles ---------------------------------------------------------------
    def inject_particles_spatial_uniform(self, nptl, dt, dist_flag, particle_v0, ct_mhd,
                                         part_box, power_index=7.0):
        box = (C.c_double * 6)(*part_box)
        self._check(self.lib.gpat_inject_particles_spatial_uniform(
            self.h, int(nptl), dt, dist_flag, particle_v0, ct_mhd, box, power_index))

    def locate_shock_xpos(self) -> np.ndarray:
        """locate_shock_xpos on frame 1: (nzg, nyg) 1-based x indices."""
        S = np.zeros((self.nzg, self.nyg), np.int32)
        self._check(self.lib.gpat_locate_shock_xpos(self.h, S.ctypes.data_as(C.POINTER(C.c_int32))))
        return S

    def inject_particles_at_shock(self, nptl, dt, dist_flag, particle_v0, ct_mhd,
                                  power_index=7.0):
        self._check(self.lib.gpat_inject_particles_at_shock(
            self.h, int(nptl), dt, dist_flag, particle_v0, ct_mhd, power_index))

    def inject_particles_at_x(self, nptl, xpos, dt, dist_flag, particle_v0, ct_mhd,
                              power_index=7.0):
        self._check(self.lib.gpat_inject_particles_at_x(
            self.h, int(nptl), xpos, dt, dist_flag, particle_v0, ct_mhd, power_index))

    def set_fluctuations(self, var_flag=0, db2_slab=None, db2_2d=None, lc_slab=None, lc_2d=None):
        """Turbulence variance / correlation length arrays, each (nzg, nyg, nxg)
        FP32 over the ghost-padded nodes (None keeps that component)."""
        keep = []

        def ptr(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float32)
            keep.append(a)
            return a.ctypes.data_as(C.POINTER(C.c_float))

        self._check(self.lib.gpat_set_fluctuations(self.h, var_flag, ptr(db2_slab), ptr(db2_2d),
                                                   ptr(lc_slab), ptr(lc_2d)))

    def read_magnetic_fluctuation(self, path, var_flag=0):
        self._check(self.lib.gpat_read_magnetic_fluctuation(self.h, str(path).encode(), var_flag))

    def read_correlation_length(self, path, var_flag=0):
        self._check(self.lib.gpat_read_correlation_length(self.h, str(path).encode(), var_flag))

    def get_fluctuations(self, var_flag=0) -> np.ndarray:
        """The (nzg, nyg, nxg, 16) records {db2_slab, db2_2d, lc_slab, lc_2d} x
        {value, d/dx, d/dy, d/dz}."""
        out = np.zeros((self.nzg, self.nyg, self.nxg, 16), np.float32)
        self._check(self.lib.gpat_get_fluctuations(self.h, var_flag,
                                                   out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def _grid_counts(self):
        return [self.nxg, self.nyg, self.nzg][:self.params.ndim]

    def set_grid_positions(self, xpos, ypos=None, zpos=None):
        """Node positions of a non-uniform grid (ghost nodes included: nxg,
        nyg, nzg values); set before calc_fields_gradients."""
        keep = [None if a is None else np.ascontiguousarray(a, np.float64)
                for a in (xpos, ypos, zpos)]
        for a, n in zip(keep, self._grid_counts()):
            if a is None or len(a) != n:
                raise ValueError(f"expected {n} grid positions")
        ptrs = [None if a is None else a.ctypes.data_as(C.POINTER(C.c_double)) for a in keep]
        self._check(self.lib.gpat_set_grid_positions(self.h, *ptrs))

    def read_grid_positions(self, dir_mhd_data):
        """read_global_grid_positions: <dir>xpos.dat, ypos.dat, zpos.dat."""
        d = str(dir_mhd_data)
        if not d.endswith("/"):
            d += "/"
        self._check(self.lib.gpat_read_grid_positions(self.h, d.encode()))

    def get_grid_positions(self):
        out = [np.zeros(n, np.float64) for n in self._grid_counts()]
        ptrs = [a.ctypes.data_as(C.POINTER(C.c_double)) for a in out] + \
               [None] * (3 - len(out))
        self._check(self.lib.gpat_get_grid_positions(self.h, *ptrs))
        return out

    def init_acc_surface(self, norm1, norm2=None, is_intersection=True):
        """init_acc_surface: norm "+y" etc.; a second surface when norm2."""
        self._check(self.lib.gpat_init_acc_surface(
            self.h, norm1.encode(), norm2.encode() if norm2 else None, int(is_intersection)))

    def set_acc_surface(self, var_flag, surface1, surface2=None):
        """Surface heights, numpy arrays (n2, n1) over the ghost-padded plane
        (first index fastest)."""
        keep = [None if a is None else np.ascontiguousarray(a, np.float64)
                for a in (surface1, surface2)]
        ptr = [None if a is None else a.ctypes.data_as(C.POINTER(C.c_double)) for a in keep]
        self._check(self.lib.gpat_set_acc_surface(self.h, var_flag, *ptr))

    def read_acc_surface(self, var_flag, filename1, filename2=None):
        self._check(self.lib.gpat_read_acc_surface(
            self.h, var_flag, str(filename1).encode(),
            str(filename2).encode() if filename2 else None))

    def count_cells_large(self, quantity, qmin, part_box) -> int:
        """get_ncells_large_jz / _absj / _divv / _rho (quantity: _abi.LARGE_*)."""
        box = (C.c_double * 6)(*part_box)
        n = C.c_int64()
        self._check(self.lib.gpat_count_cells_large(self.h, quantity, qmin, box, C.byref(n)))
        return n.value

    def inject_particles_at_large(self, quantity, nptl, dt, dist_flag, particle_v0, ct_mhd,
                                  inject_same_nptl, qmin, ncells_norm, part_box,
                                  power_index=7.0) -> int:
        """inject_particles_at_large_jz / _absj / _divv / _rho; returns the
        number of particles it injected."""
        box = (C.c_double * 6)(*part_box)
        n = C.c_int64()
        self._check(self.lib.gpat_inject_particles_at_large(
            self.h, quantity, int(nptl), dt, dist_flag, particle_v0, ct_mhd,
            int(bool(inject_same_nptl)), qmin, int(ncells_norm), box, power_index, C.byref(n)))
        return n.value

    def put_particles(self, ps: ParticleSet):
        s = ps.ctypes()
        self._check(self.lib.gpat_put_particles(self.h, C.byref(s), len(ps)))

    def get_particles(self, out: ParticleSet | None = None) -> ParticleSet:
        """Copies the particle set to the host.  With ``out`` (capacity >=
        nptl_current, e.g. pinned buffers) it fills those arrays and returns
        a view of the first nptl_current entries."""
        n = self.counters().nptl_current
        ps = ParticleSet.empty(n) if out is None else out
        if len(ps) < n:
            raise ValueError(f"output capacity {len(ps)} < {n} particles")
        s = ps.ctypes()
        got = C.c_int64()
        self._check(self.lib.gpat_get_particles(self.h, C.byref(s), len(ps), C.byref(got)))
        return ps if out is None else ParticleSet({k: v[:n] for k, v in ps.arrays.items()})

    def particle_distributions_mu(self, nmu: int):
        """fglobal(nmu, npp_global) and counts, as numpy (npp_global, nmu)."""
        npp = self.params.npp_global
        f = np.zeros((npp, nmu), np.float64)
        c = np.zeros((npp, nmu), np.uint64)
        self._check(self.lib.gpat_calc_particle_distributions_mu(
            self.h, nmu, f.ctypes.data_as(C.POINTER(C.c_double)),
            c.ctypes.data_as(C.POINTER(C.c_uint64))))
        return f, c

    def escaped_distributions_mu(self, nmu: int):
        """fescaped(nmu, npp_global, 2 ndim) as numpy (2 ndim, npp_global, nmu)."""
        npp, nf = self.params.npp_global, 2 * self.params.ndim
        f = np.zeros((nf, npp, nmu), np.float64)
        c = np.zeros((nf, npp, nmu), np.uint64)
        self._check(self.lib.gpat_calc_escaped_distributions_mu(
            self.h, nmu, f.ctypes.data_as(C.POINTER(C.c_double)),
            c.ctypes.data_as(C.POINTER(C.c_uint64))))
        return f, c

    def local_escaped_distribution(self, pmin, pmax, npbins, nmu=1, rx=1, ry=1, rz=1):
        """(fx, fy, fz), (cx, cy, cz): numpy (2, nrz, nry, npbins, nmu),
        (2, nrz, nrx, npbins, nmu) and (2, nry, nrx, npbins, nmu), i.e.
        Fortran fx(nmu, npbins, nry, nrz, 2) etc.; faces beyond ndim are
        None."""
        spec = _abi.LocalDist(pmin, pmax, npbins, nmu, rx, ry, rz, 0)
        dims = (C.c_int32 * 5)()
        self._check(self.lib.gpat_local_distribution_dims(self.h, C.byref(spec), dims))
        nmu_, npb, nrx, nry, nrz = list(dims)
        shapes = [(2, nrz, nry, npb, nmu_), (2, nrz, nrx, npb, nmu_), (2, nry, nrx, npb, nmu_)]
        nd = self.params.ndim
        f = [np.zeros(s, np.float64) if k < nd else None for k, s in enumerate(shapes)]
        c = [np.zeros(s, np.uint64) if k < nd else None for k, s in enumerate(shapes)]
        dp = lambda a: None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))
        up = lambda a: None if a is None else a.ctypes.data_as(C.POINTER(C.c_uint64))
        self._check(self.lib.gpat_calc_local_escaped_distribution(
            self.h, C.byref(spec), dp(f[0]), dp(f[1]), dp(f[2]), up(c[0]), up(c[1]), up(c[2])))
        return tuple(f), tuple(c)

    def get_escaped_particles(self) -> ParticleSet:
        """escaped_ptls: particles removed through an open boundary by mover
        calls with dump_escaped_dist since the last reset_escaped_particles."""
        got = C.c_int64()
        empty = ParticleSet.empty(0)
        rc = self.lib.gpat_get_escaped_particles(self.h, C.byref(empty.ctypes()), 0,
                                                 C.byref(got))
        if rc not in (_abi.GPAT_OK, _abi.GPAT_ERR_CAPACITY):
            self._check(rc)
        ps = ParticleSet.empty(got.value)
        self._check(self.lib.gpat_get_escaped_particles(self.h, C.byref(ps.ctypes()), len(ps),
                                                        C.byref(got)))
        return ps

    # -- particle tracking -------------------------------------------------------
    def init_particle_tracking(self, tags, nsteps_interval=10):
        """init_particle_tracking: tags is tags_tracking as (nptl_tracking,
        nrows), one row per tracked particle: origin, tag_injected and
        tag_splitted after each split."""
        t = np.ascontiguousarray(tags, dtype=np.int32)
        if t.ndim != 2:
            raise ValueError("tags must be (nptl_tracking, nrows)")
        self._check(self.lib.gpat_init_particle_tracking(
            self.h, t.ctypes.data_as(C.POINTER(C.c_int32)), t.shape[1], t.shape[0],
            nsteps_interval))

    def read_particle_tracking(self, path, nsteps_interval=10):
        self._check(self.lib.gpat_read_particle_tracking(self.h, str(path).encode(),
                                                         nsteps_interval))

    def tracking_dims(self):
        """(nsteps_tracking_max, nptl_tracking, dropped records)."""
        s, n, d = C.c_int64(), C.c_int32(), C.c_int64()
        self._check(self.lib.gpat_tracking_dims(self.h, C.byref(s), C.byref(n), C.byref(d)))
        return s.value, n.value, d.value

    def get_tracked_particles(self) -> dict:
        """sync_tracked_particles and the datasets of dump_tracked_particles:
        each field shaped (nptl_tracking, nsteps_tracking_max)."""
        nsteps, ntrk, _ = self.tracking_dims()
        ps = ParticleSet.empty(nsteps * ntrk)
        self._check(self.lib.gpat_get_tracked_particles(self.h, C.byref(ps.ctypes())))
        return {k: v.reshape(ntrk, nsteps) for k, v in ps.arrays.items()}

    def free_particle_tracking(self):
        self._check(self.lib.gpat_free_particle_tracking(self.h))

    @property
    def nptl_current(self) -> int:
        return self.counters().nptl_current

    # -- the mover path -----------------------------------------------------------
    def particle_mover(self, focused_transport=False, nlgc=False, kperp_kpara=0.01,
                       nsteps_interval=10, mhd_tframe=1, num_fine_steps=1,
                       dump_escaped_dist=False):
        self._check(self.lib.gpat_particle_mover(
            self.h, int(focused_transport), int(nlgc), kperp_kpara, nsteps_interval,
            mhd_tframe, num_fine_steps, int(dump_escaped_dist)))

    def set_mover_tiles(self, bx=0, by=0, bz=0, hx=0, hy=0, hz=0, threads=0, items=0):
        """Brick shape of the split-precision mover (gpat_set_mover_tiles):
        bx = 0 gathers field records from device memory, bx > 0 stages
        bricks of bx x by x bz cells plus hx, hy, hz halo cells per side in
        shared memory."""
        self._check(self.lib.gpat_set_mover_tiles(self.h, bx, by, bz, hx, hy, hz, threads, items))

    def mover_tiles(self) -> dict:
        out = (C.c_int * 8)()
        self._check(self.lib.gpat_get_mover_tiles(self.h, out))
        return dict(zip(("bx", "by", "bz", "hx", "hy", "hz", "threads", "items"), list(out)))

    def split_particle(self, split_ratio=2.72, pmin_split=2.0, nsteps_interval=10):
        self._check(self.lib.gpat_split_particle(self.h, split_ratio, pmin_split, nsteps_interval))

    def calc_particle_distributions(self):
        """Global f(p): (fglobal[npp], counts[npp])."""
        npp = self.params.npp_global
        f = np.zeros(npp, dtype=np.float64)
        c = np.zeros(npp, dtype=np.uint64)
        self._check(self.lib.gpat_calc_particle_distributions(
            self.h, f.ctypes.data_as(C.POINTER(C.c_double)),
            c.ctypes.data_as(C.POINTER(C.c_uint64))))
        return f, c

    def local_distribution(self, pmin, pmax, npbins, nmu=1, rx=1, ry=1, rz=1):
        """One local distribution: (flocal, counts) shaped (nrz, nry, nrx,
        npbins, nmu), i.e. Fortran flocal(nmu, npbins, nrx, nry, nrz)."""
        spec = _abi.LocalDist(pmin, pmax, npbins, nmu, rx, ry, rz, 0)
        dims = (C.c_int32 * 5)()
        self._check(self.lib.gpat_local_distribution_dims(self.h, C.byref(spec), dims))
        shape = tuple(reversed(list(dims)))
        f = np.zeros(shape, np.float64)
        c = np.zeros(shape, np.uint64)
        self._check(self.lib.gpat_calc_local_distribution(
            self.h, C.byref(spec), f.ctypes.data_as(C.POINTER(C.c_double)),
            c.ctypes.data_as(C.POINTER(C.c_uint64))))
        return f, c

    def calc_escaped_distributions(self):
        """(fescaped, counts) shaped (2 * ndim, npp_global)."""
        npp = self.params.npp_global
        f = np.zeros((2 * self.ndim, npp), np.float64)
        c = np.zeros((2 * self.ndim, npp), np.uint64)
        self._check(self.lib.gpat_calc_escaped_distributions(
            self.h, f.ctypes.data_as(C.POINTER(C.c_double)),
            c.ctypes.data_as(C.POINTER(C.c_uint64))))
        return f, c

    def reset_escaped_particles(self):
        self._check(self.lib.gpat_reset_escaped_particles(self.h))

    def pbins_edges(self) -> np.ndarray:
        e = np.zeros(self.params.npp_global + 1, dtype=np.float64)
        self._check(self.lib.gpat_pbins_edges(self.h, e.ctypes.data_as(C.POINTER(C.c_double))))
        return e

    def quick_check(self) -> dict:
        out = (C.c_double * 8)()
        self._check(self.lib.gpat_quick_check(self.h, out))
        keys = ("nptl_current", "nptl_split", "ntot", "leak", "leak_negp", "pdt_min",
                "pdt_max", "pdt_avg")
        return dict(zip(keys, list(out)))

    def counters(self) -> _abi.Counters:
        c = _abi.Counters()
        self._check(self.lib.gpat_get_counters(self.h, C.byref(c)))
        return c

    def set_counters(self, c: _abi.Counters):
        self._check(self.lib.gpat_set_counters(self.h, C.byref(c)))


class Batch:
    """Independent runs moved together (gpat_batch_*): one persistent,
    graph-replayed launch per chunk for all of them."""

    def __init__(self, engines):
        self.engines = list(engines)
        self.lib = self.engines[0].lib
        self.b = _abi.Batch()
        arr = (_abi.Handle * len(self.engines))(*[e.h for e in self.engines])
        rc = self.lib.gpat_batch_create(arr, len(self.engines), C.byref(self.b))
        if rc != _abi.GPAT_OK:
            raise GPATError(rc, "gpat_batch_create failed")

    def _check(self, rc: int):
        if rc != _abi.GPAT_OK:
            raise GPATError(rc, self.lib.gpat_batch_last_error(self.b).decode())

    def _frames(self, mhd_tframe):
        if isinstance(mhd_tframe, int):
            mhd_tframe = [mhd_tframe] * len(self.engines)
        return (C.c_int * len(self.engines))(*mhd_tframe)

    def particle_mover(self, mhd_tframe=1, nlgc=False, kperp_kpara=0.01, nsteps_interval=10,
                       num_fine_steps=1):
        self._check(self.lib.gpat_batch_particle_mover(
            self.b, self._frames(mhd_tframe), int(nlgc), kperp_kpara, nsteps_interval,
            num_fine_steps))

    def autotune(self, mhd_tframe=1, nlgc=False, kperp_kpara=0.01, nsteps_interval=10,
                 num_fine_steps=1, cache=None) -> dict:
        """gpat_batch_autotune.  cache: a JSON file of earlier choices keyed by
        the GPU and a hash of the runs' grids, sizes and parameters; a hit
        applies the stored choice without timing."""
        key = self._cache_key(nlgc) if cache else None
        if cache:
            table = _read_cache(cache)
            if key in table:
                c = table[key]
                self.set_tuning(c["minb"], c["grab"], c["chunk_pushes"])
                return dict(c, cached=True)
        t = _abi.BatchTuning()
        self._check(self.lib.gpat_batch_autotune(
            self.b, self._frames(mhd_tframe), int(nlgc), kperp_kpara, nsteps_interval,
            num_fine_steps, C.byref(t)))
        out = dict(minb=t.minb, grab=t.grab, pushes_per_s=t.pushes_per_s,
                   chunk_pushes=t.chunk_pushes, default_pushes_per_s=t.default_pushes_per_s)
        if cache:
            table = _read_cache(cache)
            table[key] = out
            _write_cache(cache, table)
        return out

    def _cache_key(self, nlgc) -> str:
        import hashlib
        import torch
        gpu = torch.cuda.get_device_name(self.engines[0].device) if torch.cuda.is_available() else "?"
        desc = [(e.cfg.nx, e.cfg.ny, e.cfg.nz, e.nptl_current, e.params.kpara0, e.params.kret,
                 e.params.ndim, e.params.bin_interval) for e in self.engines]
        return gpu + ":" + hashlib.sha1(repr((desc, bool(nlgc))).encode()).hexdigest()[:16]

    def tuning(self) -> dict:
        t = _abi.BatchTuning()
        self._check(self.lib.gpat_batch_get_tuning(self.b, C.byref(t)))
        return dict(minb=t.minb, grab=t.grab, pushes_per_s=t.pushes_per_s,
                    chunk_pushes=t.chunk_pushes)

    def set_tuning(self, minb, grab, chunk_pushes=0):
        t = _abi.BatchTuning(minb, grab, 0.0, chunk_pushes, 0, 0.0)
        self._check(self.lib.gpat_batch_set_tuning(self.b, C.byref(t)))

    def stats(self) -> dict:
        ms, pushes, launches = C.c_double(), C.c_uint64(), C.c_int64()
        self._check(self.lib.gpat_batch_stats(self.b, C.byref(ms), C.byref(pushes),
                                              C.byref(launches)))
        return dict(ms=ms.value, pushes=pushes.value, graph_launches=launches.value)

    def close(self):
        if self.b:
            self.lib.gpat_batch_destroy(self.b)
            self.b = _abi.Batch()


class Mlp:
    """The learned-splitting importance network (gpat_mlp_*)."""

    def __init__(self, device: int = 0, seed: int = 1, record_capacity: int = 0):
        self.lib = _abi.load()
        self.m = _abi.Mlp()
        rc = self.lib.gpat_mlp_create(device, seed, int(record_capacity), C.byref(self.m))
        if rc != _abi.GPAT_OK:
            raise GPATError(rc, "gpat_mlp_create failed")

    def _check(self, rc: int):
        if rc != _abi.GPAT_OK:
            raise GPATError(rc, self.lib.gpat_mlp_last_error(self.m).decode())

    @staticmethod
    def _f32(a):
        a = np.ascontiguousarray(a, dtype=np.float32)
        return a, a.ctypes.data_as(C.POINTER(C.c_float))

    def set_params(self, params=None, norm=None):
        p, pp = self._f32(params) if params is not None else (None, None)
        q, qq = self._f32(norm) if norm is not None else (None, None)
        self._check(self.lib.gpat_mlp_set_params(self.m, pp, qq))

    def get_params(self):
        p = np.zeros(_abi.MLP_PARAMS, np.float32)
        q = np.zeros(2 * _abi.MLP_FEATURES, np.float32)
        self._check(self.lib.gpat_mlp_get_params(self.m, self._f32(p)[1], self._f32(q)[1]))
        return p, q

    def forward(self, x) -> np.ndarray:
        x, xp = self._f32(x)
        z = np.zeros(len(x), np.float32)
        self._check(self.lib.gpat_mlp_forward(self.m, xp, len(x),
                                              z.ctypes.data_as(C.POINTER(C.c_float))))
        return z

    def loss_grad(self, x, y):
        x, xp = self._f32(x)
        y, yp = self._f32(y)
        loss = C.c_float()
        g = np.zeros(_abi.MLP_PARAMS, np.float32)
        self._check(self.lib.gpat_mlp_loss_grad(self.m, xp, yp, len(x), C.byref(loss),
                                                g.ctypes.data_as(C.POINTER(C.c_float))))
        return float(loss.value), g

    def set_records(self, x, labels):
        x, xp = self._f32(x)
        y, yp = self._f32(labels)
        self._check(self.lib.gpat_mlp_set_records(self.m, xp, yp, len(x)))

    def clear_records(self):
        self._check(self.lib.gpat_mlp_clear_records(self.m))

    def record(self, eng, t_norm) -> int:
        n = C.c_int64()
        self._check(self.lib.gpat_mlp_record(self.m, eng.h, t_norm, C.byref(n)))
        return n.value

    def label(self, eng, p_threshold):
        npos, nrec = C.c_int64(), C.c_int64()
        self._check(self.lib.gpat_mlp_label(self.m, eng.h, p_threshold, C.byref(npos),
                                            C.byref(nrec)))
        return npos.value, nrec.value

    def train(self, epochs=3, batch=8192, lr=2e-3, neg_keep=1.0, seed=1) -> float:
        loss = C.c_double()
        self._check(self.lib.gpat_mlp_train(self.m, epochs, batch, lr, neg_keep, seed,
                                            C.byref(loss)))
        return loss.value

    def score(self, eng, t_norm):
        """(mean z, log sum w exp(z), log sum w) over the run's live particles."""
        z, lse, lsw = C.c_double(), C.c_double(), C.c_double()
        self._check(self.lib.gpat_mlp_score(self.m, eng.h, t_norm, C.byref(z), C.byref(lse),
                                            C.byref(lsw)))
        return z.value, lse.value, lsw.value

    def close(self):
        if self.m:
            self.lib.gpat_mlp_destroy(self.m)
            self.m = _abi.Mlp()


def window_params(log_sum_wexpz, log_sum_w, target, defensive=0.1):
    """(z_ref, z_floor) that aim weighted splitting at `target` particles with
    defensive importance exp(z) + defensive * (weighted mean of exp(z)):
    no roulette survivor then weighs more than about
    (1 + defensive) / defensive * sum(w) / target.  defensive = 0 gives the
    bare importance exp(z) (z_floor = -inf)."""
    if defensive <= 0.0:
        return log_sum_wexpz - math.log(target), -math.inf
    z_floor = math.log(defensive) + log_sum_wexpz - log_sum_w
    return log_sum_wexpz + math.log1p(defensive) - math.log(target), z_floor


class FusedWindow:
    """z_ref and z_floor for learned splitting inside the mover
    (set_mover_learned), interval after interval.  The mover judges the
    particles that finish an interval with sums taken in the interval
    before (the judged particles' sums are only complete at its end), and
    the network's outputs drift as time advances and particles move: the
    log-sum of w exp(z) is therefore carried one interval ahead by its last
    change (at most `max_step` in magnitude), which keeps the population
    near `target`.  Usage: start() with Mlp.score's sums before the first
    interval, params() before each mover call, update() with
    mover_learned_stats after it."""

    def __init__(self, target, defensive=0.1, max_step=2.0):
        self.target, self.defensive, self.max_step = target, defensive, max_step
        self.lse = self.lsw = self.prev = None

    def start(self, log_sum_wexpz, log_sum_w):
        self.lse, self.lsw, self.prev = log_sum_wexpz, log_sum_w, None

    def update(self, stats: dict):
        if stats["judged"] > 0 and math.isfinite(stats["log_sum_wexpz"]):
            self.prev = self.lse
            self.lse, self.lsw = stats["log_sum_wexpz"], stats["log_sum_w"]

    def params(self):
        lse = self.lse
        if self.prev is not None:
            lse += max(-self.max_step, min(self.max_step, self.lse - self.prev))
        return window_params(lse, self.lsw, self.target, self.defensive)


def weighted_split(eng, mlp: Mlp, t_norm, w_ref, z_ref, window_ratio=4.0, max_level=4,
                   z_floor=-math.inf):
    """gpat_weighted_split; returns (children created, particles killed)."""
    ns, nk = C.c_int64(), C.c_int64()
    eng._check(eng.lib.gpat_weighted_split(eng.h, mlp.m, t_norm, w_ref, z_ref, z_floor,
                                           window_ratio, max_level, C.byref(ns), C.byref(nk)))
    return ns.value, nk.value


def set_mover_learned(eng, mlp, t_norm=0.0, w_ref=1.0, z_ref=0.0, window_ratio=4.0,
                      max_level=3, z_floor=-math.inf):
    """gpat_set_mover_learned: learned splitting of particles as they finish
    an interval, inside the mover launch; mlp = None turns it off."""
    eng._check(eng.lib.gpat_set_mover_learned(eng.h, mlp.m if mlp is not None else None, t_norm,
                                              w_ref, z_ref, z_floor, window_ratio, max_level))


def mover_learned_stats(eng) -> dict:
    """gpat_get_mover_learned after a mover call."""
    lse, lsw = C.c_double(), C.c_double()
    j, ns, nk = C.c_int64(), C.c_int64(), C.c_int64()
    eng._check(eng.lib.gpat_get_mover_learned(eng.h, C.byref(lse), C.byref(lsw), C.byref(j),
                                              C.byref(ns), C.byref(nk)))
    return dict(log_sum_wexpz=lse.value, log_sum_w=lsw.value, judged=j.value, nsplit=ns.value,
                nkilled=nk.value)


def _read_cache(path) -> dict:
    import json
    try:
        return json.loads(Path(path).read_text())
    except (OSError, ValueError):
        return {}


def _write_cache(path, table: dict):
    import json
    Path(path).write_text(json.dumps(table, indent=1, sort_keys=True))


def tail_weights(eng, p_threshold):
    """(count, sum w, sum w^2) of live particles with p > p_threshold."""
    n, w, w2 = C.c_int64(), C.c_double(), C.c_double()
    eng._check(eng.lib.gpat_tail_weights(eng.h, p_threshold, C.byref(n), C.byref(w),
                                         C.byref(w2)))
    return n.value, w.value, w2.value


def tail_by_ancestor(eng, p_threshold, n_injected):
    """Tail statistics of a run with splitting, one sample per injected
    particle.  Copies split from one parent share its history, so the
    particles of a lineage are not independent samples: the tail weight W_a
    of all live descendants (same tag_injected) of each of the n_injected
    ancestors is.  Returns the tail fraction sum(W_a) / n_injected, its Monte
    Carlo error sqrt(sum W_a^2) / n_injected, the effective sample size
    (sum W_a)^2 / sum W_a^2, and the numbers of tail particles and of
    ancestors with descendants in the tail."""
    ps = eng.get_particles()
    m = (ps["count_flag"] == 1) & (ps["p"] > p_threshold)
    tags = ps["tag_injected"][m].astype(np.int64)
    w = ps["weight"][m]
    if len(w) == 0:
        return dict(fraction=0.0, sigma=0.0, ess=0.0, particles=0, ancestors=0)
    _, inv = np.unique(tags, return_inverse=True)
    W = np.bincount(inv, weights=w)
    s1, s2 = float(W.sum()), float((W * W).sum())
    return dict(fraction=s1 / n_injected, sigma=math.sqrt(s2) / n_injected,
                ess=s1 * s1 / s2 if s2 > 0 else 0.0, particles=int(m.sum()),
                ancestors=int(len(W)))
