"""ctypes binding of the CPU oracle (oracle/gpat_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
the CPU-baseline leg of bench.py as the checker.  The product never loads it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
LIB_PATH = ORACLE_DIR / "_build" / "libgpat_oracle.so"

d, i32, i64, u32, u64 = C.c_double, C.c_int32, C.c_int64, C.c_uint32, C.c_uint64
P = C.POINTER


class OrcMhdConfig(C.Structure):
    _fields_ = [(n, d) for n in ("dx", "dy", "dz", "xmin", "ymin", "zmin", "xmax", "ymax", "zmax",
                                 "lx", "ly", "lz", "dt_out")] + \
               [(n, i32) for n in ("nx", "ny", "nz", "nxs", "nys", "nzs", "topox", "topoy", "topoz",
                                   "nvar", "bcx", "bcy", "bcz")]


class OrcParams(C.Structure):
    _fields_ = [
        ("b0", d), ("p0", d), ("pmin", d), ("pmax", d),
        ("gamma_turb", d), ("pindex", d), ("kpara0", d), ("kret", d),
        ("dt_min_rel", d), ("dt_max_rel", d),
        ("acc_region", d * 6),
        ("drift1", d), ("drift2", d),
        ("momentum_dependency", i32), ("mag_dependency", i32), ("acc_region_flag", i32),
        ("charge", i32),
        ("check_drift_2d", i32), ("ndim", i32), ("pbcx", i32), ("pbcy", i32), ("pbcz", i32),
        ("npp_global", i32),
        ("seed", u64),
        ("noise", i32), ("focused_transport", i32), ("nlgc", i32), ("dpp_wave", i32),
        ("duu0", d), ("kperp_kpara", d), ("dpp_shear", i32), ("weak_scattering", i32),
        ("tau0", d), ("deltab_flag", i32), ("correlation_flag", i32),
        ("spherical_coord", i32), ("nonuniform_grid", i32), ("include_3rd_dim", i32),
    ]

# Mover arguments of the reference carried in OrcParams rather than in the
# engine's parameter block.
_MOVER_ARGS = ("focused_transport", "nlgc", "kperp_kpara")


FIELDS = [
    ("x", "f8"), ("y", "f8"), ("z", "f8"), ("p", "f8"), ("v", "f8"), ("mu", "f8"),
    ("weight", "f8"), ("t", "f8"), ("dt", "f8"),
    ("split_times", "i1"), ("count_flag", "i1"),
    ("origin", "i4"), ("nsteps_tracked", "i4"), ("nsteps_pushed", "i4"),
    ("tag_injected", "i4"), ("tag_splitted", "i4"), ("rng_ctr", "u4"),
]
_CT = {"f8": C.c_double, "i1": C.c_int8, "i4": C.c_int32, "u4": C.c_uint32}


class OrcParticles(C.Structure):
    _fields_ = [(n, P(_CT[t])) for n, t in FIELDS]


class OrcCounters(C.Structure):
    _fields_ = [("leak_hi", u64), ("leak_lo", u64), ("leak_negp_hi", u64), ("leak_negp_lo", u64),
                ("steps", u64), ("nptl_escaped", i64), ("nptl_split", i64), ("tag_max", i64)]

    def leak(self) -> float:
        return fixed_to_double(self.leak_hi, self.leak_lo)

    def leak_negp(self) -> float:
        return fixed_to_double(self.leak_negp_hi, self.leak_negp_lo)


def fixed_to_double(hi: int, lo: int) -> float:
    return float(hi) + float(lo) * (1.0 / 18446744073709551616.0)


_lib = None


def build() -> Path:
    """Compiles the oracle with its Makefile (gcc, -ffp-contract=off)."""
    src = ORACLE_DIR / "gpat_oracle.c"
    if not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-C", str(ORACLE_DIR), "-B", "_build/libgpat_oracle.so"],
                       check=True, capture_output=True)
    return LIB_PATH


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB_PATH))
        lib.orc_philox4x32_10.argtypes = [P(u32), P(u32), P(u32)]
        lib.orc_u01.restype = d
        lib.orc_u01.argtypes = [u32, u32]
        lib.orc_calc_fields_gradients.argtypes = [P(C.c_float), C.c_int, C.c_int, C.c_int, C.c_int,
                                                  d, d, d]
        lib.orc_get_interp_paramters.argtypes = [C.c_int, d, d, d, P(i32), P(d)]
        lib.orc_interp_fields.argtypes = [P(C.c_float), P(C.c_float), C.c_int, C.c_int, C.c_int,
                                          C.c_int, P(i32), P(d), d, P(d)]
        lib.orc_calc_spatial_diffusion_coefficients.argtypes = [P(OrcParams), d, d, P(d), P(d),
                                                                P(d)]
        lib.orc_calc_aux_gradients.argtypes = [P(C.c_float), C.c_int, C.c_int, C.c_int, C.c_int,
                                               d, d, d]
        lib.orc_particle_mover.restype = i64
        lib.orc_particle_mover.argtypes = [P(OrcParams), P(OrcMhdConfig), P(C.c_float),
                                           P(C.c_float), P(C.c_float), P(C.c_float), C.c_int,
                                           P(OrcParticles), i64, d, d, C.c_int, C.c_int, C.c_int,
                                           P(OrcCounters)]
        lib.orc_remove_particles.restype = i64
        lib.orc_remove_particles.argtypes = [P(OrcParticles), i64, P(OrcCounters)]
        lib.orc_split_particle.restype = i64
        lib.orc_split_particle.argtypes = [P(OrcParams), P(OrcParticles), i64, i64, d, d,
                                           P(OrcCounters)]
        lib.orc_pbins_edges.argtypes = [P(OrcParams), P(d)]
        lib.orc_calc_particle_distributions.argtypes = [P(OrcParams), P(OrcParticles), i64,
                                                        P(u64), P(u64), P(u64), P(d)]
        lib.orc_inject_spatial_uniform.restype = i64
        lib.orc_inject_spatial_uniform.argtypes = [P(OrcParams), P(OrcParticles), i64, i64, i64, d,
                                                   C.c_int, d, d, d, P(d), d, P(OrcCounters)]
        lib.orc_inject_at_x.restype = i64
        lib.orc_inject_at_x.argtypes = [P(OrcParams), P(OrcMhdConfig), P(OrcParticles), i64, i64,
                                        i64, d, d, C.c_int, d, d, d, P(OrcCounters)]
        lib.orc_locate_shock_xpos.argtypes = [P(C.c_float), C.c_int, C.c_int, C.c_int, P(i32)]
        lib.orc_inject_at_shock.restype = i64
        lib.orc_inject_at_shock.argtypes = [P(OrcParams), P(OrcMhdConfig), P(i32), C.c_int,
                                            C.c_int, P(OrcParticles), i64, i64, i64, d, C.c_int,
                                            d, d, d, P(OrcCounters)]
        lib.orc_count_cells_large.restype = i64
        lib.orc_count_cells_large.argtypes = [P(OrcParams), P(OrcMhdConfig), P(C.c_float),
                                              P(C.c_float), C.c_int, d, P(d)]
        lib.orc_inject_at_large.restype = i64
        lib.orc_inject_at_large.argtypes = [P(OrcParams), P(OrcMhdConfig), P(C.c_float),
                                            P(C.c_float), P(OrcParticles), i64, i64, i64, d,
                                            C.c_int, d, d, d, C.c_int, d, P(d), d,
                                            P(OrcCounters)]
        lib.orc_quick_check.argtypes = [P(OrcParticles), i64, P(d)]
        lib.orc_set_escaped_histogram.argtypes = [C.c_int, d, d, P(u64), P(u64), P(u64)]
        lib.orc_set_escaped_store.argtypes = [P(OrcParticles), i64, P(i64)]
        lib.orc_calc_local_distribution.argtypes = [P(OrcMhdConfig), C.c_int, C.c_int, C.c_int,
                                                    d, d, C.c_int,
                                                    C.c_int, C.c_int, C.c_int, C.c_int,
                                                    P(OrcParticles), i64, P(u64), P(u64), P(u64),
                                                    P(d)]
        lib.orc_calc_local_escaped_distribution.argtypes = (
            [P(OrcMhdConfig), C.c_int, C.c_int, C.c_int, d, d] + [C.c_int] * 5 +
            [P(OrcParticles), i64] + [P(u64)] * 9)
        lib.orc_calc_distribution_mu.argtypes = [P(OrcParams), P(OrcParticles), i64, C.c_int,
                                                 C.c_int, C.c_int, P(u64), P(u64), P(u64)]
        lib.orc_set_grid_positions.argtypes = [P(d), P(d), P(d), C.c_int, C.c_int, C.c_int]
        lib.orc_set_acc_surface.argtypes = [C.c_int] * 6 + [P(d)] * 4 + [C.c_int] * 3
        lib.orc_set_tracking.argtypes = [P(i32), C.c_int, C.c_int, i64, P(OrcParticles)]
        lib.orc_tracking_dropped.restype = i64
        lib.orc_nsteps_tracking_max.restype = i64
        lib.orc_nsteps_tracking_max.argtypes = [d, C.c_int]
        lib.orc_uniform_grid_positions.argtypes = [C.c_int, d, d, P(d)]
        lib.orc_binary_search.restype = C.c_int
        lib.orc_binary_search.argtypes = [P(d), C.c_int, d]
        lib.orc_calc_fields_gradients_nonuniform.argtypes = [P(C.c_float), C.c_int, C.c_int,
                                                             C.c_int, C.c_int]
        lib.orc_calc_aux_gradients_nonuniform.argtypes = [P(C.c_float), C.c_int, C.c_int,
                                                          C.c_int, C.c_int]
        lib.orc_grid_interp_paramters.argtypes = [P(OrcParams), P(OrcMhdConfig), d, d, d, P(i32),
                                                  P(d)]
        _lib = lib
    return _lib


def params_from(p) -> OrcParams:
    """Copies the shared fields of an engine gpat_params_t (or a dict)."""
    o = OrcParams()
    get = (lambda k: p[k]) if isinstance(p, dict) else (lambda k: getattr(p, k))
    for name, _ in OrcParams._fields_:
        if name in _MOVER_ARGS:
            continue
        v = get(name)
        if name == "acc_region":
            o.acc_region = (C.c_double * 6)(*tuple(v))
        else:
            setattr(o, name, v)
    return o


def config_from(c) -> OrcMhdConfig:
    o = OrcMhdConfig()
    for name, _ in OrcMhdConfig._fields_:
        setattr(o, name, getattr(c, name))
    return o


class Particles:
    """Oracle particle storage (numpy SoA with spare capacity)."""

    def __init__(self, capacity: int, arrays: dict | None = None):
        self.cap = capacity
        self.a = {k: np.zeros(capacity, dtype=t) for k, t in FIELDS}
        self.n = 0
        if arrays is not None:
            n = len(arrays["x"])
            assert n <= capacity
            for k, _ in FIELDS:
                self.a[k][:n] = arrays[k]
            self.n = n
        self.c = OrcParticles()
        for k, t in FIELDS:
            setattr(self.c, k, self.a[k].ctypes.data_as(P(_CT[t])))

    def view(self) -> dict:
        return {k: v[:self.n].copy() for k, v in self.a.items()}


def full_fields(frame8: np.ndarray, ndim: int, cfg, nonuniform: bool = False) -> np.ndarray:
    """32-variable array with the reference's gradients from an 8-var frame
    (calc_fields_gradients_nonuniform on the positions of set_grid_positions
    when nonuniform)."""
    nzg, nyg, nxg, _ = frame8.shape
    full = np.zeros((nzg, nyg, nxg, 32), dtype=np.float32)
    full[..., :8] = frame8
    lib = load()
    if nonuniform:
        lib.orc_calc_fields_gradients_nonuniform(full.ctypes.data_as(P(C.c_float)), ndim, nxg,
                                                 nyg, nzg)
    else:
        lib.orc_calc_fields_gradients(full.ctypes.data_as(P(C.c_float)), ndim, nxg, nyg, nzg,
                                      cfg.dx, cfg.dy, cfg.dz)
    return full


def set_grid_positions(xpos, ypos=None, zpos=None) -> None:
    """Node positions (ghost nodes included) for spherical and non-uniform
    grids; None clears an axis."""
    keep = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (xpos, ypos, zpos)]
    ptrs = [None if a is None else a.ctypes.data_as(P(d)) for a in keep]
    ns = [0 if a is None else len(a) for a in keep]
    load().orc_set_grid_positions(*ptrs, *ns)


def uniform_grid_positions(n: int, step: float, origin: float) -> np.ndarray:
    """calc_global_grid_positions: step * (j - 2) + origin for j = 0..n-1."""
    out = np.zeros(n, np.float64)
    load().orc_uniform_grid_positions(n, step, origin, out.ctypes.data_as(P(d)))
    return out


_AXES = {"x": 0, "y": 1, "z": 2}


def set_acc_surface(norm1=None, s11=None, s12=None, norm2=None, s21=None, s22=None,
                    intersection=True, shape=(0, 0, 0)) -> None:
    """Acceleration-region surfaces of 3D runs; norm1 = "+y" etc., the
    arrays ghost-padded with the first index fastest (numpy arrays of shape
    (n2, n1)); shape = (nxg, nyg, nzg).  norm1 None turns them off."""
    if norm1 is None:
        load().orc_set_acc_surface(0, 0, 0, 0, 0, 0, None, None, None, None, 0, 0, 0)
        return
    keep = [None if a is None else np.ascontiguousarray(a, np.float64)
            for a in (s11, s12, s21, s22)]
    ptr = [None if a is None else a.ctypes.data_as(P(d)) for a in keep]
    sgn = lambda n: 1 if n[0] == "+" else -1
    n2 = norm2 or norm1
    load().orc_set_acc_surface(_AXES[norm1[1]], sgn(norm1), _AXES[n2[1]], sgn(n2),
                               int(norm2 is not None), int(intersection), *ptr, *shape)


def binary_search(a, v: float) -> int:
    a = np.ascontiguousarray(a, np.float64)
    return load().orc_binary_search(a.ctypes.data_as(P(d)), len(a), v)


def grid_interp_paramters(params: OrcParams, cfg: OrcMhdConfig, x: float, y: float, z: float):
    pos = (i32 * 3)()
    w = (d * 8)()
    load().orc_grid_interp_paramters(C.byref(params), C.byref(cfg), x, y, z, pos, w)
    return list(pos), np.array(list(w))


def aux_fields(db2_slab, db2_2d, lc_slab, lc_2d, ndim: int, cfg,
               nonuniform: bool = False) -> np.ndarray:
    """16-float fluctuation records {db2_slab, db2_2d, lc_slab, lc_2d} x
    {value, d/dx, d/dy, d/dz} from four (nzg, nyg, nxg) arrays (None: the
    reference's initial value 1), gradients as the reference computes them."""
    shape = np.shape(db2_slab if db2_slab is not None else lc_slab)
    aux = np.ones(shape + (16,), dtype=np.float32)
    for g, a in enumerate((db2_slab, db2_2d, lc_slab, lc_2d)):
        if a is not None:
            aux[..., 4 * g] = a
    nzg, nyg, nxg = shape
    if nonuniform:
        load().orc_calc_aux_gradients_nonuniform(aux.ctypes.data_as(P(C.c_float)), ndim, nxg,
                                                 nyg, nzg)
    else:
        load().orc_calc_aux_gradients(aux.ctypes.data_as(P(C.c_float)), ndim, nxg, nyg, nzg,
                                      cfg.dx, cfg.dy, cfg.dz)
    return aux


def philox(ctr, key):
    lib = load()
    c = (u32 * 4)(*ctr)
    k = (u32 * 2)(*key)
    o = (u32 * 4)()
    lib.orc_philox4x32_10(c, k, o)
    return list(o)


def mover(params: OrcParams, cfg: OrcMhdConfig, f1: np.ndarray, parts: Particles, t0: float,
          dtf: float, nsteps_interval: int = 10, num_fine_steps: int = 1, nthreads: int = 0,
          counters: OrcCounters | None = None, f2: np.ndarray | None = None,
          focused_transport: bool = False, nlgc: bool = False,
          kperp_kpara: float = 0.01, aux1: np.ndarray | None = None,
          aux2: np.ndarray | None = None) -> OrcCounters:
    """particle_mover(focused_transport, nlgc, kperp_kpara, ...) on one rank."""
    lib = load()
    params = OrcParams.from_buffer_copy(params)
    params.focused_transport = int(bool(focused_transport))
    params.nlgc = int(bool(nlgc))
    params.kperp_kpara = kperp_kpara
    cnt = counters if counters is not None else OrcCounters()
    fp1 = f1.ctypes.data_as(P(C.c_float))
    fp2 = (f2 if f2 is not None else f1).ctypes.data_as(P(C.c_float))
    a1 = aux1.ctypes.data_as(P(C.c_float)) if aux1 is not None else None
    a2 = aux2.ctypes.data_as(P(C.c_float)) if aux2 is not None else a1
    parts.n = lib.orc_particle_mover(C.byref(params), C.byref(cfg), fp1, fp2, a1, a2,
                                     1 if f2 is not None else 0, C.byref(parts.c), parts.n, t0,
                                     dtf, nsteps_interval, num_fine_steps, nthreads, C.byref(cnt))
    return cnt


def split(params: OrcParams, parts: Particles, split_ratio: float, pmin_split: float,
          counters: OrcCounters) -> None:
    lib = load()
    parts.n = lib.orc_split_particle(C.byref(params), C.byref(parts.c), parts.n, parts.cap,
                                     split_ratio, pmin_split, C.byref(counters))


def histogram(params: OrcParams, parts: Particles):
    lib = load()
    npp = params.npp_global
    counts = np.zeros(npp, np.uint64)
    whi = np.zeros(npp, np.uint64)
    wlo = np.zeros(npp, np.uint64)
    f = np.zeros(npp, np.float64)
    lib.orc_calc_particle_distributions(
        C.byref(params), C.byref(parts.c), parts.n, counts.ctypes.data_as(P(u64)),
        whi.ctypes.data_as(P(u64)), wlo.ctypes.data_as(P(u64)), f.ctypes.data_as(P(d)))
    return f, counts


def inject_at_x(params: OrcParams, cfg: OrcMhdConfig, parts: Particles, nptl: int, xpos: float,
                dt: float, dist_flag: int, particle_v0: float, t_frame: float,
                counters: OrcCounters, power_index: float = 7.0):
    lib = load()
    parts.n = lib.orc_inject_at_x(C.byref(params), C.byref(cfg), C.byref(parts.c), parts.n,
                                  parts.cap, nptl, xpos, dt, dist_flag, particle_v0, t_frame,
                                  power_index, C.byref(counters))


def locate_shock_xpos(full: np.ndarray) -> np.ndarray:
    """Per (y, z) row of a (nzg, nyg, nxg, 32) frame the 1-based x index of
    the largest |dvx/dx|, shaped (nzg, nyg)."""
    nzg, nyg, nxg, _ = full.shape
    S = np.zeros((nzg, nyg), np.int32)
    f = np.ascontiguousarray(full, np.float32)
    load().orc_locate_shock_xpos(f.ctypes.data_as(P(C.c_float)), nxg, nyg, nzg,
                                 S.ctypes.data_as(P(i32)))
    return S


def inject_at_shock(params: OrcParams, cfg: OrcMhdConfig, full: np.ndarray, parts: Particles,
                    nptl: int, dt: float, dist_flag: int, particle_v0: float, t_frame: float,
                    counters: OrcCounters, power_index: float = 7.0):
    S = locate_shock_xpos(full)
    parts.n = load().orc_inject_at_shock(C.byref(params), C.byref(cfg), S.ctypes.data_as(P(i32)),
                                         S.shape[1], S.shape[0], C.byref(parts.c), parts.n,
                                         parts.cap, nptl, dt, dist_flag, particle_v0, t_frame,
                                         power_index, C.byref(counters))


def inject_spatial_uniform(params: OrcParams, parts: Particles, nptl: int, dt: float,
                           dist_flag: int, particle_v0: float, t_frame: float, dt_mhd: float,
                           box, counters: OrcCounters, power_index: float = 7.0):
    lib = load()
    b = (d * 6)(*box)
    parts.n = lib.orc_inject_spatial_uniform(C.byref(params), C.byref(parts.c), parts.n,
                                             parts.cap, nptl, dt, dist_flag, particle_v0,
                                             t_frame, dt_mhd, b, power_index, C.byref(counters))


def count_cells_large(params: OrcParams, cfg: OrcMhdConfig, full: np.ndarray, quantity: int,
                      qmin: float, box, aux: np.ndarray | None = None) -> int:
    """get_ncells_large_* (quantity 0 jz, 1 absj, 2 divv, 3 rho, 4 db2)."""
    ap = aux.ctypes.data_as(P(C.c_float)) if aux is not None else None
    return load().orc_count_cells_large(C.byref(params), C.byref(cfg),
                                        full.ctypes.data_as(P(C.c_float)), ap, quantity, qmin,
                                        (d * 6)(*box))


def inject_at_large(params: OrcParams, cfg: OrcMhdConfig, full: np.ndarray, parts: Particles,
                    nptl: int, dt: float, dist_flag: int, particle_v0: float, t_frame: float,
                    dt_mhd: float, quantity: int, qmin: float, box, counters: OrcCounters,
                    power_index: float = 7.0, aux: np.ndarray | None = None):
    """inject_particles_at_large_* for nptl particles (nptl_inject given)."""
    lib = load()
    ap = aux.ctypes.data_as(P(C.c_float)) if aux is not None else None
    parts.n = lib.orc_inject_at_large(C.byref(params), C.byref(cfg),
                                      full.ctypes.data_as(P(C.c_float)), ap, C.byref(parts.c),
                                      parts.n, parts.cap, nptl, dt, dist_flag, particle_v0,
                                      t_frame, dt_mhd, quantity, qmin, (d * 6)(*box),
                                      power_index, C.byref(counters))


def quick_check(parts: Particles):
    lib = load()
    out = (d * 4)()
    lib.orc_quick_check(C.byref(parts.c), parts.n, out)
    return list(out)


class EscapedHistogram:
    """Attaches an escaped-particle distribution to the oracle's
    remove_particles (npp bins x 6 faces); detach() turns it off."""

    def __init__(self, npp: int, pmin: float, pmax: float):
        self.npp = npp
        self.counts = np.zeros(6 * npp, np.uint64)
        self.whi = np.zeros(6 * npp, np.uint64)
        self.wlo = np.zeros(6 * npp, np.uint64)
        load().orc_set_escaped_histogram(npp, pmin, pmax, self.counts.ctypes.data_as(P(u64)),
                                         self.whi.ctypes.data_as(P(u64)),
                                         self.wlo.ctypes.data_as(P(u64)))

    def detach(self):
        load().orc_set_escaped_histogram(0, 1.0, 2.0, None, None, None)

    def weights(self) -> np.ndarray:
        return np.array([fixed_to_double(int(h), int(l)) for h, l in zip(self.whi, self.wlo)])


class Tracking:
    """init_particle_tracking for the oracle: tags is tags_tracking as
    (nptl_tracking, nrows), one row per tracked particle.  While attached,
    injection, the mover and split_particle record into particles_tracked;
    detach() turns tracking off."""

    def __init__(self, tags, dt_min_rel: float, nsteps_interval: int):
        lib = load()
        self.tags = np.ascontiguousarray(tags, dtype=np.int32)
        self.ntrk, self.nrows = self.tags.shape
        self.nsteps_max = lib.orc_nsteps_tracking_max(dt_min_rel, nsteps_interval)
        self.rec = Particles(self.nsteps_max * self.ntrk)
        lib.orc_set_tracking(self.tags.ctypes.data_as(P(i32)), self.nrows, self.ntrk,
                             self.nsteps_max, C.byref(self.rec.c))

    def dropped(self) -> int:
        return load().orc_tracking_dropped()

    def sync(self) -> dict:
        """sync_tracked_particles, then every field shaped (nptl_tracking,
        nsteps_tracking_max)."""
        load().orc_sync_tracked()
        return {k: v.reshape(self.ntrk, self.nsteps_max).copy() for k, v in self.rec.a.items()}

    def detach(self):
        load().orc_set_tracking(None, 0, 0, 0, None)


class EscapedStore:
    """Attaches a store for the particles remove_particles drops through an
    open boundary (escaped_ptls); detach() turns it off."""

    def __init__(self, capacity: int):
        self.parts = Particles(capacity)
        self.n = C.c_int64(0)
        load().orc_set_escaped_store(C.byref(self.parts.c), capacity, C.byref(self.n))

    def detach(self):
        load().orc_set_escaped_store(None, 0, None)

    def view(self) -> dict:
        return {k: v[:self.n.value].copy() for k, v in self.parts.a.items()}


def local_distribution(cfg: OrcMhdConfig, ndim: int, parts: Particles, pmin: float, pmax: float,
                       npbins: int, nmu: int = 1, rx: int = 1, ry: int = 1, rz: int = 1,
                       spherical: bool = False, nonuniform: bool = False):
    nz = cfg.nz if ndim == 3 else 1
    nb = nmu * npbins * ((cfg.nx + rx - 1) // rx) * ((cfg.ny + ry - 1) // ry) * ((nz + rz - 1) // rz)
    counts = np.zeros(nb, np.uint64)
    whi = np.zeros(nb, np.uint64)
    wlo = np.zeros(nb, np.uint64)
    f = np.zeros(nb, np.float64)
    load().orc_calc_local_distribution(C.byref(cfg), ndim, int(spherical), int(nonuniform),
                                       pmin, pmax, npbins, nmu, rx, ry, rz,
                                       C.byref(parts.c), parts.n, counts.ctypes.data_as(P(u64)),
                                       whi.ctypes.data_as(P(u64)), wlo.ctypes.data_as(P(u64)),
                                       f.ctypes.data_as(P(d)))
    return f, counts


def _unpack(counts, whi, wlo):
    return np.array([fixed_to_double(int(h), int(l)) for h, l in zip(whi, wlo)]), counts


def distribution_mu(params: OrcParams, parts: Particles, nmu: int, by_face: bool = False,
                    nfaces: int = 1):
    """fglobal(nmu, npp_global) (or, by_face, fescaped(nmu, npp, nfaces))
    flattened in Fortran order: (weights, counts)."""
    nb = nmu * params.npp_global * (nfaces if by_face else 1)
    c, h, l = (np.zeros(nb, np.uint64) for _ in range(3))
    load().orc_calc_distribution_mu(C.byref(params), C.byref(parts.c), parts.n, nmu,
                                    int(by_face), nfaces, c.ctypes.data_as(P(u64)),
                                    h.ctypes.data_as(P(u64)), l.ctypes.data_as(P(u64)))
    return _unpack(c, h, l)


def local_escaped_distribution(cfg: OrcMhdConfig, ndim: int, parts: Particles, pmin: float,
                               pmax: float, npbins: int, nmu: int = 1, rx: int = 1, ry: int = 1,
                               rz: int = 1, spherical: bool = False, nonuniform: bool = False):
    """[(weights, counts)] for the x, y and z faces (None beyond ndim), each
    flattened in Fortran order (nmu, npbins, n1, n2, 2)."""
    nz = cfg.nz if ndim == 3 else 1
    nrx, nry, nrz = (cfg.nx + rx - 1) // rx, (cfg.ny + ry - 1) // ry, (nz + rz - 1) // rz
    mp = nmu * npbins
    sizes = [mp * nry * nrz * 2, mp * nrx * nrz * 2, mp * nrx * nry * 2]
    arrs = [[np.zeros(sz, np.uint64) for _ in range(3)] if k < ndim else [None] * 3
            for k, sz in enumerate(sizes)]
    ptrs = [None if a is None else a.ctypes.data_as(P(u64)) for trio in arrs for a in trio]
    load().orc_calc_local_escaped_distribution(C.byref(cfg), ndim, int(spherical),
                                               int(nonuniform), pmin, pmax, npbins, nmu, rx, ry,
                                               rz, C.byref(parts.c), parts.n, *ptrs)
    return [None if trio[0] is None else _unpack(*trio) for trio in arrs]
