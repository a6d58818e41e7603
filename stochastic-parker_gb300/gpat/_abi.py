"""ctypes declarations of the engine's C ABI (include/gpat_engine.h)."""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

from . import build as _build

GPAT_OK = 0
GPAT_ERR_ARG = -1
GPAT_ERR_OOM = -2
GPAT_ERR_CAPACITY = -3
GPAT_ERR_TIMEOUT = -4
GPAT_ERR_CUDA = -5
GPAT_ERR_UNSUPPORTED = -6
GPAT_ERR_IO = -7
GPAT_ERR_STATE = -8
GPAT_ERR_DEVICE = -9

ERROR_NAMES = {
    GPAT_ERR_ARG: "GPAT_ERR_ARG", GPAT_ERR_OOM: "GPAT_ERR_OOM",
    GPAT_ERR_CAPACITY: "GPAT_ERR_CAPACITY", GPAT_ERR_TIMEOUT: "GPAT_ERR_TIMEOUT",
    GPAT_ERR_CUDA: "GPAT_ERR_CUDA", GPAT_ERR_UNSUPPORTED: "GPAT_ERR_UNSUPPORTED",
    GPAT_ERR_IO: "GPAT_ERR_IO", GPAT_ERR_STATE: "GPAT_ERR_STATE",
    GPAT_ERR_DEVICE: "GPAT_ERR_DEVICE",
}

LARGE_JZ, LARGE_ABSJ, LARGE_DIVV, LARGE_RHO, LARGE_DB2 = 0, 1, 2, 3, 4
PREC_FP64 = 0
PREC_MIXED = 1
NOISE_UNIFORM = 0
NOISE_GAUSS = 1

d, i32, i64, u32, u64 = C.c_double, C.c_int32, C.c_int64, C.c_uint32, C.c_uint64
P = C.POINTER


class MhdConfig(C.Structure):
    """mhd_configuration (mhd_config.f90:16-27): 13 doubles, 13 int32."""
    _fields_ = [(n, d) for n in ("dx", "dy", "dz", "xmin", "ymin", "zmin", "xmax", "ymax", "zmax",
                                 "lx", "ly", "lz", "dt_out")] + \
               [(n, i32) for n in ("nx", "ny", "nz", "nxs", "nys", "nzs", "topox", "topoy", "topoz",
                                   "nvar", "bcx", "bcy", "bcz")]


class Params(C.Structure):
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
        ("noise", i32), ("precision", i32),
        ("nptl_max", i64),
        ("time_interp", i32),
        ("dpp_wave", i32), ("dpp_shear", i32), ("deltab_flag", i32), ("correlation_flag", i32),
        ("include_3rd_dim", i32), ("spherical_coord", i32), ("nonuniform_grid", i32),
        ("bin_interval", i32), ("weak_scattering", i32),
        ("duu0", d), ("tau0", d),
    ]


PARTICLE_FIELDS = [
    ("x", "f8"), ("y", "f8"), ("z", "f8"), ("p", "f8"), ("v", "f8"), ("mu", "f8"),
    ("weight", "f8"), ("t", "f8"), ("dt", "f8"),
    ("split_times", "i1"), ("count_flag", "i1"),
    ("origin", "i4"), ("nsteps_tracked", "i4"), ("nsteps_pushed", "i4"),
    ("tag_injected", "i4"), ("tag_splitted", "i4"),
    ("rng_ctr", "u4"),
]
_CT = {"f8": C.c_double, "i1": C.c_int8, "i4": C.c_int32, "u4": C.c_uint32}


class Particles(C.Structure):
    """particle_type as structure-of-arrays (gpat_particles_t)."""
    _fields_ = [(n, P(_CT[t])) for n, t in PARTICLE_FIELDS]


class LocalDist(C.Structure):
    """gpat_local_dist_t: one set of local distribution parameters."""
    _fields_ = [("pmin", d), ("pmax", d), ("npbins", i32), ("nmu", i32), ("rx", i32),
                ("ry", i32), ("rz", i32), ("reserved", i32)]


class Counters(C.Structure):
    _fields_ = [
        ("nptl_current", i64), ("nptl_split", i64), ("nptl_escaped", i64), ("tag_max", i64),
        ("leak", d), ("leak_negp", d),
        ("leak_hi", u64), ("leak_lo", u64), ("leak_negp_hi", u64), ("leak_negp_lo", u64),
        ("steps", u64),
        ("last_mover_ms", d), ("last_mover_steps", u64), ("last_mover_launches", i64),
    ]


Handle = C.c_void_p
Batch = C.c_void_p
Mlp = C.c_void_p
MLP_FEATURES = 8
MLP_PARAMS = 8961


class BatchTuning(C.Structure):
    _fields_ = [("minb", i32), ("grab", i32), ("pushes_per_s", d), ("chunk_pushes", i32),
                ("reserved", i32), ("default_pushes_per_s", d)]


# name -> (restype, argtypes); every symbol include/gpat_engine.h declares.
SIGNATURES = {
    "gpat_version": (C.c_char_p, []),
    "gpat_read_particle_params": (C.c_int, [C.c_char_p, P(Params)]),
    "gpat_get_variable": (C.c_int, [C.c_char_p, C.c_char_p, P(d)]),
    "gpat_load_mhd_config": (C.c_int, [C.c_char_p, P(MhdConfig)]),
    "gpat_create": (C.c_int, [P(Params), P(MhdConfig), C.c_int, P(Handle)]),
    "gpat_destroy": (C.c_int, [Handle]),
    "gpat_last_error": (C.c_char_p, [Handle]),
    "gpat_set_tstamps": (C.c_int, [Handle, P(d), C.c_int]),
    "gpat_calc_tstamps_mhd": (C.c_int, [Handle, C.c_int, C.c_int]),
    "gpat_set_fields": (C.c_int, [Handle, C.c_int, P(C.c_float), C.c_int]),
    "gpat_read_field_data": (C.c_int, [Handle, C.c_char_p, C.c_int]),
    "gpat_calc_fields_gradients": (C.c_int, [Handle, C.c_int]),
    "gpat_copy_fields": (C.c_int, [Handle]),
    "gpat_get_fields": (C.c_int, [Handle, C.c_int, P(C.c_float)]),
    "gpat_inject_particles_spatial_uniform": (
        C.c_int, [Handle, i64, d, C.c_int, d, C.c_int, P(d), d]),
    "gpat_inject_particles_at_x": (C.c_int, [Handle, i64, d, d, C.c_int, d, C.c_int, d]),
    "gpat_batch_create": (C.c_int, [P(Handle), C.c_int, P(Batch)]),
    "gpat_batch_destroy": (C.c_int, [Batch]),
    "gpat_batch_last_error": (C.c_char_p, [Batch]),
    "gpat_batch_particle_mover": (C.c_int, [Batch, P(C.c_int), C.c_int, d, C.c_int, C.c_int]),
    "gpat_batch_autotune": (C.c_int, [Batch, P(C.c_int), C.c_int, d, C.c_int, C.c_int,
                                      P(BatchTuning)]),
    "gpat_batch_get_tuning": (C.c_int, [Batch, P(BatchTuning)]),
    "gpat_batch_set_tuning": (C.c_int, [Batch, P(BatchTuning)]),
    "gpat_batch_stats": (C.c_int, [Batch, P(d), P(u64), P(i64)]),
    "gpat_mlp_create": (C.c_int, [C.c_int, u64, i64, P(Mlp)]),
    "gpat_mlp_destroy": (C.c_int, [Mlp]),
    "gpat_mlp_last_error": (C.c_char_p, [Mlp]),
    "gpat_mlp_set_params": (C.c_int, [Mlp, P(C.c_float), P(C.c_float)]),
    "gpat_mlp_get_params": (C.c_int, [Mlp, P(C.c_float), P(C.c_float)]),
    "gpat_mlp_forward": (C.c_int, [Mlp, P(C.c_float), i64, P(C.c_float)]),
    "gpat_mlp_loss_grad": (C.c_int, [Mlp, P(C.c_float), P(C.c_float), i64, P(C.c_float),
                                     P(C.c_float)]),
    "gpat_mlp_clear_records": (C.c_int, [Mlp]),
    "gpat_mlp_set_records": (C.c_int, [Mlp, P(C.c_float), P(C.c_float), i64]),
    "gpat_mlp_record": (C.c_int, [Mlp, Handle, d, P(i64)]),
    "gpat_mlp_label": (C.c_int, [Mlp, Handle, d, P(i64), P(i64)]),
    "gpat_mlp_train": (C.c_int, [Mlp, C.c_int, i64, d, d, u64, P(d)]),
    "gpat_mlp_score": (C.c_int, [Mlp, Handle, d, P(d), P(d), P(d)]),
    "gpat_weighted_split": (C.c_int, [Handle, Mlp, d, d, d, d, d, C.c_int, P(i64), P(i64)]),
    "gpat_tail_weights": (C.c_int, [Handle, d, P(i64), P(d), P(d)]),
    "gpat_set_fluctuations": (C.c_int, [Handle, C.c_int, P(C.c_float), P(C.c_float),
                                        P(C.c_float), P(C.c_float)]),
    "gpat_read_magnetic_fluctuation": (C.c_int, [Handle, C.c_char_p, C.c_int]),
    "gpat_read_correlation_length": (C.c_int, [Handle, C.c_char_p, C.c_int]),
    "gpat_get_fluctuations": (C.c_int, [Handle, C.c_int, P(C.c_float)]),
    "gpat_set_grid_positions": (C.c_int, [Handle, P(C.c_double), P(C.c_double), P(C.c_double)]),
    "gpat_read_grid_positions": (C.c_int, [Handle, C.c_char_p]),
    "gpat_get_grid_positions": (C.c_int, [Handle, P(C.c_double), P(C.c_double), P(C.c_double)]),
    "gpat_init_acc_surface": (C.c_int, [Handle, C.c_char_p, C.c_char_p, C.c_int]),
    "gpat_get_escaped_particles": (C.c_int, [Handle, P(Particles), C.c_int64, P(C.c_int64)]),
    "gpat_set_acc_surface": (C.c_int, [Handle, C.c_int, P(C.c_double), P(C.c_double)]),
    "gpat_read_acc_surface": (C.c_int, [Handle, C.c_int, C.c_char_p, C.c_char_p]),
    "gpat_count_cells_large": (C.c_int, [Handle, C.c_int, d, P(d), P(i64)]),
    "gpat_inject_particles_at_large": (C.c_int, [Handle, C.c_int, i64, d, C.c_int, d, C.c_int,
                                                 C.c_int, d, i64, P(d), d, P(i64)]),
    "gpat_put_particles": (C.c_int, [Handle, P(Particles), i64]),
    "gpat_get_particles": (C.c_int, [Handle, P(Particles), i64, P(i64)]),
    "gpat_particle_mover": (C.c_int, [Handle, C.c_int, C.c_int, d, C.c_int, C.c_int, C.c_int,
                                      C.c_int]),
    "gpat_split_particle": (C.c_int, [Handle, d, d, C.c_int]),
    "gpat_set_mover_learned": (C.c_int, [Handle, C.c_void_p, d, d, d, d, d, C.c_int]),
    "gpat_get_mover_learned": (C.c_int, [Handle, C.POINTER(d), C.POINTER(d), C.POINTER(C.c_int64),
                                         C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "gpat_set_mover_tiles": (C.c_int, [Handle] + [C.c_int] * 8),
    "gpat_get_mover_tiles": (C.c_int, [Handle, C.POINTER(C.c_int)]),
    "gpat_split_particle_noalloc": (C.c_int, [P(Particles), i64, i64, d, d, d, d, C.c_void_p,
                                              P(i64), P(i64)]),
    "gpat_calc_particle_distributions": (C.c_int, [Handle, P(d), P(u64)]),
    "gpat_local_distribution_dims": (C.c_int, [Handle, P(LocalDist), P(i32)]),
    "gpat_calc_local_distribution": (C.c_int, [Handle, P(LocalDist), P(d), P(u64)]),
    "gpat_calc_escaped_distributions": (C.c_int, [Handle, P(d), P(u64)]),
    "gpat_reset_escaped_particles": (C.c_int, [Handle]),
    "gpat_init_particle_tracking": (C.c_int, [Handle, P(C.c_int32), C.c_int32, C.c_int32,
                                              C.c_int32]),
    "gpat_read_particle_tracking": (C.c_int, [Handle, C.c_char_p, C.c_int32]),
    "gpat_tracking_dims": (C.c_int, [Handle, P(C.c_int64), P(C.c_int32), P(C.c_int64)]),
    "gpat_get_tracked_particles": (C.c_int, [Handle, P(Particles)]),
    "gpat_free_particle_tracking": (C.c_int, [Handle]),
    "gpat_load_tstamps_mhd": (C.c_int, [Handle, C.c_int, C.c_int, C.c_int, C.c_char_p]),
    "gpat_get_pmax_global": (C.c_int, [Handle, P(C.c_double)]),
    "gpat_locate_shock_xpos": (C.c_int, [Handle, P(C.c_int32)]),
    "gpat_inject_particles_at_shock": (C.c_int, [Handle, C.c_int64, C.c_double, C.c_int,
                                                 C.c_double, C.c_int, C.c_double]),
    "gpat_calc_particle_distributions_mu": (C.c_int, [Handle, C.c_int32, P(C.c_double),
                                                      P(C.c_uint64)]),
    "gpat_calc_escaped_distributions_mu": (C.c_int, [Handle, C.c_int32, P(C.c_double),
                                                     P(C.c_uint64)]),
    "gpat_calc_local_escaped_distribution": (C.c_int, [Handle, P(LocalDist)] +
                                             [P(C.c_double)] * 3 + [P(C.c_uint64)] * 3),
    "gpat_pbins_edges": (C.c_int, [Handle, P(d)]),
    "gpat_quick_check": (C.c_int, [Handle, P(d)]),
    "gpat_get_counters": (C.c_int, [Handle, P(Counters)]),
    "gpat_set_counters": (C.c_int, [Handle, P(Counters)]),
    "gpat_stream": (C.c_void_p, [Handle]),
}

_lib = None


def lib_path() -> Path:
    return _build.LIB_PATH


def load(path: str | Path | None = None) -> C.CDLL:
    """Loads the engine library; raises if it has not been built.

    The first load without a path fixes the process-wide library; the
    GPAT_ENGINE_LIB environment variable points it at another build."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    env = os.environ.get("GPAT_ENGINE_LIB")
    p = Path(path) if path else (Path(env) if env else lib_path())
    if not p.exists():
        raise RuntimeError(
            f"GPAT engine library not found at {p}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib
