"""C ABI and host logic without a GPU: the library loads, exports every
symbol include/gpat_engine.h declares, and its host-only entry points (the
conf.dat and mhd_config readers, argument checks) behave like the
reference's."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from gpat import _abi, fields
from gpat.engine import make_mhd_config, make_params, read_particle_params, load_mhd_config

HEADER = Path(__file__).resolve().parent.parent / "include" / "gpat_engine.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(gpat_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(engine_lib):
    names = declared_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(engine_lib, n), n
    assert set(names) == set(_abi.SIGNATURES), "ctypes table out of sync with the header"
    assert engine_lib.gpat_version().startswith(b"gpat-gb300")


def test_fortran_shim_binds_exported_symbols(engine_lib):
    """Every bind(c, name=...) of the Fortran shim names an exported entry
    point (no Fortran compiler is needed to check the names)."""
    shim = HEADER.parent.parent / "stochastic-parker_gb300" / "fortran" / "gpat_gpu.f90"
    names = re.findall(r'bind\(c,\s*name="(gpat_[a-z0-9_]+)"\)', shim.read_text())
    assert len(names) >= 30
    for n in names:
        assert hasattr(engine_lib, n), n


def test_header_compiles_as_c(tmp_path):
    """include/gpat_engine.h is plain C99: no C++ or torch types."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "hdr.c"
    src.write_text('#include "gpat_engine.h"\n'
                   "int main(void) { gpat_params_t p; gpat_particles_t s; gpat_counters_t c;\n"
                   "  gpat_local_dist_t l; (void)p; (void)s; (void)c; (void)l; return GPAT_OK; }\n")
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                        "-I", str(HEADER.parent), "-c", str(src), "-o", str(tmp_path / "hdr.o")],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr


def test_struct_layouts_match_header():
    # gpat_mhd_config_t: 13 doubles + 13 int32 (+4 bytes tail padding)
    assert C.sizeof(_abi.MhdConfig) == 160
    assert _abi.MhdConfig.bcz.offset == 152
    assert C.sizeof(_abi.Particles) == 17 * C.sizeof(C.c_void_p)


CONF = """!< Configuration file written for the tests
!< Initial magnetic field strength
b0 = 2.0
!< momentum normalisation
p0 = 0.1
pmin = 1.0E-2
pmax = 1.0d1
momentum_dependency = 1
!< turbulence spectral index
gamma_turb = 1.6666667
mag_dependency = 0
kpara0 = 0.01 ; trailing C-style terminator
kret = 0.03
dt_min = 1E-8
dt_min_rel = 1E-7
dt_max_rel = 1E-2
npp_global = 96
nmu_global = 32
acc_region_flag = 1
acc_xmin = -1.0
acc_xmax = -0.5
acc_ymin = 0.08
acc_ymax = 1.0
acc_zmin = 0.0
acc_zmax = 1.0
pbcx = 1
pbcy = 0
pbcz = 0
"""


def test_read_particle_params_reference_order(tmp_path, engine_lib):
    f = tmp_path / "conf.dat"
    f.write_text(CONF)
    p = read_particle_params(f)
    assert (p.b0, p.p0, p.pmin, p.pmax) == (2.0, 0.1, 0.01, 10.0)
    assert p.momentum_dependency == 1 and p.mag_dependency == 0
    assert p.gamma_turb == 1.6666667 and p.pindex == pytest.approx(3.0 - 1.6666667)
    assert p.kpara0 == 0.01 and p.kret == 0.03
    # 'dt_min' line does not match 'dt_min_rel' (substring search is by key)
    assert p.dt_min_rel == 1e-7 and p.dt_max_rel == 1e-2
    assert p.acc_region_flag == 1
    assert tuple(p.acc_region) == (-1.0, -0.5, 0.08, 1.0, 0.0, 1.0)
    assert (p.pbcx, p.pbcy, p.pbcz) == (1, 0, 0)
    assert p.npp_global == 96


def test_read_particle_params_forward_scan_and_missing(tmp_path, engine_lib):
    # gamma_turb appears before momentum_dependency: the forward scan from
    # the momentum_dependency match never sees it and reads -1 (as
    # read_config.f90:20-44 does); the sample config/conf.dat has no
    # gamma_turb key at all, which gives the same -1.
    text = CONF.replace("gamma_turb = 1.6666667\n", "")
    text = text.replace("pmax = 1.0d1\n", "pmax = 1.0d1\ngamma_turb = 1.5\n")
    f = tmp_path / "conf.dat"
    f.write_text(text)
    p = read_particle_params(f)
    assert p.gamma_turb == -1.0 and p.pindex == 4.0
    # A key missing at the end leaves the scan at EOF: everything after it
    # reads -1 too.
    f2 = tmp_path / "conf2.dat"
    f2.write_text(CONF.split("kret")[0])
    p2 = read_particle_params(f2)
    assert p2.kpara0 == 0.01 and p2.kret == -1.0 and p2.dt_min_rel == -1.0
    assert p2.acc_region_flag == -1   # not 1: default acc region kept
    assert tuple(p2.acc_region) == (0.0, 1.0, 0.0, 1.0, 0.0, 1.0)


def test_get_variable_single_key(tmp_path, engine_lib):
    f = tmp_path / "conf.dat"
    f.write_text(CONF)
    v = C.c_double()
    assert engine_lib.gpat_get_variable(str(f).encode(), b"nmu_global", C.byref(v)) == 0
    assert v.value == 32.0
    assert engine_lib.gpat_get_variable(str(f).encode(), b"no_such_key", C.byref(v)) == 0
    assert v.value == -1.0
    assert engine_lib.gpat_get_variable(b"/nonexistent/conf.dat", b"b0", C.byref(v)) == \
        _abi.GPAT_ERR_IO


def test_mhd_config_file_roundtrip(tmp_path, engine_lib):
    cfg = make_mhd_config(512, 64, 1, 0.0, 1.0, 0.0, 0.125, dt_out=0.1)
    cfg.bcx, cfg.bcy, cfg.bcz = 1, 0, 0
    path = tmp_path / "mhd_config.dat"
    fields.write_mhd_config(path, cfg)
    assert path.stat().st_size == 156
    got = load_mhd_config(path)
    for name, _ in _abi.MhdConfig._fields_:
        assert getattr(got, name) == getattr(cfg, name), name


def test_create_rejects_out_of_scope_options(engine_lib):
    cfg = make_mhd_config(16, 16, 1, 0.0, 1.0, 0.0, 1.0)
    h = _abi.Handle()
    for kw, code in ((dict(ndim=4), _abi.GPAT_ERR_UNSUPPORTED),
                     (dict(ndim=1, precision=1), _abi.GPAT_ERR_UNSUPPORTED),
                     (dict(dpp_wave=1, precision=1), _abi.GPAT_ERR_UNSUPPORTED),
                     (dict(dpp_shear=1, precision=1), _abi.GPAT_ERR_UNSUPPORTED),
                     (dict(deltab_flag=1, precision=1), _abi.GPAT_ERR_UNSUPPORTED),
                     (dict(correlation_flag=1, precision=1), _abi.GPAT_ERR_UNSUPPORTED),
                     (dict(include_3rd_dim=1, precision=1), _abi.GPAT_ERR_UNSUPPORTED),
                     (dict(include_3rd_dim=1, ndim=3, precision=0), _abi.GPAT_ERR_ARG),
                     (dict(spherical_coord=1, precision=1), _abi.GPAT_ERR_UNSUPPORTED),
                     (dict(nonuniform_grid=1, precision=1), _abi.GPAT_ERR_UNSUPPORTED),
                     (dict(precision=7), _abi.GPAT_ERR_ARG),
                     (dict(nptl_max=0), _abi.GPAT_ERR_ARG),
                     (dict(npp_global=0), _abi.GPAT_ERR_ARG)):
        p = make_params(**kw)
        assert engine_lib.gpat_create(C.byref(p), C.byref(cfg), 0, C.byref(h)) == code, kw
    assert engine_lib.gpat_create(None, None, 0, C.byref(h)) == _abi.GPAT_ERR_ARG


def test_frames_have_reference_layout():
    frame = fields.planar_shock_2d(32, 8, 0.0, 1.0, 0.0, 0.25, r=4.0, w=0.01)
    assert frame.shape == (1, 12, 36, 8) and frame.dtype == np.float32
    # node i (C index) sits at x = xmin + (i - 2) dx: upstream/downstream
    vx = frame[0, 0, :, 0]
    assert vx[0] == pytest.approx(1.0) and vx[-1] == pytest.approx(0.25, rel=1e-6)
    assert np.all(frame[..., 7] == np.sqrt(frame[..., 4].astype(np.float64) ** 2).astype(np.float32))


# --- Fortran bind(c) interfaces against the C prototypes -------------------
# Each dummy argument of a bind(c) interface in the shim is reduced to the C
# type it passes (value or reference, element type), and so is each parameter
# of the header's prototype; the two lists must agree.  An int passed where
# the header takes int64_t, a missing `value`, or a dropped argument fails
# here without a Fortran compiler.

_F_KIND = {"c_int": "i32", "c_int32_t": "i32", "c_int64_t": "i64", "c_int8_t": "i8",
           "c_double": "f64", "c_float": "f32", "c_char": "char"}


def _fortran_interfaces(text):
    out = {}
    blocks = re.findall(
        r'^\s*(?:(integer\(c_int\)|type\(c_ptr\))\s+function|subroutine)\s+(\w+)\s*\(([^)]*)\)'
        r'[\s&]*bind\(c,\s*name="(gpat_\w+)"\)(.*?)^\s*end\s+(?:function|subroutine)',
        text, flags=re.M | re.S | re.I)
    for result, _, args, cname, body in blocks:
        names = [a.strip().lower() for a in args.replace("&", " ").split(",") if a.strip()]
        decl = {}
        for line in body.splitlines():
            if "::" not in line or line.strip().lower().startswith("import"):
                continue
            spec, vars_ = line.split("::", 1)
            spec = spec.strip().lower()
            for v in vars_.split(","):
                decl[v.strip().lower().split("(")[0]] = spec
        kinds = []
        for n in names:
            spec = decl[n]
            by_value = "value" in spec
            m = re.match(r"(integer|real|character|type)\((?:kind=)?(\w+)\)", spec)
            base = m.group(2)
            if m.group(1) == "type":
                k = "ptr" if base == "c_ptr" else base
            else:
                k = _F_KIND[base]
            kinds.append(k if by_value else k + "*")
        ret = {"integer(c_int)": "i32", "type(c_ptr)": "ptr"}.get(result.lower(), "void")
        out[cname] = (ret, kinds)
    return out


_C_BASE = {"int": "i32", "int32_t": "i32", "int64_t": "i64", "uint64_t": "i64",
           "int8_t": "i8", "double": "f64", "float": "f32", "char": "char", "void": "void"}


def _c_kind(decl):
    d = decl.replace("const", " ").strip()
    stars = d.count("*") + d.count("[")      # an array parameter is a pointer
    words = d.replace("*", " ").split()
    base = words[0]
    if base in ("gpat_handle_t", "gpat_batch_t", "gpat_mlp_t") or (base == "void" and stars):
        k, stars = "ptr", stars - 1          # opaque handles and void * travel as c_ptr
    else:
        k = _C_BASE.get(base, base)
    return k + "*" * stars


def _c_prototypes(text):
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    out = {}
    for ret, name, args in re.findall(r"([\w\s\*]+?)\b(gpat_\w+)\s*\(([^;{]*?)\)\s*;", text):
        params = [a.strip() for a in args.split(",") if a.strip() and a.strip() != "void"]
        out[name] = (_c_kind(ret.strip().split("\n")[-1]), [_c_kind(p) for p in params])
    return out


def _same_kind(f, c):
    if f == c:
        return True
    # a c_ptr by value stands for any single pointer (e.g. an optional
    # file name or a device array)
    return f == "ptr" and c.endswith("*") and c.count("*") == 1


def test_fortran_interfaces_match_c_prototypes():
    shim = HEADER.parent.parent / "stochastic-parker_gb300" / "fortran" / "gpat_gpu.f90"
    fort = _fortran_interfaces(shim.read_text())
    cproto = _c_prototypes(HEADER.read_text())
    bound = set(re.findall(r'bind\(c,\s*name="(gpat_\w+)"\)', shim.read_text()))
    assert set(fort) == bound, bound - set(fort)
    for name, (fret, fargs) in sorted(fort.items()):
        assert name in cproto, name
        cret, cargs = cproto[name]
        assert len(fargs) == len(cargs), (name, fargs, cargs)
        for i, (f, c) in enumerate(zip(fargs, cargs)):
            assert _same_kind(f, c), (name, i, f, c)
        if fret == "ptr":
            assert cret.endswith("*"), (name, cret)
        else:
            assert fret == cret, (name, fret, cret)


def test_fortran_interface_check_catches_a_mismatch():
    """The check above fails on an int count where the header has int64_t."""
    shim = HEADER.parent.parent / "stochastic-parker_gb300" / "fortran" / "gpat_gpu.f90"
    text = shim.read_text()
    fort = _fortran_interfaces(text)
    name = next(n for n, (_, a) in fort.items() if "i64" in a)
    i = fort[name][1].index("i64")
    cargs = _c_prototypes(HEADER.read_text())[name][1]
    assert cargs[i] == "i64"
    assert not _same_kind("i32", cargs[i])


def _py_kind(t):
    """The kind of a ctypes argument type, in the notation of _c_kind."""
    if t is C.c_void_p:
        return "ptr"
    if t is C.c_char_p:
        return "char*"
    scalars = {C.c_int: "i32", C.c_int32: "i32", C.c_int64: "i64", C.c_uint64: "i64",
               C.c_int8: "i8", C.c_uint32: "u32", C.c_double: "f64", C.c_float: "f32",
               C.c_char: "char"}
    for k, v in scalars.items():
        if t is k:
            return v
    if isinstance(t, type) and issubclass(t, C._Pointer):
        return _py_kind(t._type_) + "*"
    if isinstance(t, type) and issubclass(t, C.Structure):
        return "struct"
    raise AssertionError(f"unmapped ctypes type {t}")


def _py_matches_c(p, c):
    if p == c:
        return True
    c = c.replace("uint32_t", "u32").replace("uint8_t", "i8")
    if p == c:
        return True
    # a structure pointer stands for the header's gpat_*_t pointer of the
    # same depth; an opaque handle pointer for void *
    if p.startswith("struct") and c.startswith("gpat_"):
        return p.count("*") == c.count("*")
    return p == "ptr" and c.endswith("*") and c.count("*") == 1


def _binding_mismatches(signatures):
    cproto = _c_prototypes(HEADER.read_text())
    bad = sorted(set(signatures) ^ set(cproto))
    for name, (_, args) in sorted(signatures.items()):
        if name not in cproto:
            continue
        cargs = cproto[name][1]
        if len(args) != len(cargs):
            bad.append((name, len(args), len(cargs)))
            continue
        for i, (t, c) in enumerate(zip(args, cargs)):
            if not _py_matches_c(_py_kind(t), c):
                bad.append((name, i, _py_kind(t), c))
    return bad


def test_python_bindings_match_c_prototypes():
    """Every ctypes declaration in gpat/_abi.py has the header prototype's
    argument count, scalar types and pointer depths, so a changed signature
    cannot go unnoticed by the Python callers."""
    assert _binding_mismatches(_abi.SIGNATURES) == []


def test_python_binding_check_catches_a_mismatch():
    """Dropping an argument or narrowing an int64_t to int fails the check."""
    sigs = dict(_abi.SIGNATURES)
    res, args = sigs["gpat_weighted_split"]
    sigs["gpat_weighted_split"] = (res, args[:5] + args[6:])          # no z_floor
    res, args = sigs["gpat_put_particles"]
    sigs["gpat_put_particles"] = (res, args[:2] + [C.c_int])           # int64_t n as int
    bad = _binding_mismatches(sigs)
    assert any(b[0] == "gpat_weighted_split" for b in bad)
    assert any(b[0] == "gpat_put_particles" for b in bad)
