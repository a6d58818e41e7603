"""gpat_split_particle_noalloc: the split for callers that cannot allocate
device memory (their particle arrays live in device memory they manage, and
they may not call cudaMalloc in the time loop).  The caller passes its own
device arrays; the entry point allocates nothing.  Its output must equal the
handle-based gpat_split_particle's, particle for particle, on two calls in a
row (the second call reuses the fixed scratch the first one left behind).

This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from gpat import _abi
from gpat.engine import Engine, make_mhd_config, make_params

pytestmark = pytest.mark.gpu

TORCH_DTYPES = {"f8": "float64", "i1": "int8", "i4": "int32", "u4": "int32"}


def _device_arrays(torch, ps, capacity):
    """The caller's own device arrays (allocated here, by the test)."""
    out = {}
    for name, t in _abi.PARTICLE_FIELDS:
        a = np.ascontiguousarray(ps.arrays[name])
        if t == "u4":
            a = a.view(np.int32)
        buf = torch.zeros(capacity, dtype=getattr(torch, TORCH_DTYPES[t]), device="cuda")
        buf[:len(a)] = torch.from_numpy(a).to("cuda")
        out[name] = buf
    return out


def _as_struct(arrays):
    s = _abi.Particles()
    for name, t in _abi.PARTICLE_FIELDS:
        setattr(s, name, C.cast(C.c_void_p(arrays[name].data_ptr()), C.POINTER(_abi._CT[t])))
    return s


def _to_host(arrays, n):
    out = {}
    for name, t in _abi.PARTICLE_FIELDS:
        a = arrays[name][:n].cpu().numpy()
        out[name] = a.view(np.uint32) if t == "u4" else a
    return out


def test_split_noalloc_matches_split_particle_twice():
    torch = pytest.importorskip("torch")
    lib = _abi.load()
    cap = 20000
    p0, pmax, ratio, pmin_split = 0.1, 100.0, 2.72, 2.0
    cfg = make_mhd_config(32, 32, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.02)
    eng = Engine(make_params(p0=p0, pmin=p0, pmax=pmax, nptl_max=cap, ndim=2), cfg, 0)
    eng.set_tstamps([0.0, 0.02])
    eng.inject_particles_at_x(6000, 0.5, 1e-6, 1, 1.0, 1)
    start = eng.get_particles()
    rng = np.random.default_rng(1234)
    start.arrays["p"][:] = p0 * np.exp(rng.uniform(0.0, 3.0, len(start)))
    eng.put_particles(start)

    dev = _device_arrays(torch, start, cap)
    st = _as_struct(dev)
    n = len(start)
    for call in range(2):
        eng.split_particle(ratio, pmin_split, 10)
        ref = eng.get_particles()
        torch.cuda.synchronize()
        n_out, n_split = C.c_int64(), C.c_int64()
        rc = lib.gpat_split_particle_noalloc(C.byref(st), n, cap, ratio, pmin_split, p0, pmax,
                                             None, C.byref(n_out), C.byref(n_split))
        assert rc == _abi.GPAT_OK, (call, rc)
        assert n_out.value == len(ref) and n_split.value == len(ref) - n > 0
        got = _to_host(dev, n_out.value)
        for name, _ in _abi.PARTICLE_FIELDS:
            assert np.array_equal(got[name], ref.arrays[name]), (call, name)
        n = n_out.value
    eng.close()


def test_split_noalloc_warm_up_call():
    """The n = 0 call a driver makes on each device before its time loop (it
    loads the device code and looks up the scratch) returns GPAT_OK."""
    torch = pytest.importorskip("torch")
    lib = _abi.load()
    dev = {name: torch.zeros(16, dtype=getattr(torch, TORCH_DTYPES[t]), device="cuda")
           for name, t in _abi.PARTICLE_FIELDS}
    st = _as_struct(dev)
    n_out, n_split = C.c_int64(-1), C.c_int64(-1)
    rc = lib.gpat_split_particle_noalloc(C.byref(st), 0, 16, 2.72, 2.0, 0.1, 100.0, None,
                                         C.byref(n_out), C.byref(n_split))
    assert rc == _abi.GPAT_OK and n_out.value == 0 and n_split.value == 0


def test_split_noalloc_capacity_like_split_particle():
    """capacity below n + candidates: GPAT_ERR_CAPACITY, n_out = capacity, and
    the same particles as gpat_split_particle on a handle with that nptl_max."""
    torch = pytest.importorskip("torch")
    from gpat.engine import GPATError
    lib = _abi.load()
    p0, pmax, ratio, pmin_split = 0.1, 100.0, 2.72, 2.0
    n0, cap = 3000, 4000
    cfg = make_mhd_config(32, 32, 1, 0.0, 1.0, 0.0, 1.0, dt_out=0.02)
    eng = Engine(make_params(p0=p0, pmin=p0, pmax=pmax, nptl_max=cap, ndim=2), cfg, 0)
    eng.set_tstamps([0.0, 0.02])
    eng.inject_particles_at_x(n0, 0.5, 1e-6, 1, 1.0, 1)
    start = eng.get_particles()
    start.arrays["p"][:] = p0 * np.exp(np.random.default_rng(99).uniform(0.0, 3.0, n0))
    eng.put_particles(start)
    # split_times is 0 after injection: candidates have p > pmin_split p0
    wanted = int(np.sum(start.arrays["p"] > pmin_split * p0))
    assert n0 + wanted > cap
    with pytest.raises(GPATError):
        eng.split_particle(ratio, pmin_split, 10)
    ref = eng.get_particles()
    assert len(ref) == cap
    dev = _device_arrays(torch, start, cap)
    st = _as_struct(dev)
    torch.cuda.synchronize()
    n_out, n_split = C.c_int64(), C.c_int64()
    rc = lib.gpat_split_particle_noalloc(C.byref(st), n0, cap, ratio, pmin_split, p0, pmax, None,
                                         C.byref(n_out), C.byref(n_split))
    assert rc == _abi.GPAT_ERR_CAPACITY and n_out.value == cap and n_split.value == cap - n0
    got = _to_host(dev, cap)
    for name, _ in _abi.PARTICLE_FIELDS:
        assert np.array_equal(got[name], ref.arrays[name]), name
    eng.close()


def test_split_noalloc_rejects_sizes_beyond_its_scratch():
    lib = _abi.load()
    st = _abi.Particles()
    n_out = C.c_int64()
    too_many = (1 << 26) + 1
    assert lib.gpat_split_particle_noalloc(C.byref(st), too_many, too_many, 2.0, 2.0, 0.1, 10.0,
                                           None, C.byref(n_out), None) == _abi.GPAT_ERR_ARG
