"""Builds the engine's shared library (CUDA kernels + C ABI) for sm_103a.

The library is compiled in-tree into ``gpat/_lib/libgpat_engine.so`` with
nvcc, one translation unit per process, then linked.  ``mover_fp64.cu`` and
``particles.cu`` are compiled with ``-fmad=false`` so the FP64 mover and the
injection keep the reference's separately rounded operations; the
split-precision mover contracts freely to FMA.  Host code is compiled with
``-ffp-contract=off``: on Arm hosts the compiler would otherwise fuse the
box and grid arithmetic (xmin + nx * dx, ...) into FMAs and the bounds the
kernels receive would differ in the last bit from an x86 build.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
PROJECT_DIR = PKG_DIR.parent                  # stochastic-parker_gb300/
REPO_DIR = PROJECT_DIR.parent
CSRC = PROJECT_DIR / "csrc"
INCLUDE = REPO_DIR / "include"
LIB_DIR = PKG_DIR / "_lib"
BUILD_DIR = PROJECT_DIR / "_build"
LIB_PATH = LIB_DIR / "libgpat_engine.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = {
    "gpat_engine.cpp": [],
    "fields.cu": [],
    "particles.cu": ["-fmad=false"],   # injection draws match the oracle bit for bit
    "mover_fp64.cu": ["-fmad=false"],
    "mover_mixed.cu": [],
    "mover_tile.cu": [],
    "noalloc.cu": [],
    "learned.cu": [],
}


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the engine needs the CUDA toolkit to build")


def _compile(src: str, extra: list[str], nvcc: str, verbose_ptxas: bool, build_dir: Path) -> Path:
    out = build_dir / (src.replace(".", "_") + ".o")
    cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off",
           "-I", str(INCLUDE), "-I", str(CSRC), *extra, "-c", str(CSRC / src), "-o", str(out)]
    if src.endswith(".cpp"):
        cmd[1:1] = ["-x", "cu"]
    if verbose_ptxas and src.endswith(".cu"):
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    if verbose_ptxas:
        (build_dir / (src + ".ptxas.txt")).write_text(res.stderr)
    return out


def build(force: bool = False, verbose_ptxas: bool = False, defines: dict | None = None,
          lib_path: Path | None = None) -> Path:
    """Compiles and links the engine; returns the library path.

    ``defines`` adds -D macros (tuning knobs such as GPAT_MIXED_MINB_2D) and
    ``lib_path`` writes the library elsewhere, so variants can sit side by
    side; load one with ``gpat._abi.load(path)``."""
    out_path = Path(lib_path) if lib_path else LIB_PATH
    srcs = [CSRC / s for s in SOURCES] + [INCLUDE / "gpat_engine.h",
                                          CSRC / "gpat_internal.h", CSRC / "device_common.cuh",
                                          CSRC / "grid_common.cuh", CSRC / "track_common.cuh",
                                          CSRC / "mixed_body.cuh", CSRC / "cell_index.cuh",
                                          CSRC / "mlp_mma.cuh", CSRC / "learned_dev.cuh"]
    if out_path.exists() and not force and not defines:
        lib_mtime = out_path.stat().st_mtime
        if all(s.stat().st_mtime <= lib_mtime for s in srcs):
            return out_path
    nvcc = nvcc_path()
    build_dir = BUILD_DIR if not lib_path else BUILD_DIR / out_path.stem
    build_dir.mkdir(parents=True, exist_ok=True)
    out_path.parent.mkdir(parents=True, exist_ok=True)
    dflags = [f"-D{k}={v}" for k, v in (defines or {}).items()]
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1] + dflags, nvcc, verbose_ptxas,
                                               build_dir), SOURCES.items()))
    tmp = out_path.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, out_path)
    if not lib_path:
        build_driver()
    return out_path


DRIVER_SRC = CSRC / "gpat_run.cpp"
DRIVER_PATH = LIB_DIR / "gpat_run"


def build_driver(force: bool = False) -> Path:
    """Compiles the C++ replay driver against the engine library (C ABI only)."""
    if DRIVER_PATH.exists() and not force and \
            DRIVER_PATH.stat().st_mtime >= max(DRIVER_SRC.stat().st_mtime, LIB_PATH.stat().st_mtime):
        return DRIVER_PATH
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("no C++ compiler for gpat_run")
    cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-ffp-contract=off", "-I", str(INCLUDE), str(DRIVER_SRC),
           "-L", str(LIB_DIR), "-lgpat_engine", "-Wl,-rpath,$ORIGIN", "-o", str(DRIVER_PATH)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"gpat_run build failed:\n{res.stdout}\n{res.stderr}")
    return DRIVER_PATH


if __name__ == "__main__":
    print(build(force=True, verbose_ptxas=True))
