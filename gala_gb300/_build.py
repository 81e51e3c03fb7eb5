"""Build the CUDA library ``gala_gb300/_build/libgala_gb300.so`` for sm_103a.

The library is compiled in-tree with nvcc (one process per translation unit, in
parallel) and linked with the static CUDA runtime.  FP64 translation units that
reproduce gala's arithmetic are compiled with ``-fmad=false`` so that no
multiply-add is contracted; the FP32 / tensor-core units keep contraction on.
``build(debug=True)`` makes the debug library ``libgala_gb300_debug.so`` from the
same sources with ``-DGX_DEBUG_CHECKS`` (device-side check records,
gx_debug_read), its objects kept apart in ``_build/debug``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libgala_gb300.so"
LIB_DEBUG = OUT / "libgala_gb300_debug.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]

# translation unit -> extra flags
UNITS = {
    "gx_host.cu": ["-fmad=false"],
    "gx_fixed.cu": ["-fmad=false"],
    "gx_dop853.cu": ["-fmad=false"],
    "gx_nbody.cu": ["-fmad=false"],
    "gx_nbody_wide.cu": ["-fmad=false"],
    "gx_lfnbody.cu": ["-fmad=false"],
    "gx_orbit.cu": ["-fmad=false"],
    "gx_peaks.cu": [],
    "gx_batch.cu": [],
    "gx_dop853_fp32.cu": [],
    "gx_nbody_fp32.cu": [],
    "gx_nbody_wide_fp32.cu": [],
    "gx_stream32.cu": [],
    "gx_mlp_train.cu": [],
    "gx_mlp_infer.cu": [],
    "gx_mlp_tc.cu": [],
}


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build gala_gb300")


def _sources_newer(target: Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    deps = list(CSRC.glob("*")) + [PKG.parent / "include" / "gala_gb300.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build(force: bool = False, verbose: bool = False, debug: bool = False) -> Path:
    """Compile every CUDA translation unit and link the shared library (the
    debug library with ``debug=True``).

    Processes that build at once (ranks of one job, parallel test workers)
    take turns on a lock file; a process that waited finds the library fresh
    and returns."""
    import fcntl

    lib = LIB_DEBUG if debug else LIB
    if not force and not _sources_newer(lib):
        return lib
    OUT.mkdir(exist_ok=True)
    with open(OUT / ".build.lock", "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        try:
            if not force and not _sources_newer(lib):
                return lib
            return _build_locked(verbose, debug)
        finally:
            fcntl.flock(lock, fcntl.LOCK_UN)


def _build_locked(verbose: bool, debug: bool = False) -> Path:
    cc = nvcc()
    objdir = OUT / "debug" if debug else OUT
    objdir.mkdir(exist_ok=True)
    lib = LIB_DEBUG if debug else LIB
    flags = ["-DGX_DEBUG_CHECKS"] if debug else []

    def compile_unit(item):
        name, extra = item
        obj = objdir / (Path(name).stem + ".o")
        cmd = [cc, *ARCH, *COMMON, *flags, *extra, "-c", str(CSRC / name), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(len(UNITS), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_unit, UNITS.items()))
    tmp = OUT / f"{lib.name}.{os.getpid()}.tmp"
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, debug="--debug" in sys.argv))
