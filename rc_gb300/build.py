"""Build librc_gb300.so in-tree with nvcc for sm_103a.

Each .cu under rc_gb300/csrc compiles to an object in parallel (one -gencode,
-lineinfo), then one shared library is linked next to this file.  The build
is skipped when the library is newer than every source.

    python -m rc_gb300.build [--force] [--ptxas-v]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librc_gb300.so")
# the bounds-checked variant (-DGB_CHECKED), built on request
LIB_CHECKED = os.path.join(HERE, "librc_gb300_checked.so")
BUILD_CHECKED = os.path.join(HERE, "_build_checked")
# the MS5 binding variant (-DGB_MS5_ABI: MS5's kern_scatter and kern_fft,
# include/rc_gb300_ms5.h), built on request
LIB_MS5 = os.path.join(HERE, "librc_gb300_ms5.so")
BUILD_MS5 = os.path.join(HERE, "_build_ms5")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build rc_gb300")
    return cand


def cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h")) + [
        os.path.abspath(__file__)]


def up_to_date(lib: str = LIB) -> bool:
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force: bool = False, ptxas_verbose: bool = False, verbose: bool = False,
          checked: bool = False, ms5: bool = False) -> str:
    """Build the library; checked=True builds the bounds-checked variant
    (librc_gb300_checked.so, -DGB_CHECKED), ms5=True the MS5 binding variant
    (librc_gb300_ms5.so, -DGB_MS5_ABI) instead."""
    lib_out, build_dir = ((LIB_CHECKED, BUILD_CHECKED) if checked else
                          (LIB_MS5, BUILD_MS5) if ms5 else (LIB, BUILD))
    if not force and up_to_date(lib_out):
        return lib_out
    os.makedirs(build_dir, exist_ok=True)
    cc = nvcc()
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE,
                    "--expt-relaxed-constexpr"]
    if checked:
        flags += ["-DGB_CHECKED"]
    if ms5:
        flags += ["-DGB_MS5_ABI"]
    if ptxas_verbose:
        flags += ["-Xptxas", "-v"]

    def one(src):
        obj = os.path.join(build_dir, os.path.basename(src)[:-3] + ".o")
        cmd = [cc] + flags + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        results = list(ex.map(one, sources()))
    if verbose or ptxas_verbose:
        for obj, err in results:
            if err.strip():
                print(f"--- {os.path.basename(obj)}\n{err}", file=sys.stderr)
    objs = [o for o, _ in results]
    libdir = os.path.join(cuda_home(), "lib64")
    tmp = lib_out + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + [
        "-L", libdir, "-lcufft", "-lpthread", "-Xlinker", "-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib_out)
    return lib_out


STRATEGY_SRC = os.path.join(HERE, "host", "gridding_strategy.cpp")


def strategy_program(out_dir: str | None = None, ms5: bool = False) -> str:
    """Compile host/gridding_strategy.cpp (the MS6 gridding strategy on the C++
    host layer, include/rc_kernels.hpp) against librc_gb300.so (or, ms5=True,
    librc_gb300_ms5.so with -DGB_MS5_ABI); returns the executable's path.
    Rebuilt when older than its sources or the library."""
    lib_out = build(ms5=ms5)
    out_dir = out_dir or BUILD
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "gridding_strategy_ms5" if ms5 else "gridding_strategy")
    deps = [STRATEGY_SRC, lib_out] + glob.glob(os.path.join(INCLUDE, "*"))
    if os.path.exists(exe) and all(os.path.getmtime(d) <= os.path.getmtime(exe) for d in deps):
        return exe
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-Wall", "-Wextra", "-pthread",
           "-I", INCLUDE, STRATEGY_SRC, "-L", HERE,
           "-lrc_gb300_ms5" if ms5 else "-lrc_gb300", "-Wl,-rpath," + HERE, "-o", exe + ".tmp"]
    if ms5:
        cmd.insert(1, "-DGB_MS5_ABI")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 or "warning" in r.stderr:
        raise RuntimeError(f"g++ failed on {STRATEGY_SRC}:\n{r.stderr}")
    os.replace(exe + ".tmp", exe)
    return exe


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--ptxas-v", action="store_true")
    a = ap.parse_args(argv)
    print(build(force=a.force, ptxas_verbose=a.ptxas_v, verbose=True))


if __name__ == "__main__":
    main()
