"""Builds libgspec.so (the CUDA kernels + C ABI) in-tree for sm_103a.

Each translation unit is compiled by its own nvcc process in parallel and
then linked into ``psrdada_cpp_gb300/libgspec.so``.  No cmake, one -gencode.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / os.environ.get("GSPEC_BUILD_DIR", "_build")
LIB = Path(os.environ["GSPEC_LIB"]) if os.environ.get("GSPEC_LIB") else PKG / "libgspec.so"
# extra nvcc flags (e.g. -D tuning knobs) and a separate object folder for variant builds
EXTRA = os.environ.get("GSPEC_NVCC_FLAGS", "").split()
SOURCES = ["gspec_kernels.cu", "gspec_fourstep.cu", "gspec_engine.cu", "gspec_noalloc.cu", "gspec_server.cu",
           "gspec_batch.cu", "gspec_tc.cu", "gspec_dummy.cu",
           "gspec_vlbi.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")


def nvcc_flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                   "-I", str(PKG.parent / "include")] + EXTRA + list(extra)


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False, ptxas_v: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "gspec.h"]
    objs, procs = [], []
    for src in SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + headers):
            cmd = [NVCC] + nvcc_flags(["-Xptxas", "-v"] if ptxas_v else []) + ["-c", str(CSRC / src), "-o", str(obj)]
            if verbose:
                print(" ".join(cmd), flush=True)
            procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0 or verbose or ptxas_v:
            sys.stdout.write(out)
        if p.returncode != 0:
            failed.append(src)
    if failed:
        raise RuntimeError(f"nvcc failed for {failed}")
    if force or procs or _stale(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs] + ["-lcudart", "-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv, ptxas_v="--ptxas" in sys.argv)
