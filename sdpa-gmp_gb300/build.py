"""Build the CUDA library ``libsdpg.so`` in-tree with nvcc for sm_103a.

Every ``csrc/*.cu`` translation unit is compiled in parallel into
``_build/`` and linked into ``sdpa-gmp_gb300/libsdpg.so``.  Only one
``-gencode`` (compute_103a / sm_103a) is emitted.  The command-line driver
``sdpa-gmp_gb300/sdpa_gmp_gb300`` (``cli/sdpa_gmp_gb300.cpp``) is linked
against it with g++.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libsdpg.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "--expt-relaxed-constexpr", "-I" + CSRC, "-I" + os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _digest(paths: list[str], extra: str) -> str:
    h = hashlib.sha256(extra.encode())
    for p in sorted(paths):
        with open(p, "rb") as f:
            h.update(p.encode())
            h.update(f.read())
    return h.hexdigest()


def build(verbose: bool = False, force: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
                     + glob.glob(os.path.join(ROOT, "include", "*.h")))
    cli = sorted(glob.glob(os.path.join(PKG, "cli", "*.cpp")))
    flags = " ".join(ARCH + CFLAGS)
    stamp = os.path.join(BUILD, "libsdpg.stamp")
    digest = _digest(sources + headers + cli, flags + os.uname().machine)
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return LIB
    hdr_digest = _digest(headers, flags)

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        dstamp = obj + ".stamp"
        d = hashlib.sha256((hdr_digest + open(src).read() + os.uname().machine).encode()).hexdigest()
        if not force and os.path.exists(obj) and os.path.exists(dstamp) and open(dstamp).read() == d:
            return obj
        cmd = [nvcc] + ARCH + CFLAGS + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        with open(dstamp, "w") as f:
            f.write(d)
        return obj

    with cf.ThreadPoolExecutor(max_workers=max(2, min(len(sources), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_one, sources))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_cli()
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB


def build_cli() -> str:
    """The command-line driver ``sdpa_gmp_gb300`` beside the library (rpath $ORIGIN)."""
    src = os.path.join(PKG, "cli", "sdpa_gmp_gb300.cpp")
    exe = os.path.join(PKG, "sdpa_gmp_gb300")
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), src, "-o", exe + ".tmp",
           "-L" + PKG, "-lsdpg", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(exe + ".tmp", exe)
    return exe


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
