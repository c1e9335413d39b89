"""Build libgategpu.so (the CUDA transport path) in-tree for sm_103a.

Each .cu file under ``csrc/`` compiles in parallel to an object file under
``_build/``; the objects link into ``opengate_gb300/_lib/libgategpu.so``.
``-fmad=false`` keeps each a*b+c as a rounded multiply followed by a rounded
add (fused only where the source calls fma), which the bit-reproducibility of
a history relies on.
"""

import os
import pathlib
import shutil
import subprocess
import sys

PKG = pathlib.Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG.parent / "_build" / "csrc"
LIB_DIR = PKG / "_lib"
LIB = LIB_DIR / "libgategpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def sources():
    return sorted(CSRC.glob("*.cu"))


def _stale(target, deps):
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose=False, ptxas_verbose=False):
    BUILD.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [PKG.parent / "include" / "gate_gpu.h"]
    objs, procs = [], []
    for src in sources():
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if not _stale(obj, [src] + headers) and not ptxas_verbose:
            continue
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
        if ptxas_verbose:
            cmd.insert(1, "-Xptxas=-v")
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((cmd, subprocess.Popen(cmd)))
    for cmd, p in procs:
        if p.wait() != 0:
            raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", *[str(o) for o in objs], "-o", str(LIB)]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_verbose="-v" in sys.argv)
