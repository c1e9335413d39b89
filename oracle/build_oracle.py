"""Build the CPU oracle shared libraries (test infrastructure only).

Produces ``oracle/_build/libggo32.so`` (float transport arithmetic) and
``oracle/_build/libggo64.so`` (double).  ``-ffp-contract=off`` keeps every
``a*b+c`` as a separately rounded multiply and add, the same rule the CUDA
kernels are compiled with (``-fmad=false``), so both execute identical
floating-point operation sequences.
"""

import pathlib
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
OUT = HERE / "_build"


def build(verbose=False):
    OUT.mkdir(exist_ok=True)
    src = HERE / "gg_oracle.c"
    procs = []
    for name, extra in (("libggo32.so", []), ("libggo64.so", ["-DGGO_DOUBLE"])):
        target = OUT / name
        if target.exists() and target.stat().st_mtime >= src.stat().st_mtime:
            continue
        cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
               "-fno-fast-math", "-fno-strict-aliasing", *extra, str(src), "-o", str(target), "-lm"]
        if verbose:
            print(" ".join(cmd))
        procs.append((cmd, subprocess.Popen(cmd)))
    for cmd, p in procs:
        if p.wait() != 0:
            raise RuntimeError("oracle build failed: " + " ".join(cmd))
    return OUT


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
