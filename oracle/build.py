"""Build recipe for the CPU oracle (test infrastructure only).

Compiles the C restatement in this directory into ``oracle/_build/liborc.so`` with
gcc.  ``-ffp-contract=off`` and the absence of fast-math keep every floating-point
operation a single IEEE operation, which the bit-for-bit comparison with the GPU path
depends on.  The reference project has no C/C++ source for this path (its radmc3d
branch shells out to the external RADMC-3D binary), so there is no ``oracle/_ref``
build.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liborc.so")
SOURCES = ["mcrt_oracle.c", "geom_ds.c", "raytrace_oracle.c", "mcscat_oracle.c"]
CFLAGS = ["-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
          "-fno-fast-math", "-Wall", "-Wno-unused-function"]


def needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for f in SOURCES + ["mcrt_oracle.h", "raytrace_oracle.h", "mc_internal.h"]:
        p = os.path.join(HERE, f)
        if os.path.exists(p) and os.path.getmtime(p) > t:
            return True
    return False


def build(force=False, verbose=False):
    if not force and not needs_build():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, f) for f in SOURCES if os.path.exists(os.path.join(HERE, f))]
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc"] + CFLAGS + srcs + ["-o", tmp, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
