"""In-tree build of the CUDA library ``pdspy_gb300/_build/libpdgpu.so`` (sm_103a).

Each translation unit is compiled by nvcc in parallel and linked into one shared
library that exports the C ABI declared in ``include/pdgpu.h``.  The Monte Carlo and
ray-tracing units are compiled with ``--fmad=false`` and host ``-ffp-contract=off`` so that every
floating-point operation is a single IEEE operation (the walk is bit-reproducible and
comparable operation for operation with the CPU oracle); the other units use the
default contraction.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libpdgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, extra flags)
UNITS = [
    ("mctherm.cu", ["--fmad=false", "-Xcompiler", "-ffp-contract=off"]),
    ("raytrace.cu", ["--fmad=false", "-Xcompiler", "-ffp-contract=off"]),
    ("mcscat.cu", ["--fmad=false", "-Xcompiler", "-ffp-contract=off"]),
    ("dft.cu", []),
]
HEADERS = ["mc_common.h", "mc_device.cuh", "mc_geom.cuh", "mc_geom_ds.cuh", "mc_host.h"]


def nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    for c in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pdspy_gb300")


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, u) for u, _ in UNITS] + [os.path.join(CSRC, h) for h in HEADERS]
    deps.append(os.path.join(ROOT, "include", "pdgpu.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps)


def _compile(unit, flags, verbose):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OUT, unit + ".o")
    cmd = [nvcc()] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                             "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj] + flags
    if verbose:
        cmd += ["-Xptxas", "-v"]
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (unit, r.stdout, r.stderr))
    if verbose and r.stderr:
        print(r.stderr)
    return obj


def build(force=False, verbose=False):
    """Compile and link the library if a source changed; returns its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    with ThreadPoolExecutor(max_workers=max(1, len(UNITS))) as ex:
        objs = list(ex.map(lambda u: _compile(u[0], u[1], verbose), UNITS))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
