"""Builds liblpmgpu.so for sm_103a (nvcc, translation units in parallel).

Outputs stay in lpm-mac_gb300/_build/ (git-ignored).  Run as a script or call
``build()``; a rebuild happens only when a source is newer than the library.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liblpmgpu.so")
SOURCES = ["lpm_capi.cu", "lpm_force.cu", "lpm_tangent.cu", "lpm_cg.cu", "lpm_laws.cu", "lpm_noalloc.cu", "lpm_adjoint.cu", "lpm_search.cu", "lpm_mfree.cu", "lpm_coarse.cu"]
HEADERS = ["lpm_internal.cuh", "lpm_device.cuh", "lpm_cgvec.cuh", "lpm_df.cuh", "lpm_graph.cuh", "lpm_grid.cuh", "lpm_coarse.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no fused multiply-add contraction, so host-side lengths (the
# initial bond lengths) round like the reference's
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS] + [os.path.join(ROOT, "include", "lpm_gpu.h")]
    return any(os.path.getmtime(p) > t for p in deps)


def build(force=False, verbose=False, ptxas_info=False):
    """Compiles every translation unit and links the shared library."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_info else []

    def compile_one(src):
        obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc] + ARCH + FLAGS + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose or ptxas_info:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
