"""Builds the in-tree CUDA library cfd3d_gb300/_build/libcfd3d_gb300.so for sm_103a.

Translation units are compiled in parallel (one nvcc per .cu file) and linked with
nvcc; no PyTorch headers are involved -- the library exposes the plain C ABI of
include/cfd3d.h.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libcfd3d_gb300.so")
UNITS = ["adjoint_face.cu", "adjoint.cu", "engine.cu", "setup.cu", "flux.cu", "flux_mixed.cu", "peak.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-I", os.path.join(ROOT, "include")]
# the adjoint's dual-number kernels are large and off the iteration's path: the device
# compiler's fast-compile mode keeps their build at seconds instead of minutes
UNIT_FLAGS = {"adjoint.cu": ["-Ofc", "mid"], "adjoint_face.cu": ["-Ofc", "mid"]}


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    files = [os.path.join(SRC, f) for f in os.listdir(SRC)] + [os.path.join(ROOT, "include", "cfd3d.h")]
    return max(os.path.getmtime(f) for f in files)


def build(force=False, verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps():
        return LIB
    nv = nvcc()

    def compile_one(u):
        obj = os.path.join(OUT, u.replace(".cu", ".o"))
        cmd = [nv, *ARCH, *FLAGS, *UNIT_FLAGS.get(u, []), *extra, "-c", os.path.join(SRC, u), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {u}:\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(len(UNITS)) as ex:
        objs = list(ex.map(compile_one, UNITS))
    tmp = LIB + ".tmp"
    cmd = [nv, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv,
          extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else [])
    print(LIB)
