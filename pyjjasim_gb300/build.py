"""Builds libjja_gb300.so in-tree (pyjjasim_gb300/_lib/) for sm_103a.

Two translation units, compiled in parallel: the host factorisation (g++) and the CUDA
kernels + C ABI (nvcc, ``-gencode arch=compute_103a,code=sm_103a``), linked by nvcc.
Used by ``__graft_entry__.build()`` and by ``pyjjasim_gb300._native`` when the library is
missing. No cmake; plain subprocess calls so it runs the same on x86 and aarch64 hosts.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libjja_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand) and not shutil.which(cand):
        raise RuntimeError("nvcc not found; set NVCC or put CUDA's bin directory on PATH")
    return cand


def sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith((".cu", ".cuh", ".cpp", ".h"))] + \
        [os.path.join(ROOT, "include", "jja_gb300.h")]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in sources())


def build(force=False, verbose=False, extra_nvcc=()):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    obj_cpp = os.path.join(OUT_DIR, "jja_factor.o")
    obj_cu = os.path.join(OUT_DIR, "jja_gb300.o")
    cmds = [
        ["g++", "-O3", "-std=c++17", "-fPIC", "-Wall", "-c", os.path.join(CSRC, "jja_factor.cpp"), "-o", obj_cpp] + inc,
        [nvcc, "-O3", "-std=c++17", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-c", os.path.join(CSRC, "jja_gb300.cu"), "-o", obj_cu, *extra_nvcc] + inc,
    ]

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, file=sys.stderr)

    with ThreadPoolExecutor(2) as ex:
        list(ex.map(run, cmds))
    tmp = LIB + ".tmp"
    run([nvcc, "-shared", *ARCH, obj_cpp, obj_cu, "-o", tmp, "-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, extra_nvcc=["-Xptxas", "-v"] if "-v" in sys.argv else ()))
