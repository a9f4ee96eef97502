"""In-tree build of the CUDA library ``optifax_gb300/_lib/liboptifax.so`` for sm_103a.

The translation units are compiled in parallel with nvcc and linked into one
shared library exporting the C ABI declared in include/optifax.h.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "liboptifax.so")
SOURCES = ["ofx_api.cu", "ofx_k_heun_large.cu", "ofx_k_heun_small.cu", "ofx_k_rk23.cu", "ofx_k_heun_nee.cu", "ofx_noalloc.cu", "ofx_fp64.cu", "ofx_f32x2.cu", "ofx_gemm.cu", "ofx_fno.cu", "ofx_setup.cu", "ofx_gnlse.cu"]
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-I" + os.path.join(HERE, "..", "include")]
# per-file flags: the float-float kernel's error-free transformations must not be
# contracted into fused multiply-adds (every intended one is an explicit fmaf)
EXTRA_FLAGS = {"ofx_f32x2.cu": ["-fmad=false"]}


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the optifax CUDA library cannot be built")


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh"))] + \
        [os.path.join(HERE, "..", "include", "optifax.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force: bool = False, verbose: bool = False, jobs: int = 0) -> str:
    if not force and up_to_date():
        return LIB
    nvcc = _nvcc()
    os.makedirs(OUT_DIR, exist_ok=True)
    objs = [os.path.join(OUT_DIR, os.path.splitext(s)[0] + ".o") for s in SOURCES]

    def compile_one(i):
        cmd = [nvcc] + NVCC_FLAGS + EXTRA_FLAGS.get(SOURCES[i], []) + ["-c", os.path.join(CSRC, SOURCES[i]),
                                                                       "-o", objs[i]]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {SOURCES[i]}:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=jobs or len(SOURCES)) as ex:
        for msg in ex.map(compile_one, range(len(SOURCES))):
            if verbose and msg:
                print(msg, file=sys.stderr)
    tmp = LIB + ".tmp"
    cmd = [nvcc, GENCODE, "-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
