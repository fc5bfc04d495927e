"""Builds libplb_gb300.so in-tree (plbpd_gb300/_lib/) with nvcc for sm_103a.

Every translation unit compiles in parallel; the shared library links the
CUDA runtime statically.  Device code is built with -fmad=false (every fused
multiply-add in the kernels is written out as __fmaf_rn) and host code with
-ffp-contract=off, so each floating-point operation rounds where the source
says it does.  A stamp of the sources and flags skips rebuilds when nothing
changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libplb_gb300.so")
SOURCES = ["capi.cu", "kernels_ref.cu", "kernels_ref_cluster.cu", "kernels_native.cu", "kernels_trt.cu", "kernels_h2_q9.cu", "kernels_h2_q19.cu",
           "kernels_h2_q27.cu", "kernels_pair32_q9.cu", "kernels_pair32_q19.cu",
           "kernels_pair32_q27.cu", "kernels_util.cu", "kernels_static.cu", "facade.cpp", "server.cpp"]
HEADERS = ["lattice.cuh", "tail_exact.h", "engine.h", "native_impl.cuh", "ref_ops.cuh", "admission.h"]
FACADE_HEADERS = ["Boundary.hpp", "CalcMoments.hpp", "Collision.hpp", "CollisionSRT.hpp", "CollisionTRT.hpp", "Domain.hpp",
                  "EqlbDist.hpp", "Field.hpp", "Flow.hpp", "LBDynamics.hpp", "LBModel.hpp", "PLBPD.hpp", "SimData.hpp",
                  "Streaming.hpp"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
                     "-Xptxas", "-v" if os.environ.get("PLB_PTXAS_VERBOSE") else "-O3",
                     "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stamp() -> str:
    h = hashlib.sha256()
    for name in SOURCES + HEADERS:
        with open(os.path.join(CSRC, name), "rb") as f:
            h.update(f.read())
    with open(os.path.join(ROOT, "include", "plb.h"), "rb") as f:
        h.update(f.read())
    for name in FACADE_HEADERS:
        with open(os.path.join(ROOT, "include", "plbpd", name), "rb") as f:
            h.update(f.read())
    h.update(" ".join(NVCC_FLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles the library if needed and returns its path."""
    os.makedirs(OUT, exist_ok=True)
    stamp_file = os.path.join(OUT, "stamp")
    stamp = _stamp()
    if not force and os.path.exists(LIB) and os.path.exists(stamp_file):
        with open(stamp_file) as f:
            if f.read().strip() == stamp:
                return LIB
    cc = nvcc()

    def compile_one(src: str) -> str:
        obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
        cmd = [cc] + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    r = subprocess.run([cc] + ARCH + ["-shared", "-o", tmp] + objs, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp_file, "w") as f:
        f.write(stamp)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
