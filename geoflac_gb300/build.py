"""In-tree build of the CUDA library (sm_103a) behind include/geoflac_gb300.h.

Compiles every translation unit in parallel with nvcc / g++ and links
``geoflac_gb300/libgeoflac_gb300.so``.  The FP64 kernels are compiled with
``-fmad=false`` (no contraction of a*b+c into one rounding, as in the
serial reference); the mixed-precision kernels use contraction and the
approximate FP32 division and square root (2 ulp).  Host C++ is
compiled with ``-ffp-contract=off`` so that x86 and Arm hosts round alike.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgeoflac_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]

UNITS = [
    ("gf_fp64.cu", ["-fmad=false"]),
    ("gf_mixed.cu", ["-fmad=true", "-prec-div=false", "-prec-sqrt=false"]),
    ("gf_capi.cu", ["-fmad=false"]),
    ("gf_noalloc.cu", ["-fmad=false"]),
    ("gf_remesh.cu", ["-fmad=false"]),
    ("gf_io.cu", ["-fmad=false"]),
    ("gf_batch.cu", ["-fmad=true", "-prec-div=false", "-prec-sqrt=false"]),
    ("fno_gemm.cu", ["-fmad=true"]),
    ("fno_ops.cu", ["-fmad=true"]),
    ("host_inp.cpp", None),
    ("host_setup.cpp", None),
]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_lib_dir(nvcc: str) -> str:
    root = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    for sub in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        p = os.path.join(root, sub)
        if os.path.exists(os.path.join(p, "libcudart.so")):
            return p
    return os.path.join(root, "lib64")


def _needs(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_v: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    jobs = []
    objs = []
    for src, extra in UNITS:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if not force and not _needs(obj, [path] + headers):
            continue
        if extra is None:
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-c", path, "-o", obj]
        else:
            cmd = [nvcc] + ARCH + NVCC_COMMON + extra + (["-Xptxas", "-v"] if ptxas_v else []) + ["-c", path, "-o", obj]
        jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0 or ptxas_v:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"compile failed: {' '.join(cmd)}")
    if force or jobs or not os.path.exists(LIB):
        link = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-L" + _cuda_lib_dir(nvcc), "-lcudart"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, ptxas_v="--ptxas" in sys.argv, force="-f" in sys.argv)
    print(LIB)
