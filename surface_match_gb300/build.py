"""In-tree build of libsurface_match.so (CUDA sm_103a + the C++ Detector shim).

Translation units compile in parallel with nvcc; the float-exactness flags are part of
the product's contract: ``--fmad=false`` on the device and ``-ffp-contract=off`` on the
host keep the quantised PPF keys, alpha angles and vote bins bit-identical to the CPU
restatement that checks them.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.abspath(os.path.join(HERE, "..", "include"))
LIB = os.path.join(HERE, "libsurface_match.so")

CU_SOURCES = ["sort.cu", "kdtree.cu", "prep.cu", "vote.cu", "vote_pipe.cu", "cluster.cu", "icp.cu", "api.cu", "noalloc.cu", "batch.cu", "server.cu",
              "probe.cu", "mls.cu"]
CPP_SOURCES: list = []
HEADERS = ["sm_math.h", "sm_linalg.h", "sm_icp.h", "sm_grid.h", "sm_device.cuh", "sm_vote.cuh",
           "sm_kdtree.cuh",
           "sm_engine.h", "sm_stages.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-prec-div=true",
              "-prec-sqrt=true", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
              "-I", INCLUDE, "-I", CSRC]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
             "-I", INCLUDE, "-I", CSRC]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_root():
    return os.path.dirname(os.path.dirname(nvcc()))


def _newest(paths):
    return max(os.path.getmtime(p) for p in paths if os.path.exists(p))


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in CU_SOURCES + CPP_SOURCES]
    deps = srcs + [os.path.join(CSRC, h) for h in HEADERS] + \
        [os.path.join(INCLUDE, "surface_match.h"), os.path.join(INCLUDE, "ppf.h"), __file__]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest(deps):
        return LIB
    header_time = _newest([d for d in deps if not d.endswith((".cu", ".cpp"))])

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        if not force and os.path.exists(obj) and \
                os.path.getmtime(obj) >= max(os.path.getmtime(src), header_time):
            return obj, ""
        if src.endswith(".cu"):
            cmd = [nvcc()] + ARCH + NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_info else []) + \
                ["-c", src, "-o", obj]
        else:
            cmd = ["g++"] + CXX_FLAGS + ["-I", os.path.join(_cuda_root(), "include"), "-c",
                                         src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        results = list(ex.map(compile_one, srcs))
    if verbose or ptxas_info:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
