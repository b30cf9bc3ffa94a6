"""Build libtdda.so (the CUDA product path) in-tree for sm_103a.

    python topo-dda-forwin64_gb300/build.py            # incremental
    python topo-dda-forwin64_gb300/build.py --force    # rebuild everything

Translation units are compiled in parallel with nvcc, one -gencode
(compute_103a / sm_103a), then linked with the CUDA runtime into
topo-dda-forwin64_gb300/libtdda.so.  No PyTorch, no cmake.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtdda.so")

UNITS = ["tdda_kernels.cu", "tdda_api.cu", "tdda_pass_generic.cu", "tdda_pass_z.cu", "tdda_pass_xy.cu",
         "tdda_pass_zy.cu", "tdda_server.cu", "tdda_pass_xy2.cu", "tdda_pass_dd.cu", "tdda_pass_dd_128.cu", "tdda_pass_dd_192.cu",
         "tdda_pass_dd_160.cu", "tdda_pass_dd_40.cu"]
HEADERS = ["tdda_fft.cuh", "tdda_fft_ct.cuh", "tdda_internal.cuh", "tdda_device.cuh", "tdda_passes.cuh",
           "tdda_tensor.cuh", "tdda_session.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    include = os.path.join(ROOT, "include")
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(include, "tdda.h")]
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-I", include,
                    "--expt-relaxed-constexpr"]
    jobs = []
    objs = []
    for u in UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + hdrs):
            jobs.append([nv] + flags + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        for cmd, res in zip(jobs, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs)):
            if verbose or res.returncode:
                sys.stderr.write(res.stdout + res.stderr)
            if res.returncode:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or _newer(LIB, objs):
        cmd = [nv] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lpthread"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode:
            sys.stderr.write(res.stdout + res.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    print(build(a.force, a.verbose))
