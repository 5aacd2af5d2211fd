"""Build libkdgr.so in-tree (sm_103a device code, host C++).

Translation units compile in parallel; object files go to ``_build/`` next
to this file and the library to ``libkdgr.so``.  Flags per unit:

* ``render_exact.cu``: ``--fmad=false`` with IEEE division and square root;
  the kernel also spells every operation as an ``__f*_rn`` intrinsic, so the
  oracle-matching arithmetic does not depend on the flag;
* ``render_fast.cu``: default contraction (FMA) for the fast forms;
* host ``.cpp``: ``-ffp-contract=off`` -- the kd-tree builder and the camera
  set-up must round exactly like the reference host code.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libkdgr.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_UNITS = {
    "render_exact.cu": ["--fmad=false", "-prec-div=true", "-prec-sqrt=true"],
    "render_fast.cu": [],
    "kdgr_noalloc.cu": [],
    "scene_pack.cu": ["--fmad=false", "-prec-div=true", "-prec-sqrt=true"],
    "kdbuild_gpu.cu": ["--fmad=false", "-prec-div=true", "-prec-sqrt=true"],
}
CPP_UNITS = ["kdbuild.cpp", "kdgr_tree_api.cpp", "kdgr_api.cpp", "kdgr_batch_api.cpp", "kdgr_reference_api.cpp",
             "kdgr_server.cpp", "kdgr_debug.cpp", "kdgr_ingest.cpp", "kdgr_hybrid.cpp"]


def _cuda_home() -> str:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    inc = ["-I" + os.path.join(REPO, "include"), "-I" + CSRC]
    jobs = []
    # KDGR_NVCC_DEFINES: extra -D options (e.g. "KDGR_FAST_HITS=2 KDGR_FAST_STACK=16") for
    # compile-time variants of the fast kernel
    defs = ["-D" + d for d in os.environ.get("KDGR_NVCC_DEFINES", "").split()]
    for src, extra in CU_UNITS.items():
        obj = os.path.join(OUT_DIR, src + ".o")
        cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", *inc, *extra, *defs,
               "-c", os.path.join(CSRC, src), "-o", obj]
        if ptxas_info:
            cmd.insert(1, "-Xptxas=-v")
        jobs.append((cmd, obj))
    for src in CPP_UNITS:
        obj = os.path.join(OUT_DIR, src + ".o")
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-pthread", *inc,
               "-I" + os.path.join(cuda, "include"), "-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append((cmd, obj))
    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        logs = list(ex.map(lambda j: _run(j[0]), jobs))
    if verbose or ptxas_info:
        for l in logs:
            if l.strip():
                print(l, file=sys.stderr)
    objs = [o for _, o in jobs]
    tmp = LIB + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", tmp, *objs, "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv))
