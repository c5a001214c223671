"""Builds the engine's shared library for sm_103a with nvcc.

    python -m gpuvoxels_gb300.build          # -> gpuvoxels_gb300/_build/libgpuvoxels_gb300.so

All translation units compile in parallel into one in-tree shared library.
Device code is compiled with -fmad=false and host code with
-ffp-contract=off: every multiply and add rounds separately, as in the
reference CPU path, which is what the parity bar (1e-6 voxel sizes after
1,000 steps) is measured against.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgpuvoxels_gb300.so")
WORKER = os.path.join(OUT_DIR, "vx3_node_worker")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["kernels_exact.cu", "kernels_fast.cu", "engine.cu", "noalloc.cu", "world.cpp", "xml_dom.cpp", "capi.cpp", "history.cpp"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build gpuvoxels_gb300")


def _flags(src: str):
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I", CSRC,
              "-I", os.path.join(HERE, "..", "include")]
    if src.endswith(".cu"):
        fmad = "-fmad=true" if src == "kernels_fast.cu" else "-fmad=false"
        # GVX_NVCC_DEFINES: extra -D tuning knobs for the kernels, e.g. "GVX_LINKS_MIN_BLOCKS=3"
        defs = ["-D" + x for x in os.environ.get("GVX_NVCC_DEFINES", "").split()]
        return common + ARCH + ["-lineinfo", fmad, "-Xptxas", "-warn-spills"] + defs
    return common


def needs_build() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(WORKER):
        return True
    t = min(os.path.getmtime(LIB), os.path.getmtime(WORKER))
    for d in (CSRC, os.path.join(HERE, "..", "include")):
        for f in os.listdir(d):
            if os.path.getmtime(os.path.join(d, f)) > t:
                return True
    return False


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not needs_build():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    exe = nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(OUT_DIR, src + ".o")
        cmd = [exe, "-c", os.path.join(CSRC, src), "-o", obj] + _flags(src)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [exe, "-shared", "-o", tmp] + objs + ARCH + ["-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    # the worker executable (vx3_node_worker process contract) over the library
    cmd = [exe, os.path.join(CSRC, "worker_main.cpp"), "-o", WORKER + ".tmp", "-O2", "-std=c++17", "-I", CSRC,
           "-I", os.path.join(HERE, "..", "include"), "-L", OUT_DIR, "-lgpuvoxels_gb300", "-Xlinker", "-rpath,$ORIGIN",
           "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"worker link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(WORKER + ".tmp", WORKER)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
