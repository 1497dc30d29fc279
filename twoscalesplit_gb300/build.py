"""Build libtss.so in-tree: the sm_103a kernels and the host solver behind the C ABI.

Flags that matter for results: --fmad=false, -prec-div=true, -prec-sqrt=true (no
fast math), so every FP32 expression rounds exactly as written, as the
reference's Release build (FastMath=false) evaluated it.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtss.so")
SOURCES = ["grid.cu", "grid_noalloc.cu", "sph.cu", "sph_fast.cu", "solver.cu", "pool.cu", "render.cu", "serve.cpp"]
HEADERS = ["tss_device.cuh", "arith.cuh", "gather.cuh", "gathers.cuh", "grid.cuh", "sph.cuh", "solver_impl.cuh",
           "extent.hpp"]
ARCH = os.environ.get("TSS_CUDA_ARCH", "103a")


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def flags():
    return ["-std=c++17", "-O3", f"-gencode=arch=compute_{ARCH},code=sm_{ARCH}", "-lineinfo", "--fmad=false",
            "-prec-div=true", "-prec-sqrt=true", "-ftz=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(HERE, "..", "include", "tss.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, ptxas_info=False):
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    procs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [cc, *flags(), "-c", os.path.join(CSRC, src), "-o", obj]
        if ptxas_info:
            cmd.insert(1, "-Xptxas=-v")
        if verbose:
            print(" ".join(cmd))
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0 or (ptxas_info and out):
            sys.stderr.write(out.decode(errors="replace"))
        if p.returncode != 0:
            failed.append(src)
    if failed:
        raise RuntimeError(f"nvcc failed for {failed}")
    tmp = LIB + ".tmp"
    # cudart is linked statically (nvcc's default), so the library needs only the driver
    subprocess.check_call([cc, "-shared", f"-gencode=arch=compute_{ARCH},code=sm_{ARCH}", "-o", tmp, *objs])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
    print("built", LIB)
