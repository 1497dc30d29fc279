"""Build the oracle libraries (TEST INFRASTRUCTURE: never loaded by the product).

  liboracle.so        -- tss_oracle.cpp, the CPU restatement of the step (g++,
                         OpenMP, -ffp-contract=off so FP32 follows the reference's
                         operation order without fused multiply-adds)
  _ref/librefcpu.so   -- the reference's own kernel source compiled for the CPU
                         (refcpu/build_ref.sh); only when the reference checkout is
                         present, i.e. on the build machine, not on the GPU machine
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REFCPU_SO = os.path.join(HERE, "_ref", "librefcpu.so")
REFERENCE_ROOT = os.environ.get("TSS_REFERENCE_ROOT", "/root/reference")


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force=False):
    src = os.path.join(HERE, "tss_oracle.cpp")
    hdr = os.path.join(HERE, "..", "include", "tss.h")
    if not force and not _stale(ORACLE_SO, [src, hdr]):
        return ORACLE_SO
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-fPIC", "-shared", "-o", ORACLE_SO, src]
    subprocess.check_call(cmd)
    return ORACLE_SO


def build_refcpu(force=False):
    """Returns the library path, or None when the reference sources are absent."""
    cur = os.path.join(REFERENCE_ROOT, "TwoScale2D", "WCSPHSolver.cu")
    if not os.path.exists(cur):
        return None
    deps = [os.path.join(HERE, "refcpu", f) for f in ("cuda_shim.h", "refcpu_harness.inc", "build_ref.sh")]
    if not force and not _stale(REFCPU_SO, deps):
        return REFCPU_SO
    subprocess.check_call(["sh", os.path.join(HERE, "refcpu", "build_ref.sh"), REFERENCE_ROOT])
    return REFCPU_SO


def build(force=False):
    build_oracle(force)
    build_refcpu(force)


if __name__ == "__main__":
    build(force="--force" in sys.argv)
