"""Build the oracle libraries (TEST INFRASTRUCTURE: never loaded by the product).

  liboracle.so        -- tss_oracle.cpp, the CPU restatement of the step (g++,
                         OpenMP, -ffp-contract=off so FP32 follows the reference's
                         operation order without fused multiply-adds)
  _ref/librefcpu.so   -- the reference's own kernel source compiled for the CPU
                         (refcpu/build_ref.sh); only when a reference checkout is
                         given, i.e. on the build machine, not on the GPU machine
  _ref/refkern.cubin  -- the reference's own kernel source compiled for sm_103a
                         (refgpu/build_refgpu.sh); only where the checkout is
                         present.  Device code only: it travels to the GPU machine.
  librefgpu.so        -- refgpu/refgpu_launcher.cu, the host side that loads that
                         cubin and runs the reference's step on the GPU (nvcc;
                         built wherever nvcc is, including the GPU machine)
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REFCPU_SO = os.path.join(HERE, "_ref", "librefcpu.so")
REFGPU_CUBIN = os.path.join(HERE, "_ref", "refkern.cubin")
REFGPU_SO = os.path.join(HERE, "librefgpu.so")


def reference_root(root=None):
    """The reference checkout to build from: `root`, else $TSS_REFERENCE_ROOT, else
    None (then only the prebuilt files are used)."""
    root = root or os.environ.get("TSS_REFERENCE_ROOT")
    if root and os.path.exists(os.path.join(root, "TwoScale2D", "WCSPHSolver.cu")):
        return root
    if root:
        sys.stderr.write(f"oracle: no reference sources under {root}; using the prebuilt files if any\n")
    return None


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


def build_refcpu(force=False, root=None):
    """Returns the library path: built from the reference checkout (`root` or
    $TSS_REFERENCE_ROOT) when given, else the prebuilt library if any, else None."""
    ref = reference_root(root)
    if ref is None:
        return REFCPU_SO if os.path.exists(REFCPU_SO) else None
    deps = [os.path.join(HERE, "refcpu", f) for f in ("cuda_shim.h", "refcpu_harness.inc", "build_ref.sh")]
    if not force and not _stale(REFCPU_SO, deps):
        return REFCPU_SO
    subprocess.check_call(["sh", os.path.join(HERE, "refcpu", "build_ref.sh"), ref])
    return REFCPU_SO


def build_refgpu_cubin(force=False, root=None):
    """Returns the cubin path: built from the reference checkout (`root` or
    $TSS_REFERENCE_ROOT) when given, else the cubin built on the build machine if it
    is there, else None."""
    ref = reference_root(root)
    if ref is None:
        return REFGPU_CUBIN if os.path.exists(REFGPU_CUBIN) else None
    deps = [os.path.join(HERE, "refgpu", f) for f in ("refgpu_shim.cuh", "refgpu_entry.inc", "build_refgpu.sh")]
    if not force and not _stale(REFGPU_CUBIN, deps):
        return REFGPU_CUBIN
    subprocess.check_call(["sh", os.path.join(HERE, "refgpu", "build_refgpu.sh"), ref])
    return REFGPU_CUBIN


def build_refgpu_launcher(force=False):
    """Returns the launcher library path (nvcc; links the CUDA driver library)."""
    src = os.path.join(HERE, "refgpu", "refgpu_launcher.cu")
    hdr = os.path.join(HERE, "..", "include", "tss.h")
    if not force and not _stale(REFGPU_SO, [src, hdr]):
        return REFGPU_SO
    sys.path.insert(0, os.path.join(HERE, ".."))
    from twoscalesplit_gb300 import build as tb
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(tb.nvcc())), "lib64")
    cmd = [tb.nvcc(), "-std=c++17", "-O2", f"-gencode=arch=compute_{tb.ARCH},code=sm_{tb.ARCH}",
           "-Xcompiler", "-fPIC", "-shared", "-I", os.path.join(HERE, "..", "include"), "-o", REFGPU_SO, src,
           "-L", cuda_lib, "-L", os.path.join(cuda_lib, "stubs"), "-lcuda"]
    subprocess.check_call(cmd)
    return REFGPU_SO


def build(force=False, root=None):
    build_oracle(force)
    if reference_root(root) is None:
        sys.stderr.write("oracle: no reference checkout given (pass it, or set TSS_REFERENCE_ROOT): the "
                         "reference's kernels are not rebuilt\n")
    build_refcpu(force, root)
    build_refgpu_cubin(force, root)
    build_refgpu_launcher(force)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    build(force="--force" in sys.argv, root=args[0] if args else None)
