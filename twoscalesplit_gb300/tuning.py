"""Launch shapes per GPU: the autotuner's choices kept on disk.

tss_solver_autotune times the candidate launch shapes of the four gathers (64, 128
or 256 threads per block; grids covering the list or one persistent wave; one
particle per warp) on a handle's own steps, picks the fastest per gather, and
installs that choice unless the default shape or one particle per warp
throughout runs whole steps faster.  This module keeps the
chosen shape per (GPU model, workload class) in a JSON file, so that later handles
of the same class start with it instead of tuning again.  The reference had one
hard-coded shape (256-thread blocks, TwoScale2D/WCSPHSolver.cu:2421,2437).
"""
import json
import math
import os
import tempfile


def default_cache_path():
    return os.environ.get("TSS_LAUNCH_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "twoscalesplit_gb300", "launch.json"))


def workload_class(kind, n_low):
    """`kind` (single, batch, pool) and the power of two nearest the low-res count."""
    return f"{kind}/2^{int(round(math.log2(max(int(n_low), 1))))}"


def gpu_name():
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(torch.cuda.current_device())
    except Exception:
        pass
    return "cuda"


def load(path=None):
    p = path or default_cache_path()
    try:
        with open(p) as f:
            d = json.load(f)
        return d if isinstance(d, dict) else {}
    except (OSError, ValueError):
        return {}


def store(cache, path=None):
    """Write the cache atomically (a reader sees the old or the new file)."""
    p = path or default_cache_path()
    os.makedirs(os.path.dirname(os.path.abspath(p)), exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=os.path.dirname(os.path.abspath(p)), suffix=".tmp")
    with os.fdopen(fd, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, p)


def tuned_launch(solver, kind, n_low, path=None, steps_per_trial=3, retune=False):
    """Install the cached shape of this GPU and workload class on `solver`, or tune
    it there (the trial steps advance the solver's state) and cache the result.
    Returns (shape, steps the tuning took)."""
    key = f"{gpu_name()}|{workload_class(kind, n_low)}"
    cache = load(path)
    if not retune and key in cache:
        solver.set_launch(cache[key])
        return cache[key], 0
    shape, taken = solver.autotune(steps_per_trial)
    cache[key] = shape
    store(cache, path)
    return shape, taken
