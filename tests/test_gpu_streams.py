"""GPU: the C ABI waits for one solver's own work, not for the whole device.

The reference checked for errors after every launch with CheckLastError
(CUDA/cuda.h:24-35) on the default stream of a single-solver process.  Here a
host application may run other solvers, or its own kernels, on other streams:
tss_solver_counts / _sync / _download / _copy must return once this solver's work
is done, while unrelated streams still have work queued; and steps enqueued on
different streams must still run in order.
"""
import time

import numpy as np
import pytest

from twoscalesplit_gb300 import _abi, scenes
from twoscalesplit_gb300.solver import Solver

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from twoscalesplit_gb300 import build
    build.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"


def test_queries_do_not_wait_for_unrelated_streams():
    import torch
    sc = scenes.dam_break_small(16, 32, seed=1)
    sol = Solver.from_scene(sc)
    sol.step(3)
    sol.sync()
    other = torch.cuda.Stream()
    # about a second of a bounded spin on a stream the solver knows nothing about
    cycles = int(2.5e9)
    with torch.cuda.stream(other):
        torch.cuda._sleep(cycles)
    t0 = time.perf_counter()
    sol.step(2)
    c = sol.counts()
    sol.sync()
    d = sol.download(_abi.TSS_SCALE_LOW)
    dens = sol.copy(_abi.TSS_SCALE_LOW, _abi.TSS_BUF_DENSITY)
    elapsed = time.perf_counter() - t0
    still_busy = not other.query()
    other.synchronize()
    assert c["steps"] == 5 and d["id"].shape[0] == sc.n_low and dens.shape[0] == sc.n_low
    assert still_busy, f"the solver's queries waited for an unrelated stream ({elapsed:.3f} s)"


def test_steps_on_different_streams_run_in_order():
    import torch
    sc = scenes.dam_break_small(16, 32, seed=4)
    sc.config.roi[:] = [0.3, -np.inf, np.inf, np.inf]
    ref = Solver.from_scene(sc)
    ref.step(12)
    ref.sync()
    sol = Solver.from_scene(sc)
    streams = [torch.cuda.Stream(), torch.cuda.Stream(), None]
    for k in range(12):
        s = streams[k % 3]
        sol.step(1, stream=s.cuda_stream if s is not None else None)
    sol.sync()
    for scale in (_abi.TSS_SCALE_LOW, _abi.TSS_SCALE_HIGH):
        a, b = ref.download(scale), sol.download(scale)
        assert a["id"].shape[0] > 0
        for k in ("id", "pos", "vel", "state"):
            assert np.array_equal(a[k], b[k]), (scale, k)


@pytest.mark.parametrize("arith", ["exact", "fast"])
def test_branched_step_graph_equals_sequential(arith):
    """Outside profiling a step graph runs the two grid builds and the two density
    passes as parallel branches; with profiling on it runs every stage in order.
    Both must give the same state, bit for bit (a batch too: its pool kernels take
    the same branches)."""
    from twoscalesplit_gb300.solver import Batch
    sc = scenes.dam_break_small(24, 48, seed=9)
    sc.config.roi[:] = [0.3, -np.inf, np.inf, np.inf]
    seq, par = Solver.from_scene(sc), Solver.from_scene(sc)
    for sol in (seq, par):
        sol.set_arith(arith)
    seq.profile(True)
    seq.step(40)
    par.step(40)
    seq.sync()
    par.sync()
    assert par.counts()["n_high"] > 0
    for scale in (_abi.TSS_SCALE_LOW, _abi.TSS_SCALE_HIGH):
        a, b = seq.download(scale), par.download(scale)
        for k in ("id", "pos", "vel", "state", "dens", "pres"):
            assert np.array_equal(a[k], b[k]), (scale, k)
    scs = [scenes.dam_break_small(12 + 4 * k, 24, seed=k) for k in range(3)]
    bs, bp = Batch(scs), Batch(scs)
    for bb in (bs, bp):
        bb.set_arith(arith)
    bs.profile(True)
    bs.step(30)
    bp.step(30)
    for k in range(len(scs)):
        for scale in (_abi.TSS_SCALE_LOW, _abi.TSS_SCALE_HIGH):
            x, y = bs.download_scene(k, scale), bp.download_scene(k, scale)
            for name in ("id", "pos", "vel", "state"):
                assert np.array_equal(x[name], y[name]), (k, scale, name)
