"""Launch shapes, the autotuner and the step-bucket graphs: none of them may change a
result.  Every gather walks its list with a grid-stride loop over a device-side
count, so any block size and grid gives the same sums in the same order; the step
graphs of 2, 4 and 8 steps replay the same kernels as the one-step graph."""
import itertools
import math

import numpy as np
import pytest

from twoscalesplit_gb300 import scenes
from twoscalesplit_gb300._abi import GATHER_NAMES, TSS_SCALE_HIGH, TSS_SCALE_LOW, TssError
from twoscalesplit_gb300.solver import Batch, Solver

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from twoscalesplit_gb300 import build
    build.build()


def _scene(seed=3, relax=4):
    sc = scenes.dam_break_small(24, 40, seed=seed, relax_iters=relax)
    sc.config.roi[:] = [0.2, -math.inf, math.inf, math.inf]
    return sc


def _state(sol):
    return [sol.download(s) for s in (TSS_SCALE_LOW, TSS_SCALE_HIGH)]


def _assert_same(a, b):
    for sa, sb in zip(a, b):
        for name in ("id", "pos", "vel", "state"):
            assert np.array_equal(sa[name], sb[name]), name


def _shape(threads, persistent, per_warp=False):
    return {g: {"threads": threads, "persistent": persistent, "per_warp": per_warp} for g in GATHER_NAMES}


def test_default_shape_is_the_reference_block_size():
    sol = Solver.from_scene(_scene())
    assert sol.launch == _shape(256, False)


@pytest.mark.parametrize("threads,persistent,per_warp",
                         list(itertools.product([64, 128, 256], [False, True], [False, True])))
def test_every_shape_gives_the_same_steps(threads, persistent, per_warp):
    sc = _scene()
    ref = Solver.from_scene(sc)
    ref.step(60)
    sol = Solver.from_scene(sc)
    sol.set_launch(_shape(threads, persistent, per_warp))
    sol.step(60)
    sol.sync()
    assert sol.counts()["n_high"] > 0
    _assert_same(_state(ref), _state(sol))


@pytest.mark.parametrize("threads,persistent,per_warp", [(64, True, True), (128, False, False), (256, True, True)])
def test_every_shape_gives_the_same_steps_in_the_tolerance_arithmetic(threads, persistent, per_warp):
    sc = _scene()
    ref = Solver.from_scene(sc)
    ref.set_arith("fast")
    ref.step(60)
    sol = Solver.from_scene(sc)
    sol.set_arith("fast")
    sol.set_launch(_shape(threads, persistent, per_warp))
    sol.step(60)
    sol.sync()
    assert sol.counts()["n_high"] > 0
    _assert_same(_state(ref), _state(sol))


def test_shape_of_a_batch_does_not_change_its_scenes():
    scs = [_scene(seed=s, relax=0) for s in (5, 6, 7)]
    a, b = Batch(scs), Batch(scs)
    mixed = {g: {"threads": t, "persistent": p, "per_warp": w}
             for g, t, p, w in zip(GATHER_NAMES, (64, 128, 256, 64), (True, False, True, False),
                                   (True, True, False, True))}
    b.set_launch(mixed)
    a.step(50)
    b.step(50)
    for k in range(len(scs)):
        for scale in (TSS_SCALE_LOW, TSS_SCALE_HIGH):
            x, y = a.download_scene(k, scale), b.download_scene(k, scale)
            for name in ("id", "pos", "vel", "state"):
                assert np.array_equal(x[name], y[name]), (k, scale, name)


def test_autotune_installs_a_valid_shape_and_keeps_the_trajectory():
    sc = _scene(seed=11)
    tuned = Solver.from_scene(sc)
    shape, taken = tuned.autotune(steps_per_trial=2)
    assert taken == 10 * 3
    assert tuned.launch == shape
    for g in GATHER_NAMES:
        assert shape[g]["threads"] in (64, 128, 256)
    tuned.step(7)
    ref = Solver.from_scene(sc)
    ref.step(taken + 7)
    assert tuned.counts()["steps"] == ref.counts()["steps"] == taken + 7
    _assert_same(_state(ref), _state(tuned))


def test_invalid_shape_is_rejected_and_the_old_one_kept():
    sol = Solver.from_scene(_scene())
    with pytest.raises(TssError):
        sol.set_launch(_shape(96, False))
    assert sol.launch == _shape(256, False)


def test_step_buckets_equal_single_steps():
    sc = _scene(seed=9)
    one = Solver.from_scene(sc)
    for _ in range(29):
        one.step(1)
    many = Solver.from_scene(sc)
    many.step(13)   # 8 + 4 + 1
    many.step(16)   # 8 + 8
    assert many.counts()["steps"] == 29
    _assert_same(_state(one), _state(many))


def test_read_positions_equals_download_and_refuses_pageable_memory():
    import torch
    sc = _scene(seed=13, relax=0)
    sol = Solver.from_scene(sc)
    sol.step(25)
    n_high = sol.counts()["n_high"]
    assert n_high > 0
    low = torch.zeros((sc.n_low, 2), dtype=torch.float32).pin_memory()
    high = torch.zeros((sc.cap_high, 2), dtype=torch.float32).pin_memory()
    counts = torch.zeros(2, dtype=torch.int32).pin_memory()
    stream = torch.cuda.current_stream().cuda_stream
    sol.read_positions(low, high, counts, stream=stream)
    torch.cuda.synchronize()
    assert counts.tolist() == [sc.n_low, n_high]
    assert np.array_equal(low.numpy(), sol.download(TSS_SCALE_LOW)["pos"])
    assert np.array_equal(high.numpy()[:n_high], sol.download(TSS_SCALE_HIGH)["pos"])
    short = torch.zeros((3, 2), dtype=torch.float32).pin_memory()  # entries past the capacity are not written
    sol.read_positions(short, high, counts, stream=stream)
    torch.cuda.synchronize()
    assert np.array_equal(short.numpy(), low.numpy()[:3])
    # a destination 8 bytes past a 16-byte boundary
    big = torch.zeros((sc.n_low + 1, 2), dtype=torch.float32).pin_memory()
    shifted = big[1:]
    assert shifted.data_ptr() % 16 == 8
    sol.read_positions(shifted, high, counts, stream=stream)
    torch.cuda.synchronize()
    assert np.array_equal(shifted.numpy(), low.numpy()) and not big[0].any()
    with pytest.raises(TssError):
        sol.read_positions(torch.zeros((sc.n_low, 2), dtype=torch.float32), high, counts, stream=stream)


@pytest.mark.parametrize("relax", [0, 4])
def test_one_particle_per_warp_through_merges_and_the_guard(relax):
    """The moving region of interest with merging, the tether guard and (without
    Q1) the low-res cross term, one particle per warp against one per thread."""
    sc = scenes.adaptive_dam_break(40, 80, 0.01, roi_velocity=(20.0, 5.0), roi_start=(0.0, 0.05), steps=120,
                                   relax_iters=relax)
    ref = Solver.from_scene(sc)
    sol = Solver.from_scene(sc)
    sol.set_launch(_shape(128, False, True))
    ref.step(120)
    sol.step(120)
    c = sol.counts()
    assert c["total_split"] > 0 and c["total_removed"] > 0
    assert c == ref.counts()
    _assert_same(_state(ref), _state(sol))


def test_overlapped_read_back_gives_every_steps_positions():
    """tss_solver_read_positions_async, two host buffers in turn while the steps go
    on, against the ordered read-back of the same steps; a later call with larger
    capacities regrows the staging buffers."""
    import torch
    sc = _scene(seed=17, relax=0)
    stream = torch.cuda.current_stream().cuda_stream
    ref = Solver.from_scene(sc)
    want = []
    lo = torch.zeros((sc.n_low, 2), dtype=torch.float32).pin_memory()
    hi = torch.zeros((sc.cap_high, 2), dtype=torch.float32).pin_memory()
    cn = torch.zeros(2, dtype=torch.int32).pin_memory()
    for _ in range(30):
        ref.step(1, stream=stream)
        ref.read_positions(lo, hi, cn, stream=stream)
        torch.cuda.synchronize()
        want.append((lo.numpy().copy(), hi.numpy()[:cn[1]].copy(), cn.tolist()))
    sol = Solver.from_scene(sc)
    small = 7  # the first calls stage 7 high-res entries at most, later ones all of them
    bufs = [(torch.zeros((sc.n_low, 2), dtype=torch.float32).pin_memory(),
             torch.zeros((sc.cap_high, 2), dtype=torch.float32).pin_memory(),
             torch.zeros(2, dtype=torch.int32).pin_memory()) for _ in range(2)]
    tickets = [None, None]
    got = [None] * 30

    def collect(b, k):
        sol.read_wait(tickets[b])
        n = bufs[b][2].tolist()
        m = n[1] if k >= 10 else min(n[1], small)
        got[k] = (bufs[b][0].numpy().copy(), bufs[b][1].numpy()[:m].copy(), n)

    for k in range(30):
        b = k % 2
        if tickets[b] is not None:
            collect(b, k - 2)
        sol.step(1, stream=stream)
        high = bufs[b][1] if k >= 10 else bufs[b][1][:small]
        tickets[b] = sol.read_positions_async(bufs[b][0], high, bufs[b][2], stream=stream)
    for k in (28, 29):
        collect(k % 2, k)
    assert want[-1][2][1] > small
    for k in range(30):
        assert got[k][2] == want[k][2], k
        assert np.array_equal(got[k][0], want[k][0]), k
        m = len(got[k][1])
        assert np.array_equal(got[k][1], want[k][1][:m]), k
    with pytest.raises(TssError):
        sol.read_wait(tickets[1] + 1)  # not issued


def test_overlapped_read_back_of_a_batch():
    """A batch's list lengths are on the device only: its overlapped read-back goes
    by kernel for both lists and must equal the ordered one."""
    import torch
    scs = [_scene(seed=s, relax=0) for s in (21, 22)]
    stream = torch.cuda.current_stream().cuda_stream
    a, b = Batch(scs), Batch(scs)
    n_low = sum(sc.n_low for sc in scs)
    cap_h = sum(sc.cap_high for sc in scs)
    bufs = [(torch.zeros((n_low, 2), dtype=torch.float32).pin_memory(),
             torch.zeros((cap_h, 2), dtype=torch.float32).pin_memory(),
             torch.zeros(2, dtype=torch.int32).pin_memory()) for _ in range(2)]
    for k in range(12):
        a.step(1, stream=stream)
        b.step(1, stream=stream)
        a.read_positions(bufs[0][0], bufs[0][1], bufs[0][2], stream=stream)
        t = b.read_positions_async(bufs[1][0], bufs[1][1], bufs[1][2], stream=stream)
        b.read_wait(t)
        torch.cuda.synchronize()
        n = bufs[0][2].tolist()
        assert bufs[1][2].tolist() == n
        assert np.array_equal(bufs[0][0].numpy(), bufs[1][0].numpy())
        assert np.array_equal(bufs[0][1].numpy()[:n[1]], bufs[1][1].numpy()[:n[1]])
    assert n[1] > 0
