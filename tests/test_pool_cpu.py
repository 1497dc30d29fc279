"""Host-side logic of scene pools and the serving loop, on the CPU: the page
allocator (compiled C++ against its header), pool sizing and scene footprints from
the library's host-only calls, and the latency/FIFO helpers of the serving bench."""
import ctypes
import math
import os
import subprocess

import numpy as np
import pytest

from twoscalesplit_gb300 import _abi, build, scenes
from twoscalesplit_gb300.serving import (fifo_schedule, footprint, latency_summary, pool_bytes, pool_config,
                                         pool_config_for_budget)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def _lib():
    build.build()


def test_extent_allocator(tmp_path):
    exe = str(tmp_path / "extent_test")
    subprocess.check_call(["g++", "-std=c++17", "-O1", os.path.join(ROOT, "tests", "cpp", "extent_test.cpp"), "-o", exe])
    assert subprocess.check_output([exe], timeout=120).decode().strip() == "ok"


def test_scene_footprint_is_rounded_to_pages():
    sc = scenes.mixed_scene(np.random.default_rng(3), n_min=3000, n_max=3001)
    f = footprint(sc)
    cells_low = sc.config.dims_low[0] * sc.config.dims_low[1]
    cells_high = sc.config.dims_high[0] * sc.config.dims_high[1]
    assert f["low_slots"] == -(-sc.n_low // _abi.TSS_POOL_SLOT_PAGE) * _abi.TSS_POOL_SLOT_PAGE
    assert f["high_particles"] == 4 * sc.n_low
    assert f["low_cells"] == -(-(cells_low + 1) // _abi.TSS_POOL_CELL_PAGE) * _abi.TSS_POOL_CELL_PAGE
    assert f["high_cells"] == -(-cells_high // _abi.TSS_POOL_CELL_PAGE) * _abi.TSS_POOL_CELL_PAGE
    assert f["wall_particles"] == -(-sc.n_wall // _abi.TSS_POOL_WALL_PAGE) * _abi.TSS_POOL_WALL_PAGE


@pytest.mark.parametrize("r_low,r_high,ok", [(2.0 ** -40, 2.0 ** -41, False), (2.0 ** -39, 2.0 ** -40, True),
                                              (2.0 ** 40, 2.0 ** 39, True), (2.0 ** 41, 2.0 ** 40, False),
                                              (0.01, 0.0, False), (0.01, math.inf, False)])
def test_support_radii_outside_the_exact_division_range_are_refused(r_low, r_high, ok):
    """The pair kernels divide by the radii through their reciprocal splits, which is
    exact for radii in [2^-40, 2^40]; the configuration check refuses the rest."""
    sc = scenes.mixed_scene(np.random.default_rng(3), n_min=3000, n_max=3001)
    sc.config.r_low, sc.config.r_high = r_low, r_high
    if ok:
        footprint(sc)
    else:
        with pytest.raises(_abi.TssError):
            footprint(sc)


def test_pool_bytes_grow_with_capacity_and_budget_fits():
    b1 = pool_bytes(pool_config(1 << 16))
    b2 = pool_bytes(pool_config(1 << 17))
    assert b2 > b1 > 0
    for budget in (64 << 20, 3 << 30, 150 << 30):
        c = pool_config_for_budget(budget, 1.2, 0.3)
        b = pool_bytes(c)
        assert b <= budget
        if budget < (100 << 30):  # below the int32 limits the budget is used up to ~0.2 %
            assert b >= 0.99 * budget
        assert c.low_slots % _abi.TSS_POOL_SLOT_PAGE == 0
        assert 4 * c.low_slots < 2 ** 31 and c.high_cells < 2 ** 31


def test_invalid_pool_configs_are_refused():
    lib = _abi.load_library()
    b = ctypes.c_size_t(0)
    bad = pool_config(1 << 16, max_scenes=0)
    assert lib.tss_pool_bytes(ctypes.byref(bad), ctypes.byref(b)) == _abi.TSS_INVALID_ARG
    bad = pool_config(1 << 30)  # 4 x slots would overflow the int32 slot space
    assert lib.tss_pool_bytes(ctypes.byref(bad), ctypes.byref(b)) == _abi.TSS_INVALID_ARG


def test_fifo_schedule_and_latency_summary():
    arr = [0.0, 0.5, 0.6, 10.0]
    svc = [1.0, 1.0, 1.0, 0.5]
    done = fifo_schedule(arr, svc)
    assert np.allclose(done, [1.0, 2.0, 3.0, 10.5])
    stats = [{"arrival_s": a, "done_s": d, "status": _abi.TSS_OK} for a, d in zip(arr, done)]
    stats.append({"arrival_s": 0.0, "done_s": -1.0, "status": _abi.TSS_INVALID_ARG})
    s = latency_summary(stats)
    assert s["served"] == 4
    assert math.isclose(s["p50_s"], np.percentile([1.0, 1.5, 2.4, 0.5], 50))


def test_serving_trace_distributions():
    tr = scenes.serving_trace(40, rate_per_s=100.0, seed=1, n_min=1000, n_max=20000, h_min=200, h_max=5000)
    arr = [t for _, _, t in tr]
    assert arr == sorted(arr) and arr[0] > 0
    assert all(200 <= h <= 5000 for _, h, _ in tr)
    n = np.array([sc.n_low for sc, _, _ in tr])
    assert n.min() >= 500 and n.max() <= 30000
    assert scenes.mean_work(1000, 500000, 200, 5000) == pytest.approx((499000 / math.log(500)) * 2600)


def test_launch_cache_roundtrip(tmp_path):
    from twoscalesplit_gb300 import tuning

    class FakeSolver:
        def __init__(self):
            self.set = None
            self.tuned = 0

        def autotune(self, steps_per_trial):
            self.tuned += 1
            return {"force_low": {"threads": 128, "persistent": False}}, 6 * (steps_per_trial + 1)

        def set_launch(self, shape):
            self.set = shape

    path = str(tmp_path / "launch.json")
    assert tuning.workload_class("single", 999698) == "single/2^20"
    s = FakeSolver()
    shape, taken = tuning.tuned_launch(s, "single", 1000, path=path, steps_per_trial=2)
    assert taken == 18 and s.tuned == 1 and s.set is None
    s2 = FakeSolver()
    shape2, taken2 = tuning.tuned_launch(s2, "single", 1100, path=path)
    assert taken2 == 0 and s2.tuned == 0 and s2.set == shape == shape2
    s3 = FakeSolver()
    tuning.tuned_launch(s3, "batch", 1000, path=path)
    assert s3.tuned == 1 and len(tuning.load(path)) == 2
