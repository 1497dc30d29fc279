"""Pools and the serving loop: a scene admitted into a pool, advanced together with
whatever else is admitted, placed in pages that other scenes used before, and
extracted at its horizon must give the state it gives alone, bit for bit (the
per-scene sums and orders do not depend on the other scenes or on placement);
the tolerance for these FP32 arrays is therefore exact equality, tighter than the
1e-5 relative bound.  The serving loop must admit by free pool memory, first come
first served, and reject what can never fit."""
import math

import numpy as np
import pytest

from twoscalesplit_gb300 import scenes
from twoscalesplit_gb300._abi import TSS_INVALID_ARG, TSS_OK, TSS_SCALE_HIGH, TSS_SCALE_LOW
from twoscalesplit_gb300.serving import Pool, Request, Server, footprint, pool_config
from twoscalesplit_gb300.solver import Solver

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from twoscalesplit_gb300 import build
    build.build()


def _scenes(relax, n=4, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        if relax:
            sc = scenes.dam_break_small(10 + 4 * k, 20 + 3 * k, seed=seed + k, relax_iters=relax)
            sc.config.roi[:] = [0.2 + 0.05 * k, -math.inf, math.inf, math.inf]
        else:
            sc = scenes.mixed_scene(rng, n_min=1500, n_max=6000)
        out.append(sc)
    return out


def _by_id(d):
    o = np.argsort(d["id"], kind="stable")
    return {k: v[o] for k, v in d.items()}


def _alone(sc, steps):
    sol = Solver.from_scene(sc)
    sol.step(steps)
    sol.sync()
    return [sol.download(TSS_SCALE_LOW), sol.download(TSS_SCALE_HIGH)]


def _assert_same(mine, theirs, tag):
    for scale in (0, 1):
        a, b = _by_id(mine[scale]), _by_id(theirs[scale])
        assert a["id"].shape == b["id"].shape, (tag, scale)
        assert np.array_equal(a["id"], b["id"]), (tag, scale)
        for name in ("pos", "vel", "state", "dens", "pres"):
            assert np.array_equal(a[name], b[name]), (tag, scale, name)


@pytest.mark.parametrize("relax", [0, 4])
def test_pool_admit_retire_extract_equal_alone(relax):
    A, B, C, D = _scenes(relax)
    total = sum(footprint(s)["low_slots"] for s in (A, B, C, D))
    cfg = pool_config(low_slots=total, low_cells=sum(footprint(s)["low_cells"] for s in (A, B, C, D)),
                      high_cells=sum(footprint(s)["high_cells"] for s in (A, B, C, D)),
                      wall_particles=sum(footprint(s)["wall_particles"] for s in (A, B, C, D)), max_scenes=8,
                      relax_iters=relax)
    pool = Pool(cfg)
    a = pool.admit(A)
    pool.step(5)
    b = pool.admit(B)
    pool.step(7)
    got_a = pool.extract(a)                  # A: 12 steps
    pool.retire(a)
    c = pool.admit(C)                        # placed in A's pages, before the next step
    d = pool.admit(D)
    pool.step(10)
    got_b = pool.extract(b)                  # B: 17 steps
    pool.retire(b)
    pool.step(3)
    got_c = pool.extract(c)                  # C: 13 steps
    got_d = pool.extract(d)
    pool.sync()
    assert pool.counts()["error_bits"] == 0
    _assert_same(_alone(A, 12), got_a, "A")
    _assert_same(_alone(B, 17), got_b, "B")
    _assert_same(_alone(C, 13), got_c, "C")
    _assert_same(_alone(D, 13), got_d, "D")
    assert sum(x[1]["id"].shape[0] for x in (got_a, got_b, got_c)) > 0  # splits happened


@pytest.mark.parametrize("arith", ["exact", "fast"])
def test_pool_whose_neighbour_list_columns_pass_2_31_entries(arith):
    """A pool sized for 300M high-res particles: entry c of a particle's neighbour
    list lies c x 300M entries into the list array, past 2^31 from c = 8 on, so a
    32-bit index would wrap into other arrays.  The scene must still give its state
    alone, bit for bit, in either arithmetic (about 33 GB of device memory)."""
    rng = np.random.default_rng(5)
    sc = scenes.mixed_scene(rng, n_min=4000, n_max=6000)
    f = footprint(sc)
    cfg = pool_config(low_slots=f["low_slots"], high_particles=300_000_000, low_cells=f["low_cells"],
                      high_cells=f["high_cells"], wall_particles=f["wall_particles"], max_scenes=2)
    assert 8 * cfg.high_particles > 2**31
    pool = Pool(cfg)
    pool.set_arith(arith)
    sid = pool.admit(sc)
    pool.step(40)
    got = pool.extract(sid)
    pool.sync()
    assert pool.counts()["error_bits"] == 0
    sol = Solver.from_scene(sc)
    sol.set_arith(arith)
    sol.step(40)
    sol.sync()
    _assert_same([sol.download(TSS_SCALE_LOW), sol.download(TSS_SCALE_HIGH)], got, arith)
    assert got[1]["id"].shape[0] > 0  # splits happened: the high-res lists were in use
    pool.close()


def test_pool_download_scene_matches_extract_and_frees_pages():
    scs = _scenes(0, n=3, seed=5)
    fp = [footprint(s) for s in scs]
    cfg = pool_config(low_slots=sum(f["low_slots"] for f in fp), low_cells=sum(f["low_cells"] for f in fp),
                      high_cells=sum(f["high_cells"] for f in fp),
                      wall_particles=sum(f["wall_particles"] for f in fp), max_scenes=4)
    pool = Pool(cfg)
    free0 = pool.free()
    ids = [pool.admit(s) for s in scs]
    assert None not in ids
    assert pool.admit(scs[0]) is None  # full: TSS_CAPACITY, nothing admitted
    pool.step(20)
    for sid in ids:
        ex = pool.extract(sid)
        for scale in (0, 1):
            dl = pool.download_scene(sid, scale)
            assert np.array_equal(dl["id"], ex[scale]["id"])
            assert np.array_equal(dl["pos"], ex[scale]["pos"])
    for sid in ids:
        pool.retire(sid)
    assert pool.free() == free0
    pool.step(1)  # an empty step after the retirements
    pool.sync()
    assert pool.counts()["n_low"] == 0 and pool.counts()["n_high"] == 0


def test_server_results_equal_alone_and_admission_waits_for_memory():
    scs = _scenes(0, n=6, seed=11)
    fp = [footprint(s) for s in scs]
    # room for the two largest scenes at a time, not three
    big = sorted(fp, key=lambda f: f["low_slots"])[-2:]
    cfg = pool_config(low_slots=sum(f["low_slots"] for f in big), low_cells=sum(f["low_cells"] for f in big) + 64,
                      high_cells=max(f["high_cells"] for f in fp) * 2 + 64,
                      wall_particles=max(f["wall_particles"] for f in fp) * 2 + 64, max_scenes=16)
    too_big = scenes.mixed_scene(np.random.default_rng(99), n_min=200000, n_max=200001)
    horizons = [23, 41, 17, 30, 9, 35]
    reqs = [Request(sc, h, 0.002 * k, want_result=True) for k, (sc, h) in enumerate(zip(scs, horizons))]
    reqs.insert(3, Request(too_big, 10, 0.004, want_result=False))
    sv = Server(cfg, max_steps_per_launch=6, max_in_flight=2, staging_bytes=64 << 20)
    stats, summ, res = sv.run(reqs)
    assert stats[3]["status"] == TSS_INVALID_ARG          # can never fit: rejected
    served = [k for k in range(len(reqs)) if k != 3]
    for k in served:
        s = stats[k]
        assert s["status"] == TSS_OK, (k, s)
        assert s["arrival_s"] <= s["admit_s"] + 1e-3 and s["admit_s"] <= s["done_s"] + 1e-3
        _assert_same(_alone(reqs[k].scene, reqs[k].horizon), res[k], f"request {k}")
        assert s["n_low"] == reqs[k].scene.n_low
    assert summ["served"] == len(served)
    assert 1 <= summ["max_active"] < len(served)
    assert summ["scene_steps"] == sum(reqs[k].horizon for k in served)
    # memory-bound admission: some request waited for an earlier one to finish
    done_first = min(stats[k]["done_s"] for k in served)
    assert any(stats[k]["admit_s"] >= done_first - 1e-3 for k in served)


def test_pool_moving_roi_and_merge_start_at_each_scenes_own_step():
    # scenes with a translating region of interest and merging, admitted at different
    # pool steps: each one's region starts moving at its own first step, so each
    # equals the same scene run alone
    A = scenes.adaptive_dam_break(30, 60, 0.4 / 30, roi_velocity=(14.0, 3.0), roi_start=(0.0, 0.05), steps=60)
    B = scenes.adaptive_dam_break(24, 40, 0.4 / 24, roi_velocity=(-9.0, 2.0), roi_start=(0.25, 0.1), steps=60,
                                  seed=4)
    fa, fb = footprint(A), footprint(B)
    cfg = pool_config(low_slots=fa["low_slots"] + fb["low_slots"], low_cells=fa["low_cells"] + fb["low_cells"],
                      high_cells=fa["high_cells"] + fb["high_cells"],
                      wall_particles=fa["wall_particles"] + fb["wall_particles"], max_scenes=4)
    pool = Pool(cfg)
    a = pool.admit(A)
    pool.step(17)
    b = pool.admit(B)
    pool.step(40)
    got_a, got_b = pool.extract(a), pool.extract(b)
    pool.sync()
    for got in (got_a, got_b):
        got[1] = {k: v[got[1]["state"] != 2] for k, v in got[1].items()}  # removed in the last step
    _assert_same(_alone(A, 57), got_a, "A")
    _assert_same(_alone(B, 40), got_b, "B")
    c = pool.counts()
    assert c["total_split"] > 0 and c["total_removed"] > 0
