"""Edge cases of the step and of pools on the GPU: empty and one-particle scenes,
scenes without walls, particles outside the domain (their cells clamp to the border
cells, WCSPHSolver.cu:265-289), and the pool calls' argument errors.  Every
trajectory is compared with the FP32 oracle bit for bit."""
import math

import numpy as np
import pytest

import oracle as O
from twoscalesplit_gb300 import scenes, serving
from twoscalesplit_gb300._abi import TSS_SCALE_HIGH, TSS_SCALE_LOW, TssError
from twoscalesplit_gb300.solver import Solver

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from twoscalesplit_gb300 import build
    build.build()


def _equal_oracle(sol, orc, where):
    for s in (TSS_SCALE_LOW, TSS_SCALE_HIGH):
        st = orc.state(s)
        d = sol.download(s)
        assert np.array_equal(d["id"], st["id"]), (where, s)
        assert np.array_equal(d["state"], st["state"]), (where, s)
        for k in ("pos", "vel"):
            assert np.array_equal(d[k], st[k].astype(np.float32)), (where, s, k)


def _run_both(sc, steps, check_every=5):
    sol = Solver.from_scene(sc)
    orc = O.Oracle(sc, 32)
    for k in range(steps):
        sol.step(1)
        orc.step()
        if k % check_every == check_every - 1:
            sol.sync()
            _equal_oracle(sol, orc, k)
    return sol, orc


def _small(seed=4, **kw):
    sc = scenes.dam_break_small(12, 20, seed=seed, relax_iters=4, **kw)
    sc.config.roi[:] = [0.2, -math.inf, math.inf, math.inf]
    return sc


def test_empty_scene_steps_without_error():
    sc = _small()
    sc.low_pos = np.zeros((0, 2), np.float32)
    sc.low_vel = np.zeros((0, 2), np.float32)
    sol = Solver.from_scene(sc)
    sol.step(7)
    sol.sync()
    c = sol.counts()
    assert c["n_low"] == 0 and c["n_high"] == 0 and c["steps"] == 7


def test_scene_without_walls_matches_oracle():
    sc = _small(seed=5)
    sc.wall_pos = np.zeros((0, 2), np.float32)
    sol, _ = _run_both(sc, 30)
    assert sol.counts()["n_high"] > 0


def test_single_particle_matches_oracle():
    sc = _small(seed=6)
    sc.low_pos = np.array([[0.35, 0.5]], np.float32)  # inside the ROI: it splits
    sc.low_vel = np.array([[0.1, 0.0]], np.float32)
    sol, _ = _run_both(sc, 12, check_every=3)
    assert sol.counts()["n_high"] == 4


def test_particles_outside_the_domain_match_oracle():
    sc = _small(seed=7)
    pos = sc.low_pos.copy()
    # clear of the wall layers (within r of a wall particle the wall weight has
    # 1/d^2, and a particle on one makes the reference's arithmetic non-finite)
    pos[:6] = [[-0.15 - 0.02 * k, 0.3 + 0.02 * k] for k in range(6)]   # left of the domain, interacting
    pos[6:12] = [[0.3 + 0.02 * k, 1.2 + 0.01 * k] for k in range(6)]   # above it, inside the ROI: they split
    pos[12:16] = [[1.3, 0.2], [-0.2, -0.3], [0.5, 1.5], [2.0, 2.0]]
    sc.low_pos = pos
    _run_both(sc, 20)


def test_pool_argument_errors_and_one_particle_scene():
    sc = _small(seed=8)
    one = _small(seed=9)
    one.low_pos = np.array([[0.6, 0.5]], np.float32)
    one.low_vel = np.zeros((1, 2), np.float32)
    cfg = serving.pool_config(low_slots=1024, wall_particles=4 * sc.n_wall, max_scenes=4, relax_iters=4)
    pool = serving.Pool(cfg)
    a = pool.admit(sc)
    b = pool.admit(one)
    assert a is not None and b is not None and a != b
    with pytest.raises(TssError):
        pool.extract(b)          # the scene has not taken a step
    with pytest.raises(TssError):
        pool.retire(57)          # no such scene
    pool.step(6)
    pool.sync()
    alone = Solver.from_scene(one)
    alone.step(6)
    got = pool.extract(b)
    for s, scale in ((0, TSS_SCALE_LOW), (1, TSS_SCALE_HIGH)):
        d = alone.download(scale)
        order = np.argsort(got[s]["id"], kind="stable")
        assert np.array_equal(got[s]["id"][order], d["id"])
        for k in ("pos", "vel", "state"):
            assert np.array_equal(got[s][k][order], d[k]), (s, k)
    # 256-slot pages: the two scenes hold two of the four pages, so a 700-particle
    # scene (three pages) fits the pool but not now
    mid = scenes.dam_break_small(20, 35, seed=10, relax_iters=4)
    assert not pool.can_admit(mid)
    assert pool.admit(mid) is None
    pool.retire(a)
    pool.retire(b)
    with pytest.raises(TssError):
        pool.retire(b)           # already retired
    assert pool.can_admit(mid)
    too_big = scenes.dam_break_small(40, 40, seed=11, relax_iters=4)
    with pytest.raises(TssError):
        pool.can_admit(too_big)  # more low-res particles than the pool has slots: never fits
