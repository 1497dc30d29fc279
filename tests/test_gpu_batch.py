"""Batches of independent scenes: each scene advanced inside a batch must give the
same result as the same scene advanced alone, bit for bit (the per-scene sums and
orders do not depend on the other scenes)."""
import math

import numpy as np
import pytest

import oracle as O
from twoscalesplit_gb300 import scenes
from twoscalesplit_gb300._abi import TSS_SCALE_HIGH, TSS_SCALE_LOW
from twoscalesplit_gb300.solver import Batch, Solver

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from twoscalesplit_gb300 import build
    build.build()


def _mixed_scenes(relax):
    out = []
    for k, (nx, ny, seed) in enumerate([(16, 32, 1), (10, 24, 2), (24, 40, 3), (12, 12, 4)]):
        sc = scenes.dam_break_small(nx, ny, seed=seed, relax_iters=relax, calibrate_mass=(k % 2 == 0))
        sc.config.roi[:] = [0.25 + 0.05 * k, -math.inf, math.inf, math.inf]
        if k == 3:
            sc.config.flags = 0  # a scene without the Q1 compatibility switch
        out.append(sc)
    return out


@pytest.mark.parametrize("relax,arith", [(0, "exact"), (4, "exact"), (0, "fast"), (4, "fast")])
def test_batch_scenes_equal_alone(relax, arith):
    """in either arithmetic: the tolerance arithmetic's pair terms are rounded the
    same way in the batched and the single-scene kernel forms"""
    scs = _mixed_scenes(relax)
    batch = Batch(scs)
    alone = [Solver.from_scene(sc) for sc in scs]
    for s in [batch] + alone:
        s.set_arith(arith)
    steps = 90
    batch.step(steps)
    for a in alone:
        a.step(steps)
    batch.sync()
    lo, hi = batch.scene_counts()
    assert hi.sum() > 0
    for k, a in enumerate(alone):
        for scale in (TSS_SCALE_LOW, TSS_SCALE_HIGH):
            mine = a.download(scale)
            theirs = batch.download_scene(k, scale)
            assert np.array_equal(mine["id"], theirs["id"]), (k, scale)
            for name in ("pos", "vel", "state"):
                assert np.array_equal(mine[name], theirs[name]), (k, scale, name)
        assert hi[k] == a.counts()["n_high"]


def test_batch_of_one_equals_plain_solver_and_oracle():
    sc = scenes.dam_break_small(16, 32, seed=8, relax_iters=4)
    sc.config.roi[:] = [0.3, -math.inf, math.inf, math.inf]
    b = Batch([sc])
    orc = O.Oracle(sc, 32)
    b.step(60)
    for _ in range(60):
        orc.step()
    for scale in (TSS_SCALE_LOW, TSS_SCALE_HIGH):
        d = b.download(scale)
        st = orc.state(scale)
        assert np.array_equal(d["id"], st["id"])
        assert np.array_equal(d["pos"], st["pos"].astype(np.float32))
