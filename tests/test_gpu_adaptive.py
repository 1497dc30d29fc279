"""The moving region of interest with merging (TSS_FLAG_MERGE): the GPU step must
equal the oracle's FP32 step bit for bit while particles split at the region's
leading edge and merge back at its trailing edge, and the mass
m * #(low state 0) + m/4 * #(high) must stay exactly what it was (m/4 is exact in
FP32, so the check is on counts: 4 * #(low state 0) + #(high) == 4 * N_low)."""
import numpy as np
import pytest

import oracle as O
from twoscalesplit_gb300 import scenes
from twoscalesplit_gb300._abi import TSS_SCALE_HIGH, TSS_SCALE_LOW
from twoscalesplit_gb300.solver import Solver

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from twoscalesplit_gb300 import build
    build.build()


@pytest.mark.parametrize("relax,q1", [(0, True), (4, False)])
def test_moving_roi_merge_matches_oracle_and_conserves_mass(relax, q1):
    sc = scenes.adaptive_dam_break(40, 80, 0.01, roi_velocity=(20.0, 5.0), roi_start=(0.0, 0.05), steps=240,
                                   relax_iters=relax)
    if q1:
        sc.config.flags |= 1  # the reference's high-res density term (TSS_FLAG_Q1_COMPAT)
    sol = Solver.from_scene(sc)
    orc = O.Oracle(sc, 32)
    n = sc.n_low
    splits = removed = 0
    for s in range(240):
        sol.step(1)
        orc.step()
        c = sol.counts()
        splits += c["n_split_last"]
        removed += c["n_removed_last"]
        if s % 20 == 19 or s == 239:
            for scale in (TSS_SCALE_LOW, TSS_SCALE_HIGH):
                d = sol.download(scale)
                st = orc.state(scale)
                assert np.array_equal(d["id"], st["id"]), (s, scale)
                assert np.array_equal(d["state"], st["state"]), (s, scale)
                assert np.array_equal(d["pos"], st["pos"].astype(np.float32)), (s, scale)
                assert np.array_equal(d["vel"], st["vel"].astype(np.float32)), (s, scale)
            low = sol.download(TSS_SCALE_LOW)
            assert 4 * int((low["state"] == 0).sum()) + c["n_high"] == 4 * n, s
            assert not (sol.download(TSS_SCALE_HIGH)["state"] == 2).any()
    sol.sync()
    assert splits > 0 and removed > 0 and removed % 4 == 0


def test_fixed_roi_without_merge_is_unchanged():
    # roi_velocity 0 and no merge flag: the reference's behaviour, children are never removed
    sc = scenes.dam_break_small(20, 40, seed=3, relax_iters=0)
    sol = Solver.from_scene(sc)
    orc = O.Oracle(sc, 32)
    for _ in range(60):
        sol.step(1)
        orc.step()
        assert sol.counts()["n_removed_last"] == 0
    for scale in (TSS_SCALE_LOW, TSS_SCALE_HIGH):
        d = sol.download(scale)
        st = orc.state(scale)
        assert np.array_equal(d["id"], st["id"])
        assert np.array_equal(d["pos"], st["pos"].astype(np.float32))


def test_tether_guard_matches_oracle_where_the_reference_divides_zero_by_zero():
    # a droplet scene whose children collapse onto their parent by step 5 (half its
    # usual time step): with the guard the GPU stays finite and equals the oracle
    sc = scenes.mixed_batch(47, seed=0)[46]
    sc.config.dt = np.float32(sc.config.dt * 0.5)
    sc.config.flags |= 0x4
    sol = Solver.from_scene(sc)
    orc = O.Oracle(sc, 32)
    for _ in range(8):
        sol.step(1)
        orc.step()
    sol.sync()
    for scale in (TSS_SCALE_LOW, TSS_SCALE_HIGH):
        d = sol.download(scale)
        st = orc.state(scale)
        assert np.isfinite(d["pos"]).all()
        assert np.array_equal(d["id"], st["id"])
        assert np.array_equal(d["pos"], st["pos"].astype(np.float32))
