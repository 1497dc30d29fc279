"""CPU tests of the oracle: pinned against the reference's own kernels.

The reference has no tests or golden vectors.  The fixtures in tests/golden were
produced by the reference's kernel source compiled for the CPU
(tests/golden/make_golden.py); where that build is present (the machine with the
reference checkout) the oracle is also compared with it step by step.
"""
import math
import os

import numpy as np
import pytest

import oracle as O
from tests._golden import dense_to_start_end, fixture_input, scene_from_fixture
from twoscalesplit_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
REF_ROI = [0.5, -math.inf, math.inf, math.inf]


# --------------------------------------------------------------------------- grid
GRID_CASES = ["random", "one_cell", "single", "empty", "ragged", "outside", "edges"]


@pytest.mark.parametrize("case", GRID_CASES)
def test_grid_matches_reference_fixture(case):
    g = np.load(os.path.join(GOLDEN, "grid_cases.npz"))
    pos = g[case + "_pos"]
    ids = np.arange(pos.shape[0], dtype=np.int32)
    order, off = O.grid(pos, ids, g["origin"], float(g["cell"]), g["dims"])
    # ids ascending -> the reference's stable sort by cell is the (cell, id) order
    assert np.array_equal(ids[order], g[case + "_sorted_id"])
    s, e = dense_to_start_end(off)
    assert np.array_equal(s, g[case + "_cell_start"])
    assert np.array_equal(e, g[case + "_cell_end"])
    assert off[0] == 0 and off[-1] == pos.shape[0]


def test_grid_unsorted_input_is_cell_multiset_equal():
    """With an arbitrary list order the reference's order inside a cell follows the
    list; ours is by id.  Per-cell id multisets must agree."""
    g = np.load(os.path.join(GOLDEN, "grid_cases.npz"))
    pos = g["random_pos"]
    rng = np.random.default_rng(3)
    ids = rng.permutation(pos.shape[0]).astype(np.int32)
    order, off = O.grid(pos[ids], ids, g["origin"], float(g["cell"]), g["dims"])
    ref_sorted = g["random_sorted_id"]
    ours = ids[order]
    for c in range(off.shape[0] - 1):
        a, b = off[c], off[c + 1]
        assert sorted(ours[a:b]) == sorted(ref_sorted[a:b])
        assert np.all(np.diff(ours[a:b]) > 0)


# --------------------------------------------------------------------------- step
@pytest.mark.parametrize("fname", ["step_q1.npz", "step_q1_relax.npz", "step_developed_51k.npz"])
def test_step_matches_reference_fixture_bit_exact(fname):
    g = np.load(os.path.join(GOLDEN, fname))
    sc = scene_from_fixture(g)
    orc = O.Oracle(sc, 32)
    for s, tag in ((0, "low"), (1, "high")):
        st = fixture_input(g, tag)
        orc.set_scale(s, st["id"], st["pos"], st["vel"], st["state"], st["dens"], st["pres"])
    orc.set_fresh(g["fresh"])
    assert orc.step() == 0
    for s, tag in ((0, "low"), (1, "high")):
        sid = orc.get(s, "sorted_id")
        assert np.array_equal(sid, g[f"out_{tag}_sorted_id"]), tag
        cs, ce = dense_to_start_end(orc.get(s, "cell_off"))
        assert np.array_equal(cs, g[f"out_{tag}_cell_start"]), tag
        assert np.array_equal(ce, g[f"out_{tag}_cell_end"]), tag
        for name in ("dens", "pres"):
            assert np.array_equal(orc.get(s, name).astype(np.float32), g[f"out_{tag}_{name}"][sid]), (tag, name)
        acc = orc.get(s, "acc").astype(np.float32)
        assert np.array_equal(acc, g[f"out_{tag}_acc"].reshape(-1, 2)[sid]), (tag, "acc")
        st = orc.state(s)
        ids = st["id"]
        assert sorted(ids) == sorted(g[f"out_{tag}_ids"]), tag
        for name in ("pos", "vel"):
            assert np.array_equal(st[name].astype(np.float32), g[f"out_{tag}_{name}"].reshape(-1, 2)[ids]), \
                (tag, name)
        assert np.array_equal(st["state"], g[f"out_{tag}_state"][ids]), tag
    assert np.array_equal(orc.get(0, "split"), g["out_split"])
    counts = g["out_counts"]
    assert orc.get(1, "id").shape[0] == counts[1]
    assert int((orc.get(0, "state") == 1).sum()) == counts[2]


@pytest.mark.skipif(not O.refcpu_available(), reason="needs the reference checkout")
@pytest.mark.parametrize("relax", [0, 4])
def test_oracle_tracks_reference_kernels_many_steps(relax):
    # the literal mass (1000 dx^2) starts violently, so splits at x > 0.5 come early
    sc = scenes.dam_break_small(16, 32, seed=11, relax_iters=relax, calibrate_mass=False)
    sc.config.roi[:] = REF_ROI
    orc = O.Oracle(sc, 32)
    ref = O.RefCPU(sc)
    seen_high = False
    for step in range(150):
        orc.step()
        ref.step()
        for s in (0, 1):
            st = orc.state(s)
            ids = st["id"]
            if ids.size == 0:
                continue
            seen_high |= s == 1
            for name in ("pos", "vel"):
                assert np.array_equal(st[name].astype(np.float32), ref.get(s, name).reshape(-1, 2)[ids]), \
                    (step, s, name)
            assert np.array_equal(st["state"], ref.get(s, "state")[ids])
            sid = orc.get(s, "sorted_id")
            assert np.array_equal(orc.get(s, "dens").astype(np.float32), ref.get(s, "dens")[sid])
        assert np.array_equal(orc.get(0, "split"), ref.get(0, "split"))
    assert seen_high


# --------------------------------------------------------------------------- KATs
@pytest.mark.parametrize("r", [0.016, 0.008, 1.132e-3])
def test_kernel_known_answers(r):
    C = 20.0 / (14.0 * math.pi * r * r)
    assert O.kernel_eval(0, 0.0, r) == pytest.approx(4 * C, rel=1e-14)  # W(0) = 4C
    assert O.kernel_eval(0, r, r) == 0.0  # q = 2
    assert O.kernel_eval(1, r * 1.0000001, r) == 0.0
    # 2D normalisation: 2 pi int_0^r W(s) s ds = 1
    s = np.linspace(0.0, r, 20001)
    w = np.array([O.kernel_eval(0, x, r) for x in s])
    integral = 2 * math.pi * np.trapezoid(w * s, s)
    assert integral == pytest.approx(1.0, abs=1e-6)
    # gradient is the derivative of W
    for x in (0.1 * r, 0.3 * r, 0.6 * r, 0.9 * r):
        h = 1e-7 * r
        num = (O.kernel_eval(0, x + h, r) - O.kernel_eval(0, x - h, r)) / (2 * h)
        assert O.kernel_eval(1, x, r) == pytest.approx(num, rel=1e-5)
    # wall weight: continuous at q = 2/3 and q = 1, zero from q = 2
    cs = 39.6
    for q in (2.0 / 3.0, 1.0):
        d = q * r / 2
        a, b = O.kernel_eval(2, d * (1 - 1e-9), r, cs), O.kernel_eval(2, d * (1 + 1e-9), r, cs)
        assert a == pytest.approx(b, rel=1e-6)
    assert O.kernel_eval(2, r, r, cs) == 0.0


def _lattice_scene(nx, ny, dx, jitter=False, gravity=9.81, walls=True):
    sc = scenes.dam_break_small(nx, ny, dx=dx, seed=0)
    if not jitter:
        sc.low_pos = scenes.particle_box(0.5 * dx, 0.5 * dx, dx, nx, ny) + np.float32(0.3)
    sc.config.gravity = gravity
    if not walls:
        sc.wall_pos = np.zeros((0, 2), np.float32)
    sc.config.roi[:] = [10.0, 10.0, 11.0, 11.0]  # no splits
    return sc


def test_lattice_density_and_tait():
    dx = 0.01
    sc = _lattice_scene(30, 30, dx, walls=False)
    orc = O.Oracle(sc, 64)
    orc.step()
    sid = orc.get(0, "sorted_id")
    dens = orc.get(0, "dens")
    pres = orc.get(0, "pres")
    # interior particle: independent evaluation of m * sum (W_r + W_rh) / 2
    i = np.nonzero(sid == 15 * 30 + 15)[0][0]
    r, rh = sc.config.r_low, sc.config.r_high  # the float32 values the solver uses
    m = float(np.float32(sc.mass_low))
    p = sc.low_pos.astype(np.float64)
    d = np.linalg.norm(p - p[15 * 30 + 15], axis=1)
    w = [0.5 * (O.kernel_eval(0, x, r) + O.kernel_eval(0, x, rh)) for x in d[d <= r]]
    assert dens[i] == pytest.approx(m * sum(w), rel=1e-12)
    # the generator's mass calibration puts the lattice at rest density ...
    assert dens[i] == pytest.approx(1000.0, rel=1e-4)
    # ... while the low-res kernel alone with mass rho0 dx^2 also sums to rho0
    w_r = sum(O.kernel_eval(0, x, r) for x in d[d <= r])
    assert 1000.0 * dx * dx * w_r == pytest.approx(1000.0, rel=0.01)
    # Tait: p = B((rho/rho0)^7 - 1)
    B = sc.config.tait_b
    assert pres[i] == pytest.approx(B * ((dens[i] / 1000.0) ** 7 - 1), rel=1e-9)


def test_tait_zero_at_rest_density():
    sc = _lattice_scene(4, 4, 0.01, walls=False)
    orc = O.Oracle(sc, 64)
    # choose the mass so that an isolated particle has rho0 exactly: m * W_bar(0) = rho0
    r, rh = sc.config.r_low, sc.config.r_high
    wbar0 = 0.5 * (O.kernel_eval(0, 0, r) + O.kernel_eval(0, 0, rh))
    sc2 = _lattice_scene(1, 1, 0.01, walls=False)
    sc2.mass_low = 1000.0 / wbar0
    orc = O.Oracle(sc2, 64)
    orc.step()
    assert orc.get(0, "dens")[0] == pytest.approx(1000.0, rel=1e-7)  # mass is passed as float32
    assert abs(orc.get(0, "pres")[0]) < 1e-6 * sc.config.tait_b


def test_momentum_conservation_without_walls_and_gravity():
    sc = _lattice_scene(12, 12, 0.01, jitter=True, gravity=0.0, walls=False)
    rng = np.random.default_rng(5)
    sc.low_vel = rng.normal(0, 0.5, size=sc.low_pos.shape).astype(np.float32)
    orc = O.Oracle(sc, 64)
    orc.step()
    acc = orc.get(0, "acc")
    total = np.abs(acc).sum()
    assert total > 0
    assert np.abs(acc.sum(axis=0)).max() < 1e-10 * total


def test_split_conserves_mass_and_tethers_children():
    sc = scenes.dam_break_small(16, 32, seed=2, relax_iters=4)
    sc.config.roi[:] = [0.3, -math.inf, math.inf, math.inf]
    orc = O.Oracle(sc, 32)
    m, mh = np.float32(sc.mass_low), np.float32(sc.mass_high)
    assert mh * np.float32(4) == m  # split mass is exact in FP32
    splits = 0
    for _ in range(60):
        orc.step()
        st_low = orc.get(0, "state")
        n_high = orc.get(1, "id").shape[0]
        n_trans = int((st_low == 1).sum())
        assert n_high == 4 * n_trans  # 4 children per transient parent
        # M = m * #low(state 0) + m_h * #high stays m * N_low
        assert m * np.float32((st_low == 0).sum()) + mh * np.float32(n_high) == m * np.float32(st_low.size)
        splits += orc.get(0, "split").shape[0]
        # tether: every child that existed at the start of the step is within the clamp radius
        hid = orc.get(1, "id")
        hpos = orc.get(1, "pos")
        lid = orc.get(0, "id")
        lpos = orc.get(0, "pos")
        ldens = orc.get(0, "dens_state")
        slot_to_low = {int(s): k for k, s in enumerate(lid)}
        fresh = set(orc.get(0, "split").tolist())
        for k, s in enumerate(hid):
            parent = int(s) >> 2
            if parent in fresh:
                continue  # created this step, tethered from the next one
            j = slot_to_low[parent]
            lim = 0.75 * math.sqrt(sc.mass_low / (ldens[j] * math.pi))
            assert np.linalg.norm(hpos[k] - lpos[j]) <= lim * (1 + 1e-5)
    assert splits > 0


def test_fp32_against_fp64_one_step():
    """FP32 oracle vs FP64 oracle from the same state: the arithmetic's own error."""
    sc = scenes.dam_break_small(16, 32, seed=4)
    o32, o64 = O.Oracle(sc, 32), O.Oracle(sc, 64)
    for _ in range(3):
        st = o32.state(0)
        o64.load_state(0, st)
        o64.load_state(1, o32.state(1))
        o32.step()
        o64.step()
        assert np.array_equal(o32.get(0, "sorted_id"), o64.get(0, "sorted_id"))
        d32, d64 = o32.get(0, "dens"), o64.get(0, "dens")
        assert np.max(np.abs(d32 - d64) / np.abs(d64)) < 1e-5


def test_moving_roi_merge_conserves_mass_exactly():
    """Builder-defined removal (TSS_FLAG_MERGE): split parents that leave the moving
    region of interest merge back and their children are removed; the mass
    m * #(low state 0) + m/4 * #(high) is conserved exactly (a count identity,
    since m/4 is exact in FP32), in FP32 and FP64."""
    from twoscalesplit_gb300 import scenes
    for precision in (32, 64):
        sc = scenes.adaptive_dam_break(30, 60, 0.4 / 30, roi_velocity=(16.0, 4.0), roi_start=(0.0, 0.05), steps=150)
        orc = O.Oracle(sc, precision)
        n = sc.n_low
        seen_high, seen_merge = 0, 0
        prev_transient = 0
        for s in range(150):
            orc.step()
            st = orc.get(0, "state")
            nh = orc.get(1, "id").shape[0]
            assert 4 * int((st == 0).sum()) + nh == 4 * n, (precision, s)
            assert nh == 4 * int((st == 1).sum())
            seen_high = max(seen_high, nh)
            seen_merge += int(prev_transient > (st == 1).sum())
            prev_transient = int((st == 1).sum())
        assert seen_high > 0 and seen_merge > 0


def test_tether_guard_removes_the_zero_distance_nan():
    """A mixed-workload droplet scene whose split children collapse onto their
    parent: with the reference's tether a child landing exactly on the parent gets
    0/0 = NaN; with TSS_FLAG_TETHER_GUARD it keeps its position and the scene stays
    finite."""
    import copy
    from twoscalesplit_gb300 import scenes
    sc0 = scenes.mixed_batch(47, seed=0)[46]
    sc0.config.dt = np.float32(sc0.config.dt * 0.5)
    finite = {}
    for guard in (False, True):
        sc = copy.deepcopy(sc0)
        if guard:
            sc.config.flags |= 0x4
        else:
            sc.config.flags &= ~0x4
        orc = O.Oracle(sc, 32)
        for _ in range(8):
            orc.step()
        finite[guard] = bool(np.isfinite(orc.get(1, "pos")).all())
    assert finite == {False: False, True: True}


@pytest.mark.skipif(not O.refcpu_available(), reason="needs the reference checkout")
def test_older_placement_matches_the_older_snapshots_own_code():
    """TSS_FLAG_OLDER_PLACEMENT places each split's children exactly where the older
    snapshot's initSubParticlesAndAddToList (TwoScale2D-master/TwoScale2D/
    WCSPHSolver.cu:813-867, compiled here from the checkout) places them: at the
    parent's predicted position +-DIR_LEN * r, with its predicted velocity."""
    from twoscalesplit_gb300._abi import TSS_FLAG_OLDER_PLACEMENT
    sc = scenes.dam_break_small(16, 32, seed=1, relax_iters=4)
    sc.config.flags |= TSS_FLAG_OLDER_PLACEMENT
    sc.config.roi[:] = [0.3, -math.inf, math.inf, math.inf]
    o = O.Oracle(sc, 32)
    checked = 0
    for _ in range(60):
        o.step()
        split = o.get(0, "split")
        if split.size == 0:
            continue
        lo, hi = o.state(0), o.state(1)
        lpos = dict(zip(lo["id"].tolist(), lo["pos"].astype(np.float32)))
        lvel = dict(zip(lo["id"].tolist(), lo["vel"].astype(np.float32)))
        hix = {int(i): k for k, i in enumerate(hi["id"].tolist())}
        for pid in split.tolist():
            rp, rv = O.ref_older_children(np.float32(sc.config.r_low), pid, lpos[pid], lvel[pid])
            for c in range(4):
                k = hix[4 * pid + c]
                assert np.array_equal(hi["pos"][k].astype(np.float32), rp[c]), (pid, c)
                assert np.array_equal(hi["vel"][k].astype(np.float32), rv[c]), (pid, c)
            checked += 1
    assert checked > 0


def test_relaxed_cfg0_runs_its_horizon():
    """dam_break_5k with the older snapshot's placement and relaxation (4 x dt/10)
    runs all its 2,000 steps finite, with the densities near rest density; with the
    current tree's placement the same relaxation goes non-finite within 500 steps
    (its first sub-step finds the children at 2-3 rest densities)."""
    sc = scenes.dam_break_5k_relaxed(seed=0)
    o = O.Oracle(sc, 32)
    for _ in range(sc.steps):
        o.step()
    p0, p1 = o.state(0)["pos"], o.state(1)["pos"]
    assert np.isfinite(p0).all() and np.isfinite(p1).all() and p1.shape[0] > 1000
    d0, d1 = o.get(0, "dens"), o.get(1, "dens")
    assert np.abs(d0 / 1000 - 1).mean() < 0.02 and np.abs(d1 / 1000 - 1).mean() < 0.1
