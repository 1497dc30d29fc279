"""GPU parity: the sm_103a kernels (through the C ABI) against the reference's own
kernels (golden fixtures) and the CPU oracle.

Integer work (cell indices, sorted permutations, cell ranges, split sets) must be
bit-exact.  Densities, forces and positions are required within 1e-5 relative in
FP32 (TOL below); the kernels keep the reference's operation order and are built
without fused multiply-adds, so in practice they are bit-identical to the FP32
oracle, and the tests check that too.
"""
import ctypes
import math
import os

import numpy as np
import pytest

import oracle as O
from tests._golden import dense_to_start_end, fixture_input, scene_from_fixture
from twoscalesplit_gb300 import _abi, scenes
from twoscalesplit_gb300._abi import TSS_SCALE_HIGH, TSS_SCALE_LOW, TssError
from twoscalesplit_gb300.solver import Solver

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-5  # FP32 relative tolerance for densities, forces, positions


@pytest.fixture(scope="module", autouse=True)
def _built():
    from twoscalesplit_gb300 import build
    build.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"


def _torch():
    import torch
    return torch


# --------------------------------------------------------------------------- grid
def _grid_gpu(pos, ids, origin, cell, dims, timing=None):
    torch = _torch()
    lib = _abi.load_library()
    n = ids.shape[0]
    dpos = torch.from_numpy(np.ascontiguousarray(pos, np.float32).reshape(-1)).cuda()
    did = torch.from_numpy(np.ascontiguousarray(ids, np.int32)).cuda()
    order = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    off = torch.full((dims[0] * dims[1] + 1,), -7, dtype=torch.int32, device="cuda")
    ws = ctypes.c_size_t(0)
    assert lib.tss_grid_workspace_size(n, int(dims[0]), int(dims[1]), ctypes.byref(ws)) == 0
    work = torch.empty(ws.value, dtype=torch.uint8, device="cuda")
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    torch.cuda.synchronize()
    ev[0].record()
    st = lib.tss_grid_build(ctypes.c_void_p(dpos.data_ptr()), ctypes.c_void_p(did.data_ptr()), n,
                            float(origin[0]), float(origin[1]), float(cell), int(dims[0]), int(dims[1]),
                            ctypes.c_void_p(order.data_ptr()), ctypes.c_void_p(off.data_ptr()),
                            ctypes.c_void_p(work.data_ptr()), ws.value,
                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    ev[1].record()
    assert st == 0
    torch.cuda.synchronize()
    if timing is not None:
        timing.append(ev[0].elapsed_time(ev[1]))
    return order.cpu().numpy()[:n], off.cpu().numpy()


@pytest.mark.parametrize("case", ["random", "one_cell", "single", "empty", "ragged", "outside", "edges"])
def test_grid_build_matches_reference_fixture(case):
    g = np.load(os.path.join(GOLDEN, "grid_cases.npz"))
    pos = g[case + "_pos"]
    ids = np.arange(pos.shape[0], dtype=np.int32)
    order, off = _grid_gpu(pos, ids, g["origin"], float(g["cell"]), g["dims"])
    assert np.array_equal(ids[order], g[case + "_sorted_id"])
    s, e = dense_to_start_end(off)
    assert np.array_equal(s, g[case + "_cell_start"])
    assert np.array_equal(e, g[case + "_cell_end"])


@pytest.mark.parametrize("n,cells,spread", [(1_000_003, 1024, 1.0), (300_000, 4096, 0.001), (50_000, 2, 1.0),
                                            (4097, 3000, 1.0)])
def test_grid_build_matches_oracle_adversarial(n, cells, spread):
    rng = np.random.default_rng(n)
    pos = (rng.uniform(0, spread, size=(n, 2))).astype(np.float32)
    ids = rng.permutation(4 * n)[:n].astype(np.int32)  # unique, unsorted, sparse
    dims = (cells, cells)
    order, off = _grid_gpu(pos, ids, (0.0, 0.0), 1.0 / cells, dims)
    o_order, o_off = O.grid(pos, ids, (0.0, 0.0), 1.0 / cells, dims)
    assert np.array_equal(off, o_off)
    assert np.array_equal(order, o_order)


@pytest.mark.parametrize("case", ["border_clamped", "one_cluster", "around_threshold"])
def test_grid_build_crowded_cells_bounded(case):
    """Cells far fuller than a grid's few particles per cell -- points outside the
    domain clamped into its border cells (computeGridCoordinate,
    WCSPHSolver.cu:247-248), a collapsed cluster, cells straddling the size where the
    in-cell ordering switches from counting to a block sort -- give exactly the
    stable (cell, id) order of the oracle, and the build stays fast (its time is
    printed; an ordering quadratic in the cell size would take minutes here)."""
    rng = np.random.default_rng({"border_clamped": 11, "one_cluster": 12, "around_threshold": 13}[case])
    if case == "border_clamped":  # 1.2M points, ~300k in each corner cell of a 64x64 grid on [0,1]^2
        n, dims, lo, hi = 1_200_000, (64, 64), -100.0, 101.0
    elif case == "one_cluster":  # 400k points in ~650 cells of a 512x512 grid: ~600 per cell
        n, dims, lo, hi = 400_000, (512, 512), 0.0, 0.05
    else:  # ~38 per cell on average: cells both below and above the switch
        n, dims, lo, hi = 100_000, (512, 512), 0.0, 0.1
    pos = rng.uniform(lo, hi, size=(n, 2)).astype(np.float32)
    ids = rng.permutation(2 * n)[:n].astype(np.int32)
    ms = []
    order, off = _grid_gpu(pos, ids, (0.0, 0.0), 1.0 / dims[0], dims, timing=ms)
    o_order, o_off = O.grid(pos, ids, (0.0, 0.0), 1.0 / dims[0], dims)
    assert np.array_equal(off, o_off)
    assert np.array_equal(order, o_order)
    counts = np.diff(off)
    print(f"{case}: n={n}, largest cell {counts.max()}, build {ms[0]:.3f} ms")
    assert counts.max() > 32
    assert ms[0] < 1000.0


# --------------------------------------------------------------------------- helpers
def _load_state(sol, scale, st):
    sol.upload(scale, {"id": st["id"], "pos": st["pos"], "vel": st["vel"], "state": st["state"],
                       "dens": st.get("dens"), "pres": st.get("pres")})


def _assert_state_equal(gpu, orc, scale, where, exact=True):
    st = orc.state(scale)
    d = gpu.download(scale)
    assert np.array_equal(d["id"], st["id"]), (where, scale, "id")
    assert np.array_equal(d["state"], st["state"]), (where, scale, "state")
    for k in ("pos", "vel"):
        a, b = d[k], st[k].astype(np.float32)
        if exact:
            assert np.array_equal(a, b), (where, scale, k, np.abs(a - b).max() if a.size else 0)
        else:
            scale_ref = np.abs(b).max() if b.size else 1.0
            assert np.abs(a - b).max(initial=0) <= TOL * max(scale_ref, 1e-30), (where, scale, k)


def _compare_step_buffers(gpu, orc, where):
    for s in (TSS_SCALE_LOW, TSS_SCALE_HIGH):
        sid = gpu.copy(s, _abi.TSS_BUF_SORTED_ID)
        assert np.array_equal(sid, orc.get(s, "sorted_id")), (where, s, "sorted id")
        assert np.array_equal(gpu.copy(s, _abi.TSS_BUF_CELL_OFFSET), orc.get(s, "cell_off")), (where, s, "cells")
        for which, name in ((_abi.TSS_BUF_DENSITY, "dens"), (_abi.TSS_BUF_PRESSURE, "pres"),
                            (_abi.TSS_BUF_ACCEL, "acc")):
            a = gpu.copy(s, which)
            b = orc.get(s, name).astype(np.float32)
            assert np.array_equal(a, b), (where, s, name, np.abs(a - b).max() if a.size else 0)
    assert np.array_equal(gpu.copy(TSS_SCALE_LOW, _abi.TSS_BUF_SPLIT), orc.get(0, "split")), (where, "split")


# --------------------------------------------------------------------------- step vs reference
@pytest.mark.parametrize("fname", ["step_q1.npz", "step_q1_relax.npz", "step_developed_51k.npz"])
def test_step_matches_reference_fixture(fname):
    g = np.load(os.path.join(GOLDEN, fname))
    sc = scene_from_fixture(g)
    sol = Solver.from_scene(sc)
    for s, tag in ((TSS_SCALE_LOW, "low"), (TSS_SCALE_HIGH, "high")):
        _load_state(sol, s, fixture_input(g, tag))
    sol.set_fresh(g["fresh"])
    sol.step(1)
    sol.sync()
    for s, tag in ((TSS_SCALE_LOW, "low"), (TSS_SCALE_HIGH, "high")):
        sid = sol.copy(s, _abi.TSS_BUF_SORTED_ID)
        assert np.array_equal(sid, g[f"out_{tag}_sorted_id"]), tag
        cs, ce = dense_to_start_end(sol.copy(s, _abi.TSS_BUF_CELL_OFFSET))
        assert np.array_equal(cs, g[f"out_{tag}_cell_start"]) and np.array_equal(ce, g[f"out_{tag}_cell_end"])
        for which, name in ((_abi.TSS_BUF_DENSITY, "dens"), (_abi.TSS_BUF_PRESSURE, "pres")):
            a = sol.copy(s, which)
            ref = g[f"out_{tag}_{name}"][sid]
            assert np.all(np.abs(a - ref) <= TOL * np.abs(ref)), (tag, name)
            assert np.array_equal(a, ref), (tag, name, "bit-exact")
        acc = sol.copy(s, _abi.TSS_BUF_ACCEL)
        assert np.array_equal(acc, g[f"out_{tag}_acc"].reshape(-1, 2)[sid]), (tag, "acc")
        d = sol.download(s)
        assert sorted(d["id"].tolist()) == sorted(g[f"out_{tag}_ids"].tolist())
        for k in ("pos", "vel"):
            assert np.array_equal(d[k], g[f"out_{tag}_{k}"].reshape(-1, 2)[d["id"]]), (tag, k)
        assert np.array_equal(d["state"], g[f"out_{tag}_state"][d["id"]])
    assert np.array_equal(sol.copy(TSS_SCALE_LOW, _abi.TSS_BUF_SPLIT), g["out_split"])
    c = sol.counts()
    assert c["n_high"] == g["out_counts"][1]


# --------------------------------------------------------------------------- multi-step vs oracle
@pytest.mark.parametrize("relax,flags,roi", [(4, 1, None), (0, 1, "ref"), (4, 0, None), (4, 1 | 8, None)])
def test_multistep_matches_oracle(relax, flags, roi):
    sc = scenes.dam_break_small(16, 32, seed=21, relax_iters=relax, flags=flags, calibrate_mass=(roi != "ref"))
    if roi == "ref":
        sc.config.roi[:] = [0.5, -math.inf, math.inf, math.inf]
    else:
        sc.config.roi[:] = [0.3, -math.inf, math.inf, math.inf]
    sol = Solver.from_scene(sc)
    orc = O.Oracle(sc, 32)
    high_seen = 0
    for k in range(120):
        sol.step(1)
        orc.step()
        if k % 10 == 9 or k < 3:
            sol.sync()
            _compare_step_buffers(sol, orc, k)
            _assert_state_equal(sol, orc, TSS_SCALE_LOW, k)
            _assert_state_equal(sol, orc, TSS_SCALE_HIGH, k)
            assert np.array_equal(sol.get_fresh(), orc.get(0, "fresh"))
            high_seen = max(high_seen, sol.counts()["n_high"])
    assert high_seen > 0


def test_dam_break_5k_tracks_oracle_300_steps():
    sc = scenes.dam_break_5k(seed=3)
    sol = Solver.from_scene(sc)
    orc = O.Oracle(sc, 32)
    for k in range(300):
        orc.step()
    sol.step(300)
    sol.sync()
    _compare_step_buffers(sol, orc, 299)
    _assert_state_equal(sol, orc, TSS_SCALE_LOW, 299)
    _assert_state_equal(sol, orc, TSS_SCALE_HIGH, 299)
    assert sol.counts()["n_high"] > 0


def test_relaxed_cfg0_tracks_oracle():
    """dam_break_5k with the older snapshot's child placement and relaxation: the GPU
    equals the FP32 oracle bit for bit through splits and relaxation sub-steps."""
    sc = scenes.dam_break_5k_relaxed(seed=3)
    sol = Solver.from_scene(sc)
    orc = O.Oracle(sc, 32)
    for k in range(400):
        orc.step()
    sol.step(400)
    sol.sync()
    _compare_step_buffers(sol, orc, 399)
    _assert_state_equal(sol, orc, TSS_SCALE_LOW, 399)
    _assert_state_equal(sol, orc, TSS_SCALE_HIGH, 399)
    assert np.array_equal(sol.get_fresh(), orc.get(0, "fresh"))
    assert sol.counts()["n_high"] > 0


def test_fp64_error_statement():
    """One step from a developed state: FP32 GPU vs the FP64 oracle."""
    sc = scenes.dam_break_small(20, 40, seed=5, relax_iters=4)
    sol = Solver.from_scene(sc)
    sol.step(150)
    o64 = O.Oracle(sc, 64)
    for s in (TSS_SCALE_LOW, TSS_SCALE_HIGH):
        d = sol.download(s)
        o64.set_scale(s, d["id"], d["pos"], d["vel"], d["state"], d["dens"], d["pres"])
    o64.set_fresh(sol.get_fresh())
    sol.step(1)
    sol.sync()
    o64.step()
    report = {}
    for s in (TSS_SCALE_LOW, TSS_SCALE_HIGH):
        sid = sol.copy(s, _abi.TSS_BUF_SORTED_ID)
        assert np.array_equal(sid, o64.get(s, "sorted_id"))
        dg, d64 = sol.copy(s, _abi.TSS_BUF_DENSITY), o64.get(s, "dens")
        report[f"dens{s}"] = float(np.max(np.abs(dg - d64) / np.abs(d64)))
        ag, a64 = sol.copy(s, _abi.TSS_BUF_ACCEL), o64.get(s, "acc")
        report[f"acc{s}"] = float(np.max(np.linalg.norm(ag - a64, axis=1)) / np.max(np.linalg.norm(a64, axis=1)))
        st64 = o64.state(s)
        dd = sol.download(s)
        report[f"pos{s}"] = float(np.max(np.abs(dd["pos"] - st64["pos"])) / np.max(np.abs(st64["pos"])))
    print("FP32 vs FP64 relative errors:", report)
    assert report["dens0"] < 1e-5 and report["dens1"] < 1e-5
    assert report["acc0"] < 1e-4 and report["acc1"] < 1e-4
    assert report["pos0"] < 1e-6 and report["pos1"] < 1e-6


def test_1m_dam_break_one_step_parity_and_invariants():
    sc = scenes.dam_break_1m(seed=0)
    sol = Solver.from_scene(sc)
    orc = O.Oracle(sc, 32)
    sol.step(1)
    sol.sync()
    orc.step()
    sid = sol.copy(TSS_SCALE_LOW, _abi.TSS_BUF_SORTED_ID)
    assert np.array_equal(sid, orc.get(0, "sorted_id"))
    off = sol.copy(TSS_SCALE_LOW, _abi.TSS_BUF_CELL_OFFSET)
    assert np.array_equal(off, orc.get(0, "cell_off"))
    for which, name in ((_abi.TSS_BUF_DENSITY, "dens"), (_abi.TSS_BUF_ACCEL, "acc")):
        assert np.array_equal(sol.copy(TSS_SCALE_LOW, which), orc.get(0, name).astype(np.float32))
    # size-independent properties after more steps on the GPU alone
    sol.step(20)
    sol.sync()
    d = sol.download(TSS_SCALE_LOW)
    assert np.array_equal(np.sort(d["id"]), np.arange(sc.n_low))  # a permutation of all slots
    off = sol.copy(TSS_SCALE_LOW, _abi.TSS_BUF_CELL_OFFSET)
    assert off[0] == 0 and off[-1] == sc.n_low and np.all(np.diff(off) >= 0)
    c = sol.counts()
    m, mh = np.float32(sc.mass_low), np.float32(sc.mass_high)
    assert m * np.float32((d["state"] == 0).sum()) + mh * np.float32(c["n_high"]) == m * np.float32(sc.n_low)


def test_1m_developed_multistep_parity():
    """The 1M dam break once its front carries parents through the region of interest
    (20,000 steps on the GPU, ~400k high-res particles, tens of splits per step):
    three more steps bit-exact against the FP32 oracle started from the same state --
    sorted ids, cell offsets, densities, pressures, accelerations, split sets, both
    lists after each step."""
    sc = scenes.dam_break_1m(seed=0)
    sc.config.flags |= _abi.TSS_FLAG_TETHER_GUARD
    sol = Solver.from_scene(sc)
    sol.step(20000)
    sol.sync()
    orc = O.Oracle(sc, 32)
    for s in (TSS_SCALE_LOW, TSS_SCALE_HIGH):
        d = sol.download(s)
        orc.set_scale(s, d["id"], d["pos"], d["vel"], d["state"], d["dens"], d["pres"])
    orc.set_fresh(sol.get_fresh())
    orc.set_steps(sol.counts()["steps"])
    assert sol.counts()["n_high"] > 100_000
    splits = 0
    for k in range(3):
        sol.step(1)
        sol.sync()
        orc.step()
        _compare_step_buffers(sol, orc, k)
        _assert_state_equal(sol, orc, TSS_SCALE_LOW, k)
        _assert_state_equal(sol, orc, TSS_SCALE_HIGH, k)
        splits += sol.copy(TSS_SCALE_LOW, _abi.TSS_BUF_SPLIT).shape[0]
    assert splits > 0


def test_determinism_bitwise():
    sc = scenes.dam_break_5k(seed=9)
    a, b = Solver.from_scene(sc), Solver.from_scene(sc)
    a.step(80)
    b.step(80)
    for s in (TSS_SCALE_LOW, TSS_SCALE_HIGH):
        da, db = a.download(s), b.download(s)
        for k in da:
            assert np.array_equal(da[k], db[k]), (s, k)


def test_capacity_error_is_reported():
    sc = scenes.dam_break_small(16, 32, seed=1, cap_high=8)
    sc.config.roi[:] = [0.0, -math.inf, math.inf, math.inf]  # everything splits at once
    sol = Solver.from_scene(sc)
    sol.step(1)
    with pytest.raises(TssError) as ei:
        sol.sync()
    assert ei.value.status == _abi.TSS_CAPACITY
    assert sol.counts()["n_high"] <= 8


def test_numeric_error_is_reported():
    sc = scenes.dam_break_small(8, 8, seed=1)
    sol = Solver.from_scene(sc)
    d = sol.download(TSS_SCALE_LOW)
    d["pos"][3] = np.nan
    sol.upload(TSS_SCALE_LOW, d)
    sol.step(1)
    with pytest.raises(TssError) as ei:
        sol.sync()
    assert ei.value.status == _abi.TSS_NUMERIC


def test_reference_shaped_api_matches_solver():
    from twoscalesplit_gb300 import solver as S
    sc = scenes.dam_break_small(12, 24, seed=0)
    cfg = S.WCSPHConfig(*sc.config.domain_origin, *sc.config.domain_end, sc.config.r_low, sc.config.r_high,
                        sc.config.rest_density, sc.config.tait_b, sc.config.speed_sound, sc.config.alpha,
                        sc.config.tension, sc.config.dt)
    assert cfg.DomainDimensions == list(sc.config.dims_low)
    fluid = S.CreateParticleBox(0.5 * sc.dx, 0.5 * sc.dx, sc.dx, 12, 24, sc.mass_low)
    high = S.ParticleSystem(4 * fluid.GetMaxParticles(), fluid.GetMass() / 4.0)
    walls = S.ParticleSystem(sc.n_wall, sc.mass_wall)
    for p in sc.wall_pos:
        walls.PushParticle(p)
    solver = S.WCSPHSolver(cfg, fluid, high, walls)
    solver.Bind()
    for _ in range(40):
        solver.AdvanceTS()
    cfg.cfg.roi[:] = list(cfg.cfg.roi)
    twin = Solver(cfg.cfg, fluid.host_positions(), sc.mass_low, 4 * 12 * 24, sc.mass_low / 4.0, sc.wall_pos,
                  sc.mass_wall)
    twin.step(40)
    assert np.array_equal(fluid.Positions(), twin.download(TSS_SCALE_LOW)["pos"])
    assert fluid.GetNumParticles() == 12 * 24
    with pytest.raises(ValueError):
        S.WCSPHConfig(1.0, 0.0, 0.0, 1.0, 0.1, 0.05, 1000, 1, 1, 0, 0, 1e-4)


def test_step_on_caller_stream():
    torch = _torch()
    sc = scenes.dam_break_small(10, 20, seed=2)
    a, b = Solver.from_scene(sc), Solver.from_scene(sc)
    s = torch.cuda.Stream()
    a.step(25, stream=s.cuda_stream)
    b.step(25)
    s.synchronize()
    assert np.array_equal(a.download(0)["pos"], b.download(0)["pos"])
