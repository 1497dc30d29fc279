"""GPU: the tolerance arithmetic (TSS_ARITH_FAST) against the oracle, one step at a time.

Each check loads one state -- a developed state of a dam break, with split parents
and their children -- into the solver in the fast arithmetic, into the FP32 oracle
(the reference's arithmetic) and into the FP64 oracle, takes one step in each and
compares (per-step resync: the next check starts again from the exact path's
state):

  * the integer work bit for bit: sorted ids, cell offsets and split sets.  A
    split decision may differ only for a particle whose predicted position lies
    within rounding of the region's edge; such ties are counted and printed, and
    each one is checked to be one;
  * densities within TOL = 1e-5 relative, per particle;
  * positions within TOL relative, per particle;
  * accelerations within TOL of each particle's error scale (the FP64 oracle's
    "acc_scale"): the sum of the magnitudes of the acceleration's summands (m times
    each pair's pressure/viscosity term, sigma times each tension term, each wall
    term, g), a pressure term counted with how far it moves when the two densities
    move by their own relative amount (the Tait equation's d(p/rho^2)/d rho times
    rho).  A result within TOL of that scale is the exact sum for densities and
    summands each within TOL relative -- the per-step tolerance in backward form.
    It is the form an FP32 evaluation can meet at all: the reference's own FP32
    arithmetic misses the FP64 result by up to ~2 % of |a| where a particle's
    pressure terms nearly cancel, and near rest density the Tait equation turns a
    density's last-place rounding into a large relative change of its pressure.

    Where the reference's own FP32 rounding is the larger error -- its gradient
    takes (2-q)^2 - 4(1-q)^2 as a difference of two numbers near 4, which cancels
    for close pairs (collapsing children), while the expanded form q(4-3q) does not
    -- a fast result further than TOL from it must be no further from the FP64
    result than the reference's is; such particles are counted and printed.

The errors of both arithmetics against FP64 are printed beside (the FP64 error
statement), in the same scale; the fast arithmetic's must stay within twice the
exact arithmetic's.
"""
import math

import numpy as np
import pytest

import oracle as O
from twoscalesplit_gb300 import _abi, scenes
from twoscalesplit_gb300._abi import TSS_SCALE_HIGH, TSS_SCALE_LOW
from twoscalesplit_gb300.solver import Solver

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _built():
    from twoscalesplit_gb300 import build
    build.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"


def _state(sol):
    return {s: sol.download(s) for s in (0, 1)}, sol.get_fresh(), sol.counts()["steps"]


def _load_solver(sc, st, fresh, mode):
    sol = Solver.from_scene(sc)
    sol.set_arith(mode)
    for s in (0, 1):
        d = st[s]
        sol.upload(s, {"id": d["id"], "pos": d["pos"], "vel": d["vel"], "state": d["state"],
                       "dens": d.get("dens"), "pres": d.get("pres")})
    sol.set_fresh(fresh)
    return sol


def _load_oracle(sc, st, fresh, steps, prec, scale=False):
    o = O.Oracle(sc, prec)
    for s in (0, 1):
        d = st[s]
        o.set_scale(s, d["id"], d["pos"], d["vel"], d["state"], d["dens"], d["pres"])
    o.set_fresh(fresh)
    o.set_steps(steps)
    o.set_want_scale(scale)
    return o


def _by_id(ids, vals, slots):
    out = np.full((slots,) + vals.shape[1:], np.nan)
    out[ids] = vals
    return out


def _roi_distance(sc, steps, p):
    """distance of a predicted position to the edge of the step's region of interest"""
    cfg = sc.config
    kf = np.float32(steps)
    vdt = np.float32(cfg.roi_velocity[0]) * np.float32(cfg.dt), np.float32(cfg.roi_velocity[1]) * np.float32(cfg.dt)
    x0, x1 = np.float32(cfg.roi[0]) + kf * vdt[0], np.float32(cfg.roi[2]) + kf * vdt[0]
    y0, y1 = np.float32(cfg.roi[1]) + kf * vdt[1], np.float32(cfg.roi[3]) + kf * vdt[1]
    return min(abs(p[0] - x0), abs(p[0] - x1), abs(p[1] - y0), abs(p[1] - y1))


def _check_one_step(sc, st, fresh, steps, report):
    fast = _load_solver(sc, st, fresh, "fast")
    exact = _load_solver(sc, st, fresh, "exact")
    for sol in (fast, exact):
        sol.step(1)
        sol.sync()
    o32 = _load_oracle(sc, st, fresh, steps, 32)
    o64 = _load_oracle(sc, st, fresh, steps, 64, scale=True)
    o32.step()
    o64.step()
    slots = {0: sc.n_low, 1: sc.cap_high}
    # split sets: equal up to ties at the region's edge
    s_fast, s_32 = set(fast.copy(0, _abi.TSS_BUF_SPLIT).tolist()), set(o32.get(0, "split").tolist())
    ties = s_fast ^ s_32
    if ties:
        sid = o32.get(0, "sorted_id")
        nxt = o32.state(0)
        pos_by_id = _by_id(nxt["id"], nxt["pos"], slots[0])
        for t in ties:
            assert t in set(sid.tolist())
            p = pos_by_id[t]
            assert _roi_distance(sc, steps, p) <= 4 * TOL * max(1.0, float(np.abs(p).max())), ("split tie", t, p)
    report["ties"] = report.get("ties", 0) + len(ties)
    report["splits"] = report.get("splits", 0) + len(s_32)
    for s in (TSS_SCALE_LOW, TSS_SCALE_HIGH):
        sid = fast.copy(s, _abi.TSS_BUF_SORTED_ID)
        assert np.array_equal(sid, o32.get(s, "sorted_id")), (s, "sorted ids")
        assert np.array_equal(fast.copy(s, _abi.TSS_BUF_CELL_OFFSET), o32.get(s, "cell_off")), (s, "cells")
        if sid.size == 0:
            continue
        n = slots[s]
        d32 = o32.get(s, "dens")
        df = fast.copy(s, _abi.TSS_BUF_DENSITY).astype(np.float64)
        rel_d = np.abs(df - d32) / np.abs(d32)
        assert rel_d.max() <= TOL, (s, "density", rel_d.max())
        # accelerations against each particle's error scale (FP64 oracle, by id)
        scale64 = _by_id(o64.get(s, "sorted_id"), o64.get(s, "acc_scale"), n)[sid]
        a64 = _by_id(o64.get(s, "sorted_id"), o64.get(s, "acc"), n)[sid]
        af = fast.copy(s, _abi.TSS_BUF_ACCEL).reshape(-1, 2).astype(np.float64)
        ae = exact.copy(s, _abi.TSS_BUF_ACCEL).reshape(-1, 2).astype(np.float64)
        a32 = o32.get(s, "acc")
        assert np.array_equal(ae, a32), (s, "exact arithmetic is bit-exact")
        ok64 = np.isfinite(scale64)  # present in the FP64 step too (its sort may differ at a cell edge)
        err_f32 = np.linalg.norm(af - a32, axis=1) / scale64
        err_f64 = np.linalg.norm(af - a64, axis=1) / scale64
        err_ref = np.linalg.norm(a32 - a64, axis=1) / scale64
        # within TOL of the reference's FP32 result -- or, where the reference's own
        # rounding is the larger error (its kernel gradient takes (2-q)^2 - 4(1-q)^2
        # as a difference of two numbers near 4, which cancels for close pairs), no
        # further from the FP64 result than the reference is
        closer = ok64 & (err_f64 <= np.maximum(err_ref, TOL))
        bad = ~((err_f32 <= TOL) | closer)
        assert not bad.any(), (s, "acceleration", np.nanmax(err_f32[bad]), int(bad.sum()))
        report[f"ref_less_accurate{s}"] = report.get(f"ref_less_accurate{s}", 0) + int(((err_f32 > TOL) & closer).sum())
        for name, a in (("fast", af), ("exact", ae)):
            e64 = np.linalg.norm(a - a64, axis=1)[ok64] / scale64[ok64]
            key = f"{name}_vs_fp64_acc{s}"
            report[key] = max(report.get(key, 0.0), float(e64.max()))
        report[f"fast_vs_fp32_acc{s}"] = max(report.get(f"fast_vs_fp32_acc{s}", 0.0), float(np.nanmax(err_f32)))
        report[f"fast_vs_fp32_dens{s}"] = max(report.get(f"fast_vs_fp32_dens{s}", 0.0), float(rel_d.max()))
        d64 = _by_id(o64.get(s, "sorted_id"), o64.get(s, "dens"), n)[sid]
        okd = np.isfinite(d64)
        report[f"fast_vs_fp64_dens{s}"] = max(report.get(f"fast_vs_fp64_dens{s}", 0.0),
                                             float((np.abs(df - d64)[okd] / d64[okd]).max()))
        # positions after the step, by id (the split sets are equal or the ties are at the edge)
        pf = fast.download(s)
        p32 = o32.state(s)
        common = np.intersect1d(pf["id"], p32["id"])
        xf = _by_id(pf["id"], pf["pos"].astype(np.float64), n)[common]
        x32 = _by_id(p32["id"], p32["pos"], n)[common]
        rel_x = np.linalg.norm(xf - x32, axis=1) / np.maximum(np.linalg.norm(x32, axis=1), 1e-30)
        assert rel_x.max() <= TOL, (s, "position", rel_x.max())
        report[f"fast_vs_fp32_pos{s}"] = max(report.get(f"fast_vs_fp32_pos{s}", 0.0), float(rel_x.max()))
    fast.close()
    exact.close()


@pytest.mark.parametrize("name,develop,checks", [("dam_break_48x96_x0.45", 2000, 6), ("dam_break_5k", 1500, 3)])
def test_fast_arith_per_step_resync(name, develop, checks):
    if name == "dam_break_5k":
        sc = scenes.dam_break_5k(seed=3)
    else:
        sc = scenes.dam_break_small(48, 96, seed=6, relax_iters=0)
        sc.config.roi[:] = [0.45, -math.inf, math.inf, math.inf]  # the flow crosses it: splits in most steps
    sc.config.flags |= _abi.TSS_FLAG_TETHER_GUARD
    ref = Solver.from_scene(sc)  # the exact path develops the states
    ref.step(develop)
    report = {}
    for _ in range(checks):
        st, fresh, steps = _state(ref)
        assert st[1]["id"].size > 0, "the developed state has high-res particles"
        _check_one_step(sc, st, fresh, steps, report)
        ref.step(1)
    print(name, {k: (f"{v:.2e}" if isinstance(v, float) else v) for k, v in sorted(report.items())})
    for s in (0, 1):  # no less accurate than the reference's own FP32 arithmetic, against FP64
        if f"exact_vs_fp64_acc{s}" in report:
            assert report[f"fast_vs_fp64_acc{s}"] <= 2.0 * max(report[f"exact_vs_fp64_acc{s}"], TOL / 10), s
    assert report["splits"] > 0 or name == "dam_break_5k"


def test_fast_arith_switch():
    sc = scenes.dam_break_small(16, 32, seed=1)
    sol = Solver.from_scene(sc)
    assert sol.arith == "exact"
    sol.set_arith("fast")
    assert sol.arith == "fast"
    sol.step(3)
    sol.set_arith("exact")
    sol.step(3)
    sol.sync()
    assert sol.lib.tss_solver_set_arith(sol.h, 7) == _abi.TSS_INVALID_ARG
    with pytest.raises(ValueError):
        sol.set_arith("approximate")
