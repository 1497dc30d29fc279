"""Generate the golden fixtures in this directory from the REFERENCE's own kernels.

The reference (TwoScale2D/WCSPHSolver.cu) has no tests or golden vectors.  These
fixtures come from its kernel source compiled for the CPU (oracle/refcpu, built
from the reference checkout by oracle/refcpu/build_ref.sh) and run headless:

  grid_cases.npz      computeParticleHash + thrust::sort_by_key (stable) +
                      computeCellStartEndIndices (WCSPHSolver.cu:1246-1340) on
                      adversarial key sets: random, one cell, n=1, n=0, n not a
                      multiple of 256, out-of-domain (clamped) and on-edge points
  step_q1.npz         one AdvanceTS (WCSPHSolver.cu:2726-2810) from a developed
                      dam-break state with high-res particles and transient parents
  step_q1_relax.npz   the same with the relaxation of the previous step's children
                      (TwoScale2D-master/TwoScale2D/WCSPHSolver.cu:2380-2446)
  step_developed_51k.npz
                      one AdvanceTS of the reference's kernels from a developed
                      51,200-particle dam break (160 x 320 lattice, region x > 0.5,
                      mass calibrated to rest density): 7,000 steps of flow, 5,644
                      split parents and 22,576 children, Q1 on.  The state is
                      developed by the oracle (bit-identical to the reference's
                      kernels on this schedule, tests/test_oracle_cpu.py) and the
                      recorded step is the reference's own

Run from the repository root with the reference checkout named:
    TSS_REFERENCE_ROOT=<checkout> python tests/golden/make_golden.py
"""
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from twoscalesplit_gb300 import scenes  # noqa: E402
from twoscalesplit_gb300._abi import config_init  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROI = [0.5, -math.inf, math.inf, math.inf]  # the reference's hard-coded x > 0.5


def grid_cases():
    rng = np.random.default_rng(12345)
    cfg = config_init(0.0, 0.0, 1.0, 1.0, 0.0625, 0.03125, 1000.0, 1.0, 1.0, 0.0, 0.0, 1e-4)
    r = 0.0625
    cases = {}
    cases["random"] = rng.uniform(0.0, 1.0, size=(3000, 2))
    cases["one_cell"] = np.full((500, 2), 0.3) + rng.uniform(0, 1e-3, size=(500, 2))
    cases["single"] = np.array([[0.51, 0.27]])
    cases["empty"] = np.zeros((0, 2))
    cases["ragged"] = rng.uniform(0.0, 1.0, size=(1013, 2))
    cases["outside"] = rng.uniform(-0.5, 1.5, size=(777, 2))
    k = rng.integers(0, 16, size=(400, 2))
    cases["edges"] = k * r  # exactly on cell boundaries
    out = {"origin": np.array(cfg.domain_origin[:], np.float32), "cell": np.float32(r),
           "dims": np.array(cfg.dims_low[:], np.int32)}
    for name, p in cases.items():
        p = p.astype(np.float32)
        ids = np.arange(p.shape[0], dtype=np.int32)
        sid, sh, cs, ce = O.ref_grid(cfg, p, ids)
        out[name + "_pos"] = p
        out[name + "_sorted_id"] = sid
        out[name + "_sorted_hash"] = sh
        out[name + "_cell_start"] = cs
        out[name + "_cell_end"] = ce
    np.savez_compressed(os.path.join(HERE, "grid_cases.npz"), **out)


def _ref_state(ref, scale):
    ids = ref.get(scale, "ids_active")
    return dict(id=ids, pos=ref.get(scale, "pos")[ids], vel=ref.get(scale, "vel")[ids],
                state=ref.get(scale, "state")[ids], dens=ref.get(scale, "dens")[ids],
                pres=ref.get(scale, "pres")[ids])


def step_case(fname, relax_iters, warm_steps, nx=20, ny=40, calibrate_mass=False, seed=7, develop_oracle=False):
    sc = scenes.dam_break_small(nx, ny, seed=seed, relax_iters=relax_iters, calibrate_mass=calibrate_mass)
    sc.config.roi[:] = REF_ROI
    ref = O.RefCPU(sc)
    if develop_oracle:  # the oracle develops the state, the reference's kernels take the recorded step
        orc = O.Oracle(sc, 32)
        for _ in range(warm_steps):
            orc.step()
        for s in (0, 1):
            st = orc.state(s)
            dens, pres = (st["dens_state"], st["pres_state"]) if relax_iters > 0 else (None, None)
            ref.set_scale(s, st["id"], st["pos"].astype(np.float32), st["vel"].astype(np.float32), st["state"],
                          dens, pres)
        ref.set_fresh(orc.get(0, "fresh"))
        fresh = orc.get(0, "fresh")
        inp = {s: {"id": orc.state(s)["id"], "pos": orc.state(s)["pos"].astype(np.float32),
                   "vel": orc.state(s)["vel"].astype(np.float32), "state": orc.state(s)["state"],
                   "dens": orc.state(s)["dens_state"].astype(np.float32),
                   "pres": orc.state(s)["pres_state"].astype(np.float32)} for s in (0, 1)}
    else:
        for _ in range(warm_steps):
            ref.step()
        fresh = ref.get(0, "split")
        inp = {s: _ref_state(ref, s) for s in (0, 1)}
    ref.step()
    out = {}
    c = sc.config
    for key in ("domain_origin", "domain_end", "dims_low", "dims_high", "roi"):
        out["cfg_" + key] = np.array(getattr(c, key)[:])
    for key in ("r_low", "r_high", "rest_density", "tait_b", "speed_sound", "alpha", "tension", "dt",
                "gravity", "relax_iters", "relax_dt_div", "flags"):
        out["cfg_" + key] = np.array(getattr(c, key))
    out["mass"] = np.array([sc.mass_low, sc.mass_high, sc.mass_wall], np.float32)
    out["cap_high"] = np.array(sc.cap_high)
    out["wall_pos"] = sc.wall_pos
    out["fresh"] = fresh
    for s, tag in ((0, "low"), (1, "high")):
        for k, v in inp[s].items():
            out[f"in_{tag}_{k}"] = v
        n_in = inp[s]["id"].shape[0]
        out[f"out_{tag}_sorted_id"] = ref.get(s, "sorted_prev")[:n_in]
        out[f"out_{tag}_cell_start"] = ref.get(s, "cell_start")
        out[f"out_{tag}_cell_end"] = ref.get(s, "cell_end")
        for k in ("pos", "vel", "acc", "dens", "pres", "state"):
            out[f"out_{tag}_{k}"] = ref.get(s, k)  # slot-indexed
        out[f"out_{tag}_ids"] = ref.get(s, "ids_active")
    out["out_split"] = ref.get(0, "split")
    out["out_counts"] = ref.get(0, "counts")
    np.savez_compressed(os.path.join(HERE, fname), **out)
    print(fname, "n_low", inp[0]["id"].shape[0], "n_high in", inp[1]["id"].shape[0], "out",
          out["out_counts"], "fresh", fresh.shape[0], "split", out["out_split"].shape[0])


if __name__ == "__main__":
    if not O.refcpu_available():
        sys.exit("the reference checkout is needed to generate the fixtures")
    grid_cases()
    step_case("step_q1.npz", 0, 120)
    step_case("step_q1_relax.npz", 4, 120)
    step_case("step_developed_51k.npz", 0, 7000, nx=160, ny=320, calibrate_mass=True, seed=11, develop_oracle=True)
