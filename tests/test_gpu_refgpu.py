"""The reference's own CUDA kernels rebuilt for sm_103a (oracle.RefGPU) against this
library on the same scene.  Agreement is within tolerance, not bitwise: the rebuilt
reference is compiled with nvcc's defaults (multiply-adds contracted), appends its
particle lists in atomic order (so from the second step its sums run in another
order) and integrates the high-res scale in place (WCSPHSolver.cu:2020-2027).
The reference's kernels hard-code the split region x > 0.5 (WCSPHSolver.cu:1835),
so the library runs the scene with that region here."""
import math

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
    if not O.refgpu_available():
        pytest.skip("the reference's kernels for sm_103a are not built (no reference checkout where built)")


def _by_slot(sol, scale, n):
    d = sol.download(scale)
    pos = np.full((n, 2), np.nan, np.float32)
    vel = np.full((n, 2), np.nan, np.float32)
    pos[d["id"]] = d["pos"]
    vel[d["id"]] = d["vel"]
    return pos, vel, d["id"]


def _pair(steps):
    sc = scenes.dam_break_5k(seed=3)
    sc.config.roi[:] = [0.5, -math.inf, math.inf, math.inf]
    ref = O.RefGPU(sc)
    sol = Solver.from_scene(sc)
    ref.step(steps)
    sol.step(steps)
    sol.sync()
    return sc, ref, sol


@pytest.mark.parametrize("steps,tol", [(1, 1e-6), (10, 1e-5), (60, 1e-4)])
def test_rebuilt_reference_tracks_the_library(steps, tol):
    sc, ref, sol = _pair(steps)
    rc, c = ref.counts(), sol.counts()
    assert rc["n_low"] == c["n_low"] == sc.n_low
    assert rc["n_high"] == c["n_high"]
    rpos, _, _ = ref.state(0)
    mpos, _, ids = _by_slot(sol, TSS_SCALE_LOW, sc.n_low)
    scale = float(np.abs(mpos).max())
    err = float(np.abs(rpos[ids] - mpos[ids]).max())
    assert err <= tol * scale, (steps, err / scale)


def test_rebuilt_reference_aggregates_after_many_steps():
    """Over hundreds of steps the two runs part particle by particle (their sums
    run in different orders in a chaotic flow), so they are compared by
    aggregates: low-res kinetic energy, centre of mass, number of splits."""
    steps = 1000
    sc, ref, sol = _pair(steps)
    rc, c = ref.counts(), sol.counts()
    assert abs(rc["n_high"] - c["n_high"]) <= max(8, c["n_high"] // 20)
    rpos, rvel, _ = ref.state(0)
    mpos, mvel, ids = _by_slot(sol, TSS_SCALE_LOW, sc.n_low)
    rpos, rvel, mpos, mvel = (a[ids].astype(np.float64) for a in (rpos, rvel, mpos, mvel))
    ke_r, ke_m = float((rvel ** 2).sum()), float((mvel ** 2).sum())
    assert abs(ke_r - ke_m) <= 1e-2 * ke_m, (ke_r, ke_m)
    com_r, com_m = rpos.mean(axis=0), mpos.mean(axis=0)
    assert np.abs(com_r - com_m).max() <= 1e-4 * np.abs(com_m).max(), (com_r, com_m)
