"""Headless splat renderer: the CPU restatement of the reference's shader math
(oracle.splat) and the GPU rasterizer (tss_render_splats / tss_solver_render),
compared bit for bit -- each pixel blends the splats covering it in drawing order
with the same FP32 expressions, so the images must be identical (tolerance: exact
equality)."""
import math

import numpy as np
import pytest

import oracle as O
from twoscalesplit_gb300 import scenes


def _cleared(w, h):
    img = np.zeros((h, w, 4), np.float32)
    img[..., :3] = 1.0
    return img


def test_cpu_splat_semantics():
    # one particle at the centre of a 64x64 view of [0,1]^2, radius 0.1 NDC = 3.2 px
    img = O.splat((0.0, 0.0, 1.0, 1.0), 64, 64, np.array([[0.5, 0.5]]), rgb=(0.0, 0.0, 0.0), point_size=0.1)
    covered = img[..., 3] > 0
    assert covered.sum() == 32  # pixel centres within 3.2 px of the image centre
    assert np.allclose(img[covered, :3], 0.5) and np.allclose(img[covered, 3], 0.25)
    assert np.all(img[~covered, :3] == 1.0) and np.all(img[~covered, 3] == 0.0)
    # blending is ordered: the later splat weighs 1/2, the earlier 1/4
    two = O.splat((0.0, 0.0, 1.0, 1.0), 8, 8, np.array([[0.5, 0.5], [0.5, 0.5]]), dens=np.array([1000.0, 600.0]),
                  point_size=0.2)
    c = two[4, 4]
    blue, red = np.array([0.0, 0.0, 0.5]), np.array([0.5, 0.0, 0.0])  # jet(0) and jet(1)
    assert np.allclose(c[:3], 0.5 * np.array([0.5, 0.0, 0.0]) + 0.25 * np.array([0.0, 0.0, 0.5]) + 0.25)
    del blue, red
    # the jet map at the visual quantity's ends (QuantityRendererFragmentShader.glsl:32-40)
    assert math.isclose(float(two[4, 4, 3]), 0.375)


@pytest.mark.gpu
def test_gpu_splats_equal_cpu_restatement():
    import torch
    from twoscalesplit_gb300 import build, render
    build.build()
    rng = np.random.default_rng(5)
    W, H = 203, 157
    v = render.view(0.1, -0.05, 0.9, 1.05, W, H)
    n = 20000
    pos = rng.uniform(0.0, 1.0, size=(n, 2)).astype(np.float32)
    pos[:50] = np.nan                                   # skipped
    pos[50:60] = [[5.0, 5.0]]                           # off screen
    pos[60:6060] = pos[60]                              # one tile with > 4096 splats (selection path)
    dens = rng.uniform(500.0, 1600.0, size=n).astype(np.float32)
    img = render.splats(v, torch.from_numpy(pos).cuda(), torch.from_numpy(dens).cuda(), point_size=0.02)
    img = render.splats(v, torch.from_numpy(pos[::7].copy()).cuda(), None, rgb=(0.2, 0.4, 0.6), point_size=0.013,
                        img=img)
    torch.cuda.synchronize()
    ref = O.splat((0.1, -0.05, 0.9, 1.05), W, H, pos, dens=dens, point_size=0.02)
    ref = O.splat((0.1, -0.05, 0.9, 1.05), W, H, pos[::7], rgb=(0.2, 0.4, 0.6), point_size=0.013, img=ref)
    got = img.cpu().numpy()
    assert np.array_equal(got, ref)


@pytest.mark.gpu
def test_solver_frame_equals_cpu_restatement():
    import torch
    from twoscalesplit_gb300 import build
    from twoscalesplit_gb300._abi import TSS_SCALE_HIGH, TSS_SCALE_LOW
    from twoscalesplit_gb300.solver import Solver
    build.build()
    sc = scenes.dam_break_small(20, 40, seed=2, relax_iters=0, roi=[0.2, -math.inf, math.inf, math.inf])
    sol = Solver.from_scene(sc)
    sol.step(30)
    W = H = 300
    view = (0.0, 0.0, 1.0, 1.0, W, H)
    sizes = (0.01, 0.006, 0.01)
    img = sol.render(view, sizes)
    torch.cuda.synchronize()
    low, high = sol.download(TSS_SCALE_LOW), sol.download(TSS_SCALE_HIGH)
    assert high["id"].shape[0] > 0
    rho0 = float(sc.config.rest_density)
    ref = O.splat(view[:4], W, H, low["pos"], dens=low["dens"], rest_density=rho0, point_size=sizes[0])
    ref = O.splat(view[:4], W, H, high["pos"], dens=high["dens"], rest_density=rho0, point_size=sizes[1], img=ref)
    ref = O.splat(view[:4], W, H, sc.wall_pos, rgb=(0.0, 0.0, 0.0), point_size=sizes[2], img=ref)
    assert np.array_equal(img.cpu().numpy(), ref)
