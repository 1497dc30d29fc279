"""Seeded scene generators: the dam-break workloads the solver is measured on.

The lattice and wall generators restate the reference's CreateParticleBox and
CreateParticleBoxCanvas (TwoScale2D/ParticleSystem.cpp:123-179); the dam-break
parameters follow the reference's scene setup (TwoScale2D/main.cpp:144-175) with
the constants of the named workloads:

  dam_break_5k    50x100 lattice (5,000 low-res particles), spacing 0.008,
                  [0,0.4]x[0,0.8] in the unit box, ROI [0.4,0.7]x[0,0.3], dt 1e-4,
                  2,000 steps, children relaxed 4 x dt/10 before coupling
  dam_break_1m    707x1414 lattice (999,698 particles), spacing 5.66e-4,
                  ROI [0.4,0.9]x[0,0.5], high-res pool 4M, 500 steps

Common constants: rest density 1000, Tait gamma 7, c = 10*sqrt(2*9.81*0.8),
B = rho0*c^2/7, alpha 0.05, sigma 0.08 (main.cpp:153), gravity 9.81, support
2 x spacing, high-res support and spacing halved, mass/4 per child.  Walls are 3
layers of fixed particles around [0,1]^2 at half the fluid spacing; the grid
domain is padded by 4 wall spacings so that the walls lie inside it.  Every
lattice coordinate is jittered by U(+-1e-4 * spacing) from the seed.
dt for dam_break_1m keeps the Courant number of dam_break_5k: dt = 1e-4 * dx/0.008.

Two choices keep these scenes physical (both are switches):
  * mass: with support 2 x spacing the pair kernel (W_r + W_rh)/2 sums to 1.41/dx^2
    on the lattice, so mass 1000*dx^2 starts the fluid at 1.41 rho0, i.e. at a
    pressure of ~10 B, and the block explodes through its walls within ~100
    steps.  `calibrate_mass` (default on) scales the mass by rho0 / (lattice
    density), 0.709, so the lattice starts at rest density.
  * relaxation: the older snapshot's relaxation (4 x dt/10 with the single-scale
    high-res kernel) applied to children placed as the current tree places them
    (0.5*sqrt(m/(2 rho pi)) from the parent) gives them 2-3 rho0 in the first
    sub-step and throws them apart.  The workloads run with relax_iters = 0, as
    the current reference tree does (its relaxTransient call is commented out,
    WCSPHSolver.cu:2738); relax_iters=4 selects the relaxation.
"""
import dataclasses
import math

import numpy as np

from ._abi import TSS_FLAG_MERGE, TSS_FLAG_OLDER_PLACEMENT, TSS_FLAG_TETHER_GUARD, TssConfig, config_init

REST_DENSITY = 1000.0
GAMMA = 7
SPEED_SOUND = 10.0 * math.sqrt(2.0 * 9.81 * 0.8)
TAIT_B = REST_DENSITY * SPEED_SOUND ** 2 / GAMMA
ALPHA = 0.05
SIGMA = 0.08


@dataclasses.dataclass
class Scene:
    name: str
    config: TssConfig
    low_pos: np.ndarray        # float32 [n, 2]
    low_vel: np.ndarray        # float32 [n, 2]
    mass_low: float
    mass_high: float
    cap_high: int
    wall_pos: np.ndarray       # float32 [nw, 2]
    mass_wall: float
    steps: int
    dx: float

    @property
    def n_low(self):
        return int(self.low_pos.shape[0])

    @property
    def n_wall(self):
        return int(self.wall_pos.shape[0])


def particle_box(xs, ys, dx, dim_x, dim_y):
    """CreateParticleBox (ParticleSystem.cpp:123-148): row-major lattice, j outer."""
    f = np.float32
    i = np.arange(dim_x, dtype=np.float32)
    j = np.arange(dim_y, dtype=np.float32)
    gx = f(xs) + f(dx) * i[None, :]
    gy = f(ys) + f(dx) * j[:, None]
    pos = np.empty((dim_y, dim_x, 2), dtype=np.float32)
    pos[..., 0] = np.broadcast_to(gx, (dim_y, dim_x))
    pos[..., 1] = np.broadcast_to(gy, (dim_y, dim_x))
    return pos.reshape(-1, 2)


def particle_box_canvas(xs, ys, dx, dim_x, dim_y, off_x, off_y):
    """CreateParticleBoxCanvas (ParticleSystem.cpp:150-179): the ring of lattice
    points around a dim_x x dim_y interior, off_x/off_y layers thick."""
    f = np.float32
    out = []
    for j in range(-off_y, dim_y + off_y):
        i = np.arange(-off_x, dim_x + off_x)
        if 0 <= j < dim_y:
            i = i[(i < 0) | (i >= dim_x)]
        p = np.empty((i.size, 2), dtype=np.float32)
        p[:, 0] = f(xs) + f(dx) * i.astype(np.float32)
        p[:, 1] = f(ys) + f(dx) * f(j)
        out.append(p)
    return np.concatenate(out, axis=0)


def lattice_pair_kernel_sum(dx, r, rh):
    """sum_j (W_r + W_rh)(|x_ij|) / 2 over an infinite square lattice of spacing dx."""
    k = int(math.ceil(r / dx)) + 1
    a = np.arange(-k, k + 1, dtype=np.float64)
    d = np.hypot(*np.meshgrid(a * dx, a * dx)).ravel()
    d = d[d <= r]

    def w(d, s):
        q = 2.0 * d / s
        c = 20.0 / (14.0 * math.pi * s * s)
        return np.where(q < 1, c * ((2 - q) ** 3 - 4 * (1 - q) ** 3), np.where(q < 2, c * (2 - q) ** 3, 0.0))

    return float(np.sum(0.5 * (w(d, r) + w(d, rh))))


def _dam_break(name, nx, ny, dx, roi, dt, steps, cap_high, relax_iters, seed, flags=None, calibrate_mass=True):
    rng = np.random.default_rng(seed)
    dx = float(np.float32(dx))
    low = particle_box(0.5 * dx, 0.5 * dx, dx, nx, ny)
    low = low + rng.uniform(-1e-4 * dx, 1e-4 * dx, size=low.shape).astype(np.float32)
    low = low.astype(np.float32)
    wdx = 0.5 * dx
    nw = int(math.ceil(1.0 / wdx)) + 1
    walls = particle_box_canvas(0.0, 0.0, wdx, nw, nw, 3, 3)
    pad = 4 * wdx
    r = 2.0 * dx
    cfg = config_init(-pad, -pad, (nw - 1) * wdx + pad, (nw - 1) * wdx + pad, r, 0.5 * r,
                      REST_DENSITY, TAIT_B, SPEED_SOUND, ALPHA, SIGMA, dt)
    cfg.roi[:] = roi
    cfg.relax_iters = relax_iters
    if flags is not None:
        cfg.flags = flags
    m = REST_DENSITY * dx * dx
    if calibrate_mass:
        m = REST_DENSITY / lattice_pair_kernel_sum(dx, float(cfg.r_low), float(cfg.r_high))
    return Scene(name=name, config=cfg, low_pos=low, low_vel=np.zeros_like(low), mass_low=m,
                 mass_high=m / 4.0, cap_high=cap_high, wall_pos=walls,
                 mass_wall=REST_DENSITY * wdx * wdx, steps=steps, dx=dx)


def dam_break_5k(seed=0, relax_iters=0, **kw):
    return _dam_break("dam_break_5k", 50, 100, 0.008, [0.4, 0.0, 0.7, 0.3], 1e-4, 2000,
                      4 * 5000, relax_iters, seed, **kw)


def dam_break_5k_relaxed(seed=0, **kw):
    """dam_break_5k with its children relaxed before they couple, as the older
    snapshot does: placed at +-DIR_LEN * r on the diagonals
    (TSS_FLAG_OLDER_PLACEMENT; TwoScale2D-master/TwoScale2D/WCSPHSolver.cu:840-850)
    and relaxed 4 x dt/10 (2380-2446) at the start of the step after their split.
    With the current tree's placement the relaxation starts them at 2-3 rest
    densities and the scene goes non-finite within 500 steps; with this one it runs
    its 2,000 steps."""
    sc = dam_break_5k(seed=seed, relax_iters=4, **kw)
    sc.config.flags |= TSS_FLAG_OLDER_PLACEMENT
    sc.name = "dam_break_5k_relaxed"
    return sc


def dam_break_1m(seed=0, relax_iters=0, **kw):
    dx = 5.66e-4
    return _dam_break("dam_break_1m", 707, 1414, dx, [0.4, 0.0, 0.9, 0.5], 1e-4 * dx / 0.008, 500,
                      4_000_000, relax_iters, seed, **kw)


def adaptive_dam_break(nx, ny, dx, roi_size=0.3, roi_start=(0.05, 0.05), roi_velocity=(0.5, 0.0), steps=2000,
                       seed=0, cap_high=None, relax_iters=0, flags=None):
    """A dam break filling [0, nx*dx]x[0, ny*dx] whose region of interest (a square
    of side roi_size, lower-left corner roi_start) translates at roi_velocity units
    per second, with TSS_FLAG_MERGE: particles split as the region reaches them and
    merge back as it leaves them.  dt at dam_break_5k's Courant number; the tether
    guard on (TSS_FLAG_TETHER_GUARD) and the Q1 compatibility path off (its term
    depends on the sorted order of the high-res list, so an FP64 evaluation of the
    same state, whose cell hashing may order a boundary particle differently, is not
    comparable with it)."""
    dt = 1e-4 * dx / 0.008
    roi = [roi_start[0], roi_start[1], roi_start[0] + roi_size, roi_start[1] + roi_size]
    sc = _dam_break(f"adaptive_dam_break_{nx}x{ny}", nx, ny, dx, roi, dt, steps,
                    cap_high if cap_high is not None else 4 * nx * ny, relax_iters, seed,
                    flags=0 if flags is None else flags)
    sc.config.roi_velocity[:] = list(roi_velocity)
    sc.config.flags |= TSS_FLAG_MERGE | TSS_FLAG_TETHER_GUARD
    return sc


def adaptive_8m(seed=0, **kw):
    """The adaptive stress workload: 2000x4000 lattice at spacing 2e-4 (8M low-res
    particles), a 0.3x0.3 region of interest translating at 0.5 units/s, high-res
    pool of 32M, 2000 steps."""
    return adaptive_dam_break(2000, 4000, 2e-4, cap_high=32_000_000, seed=seed, **kw)


def dam_break_small(nx, ny, dx=None, seed=0, roi=None, relax_iters=4, cap_high=None, **kw):
    """A dam break of any lattice size filling [0,0.4]x[0,0.8] (test cases)."""
    if dx is None:
        dx = 0.4 / nx
    roi = roi if roi is not None else [0.4, 0.0, 0.7, 0.3]
    return _dam_break(f"dam_break_{nx}x{ny}", nx, ny, dx, roi, 1e-4 * dx / 0.008, 100,
                      cap_high if cap_high is not None else 4 * nx * ny, relax_iters, seed, **kw)


def _box_scene(name, fluid, dx, roi, steps, cap_factor, seed_rng, relax_iters=0, calibrate_mass=True):
    """A scene in the unit box from fluid lattice points (before jitter)."""
    dx = float(np.float32(dx))
    low = fluid + seed_rng.uniform(-1e-4 * dx, 1e-4 * dx, size=fluid.shape)
    low = low.astype(np.float32)
    wdx = 0.5 * dx
    nw = int(math.ceil(1.0 / wdx)) + 1
    walls = particle_box_canvas(0.0, 0.0, wdx, nw, nw, 3, 3)
    pad = 4 * wdx
    r = 2.0 * dx
    cfg = config_init(-pad, -pad, (nw - 1) * wdx + pad, (nw - 1) * wdx + pad, r, 0.5 * r,
                      REST_DENSITY, TAIT_B, SPEED_SOUND, ALPHA, SIGMA, 1e-4 * dx / 0.008)
    cfg.roi[:] = roi
    cfg.relax_iters = relax_iters
    # The four children of a split start below rest density, attract, and can land
    # exactly on their parent, where the reference's tether divides 0 by 0: without
    # the guard about a third of the large scenes with large regions of interest go
    # non-finite within a few thousand steps (the oracle agrees bit for bit).
    cfg.flags |= TSS_FLAG_TETHER_GUARD
    m = REST_DENSITY * dx * dx
    if calibrate_mass:
        m = REST_DENSITY / lattice_pair_kernel_sum(dx, float(cfg.r_low), float(cfg.r_high))
    n = low.shape[0]
    return Scene(name=name, config=cfg, low_pos=low, low_vel=np.zeros_like(low), mass_low=m, mass_high=m / 4.0,
                 cap_high=int(cap_factor * n), wall_pos=walls, mass_wall=REST_DENSITY * wdx * wdx, steps=steps,
                 dx=dx)


def mixed_scene(rng, n_min=2000, n_max=200000, steps=1000, cap_factor=4.0):
    """One scene of the mixed-size batch workload: a dam break (block width
    U[0.2,0.5], height U[0.4,0.9]) or a droplet (radius U[0.1,0.3], centre height
    U[0.5,0.8]) above a pool of depth U[0.1,0.4]; low-res count log-uniform in
    [n_min, n_max]; spacing from the count and the fluid area; the region of
    interest a rectangle covering U[10%,40%] of the box at a uniform position; dt
    at the Courant number of dam_break_5k; mass calibrated to rest density; the
    tether guard on (TSS_FLAG_TETHER_GUARD)."""
    n_target = math.exp(rng.uniform(math.log(n_min), math.log(n_max)))
    if rng.uniform() < 0.5:
        w, h = rng.uniform(0.2, 0.5), rng.uniform(0.4, 0.9)
        dx = math.sqrt(w * h / n_target)
        nx, ny = max(1, int(round(w / dx))), max(1, int(round(h / dx)))
        fluid = particle_box(0.5 * dx, 0.5 * dx, dx, nx, ny).astype(np.float64)
        kind = "dam"
    else:
        rad, cy, depth = rng.uniform(0.1, 0.3), rng.uniform(0.5, 0.8), rng.uniform(0.1, 0.4)
        dx = math.sqrt((math.pi * rad * rad + depth) / n_target)
        n1 = int(math.ceil(1.0 / dx))
        g = particle_box(0.5 * dx, 0.5 * dx, dx, n1, n1).astype(np.float64)
        g = g[(g[:, 0] < 1.0) & (g[:, 1] < 1.0)]
        pool = g[:, 1] < depth
        drop = ((g[:, 0] - 0.5) ** 2 + (g[:, 1] - cy) ** 2 < rad * rad) & (g[:, 1] > depth + dx)
        fluid = g[pool | drop]
        kind = "droplet"
    frac = rng.uniform(0.1, 0.4)
    aw = min(1.0, math.sqrt(frac) * rng.uniform(0.7, 1.4))
    ah = min(1.0, frac / aw)
    x0, y0 = rng.uniform(0.0, 1.0 - aw), rng.uniform(0.0, 1.0 - ah)
    return _box_scene(f"{kind}_{fluid.shape[0]}", fluid, dx, [x0, y0, x0 + aw, y0 + ah], steps, cap_factor, rng)


def mixed_batch(n_scenes=512, seed=0, **kw):
    """The batch workload: n_scenes independent mixed scenes (seeded)."""
    rng = np.random.default_rng(seed)
    return [mixed_scene(rng, **kw) for _ in range(n_scenes)]


def serving_trace(n_requests, rate_per_s, seed=0, n_min=1000, n_max=500000, h_min=200, h_max=5000):
    """The serving workload: n_requests scene requests with Poisson arrivals at
    rate_per_s, scenes as in mixed_scene with low-res counts log-uniform in
    [n_min, n_max], horizons uniform in {h_min..h_max} steps.  Returns
    [(scene, horizon, arrival_s)] in arrival order."""
    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    for _ in range(n_requests):
        t += rng.exponential(1.0 / rate_per_s)
        sc = mixed_scene(rng, n_min=n_min, n_max=n_max)
        out.append((sc, int(rng.integers(h_min, h_max + 1)), t))
    return out


def mean_work(n_min=1000, n_max=500000, h_min=200, h_max=5000):
    """E[n_low * horizon] of serving_trace's distributions (independent draws):
    the log-uniform mean (b - a) / ln(b / a) times the mean horizon."""
    return (n_max - n_min) / math.log(n_max / n_min) * (h_min + h_max) / 2.0


SCENES = {"dam_break_5k": dam_break_5k, "dam_break_5k_relaxed": dam_break_5k_relaxed, "dam_break_1m": dam_break_1m,
          "adaptive_8m": adaptive_8m}


def make_scene(name, seed=0, **kw):
    return SCENES[name](seed=seed, **kw)
