"""Helpers to rebuild scenes and states from the golden step fixtures."""
import numpy as np

from twoscalesplit_gb300._abi import TssConfig
from twoscalesplit_gb300.scenes import Scene


def scene_from_fixture(g):
    c = TssConfig()
    for key in ("domain_origin", "domain_end", "dims_low", "dims_high", "roi"):
        getattr(c, key)[:] = list(g["cfg_" + key])
    for key in ("r_low", "r_high", "rest_density", "tait_b", "speed_sound", "alpha", "tension", "dt",
                "gravity", "relax_dt_div"):
        setattr(c, key, float(g["cfg_" + key]))
    c.relax_iters = int(g["cfg_relax_iters"])
    c.flags = int(g["cfg_flags"])
    m = g["mass"]
    n_low = g["out_low_state"].shape[0]
    return Scene(name="fixture", config=c, low_pos=np.zeros((n_low, 2), np.float32),
                 low_vel=np.zeros((n_low, 2), np.float32), mass_low=float(m[0]), mass_high=float(m[1]),
                 cap_high=int(g["cap_high"]), wall_pos=g["wall_pos"], mass_wall=float(m[2]), steps=1, dx=0.0)


def fixture_input(g, tag):
    return {k: g[f"in_{tag}_{k}"] for k in ("id", "pos", "vel", "state", "dens", "pres")}


def dense_to_start_end(off):
    """Dense offsets -> the reference's cellStart/cellEnd (-1 for empty cells)."""
    off = np.asarray(off)
    s = off[:-1].copy()
    e = off[1:].copy()
    empty = s == e
    s[empty] = -1
    e[empty] = -1
    return s, e
