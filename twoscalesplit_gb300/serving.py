"""Pools and the serving loop over the C ABI (include/tss.h).

`Pool` is a solver handle whose scenes are admitted and retired between steps
(tss_pool_*); `Server` replays a trace of scene requests in real time through the
library's serving loop (tss_server_run): admission by free pool memory, continuous
batching of every admitted scene, extraction and retirement at each scene's
horizon.  Neither has a counterpart in the reference, whose solver held one scene
per process (TwoScale2D/WCSPHSolver.cu:2728); each scene keeps the reference's
step semantics.
"""
import ctypes
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._abi import TssError, check, fptr, load_library
from .solver import Batch


def scene_desc(scene, keep):
    """tss_scene_desc of a scenes.Scene; the arrays it points at are appended to `keep`."""
    lp = np.ascontiguousarray(scene.low_pos, np.float32).reshape(-1, 2)
    lv = None if scene.low_vel is None else np.ascontiguousarray(scene.low_vel, np.float32).reshape(-1, 2)
    wp = np.ascontiguousarray(scene.wall_pos, np.float32).reshape(-1, 2)
    keep += [lp, lv, wp, scene.config]
    return _abi.TssSceneDesc(ctypes.pointer(scene.config), lp.shape[0], fptr(lp), fptr(lv), scene.mass_low,
                             scene.mass_high, wp.shape[0], fptr(wp), scene.mass_wall)


def footprint(scene):
    """Pool resources a scene takes (rounded to pages); host only."""
    lib = load_library()
    keep = []
    d = scene_desc(scene, keep)
    f = _abi.TssFootprint()
    check(lib.tss_scene_footprint(ctypes.byref(d), ctypes.byref(f)))
    return f.as_dict()


def pool_bytes(cfg):
    lib = load_library()
    b = ctypes.c_size_t(0)
    check(lib.tss_pool_bytes(ctypes.byref(cfg), ctypes.byref(b)))
    return b.value


def pool_config(low_slots, high_particles=None, low_cells=None, high_cells=None, wall_particles=0, max_scenes=1024,
                relax_iters=0):
    c = _abi.TssPoolConfig()
    c.low_slots = int(low_slots)
    c.high_particles = int(4 * low_slots if high_particles is None else high_particles)
    c.low_cells = int(2 * low_slots if low_cells is None else low_cells)
    c.high_cells = int(4 * c.low_cells if high_cells is None else high_cells)
    c.wall_particles = int(wall_particles)
    c.max_scenes = int(max_scenes)
    c.relax_iters = int(relax_iters)
    return c


def pool_config_for_budget(nbytes, low_cells_per_slot, walls_per_slot, max_scenes=4096, relax_iters=0):
    """The largest pool within `nbytes` of device memory with these proportions."""
    lib = load_library()
    c = _abi.TssPoolConfig()
    check(lib.tss_pool_config_for_budget(int(nbytes), float(low_cells_per_slot), float(walls_per_slot),
                                         int(max_scenes), int(relax_iters), ctypes.byref(c)))
    return c


class Pool(Batch):
    """A pool of scenes (tss_pool_create): scenes are admitted and retired between
    steps; step() advances all admitted scenes together."""

    def __init__(self, cfg):
        self.lib = load_library()
        self.cfg = cfg
        self.scenes = {}
        h = ctypes.c_void_p()
        check(self.lib.tss_pool_create(ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h

    def can_admit(self, scene):
        """True if the pool has room for the scene now, False if not (TSS_CAPACITY)."""
        keep = []
        d = scene_desc(scene, keep)
        st = self.lib.tss_pool_can_admit(self.h, ctypes.byref(d))
        if st == _abi.TSS_CAPACITY:
            return False
        self._check(st)
        return True

    def admit(self, scene, stream=None):
        """Scene id, or None when the pool has no room now (TSS_CAPACITY)."""
        keep = []
        d = scene_desc(scene, keep)
        sid = ctypes.c_int(-1)
        st = self.lib.tss_pool_admit(self.h, ctypes.byref(d), ctypes.c_void_p(stream) if stream else None,
                                     ctypes.byref(sid))
        if st == _abi.TSS_CAPACITY:
            return None
        self._check(st)
        self.scenes[sid.value] = scene
        return sid.value

    def retire(self, sid, stream=None):
        self._check(self.lib.tss_pool_retire(self.h, int(sid), ctypes.c_void_p(stream) if stream else None))
        self.scenes.pop(sid, None)

    def free(self):
        f = _abi.TssFootprint()
        self._check(self.lib.tss_pool_free(self.h, ctypes.byref(f)))
        return f.as_dict()

    def scene_counts(self):
        n = ctypes.c_int(0)
        self._check(self.lib.tss_solver_num_scenes(self.h, ctypes.byref(n)))
        lo = np.zeros(max(n.value, 1), np.int32)
        hi = np.zeros(max(n.value, 1), np.int32)
        self._check(self.lib.tss_solver_scene_counts(self.h, _abi.iptr(lo), _abi.iptr(hi)))
        return lo, hi

    def extract(self, sid, stream=None):
        """The scene's state after the last step, through tss_pool_extract into device
        buffers (torch CUDA tensors), then copied to the host."""
        import torch
        n = self.scenes[sid].n_low
        caps = (n, 4 * n)
        dev = torch.device("cuda")
        bufs = []
        res = _abi.TssSceneResult()
        for k in range(2):
            m = max(caps[k], 1)
            b = {"id": torch.empty(m, dtype=torch.int32, device=dev), "pos": torch.empty((m, 2), dtype=torch.float32, device=dev),
                 "vel": torch.empty((m, 2), dtype=torch.float32, device=dev),
                 "state": torch.empty(m, dtype=torch.uint8, device=dev),
                 "dens": torch.empty(m, dtype=torch.float32, device=dev), "pres": torch.empty(m, dtype=torch.float32, device=dev)}
            bufs.append(b)
            res.cap[k] = caps[k]
            for name in ("id", "pos", "vel", "state", "dens", "pres"):
                getattr(res, name)[k] = b[name].data_ptr()
        counts = torch.zeros(3, dtype=torch.int32, device=dev)
        s = stream if stream else torch.cuda.current_stream().cuda_stream
        self._check(self.lib.tss_pool_extract(self.h, int(sid), ctypes.byref(res), ctypes.c_void_p(counts.data_ptr()),
                                              ctypes.c_void_p(s)))
        torch.cuda.synchronize()
        c = counts.cpu().numpy()
        return [{name: t[: int(c[k])].cpu().numpy() for name, t in bufs[k].items()} for k in range(2)]


@dataclass
class Request:
    scene: object
    horizon: int
    arrival_s: float
    want_result: bool = False


class Server:
    """The library's serving loop (tss_server_*) over a pool of `cfg`."""

    def __init__(self, cfg, max_steps_per_launch=8, max_in_flight=2, staging_bytes=1 << 30, arith="exact"):
        self.lib = load_library()
        sc = _abi.TssServerConfig()
        sc.pool = cfg
        sc.max_steps_per_launch = int(max_steps_per_launch)
        sc.max_in_flight = int(max_in_flight)
        sc.staging_bytes = int(staging_bytes)
        h = ctypes.c_void_p()
        check(self.lib.tss_server_create(ctypes.byref(sc), ctypes.byref(h)))
        self.h = h
        if arith not in ("exact", "fast"):
            raise ValueError("arith must be 'exact' or 'fast'")
        check(self.lib.tss_server_set_arith(h, _abi.TSS_ARITH_FAST if arith == "fast" else _abi.TSS_ARITH_EXACT))

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.tss_server_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, requests):
        """Replay `requests` (Request objects) in real time.  Returns (stats, summary,
        results): per-request dicts, the run summary, and for requests that asked for
        it the final state [low, high] (dicts of arrays, scene-local ids)."""
        n = len(requests)
        reqs = (_abi.TssRequest * max(n, 1))()
        stats = (_abi.TssRequestStats * max(n, 1))()
        keep = []
        results = [None] * n
        res_structs = []
        for k, r in enumerate(requests):
            reqs[k].scene = scene_desc(r.scene, keep)
            reqs[k].horizon = int(r.horizon)
            reqs[k].arrival_s = float(r.arrival_s)
            if r.want_result:
                nl = r.scene.n_low
                arrs = []
                rs = _abi.TssSceneResult()
                for s, cap in enumerate((nl, 4 * nl)):
                    m = max(cap, 1)
                    a = {"id": np.zeros(m, np.int32), "pos": np.zeros((m, 2), np.float32),
                         "vel": np.zeros((m, 2), np.float32), "state": np.zeros(m, np.uint8),
                         "dens": np.zeros(m, np.float32), "pres": np.zeros(m, np.float32)}
                    arrs.append(a)
                    rs.cap[s] = cap
                    for name, v in a.items():
                        getattr(rs, name)[s] = v.ctypes.data
                res_structs.append(rs)
                results[k] = (arrs, rs)
                reqs[k].result = ctypes.pointer(rs)
        summ = _abi.TssServeSummary()
        st = self.lib.tss_server_run(self.h, n, reqs, stats, ctypes.byref(summ))
        if st != _abi.TSS_OK:
            buf = ctypes.create_string_buffer(512)
            self.lib.tss_server_last_error(self.h, buf, 512)
            raise TssError(st, "tss_server_run: " + buf.value.decode(errors="replace"))
        out_stats = []
        for k in range(n):
            s = stats[k]
            out_stats.append({"arrival_s": s.arrival_s, "admit_s": s.admit_s, "done_s": s.done_s,
                              "first_step": s.first_step, "status": s.status, "n_low": s.n_low, "n_high": s.n_high})
        out_res = [None] * n
        for k in range(n):
            if results[k] is None:
                continue
            arrs, rs = results[k]
            out_res[k] = [{name: v[: rs.n[s]] for name, v in arrs[s].items()} for s in range(2)]
        return out_stats, summ.as_dict(), out_res


def latency_summary(stats):
    """p50/p99/mean completion latency (done - arrival) of the served requests
    (those that completed, including any whose scene went non-finite)."""
    lat = np.array([s["done_s"] - s["arrival_s"] for s in stats if s["status"] in (_abi.TSS_OK, _abi.TSS_NUMERIC)])
    if lat.size == 0:
        return {"p50_s": None, "p99_s": None, "mean_s": None, "served": 0}
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "served": int(lat.size)}


def fifo_schedule(arrivals, service):
    """Completion times of one-at-a-time, first-come-first-served service: each
    request starts when it has arrived and the previous one is done."""
    t = 0.0
    done = np.zeros(len(arrivals))
    for k in np.argsort(np.asarray(arrivals), kind="stable"):
        t = max(t, arrivals[k]) + service[k]
        done[k] = t
    return done
