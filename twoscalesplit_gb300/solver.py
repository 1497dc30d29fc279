"""Host-side mirror of the reference's solver interface over the C ABI.

`Solver` is a thin handle on tss_solver (include/tss.h).  `WCSPHConfig`,
`ParticleSystem`, `CreateParticleBox`, `CreateParticleBoxCanvas` and `WCSPHSolver`
keep the names, argument meaning and error behaviour of the reference classes
(TwoScale2D/WCSPHSolver.h:14-131, TwoScale2D/ParticleSystem.h:17-86), so code
written against the reference reads the same; the device work all happens in the
CUDA library, which must be present (there is no CPU path).
"""
import ctypes

import numpy as np

from . import _abi
from ._abi import (TSS_SCALE_HIGH, TSS_SCALE_LOW, TssBuffers, TssCounts, TssScaleState, check, fptr, iptr,
                   load_library, u8ptr)


class Solver:
    """One two-scale scene resident on the GPU."""

    def __init__(self, config, low_pos, mass_low, cap_high, mass_high, wall_pos, mass_wall, low_vel=None):
        self.lib = load_library()
        self.config = config
        low_pos = np.ascontiguousarray(low_pos, np.float32).reshape(-1, 2)
        low_vel = None if low_vel is None else np.ascontiguousarray(low_vel, np.float32).reshape(-1, 2)
        wall_pos = np.ascontiguousarray(wall_pos, np.float32).reshape(-1, 2)
        self.n_low = low_pos.shape[0]
        self.cap_high = int(cap_high)
        h = ctypes.c_void_p()
        st = self.lib.tss_solver_create(ctypes.byref(config), self.n_low, fptr(low_pos), fptr(low_vel),
                                        float(mass_low), self.cap_high, float(mass_high), wall_pos.shape[0],
                                        fptr(wall_pos), float(mass_wall), ctypes.byref(h))
        check(st)
        self.h = h

    @classmethod
    def from_scene(cls, scene):
        return cls(scene.config, scene.low_pos, scene.mass_low, scene.cap_high, scene.mass_high, scene.wall_pos,
                   scene.mass_wall, low_vel=scene.low_vel)

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.tss_solver_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        check(st, self.h, self.lib)

    def step(self, n=1, stream=None):
        """Enqueue n steps on a cudaStream_t handle (int; None or 0 = the default stream)."""
        self._check(self.lib.tss_solver_step(self.h, int(n), ctypes.c_void_p(stream) if stream else None))

    def sync(self):
        self._check(self.lib.tss_solver_sync(self.h))

    def counts(self):
        c = TssCounts()
        self._check(self.lib.tss_solver_counts(self.h, ctypes.byref(c)))
        return {"n_low": c.n_low, "n_high": c.n_high, "n_transient_low": c.n_transient_low,
                "n_split_last": c.n_split_last, "steps": c.steps, "error_bits": c.error_bits,
                "n_removed_last": c.n_removed_last, "total_split": c.total_split, "total_removed": c.total_removed}

    def download(self, scale):
        c = self.counts()
        n = c["n_low"] if scale == TSS_SCALE_LOW else c["n_high"]
        out = {"id": np.zeros(n, np.int32), "pos": np.zeros((n, 2), np.float32), "vel": np.zeros((n, 2), np.float32),
               "state": np.zeros(n, np.uint8), "dens": np.zeros(n, np.float32), "pres": np.zeros(n, np.float32)}
        s = TssScaleState(n, iptr(out["id"]), fptr(out["pos"]), fptr(out["vel"]), u8ptr(out["state"]),
                          fptr(out["dens"]), fptr(out["pres"]))
        self._check(self.lib.tss_solver_download(self.h, scale, ctypes.byref(s)))
        return out

    def upload(self, scale, st):
        ids = np.ascontiguousarray(st["id"], np.int32)
        pos = np.ascontiguousarray(st["pos"], np.float32).reshape(-1, 2)
        vel = np.ascontiguousarray(st["vel"], np.float32).reshape(-1, 2)
        state = np.ascontiguousarray(st["state"], np.uint8)
        dens = st.get("dens")
        pres = st.get("pres")
        dens = None if dens is None else np.ascontiguousarray(dens, np.float32)
        pres = None if pres is None else np.ascontiguousarray(pres, np.float32)
        s = TssScaleState(ids.shape[0], iptr(ids), fptr(pos), fptr(vel), u8ptr(state), fptr(dens), fptr(pres))
        self._check(self.lib.tss_solver_upload(self.h, scale, ctypes.byref(s)))

    def get_fresh(self):
        n = ctypes.c_int(0)
        self._check(self.lib.tss_solver_get_fresh(self.h, ctypes.byref(n), None))
        out = np.zeros(n.value, np.int32)
        self._check(self.lib.tss_solver_get_fresh(self.h, ctypes.byref(n), iptr(out)))
        return out

    def set_fresh(self, parents):
        parents = np.ascontiguousarray(parents, np.int32)
        self._check(self.lib.tss_solver_set_fresh(self.h, parents.shape[0], iptr(parents)))

    _DTYPES = {_abi.TSS_BUF_SORTED_ID: np.int32, _abi.TSS_BUF_CELL_OFFSET: np.int32, _abi.TSS_BUF_DENSITY: np.float32,
               _abi.TSS_BUF_PRESSURE: np.float32, _abi.TSS_BUF_ACCEL: np.float32, _abi.TSS_BUF_SPLIT: np.int32,
               _abi.TSS_BUF_WALL_CELL_OFFSET: np.int32}

    def copy(self, scale, which):
        n = ctypes.c_size_t(0)
        self._check(self.lib.tss_solver_copy(self.h, scale, which, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, self._DTYPES[which])
        self._check(self.lib.tss_solver_copy(self.h, scale, which, out.ctypes.data_as(ctypes.c_void_p), n.value,
                                             ctypes.byref(n)))
        if which == _abi.TSS_BUF_ACCEL:
            out = out.reshape(-1, 2)
        return out

    def profile(self, enable=True):
        self._check(self.lib.tss_solver_profile(self.h, 1 if enable else 0))

    def stage_times(self):
        """Device ms of each stage of the last step (profiling must be on)."""
        ms = np.zeros(_abi.TSS_NUM_STAGES, np.float32)
        self._check(self.lib.tss_solver_stage_times(self.h, fptr(ms), ms.shape[0]))
        return dict(zip(_abi.STAGE_NAMES, ms.tolist()))

    def read_positions(self, host_low, host_high, counts, stream=None):
        """Enqueue the asynchronous position read-back (tss_solver_read_positions)
        into page-locked torch CPU tensors: host_low (cap_low, 2) and host_high
        (cap_high, 2) float32, counts (2,) int32.  Wait on the stream (or an event
        recorded after it) before reading them."""
        self._check(self.lib.tss_solver_read_positions(
            self.h, ctypes.c_void_p(host_low.data_ptr()), int(host_low.shape[0]),
            ctypes.c_void_p(host_high.data_ptr()), int(host_high.shape[0]), ctypes.c_void_p(counts.data_ptr()),
            ctypes.c_void_p(stream) if stream else None))

    def read_positions_async(self, host_low, host_high, counts, stream=None):
        """The read-back overlapped with the following steps
        (tss_solver_read_positions_async): returns a ticket; read the buffers after
        read_wait(ticket)."""
        t = ctypes.c_int64(0)
        self._check(self.lib.tss_solver_read_positions_async(
            self.h, ctypes.c_void_p(host_low.data_ptr()), int(host_low.shape[0]),
            ctypes.c_void_p(host_high.data_ptr()), int(host_high.shape[0]), ctypes.c_void_p(counts.data_ptr()),
            ctypes.c_void_p(stream) if stream else None, ctypes.byref(t)))
        return t.value

    def read_wait(self, ticket):
        """Blocks until the read-back with this ticket has written host memory."""
        self._check(self.lib.tss_solver_read_wait(self.h, ctypes.c_int64(ticket)))

    @property
    def launch(self):
        """Launch shape of the gathers: {gather: {"threads": t, "persistent": bool}}."""
        l = _abi.TssLaunch()
        self._check(self.lib.tss_solver_get_launch(self.h, ctypes.byref(l)))
        return l.as_dict()

    def set_launch(self, shape):
        self._check(self.lib.tss_solver_set_launch(self.h, ctypes.byref(_abi.TssLaunch.from_dict(shape))))

    @property
    def arith(self):
        """The gathers' arithmetic: "exact" (the reference's bits, the default) or
        "fast" (within the step's 1e-5 tolerance; tss_solver_set_arith)."""
        m = ctypes.c_int(0)
        self._check(self.lib.tss_solver_get_arith(self.h, ctypes.byref(m)))
        return "fast" if m.value == _abi.TSS_ARITH_FAST else "exact"

    def set_arith(self, mode):
        if mode not in ("exact", "fast"):
            raise ValueError("arith must be 'exact' or 'fast'")
        self._check(self.lib.tss_solver_set_arith(
            self.h, _abi.TSS_ARITH_FAST if mode == "fast" else _abi.TSS_ARITH_EXACT))

    def autotune(self, steps_per_trial=3):
        """Time every candidate launch shape on this handle's own steps and install
        the fastest per gather (tss_solver_autotune).  The trial steps advance the
        state (results do not depend on the shape).  Returns (shape, steps taken)."""
        l = _abi.TssLaunch()
        n = ctypes.c_int(0)
        self._check(self.lib.tss_solver_autotune(self.h, int(steps_per_trial), ctypes.byref(l), ctypes.byref(n)))
        return l.as_dict(), n.value

    def render(self, view, point_sizes=(0.005, 0.003, 0.005), stream=None):
        """One frame (tss_solver_render): a torch CUDA tensor (height, width, 4),
        row 0 at the bottom.  `view` is (xs, ys, xe, ye, width, height)."""
        import torch
        v = _abi.TssView(*[float(x) for x in view[:4]], int(view[4]), int(view[5]))
        img = torch.empty((v.height, v.width, 4), dtype=torch.float32, device="cuda")
        ps = np.asarray(point_sizes, np.float32)
        s = stream if stream else torch.cuda.current_stream().cuda_stream
        self._check(self.lib.tss_solver_render(self.h, ctypes.byref(v), fptr(ps), ctypes.c_void_p(img.data_ptr()),
                                               ctypes.c_void_p(s)))
        return img

    def device_buffers(self):
        b = TssBuffers()
        self._check(self.lib.tss_solver_device_buffers(self.h, ctypes.byref(b)))
        return b


class Batch(Solver):
    """Many independent scenes advanced together (tss_batch_create): one grid build
    and one launch of each kernel per step for all of them.  Each scene's results
    equal those of the same scene run alone."""

    def __init__(self, scenes, cap_high=None):
        self.lib = load_library()
        self.scenes = list(scenes)
        self._keep = []
        descs = (_abi.TssSceneDesc * len(self.scenes))()
        for k, sc in enumerate(self.scenes):
            lp = np.ascontiguousarray(sc.low_pos, np.float32).reshape(-1, 2)
            lv = np.ascontiguousarray(sc.low_vel, np.float32).reshape(-1, 2)
            wp = np.ascontiguousarray(sc.wall_pos, np.float32).reshape(-1, 2)
            self._keep += [lp, lv, wp, sc.config]
            descs[k] = _abi.TssSceneDesc(ctypes.pointer(sc.config), lp.shape[0], fptr(lp), fptr(lv), sc.mass_low,
                                         sc.mass_high, wp.shape[0], fptr(wp), sc.mass_wall)
        self.cap_high = int(cap_high if cap_high is not None else sum(sc.cap_high for sc in self.scenes))
        self.n_low = sum(sc.n_low for sc in self.scenes)
        h = ctypes.c_void_p()
        check(self.lib.tss_batch_create(len(self.scenes), descs, self.cap_high, ctypes.byref(h)))
        self.h = h
        self._keep = []

    def scene_counts(self):
        n = len(self.scenes)
        lo = np.zeros(n, np.int32)
        hi = np.zeros(n, np.int32)
        self._check(self.lib.tss_solver_scene_counts(self.h, iptr(lo), iptr(hi)))
        return lo, hi

    def download_scene(self, scene, scale):
        lo, hi = self.scene_counts()
        n = int(lo[scene] if scale == TSS_SCALE_LOW else hi[scene])
        out = {"id": np.zeros(n, np.int32), "pos": np.zeros((n, 2), np.float32), "vel": np.zeros((n, 2), np.float32),
               "state": np.zeros(n, np.uint8), "dens": np.zeros(n, np.float32), "pres": np.zeros(n, np.float32)}
        st = TssScaleState(n, iptr(out["id"]), fptr(out["pos"]), fptr(out["vel"]), u8ptr(out["state"]),
                           fptr(out["dens"]), fptr(out["pres"]))
        self._check(self.lib.tss_solver_download_scene(self.h, scene, scale, ctypes.byref(st)))
        return out


# ---------------------------------------------------------------------------
# Reference-shaped interface
# ---------------------------------------------------------------------------
class WCSPHConfig:
    """WCSPHConfig(xs, ys, xe, ye, effectiveRadius, effectiveRadiusHigh, restDensity,
    taitCoeff, speedSound, alpha, tensionCoefficient, timeStep); raises like the
    reference (WCSPHSolver.cu:2312-2316) on an empty domain."""

    def __init__(self, xs, ys, xe, ye, effectiveRadius, effectiveRadiusHigh, restDensity, taitCoeff, speedSound,
                 alpha, tensionCoefficient, timeStep):
        self.cfg = _abi.config_init(xs, ys, xe, ye, effectiveRadius, effectiveRadiusHigh, restDensity, taitCoeff,
                                    speedSound, alpha, tensionCoefficient, timeStep)

    def __getattr__(self, name):
        aliases = {"DomainOrigin": "domain_origin", "DomainEnd": "domain_end", "DomainDimensions": "dims_low",
                   "DomainDimensionsHigh": "dims_high", "EffectiveRadius": "r_low", "EffectiveRadiusHigh": "r_high",
                   "RestDensity": "rest_density", "TaitCoeffitient": "tait_b", "SpeedSound": "speed_sound",
                   "Alpha": "alpha", "TensionCoefficient": "tension", "TimeStep": "dt"}
        if name in aliases:
            v = getattr(self.cfg, aliases[name])
            return list(v) if hasattr(v, "__len__") else v
        raise AttributeError(name)


class ParticleSystem:
    """ParticleSystem(maxParticles, mass) (ParticleSystem.h:17-78).  Host-side until a
    WCSPHSolver takes it; afterwards its accessors read the solver's state."""

    def __init__(self, maxParticles, mass):
        self._max = int(maxParticles)
        self._mass = float(mass)
        self._pos = []
        self._solver = None
        self._scale = None

    def PushParticle(self, position):
        if self._solver is not None:
            raise RuntimeError("Positions is not mapped")
        if len(self._pos) >= self._max:
            raise RuntimeError("particle system is full")
        self._pos.append((float(position[0]), float(position[1])))

    def GetMass(self):
        return self._mass

    def GetMaxParticles(self):
        return self._max

    def GetNumParticles(self):
        if self._solver is None:
            return len(self._pos)
        c = self._solver._s.counts()
        return c["n_low"] if self._scale == TSS_SCALE_LOW else c["n_high"]

    def _state(self):
        if self._solver is None:
            n = len(self._pos)
            return {"id": np.arange(n, dtype=np.int32), "pos": np.array(self._pos, np.float32).reshape(-1, 2)}
        return self._solver._s.download(self._scale)

    def Positions(self):
        return self._state()["pos"]

    def Velocities(self):
        return self._state().get("vel")

    def Densities(self):
        return self._state().get("dens")

    def Pressures(self):
        return self._state().get("pres")

    def ParticleIDs(self):
        return self._state()["id"]

    def host_positions(self):
        return np.array(self._pos, np.float32).reshape(-1, 2)


def CreateParticleBox(xs, ys, dx, dimX, dimY, particleMass):
    """ParticleSystem.cpp:123-148."""
    from .scenes import particle_box
    ps = ParticleSystem(dimX * dimY, particleMass)
    ps._pos = [tuple(p) for p in particle_box(xs, ys, dx, dimX, dimY).tolist()]
    return ps


def CreateParticleBoxCanvas(xs, ys, dx, dimX, dimY, offX, offY, particleMass):
    """ParticleSystem.cpp:150-179."""
    from .scenes import particle_box_canvas
    p = particle_box_canvas(xs, ys, dx, dimX, dimY, offX, offY)
    ps = ParticleSystem(p.shape[0], particleMass)
    ps._pos = [tuple(q) for q in p.tolist()]
    return ps


class WCSPHSolver:
    """WCSPHSolver(config, fluidParticles, fluidParticlesHigh, boundaryParticles)
    (WCSPHSolver.h:37-131).  Bind() uploads everything and builds the wall grid;
    AdvanceTS() advances one step.  Advance()/AdvanceHigh() are empty, as in the
    reference (WCSPHSolver.cu:2649-2724)."""

    def __init__(self, config, fluidParticles, fluidParticlesHigh, boundaryParticles):
        self._config = config.cfg if isinstance(config, WCSPHConfig) else config
        self._low, self._high, self._walls = fluidParticles, fluidParticlesHigh, boundaryParticles
        self._s = None

    def Bind(self):
        if self._s is not None:
            return
        lp = self._low.host_positions()
        self._s = Solver(self._config, lp, self._low.GetMass(), self._high.GetMaxParticles(), self._high.GetMass(),
                         self._walls.host_positions(), self._walls.GetMass())
        self._low._solver, self._low._scale = self, TSS_SCALE_LOW
        self._high._solver, self._high._scale = self, TSS_SCALE_HIGH

    def Unbind(self):
        pass

    def AdvanceTS(self):
        if self._s is None:
            self.Bind()
        self._s.step(1)

    def Advance(self):
        pass

    def AdvanceHigh(self):
        pass

    @property
    def solver(self):
        return self._s
