"""ORACLE -- test infrastructure only.

Python handles for
  * Oracle: the CPU restatement of the two-scale WCSPH step (tss_oracle.cpp),
    FP32 (the reference's arithmetic, bit for bit) or FP64 (error reference);
  * RefCPU: the reference's own kernel source compiled for the CPU and driven by
    a headless harness (refcpu/), available only where the reference checkout is;
  * RefGPU: the reference's own kernels compiled for sm_103a (a cubin built where
    the checkout is) run on the GPU by a headless restatement of AdvanceTS
    (refgpu/), for timing the reference beside the library.

Only the tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg and
reference arm import this package; the product (twoscalesplit_gb300) never does.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_ORC = None
_REF = None


def _orc_lib():
    global _ORC
    if _ORC is None:
        path = _build.build_oracle()
        lib = ctypes.CDLL(path)
        vp, i, f = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        lib.orc_create.restype = vp
        lib.orc_create.argtypes = [vp, i, f, f, i, i, i, vp, f]
        lib.orc_destroy.argtypes = [vp]
        lib.orc_set_scale.argtypes = [vp, i, i, vp, vp, vp, vp, vp, vp]
        lib.orc_set_fresh.argtypes = [vp, i, vp]
        lib.orc_set_steps.argtypes = [vp, ctypes.c_longlong]
        lib.orc_set_want_scale.argtypes = [vp, i]
        lib.orc_splat.argtypes = [vp, i, i, i, vp, vp, i, f, vp, f, vp]
        lib.orc_step.argtypes = [vp]
        lib.orc_get.argtypes = [vp, i, ctypes.c_char_p, vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
        lib.orc_set_threads.argtypes = [i]
        lib.orc_max_threads.restype = i
        lib.orc_grid.argtypes = [i, vp, vp, f, f, f, i, i, vp, vp]
        lib.orc_eval.restype = ctypes.c_double
        lib.orc_eval.argtypes = [i, ctypes.c_double, ctypes.c_double, ctypes.c_double, i]
        _ORC = lib
    return _ORC


def _ref_lib():
    global _REF
    if _REF is None:
        path = _build.build_refcpu()
        if path is None:
            return None
        lib = ctypes.CDLL(path)
        vp, i, f = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        lib.ref_create.restype = vp
        lib.ref_create.argtypes = [vp, i, f, i, f, i, vp, f]
        lib.ref_destroy.argtypes = [vp]
        lib.ref_set_scale.argtypes = [vp, i, i, vp, vp, vp, vp, vp, vp]
        lib.ref_set_fresh.argtypes = [vp, i, vp]
        lib.ref_step.argtypes = [vp]
        lib.ref_get.argtypes = [vp, i, ctypes.c_char_p, vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
        lib.ref_grid.argtypes = [vp, i, vp, vp, vp, vp, vp, vp]
        lib.ref_older_children.argtypes = [f, i, f, f, f, f, vp, vp]
        _REF = lib
    return _REF


def ref_older_children(r, pid, pos, vel):
    """The older snapshot's own child placement (initSubParticlesAndAddToList,
    TwoScale2D-master/TwoScale2D/WCSPHSolver.cu:813-867) compiled for the CPU: the
    four children's positions and velocities (4 x 2 float32 each)."""
    lib = _ref_lib()
    p8 = np.zeros(8, np.float32)
    v8 = np.zeros(8, np.float32)
    lib.ref_older_children(float(r), int(pid), float(pos[0]), float(pos[1]), float(vel[0]), float(vel[1]),
                           _p(p8), _p(v8))
    return p8.reshape(4, 2), v8.reshape(4, 2)


def refcpu_available():
    return _ref_lib() is not None


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def set_threads(n):
    _orc_lib().orc_set_threads(int(n))


def max_threads():
    return _orc_lib().orc_max_threads()


def kernel_eval(what, d, r, cs=0.0, precision=64):
    """0: W_r(d); 1: x-component of grad W_r at (d, 0); 2: wall weight Gamma_r(d)."""
    return _orc_lib().orc_eval(int(what), float(d), float(r), float(cs), int(precision))


def grid(pos, ids, origin, cell, dims):
    """(cell, id) order and dense cell offsets, FP32 (orc_grid)."""
    lib = _orc_lib()
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    ids = np.ascontiguousarray(ids, dtype=np.int32)
    n = ids.shape[0]
    order = np.empty(n, np.int32)
    off = np.empty(dims[0] * dims[1] + 1, np.int32)
    lib.orc_grid(n, _p(pos), _p(ids), origin[0], origin[1], cell, dims[0], dims[1], _p(order), _p(off))
    return order, off


def splat(view, width, height, pos, dens=None, nvalid=None, rest_density=1000.0, rgb=None, point_size=0.005,
          img=None):
    """The CPU restatement of the headless splat renderer: blends the particles, in
    order, into img (height x width x 4 float32, row 0 at the bottom; a new image
    cleared to (1, 1, 1, 0) when None) and returns it."""
    lib = _orc_lib()
    if img is None:
        img = np.zeros((height, width, 4), np.float32)
        img[..., :3] = 1.0
    img = np.ascontiguousarray(img, np.float32)
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 2)
    n = pos.shape[0]
    v = np.asarray(view, np.float32)
    d = None if dens is None else np.ascontiguousarray(dens, np.float32)
    c = None if rgb is None else np.asarray(rgb, np.float32)
    lib.orc_splat(_p(v), width, height, n, _p(pos), _p(d), n if nvalid is None else int(nvalid),
                  float(rest_density), _p(c), float(point_size), _p(img))
    return img


class Oracle:
    """One scene in the CPU oracle.  State arrays are in list order."""

    def __init__(self, scene, precision=32):
        self.lib = _orc_lib()
        self.scene = scene
        self.precision = precision
        walls = np.ascontiguousarray(scene.wall_pos, dtype=np.float32)
        self._cfg = scene.config
        self.h = self.lib.orc_create(ctypes.byref(scene.config), precision, scene.mass_low, scene.mass_high,
                                     scene.n_low, scene.cap_high, walls.shape[0], _p(walls), scene.mass_wall)
        n = scene.n_low
        self.set_scale(0, np.arange(n, dtype=np.int32), scene.low_pos, scene.low_vel, np.zeros(n, np.uint8))
        self.set_scale(1, np.zeros(0, np.int32), np.zeros((0, 2)), np.zeros((0, 2)), np.zeros(0, np.uint8))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def set_scale(self, scale, ids, pos, vel, state, dens=None, pres=None):
        ids = np.ascontiguousarray(ids, np.int32)
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1)
        vel = np.ascontiguousarray(vel, np.float64).reshape(-1)
        state = np.ascontiguousarray(state, np.uint8)
        dens = None if dens is None else np.ascontiguousarray(dens, np.float64)
        pres = None if pres is None else np.ascontiguousarray(pres, np.float64)
        st = self.lib.orc_set_scale(self.h, scale, ids.shape[0], _p(ids), _p(pos), _p(vel), _p(state),
                                    _p(dens), _p(pres))
        if st != 0:
            raise ValueError(f"orc_set_scale failed ({st})")

    def set_fresh(self, parents):
        parents = np.ascontiguousarray(parents, np.int32)
        self.lib.orc_set_fresh(self.h, parents.shape[0], _p(parents))

    def set_steps(self, steps):
        """Steps taken so far (the moving region of interest's step index)."""
        self.lib.orc_set_steps(self.h, int(steps))

    def set_want_scale(self, on=True):
        """Compute each acceleration's error scale in the next steps: the sum of the
        magnitudes of its summands (get(scale, "acc_scale"))."""
        self.lib.orc_set_want_scale(self.h, 1 if on else 0)

    def step(self):
        return self.lib.orc_step(self.h)

    _INT = {"id", "sorted_src", "sorted_id", "cell_off", "split", "fresh", "wall_cell_off"}
    _U8 = {"state"}

    def get(self, scale, name):
        n = ctypes.c_size_t(0)
        self.lib.orc_get(self.h, scale, name.encode(), None, 0, ctypes.byref(n))
        if name in self._INT:
            out = np.empty(n.value, np.int32)
        elif name in self._U8:
            out = np.empty(n.value, np.uint8)
        else:
            out = np.empty(n.value, np.float64)
        self.lib.orc_get(self.h, scale, name.encode(), _p(out), n.value, ctypes.byref(n))
        if name in ("pos", "vel", "acc"):
            out = out.reshape(-1, 2)
        return out

    def state(self, scale):
        return {k: self.get(scale, k) for k in ("id", "pos", "vel", "state", "dens_state", "pres_state")}

    def load_state(self, scale, st):
        self.set_scale(scale, st["id"], st["pos"], st["vel"], st["state"], st.get("dens_state"),
                       st.get("pres_state"))


def ref_grid(config, pos_by_slot, ids):
    """The reference's own grid build (hash, stable sort, cell start/end), CPU."""
    lib = _ref_lib()
    pos = np.ascontiguousarray(pos_by_slot, np.float32)
    ids = np.ascontiguousarray(ids, np.int32)
    n = ids.shape[0]
    cells = config.dims_low[0] * config.dims_low[1]
    sid = np.empty(n, np.int32)
    sh = np.empty(n, np.int32)
    cs = np.empty(cells, np.int32)
    ce = np.empty(cells, np.int32)
    lib.ref_grid(ctypes.byref(config), n, _p(pos), _p(ids), _p(sid), _p(sh), _p(cs), _p(ce))
    return sid, sh, cs, ce


class RefCPU:
    """The reference's kernels run on the CPU (slot-indexed arrays, as the reference)."""

    def __init__(self, scene):
        self.lib = _ref_lib()
        if self.lib is None:
            raise RuntimeError("reference checkout not available")
        walls = np.ascontiguousarray(scene.wall_pos, dtype=np.float32)
        self.scene = scene
        self.h = self.lib.ref_create(ctypes.byref(scene.config), scene.n_low, scene.mass_low, 4 * scene.n_low,
                                     scene.mass_high, walls.shape[0], _p(walls), scene.mass_wall)
        n = scene.n_low
        self.set_scale(0, np.arange(n, dtype=np.int32), scene.low_pos, scene.low_vel, np.zeros(n, np.uint8))
        self.set_scale(1, np.zeros(0, np.int32), np.zeros((0, 2)), np.zeros((0, 2)), np.zeros(0, np.uint8))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_destroy(self.h)
            self.h = None

    def set_scale(self, scale, ids, pos, vel, state, dens=None, pres=None):
        ids = np.ascontiguousarray(ids, np.int32)
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1)
        vel = np.ascontiguousarray(vel, np.float32).reshape(-1)
        state = np.ascontiguousarray(state, np.uint8)
        dens = None if dens is None else np.ascontiguousarray(dens, np.float32)
        pres = None if pres is None else np.ascontiguousarray(pres, np.float32)
        st = self.lib.ref_set_scale(self.h, scale, ids.shape[0], _p(ids), _p(pos), _p(vel), _p(state),
                                    _p(dens), _p(pres))
        if st != 0:
            raise ValueError("ref_set_scale failed")

    def set_fresh(self, parents):
        parents = np.ascontiguousarray(parents, np.int32)
        self.lib.ref_set_fresh(self.h, parents.shape[0], _p(parents))

    def step(self):
        self.lib.ref_step(self.h)

    _U8 = {"state"}
    _F = {"pos", "vel", "acc", "dens", "pres"}

    def get(self, scale, name):
        n = ctypes.c_size_t(0)
        self.lib.ref_get(self.h, scale, name.encode(), None, 0, ctypes.byref(n))
        dt = np.uint8 if name in self._U8 else (np.float32 if name in self._F else np.int32)
        out = np.empty(n.value, dt)
        self.lib.ref_get(self.h, scale, name.encode(), _p(out), n.value, ctypes.byref(n))
        if name in ("pos", "vel", "acc"):
            out = out.reshape(-1, 2)
        return out


_REFGPU = None


def _refgpu_lib():
    global _REFGPU
    if _REFGPU is None:
        cubin = _build.build_refgpu_cubin()
        if cubin is None:
            return None
        try:
            lib = ctypes.CDLL(_build.build_refgpu_launcher())
        except OSError:  # no CUDA driver on this machine
            return None
        vp, i, f = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        lib.refgpu_create.restype = vp
        lib.refgpu_create.argtypes = [ctypes.c_char_p, vp, i, vp, vp, f, i, f, i, vp, f, ctypes.c_char_p, i]
        lib.refgpu_destroy.argtypes = [vp]
        lib.refgpu_step.restype = i
        lib.refgpu_step.argtypes = [vp, i, ctypes.c_char_p, i]
        lib.refgpu_counts.argtypes = [vp, vp]
        lib.refgpu_state.restype = i
        lib.refgpu_state.argtypes = [vp, i, vp, vp, vp, i]
        lib.refgpu_set_state.restype = i
        lib.refgpu_set_state.argtypes = [vp, vp, vp, vp, i, vp, vp, vp, vp, ctypes.c_char_p, i]
        _REFGPU = (lib, cubin)
    return _REFGPU


def refgpu_available():
    return _refgpu_lib() is not None


class RefGPU:
    """The reference's own kernels rebuilt for sm_103a (refgpu/), run on the GPU by
    a headless restatement of AdvanceTS; slot-indexed arrays, as the reference."""

    def __init__(self, scene, cap_high=None):
        got = _refgpu_lib()
        if got is None:
            raise RuntimeError("the reference's kernels for sm_103a are not built (no reference checkout)")
        self.lib, cubin = got
        self.scene = scene
        lp = np.ascontiguousarray(scene.low_pos, np.float32).reshape(-1)
        lv = None if scene.low_vel is None else np.ascontiguousarray(scene.low_vel, np.float32).reshape(-1)
        wp = np.ascontiguousarray(scene.wall_pos, np.float32).reshape(-1)
        err = ctypes.create_string_buffer(512)
        self.cap_high = int(cap_high if cap_high is not None else scene.cap_high)
        self.h = self.lib.refgpu_create(cubin.encode(), ctypes.byref(scene.config), scene.n_low, _p(lp), _p(lv),
                                        scene.mass_low, self.cap_high, scene.mass_high, scene.n_wall, _p(wp),
                                        scene.mass_wall, err, 512)
        if not self.h:
            raise RuntimeError("refgpu_create: " + err.value.decode(errors="replace"))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.refgpu_destroy(self.h)
            self.h = None

    def step(self, n=1):
        err = ctypes.create_string_buffer(512)
        if self.lib.refgpu_step(self.h, int(n), err, 512) != 0:
            raise RuntimeError("refgpu_step: " + err.value.decode(errors="replace"))

    def set_state(self, low, high):
        """Replace the state with another solver's (list-order dicts of id, pos, vel,
        state per scale, as Solver.download returns them): every low-res slot must be
        present; split parents (state 1) form the transient list."""
        n = self.scene.n_low
        lid = np.asarray(low["id"], np.int64)
        if lid.shape[0] != n or not np.array_equal(np.sort(lid), np.arange(n)):
            raise ValueError("set_state needs every low-res slot")
        lp = np.zeros((n, 2), np.float32)
        lv = np.zeros((n, 2), np.float32)
        ls = np.zeros(n, np.uint8)
        lp[lid], lv[lid], ls[lid] = low["pos"], low["vel"], low["state"]
        hid = np.ascontiguousarray(high["id"], np.int32)
        hp = np.ascontiguousarray(high["pos"], np.float32)
        hv = np.ascontiguousarray(high["vel"], np.float32)
        hs = np.ascontiguousarray(high["state"], np.uint8)
        err = ctypes.create_string_buffer(512)
        if self.lib.refgpu_set_state(self.h, _p(lp), _p(lv), _p(ls), hid.shape[0], _p(hid), _p(hp), _p(hv), _p(hs),
                                     err, 512) != 0:
            raise RuntimeError("refgpu_set_state: " + err.value.decode(errors="replace"))

    def counts(self):
        c = np.zeros(3, np.int32)
        self.lib.refgpu_counts(self.h, _p(c))
        return {"n_low": int(c[0]), "n_high": int(c[1]), "n_transient_low": int(c[2])}

    def state(self, scale):
        """Slot-indexed positions, velocities and states of a scale (capacity-sized)."""
        cap = self.scene.n_low if scale == 0 else self.cap_high
        pos = np.zeros((max(cap, 1), 2), np.float32)
        vel = np.zeros((max(cap, 1), 2), np.float32)
        st = np.zeros(max(cap, 1), np.uint8)
        if self.lib.refgpu_state(self.h, scale, _p(pos), _p(vel), _p(st), cap) != 0:
            raise RuntimeError("refgpu_state failed")
        return pos[:cap], vel[:cap], st[:cap]
