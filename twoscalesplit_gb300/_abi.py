"""ctypes view of the C ABI declared in include/tss.h, and the library loader.

The shared library (libtss.so, built in-tree by twoscalesplit_gb300.build) holds
the sm_103a kernels and the host solver.  There is no CPU fallback: every call
that needs the library raises TssError when it cannot be loaded.
"""
import ctypes
import math
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "libtss.so")

TSS_OK = 0
TSS_INVALID_ARG = 1
TSS_OOM = 2
TSS_CUDA_ERROR = 3
TSS_CAPACITY = 4
TSS_NUMERIC = 5
TSS_GRID_INDEX = 6
TSS_NO_DEVICE = 7
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "CUDA_ERROR", 4: "CAPACITY",
                5: "NUMERIC", 6: "GRID_INDEX", 7: "NO_DEVICE"}

TSS_FLAG_Q1_COMPAT = 0x1
TSS_FLAG_MERGE = 0x2
TSS_FLAG_TETHER_GUARD = 0x4
TSS_FLAG_OLDER_PLACEMENT = 0x8
TSS_SCALE_LOW = 0
TSS_SCALE_HIGH = 1

TSS_BUF_SORTED_ID = 0
TSS_BUF_CELL_OFFSET = 1
TSS_BUF_DENSITY = 2
TSS_BUF_PRESSURE = 3
TSS_BUF_ACCEL = 4
TSS_BUF_SPLIT = 5
TSS_BUF_WALL_CELL_OFFSET = 6

TSS_NUM_STAGES = 8
STAGE_NAMES = ["grid_high", "grid_low", "relax", "density_high", "density_low", "force_low", "split",
               "force_high"]

TSS_NUM_GATHERS = 4
GATHER_NAMES = ["density_high", "density_low", "force_low", "force_high"]

TSS_ERR_CAPACITY = 0x1
TSS_GRID_NOALLOC_MAX_BYTES = 32 << 20
TSS_ERR_NUMERIC = 0x2
TSS_ERR_GRID_INDEX = 0x4
TSS_ARITH_EXACT = 0
TSS_ARITH_FAST = 1


class TssError(RuntimeError):
    def __init__(self, status, msg=""):
        self.status = status
        super().__init__(f"tss status {STATUS_NAMES.get(status, status)}{': ' + msg if msg else ''}")


class TssConfig(ctypes.Structure):
    """struct tss_config (include/tss.h)."""
    _fields_ = [
        ("domain_origin", ctypes.c_float * 2),
        ("domain_end", ctypes.c_float * 2),
        ("dims_low", ctypes.c_int * 2),
        ("dims_high", ctypes.c_int * 2),
        ("r_low", ctypes.c_float),
        ("r_high", ctypes.c_float),
        ("rest_density", ctypes.c_float),
        ("tait_b", ctypes.c_float),
        ("speed_sound", ctypes.c_float),
        ("alpha", ctypes.c_float),
        ("tension", ctypes.c_float),
        ("dt", ctypes.c_float),
        ("gravity", ctypes.c_float),
        ("roi", ctypes.c_float * 4),
        ("relax_iters", ctypes.c_int),
        ("relax_dt_div", ctypes.c_float),
        ("flags", ctypes.c_uint),
        ("roi_velocity", ctypes.c_float * 2),
    ]

    def as_dict(self):
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out


class TssCounts(ctypes.Structure):
    _fields_ = [("n_low", ctypes.c_int), ("n_high", ctypes.c_int), ("n_transient_low", ctypes.c_int),
                ("n_split_last", ctypes.c_int), ("steps", ctypes.c_longlong), ("error_bits", ctypes.c_uint),
                ("n_removed_last", ctypes.c_int), ("total_split", ctypes.c_longlong),
                ("total_removed", ctypes.c_longlong)]


class TssScaleState(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("id", ctypes.POINTER(ctypes.c_int32)),
                ("pos", ctypes.POINTER(ctypes.c_float)), ("vel", ctypes.POINTER(ctypes.c_float)),
                ("state", ctypes.POINTER(ctypes.c_uint8)), ("dens", ctypes.POINTER(ctypes.c_float)),
                ("pres", ctypes.POINTER(ctypes.c_float))]


class TssSceneDesc(ctypes.Structure):
    _fields_ = [("config", ctypes.POINTER(TssConfig)), ("n_low", ctypes.c_int),
                ("low_pos", ctypes.POINTER(ctypes.c_float)), ("low_vel", ctypes.POINTER(ctypes.c_float)),
                ("mass_low", ctypes.c_float), ("mass_high", ctypes.c_float), ("n_wall", ctypes.c_int),
                ("wall_pos", ctypes.POINTER(ctypes.c_float)), ("mass_wall", ctypes.c_float)]


TSS_POOL_SLOT_PAGE = 256
TSS_POOL_CELL_PAGE = 64
TSS_POOL_WALL_PAGE = 64
TSS_POOL_MAX_SCENES = 65535


class TssPoolConfig(ctypes.Structure):
    """struct tss_pool_config (include/tss.h)."""
    _fields_ = [("low_slots", ctypes.c_int64), ("high_particles", ctypes.c_int64), ("low_cells", ctypes.c_int64),
                ("high_cells", ctypes.c_int64), ("wall_particles", ctypes.c_int64), ("max_scenes", ctypes.c_int32),
                ("relax_iters", ctypes.c_int32)]


class TssFootprint(ctypes.Structure):
    _fields_ = [("low_slots", ctypes.c_int64), ("high_particles", ctypes.c_int64), ("low_cells", ctypes.c_int64),
                ("high_cells", ctypes.c_int64), ("wall_particles", ctypes.c_int64)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class TssSceneResult(ctypes.Structure):
    """struct tss_scene_result: arrays of each scale (0 low, 1 high)."""
    _fields_ = [("cap", ctypes.c_int32 * 2), ("n", ctypes.c_int32 * 2), ("id", ctypes.c_void_p * 2),
                ("pos", ctypes.c_void_p * 2), ("vel", ctypes.c_void_p * 2), ("state", ctypes.c_void_p * 2),
                ("dens", ctypes.c_void_p * 2), ("pres", ctypes.c_void_p * 2)]


class TssServerConfig(ctypes.Structure):
    _fields_ = [("pool", TssPoolConfig), ("max_steps_per_launch", ctypes.c_int32), ("max_in_flight", ctypes.c_int32),
                ("staging_bytes", ctypes.c_int64)]


class TssRequest(ctypes.Structure):
    _fields_ = [("scene", TssSceneDesc), ("horizon", ctypes.c_int32), ("arrival_s", ctypes.c_double),
                ("result", ctypes.POINTER(TssSceneResult))]


class TssRequestStats(ctypes.Structure):
    _fields_ = [("arrival_s", ctypes.c_double), ("admit_s", ctypes.c_double), ("done_s", ctypes.c_double),
                ("first_step", ctypes.c_int64), ("status", ctypes.c_int32), ("n_low", ctypes.c_int32),
                ("n_high", ctypes.c_int32)]


class TssServeSummary(ctypes.Structure):
    _fields_ = [("makespan_s", ctypes.c_double), ("steps", ctypes.c_int64), ("scene_steps", ctypes.c_int64),
                ("low_particle_steps", ctypes.c_double), ("mean_active", ctypes.c_double),
                ("max_active", ctypes.c_int32), ("served", ctypes.c_int32)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class TssView(ctypes.Structure):
    """struct tss_view: display rectangle and image size."""
    _fields_ = [("xs", ctypes.c_float), ("ys", ctypes.c_float), ("xe", ctypes.c_float), ("ye", ctypes.c_float),
                ("width", ctypes.c_int), ("height", ctypes.c_int)]


class TssLaunch(ctypes.Structure):
    """struct tss_launch: threads per block, grid kind and particles per warp of each
    gather kernel."""
    _fields_ = [("threads", ctypes.c_int * TSS_NUM_GATHERS), ("persistent", ctypes.c_int * TSS_NUM_GATHERS),
                ("per_warp", ctypes.c_int * TSS_NUM_GATHERS)]

    def as_dict(self):
        return {g: {"threads": self.threads[k], "persistent": bool(self.persistent[k]),
                    "per_warp": bool(self.per_warp[k])} for k, g in enumerate(GATHER_NAMES)}

    @classmethod
    def from_dict(cls, d):
        l = cls()
        for k, g in enumerate(GATHER_NAMES):
            l.threads[k] = int(d[g]["threads"])
            l.persistent[k] = 1 if d[g]["persistent"] else 0
            l.per_warp[k] = 1 if d[g].get("per_warp", False) else 0
        return l


class TssBuffers(ctypes.Structure):
    _fields_ = [("pos", ctypes.c_void_p * 2), ("vel", ctypes.c_void_p * 2), ("dens", ctypes.c_void_p * 2),
                ("id", ctypes.c_void_p * 2), ("state", ctypes.c_void_p * 2), ("counts", ctypes.c_void_p)]


def config_init(xs, ys, xe, ye, effective_radius, effective_radius_high, rest_density, tait_coeff,
                speed_sound, alpha, tension_coefficient, time_step):
    """Python restatement of tss_config_init (same float32 arithmetic), so host code
    that only needs a configuration does not have to load the CUDA library.
    Mirrors WCSPHConfig::WCSPHConfig (TwoScale2D/WCSPHSolver.cu:2287-2332)."""
    f = np.float32
    if not (f(xs) < f(xe) and f(ys) < f(ye)):
        raise ValueError("Invalid configuration parameters")
    if not (f(effective_radius) > 0 and f(effective_radius_high) > 0):
        raise ValueError("Invalid configuration parameters")
    c = TssConfig()
    c.domain_origin[:] = [xs, ys]
    c.domain_end[:] = [xe, ye]
    for name, r in (("dims_low", effective_radius), ("dims_high", effective_radius_high)):
        dx = np.float32(np.float32(xe) - np.float32(xs)) / np.float32(r)
        dy = np.float32(np.float32(ye) - np.float32(ys)) / np.float32(r)
        getattr(c, name)[:] = [int(math.ceil(np.float32(dx))), int(math.ceil(np.float32(dy)))]
    c.r_low = effective_radius
    c.r_high = effective_radius_high
    c.rest_density = rest_density
    c.tait_b = tait_coeff
    c.speed_sound = speed_sound
    c.alpha = alpha
    c.tension = tension_coefficient
    c.dt = time_step
    c.gravity = 9.81
    c.roi[:] = [0.5, -math.inf, math.inf, math.inf]
    c.relax_iters = 0
    c.relax_dt_div = 10.0
    c.flags = TSS_FLAG_Q1_COMPAT
    c.roi_velocity[:] = [0.0, 0.0]
    return c


_LIB = None


def load_library(path=None):
    """Load libtss.so; raises TssError(TSS_NO_DEVICE...) style errors loudly if absent."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise TssError(TSS_CUDA_ERROR, f"{p} not built (run twoscalesplit_gb300.build.build())")
    lib = ctypes.CDLL(p)
    vp, i, f, u = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_uint
    fp = ctypes.POINTER(ctypes.c_float)
    ip = ctypes.POINTER(ctypes.c_int32)
    cfgp = ctypes.POINTER(TssConfig)
    sig = {
        "tss_config_init": (i, [cfgp, f, f, f, f, f, f, f, f, f, f, f, f]),
        "tss_solver_create": (i, [cfgp, i, fp, fp, f, i, f, i, fp, f, ctypes.POINTER(vp)]),
        "tss_solver_destroy": (None, [vp]),
        "tss_solver_step": (i, [vp, i, vp]),
        "tss_solver_sync": (i, [vp]),
        "tss_solver_counts": (i, [vp, ctypes.POINTER(TssCounts)]),
        "tss_solver_download": (i, [vp, i, ctypes.POINTER(TssScaleState)]),
        "tss_solver_upload": (i, [vp, i, ctypes.POINTER(TssScaleState)]),
        "tss_solver_get_fresh": (i, [vp, ctypes.POINTER(i), ip]),
        "tss_solver_set_fresh": (i, [vp, i, ip]),
        "tss_solver_copy": (i, [vp, i, i, vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
        "tss_solver_device_buffers": (i, [vp, ctypes.POINTER(TssBuffers)]),
        "tss_solver_last_error": (i, [vp, ctypes.c_char_p, i]),
        "tss_solver_profile": (i, [vp, i]),
        "tss_solver_stage_times": (i, [vp, fp, i]),
        "tss_solver_read_positions": (i, [vp, vp, i, vp, i, vp, vp]),
        "tss_solver_read_positions_async": (i, [vp, vp, i, vp, i, vp, vp, ctypes.POINTER(ctypes.c_int64)]),
        "tss_solver_read_wait": (i, [vp, ctypes.c_int64]),
        "tss_solver_get_launch": (i, [vp, ctypes.POINTER(TssLaunch)]),
        "tss_solver_set_launch": (i, [vp, ctypes.POINTER(TssLaunch)]),
        "tss_solver_autotune": (i, [vp, i, ctypes.POINTER(TssLaunch), ctypes.POINTER(i)]),
        "tss_solver_set_arith": (i, [vp, i]),
        "tss_solver_get_arith": (i, [vp, ctypes.POINTER(i)]),
        "tss_status_string": (ctypes.c_char_p, [i]),
        "tss_grid_workspace_size": (i, [i, i, i, ctypes.POINTER(ctypes.c_size_t)]),
        "tss_batch_create": (i, [i, ctypes.POINTER(TssSceneDesc), i, ctypes.POINTER(vp)]),
        "tss_solver_num_scenes": (i, [vp, ctypes.POINTER(i)]),
        "tss_solver_scene_counts": (i, [vp, ip, ip]),
        "tss_solver_download_scene": (i, [vp, i, i, ctypes.POINTER(TssScaleState)]),
        "tss_grid_build": (i, [vp, vp, i, f, f, f, i, i, vp, vp, vp, ctypes.c_size_t, vp]),
        "tss_grid_build_noalloc": (i, [vp, vp, i, f, f, f, i, i, vp, vp, vp]),
        "tss_pool_bytes": (i, [ctypes.POINTER(TssPoolConfig), ctypes.POINTER(ctypes.c_size_t)]),
        "tss_pool_config_for_budget": (i, [ctypes.c_size_t, ctypes.c_double, ctypes.c_double, i, i,
                                           ctypes.POINTER(TssPoolConfig)]),
        "tss_scene_footprint": (i, [ctypes.POINTER(TssSceneDesc), ctypes.POINTER(TssFootprint)]),
        "tss_pool_create": (i, [ctypes.POINTER(TssPoolConfig), ctypes.POINTER(vp)]),
        "tss_pool_admit": (i, [vp, ctypes.POINTER(TssSceneDesc), vp, ctypes.POINTER(i)]),
        "tss_pool_can_admit": (i, [vp, ctypes.POINTER(TssSceneDesc)]),
        "tss_pool_retire": (i, [vp, i, vp]),
        "tss_pool_free": (i, [vp, ctypes.POINTER(TssFootprint)]),
        "tss_pool_extract": (i, [vp, i, ctypes.POINTER(TssSceneResult), vp, vp]),
        "tss_server_create": (i, [ctypes.POINTER(TssServerConfig), ctypes.POINTER(vp)]),
        "tss_server_run": (i, [vp, i, ctypes.POINTER(TssRequest), ctypes.POINTER(TssRequestStats),
                               ctypes.POINTER(TssServeSummary)]),
        "tss_server_destroy": (None, [vp]),
        "tss_server_set_arith": (i, [vp, i]),
        "tss_server_last_error": (i, [vp, ctypes.c_char_p, i]),
        "tss_render_workspace_size": (i, [i, ctypes.POINTER(TssView), f, ctypes.POINTER(ctypes.c_size_t)]),
        "tss_render_clear": (i, [vp, i, i, vp]),
        "tss_render_splats": (i, [ctypes.POINTER(TssView), i, vp, vp, f, fp, f, vp, vp, ctypes.c_size_t, vp]),
        "tss_solver_render": (i, [vp, ctypes.POINTER(TssView), fp, vp, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    del u
    if path is None:
        _LIB = lib
    return lib


def check(status, solver=None, lib=None):
    if status != TSS_OK:
        msg = ""
        if solver is not None and lib is not None:
            buf = ctypes.create_string_buffer(512)
            lib.tss_solver_last_error(solver, buf, 512)
            msg = buf.value.decode(errors="replace")
        raise TssError(status, msg)


def fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) if a is not None else None


def iptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)) if a is not None else None


def u8ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)) if a is not None else None
