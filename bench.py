"""Benchmark: particle-steps/s of the two-scale WCSPH step on the 1M-particle dam break.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A "step" is one WCSPHSolver::AdvanceTS-equivalent step of the whole scene (grids,
relaxation, densities, forces, splits, integration).  The default workload,
dam_break_1m_developed, is the 1M dam break (707 x 1414 low-res particles, region
of interest [0.4,0.9]x[0,0.5], high-res pool 4M) from a developed state: the
library runs it from the initial lattice until its high-res list holds 1M
particles (~32,000 steps, untimed; make_workload), so that the timed steps carry
both scales at scale -- ~1M low-res and ~1M high-res particles, the front still
splitting.  --scene dam_break_1m times the initial lattice instead.

W warm-up steps run first, then the gathers' launch-shape autotuner (its trial
steps are warm-up too; the shape changes no result); the scene is then reset to
its start state and exactly K steps (default 500, the 1M dam break's step count)
are timed, each bracketed by CUDA events on the launching stream with L2 flushed (a
512 MiB write) between steps.  value = sum over the timed steps of the particles
processed (n_low + n_high at each step) / device time, in the exact arithmetic
(the reference's bits).  The same K steps are then timed in the tolerance
arithmetic (TSS_ARITH_FAST) and reported under "fast_arith".  e2e repeats each
timed run through the C ABI with host buffers: the start state is uploaded from
pinned memory and every step's particle positions are read back to pinned memory
(an overlapped read-back per step, double-buffered: staged on the device, then
copied to host memory while the next step runs).

With N > 1 (torchrun) every rank runs an independent replica of the scene
(replicas only: one scene does not shard); value sums the ranks' particle-steps
over the slowest rank's time.

--impl reference times the CPU restatement of the reference step (the oracle,
FP32, OpenMP over all host threads) from the same start state; the reference
itself is CUDA code with an OpenGL front end and has no CPU implementation of its
own.  Its line also carries "rebuilt_cuda": the reference's own kernels rebuilt
for sm_103a and run from the same start state by a headless restatement of
AdvanceTS.  The developed start state is made on the GPU by this library in both
arms (untimed setup).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s"
GATHER_STAGES = ("density_high", "density_low", "force_low", "force_high")
NBR_BYTES = 25
UNIT = "particle-steps/s"
MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


# ---------------------------------------------------------------------------
# algorithmic bytes (compulsory own-state traffic per particle; neighbour gathers
# are served on chip).  Per-particle and per-cell figures per stage.
# ---------------------------------------------------------------------------
def stage_bytes(stage, n_low, n_high, c_low, c_high, carry, n_fresh_children, relax_iters=0):
    cg = 16 if carry else 0
    grid = lambda n, c: n * (16 + 24 + 45 + cg) + 12 * c  # keys, scatter, reorder; scan 12 B/cell
    if stage == "grid_high":
        return grid(n_high, c_high)
    if stage == "grid_low":
        return grid(n_low, c_low)
    if stage == "relax":  # per sub-step, per child: R pos, vel (16); W dens, pres (8); W pos, vel twice (32)
        return n_fresh_children * relax_iters * 56
    # the density passes also write each particle's neighbour list (~12 16-bit
    # offsets and a count: 25 B), which the force passes read back
    if stage == "density_high":
        return n_high * (21 + NBR_BYTES) + 4 * c_high
    if stage == "density_low":
        return n_low * (21 + NBR_BYTES) + 4 * c_low
    if stage == "force_low":
        return n_low * (59 + NBR_BYTES + (12 if carry else 0)) + 4 * c_low
    if stage == "split":
        return n_low * 1
    if stage == "force_high":
        return n_high * (78 + NBR_BYTES + (12 if carry else 0)) + 4 * c_low
    return 0


def _profile_value(fname, workload, arith, stage):
    """A per-launch figure of a stage's kernel from a committed ncu summary table
    (lines: workload arith stage value), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", fname)) as f:
            for line in f:
                parts = line.split()
                if len(parts) == 4 and not line.startswith("#") and parts[:3] == [workload, arith, stage]:
                    return float(parts[3])
    except OSError:
        pass
    return None


def measured_traffic(workload, arith, stage):
    """DRAM bytes per launch of a stage's kernel (profiles/dram_traffic.txt)."""
    return _profile_value("dram_traffic.txt", workload, arith, stage)


def issue_roofline(workload, arith, stage, launch_ms, sm_mhz):
    """Instruction-issue roofline of a kernel: warp instructions per launch (ncu,
    profiles/warp_instructions.txt) over its live launch time, against 4 warp
    instructions per SM per cycle."""
    inst = _profile_value("warp_instructions.txt", workload, arith, stage)
    if inst is None or not launch_ms or not sm_mhz:
        return None
    sms = 152
    try:
        import torch
        sms = torch.cuda.get_device_properties(0).multi_processor_count
    except Exception:
        pass
    achieved = inst / (launch_ms * 1e-3)
    peak = 4.0 * sms * sm_mhz * 1e6
    return {"bound": "issue", "kernel": stage, "achieved": achieved, "peak": peak, "unit": "warp inst/s",
            "frac": achieved / peak, "warp_inst_per_launch": inst,
            "source": "profiles/warp_instructions.txt (ncu, one launch); peak = 4 per SM per cycle at the "
                      "median SM clock of the timed region"}


def hbm_peak():
    try:
        with open(MEASURED_PEAKS) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            sel = [f"--id={self.gpu}"] if self.gpu not in (None, "") else []
            self.proc = subprocess.Popen(["nvidia-smi", *sel, f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ---------------------------------------------------------------------------
def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# ---------------------------------------------------------------------------
# plain workloads: a scene and the state its timed steps start from
# ---------------------------------------------------------------------------
# name -> (scene generator, high-res particles the start state must hold)
DEVELOPED = {"dam_break_1m_developed": ("dam_break_1m", 1_000_000)}
DEVELOP_CHUNK = 1000
DEVELOP_MAX_STEPS = 80_000


def make_workload(name, seed, cache=None):
    """The scene of a plain workload and, for a developed one, the state its timed
    steps start from: the scene run from its initial state by this library (exact
    arithmetic, the tether guard on) until its high-res list holds the target count,
    checked every DEVELOP_CHUNK steps.  The 1M dam break's block fills [0,0.4]x
    [0,0.8] and its region of interest is [0.4,0.9]x[0,0.5], so from the initial
    lattice nothing splits for thousands of steps; after ~32,000 steps (0.23 s of
    flow at dt = 7.07e-6) the front has carried 250,000 parents through the region
    and the pool holds 1M children.  Returns (scene, start) with start None for
    the initial state.  `cache`: an .npz file the start state is read from when it
    exists and written to otherwise (so that a profiler run can skip the
    development)."""
    from twoscalesplit_gb300 import _abi, scenes
    if name not in DEVELOPED:
        return scenes.make_scene(name, seed=seed), None
    from twoscalesplit_gb300.solver import Solver
    base, target = DEVELOPED[name]
    sc = scenes.make_scene(base, seed=seed)
    sc.config.flags |= _abi.TSS_FLAG_TETHER_GUARD
    sc.name = name
    keys = ("id", "pos", "vel", "state", "dens", "pres")
    if cache and os.path.exists(cache):
        z = np.load(cache)
        start = {"low": {k: z["low_" + k] for k in keys}, "high": {k: z["high_" + k] for k in keys},
                 "fresh": z["fresh"], "develop_steps": int(z["develop_steps"]), "develop_s": 0.0}
        return sc, start
    sol = Solver.from_scene(sc)
    t0 = time.perf_counter()
    steps = 0
    while steps < DEVELOP_MAX_STEPS:
        sol.step(DEVELOP_CHUNK)
        steps += DEVELOP_CHUNK
        if sol.counts()["n_high"] >= target:
            break
    sol.sync()  # raises on a device error
    c = sol.counts()
    if c["n_high"] < target:
        raise RuntimeError(f"{name}: {c['n_high']} high-res particles after {steps} steps")
    start = {"low": sol.download(0), "high": sol.download(1), "fresh": sol.get_fresh(), "develop_steps": steps,
             "develop_s": time.perf_counter() - t0}
    sol.close()
    if cache:
        np.savez(cache, fresh=start["fresh"], develop_steps=steps,
                 **{f"{s}_{k}": start[s][k] for s in ("low", "high") for k in keys})
    return sc, start


def load_start(obj, sc, start):
    """Put a solver or oracle in the workload's start state."""
    from twoscalesplit_gb300.solver import Solver
    if start is None:
        low = {"id": np.arange(sc.n_low, dtype=np.int32), "pos": sc.low_pos, "vel": sc.low_vel,
               "state": np.zeros(sc.n_low, np.uint8)}
        high = {"id": np.zeros(0, np.int32), "pos": np.zeros((0, 2), np.float32),
                "vel": np.zeros((0, 2), np.float32), "state": np.zeros(0, np.uint8)}
        fresh = np.zeros(0, np.int32)
    else:
        low, high, fresh = start["low"], start["high"], start["fresh"]
    if isinstance(obj, Solver):
        obj.upload(0, low)
        obj.upload(1, high)
        obj.set_fresh(fresh)
    else:
        for s, d in ((0, low), (1, high)):
            obj.set_scale(s, d["id"], d["pos"], d["vel"], d["state"], d.get("dens"), d.get("pres"))
        obj.set_fresh(fresh)


def cpu_baseline(sc, start, budget_s, threads=None):
    """The oracle (FP32, the reference's arithmetic) timed on the host cores, from
    the workload's start state."""
    import oracle as O
    if threads:
        O.set_threads(threads)
    orc = O.Oracle(sc, 32)
    load_start(orc, sc, start)
    done, parts, t0 = 0, 0, time.perf_counter()
    while True:
        n = orc.get(0, "id").shape[0] + orc.get(1, "id").shape[0]
        orc.step()
        done += 1
        parts += n
        if time.perf_counter() - t0 >= budget_s or done >= sc.steps:
            break
    dt = time.perf_counter() - t0
    where = "the initial state" if start is None else f"the developed state ({start['develop_steps']} steps)"
    return {"value": parts / dt, "unit": UNIT, "cores": O.max_threads(), "kind": "port",
            "sample": f"{sc.name}: {done} steps from {where} ({parts} particle-steps, {dt:.1f} s), FP32 CPU "
                      f"restatement of the reference step, OpenMP"}


def survey_step_bytes(n_low, n_high, c_low, c_high, splits):
    """Algorithmic bytes of one step in the radix-sort model of the hot-path survey:
    per scale N (120 + 16 k) + 8 C with k = ceil(ceil(log2 C) / 8) digit passes,
    plus 72 per split (the config-1 figure of 0.87 GB/step assumes a full 4M pool)."""
    def k(c):
        return math.ceil(math.ceil(math.log2(max(c, 2))) / 8)
    return (n_low * (120 + 16 * k(c_low)) + 8 * c_low + n_high * (120 + 16 * k(c_high)) + 8 * c_high
            + 72 * splits)


def tuned_shape(sol, kind, n_low, args):
    """The gathers' launch shape for this GPU and workload class: from the launch
    cache, else tuned on `sol` (its trial steps advance its state: call during
    warm-up).  --no-autotune keeps the default shape."""
    if args.no_autotune:
        return sol.launch, 0
    from twoscalesplit_gb300 import tuning
    return tuning.tuned_launch(sol, kind, n_low, path=args.launch_cache)


def compact_shape(shape):
    """threads per block, 'p' for a persistent grid, 'w' for one particle per warp"""
    return {g: f"{v['threads']}{'p' if v['persistent'] else ''}{'w' if v.get('per_warp') else ''}"
            for g, v in shape.items()}


def workload_config(sc, start, args):
    """The config keys both arms report for a plain workload."""
    cfg = sc.config
    c = {"workload": sc.name, "n_low": sc.n_low, "cap_high": sc.cap_high, "dt": cfg.dt,
         "relax_iters": cfg.relax_iters, "q1_compat": bool(cfg.flags & 1),
         "tether_guard": bool(cfg.flags & 4), "seed": 0,
         "start": "initial lattice" if start is None else
                  f"developed: {start['develop_steps']} steps of the library from the initial lattice"}
    if start is not None:
        c["n_high_start"] = int(start["high"]["id"].shape[0])
    return c


def run_reference(args):
    world, rank, _ = _dist()
    if rank != 0:
        return
    budget = float(os.environ.get("TSS_REF_BUDGET_S", "150"))
    import oracle as O
    sc, start = make_workload(args.scene, 0, args.start_cache)
    orc = O.Oracle(sc, 32)
    load_start(orc, sc, start)
    for _ in range(min(args.warmup, 1)):
        orc.step()
    orc = O.Oracle(sc, 32)
    load_start(orc, sc, start)
    t0 = time.perf_counter()
    parts = 0
    steps = 0
    for _ in range(args.steps):
        parts += orc.get(0, "id").shape[0] + orc.get(1, "id").shape[0]
        orc.step()
        steps += 1
        if time.perf_counter() - t0 > budget:
            break
    dt = time.perf_counter() - t0
    v = parts / dt
    where = "the initial state" if start is None else \
        f"the developed state (made on the GPU by this library, untimed: {start['develop_steps']} steps)"
    conf = workload_config(sc, start, args)
    conf.update({"l2": "n/a (CPU)", "launch": "n/a (CPU)", "autotune_steps": 0, "parallelism": "replicas1",
                 "arith": "exact (FP32, the reference's arithmetic)"})
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": world, "steps": steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": conf,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": O.max_threads(), "kind": "port",
                             "sample": f"{sc.name}: first {steps} of the {args.steps} requested steps from {where}, "
                                       f"bounded to {budget:.0f} s"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    line["rebuilt_cuda"] = rebuilt_reference_gpu(sc, start, args)
    print(json.dumps(line), flush=True)


def rebuilt_reference_gpu(sc, start, args, budget_s=30.0):
    """The reference's own CUDA kernels rebuilt for sm_103a (oracle RefGPU: its
    kernel source as a cubin, driven by a headless restatement of AdvanceTS) timed
    on this GPU from the same start state, or why not.  Each reference step ends in
    its three synchronous count read-backs, so the wall clock per step is its step
    time; the run is bounded to `budget_s`."""
    try:
        import oracle as O
        if not O.refgpu_available():
            return {"unavailable": "the reference's kernels for sm_103a are not built here (no cubin or no driver)"}

        def fresh_ref():
            r = O.RefGPU(sc)
            if start is not None:
                r.set_state(start["low"], start["high"])
            return r

        ref = fresh_ref()
        ref.step(max(args.warmup, 1))
        del ref
        ref = fresh_ref()  # timed from the start state, like the other arms
        c0 = ref.counts()
        parts, steps = 0, 0
        t0 = time.perf_counter()
        while steps < args.steps:
            c = ref.counts()
            parts += c["n_low"] + c["n_high"]
            ref.step(1)
            steps += 1
            if time.perf_counter() - t0 > budget_s:
                break
        dt = time.perf_counter() - t0
        c = ref.counts()
        return {"value": parts / dt, "unit": UNIT, "ms_per_step": 1e3 * dt / steps, "steps": steps,
                "n_high_start": c0["n_high"], "n_high_end": c["n_high"],
                "build": "TwoScale2D/WCSPHSolver.cu kernels (lines 14-2283) for sm_103a, nvcc -O3 with the "
                         "reference's defaults (contraction on); texture fetches as bounded loads",
                "split_region": "x > 0.5, hard-coded in the reference's kernels (WCSPHSolver.cu:1835), not the "
                                "scene's region of interest",
                "timing": "wall clock per step from the workload's start state, including the reference's three "
                          "synchronous count read-backs and its thrust sorts (no rendering)"}
    except Exception as e:  # the arm's CPU line stands without it
        return {"unavailable": f"{type(e).__name__}: {e}"}


def timed_steps(sol, K, reset, flush, stream, sh, world):
    """K steps, each between CUDA events on the launching stream, L2 flushed before
    each; returns (device ms, wall s, clocks sampled meanwhile)."""
    import torch
    reset()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    _, _, local = _dist()
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")
    clocks = ClockSampler(vis[local].strip() if local < len(vis) and vis[local].strip()
                          else (str(local) if world > 1 else None))
    clocks.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    for k in range(K):
        flush.zero_()
        evs[k][0].record(stream)
        sol.step(1, stream=sh)
        evs[k][1].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - w0
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    sol.sync()  # raises on a device error (capacity, NaN, grid index)
    return sum(a.elapsed_time(b) for a, b in evs), wall, clk


def stage_average(sol, reset, flush, sh, n):
    """Stage times of the profiling graph averaged over the first n steps from the
    start state (L2 flushed before each)."""
    from twoscalesplit_gb300 import _abi
    sol.profile(True)
    reset()
    acc = {k: 0.0 for k in _abi.STAGE_NAMES}
    for _ in range(n):
        flush.zero_()
        sol.step(1, stream=sh)
        for name, v in sol.stage_times().items():
            acc[name] += v
    sol.profile(False)
    return {k: v / n for k, v in acc.items()}


def e2e_run(sol, sc, start, K, sh, world):
    """The timed steps end to end through the C ABI with host buffers: the start
    state (both lists) is uploaded from page-locked memory, and every step's
    positions (both lists) are read back into page-locked memory by
    tss_solver_read_positions_async (staged on the device on the step's stream,
    then copied to host memory on the solver's own stream while the next step
    runs), double-buffered: the host waits for step k's read-back (its ticket)
    before it reuses that buffer at step k + 2, and counts the bytes it received.
    Returns (seconds, h2d bytes, d2h bytes)."""
    import ctypes

    import torch
    from twoscalesplit_gb300 import _abi
    from twoscalesplit_gb300._abi import TssScaleState, fptr
    load_start(sol, sc, start)
    cap_h = max(sc.cap_high, 1)
    outs = [(torch.empty((sc.n_low, 2), dtype=torch.float32).pin_memory(),
             torch.empty((cap_h, 2), dtype=torch.float32).pin_memory(),
             torch.zeros(2, dtype=torch.int32).pin_memory()) for _ in range(2)]
    sol.step(1, stream=sh)  # keep the graph captured and the staging buffers allocated outside the timed region
    sol.read_wait(sol.read_positions_async(outs[0][0], outs[0][1], outs[0][2], stream=sh))
    torch.cuda.synchronize()
    if start is None:
        lists = [{"id": np.arange(sc.n_low, dtype=np.int32), "pos": sc.low_pos, "vel": sc.low_vel,
                  "state": np.zeros(sc.n_low, np.uint8)},
                 {"id": np.zeros(0, np.int32), "pos": np.zeros((0, 2), np.float32),
                  "vel": np.zeros((0, 2), np.float32), "state": np.zeros(0, np.uint8)}]
        fresh = np.zeros(0, np.int32)
    else:
        lists = [start["low"], start["high"]]
        fresh = start["fresh"]
    pinned = [{k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for k, v in d.items()
               if k in ("id", "pos", "vel", "state")} for d in lists]
    states = [TssScaleState(int(d["id"].shape[0]), _abi.iptr(d["id"].numpy()), fptr(d["pos"].numpy()),
                            fptr(d["vel"].numpy()), _abi.u8ptr(d["state"].numpy()), None, None) for d in pinned]
    lib = sol.lib
    h2d = sum(int(d["id"].shape[0]) * (4 + 8 + 8 + 1) for d in lists) + 4 * fresh.shape[0]
    d2h = 0
    tickets = [None, None]

    def received(b):
        sol.read_wait(tickets[b])
        c = outs[b][2].tolist()
        tickets[b] = None
        return 8 * (min(c[0], sc.n_low) + min(c[1], cap_h)) + 8

    if world > 1:
        torch.distributed.barrier()
    e0 = time.perf_counter()
    for s in (0, 1):
        _abi.check(lib.tss_solver_upload(sol.h, s, ctypes.byref(states[s])))
    sol.set_fresh(fresh)
    for k in range(K):
        b = k % 2
        if tickets[b] is not None:
            d2h += received(b)
        sol.step(1, stream=sh)
        tickets[b] = sol.read_positions_async(outs[b][0], outs[b][1], outs[b][2], stream=sh)
    for b in (K % 2, (K + 1) % 2):  # the older read-back first
        if tickets[b] is not None:
            d2h += received(b)
    return time.perf_counter() - e0, h2d, d2h


def run_ours(args):
    import torch
    world, rank, local = _dist()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)
    from twoscalesplit_gb300 import _abi, build
    from twoscalesplit_gb300.solver import Solver
    build.build()
    sc, start = make_workload(args.scene, rank, args.start_cache if rank == 0 else None)
    sol = Solver.from_scene(sc)
    # a dedicated stream: the graph replays, the L2 flush and the timing events all
    # go to it, so the events bracket exactly the step
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream

    def reset():
        load_start(sol, sc, start)

    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=dev)
    kind = "single" if start is None else "single_developed"
    K = args.steps
    legs = {}
    for mode in (("exact", "fast") if args.arith == "both" else (args.arith,)):
        sol.set_arith(mode)
        # warm-up (graph capture happens here), then the launch-shape autotuner on the
        # same state (its trial steps are warm-up too: the state is reset after them)
        reset()
        sol.step(max(args.warmup, 1), stream=sh)
        torch.cuda.synchronize(dev)
        reset()
        shape, tune_steps = tuned_shape(sol, kind if mode == "exact" else kind + "_fast", sc.n_low, args)
        dev_ms, wall, clk = timed_steps(sol, K, reset, flush, stream, sh, world)
        st_avg = stage_average(sol, reset, flush, sh, min(K, 50))
        e2e_s, h2d, d2h = e2e_run(sol, sc, start, K, sh, world)
        legs[mode] = {"dev_ms": dev_ms, "wall": wall, "clk": clk, "stage": st_avg, "e2e_s": e2e_s, "h2d": h2d,
                      "d2h": d2h, "shape": shape, "tune_steps": tune_steps}
    head = "exact" if "exact" in legs else "fast"
    sol.set_arith(head)
    # particles processed per step (deterministic replay of the exact steps, untimed)
    reset()
    counts = []
    c0 = sol.counts()
    for k in range(K):
        c = sol.counts()
        counts.append(c["n_low"] + c["n_high"])
        sol.step(1, stream=sh)
    c_end = sol.counts()
    parts = float(sum(counts))
    splits_per_step = (c_end["total_split"] - c0["total_split"]) / K
    times = torch.tensor([legs[head]["dev_ms"], legs[head]["e2e_s"], parts], dtype=torch.float64, device=dev)
    if world > 1:
        t_max = times.clone()
        torch.distributed.all_reduce(t_max[:2], op=torch.distributed.ReduceOp.MAX)
        tot = times.clone()
        torch.distributed.all_reduce(tot[2:], op=torch.distributed.ReduceOp.SUM)
        parts_all = float(tot[2])
        for leg in legs.values():  # the slowest rank's times (replicas of the same work)
            tl = torch.tensor([leg["dev_ms"], leg["e2e_s"]], dtype=torch.float64, device=dev)
            torch.distributed.all_reduce(tl, op=torch.distributed.ReduceOp.MAX)
            leg["dev_ms"], leg["e2e_s"] = float(tl[0]), float(tl[1])
    else:
        parts_all = parts
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    peak, peak_kind = hbm_peak()
    cfg = sc.config
    c_low, c_high = cfg.dims_low[0] * cfg.dims_low[1], cfg.dims_high[0] * cfg.dims_high[1]
    n_high_avg = float(np.mean(counts)) - sc.n_low
    carry = cfg.relax_iters > 0

    n_fresh = 4.0 * splits_per_step  # children relaxed per step

    def roofline(leg, arith):
        st_avg = leg["stage"]
        # the dominant single kernel: the gathers (a grid build or a relaxation
        # sub-step is several launches)
        top = max(GATHER_STAGES, key=lambda k: st_avg[k])
        top_bytes = stage_bytes(top, sc.n_low, n_high_avg, c_low, c_high, carry, n_fresh, cfg.relax_iters)
        top_gbs = top_bytes / (st_avg[top] * 1e-3) / 1e9 if st_avg[top] > 0 else 0.0
        step_ms = leg["dev_ms"] / K
        step_bytes = sum(stage_bytes(s, sc.n_low, n_high_avg, c_low, c_high, carry, n_fresh, cfg.relax_iters)
                         for s in _abi.STAGE_NAMES)
        sv = survey_step_bytes(sc.n_low, n_high_avg, c_low, c_high, splits_per_step)
        return top, {"bound": "hbm", "kernel": top, "achieved": top_gbs, "peak": peak, "unit": "GB/s",
                     "frac": top_gbs / peak, "peak_source": peak_kind, "traffic": measured_traffic(sc.name, arith, top),
                     "traffic_source": "profiles/dram_traffic.txt (ncu, one launch)",
                     "algorithmic_bytes_per_launch": top_bytes, "launch_ms": st_avg[top],
                     "step": {"algorithmic_bytes": step_bytes,
                              "achieved_gbs": step_bytes / (step_ms * 1e-3) / 1e9,
                              "frac": step_bytes / (step_ms * 1e-3) / 1e9 / peak,
                              "survey_model_bytes": sv,
                              "survey_model_frac": sv / (step_ms * 1e-3) / 1e9 / peak}}

    ex = legs[head]
    top, roof = roofline(ex, head)
    conf = workload_config(sc, start, args)
    conf.update({"n_high_end": c_end["n_high"], "splits_per_step": splits_per_step,
                 "l2": "flushed between timed steps (512 MiB write)", "parallelism": f"replicas{world}",
                 "launch": compact_shape(ex["shape"]), "autotune_steps": ex["tune_steps"],
                 "arith": "exact (FP32, the reference's arithmetic; bit-identical to it)" if head == "exact" else
                          "fast (TSS_ARITH_FAST, within 1e-5 of the reference per step)"})
    if start is not None:
        conf["develop_s"] = round(start["develop_s"], 2)
    line = {
        "metric": METRIC, "value": parts_all / (ex["dev_ms"] / 1e3), "unit": UNIT, "n_gpus": world, "steps": K,
        "warmup": args.warmup, "ms_per_step": ex["dev_ms"] / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": conf,
        "roofline": roof,
        "issue_roofline": issue_roofline(sc.name, head, top, ex["stage"][top], (ex["clk"] or {}).get("sm_mhz")),
        "stage_ms": {k: round(v, 5) for k, v in ex["stage"].items()},
        "e2e": {"value": parts_all / ex["e2e_s"], "unit": UNIT, "h2d_bytes_per_step": ex["h2d"] / K,
                "d2h_bytes_per_step": ex["d2h"] / K},
        # kernels per step: 2 grid sorts x 3 (scan, scatter, reorder), 4 gathers, split
        # compaction, finish (+ 3 per relaxation sub-step); the 3 memset nodes are not counted
        "gpu_launches": K * (12 + 3 * cfg.relax_iters),
        "clocks": ex["clk"],
        "wall_s_timed": ex["wall"],
    }
    if head == "exact" and "fast" in legs:
        fa = legs["fast"]
        ftop, froof = roofline(fa, "fast")
        line["fast_arith"] = {
            "what": "TSS_ARITH_FAST: per pair an approximate rsqrt and reciprocal and FMAs; densities, forces and "
                    "positions within 1e-5 of the FP32 oracle per step (tests/test_gpu_fast_arith.py)",
            "value": parts_all / (fa["dev_ms"] / 1e3), "unit": UNIT, "ms_per_step": fa["dev_ms"] / K,
            "speedup_vs_exact": ex["dev_ms"] / fa["dev_ms"],
            "e2e": {"value": parts_all / fa["e2e_s"], "unit": UNIT, "h2d_bytes_per_step": fa["h2d"] / K,
                    "d2h_bytes_per_step": fa["d2h"] / K},
            "roofline": froof,
            "issue_roofline": issue_roofline(sc.name, "fast", ftop, fa["stage"][ftop], (fa["clk"] or {}).get("sm_mhz")),
            "stage_ms": {k: round(v, 5) for k, v in fa["stage"].items()},
            "launch": compact_shape(fa["shape"]), "clocks": fa["clk"]}
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(sc, start, args.cpu_budget_s)
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_batch(args):
    """The mixed-size batch workload: `--scenes` independent scenes advanced in
    lockstep by one batch (one grid build and one launch of each kernel per step),
    against the same scenes advanced one at a time by the plain solver, in each
    arithmetic of --arith (the plain solver in the same arithmetic as the batch:
    the comparison is at the same tolerance)."""
    import torch
    from twoscalesplit_gb300 import _abi, build, scenes
    from twoscalesplit_gb300.solver import Batch, Solver
    build.build()
    dev = torch.device("cuda", 0)
    scs = scenes.mixed_batch(args.scenes, seed=0)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=dev)
    empty = {"id": np.zeros(0, np.int32), "pos": np.zeros((0, 2), np.float32), "vel": np.zeros((0, 2), np.float32),
             "state": np.zeros(0, np.uint8)}
    K = args.steps
    n_low = sum(sc.n_low for sc in scs)
    n_plain = min(len(scs), args.plain_sample)
    legs = {}
    for mode in (("exact", "fast") if args.arith == "both" else (args.arith,)):
        suffix = "" if mode == "exact" else "_fast"
        b = Batch(scs)
        b.set_arith(mode)
        init = b.download(0)
        b.step(max(args.warmup, 1), stream=sh)
        torch.cuda.synchronize(dev)
        shape, tune_steps = tuned_shape(b, "batch" + suffix, n_low, args)
        b.upload(0, init)
        b.upload(1, empty)
        b.set_fresh(np.zeros(0, np.int32))
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
        clocks = ClockSampler(None)
        clocks.start()
        for k in range(K):
            flush.zero_()
            evs[k][0].record(stream)
            b.step(1, stream=sh)
            evs[k][1].record(stream)
        torch.cuda.synchronize(dev)
        clk = clocks.stop()
        b.sync()
        batch_ms = sum(x.elapsed_time(y) for x, y in evs)
        c = b.counts()
        # where a step's time goes once the high-res lists have filled: stage times
        # (profiling graph) of 10 more steps from the final state, untimed above
        b.profile(True)
        st_sum = {k: 0.0 for k in _abi.STAGE_NAMES}
        for _ in range(10):
            flush.zero_()
            b.step(1, stream=sh)
            for name, v in b.stage_times().items():
                st_sum[name] += v
        b.profile(False)
        del b
        # the plain solver, one scene at a time, same steps, same arithmetic
        plain_ms = 0.0
        for sc in scs[:n_plain]:
            sol = Solver.from_scene(sc)
            sol.set_arith(mode)
            sol.step(max(args.warmup, 1), stream=sh)
            tuned_shape(sol, "single" + suffix, sc.n_low, args)
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sol.step(K, stream=sh)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            plain_ms += e0.elapsed_time(e1)
            del sol
        plain_ms *= len(scs) / n_plain
        legs[mode] = {"value": len(scs) * K / (batch_ms / 1e3), "ms_per_step": batch_ms / K,
                      "particle_steps_per_s": n_low * K / (batch_ms / 1e3),
                      "plain_one_at_a_time": {"scene_steps_per_s": len(scs) * K / (plain_ms / 1e3),
                                              "sampled_scenes": n_plain, "ms_per_lockstep": plain_ms / K},
                      "speedup_vs_plain": plain_ms / batch_ms, "clocks": clk,
                      "n_high_end": c["n_high"], "n_particles_end": c["n_low"] + c["n_high"],
                      "launch": compact_shape(shape), "autotune_steps": tune_steps,
                      "stage_ms_end": {k: round(v / 10, 4) for k, v in st_sum.items()}}
    head = legs["exact"] if "exact" in legs else legs["fast"]
    line = {"metric": "scene-steps/s", "value": head["value"], "unit": "scene-steps/s",
            "n_gpus": 1, "steps": K, "warmup": args.warmup, "ms_per_step": head["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"mixed_batch_{len(scs)}", "scenes": len(scs), "n_low_total": n_low,
                       "arith": "exact" if "exact" in legs else "fast",
                       "l2": "flushed between timed steps (512 MiB write)"},
            **{k: v for k, v in head.items() if k not in ("value", "ms_per_step")}}
    if "exact" in legs and "fast" in legs:
        line["fast_arith"] = legs["fast"]
    print(json.dumps(line), flush=True)


def run_serve(args):
    """The serving workload: a stream of scene requests (counts log-uniform 1k-500k,
    horizons 200-5000 steps) with Poisson arrivals at `--load` x the measured
    capacity of the 512-scene batch (low-res particle-steps/s), served by the
    library's serving loop over a pool sized from an HBM budget.  The same requests
    are also run one at a time through the plain solver (create, horizon steps,
    download of the final state), each timed; first-come-first-served completion
    times of that single server follow from those service times and the same
    arrivals.  A second, saturated run submits the first `--burst` requests at once
    and compares its makespan with the plain solver's summed service times."""
    import torch
    from twoscalesplit_gb300 import _abi, build, scenes
    from twoscalesplit_gb300.serving import (Request, Server, fifo_schedule, latency_summary, pool_bytes,
                                             pool_config_for_budget)
    from twoscalesplit_gb300.solver import Batch, Solver
    build.build()
    world, rank, local = _dist()
    if world > 1:
        return run_serve_replicas(args, world, rank, local)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    # 1. capacity of the batched step on the 512-scene mixed batch
    if args.capacity_lps:
        cap_lps, cap_src = args.capacity_lps, "given on the command line"
    else:
        cap_lps = measure_batch_capacity(dev, arith=args.arith)
        cap_src = f"mixed_batch_512, 10 steps after 3 warm-up steps, {args.arith} arithmetic"
    # 2. the request stream
    rate = args.load * cap_lps / scenes.mean_work()
    trace = scenes.serving_trace(args.requests, rate, seed=args.seed)
    n_low = np.array([sc.n_low for sc, _, _ in trace], dtype=np.float64)
    cells = np.array([sc.config.dims_low[0] * sc.config.dims_low[1] for sc, _, _ in trace], dtype=np.float64)
    walls = np.array([sc.n_wall for sc, _, _ in trace], dtype=np.float64)
    cfg = pool_config_for_budget(int(args.budget_gb * (1 << 30)), 1.25 * cells.sum() / n_low.sum() + 0.05,
                                 1.25 * walls.sum() / n_low.sum() + 0.05, max_scenes=8192)
    sv = Server(cfg, max_steps_per_launch=args.chunk, max_in_flight=2, staging_bytes=2 << 30, arith=args.arith)
    # warm-up: graph capture, first-touch of the staging rings
    warm = scenes.serving_trace(4, 1e3, seed=args.seed + 1, n_min=2000, n_max=20000, h_min=10, h_max=20)
    sv.run([Request(sc, h, t) for sc, h, t in warm])
    verify = sorted(range(len(trace)), key=lambda k: trace[k][0].n_low * trace[k][1])[:3]
    reqs = [Request(sc, h, t, want_result=(k in verify)) for k, (sc, h, t) in enumerate(trace)]
    clocks = ClockSampler(None)
    clocks.start()
    stats, summ, res = sv.run(reqs)
    clk = clocks.stop()
    lat = latency_summary(stats)
    served = [k for k, st in enumerate(stats) if st["status"] in (_abi.TSS_OK, _abi.TSS_NUMERIC)]
    numeric_served = sorted(k for k, st in enumerate(stats) if st["status"] == _abi.TSS_NUMERIC)
    numeric_plain = []
    # 3. the plain solver, one request at a time, each timed (create + steps + download)
    #    with the launch shape tuned for its size class; the classes are tuned first,
    #    on scratch solvers, so that no request takes trial steps
    suffix = "" if args.arith == "exact" else "_fast"
    if not args.no_plain and not args.no_autotune:
        from twoscalesplit_gb300 import tuning
        seen = set()
        for sc, _, _ in trace:
            cls = tuning.workload_class("single", sc.n_low)
            if cls not in seen:
                seen.add(cls)
                scratch = Solver.from_scene(sc)
                scratch.set_arith(args.arith)
                tuned_shape(scratch, "single" + suffix, sc.n_low, args)
    service = np.zeros(len(trace))
    exact = 0
    plain_steps_ms = 0.0
    # the requests the plain solver is timed on: all, or a seeded uniform sample of
    # --plain-requests (a long stream's remaining service times are then estimated
    # from the sample: service = a + b * n_low * horizon, least squares)
    timed = list(range(len(trace)))
    if args.plain_requests and args.plain_requests < len(trace):
        timed = sorted(np.random.default_rng(args.seed + 7).choice(len(trace), args.plain_requests,
                                                                   replace=False).tolist())
        timed = sorted(set(timed) | set(verify))
    for k in (timed if not args.no_plain else []):
        sc, h, _ = trace[k]
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        sol = Solver.from_scene(sc)
        sol.set_arith(args.arith)
        if not args.no_autotune:
            tuned_shape(sol, "single" + suffix, sc.n_low, args)  # from the cache: no steps
        sol.step(h)
        lo, hi = sol.download(0), sol.download(1)
        service[k] = time.perf_counter() - t0
        if sol.counts()["error_bits"] & _abi.TSS_ERR_NUMERIC:
            numeric_plain.append(k)
        if k in verify and res[k] is not None:
            same = True
            for mine, theirs in ((lo, res[k][0]), (hi, res[k][1])):
                a, b2 = np.argsort(mine["id"], kind="stable"), np.argsort(theirs["id"], kind="stable")
                same &= all(np.array_equal(mine[f][a], theirs[f][b2]) for f in ("id", "pos", "vel", "state",
                                                                               "dens", "pres"))
            exact += int(same)
        del sol
    arrivals = np.array([t for _, _, t in trace])
    horizons = np.array([h for _, h, _ in trace], dtype=np.float64)
    sampled = len(timed) < len(trace)
    if sampled and not args.no_plain:
        work = n_low * horizons
        A = np.stack([np.ones(len(timed)), work[timed]], axis=1)
        coef, *_ = np.linalg.lstsq(A, service[timed], rcond=None)
        est = coef[0] + coef[1] * work
        rest = np.setdiff1d(np.arange(len(trace)), timed)
        service[rest] = est[rest]
    scene_steps = float(horizons[served].sum())
    makespan = summ["makespan_s"] - float(arrivals.min())
    plain_part, saturated = None, None
    if not args.no_plain:
        plain_done = fifo_schedule(arrivals, service)
        plain_lat = plain_done - arrivals
        plain_makespan = float(plain_done.max() - arrivals.min())
        plain_part = {
            "scene_steps_per_s": float(horizons.sum()) / plain_makespan,
            "latency_s": {"p50_s": float(np.percentile(plain_lat, 50)), "p99_s": float(np.percentile(plain_lat, 99)),
                          "mean_s": float(plain_lat.mean())},
            "service_s_total": float(service.sum()),
            "how": "computed, not replayed: each request timed alone through the plain solver (create, horizon "
                   "steps, download), then FIFO completion times computed from those service times and the same "
                   "arrivals" + (f"; {len(timed)} of the {len(trace)} requests timed (a seeded uniform sample), "
                                 f"the others' service times estimated as a + b * n_low * horizon fitted to them "
                                 f"(a = {coef[0]:.4f} s, b = {coef[1]:.3e} s)" if sampled else "")}
        # 4. saturated: the first `burst` requests at once (all timed when sampled)
        nb = min(args.burst, len(trace))
        if sampled:
            for k in range(nb):
                if k not in set(timed):
                    sc, h, _ = trace[k]
                    torch.cuda.synchronize(dev)
                    t0 = time.perf_counter()
                    sol = Solver.from_scene(sc)
                    sol.set_arith(args.arith)
                    if not args.no_autotune:
                        tuned_shape(sol, "single" + suffix, sc.n_low, args)
                    sol.step(h)
                    sol.download(0), sol.download(1)
                    service[k] = time.perf_counter() - t0
                    del sol
        st_b, summ_b, _ = sv.run([Request(sc, h, 0.0) for sc, h, _ in trace[:nb]])
        burst_ss = float(sum(h for _, h, _ in trace[:nb]))
        saturated = {"requests": nb, "scene_steps_per_s": burst_ss / summ_b["makespan_s"],
                     "plain_scene_steps_per_s": burst_ss / float(service[:nb].sum()),
                     "speedup_vs_plain": float(service[:nb].sum()) / summ_b["makespan_s"],
                     "mean_active_scenes": summ_b["mean_active"]}
    # kernels: 12 per pool step; per request about 11 at admission (keys, slot-map
    # fill, wall grid build, counters), 2 at extraction and 4 at retirement
    gpu_launches = int(summ["steps"] * 12 + len(served) * 17)
    line = {"metric": "scene-steps/s", "value": scene_steps / makespan, "unit": "scene-steps/s", "n_gpus": 1,
            "steps": int(summ["steps"]), "warmup": 1, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"serving_{len(trace)}_poisson", "requests": len(trace),
                       "arrival_rate_per_s": rate, "load": args.load,
                       "capacity_low_particle_steps_per_s": cap_lps, "capacity_source": cap_src,
                       "n_low": "log-uniform 1k-500k", "horizon": "uniform 200-5000",
                       "hbm_budget_gb": args.budget_gb, "pool_bytes": pool_bytes(cfg),
                       "pool": {"low_slots": cfg.low_slots, "high_particles": cfg.high_particles,
                                "low_cells": cfg.low_cells, "high_cells": cfg.high_cells,
                                "wall_particles": cfg.wall_particles},
                       "max_steps_per_launch": args.chunk, "arith": args.arith,
                       "l2": "inputs of the steps are the pool state (no flush; served end to end)"},
            "served": len(served), "rejected": int(sum(1 for st in stats if st["status"] == _abi.TSS_INVALID_ARG)),
            "latency_s": lat, "low_particle_steps_per_s": float(n_low[served] @ horizons[served]) / makespan,
            "mean_active_scenes": summ["mean_active"], "max_active_scenes": summ["max_active"],
            "plain_one_at_a_time": plain_part,
            "speedup_vs_plain": None if plain_part is None else (scene_steps / makespan) / plain_part["scene_steps_per_s"],
            "saturated": saturated,
            "exact_vs_alone": None if args.no_plain else f"{exact}/{len(verify)} requests bit-identical to the plain solver",
            "non_finite": {"served": numeric_served, "plain": None if args.no_plain else numeric_plain,
                           "same_requests": None if args.no_plain else
                           [k for k in numeric_served if k in set(timed)] == sorted(numeric_plain),
                           "plain_checked": len(timed) if not args.no_plain else 0},
            "e2e": {"value": scene_steps / makespan, "unit": "scene-steps/s",
                    "h2d_bytes_per_step": float(sum(16 * sc.n_low + 8 * sc.n_wall for sc, _, _ in trace)) / max(summ["steps"], 1),
                    "d2h_bytes_per_step": float(sum(29 * 5 * sc.n_low for sc, _, _ in trace)) / max(summ["steps"], 1)},
            "gpu_launches": gpu_launches, "clocks": clk}
    print(json.dumps(line), flush=True)


def measure_batch_capacity(dev, steps=10, arith="exact"):
    """Low-res particle-steps/s of the batched step on the 512-scene mixed batch."""
    import torch
    from twoscalesplit_gb300 import scenes
    from twoscalesplit_gb300.solver import Batch
    scs = scenes.mixed_batch(512, seed=0)
    b = Batch(scs)
    b.set_arith(arith)
    b.step(3)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    b.step(steps)
    e1.record()
    torch.cuda.synchronize(dev)
    b.sync()
    return sum(sc.n_low for sc in scs) * steps / (e0.elapsed_time(e1) / 1e3)


def run_serve_replicas(args, world, rank, local):
    """The serving workload on `world` GPUs: independent replicas behind a
    deterministic least-work dispatcher, no exchange in the data path (weak
    scaling: the stream has `world` times the requests and arrival rate of the
    one-GPU stream).  Per-request statistics are merged over gloo; rank 0 prints."""
    import torch
    import torch.distributed as dist
    from twoscalesplit_gb300 import _abi, dispatch, scenes
    from twoscalesplit_gb300.serving import Request, Server, latency_summary, pool_config_for_budget
    # replicas never wait on one another, so ranks beyond the visible devices share them
    local = local % torch.cuda.device_count()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist.init_process_group("gloo")
    cap = args.capacity_lps or measure_batch_capacity(dev, arith=args.arith)
    cap = dispatch.gather(cap)[0]  # every replica uses rank 0's measurement
    rate = world * args.load * cap / scenes.mean_work()
    trace = scenes.serving_trace(args.requests * world, rate, seed=args.seed)
    n_low = np.array([sc.n_low for sc, _, _ in trace], dtype=np.float64)
    cells = np.array([sc.config.dims_low[0] * sc.config.dims_low[1] for sc, _, _ in trace], dtype=np.float64)
    walls = np.array([sc.n_wall for sc, _, _ in trace], dtype=np.float64)
    cfg = pool_config_for_budget(int(args.budget_gb * (1 << 30)), 1.25 * cells.sum() / n_low.sum() + 0.05,
                                 1.25 * walls.sum() / n_low.sum() + 0.05, max_scenes=8192)
    sv = Server(cfg, max_steps_per_launch=args.chunk, max_in_flight=2, staging_bytes=2 << 30, arith=args.arith)
    warm = scenes.serving_trace(4, 1e3, seed=args.seed + 1, n_min=2000, n_max=20000, h_min=10, h_max=20)
    sv.run([Request(sc, h, t) for sc, h, t in warm])
    reqs = [Request(sc, h, t) for sc, h, t in trace]
    dist.barrier()
    clocks = ClockSampler(str(local))
    clocks.start()
    stats, summ = dispatch.serve_replicated(reqs, lambda rs: sv.run(rs)[:2], rank, world)
    clk = clocks.stop()
    if rank == 0:
        served = [k for k, st in enumerate(stats) if st["status"] in (_abi.TSS_OK, _abi.TSS_NUMERIC)]
        horizons = np.array([h for _, h, _ in trace], dtype=np.float64)
        arrivals = np.array([t for _, _, t in trace])
        makespan = summ["makespan_s"] - float(arrivals.min())
        ss = float(horizons[served].sum())
        line = {"metric": "scene-steps/s", "value": ss / makespan, "unit": "scene-steps/s", "n_gpus": world,
                "steps": int(summ["steps"]), "warmup": 1, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": f"serving_{len(trace)}_poisson", "requests": len(trace),
                           "arrival_rate_per_s": rate, "load": args.load, "replicas": world,
                           "dispatch": "least assigned work (n_low x horizon), arrival order",
                           "capacity_low_particle_steps_per_s": cap, "hbm_budget_gb_per_gpu": args.budget_gb,
                           "parallelism": f"replicas{world}"},
                "served": len(served), "latency_s": latency_summary(stats),
                "low_particle_steps_per_s": float(n_low[served] @ horizons[served]) / makespan,
                "e2e": {"value": ss / makespan, "unit": "scene-steps/s",
                        "h2d_bytes_per_step": float(sum(16 * sc.n_low + 8 * sc.n_wall for sc, _, _ in trace))
                        / max(summ["steps"], 1),
                        "d2h_bytes_per_step": float(sum(29 * 5 * sc.n_low for sc, _, _ in trace)) / max(summ["steps"], 1)},
                "gpu_launches": int(summ["steps"] * 12 + len(served) * 17), "clocks": clk}
        print(json.dumps(line), flush=True)
    dist.destroy_process_group()


def run_adaptive(args):
    """The adaptive stress workload: 8M low-res particles, a region of interest
    translating at 0.5 units/s with merging (particles split as it reaches them and
    merge back as it leaves them), `--steps` steps in chunks of `--check-every`.
    Between chunks (untimed): the exact mass check (4 #(low state 0) + #(high) ==
    4 N_low, i.e. m #low0 + m/4 #high constant) and, on a seeded 1% sample of each
    scale, the step's FP32 densities and accelerations against the FP64 oracle
    evaluated on the same state."""
    import torch
    import oracle as O
    from twoscalesplit_gb300 import _abi, build, scenes
    from twoscalesplit_gb300.solver import Solver
    build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    name = "adaptive_8m" if args.scene in ("dam_break_1m", "dam_break_1m_developed") else args.scene
    sc = scenes.make_scene(name, seed=0)
    sol = Solver.from_scene(sc)
    sol.set_arith(args.arith)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream
    n_low = sc.n_low
    K, every = args.steps, args.check_every
    rng = np.random.default_rng(1234)
    orc = O.Oracle(sc, 64)
    clocks = ClockSampler(None)
    clocks.start()
    dev_ms, parts, done = 0.0, 0.0, 0
    checks = []
    splits = removed = 0
    while done < K:
        k = min(every, K - done)
        c0 = sol.counts()
        # particles processed: low + high at the start of each step of the chunk
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sol.step(k, stream=sh)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        dev_ms += e0.elapsed_time(e1)
        c1 = sol.counts()
        parts += k * (n_low + 0.5 * (c0["n_high"] + c1["n_high"]))
        done += k
        # untimed checks on the state after `done` steps
        low, high = sol.download(0), sol.download(1)
        mass_ok = 4 * int((low["state"] == 0).sum()) + high["id"].shape[0] == 4 * n_low
        fresh = sol.get_fresh()
        orc.set_scale(0, low["id"], low["pos"], low["vel"], low["state"])
        orc.set_scale(1, high["id"], high["pos"], high["vel"], high["state"])
        orc.set_fresh(fresh)
        orc.set_steps(done)
        orc.step()
        sol.step(1, stream=sh)  # the same step on the GPU (counted in the next chunk's budget)
        torch.cuda.synchronize(dev)
        done += 1
        c2 = sol.counts()
        splits += c2["n_split_last"]
        removed += c2["n_removed_last"]
        rec = {"step": done, "mass_exact": bool(mass_ok), "n_high": c2["n_high"], "splits": c2["n_split_last"],
               "removed": c2["n_removed_last"]}
        for scale, tag in ((0, "low"), (1, "high")):
            gid = sol.copy(scale, _abi.TSS_BUF_SORTED_ID)
            if gid.shape[0] == 0:
                continue
            gd = sol.copy(scale, _abi.TSS_BUF_DENSITY).astype(np.float64)
            ga = sol.copy(scale, _abi.TSS_BUF_ACCEL).astype(np.float64)
            oid = orc.get(scale, "sorted_id")
            od, oa = orc.get(scale, "dens"), orc.get(scale, "acc")
            # align by particle id: FP64 cell hashing may order a boundary particle
            # into the neighbouring cell
            og, oo = np.argsort(gid, kind="stable"), np.argsort(oid, kind="stable")
            assert np.array_equal(gid[og], oid[oo]), "different particle sets"
            gd, ga, od, oa = gd[og], ga[og], od[oo], oa[oo]
            m = max(1, gid.shape[0] // 100)
            pick = rng.choice(gid.shape[0], m, replace=False)
            rd = np.abs(gd[pick] - od[pick]) / np.abs(od[pick])
            amag = np.linalg.norm(oa[pick], axis=1)
            err = np.linalg.norm(ga[pick] - oa[pick], axis=1)
            scale_a = float(np.sqrt(np.mean(amag ** 2)))
            big = amag >= 0.01 * scale_a
            ra = err[big] / amag[big]
            rec[tag] = {"sample": int(m), "dens_rel_max": float(rd.max()), "dens_rel_mean": float(rd.mean()),
                        "dens_rel_p999": float(np.percentile(rd, 99.9)),
                        "dens_frac_over_1e-5": float((rd > 1e-5).mean()),
                        "acc_rel_max": float(ra.max()), "acc_rel_p99": float(np.percentile(ra, 99)),
                        "acc_rel_median": float(np.median(ra)), "acc_err_max_over_rms": float(err.max() / scale_a),
                        "acc_err_max_over_g": float(err.max() / abs(float(sc.config.gravity))),
                        "acc_rel_over": "particles with |a| >= 1% of the sample's RMS acceleration"}
        checks.append(rec)
        print(json.dumps({"check": rec}), file=sys.stderr, flush=True)
    clk = clocks.stop()
    sol.sync()
    dens_max = max(c[t]["dens_rel_max"] for c in checks for t in ("low", "high") if t in c)
    dens_p999 = max(c[t]["dens_rel_p999"] for c in checks for t in ("low", "high") if t in c)
    dens_frac = max(c[t]["dens_frac_over_1e-5"] for c in checks for t in ("low", "high") if t in c)
    acc_rms = max(c[t]["acc_err_max_over_rms"] for c in checks for t in ("low", "high") if t in c)
    acc_g = max(c[t]["acc_err_max_over_g"] for c in checks for t in ("low", "high") if t in c)
    timed_steps = K - len(checks) if K > len(checks) else K
    line = {"metric": METRIC, "value": parts / (dev_ms / 1e3), "unit": UNIT, "n_gpus": 1, "steps": K,
            "warmup": 0, "ms_per_step": dev_ms / max(done - len(checks), 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": sc.name, "n_low": n_low, "cap_high": sc.cap_high, "dt": float(sc.config.dt),
                       "arith": args.arith,
                       "roi": list(sc.config.roi), "roi_velocity": list(sc.config.roi_velocity),
                       "flags": int(sc.config.flags), "check_every": every,
                       "l2": "inputs larger than L2 (8M-particle state)"},
            "mass_exact_all_checks": all(c["mass_exact"] for c in checks),
            "splits_total": sol.counts()["total_split"], "removed_total": sol.counts()["total_removed"],
            "fp64_sample": {"dens_rel_max": dens_max, "dens_rel_p999": dens_p999, "dens_frac_over_1e-5": dens_frac,
                            "acc_err_max_over_rms": acc_rms, "acc_err_max_over_g": acc_g,
                            "checks": len(checks),
                            "tolerance": "dens 1e-5 relative"},
            "checks": checks, "clocks": clk, "gpu_launches": done * 12}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: 500 plain, 1000 batch, 2000 adaptive -- the configs' step counts)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scene", default="dam_break_1m_developed",
                    help="plain workload: dam_break_1m_developed (default), dam_break_1m or dam_break_5k")
    ap.add_argument("--start-cache", default=None,
                    help="plain workload: .npz of the developed start state (read if present, else written)")
    ap.add_argument("--cpu-budget-s", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="plain", choices=["plain", "batch", "serve", "adaptive"])
    ap.add_argument("--check-every", type=int, default=100)
    ap.add_argument("--scenes", type=int, default=512)
    ap.add_argument("--plain-sample", type=int, default=64)
    ap.add_argument("--requests", type=int, default=400)
    ap.add_argument("--load", type=float, default=0.8)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--chunk", type=int, default=8)
    ap.add_argument("--burst", type=int, default=128)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--capacity-lps", type=float, default=0.0)
    ap.add_argument("--no-plain", action="store_true", help="serve workload: skip the plain-solver comparison")
    ap.add_argument("--plain-requests", type=int, default=0,
                    help="serve workload: time the plain solver on this many sampled requests (0: all)")
    ap.add_argument("--arith", default=None, choices=["exact", "fast", "both"],
                    help="the gathers' arithmetic (plain and batch default: both; serve, adaptive: exact)")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shape of the gathers")
    ap.add_argument("--launch-cache", default=None, help="launch-shape cache file (default: the user cache)")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = {"plain": 500, "batch": 1000, "adaptive": 2000}.get(args.workload, 200)
    if args.arith is None:
        args.arith = "both" if args.workload in ("batch", "plain") else "exact"
    if args.arith == "both" and args.workload in ("serve", "adaptive"):
        sys.exit("--arith both is for the batch workload")
    if args.workload == "batch":
        run_batch(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "adaptive":
        run_adaptive(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
