"""The C++ drop-in (include/tss.hpp) builds against the library; on a GPU it runs
the reference's own scene setup headless."""
import os
import subprocess

import numpy as np
import pytest

from twoscalesplit_gb300 import _abi, build, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dam_break_main.cpp")


def _compile(out):
    # no contraction of the host arithmetic (the lattice generators' xs + dx * i): on
    # an Arm host g++ would fuse it into an FMA, one rounding short of the
    # reference's (MSVC, /fp:precise) and of the Python scene built for the oracle
    build.build()
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), SRC,
                           "-o", out,
                           _abi.LIB_PATH, f"-Wl,-rpath,{os.path.dirname(_abi.LIB_PATH)}"])


def test_cpp_dropin_compiles_and_links(tmp_path):
    _compile(str(tmp_path / "dam_break"))
    assert os.path.exists(tmp_path / "dam_break")


def _read_state(path):
    raw = open(path, "rb").read()
    consts = np.frombuffer(raw, np.float32, 9, 0)
    off, out = 36, []
    for _ in range(2):
        n = int(np.frombuffer(raw, np.int32, 1, off)[0])
        off += 4
        d = {}
        for k, dt, m in (("id", np.int32, n), ("pos", np.float32, 2 * n), ("vel", np.float32, 2 * n),
                         ("state", np.uint8, n), ("dens", np.float32, n)):
            d[k] = np.frombuffer(raw, dt, m, off)
            off += m * np.dtype(dt).itemsize
        d["pos"], d["vel"] = d["pos"].reshape(-1, 2), d["vel"].reshape(-1, 2)
        out.append(d)
    return consts, out


@pytest.mark.gpu
def test_cpp_dropin_runs_reference_scene(tmp_path):
    """The reference's own scene (main.cpp:131-208) through the C++ drop-in, 60
    frames: every particle's id, position, velocity, state and density equals the
    FP32 oracle's for the same scene, bit for bit."""
    import oracle as O
    exe = str(tmp_path / "dam_break")
    _compile(exe)
    dump = str(tmp_path / "state.bin")
    frames = 60
    out = subprocess.check_output([exe, str(frames), dump], timeout=300).decode().split()
    n_low, n_high, steps = int(out[0]), int(out[1]), int(out[2])
    assert n_low == 101 * 151 and steps == frames and n_high % 4 == 0
    consts, got = _read_state(dump)
    m, r, rh, tait, cs, alpha, tension, dt, mw = (float(x) for x in consts)
    cfg = _abi.config_init(0.0, 0.0, 1.0, 1.0, r, rh, 1000.0, tait, cs, alpha, tension, dt)
    low = scenes.particle_box(0.205, 0.105, 0.0025, 101, 151)
    walls = scenes.particle_box_canvas(0.1, 0.1, 0.0025, 321, 321, 3, 3)
    sc = scenes.Scene(name="reference_main_cpp", config=cfg, low_pos=low, low_vel=np.zeros_like(low),
                      mass_low=m, mass_high=np.float32(m) / np.float32(4.0), cap_high=4 * low.shape[0],
                      wall_pos=walls, mass_wall=mw, steps=frames, dx=0.0025)
    orc = O.Oracle(sc, 32)
    for _ in range(frames):
        orc.step()
    for s in (0, 1):
        st = orc.state(s)
        assert np.array_equal(got[s]["id"], st["id"]), s
        assert np.array_equal(got[s]["state"], st["state"]), s
        for k in ("pos", "vel"):
            assert np.array_equal(got[s][k], st[k].astype(np.float32)), (s, k)
    # densities of the last step, in list order for the particles it sorted
    d0 = orc.get(0, "dens").astype(np.float32)
    assert np.array_equal(got[0]["dens"][: d0.shape[0]], d0)
