"""The C++ drop-in (include/tss.hpp) builds against the library; on a GPU it runs
the reference's own scene setup headless."""
import os
import subprocess

import pytest

from twoscalesplit_gb300 import _abi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dam_break_main.cpp")


def _compile(out):
    build.build()
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", out,
                           _abi.LIB_PATH, f"-Wl,-rpath,{os.path.dirname(_abi.LIB_PATH)}"])


def test_cpp_dropin_compiles_and_links(tmp_path):
    _compile(str(tmp_path / "dam_break"))
    assert os.path.exists(tmp_path / "dam_break")


@pytest.mark.gpu
def test_cpp_dropin_runs_reference_scene(tmp_path):
    exe = str(tmp_path / "dam_break")
    _compile(exe)
    out = subprocess.check_output([exe, "60"], timeout=300).decode().split()
    n_low, n_high, steps = int(out[0]), int(out[1]), int(out[2])
    assert n_low == 101 * 151 and steps == 60 and n_high % 4 == 0
