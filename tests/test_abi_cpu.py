"""CPU checks of the C ABI library: it loads, exports every entry point that
include/tss.h declares, and its host-only calls behave (no GPU work here)."""
import ctypes
import math
import os
import re
import subprocess

import numpy as np
import pytest

from twoscalesplit_gb300 import _abi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(tss_[a-z_0-9]+)\s*\(", txt))
    return names


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _abi.load_library()


def test_library_exports_every_declared_entry_point(lib):
    declared = _declared()
    assert len(declared) >= 15
    out = subprocess.check_output(["nm", "-D", "--defined-only", _abi.LIB_PATH]).decode()
    exported = set(re.findall(r"\bT (tss_[a-z_0-9]+)\b", out))
    missing = declared - exported
    assert not missing, missing
    for name in declared:
        assert getattr(lib, name) is not None


def test_config_init_matches_reference_dimension_rule(lib):
    c = _abi.TssConfig()
    assert lib.tss_config_init(ctypes.byref(c), 0, 0, 1, 1, 0.016, 0.008, 1000, 1, 1, 0.05, 0.08, 1e-4) == 0
    assert list(c.dims_low) == [63, 63] and list(c.dims_high) == [125, 125]
    assert c.gravity == pytest.approx(9.81) and c.relax_dt_div == 10.0
    assert list(c.roi)[0] == 0.5 and math.isinf(c.roi[2])
    py = _abi.config_init(0, 0, 1, 1, 0.016, 0.008, 1000, 1, 1, 0.05, 0.08, 1e-4)
    for name, _ in _abi.TssConfig._fields_:
        a, b = getattr(c, name), getattr(py, name)
        assert (list(a) == list(b)) if hasattr(a, "__len__") else a == b, name
    # the reference throws on an empty domain; the ABI returns INVALID_ARG
    assert lib.tss_config_init(ctypes.byref(c), 1, 0, 0, 1, 0.1, 0.05, 1, 1, 1, 0, 0, 1) == _abi.TSS_INVALID_ARG
    with pytest.raises(ValueError):
        _abi.config_init(0, 1, 1, 0, 0.1, 0.05, 1, 1, 1, 0, 0, 1)


@pytest.mark.parametrize("xe,r", [(1.0, 0.0625), (1.032, 0.016), (0.30000001, 0.1), (7.5, 0.0011)])
def test_config_dims_match_float_ceil(lib, xe, r):
    c = _abi.TssConfig()
    lib.tss_config_init(ctypes.byref(c), 0, 0, xe, xe, r, r / 2, 1000, 1, 1, 0, 0, 1)
    f = np.float32
    assert c.dims_low[0] == math.ceil(f(f(xe) - f(0)) / f(r))


def test_status_strings_and_argument_checks(lib):
    for st in range(8):
        assert lib.tss_status_string(st)
    ws = ctypes.c_size_t(0)
    assert lib.tss_grid_workspace_size(-1, 4, 4, ctypes.byref(ws)) == _abi.TSS_INVALID_ARG
    assert lib.tss_grid_workspace_size(10, 0, 4, ctypes.byref(ws)) == _abi.TSS_INVALID_ARG
    assert lib.tss_grid_workspace_size(10, 4, 4, ctypes.byref(ws)) == 0 and ws.value > 0
    out = ctypes.c_void_p()
    c = _abi.TssConfig()
    assert lib.tss_solver_create(None, 0, None, None, 1.0, 0, 1.0, 0, None, 1.0, ctypes.byref(out)) != 0
    c = _abi.config_init(0, 0, 1, 1, 0.1, 0.05, 1000, 1, 1, 0, 0, 1e-4)
    assert lib.tss_solver_create(ctypes.byref(c), -1, None, None, 1.0, 0, 1.0, 0, None, 1.0,
                                 ctypes.byref(out)) == _abi.TSS_INVALID_ARG
    assert lib.tss_solver_step(None, 1, None) == _abi.TSS_INVALID_ARG
    t = ctypes.c_int64(0)
    assert lib.tss_solver_read_positions_async(None, None, 0, None, 0, None, None, ctypes.byref(t)) == \
        _abi.TSS_INVALID_ARG
    assert lib.tss_solver_read_wait(None, 0) == _abi.TSS_INVALID_ARG


def test_launch_struct_layout_and_argument_checks(lib, tmp_path):
    # the ctypes mirror of tss_launch has the C layout
    src = tmp_path / "sz.c"
    src.write_text('#include "tss.h"\n#include <stdio.h>\n#include <stddef.h>\n'
                   'int main(void){printf("%zu %zu\\n", sizeof(tss_launch), offsetof(tss_launch, persistent));'
                   'return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include", str(src),
                           "-o", str(exe)])
    size, off = map(int, subprocess.check_output([str(exe)]).split())
    assert size == ctypes.sizeof(_abi.TssLaunch) and off == _abi.TssLaunch.persistent.offset
    shape = {g: {"threads": t, "persistent": p, "per_warp": w}
             for g, t, p, w in zip(_abi.GATHER_NAMES, (64, 128, 256, 64), (True, False, False, True),
                                   (False, True, False, True))}
    assert _abi.TssLaunch.from_dict(shape).as_dict() == shape
    l = _abi.TssLaunch()
    assert lib.tss_solver_get_launch(None, ctypes.byref(l)) == _abi.TSS_INVALID_ARG
    assert lib.tss_solver_set_launch(None, ctypes.byref(l)) == _abi.TSS_INVALID_ARG
    n = ctypes.c_int(0)
    assert lib.tss_solver_autotune(None, 1, ctypes.byref(l), ctypes.byref(n)) == _abi.TSS_INVALID_ARG
