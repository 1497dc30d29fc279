"""tss_grid_build_noalloc: the grid build for callers that cannot allocate device
memory (for example a host application's per-frame callback, where cudaMalloc and
cudaFree can stall the whole device, or a plug-in whose device memory belongs to its
host's memory manager).  Its scratch is a fixed array inside the library; these
tests check that it gives exactly what tss_grid_build gives with caller-provided
scratch, on consecutive calls (the shared array keeps the previous call's contents,
so the second call checks that the entry point clears what it must), and that sizes
beyond the array are refused.

This file runs last (pytest collects files alphabetically); it also passes alone in
a fresh process.
"""
import ctypes

import numpy as np
import pytest

from twoscalesplit_gb300 import _abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from twoscalesplit_gb300 import build
    build.build()
    import torch
    assert torch.cuda.is_available(), "needs a CUDA device"
    return _abi.load_library()


def _inputs(n, seed):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-0.05, 1.05, size=(n, 2)).astype(np.float32)  # includes clamped points
    ids = rng.permutation(3 * n)[:n].astype(np.int32)
    return pos, ids


def _run(lib, pos, ids, dims, noalloc):
    import torch
    n = ids.shape[0]
    dpos = torch.from_numpy(pos.reshape(-1)).cuda()
    did = torch.from_numpy(ids).cuda()
    order = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    off = torch.full((dims[0] * dims[1] + 1,), -7, dtype=torch.int32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    args = (ctypes.c_void_p(dpos.data_ptr()), ctypes.c_void_p(did.data_ptr()), n, 0.0, 0.0, 1.0 / dims[0],
            dims[0], dims[1], ctypes.c_void_p(order.data_ptr()), ctypes.c_void_p(off.data_ptr()))
    if noalloc:
        st = lib.tss_grid_build_noalloc(*args, stream)
    else:
        ws = ctypes.c_size_t(0)
        assert lib.tss_grid_workspace_size(n, dims[0], dims[1], ctypes.byref(ws)) == 0
        work = torch.empty(ws.value, dtype=torch.uint8, device="cuda")
        st = lib.tss_grid_build(*args, ctypes.c_void_p(work.data_ptr()), ws.value, stream)
    assert st == _abi.TSS_OK
    torch.cuda.synchronize()
    return order.cpu().numpy()[:n], off.cpu().numpy()


def test_noalloc_grid_build_matches_workspace_entry_point_on_consecutive_calls(lib):
    # two different problems back to back through the shared array
    for n, cells, seed in ((200_000, 700, 1), (37_013, 256, 2)):
        pos, ids = _inputs(n, seed)
        ref_order, ref_off = _run(lib, pos, ids, (cells, cells), noalloc=False)
        got_order, got_off = _run(lib, pos, ids, (cells, cells), noalloc=True)
        # integer outputs: the tolerance is exact equality
        assert np.array_equal(got_off, ref_off)
        assert np.array_equal(got_order, ref_order)
        assert got_off[0] == 0 and got_off[-1] == n


def test_noalloc_grid_build_empty_and_near_the_limit(lib):
    # n = 0: every cell empty, the offsets all zero
    order, off = _run(lib, np.zeros((0, 2), np.float32), np.zeros(0, np.int32), (64, 64), noalloc=True)
    assert order.shape == (0,) and np.array_equal(off, np.zeros(64 * 64 + 1, np.int32))
    # the largest problem of this grid whose workspace still fits the array, twice in a row
    dims = (1400, 1400)
    ws = ctypes.c_size_t(0)
    lo, hi = 1, 8_000_000
    while lo < hi:
        mid = (lo + hi + 1) // 2
        assert lib.tss_grid_workspace_size(mid, dims[0], dims[1], ctypes.byref(ws)) == 0
        if ws.value <= _abi.TSS_GRID_NOALLOC_MAX_BYTES:
            lo = mid
        else:
            hi = mid - 1
    n = lo
    assert lib.tss_grid_workspace_size(n + 1, dims[0], dims[1], ctypes.byref(ws)) == 0
    assert ws.value > _abi.TSS_GRID_NOALLOC_MAX_BYTES
    pos, ids = _inputs(n, 5)
    ref_order, ref_off = _run(lib, pos, ids, dims, noalloc=False)
    for _ in range(2):
        got_order, got_off = _run(lib, pos, ids, dims, noalloc=True)
        assert np.array_equal(got_off, ref_off) and np.array_equal(got_order, ref_order)


def test_noalloc_grid_build_refuses_sizes_beyond_its_array(lib):
    ws = ctypes.c_size_t(0)
    n, dim = 4_000_000, 2048
    assert lib.tss_grid_workspace_size(n, dim, dim, ctypes.byref(ws)) == 0
    assert ws.value > _abi.TSS_GRID_NOALLOC_MAX_BYTES
    # rejected on the host before any device work: null pointers are never touched
    st = lib.tss_grid_build_noalloc(None, None, n, 0.0, 0.0, 1.0 / dim, dim, dim, None, None, None)
    assert st == _abi.TSS_CAPACITY
