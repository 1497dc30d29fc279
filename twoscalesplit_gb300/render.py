"""Headless rendering over the C ABI (include/tss.h): particle splats into a device
RGBA image, the reference's display() without OpenGL (TwoScale2D/main.cpp:65-102),
and a PPM writer for the frames."""
import ctypes

import numpy as np

from . import _abi
from ._abi import check, load_library


def view(xs, ys, xe, ye, width=1100, height=1100):
    """A display rectangle and image size (the reference's window was 1100 x 1100)."""
    return _abi.TssView(float(xs), float(ys), float(xe), float(ye), int(width), int(height))


def splats(v, pos, dens=None, rest_density=1000.0, rgb=None, point_size=0.005, img=None, stream=None):
    """Blend particles (a torch CUDA tensor n x 2) into `img` (torch CUDA tensor
    height x width x 4; a cleared image when None) with tss_render_splats."""
    import torch
    lib = load_library()
    if img is None:
        img = torch.empty((v.height, v.width, 4), dtype=torch.float32, device="cuda")
        check(lib.tss_render_clear(ctypes.c_void_p(img.data_ptr()), v.width, v.height,
                                   ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    n = int(pos.shape[0])
    ws = ctypes.c_size_t(0)
    check(lib.tss_render_workspace_size(n, ctypes.byref(v), float(point_size), ctypes.byref(ws)))
    work = torch.empty(ws.value, dtype=torch.uint8, device="cuda")
    c = None if rgb is None else np.asarray(rgb, np.float32)
    s = stream if stream else torch.cuda.current_stream().cuda_stream
    check(lib.tss_render_splats(ctypes.byref(v), n, ctypes.c_void_p(pos.data_ptr()) if n else None,
                                ctypes.c_void_p(dens.data_ptr()) if dens is not None else None, float(rest_density),
                                _abi.fptr(c), float(point_size), ctypes.c_void_p(img.data_ptr()),
                                ctypes.c_void_p(work.data_ptr()), ws.value, ctypes.c_void_p(s)))
    return img


def write_ppm(path, img):
    """Write an RGBA float image (row 0 at the bottom) as a binary PPM (top row first)."""
    a = np.asarray(img)[::-1, :, :3]
    b = np.clip(np.rint(a * 255.0), 0, 255).astype(np.uint8)
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (b.shape[1], b.shape[0]))
        f.write(b.tobytes())
