"""Headless frames: the reference renderer's dot splat on the GPU (libnbx
``nbx_render_frame``), returned as an image array or written as the reference's
P6 file (3D/CUDA/CUDA_NBody/src/Renderer.cpp:141-161)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import torch

from . import _lib as L
from ._lib import check, lib
from .barnes_hut import Context, State, _stream_ptr


def default_params(**kw) -> L.nbx_render_params:
    """Constants.h:31-38, updated with keyword overrides (width, height, render_scale,
    max_velocity_color, min_velocity_color, particle_brightness, particle_sharpness,
    dot_size, system_size)."""
    p = L.nbx_render_params()
    lib().nbx_render_params_default(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def system_size(s: State, n: int | None = None) -> float:
    """2 * BarnesHut::getSystemSize() (BarnesHut.cu:417-445; main.cu:95): twice the
    largest |coordinate| of the bodies, in FP32."""
    n = s.x.numel() if n is None else n
    m = torch.stack([s.x[:n].abs().max(), s.y[:n].abs().max(), s.z[:n].abs().max()]).max()
    return float(np.float32(2.0) * np.float32(m.item()))


class Frame:
    """Device scratch and output of one frame size; render() fills ``rgb``."""

    def __init__(self, params: L.nbx_render_params, device=None):
        self.p = params
        dev = device or torch.device("cuda")
        count = 3 * params.width * params.height
        self.accum = torch.empty(count, dtype=torch.float32, device=dev)
        self.rgb = torch.empty(count, dtype=torch.uint8, device=dev)

    def render(self, ctx: Context, s: State, n: int | None = None, stream=None) -> torch.Tensor:
        n = s.x.numel() if n is None else n
        check(lib().nbx_render_frame(ctx.h, C.byref(s.c), n, C.byref(self.p), self.accum.data_ptr(),
                                     self.rgb.data_ptr(), _stream_ptr(stream)), "nbx_render_frame", ctx.h)
        return self.rgb.view(self.p.height, self.p.width, 3)


def write_ppm(path: str, rgb) -> None:
    """The reference's frame file: 'P6\\n<w> <h>\\n255\\n' + bytes (Renderer.cpp:152-158)."""
    a = rgb.cpu().numpy() if isinstance(rgb, torch.Tensor) else np.asarray(rgb)
    h, w = a.shape[:2]
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(np.ascontiguousarray(a, np.uint8).tobytes())


def frame_path(directory: str, step: int, render_interval: int) -> str:
    """images/StepNNNNN.ppm with frame = step / renderInterval + 1 (Renderer.cpp:149-151)."""
    return os.path.join(directory, "Step%05d.ppm" % (step // render_interval + 1))
