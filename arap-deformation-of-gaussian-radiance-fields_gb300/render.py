"""Headless rendering of a Gaussian field into a device image (C ABI
``arap_render``): the published 3D Gaussian splatting forward standing in for
the rasteriser the viewer draws the deformed field with
(GaussianView.cpp:1066-1127), without a window or GL interop."""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import check
from .deform import _f32, _p, _s


def render(pos, shs, opacity, scale, rot, view, proj, campos, tan_fovx, tan_fovy, width, height,
           background=(0.0, 0.0, 0.0), sh_degree=3, scale_modifier=1.0):
    """(image [3,H,W], final transmittance [H,W], contributors [H,W]) as CUDA
    tensors.  ``view`` and ``proj`` are row-major 4x4 world->camera and
    world->clip matrices; the other attributes are activated, as skinned."""
    pos, shs, opacity, scale, rot = (_f32(t) for t in (pos, shs, opacity, scale, rot))
    N = pos.shape[0]
    vh = (C.c_float * 16)(*np.asarray(view, np.float32).reshape(16).tolist())
    ph = (C.c_float * 16)(*np.asarray(proj, np.float32).reshape(16).tolist())
    ch = (C.c_float * 3)(*np.asarray(campos, np.float32).reshape(3).tolist())
    bh = (C.c_float * 3)(*np.asarray(background, np.float32).reshape(3).tolist())
    img = torch.empty((3, int(height), int(width)), dtype=torch.float32, device="cuda")
    T = torch.empty((int(height), int(width)), dtype=torch.float32, device="cuda")
    n = torch.empty((int(height), int(width)), dtype=torch.int32, device="cuda")
    check("arap_render", _lib.load().arap_render(
        N, _p(pos), _p(shs), _p(opacity), _p(scale), _p(rot), float(scale_modifier), int(sh_degree),
        C.cast(vh, C.c_void_p), C.cast(ph, C.c_void_p), C.cast(ch, C.c_void_p), float(tan_fovx), float(tan_fovy),
        int(width), int(height), C.cast(bh, C.c_void_p), _p(img), _p(T), _p(n), _s()))
    return img, T, n
