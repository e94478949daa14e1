"""3D Gaussian splatting binary PLY files (C ABI ``arap_ply_*``).

Mirrors the reference viewer's loadPly / loadPly_Origin / savePly
(GaussianView.cpp:43-339): loading returns the activated arrays the
deformation path works on (positions, degree-3 SH interleaved per
coefficient, logistic opacities, exponentiated scales, normalised
quaternions), optionally in the viewer's Morton order; saving writes the
viewer's degree-3 layout back, without the splats outside a box or flagged too
small.  Host memory only: no GPU is needed.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def ply_info(path):
    """(count, sh_degree, has_index) of a 3DGS PLY file."""
    n = C.c_int64()
    deg = C.c_int()
    idx = C.c_int()
    check("arap_ply_info", _lib.load().arap_ply_info(str(path).encode(), C.byref(n), C.byref(deg), C.byref(idx)))
    return int(n.value), int(deg.value), bool(idx.value)


def load_ply(path, morton_order=True, with_index=False):
    """Activated splats of a 3DGS PLY file: a dict of float32 arrays pos [N,3],
    shs [N,48], opacity [N], scale [N,3], rot [N,4], box_min [3], box_max [3]
    and, with with_index, the file's ``index`` property as int32 [N]."""
    n, _, has_index = ply_info(path)
    if with_index and not has_index:
        raise ValueError("%s has no index property" % path)
    out = {
        "pos": np.empty((n, 3), np.float32),
        "shs": np.empty((n, 48), np.float32),
        "opacity": np.empty((n,), np.float32),
        "scale": np.empty((n, 3), np.float32),
        "rot": np.empty((n, 4), np.float32),
        "box_min": np.empty((3,), np.float32),
        "box_max": np.empty((3,), np.float32),
    }
    index = np.empty((n,), np.int32) if with_index else None
    check("arap_ply_load", _lib.load().arap_ply_load(
        str(path).encode(), n, 1 if morton_order else 0, _ptr(out["pos"]), _ptr(out["shs"]),
        _ptr(out["opacity"]), _ptr(out["scale"]), _ptr(out["rot"]), _ptr(out["box_min"]), _ptr(out["box_max"]),
        _ptr(index)))
    if with_index:
        out["index"] = index
    return out


def save_ply(path, pos, shs, opacity, scale, rot, box_min, box_max, too_small=None):
    """Writes the splats inside [box_min, box_max] not flagged in too_small;
    returns how many were written."""
    f = lambda a, shape: np.ascontiguousarray(np.asarray(a, np.float32).reshape(shape))
    pos = f(pos, (-1, 3))
    n = pos.shape[0]
    arrs = [pos, f(shs, (n, 48)), f(opacity, (n,)), f(scale, (n, 3)), f(rot, (n, 4)), f(box_min, (3,)),
            f(box_max, (3,))]
    small = None if too_small is None else np.ascontiguousarray(np.asarray(too_small, np.uint8).reshape(n))
    written = C.c_int64()
    check("arap_ply_save", _lib.load().arap_ply_save(
        str(path).encode(), n, *[_ptr(a) for a in arrs], _ptr(small), C.byref(written)))
    return int(written.value)
