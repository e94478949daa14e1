"""Oracle: control-target generators.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  Restated from
GaussianView.cpp:2920-2983 (UpdateAimPosition, UpdateAimPositionTwist,
UpdateAimPositionScale) and helper.cpp:1077-1100 (PointRotateByAxis), in
float32 like the reference's ``Pos`` arithmetic.  ``active`` lists the node
ids of the active blocks in block order; a repeated id is moved once per
occurrence, as the reference's loops do.
"""
from __future__ import annotations

import numpy as np

F32 = np.float32


def translate(aims, active, delta):
    out = np.asarray(aims, F32).copy()
    d = np.asarray(delta, F32)
    for i in np.asarray(active, np.int64):
        out[i] = (out[i] + d).astype(F32)
    return out


def _centroid(node_pos, active):
    p = np.asarray(node_pos, F32)[np.asarray(active, np.int64)].astype(np.float64)
    return p.mean(axis=0).astype(F32)


def point_rotate_by_axis(p, center, axis, radian):
    """PointRotateByAxis (helper.cpp:1077-1100): rotation by ``radian`` about
    the line through ``center`` with direction ``axis``."""
    p = np.asarray(p, F32)
    ct, st = F32(np.cos(F32(radian))), F32(np.sin(F32(radian)))
    ax = np.asarray(axis, F32)[:3]
    nrm = F32(np.sqrt((ax * ax).sum(dtype=F32)))
    x, y, z = ax / nrm
    a, b, c = np.asarray(center, F32)
    u = F32(1) - ct
    o = np.empty(3, F32)
    o[0] = (x * x * u + ct) * p[0] + (x * y * u - z * st) * p[1] + (x * z * u + y * st) * p[2]
    o[1] = (y * x * u + z * st) * p[0] + (y * y * u + ct) * p[1] + (y * z * u - x * st) * p[2]
    o[2] = (z * x * u - y * st) * p[0] + (z * y * u + x * st) * p[1] + (z * z * u + ct) * p[2]
    o[0] += (a * (y * y + z * z) - x * (b * y + c * z)) * u + (b * z - c * y) * st
    o[1] += (b * (x * x + z * z) - y * (a * x + c * z)) * u + (c * x - a * z) * st
    o[2] += (c * (x * x + y * y) - z * (a * x + b * y)) * u + (a * y - b * x) * st
    return o


def twist(aims, node_pos, active, axis, radian):
    out = np.asarray(aims, F32).copy()
    ctr = _centroid(node_pos, active)
    for i in np.asarray(active, np.int64):
        out[i] = point_rotate_by_axis(out[i], ctr, axis, radian)
    return out


def scale(aims, node_pos, active, s):
    out = np.asarray(aims, F32).copy()
    ctr = _centroid(node_pos, active)
    s = F32(s)
    for i in np.asarray(active, np.int64):
        out[i] = (ctr + s * (out[i] - ctr)).astype(F32)
    return out
