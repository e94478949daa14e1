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


# ------------------------------------------------- stripes node order ----
PI = 3.1415926535  # helper.hpp:47


def farthest_point_order(points):
    """farthest_control_points_sampling with node_num = len(points)
    (helper.cpp:139-177) and FetchFirstNodeIdx (helper.cpp:180-195): the
    order in which the viewer takes every mesh vertex as a node when the graph
    is built on a mesh ("Build Graph on Mesh", GaussianView.cpp:2268-2273).
    The first node has the largest float32 coordinate sum (first of equals);
    each next one the largest distance to the nodes taken (first of equals),
    distances float32(sqrt(double sum of squared float differences)) as
    pts_distance (helper.cpp:60-63)."""
    p = np.asarray(points, F32)
    n = p.shape[0]
    sums = np.zeros(n, F32)
    for j in range(3):
        sums = (sums + p[:, j]).astype(F32)
    first = int(np.argmax(sums))           # argmax returns the first maximum
    order = [first]
    dist = np.full(n, np.finfo(F32).max, F32)
    for i in range(n):
        if i == first:
            continue
        last = p[order[-1]]
        d = (p - last).astype(F32).astype(np.float64)
        dd = np.sqrt((d * d).sum(1)).astype(F32)
        dist = np.minimum(dist, dd)
        order.append(int(np.argmax(dist)))
        if len(order) == n:
            break
    return np.asarray(order, np.int64)


# ------------------------------------------------ stripes deform scripts ----
# LoadDeformScript0..6 (GaussianView.cpp:2512-2788): two blocks of nodes of
# the stripes graph, one kept at its start positions (type 0) and one moved
# (type 1) along 50 (39) steps.  Per script: the moved block (1 or 2), the
# types, the steps, and its motion.
STRIPES_SCRIPTS = {
    0: dict(moved=2, types=(0, 1), steps=50, kind="bend", center=(0.0, -1.5, 0.0), axis=(0.0, 0.0, 1.0),
            k=5.4, a="3pi2/k2", y_sign=1.0, turn=-1.0),
    1: dict(moved=2, types=(0, 1), steps=50, kind="turn", center=(0.0, -1.5, 0.0), axis=(0.0, 1.0, 0.0), turn=-1.5),
    2: dict(moved=2, types=(0, 1), steps=50, kind="bend", center=(0.0, -1.5, 0.0), axis=(0.0, 0.0, 1.0),
            k=3.0, a="pi/k-pi2/2k", y_sign=-1.0, turn=-0.5),
    3: dict(moved=1, types=(1, 0), steps=50, kind="bend", center=(0.0, 1.5, 0.0), axis=(0.0, 0.0, 1.0),
            k=3.0, a="pi/k-pi2/2k", y_sign=1.0, turn=0.5),
    4: dict(moved=2, types=(0, 1), steps=39, kind="bend", center=(0.0, -1.5, 0.0), axis=(0.0, 0.0, 1.0),
            k=8.4, a="3pi2/k2", y_sign=1.0, turn=-1.0),
    5: dict(moved=2, types=(0, 1), steps=39, kind="turn", center=(0.0, -1.5, 0.0), axis=(0.0, 1.0, 0.0), turn=-1.5),
    6: dict(moved=2, types=(0, 1), steps=50, kind="slide", dx=0.01),
}


def stripes_script_aims(script, start_pos, inter_steps=50):
    """The moved block's aims of every step of one script, float32
    [steps, m, 3], from its nodes' start positions [m, 3]: a rotation of
    turn*pi*step/inter_steps about the line through ``center`` along ``axis``,
    plus for "bend" a parabolic offset (x, y_sign*a*x^2, 0) with
    x = step*(-k/pi)/inter_steps; for "slide" a shift of -dx*step along x."""
    c = STRIPES_SCRIPTS[script]
    start = np.asarray(start_pos, F32)
    out = []
    for step in range(1, c["steps"] + 1):
        if c["kind"] == "slide":
            out.append((start - F32(c["dx"]) * F32(step) * np.array([1, 0, 0], F32)).astype(F32))
            continue
        radian = F32(c["turn"] * PI * step / inter_steps)
        rot = np.stack([point_rotate_by_axis(p, c["center"], c["axis"], radian) for p in start])
        if c["kind"] == "bend":
            k = F32(c["k"])
            a = F32(3.0 * PI * PI / (float(k) * float(k))) if c["a"] == "3pi2/k2" else \
                F32(PI / float(k) - PI * PI / (2 * float(k)))
            x = F32(step * (-float(k) / PI) / inter_steps)
            y = F32(c["y_sign"]) * a * x * x
            rot = (rot + np.array([x, y, 0.0], F32)).astype(F32)
        out.append(rot.astype(F32))
    return np.stack(out)
