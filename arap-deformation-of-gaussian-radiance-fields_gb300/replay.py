"""Replay of a deformation record (the viewer's ``deform.txt``) through the
frame pipeline.

Follows the viewer's history replay (GaussianView.cpp:1757-1916).  Adds and
deletes only change the control blocks.  Every frame of a move operation
does three things:
- moves the aims of the active blocks (UpdateAimPosition / Twist / Scale,
  GaussianView.cpp:2920-2983);
- solves with a fresh ``Deform`` over the current blocks and types
  (GaussianView.cpp:1855-1862);
- skins the Gaussians and samples, then re-anchors the aims to the moved
  nodes (ReloadAimPositions).

The record's integer steps become float32 parameters as the viewer computes
them: a twist step ``y`` turns by ``0.005f * y`` radians
(GaussianView.cpp:2936), and a scale step scales by ``0.002f * y + 1``
(GaussianView.cpp:2962).  The twist axis is the record's (x, y, z, w) with
``w`` unused (PointRotateByAxis, helper.cpp:1077-1100).

The viewer's feature update after a replay (CheckMovedGaussians,
UpdateFeatures) is not part of the deformation path and is not driven here.
"""
from __future__ import annotations

import numpy as np

from .record import OP_MOVE, OP_MOVE_CENTRE, OP_SCALE, OP_TWIST, replay_steps

TWIST_RADIAN_PER_STEP = np.float32(0.005)
SCALE_PER_STEP = np.float32(0.002)


def aim_op(step):
    """The aims operation of one 'move' entry of ``replay_steps``, in the form
    ``GaussianDeformer.apply_op`` takes: ``("translate", (x, y, z))``,
    ``("twist", (ax, ay, az), radian)`` or ``("scale", s)``."""
    op = step["op"]
    if op in (OP_MOVE_CENTRE, OP_MOVE):
        return ("translate", tuple(float(v) for v in np.asarray(step["translation"], np.float32)))
    if op == OP_TWIST:
        radian = TWIST_RADIAN_PER_STEP * np.float32(step["angle_step"])
        axis = np.asarray(step["axis"], np.float32)[:3]
        return ("twist", tuple(float(v) for v in axis), float(radian))
    if op == OP_SCALE:
        s = SCALE_PER_STEP * np.float32(step["scale_step"]) + np.float32(1)
        return ("scale", float(s))
    raise ValueError("deform record: unknown move operation %r" % (op,))


def frame_plan(h):
    """One entry per solved frame of the record, in order.  Each entry holds
    ``blocks`` (graph-node ids of every control block), ``types`` (1 active,
    0 pinned, -1 excluded), ``active`` (the active blocks' node ids in block
    order, a repeated id once per occurrence as the viewer's loops visit it),
    ``constraints_on_center`` and ``op`` (see ``aim_op``).

    Raises ValueError where the viewer would index past its block list: a
    move whose recorded types do not match the blocks present."""
    plan = []
    for s in replay_steps(h):
        if s["kind"] != "move":
            continue
        blocks, types = s["blocks"], s["types"]
        if len(types) != len(blocks):
            raise ValueError("deform record: a move gives %d block types for %d blocks"
                             % (len(types), len(blocks)))
        active = [int(v) for b, t in zip(blocks, types) if t == 1 for v in b]
        plan.append({"blocks": blocks, "types": types, "active": active,
                     "constraints_on_center": bool(s["constraints_on_center"]), "op": aim_op(s)})
    return plan


def first_controls(h):
    """(blocks, types) of the record's first solved frame, to construct the
    deformer with; (None, None) when the record moves nothing."""
    plan = frame_plan(h)
    if not plan:
        return None, None
    return plan[0]["blocks"], plan[0]["types"]


class Replay:
    """Drives a record through a deformer: anything with the methods
    ``set_controls(blocks, types, constraints_on_center)``, ``apply_op(op)``
    and ``frame(stats=...)`` of ``deform.GaussianDeformer``."""

    def __init__(self, deformer):
        self.deformer = deformer

    def run(self, h, stats=False, on_frame=None):
        """Replays every frame of ``h``.  Returns the per-frame solve
        statistics (None entries without ``stats``).  ``on_frame(i, entry,
        stats)`` is called after each frame."""
        out = []
        for i, f in enumerate(frame_plan(h)):
            self.deformer.set_controls(f["blocks"], f["types"], f["constraints_on_center"])
            self.deformer.apply_op(f["op"])
            st = self.deformer.frame(stats=stats)
            out.append(st)
            if on_frame is not None:
                on_frame(i, f, st)
        return out
