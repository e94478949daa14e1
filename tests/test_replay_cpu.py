"""Replay of a deformation record (replay.py) on CPU: the per-frame plan the
viewer's history replay follows (GaussianView.cpp:1757-1916), the float32
operation parameters (GaussianView.cpp:2920-2983), and the driver's order of
calls, run against a stand-in deformer whose solve is exact (the nodes reach
their aims) and whose aims moves are the oracle's target generators."""
import importlib

import numpy as np
import pytest

from oracle import targets

PKG = "arap-deformation-of-gaussian-radiance-fields_gb300"
rec = importlib.import_module(PKG + ".record")
rp = importlib.import_module(PKG + ".replay")


class ExactDeformer:
    """Nodes only: each frame's solve puts every node on its aim, then the
    aims are re-anchored to the nodes, as ReloadAimPositions does."""

    def __init__(self, node_pos):
        self.node_pos = np.asarray(node_pos, np.float32).copy()
        self.aims = self.node_pos.copy()
        self.active = []
        self.calls = []

    def set_controls(self, blocks, types, constraints_on_center):
        self.active = [v for b, t in zip(blocks, types) if t == 1 for v in b]
        self.calls.append(("controls", [list(b) for b in blocks], list(types), constraints_on_center))

    def apply_op(self, op):
        self.calls.append(("op",) + tuple(op))
        if not self.active:
            return
        if op[0] == "translate":
            self.aims = targets.translate(self.aims, self.active, op[1])
        elif op[0] == "twist":
            self.aims = targets.twist(self.aims, self.node_pos, self.active, op[1], op[2])
        elif op[0] == "scale":
            self.aims = targets.scale(self.aims, self.node_pos, self.active, op[1])
        else:
            raise ValueError(op[0])

    def frame(self, stats=False):
        self.calls.append(("frame",))
        self.node_pos = self.aims.copy()
        return {"frame": len([c for c in self.calls if c[0] == "frame"])} if stats else None


def _record():
    h = rec.DeformHistory()
    h.nodes_on_mesh = 0
    h.node_vertices = list(range(6))
    # add [0,1], add [2,3], move (centre) x2, twist x1, scale x1, delete block 1, move (nodes) x1
    h.operation_types = [0, 0, 1, 2, 3, -2, 4]
    h.total_operations = len(h.operation_types)
    h.move_operations = 4
    h.block_nodes = [[0, 1], [2, 3]]
    h.mouse_movements = [np.array([[0.1, 0, 0], [0.1, 0, 0]], np.float32),
                         np.array([[100, 0, 0]], np.float32),
                         np.array([[250, 0, 0]], np.float32),
                         np.array([[0, 0, 0.5]], np.float32)]
    h.blocks_types_moves = [[1, 0], [1, 0], [1, -1], [1]]
    h.energy_on_centers = [1, 0, 0, 0]
    h.twist_axis = [np.zeros(4, np.float32), np.array([0, 0, 2, 9], np.float32),
                    np.zeros(4, np.float32), np.zeros(4, np.float32)]
    return h


NODES = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0], [0, 0, 1], [2, 2, 2]], np.float32)


def test_operation_parameters_in_float32():
    tw = rp.aim_op({"op": rec.OP_TWIST, "axis": np.array([0, 0, 2, 9], np.float32), "angle_step": -37})
    assert tw[0] == "twist" and tw[1] == (0.0, 0.0, 2.0)
    assert tw[2] == float(np.float32(0.005) * np.float32(-37))
    sc = rp.aim_op({"op": rec.OP_SCALE, "scale_step": 250})
    assert sc == ("scale", float(np.float32(np.float32(0.002) * np.float32(250)) + np.float32(1)))
    assert abs(sc[1] - 1.5) < 1e-6
    mv = rp.aim_op({"op": rec.OP_MOVE, "translation": np.array([1e-5, -2.5e-4, 3.25], np.float32)})
    assert mv == ("translate", tuple(float(v) for v in np.array([1e-5, -2.5e-4, 3.25], np.float32)))
    with pytest.raises(ValueError):
        rp.aim_op({"op": 7})


def test_frame_plan():
    plan = rp.frame_plan(_record())
    assert len(plan) == 5
    assert [f["op"][0] for f in plan] == ["translate", "translate", "twist", "scale", "translate"]
    assert [f["constraints_on_center"] for f in plan] == [True, True, False, False, False]
    assert plan[0]["blocks"] == [[0, 1], [2, 3]] and plan[0]["types"] == [1, 0]
    assert plan[3]["types"] == [1, -1]
    assert plan[4]["blocks"] == [[0, 1]] and plan[4]["types"] == [1]
    assert all(f["active"] == [0, 1] for f in plan)
    assert rp.first_controls(_record()) == ([[0, 1], [2, 3]], [1, 0])
    assert rp.first_controls(rec.DeformHistory()) == (None, None)


def test_replay_with_exact_solve():
    d = ExactDeformer(NODES)
    seen = []
    st = rp.Replay(d).run(_record(), stats=True, on_frame=lambda i, f, s: seen.append((i, f["op"][0])))
    assert [s["frame"] for s in st] == [1, 2, 3, 4, 5]
    assert seen == [(0, "translate"), (1, "translate"), (2, "twist"), (3, "scale"), (4, "translate")]
    # every frame sets the controls, then moves the aims, then solves
    kinds = [c[0] for c in d.calls]
    assert kinds == ["controls", "op", "frame"] * 5
    # the expected node positions in closed form (float64)
    p = NODES.astype(np.float64)
    p[[0, 1], 0] += 0.2
    c = p[[0, 1]].mean(axis=0)
    ang = 0.005 * 100
    R = np.array([[np.cos(ang), -np.sin(ang), 0], [np.sin(ang), np.cos(ang), 0], [0, 0, 1]])
    p[[0, 1]] = (p[[0, 1]] - c) @ R.T + c
    c = p[[0, 1]].mean(axis=0)
    p[[0, 1]] = c + 1.5 * (p[[0, 1]] - c)
    p[[0, 1], 2] += 0.5
    np.testing.assert_allclose(d.node_pos, p, atol=2e-6)
    np.testing.assert_array_equal(d.node_pos[2:], NODES[2:])


def test_replay_without_stats_and_empty_record():
    d = ExactDeformer(NODES)
    assert rp.Replay(d).run(_record()) == [None] * 5
    d = ExactDeformer(NODES)
    assert rp.Replay(d).run(rec.DeformHistory()) == [] and d.calls == []


def test_mismatched_block_types_raise():
    h = _record()
    h.blocks_types_moves[0] = [1]  # one type for two blocks: the viewer indexes past it
    with pytest.raises(ValueError):
        rp.frame_plan(h)
