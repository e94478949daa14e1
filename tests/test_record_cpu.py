"""Deformation records (record.py): the viewer's deform.txt format
(GaussianView.cpp:4859-5095) and the replay bookkeeping (1757-1916), on CPU.

The dataset's one real record is pinned by tests/golden/deform_record_pinocchio.json
(made by tests/golden/make_deform_golden.py): format_deform reproduces it byte
for byte.  Here, synthetic records exercise every operation type."""
import importlib
import json
import os

import numpy as np
import pytest

rec = importlib.import_module("arap-deformation-of-gaussian-radiance-fields_gb300.record")
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "deform_record_pinocchio.json")


def _history():
    h = rec.DeformHistory()
    h.nodes_on_mesh = 1
    h.node_vertices = [5, 17, 2, 40, 33, 8]
    # add, add, twist, add, delete block 0, scale, move (centre), move (nodes)
    h.operation_types = [0, 0, 2, 0, -1, 3, 1, 4]
    h.total_operations = len(h.operation_types)
    h.move_operations = 4
    h.block_nodes = [[0, 1], [2, 3, 4], [5]]
    h.mouse_movements = [np.array([[3.0, 0, 0], [-2.7, 0, 0]], np.float32),
                         np.array([[1.9, 0, 0]], np.float32),
                         np.array([[1e-5, -2.5e-4, 3.25]], np.float32),
                         np.array([[0.1, 0.2, 0.3], [1234567.0, -0.000123456789, 7]], np.float32)]
    h.blocks_types_moves = [[1, 0], [0, 1], [1, 0], [0, -1]]
    h.energy_on_centers = [0, 0, 1, 0]
    h.twist_axis = [np.array([0, 0, 1, 0.5], np.float32), np.zeros(4, np.float32),
                    np.zeros(4, np.float32), np.zeros(4, np.float32)]
    return h


def test_round_trip_is_byte_exact(tmp_path):
    h = _history()
    a = str(tmp_path / "a.txt")
    rec.write_deform(a, h)
    h2 = rec.read_deform(a)
    b = str(tmp_path / "b.txt")
    rec.write_deform(b, h2)
    assert open(a, "rb").read() == open(b, "rb").read()
    assert h2.operation_types == h.operation_types and h2.block_nodes == h.block_nodes
    for m, m2 in zip(h.mouse_movements, h2.mouse_movements):
        np.testing.assert_allclose(m2, m, rtol=1e-5)


def test_float_tokens_as_cpp_streams_write_them():
    # std::ostream's default for a float: %g with 6 significant digits
    h = rec.DeformHistory()
    h.mouse_movements = [np.array([[-9.12547e-05, 1234567.0, 0.5]], np.float32)]
    text = rec.format_deform(h)
    assert "-9.12547e-05 1.23457e+06 0.5 " in text
    assert text.endswith("Twist_Axis: 0 ")


def test_replay_steps():
    steps = rec.replay_steps(_history())
    kinds = [s["kind"] for s in steps]
    assert kinds == ["add", "add", "move", "move", "add", "delete", "move", "move", "move", "move"]
    assert steps[0]["blocks"] == [[0, 1]] and steps[0]["types"] == [1]
    assert steps[1]["types"] == [1, 0]
    tw = steps[2]
    assert tw["op"] == rec.OP_TWIST and tw["angle_step"] == 3 and not tw["constraints_on_center"]
    np.testing.assert_array_equal(tw["axis"], [0, 0, 1, 0.5])
    assert tw["types"] == [1, 0]
    assert steps[3]["angle_step"] == -2  # truncation toward zero, as the viewer's (int) cast
    # the types a move set persist: a later block is added as type 0
    assert steps[4]["blocks"] == [[0, 1], [2, 3, 4], [5]] and steps[4]["types"] == [1, 0, 0]
    assert steps[5]["blocks"] == [[2, 3, 4], [5]] and steps[5]["types"] == [0, 0]
    sc = steps[6]
    assert sc["op"] == rec.OP_SCALE and sc["scale_step"] == 1 and sc["types"] == [0, 1]
    mv = steps[7]
    assert mv["op"] == rec.OP_MOVE_CENTRE and mv["constraints_on_center"]
    np.testing.assert_array_equal(mv["translation"], np.array([1e-5, -2.5e-4, 3.25], np.float32))
    assert steps[8]["op"] == rec.OP_MOVE and not steps[8]["constraints_on_center"]
    assert steps[9]["types"] == [0, -1]


def test_malformed_records(tmp_path):
    p = str(tmp_path / "bad.txt")
    text = rec.format_deform(_history())
    for broken in (text.replace("Block_Nodes:", "Blocks:"), text[: len(text) // 2], text + "7 "):
        open(p, "w").write(broken)
        with pytest.raises(ValueError):
            rec.read_deform(p)


def test_golden_digest_of_the_dataset_record():
    g = json.load(open(GOLDEN))
    assert g["round_trip_exact"] is True
    assert g["nodes"] == 501 and g["total_operations"] == 7 and g["move_operations"] == 3
    assert sum(g["frames_per_move"]) + len(g["block_sizes"]) == g["replay_frames"]
