"""A deform.txt replay driven through the GPU frame pipeline (replay.Replay on
deform.GaussianDeformer) against the same frames run by the oracle: aims
moved, exact Gauss-Newton solve, node update (GaussianView.cpp:1757-1916)."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PKG = "arap-deformation-of-gaussian-radiance-fields_gb300"


def _record(sc, rec):
    h = rec.DeformHistory()
    h.nodes_on_mesh = 0
    h.node_vertices = [int(v) for v in sc.node_vertex]
    active = [b for b, t in zip(sc.blocks, sc.block_type) if t == 1][0]
    pinned = [b for b, t in zip(sc.blocks, sc.block_type) if t == 0][0]
    h.block_nodes = [[int(v) for v in active], [int(v) for v in pinned]]   # the first block added is active
    h.operation_types = [0, 0, 4, 2]
    h.total_operations = 4
    h.move_operations = 2
    h.mouse_movements = [np.array([[0, 0.03, 0], [0, 0.03, 0]], np.float32), np.array([[20, 0, 0]], np.float32)]
    h.blocks_types_moves = [[1, 0], [1, 0]]
    h.energy_on_centers = [0, 0]
    h.twist_axis = [np.zeros(4, np.float32), np.array([1, 0, 0, 0], np.float32)]
    return h


def test_replay_matches_the_oracle_frames():
    import torch
    from oracle import ed, targets
    dev = importlib.import_module(PKG + ".deform")
    rec = importlib.import_module(PKG + ".record")
    rp = importlib.import_module(PKG + ".replay")
    synth = importlib.import_module(PKG + ".synth")
    sc = synth.make_scene("bend4k")
    h = _record(sc, rec)
    blocks, types = rp.first_controls(h)
    cfg = dev.default_config(max_iters=sc.iters, early_exit=0, precision=1, coarse_nodes=0)
    d = dev.GaussianDeformer(torch.as_tensor(sc.pos), torch.as_tensor(sc.rot), torch.as_tensor(sc.scale),
                             torch.as_tensor(sc.shs), sc.node_vertex, sc.k, blocks, types, config=cfg)
    st = rp.Replay(d).run(h, stats=True)
    assert len(st) == 3 and all(s["status"] == 0 for s in st)

    node = sc.pos[np.asarray(sc.node_vertex)].astype(np.float32)
    nb = ed.build_graph(node, sc.k)
    aidx, aw = ed.knn_weights(node, node, sc.k)
    for f in rp.frame_plan(h):
        act = f["active"]
        op = f["op"]
        if op[0] == "translate":
            aims = targets.translate(node, act, op[1])
        elif op[0] == "twist":
            aims = targets.twist(node, node, act, op[1], op[2])
        else:
            aims = targets.scale(node, node, act, op[1])
        pr = ed.EDProblem(node, nb, aidx, aw, f["blocks"], f["types"], aims,
                          cons_on_center=f["constraints_on_center"])
        x, _ = ed.gauss_newton(pr, max_iters=sc.iters, early_exit=False)
        rot, tr = ed.put_free_inputs(pr, x)
        node = ed.ed_blend(node, aidx, aw, rot, tr, node)
    got = d.node_pos.cpu().numpy()
    ext = float(np.ptp(sc.pos, axis=0).max())
    assert np.abs(got - node).max() <= 1e-4 * ext
