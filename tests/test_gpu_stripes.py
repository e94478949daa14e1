"""The reference's own solver inputs on the GPU: the stripes deformation
graph (200 nodes, k = 10) driven by its seven deform scripts
(LoadDeformScript0..6, GaussianView.cpp:2512-2788), step after step as the
viewer runs them (GaussianView.cpp:1917-1993), against the float64 oracle's
frames (tests/golden/stripes_scripts.npz, made by
tests/golden/make_stripes_golden.py).

Per step: the graph and anchors built on the GPU (arap_build_graph,
arap_compute_weights), one solve (at most 30 Gauss-Newton iterations with
the stop test, Deform.cpp:95-169) in the benchmarked form, the node update
(arap_update_nodes), the next step from the updated nodes.  Checked: the
graph and anchor indices exactly; every step's Gauss-Newton iteration count
and line-search halvings; the node positions at the saved steps within
2e-5 of the bar's length (errors carry from step to step)."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _t(a):
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(HERE, "golden", "stripes_scripts.npz"))


@pytest.mark.parametrize("script", range(7))
def test_stripes_script_follows_the_oracle(dev, golden, script):
    from oracle import ed, targets
    g = golden
    k = int(g["k"])
    nodes0 = g["vertices"][g["order"]]
    n = nodes0.shape[0]
    nb = dev.build_graph(_t(nodes0), k)
    aidx, aw = dev.compute_weights(_t(nodes0), _t(nodes0), k)
    np.testing.assert_array_equal(nb.cpu().numpy(), ed.build_graph(nodes0, k))
    ref_idx, ref_w = ed.knn_weights(nodes0, nodes0, k)
    np.testing.assert_array_equal(aidx.cpu().numpy().T, ref_idx)
    assert np.abs(aw.cpu().numpy().T - ref_w).max() <= 2e-6
    c = targets.STRIPES_SCRIPTS[script]
    blocks = [g["s%d_block1" % script], g["s%d_block2" % script]]
    types = g["s%d_types" % script]
    moved, kept = blocks[c["moved"] - 1], blocks[2 - c["moved"]]
    solver = dev.Solver(nb, aidx, aw, blocks, types, max_iters=30, early_exit=1, precision=1, coarse_nodes=64)
    aims_moved = g["s%d_aims" % script]
    pos = _t(nodes0)
    saved = list(g["s%d_saved" % script])
    iters, halvings, errs = [], [], []
    for step in range(aims_moved.shape[0]):
        aims = pos.clone()
        aims[_t(kept.astype(np.int64))] = _t(nodes0[kept])
        aims[_t(moved.astype(np.int64))] = _t(aims_moved[step])
        rot, tr, st = solver.solve(pos, aims)
        assert st["status"] == 0
        iters.append(st["gn_iterations"])
        halvings.append(st["iteration_halvings"])
        table = dev.node_table(rot, tr, pos)
        pos = dev.update_nodes(pos, aidx, aw, table)
        if step in saved:
            ref = g["s%d_nodes" % script][saved.index(step)]
            errs.append(float(np.abs(pos.cpu().numpy() - ref).max()) / 3.0)
    ref_h = [[int(v) for v in row if v >= 0] for row in g["s%d_halvings" % script]]
    print("script %d: GN iterations %s (oracle %s), node error by saved step %s" % (
        script, iters, g["s%d_iters" % script].tolist(), ["%.1e" % e for e in errs]))
    assert iters == g["s%d_iters" % script].tolist()
    assert halvings == ref_h
    assert max(errs) <= 2e-5
    solver.close()
