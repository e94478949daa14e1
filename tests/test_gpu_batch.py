"""Batched solves (arap_solver_batch_*): several instances of uneven node
counts in batched launches (waves) must give each instance's separate-solve
result (to reduction-order rounding), also when the batched solve is captured
in a CUDA graph and replayed, and with the autotuned CTA split."""
import numpy as np
import pytest

from tests import _helpers as H

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _t(a):
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


def _np(t):
    return t.detach().cpu().numpy()


SCENES = ["bend4k", "twist20k", "stress40k"]


@pytest.fixture(scope="module")
def instances(dev):
    from oracle import ed
    out = []
    for name in SCENES:
        sc = H.synth.make_scene(name)
        nb = ed.build_graph(sc.node_pos, sc.k)
        aidx, aw = ed.knn_weights(sc.pos[sc.node_vertex], sc.node_pos, sc.k)
        aims = H.oracle_aims(sc, sc.node_pos)
        out.append((sc, nb, aidx, aw, aims))
    return out


def _solvers(dev, instances, precision, coarse):
    solvers = []
    for sc, nb, aidx, aw, aims in instances:
        solvers.append(dev.Solver(_t(nb.astype(np.int32)), _t(aidx.T.astype(np.int32)),
                                  _t(aw.T.astype(np.float32)), sc.blocks, sc.block_type, max_iters=sc.iters,
                                  early_exit=0, precision=precision, coarse_nodes=coarse))
    return solvers


@pytest.mark.parametrize("precision,coarse", [(0, 0), (1, 32)])
def test_batch_matches_separate_solves(dev, instances, precision, coarse):
    solvers = _solvers(dev, instances, precision, coarse)
    pos = [_t(inst[0].node_pos) for inst in instances]
    aims = [_t(inst[4]) for inst in instances]
    separate = [s.solve(p, a) for s, p, a in zip(solvers, pos, aims)]
    batch = dev.SolverBatch(solvers)
    ctas = batch.ctas()
    assert ctas[0] == 0 and all(b > a for a, b in zip(ctas, ctas[1:]))
    rot_b, tr_b, st_b = batch.solve(pos, aims)
    for (rot, tr, st), rb, tb, sb in zip(separate, rot_b, tr_b, st_b):
        assert sb["status"] == 0
        assert sb["gn_iterations"] == st["gn_iterations"]
        X = np.concatenate([_np(rot), _np(tr)], axis=1)
        Xb = np.concatenate([_np(rb), _np(tb)], axis=1)
        assert H.rel_err(Xb, X) <= (2e-6 if precision == 1 else 2e-5)
        assert abs(sb["final_energy"] - st["final_energy"]) <= 1e-6 * st["final_energy"]
    batch.close()
    for s in solvers:
        s.close()


def test_batch_graph_capture_and_autotune(dev, instances):
    solvers = _solvers(dev, instances, 1, 32)
    pos = [_t(inst[0].node_pos) for inst in instances]
    aims = [_t(inst[4]) for inst in instances]
    batch = dev.SolverBatch(solvers)
    best = batch.autotune(pos, aims)
    assert best in (0.75, 1.0, 1.25, 1.5, 2.0)
    ref_rot, ref_tr, _ = batch.solve(pos, aims)
    ref = [np.concatenate([_np(r), _np(t)], axis=1) for r, t in zip(ref_rot, ref_tr)]
    rot = [torch.zeros_like(r) for r in ref_rot]
    tr = [torch.zeros_like(t) for t in ref_tr]
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side):
            batch.solve(pos, aims, rot, tr, stats=False)
    torch.cuda.current_stream().wait_stream(side)
    for replay in range(2):
        for r, t in zip(rot, tr):
            r.zero_()
            t.zero_()
        g.replay()
        torch.cuda.synchronize()
        for X0, r, t in zip(ref, rot, tr):
            X = np.concatenate([_np(r), _np(t)], axis=1)
            assert H.rel_err(X, X0) <= 1e-6, replay
    batch.close()
    for s in solvers:
        s.close()
