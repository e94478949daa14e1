"""Failure paths of the library on the GPU, made without a GPU fault.

* A grid-barrier wait of the persistent solve that runs out: the solver's
  spin limit is set to one poll, so the first barrier's waits give up; the
  kernel records ARAP_ETIMEOUT in the solver's own status word and every CTA
  leaves.  The context stays usable: the next solve is correct.
* ARAP_NOT_CONVERGED: early exit on and one iteration allowed (the reference
  only prints "exceed number of maximum iterations", Deform.cpp:112-115).
* Status words are per handle: an error raised by one solver or one caller's
  word is not seen by another.
"""
import numpy as np
import pytest

from tests import _helpers as H

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _t(a):
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


def _inputs(sc):
    from oracle import ed
    nb = ed.build_graph(sc.node_pos, sc.k)
    aidx, aw = ed.knn_weights(sc.pos[sc.node_vertex], sc.node_pos, sc.k)
    return nb, aidx, aw, H.oracle_aims(sc, sc.node_pos)


def _solver(dev, sc, nb, aidx, aw, **kw):
    return dev.Solver(_t(nb.astype(np.int32)), _t(aidx.T.astype(np.int32)), _t(aw.T.astype(np.float32)),
                      sc.blocks, sc.block_type, **kw)


@pytest.mark.parametrize("coarse", [0, 32])
def test_barrier_timeout_is_reported_and_recovered(dev, coarse):
    from oracle import ed
    sc = H.synth.make_scene("twist20k")
    nb, aidx, aw, aims = _inputs(sc)
    bad = _solver(dev, sc, nb, aidx, aw, max_iters=sc.iters, early_exit=0, precision=1, coarse_nodes=coarse,
                  spin_limit=1)
    good = _solver(dev, sc, nb, aidx, aw, max_iters=sc.iters, early_exit=0, precision=1, coarse_nodes=coarse)
    with pytest.raises(dev.ArapError) as e:
        bad.solve(_t(sc.node_pos), _t(aims))
    assert e.value.code == 4                      # ARAP_ETIMEOUT
    assert bad.status() == 0                      # read and cleared by the solve
    assert good.status() == 0                     # the other handle saw nothing
    # an asynchronous solve records the timeout in the solver's word
    bad.solve(_t(sc.node_pos), _t(aims), stats=False)
    torch.cuda.synchronize()
    assert bad.status() == 4 and good.status() == 0
    # the context is still usable and the other solver is exact
    rot, tr, st = good.solve(_t(sc.node_pos), _t(aims))
    assert st["status"] == 0
    pr = ed.EDProblem(sc.node_pos, nb, aidx, aw, sc.blocks, sc.block_type, aims)
    x, _ = ed.gauss_newton(pr, max_iters=sc.iters, early_exit=False)
    rot_r, tr_r = ed.put_free_inputs(pr, x)
    X = np.concatenate([rot.cpu().numpy(), tr.cpu().numpy()], 1)
    assert H.rel_err(X, np.concatenate([rot_r, tr_r], 1)) <= 1e-5
    bad.close()
    good.close()


def test_not_converged_is_reported():
    import importlib
    dev = importlib.import_module("arap-deformation-of-gaussian-radiance-fields_gb300.deform")
    sc = H.synth.make_scene("bend4k")
    nb, aidx, aw, aims = _inputs(sc)
    s = _solver(dev, sc, nb, aidx, aw, max_iters=1, early_exit=1, precision=1)
    _, _, st = s.solve(_t(sc.node_pos), _t(aims))   # the call itself succeeds
    assert st["status"] == 1                         # ARAP_NOT_CONVERGED
    assert st["gn_iterations"] == 1
    s2 = _solver(dev, sc, nb, aidx, aw, max_iters=30, early_exit=1, precision=1)
    _, _, st2 = s2.solve(_t(sc.node_pos), _t(aims))
    assert st2["status"] == 0 and st2["gn_iterations"] < 30
    s.close()
    s2.close()


def test_status_words_are_per_caller(dev):
    # all k+1 nearest nodes at the same distance: the reference's weights are
    # 0/0; the library writes NaNs and raises ARAP_ENONFINITE into the word
    # the caller passed, and nowhere else
    nodes = np.array([[1, 0, 0], [0, 1, 0], [-1, 0, 0], [0, -1, 0], [0, 0, 3]], np.float32)
    mine, other = dev.StatusWord(), dev.StatusWord()
    dev.device_status()
    dev.compute_weights(_t(np.zeros((1, 3), np.float32)), _t(nodes), 3, status=mine)
    assert other.read() == 0 and dev.device_status() == 0
    assert mine.read() == 2
    assert mine.read() == 0                          # cleared by the read
