"""Known answers for the ED / ARAP oracle (oracle/ed.py), on CPU.

A rigid motion of the whole graph, with R_i = R and t_i = R g_i + T - g_i for
every node, zeroes every residual row of CalcEnergyFunc (Deform.cpp:378-581):
- the orthogonality rows, since R is a rotation;
- the regulariser rows, since R (g_k - g_i) + g_i + t_i - g_k - t_k = 0;
- the constraint rows, since the weights sum to one, so
  sum_j w_j (R (v - g_j) + g_j + t_j) = R v + T.
So a Gauss-Newton solve (Deform.cpp:95-169) towards rigidly moved aims must
find that motion.  These follow from the reference's formulas alone."""
import numpy as np
import pytest

from oracle import ed


def _rotation(axis, angle):
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * K @ K


def _problem(aims_fn, cons_on_center=False, n=80, k=6, seed=0, blocks=None, types=None):
    rng = np.random.default_rng(seed)
    nodes = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    nb = ed.build_graph(nodes, k)
    aidx, aw = ed.knn_weights(nodes, nodes, k)
    if blocks is None:
        blocks, types = [np.arange(n)], [1]
    aims = aims_fn(nodes.astype(np.float64)).astype(np.float32)
    return nodes, ed.EDProblem(nodes, nb, aidx, aw, blocks, types, aims, cons_on_center=cons_on_center)


def _rigid_x(pr, R, T):
    g = pr.node_pos.astype(np.float64)[pr.free]
    X = np.zeros((pr.F, 12))
    X[:, 0:9] = R.T.reshape(1, 9)           # column-major R: columns are R's columns
    X[:, 9:12] = g @ R.T + T - g
    return X.reshape(-1)


def test_rest_state_is_a_zero():
    _, pr = _problem(lambda g: g)
    f = ed.residual(pr, ed.identity_x(pr.F))
    n_other = pr.n_rows - pr.n_ctrl_rows
    assert np.abs(f[:n_other]).max() == 0.0
    # the constraint rows are zero up to the rounding of the weights' sum
    assert np.abs(f[n_other:]).max() < 1e-13


@pytest.mark.parametrize("centre", [False, True])
def test_rigid_motion_zeroes_the_residual(centre):
    R = _rotation([1, 2, 0.5], 0.4)
    T = np.array([0.3, -0.1, 0.2])
    _, pr = _problem(lambda g: g @ R.T + T, cons_on_center=centre)
    f = ed.residual(pr, _rigid_x(pr, R, T))
    # the aims are float32, so the constraint rows keep their rounding
    assert np.abs(f).max() < 1e-5 * np.sqrt(pr.w_con) * (1 + 20 * centre)
    f_id = ed.residual(pr, ed.identity_x(pr.F))
    assert np.abs(f_id).max() > 1e-2


def test_translation_moves_only_the_constraint_rows():
    T = np.array([0.0, 0.3, 0.0])
    _, pr = _problem(lambda g: g + T)
    f = ed.residual(pr, ed.identity_x(pr.F))
    n_other = pr.n_rows - pr.n_ctrl_rows
    assert np.abs(f[:n_other]).max() == 0.0
    con = f[n_other:].reshape(-1, 3)
    np.testing.assert_allclose(con, np.tile(-np.sqrt(pr.w_con) * T, (con.shape[0], 1)), atol=1e-6)


def test_gauss_newton_recovers_a_rigid_motion():
    R = _rotation([0, 0, 1], 0.3)
    T = np.array([0.05, 0.1, -0.02])
    _, pr = _problem(lambda g: g @ R.T + T)
    x, st = ed.gauss_newton(pr, max_iters=15)
    X = x.reshape(pr.F, 12)
    assert st.final_energy < 1e-9
    np.testing.assert_allclose(X[:, 0:9], np.tile(R.T.reshape(9), (pr.F, 1)), atol=1e-5)
    g = pr.node_pos.astype(np.float64)[pr.free]
    np.testing.assert_allclose(X[:, 9:12], g @ R.T + T - g, atol=1e-5)


def test_static_block_keeps_its_nodes_and_unknowns():
    # a static (type -1) block leaves the unknowns, and its nodes' rows are
    # the 3k rows -t_k per node (Deform.cpp:520-536)
    n, k = 80, 6
    blocks = [np.arange(0, 10), np.arange(70, 80)]
    _, pr = _problem(lambda g: g, n=n, k=k, blocks=blocks, types=[-1, 1])
    assert pr.F == n - 10 and pr.static.tolist() == list(range(10))
    assert pr.n_rows == pr.F * (6 + 3 * k) + 10 * 3 * k + 3 * 10
    assert pr.n_cols == 12 * pr.F
