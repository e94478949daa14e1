"""Known answer for the skinning oracle (oracle/skin.py), on CPU.

When every node moves by one rigid motion x -> R x + T, the ED blend
(GaussianView.cpp:3022-3040) moves every endpoint by it, because the weights
sum to one.  The refit (GaussianView.cpp:3081-3166) then gives:
- mean R mu + T;
- rotation R q;
- unchanged scale, since the endpoints sit at 2 (s + 1e-3) along each axis;
- covariance R Sigma R^T;
- SH rotated by R.
This follows from the reference's formulas alone."""
import numpy as np

from oracle import ed, skin


def _sym(c6):
    """Packed (xx, xy, xz, yy, yz, zz) to the 3x3 matrix."""
    return c6[:, [0, 1, 2, 1, 3, 4, 2, 4, 5]].reshape(-1, 3, 3)


def test_rigid_node_motion_moves_gaussians_rigidly():
    rng = np.random.default_rng(3)
    N, n, k = 400, 30, 6
    pos = rng.uniform(0, 1, (N, 3)).astype(np.float32)
    rot = rng.normal(size=(N, 4))
    rot = (rot / np.linalg.norm(rot, axis=1, keepdims=True)).astype(np.float32)
    scale = np.exp(rng.normal(-3, 0.3, (N, 3))).astype(np.float32)
    shs = rng.normal(0, 0.2, (N, 48)).astype(np.float32)
    nodes = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    E = skin.end_points(pos, rot, scale)
    idx, w = ed.knn_weights(E.reshape(-1, 3), nodes, k)

    a = np.array([0.3, -1.0, 0.5]) / np.linalg.norm([0.3, -1.0, 0.5])
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    ang = 0.7
    R = np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K
    T = np.array([0.2, 0.05, -0.3])
    rot_node = np.tile(R.T.reshape(9), (n, 1))          # column-major R per node
    g = nodes.astype(np.float64)
    trans_node = g @ R.T + T - g

    e_new, p2, q2, s2, sh2 = skin.skin_gaussians(E, idx, w, rot_node, trans_node, nodes, rot, scale, shs,
                                                 float_accumulate=False)
    np.testing.assert_allclose(e_new, E.astype(np.float64) @ R.T + T, atol=2e-6)
    np.testing.assert_allclose(p2, pos.astype(np.float64) @ R.T + T, atol=2e-6)
    np.testing.assert_allclose(s2, scale, rtol=1e-5)
    # q2 = R q up to sign
    Rq = skin.quat_normalize(skin.quat_mul(skin.quat_from_matrix(R)[None], rot.astype(np.float64)))
    assert np.abs(np.abs((q2 * Rq).sum(axis=1)) - 1).max() < 1e-6
    S0 = _sym(skin.covariance6(rot, scale))
    S1 = _sym(skin.covariance6(q2, s2))
    expect = np.einsum("ij,njk,lk->nil", R, S0, R)
    rel = np.linalg.norm(S1 - expect, axis=(1, 2)) / np.linalg.norm(expect, axis=(1, 2))
    assert rel.max() < 1e-5
    np.testing.assert_allclose(sh2, skin.rotate_sh(shs, R), atol=1e-5)
