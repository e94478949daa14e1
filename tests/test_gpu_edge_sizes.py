"""Edge sizes of the frame kernels: no items at all, one item, and tiles
short of a full 128: Gaussian skinning (unplanned and planned), its adjoint
(unplanned and planned), sample skinning and the kNN weights, each against the
oracle (or the other form) on the same inputs."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _t(a):
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


def _np(t):
    return t.detach().cpu().numpy()


def _field(N, n=24, seed=0):
    rng = np.random.default_rng(seed)
    nodes = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    pos = rng.uniform(0.1, 0.9, (N, 3)).astype(np.float32)
    q = rng.standard_normal((N, 4))
    rot = (q / np.linalg.norm(q, axis=1, keepdims=True)).astype(np.float32)
    scale = np.exp(rng.normal(-3.5, 0.4, (N, 3))).astype(np.float32)
    shs = (0.2 * rng.standard_normal((N, 48))).astype(np.float32)
    from oracle import skin
    qn = rng.standard_normal((n, 4))
    R = skin.quat_to_matrix(skin.quat_normalize(qn * np.array([4, 0.3, 0.3, 0.3])))
    rt = (R + 0.02 * rng.standard_normal((n, 3, 3))).transpose(0, 2, 1).reshape(n, 9).astype(np.float32)
    tr = (0.05 * rng.standard_normal((n, 3))).astype(np.float32)
    return nodes, pos, rot, scale, shs, rt, tr


@pytest.mark.parametrize("N", [1, 5, 127, 129])
def test_skinning_at_edge_sizes(dev, N):
    from oracle import skin
    k = 4
    nodes, pos, rot, scale, shs, rt, tr = _field(N)
    ends, exyz = dev.end_points(_t(pos), _t(rot), _t(scale))
    eidx, ew = dev.compute_weights(exyz, _t(nodes), k)
    table = dev.node_table(_t(rt), _t(tr), _t(nodes))
    plan = dev.SkinPlan(eidx, ew)
    assert plan.info()["tiles"] == (N + 127) // 128
    outs = []
    for planned in (False, True):
        e = ends.clone()
        p = torch.empty((N, 3), device="cuda")
        q = _t(rot)
        s = torch.empty((N, 3), device="cuda")
        h = _t(shs)
        c = torch.empty((N, 6), device="cuda")
        if planned:
            dev.skin_gaussians_planned(plan, e, table, _t(scale), p, q, s, h, c, precision=1)
        else:
            dev.skin_gaussians(e, eidx, ew, table, _t(scale), p, q, s, h, c, precision=1)
        outs.append((_np(e), _np(p), _np(q), _np(h)))
    torch.cuda.synchronize()
    assert dev.device_status() == 0 and plan.status() == 0
    e_in = _np(ends).reshape(6, 3, N).transpose(2, 0, 1).copy()
    idx_o = _np(eidx).reshape(k, 6, N).transpose(2, 1, 0).reshape(6 * N, k)
    w_o = _np(ew).reshape(k, 6, N).transpose(2, 1, 0).reshape(6 * N, k).astype(np.float64)
    e_ref, p_ref, q_ref, s_ref, sh_ref = skin.skin_gaussians(
        e_in, idx_o, w_o, rt.astype(np.float64), tr.astype(np.float64), nodes, rot, scale, shs,
        float_accumulate=False)
    for e, p, q, h in outs:
        assert np.abs(e.reshape(6, 3, N).transpose(2, 0, 1) - e_ref).max() <= 2e-6
        assert np.abs(p - p_ref).max() <= 2e-6
        assert np.abs(1 - np.abs((q.astype(np.float64) * q_ref).sum(1))).max() <= 2e-6
        assert np.abs(h - sh_ref).max() <= 5e-5
    # the adjoint, planned against unplanned
    rng = np.random.default_rng(3)
    g_mu = _t(rng.standard_normal((N, 3)).astype(np.float32))
    g_cov = _t(rng.standard_normal((N, 6)).astype(np.float32))
    n = nodes.shape[0]
    g0 = _np(dev.skin_gaussians_backward(ends, eidx, ew, table, _t(scale), g_mu, g_cov, n))
    g1 = _np(dev.skin_gaussians_backward_planned(plan, ends, table, _t(scale), g_mu, g_cov, n))
    torch.cuda.synchronize()
    assert plan.status() == 0
    assert np.abs(g1 - g0).max() <= 1e-5 * max(1.0, np.abs(g0).max())
    plan.close()


@pytest.mark.parametrize("S", [1, 7, 129])
def test_sample_skinning_at_edge_sizes(dev, S):
    from oracle import skin
    k = 4
    nodes, _, _, _, _, rt, tr = _field(4)
    rng = np.random.default_rng(9)
    sp = rng.uniform(0.1, 0.9, (S, 3)).astype(np.float32)
    feat = (0.3 * rng.standard_normal((S, 48))).astype(np.float32)
    idx, w = dev.compute_weights(_t(sp), _t(nodes), k)
    table = dev.node_table(_t(rt), _t(tr), _t(nodes))
    quat = dev.node_quaternions(_t(rt))
    p, f = _t(sp), _t(feat)
    dev.skin_samples(p, idx, w, table, quat, f)
    p_ref, f_ref = skin.skin_samples(sp, _np(idx).T, _np(w).T, rt.astype(np.float64), tr.astype(np.float64),
                                     nodes, feat, float_accumulate=False)
    assert np.abs(_np(p) - p_ref).max() <= 2e-6
    assert np.abs(_np(f) - f_ref).max() <= 5e-5
    # positions only (no feature)
    p2 = _t(sp)
    dev.skin_samples(p2, idx, w, table)
    assert torch.equal(p2, p)


def test_empty_inputs_are_no_ops(dev):
    nodes = _t(np.random.default_rng(0).uniform(0, 1, (8, 3)).astype(np.float32))
    idx, w = dev.compute_weights(torch.empty((0, 3), device="cuda"), nodes, 4)
    assert idx.shape == (4, 0) and w.shape == (4, 0)
    table = dev.node_table(_t(np.tile(np.eye(3, dtype=np.float32).reshape(1, 9), (8, 1))),
                           torch.zeros((8, 3), device="cuda"), nodes)
    dev.skin_samples(torch.empty((0, 3), device="cuda"), idx, w, table)
    torch.cuda.synchronize()
    assert dev.device_status() == 0
