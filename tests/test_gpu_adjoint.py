"""Adjoint of the skinning map and of the ARAP energy on the GPU.

The library exposes a forward/backward pair (arap_skin_gaussians /
arap_skin_gaussians_backward, arap_solver_energy_grad); here it is wrapped as a
torch.autograd.Function (test harness only) and checked against the float64
oracle adjoint and against float64 finite differences (eps = 1e-6) on 64
random node coordinates.  Tolerance: relative 2e-3 of the gradient scale
(float32 kernels)."""
import numpy as np
import pytest

from tests import _helpers as H

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _t(a):
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


class SkinFn(torch.autograd.Function):
    """(rot [n,9], trans [n,3]) -> (mu [N,3], Sigma packed [N,6])."""

    @staticmethod
    def forward(ctx, rot, trans, dev, node_pos, ends_in, eidx, ew, scale0, q0):
        N = ends_in.shape[1]
        table = dev.node_table(rot.contiguous(), trans.contiguous(), node_pos)
        ends = ends_in.clone()
        pos = torch.empty((N, 3), device="cuda")
        q = q0.clone()
        sc = torch.empty((N, 3), device="cuda")
        cov = torch.empty((N, 6), device="cuda")
        dev.skin_gaussians(ends, eidx, ew, table, scale0, pos, q, sc, None, cov)
        ctx.save_for_backward(table, ends_in, eidx, ew, scale0)
        ctx.dev = dev
        ctx.n = rot.shape[0]
        return pos, cov

    @staticmethod
    def backward(ctx, g_pos, g_cov):
        table, ends_in, eidx, ew, scale0 = ctx.saved_tensors
        g = ctx.dev.skin_gaussians_backward(ends_in, eidx, ew, table, scale0, g_pos.contiguous(),
                                            g_cov.contiguous(), ctx.n)
        return g[:, :9], g[:, 9:], None, None, None, None, None, None, None


def _setup(dev, name, N=3000, seed=0):
    from oracle import ed, skin
    sc = H.synth.make_scene(name)
    rng = np.random.default_rng(seed)
    sel = rng.choice(sc.n_gauss, N, replace=False)
    pos, rot, scale = sc.pos[sel], sc.rot[sel], sc.scale[sel]
    n = sc.n_nodes
    q = rng.standard_normal((n, 4)) * np.array([5, .2, .2, .2])
    R = skin.quat_to_matrix(skin.quat_normalize(q)) + 0.03 * rng.standard_normal((n, 3, 3))
    X = np.zeros((n, 12))
    X[:, :9] = R.transpose(0, 2, 1).reshape(n, 9)
    X[:, 9:] = 0.02 * rng.standard_normal((n, 3))
    ends, exyz = dev.end_points(_t(pos), _t(rot), _t(scale))
    eidx, ew = dev.compute_weights(exyz, _t(sc.node_pos), sc.k)
    return sc, pos, rot, scale, X, ends, eidx, ew


def test_skin_backward_matches_oracle_and_fd(dev):
    from oracle import skin
    sc, pos, rot, scale, X, ends, eidx, ew = _setup(dev, "twist20k")
    N, n, k = pos.shape[0], sc.n_nodes, sc.k
    rng = np.random.default_rng(1)
    g_mu = rng.standard_normal((N, 3))
    g_cov = rng.standard_normal((N, 6))
    rot_t = _t(X[:, :9].astype(np.float32)).requires_grad_(True)
    tr_t = _t(X[:, 9:].astype(np.float32)).requires_grad_(True)
    mu, cov = SkinFn.apply(rot_t, tr_t, dev, _t(sc.node_pos), ends, eidx, ew, _t(scale), _t(rot))
    ((mu * _t(g_mu.astype(np.float32))).sum() + (cov * _t(g_cov.astype(np.float32))).sum()).backward()
    gX = np.concatenate([rot_t.grad.cpu().numpy(), tr_t.grad.cpu().numpy()], 1).astype(np.float64)
    # oracle adjoint on the same inputs (float32 weights/endpoints, float64 math)
    e_in = ends.cpu().numpy().reshape(6, 3, N).transpose(2, 0, 1).astype(np.float64)
    io = eidx.cpu().numpy().reshape(k, 6, N).transpose(2, 1, 0).reshape(6 * N, k)
    wo = ew.cpu().numpy().reshape(k, 6, N).transpose(2, 1, 0).reshape(6 * N, k).astype(np.float64)
    X32 = np.concatenate([X[:, :9].astype(np.float32), X[:, 9:].astype(np.float32)], 1).astype(np.float64)
    G = skin.packed_to_sym(g_cov)
    gX_ref = skin.skin_backward(e_in, io, wo, X32, sc.node_pos, scale, g_mu, G)
    scale_g = np.abs(gX_ref).max()
    assert np.abs(gX - gX_ref).max() <= 2e-3 * scale_g, np.abs(gX - gX_ref).max() / scale_g
    # float64 finite differences on 64 random node coordinates
    def L(Xv):
        m, S = skin.skin_forward_from_nodes(e_in, io, wo, Xv, sc.node_pos, scale)
        return (g_mu * m).sum() + (G * S).sum()
    eps = 1e-6
    for _ in range(64):
        a, b = rng.integers(n), rng.integers(12)
        Xp = X32.copy()
        Xp[a, b] += eps
        Xm = X32.copy()
        Xm[a, b] -= eps
        fd = (L(Xp) - L(Xm)) / (2 * eps)
        assert abs(fd - gX_ref[a, b]) <= 1e-6 * scale_g + 1e-6 * abs(fd)
        assert abs(fd - gX[a, b]) <= 2e-3 * scale_g


def test_energy_gradient_matches_fd(dev):
    # gradient of E = |f|^2 is 2 J^T f when the weighting factor is 1
    from oracle import ed
    sc = H.synth.make_scene("bend4k")
    nb = ed.build_graph(sc.node_pos, sc.k)
    aidx, aw = ed.knn_weights(sc.pos[sc.node_vertex], sc.node_pos, sc.k)
    aims = H.oracle_aims(sc, sc.node_pos)
    pr = ed.EDProblem(sc.node_pos, nb, aidx, aw.astype(np.float32).astype(np.float64), sc.blocks,
                      sc.block_type, aims)
    rng = np.random.default_rng(4)
    x = ed.identity_x(pr.F) + 0.02 * rng.standard_normal(pr.F * 12)
    solver = dev.Solver(_t(nb.astype(np.int32)), _t(aidx.T.astype(np.int32)), _t(aw.T.astype(np.float32)),
                        sc.blocks, sc.block_type, precision=1)
    g, e = solver.energy_grad(_t(sc.node_pos), _t(aims), _t(x))
    g = g.cpu().numpy()
    def E(v):
        f = ed.residual(pr, v)
        return f @ f
    for _ in range(64):
        i = rng.integers(x.size)
        xp = x.copy()
        xp[i] += 1e-6
        xm = x.copy()
        xm[i] -= 1e-6
        fd = (E(xp) - E(xm)) / 2e-6
        assert abs(fd - 2 * g[i]) <= 1e-5 * (abs(fd) + np.abs(g).max() * 1e-2)


def test_adjoint_pair_at_the_benchmark_scale(dev):
    """The forward/backward pair on the whole twist300k field: 300000
    Gaussians, 4061 nodes at the oracle's solved transforms, upstream
    gradients N(0,1) on mu [N,3] and Sigma [N,6].  The node gradient against
    the float64 oracle adjoint, float64 finite differences (eps = 1e-6) on
    64 random node coordinates (each evaluated on the Gaussians whose
    endpoints blend that node, the only ones it moves), and the energy
    gradient J^T f at the same transforms against the oracle's."""
    import os
    from oracle import ed, skin
    sc = H.synth.make_scene("twist300k")
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "solve_twist300k.npz"))
    X32 = g["x"].astype(np.float64)
    N, n, k = sc.n_gauss, sc.n_nodes, sc.k
    ends, exyz = dev.end_points(_t(sc.pos), _t(sc.rot), _t(sc.scale))
    eidx, ew = dev.compute_weights(exyz, _t(sc.node_pos), k)
    del exyz
    rng = np.random.default_rng(2)
    g_mu = rng.standard_normal((N, 3))
    g_cov = rng.standard_normal((N, 6))
    rot_t = _t(g["x"][:, :9]).requires_grad_(True)
    tr_t = _t(g["x"][:, 9:]).requires_grad_(True)
    mu, cov = SkinFn.apply(rot_t, tr_t, dev, _t(sc.node_pos), ends, eidx, ew, _t(sc.scale), _t(sc.rot))
    ((mu * _t(g_mu.astype(np.float32))).sum() + (cov * _t(g_cov.astype(np.float32))).sum()).backward()
    gX = np.concatenate([rot_t.grad.cpu().numpy(), tr_t.grad.cpu().numpy()], 1).astype(np.float64)
    e_in = ends.cpu().numpy().reshape(6, 3, N).transpose(2, 0, 1).astype(np.float64)
    io = eidx.cpu().numpy().reshape(k, 6, N).transpose(2, 1, 0).reshape(6 * N, k)
    wo = ew.cpu().numpy().reshape(k, 6, N).transpose(2, 1, 0).reshape(6 * N, k).astype(np.float64)
    G = skin.packed_to_sym(g_cov)
    gX_ref = skin.skin_backward(e_in, io, wo, X32, sc.node_pos, sc.scale, g_mu, G)
    scale_g = np.abs(gX_ref).max()
    err = np.abs(gX - gX_ref).max() / scale_g
    print("adjoint twist300k: max |dG| / max |G| = %.2e" % err)
    assert err <= 2e-3
    uses = io.reshape(N, 6 * k)
    eps = 1e-6
    for _ in range(64):
        a, b = rng.integers(n), rng.integers(12)
        sel = np.flatnonzero((uses == a).any(axis=1))
        rows = (sel[:, None] * 6 + np.arange(6)[None, :]).reshape(-1)

        def L(Xv):
            m, S = skin.skin_forward_from_nodes(e_in[sel], io[rows], wo[rows], Xv, sc.node_pos, sc.scale[sel])
            return (g_mu[sel] * m).sum() + (G[sel] * S).sum()
        Xp = X32.copy()
        Xp[a, b] += eps
        Xm = X32.copy()
        Xm[a, b] -= eps
        fd = (L(Xp) - L(Xm)) / (2 * eps)
        assert abs(fd - gX_ref[a, b]) <= 1e-6 * scale_g + 1e-6 * abs(fd)
        assert abs(fd - gX[a, b]) <= 2e-3 * scale_g
    # energy gradient at the solved transforms
    nb = ed.build_graph(sc.node_pos, k)
    aidx, aw = ed.knn_weights(sc.pos[sc.node_vertex], sc.node_pos, k)
    aims = H.oracle_aims(sc, sc.node_pos)
    pr = ed.EDProblem(sc.node_pos, nb, aidx, aw.astype(np.float32).astype(np.float64), sc.blocks, sc.block_type,
                      aims)
    x = X32[pr.free].reshape(-1)
    solver = dev.Solver(_t(nb.astype(np.int32)), _t(aidx.T.astype(np.int32)), _t(aw.T.astype(np.float32)),
                        sc.blocks, sc.block_type, precision=1)
    gE, e = solver.energy_grad(_t(sc.node_pos), _t(aims), _t(x))
    f = ed.residual(pr, x)
    gr = ed.gradient(pr, x)
    assert abs(e - f @ f) <= 1e-9 * (f @ f)
    assert H.rel_err(gE.cpu().numpy(), gr) <= 1e-8
    solver.close()


@pytest.mark.parametrize("name", ["twist20k", "stress40k"])
def test_planned_adjoint_matches_unplanned(dev, name):
    """arap_skin_gaussians_backward_planned (per-node sums over the plan's
    inverse lists) against arap_skin_gaussians_backward (shared-memory hash
    and atomics) on spatially ordered tiles (every tile within 256 nodes):
    the same gradient up to float rounding of the sums."""
    sc = H.synth.make_scene(name)
    key = np.floor((sc.pos - sc.pos.min(0)) / (np.ptp(sc.pos, 0).max() / 32)).astype(np.int64)
    perm = np.lexsort((key[:, 2], key[:, 1], key[:, 0]))
    pos0, rot0, scale0 = sc.pos[perm], sc.rot[perm], sc.scale[perm]
    N, n, k = pos0.shape[0], sc.n_nodes, sc.k
    rng = np.random.default_rng(5)
    from oracle import skin
    q = rng.standard_normal((n, 4))
    R = skin.quat_to_matrix(skin.quat_normalize(q * np.array([4, 0.3, 0.3, 0.3])))
    rot = (R + 0.02 * rng.standard_normal((n, 3, 3))).transpose(0, 2, 1).reshape(n, 9).astype(np.float32)
    tr = (0.05 * rng.standard_normal((n, 3))).astype(np.float32)
    table = dev.node_table(_t(rot), _t(tr), _t(sc.node_pos))
    ends, exyz = dev.end_points(_t(pos0), _t(rot0), _t(scale0))
    eidx, ew = dev.compute_weights(exyz, _t(sc.node_pos), k)
    plan = dev.SkinPlan(eidx, ew)
    assert plan.info()["overflow_tiles"] == 0
    g_mu = _t(rng.standard_normal((N, 3)).astype(np.float32))
    g_cov = _t(rng.standard_normal((N, 6)).astype(np.float32))
    g_ref = dev.skin_gaussians_backward(ends, eidx, ew, table, _t(scale0), g_mu, g_cov, n).cpu().numpy()
    g_pl = dev.skin_gaussians_backward_planned(plan, ends, table, _t(scale0), g_mu, g_cov, n).cpu().numpy()
    torch.cuda.synchronize()
    assert plan.status() == 0
    err = np.abs(g_pl - g_ref).max() / np.abs(g_ref).max()
    print("%s planned adjoint: max |d| / max |g| = %.2e" % (name, err))
    assert err <= 1e-4
    plan.close()
