"""GPU parity: every kernel of libarap_gb300.so against the CPU oracle.

Tolerances (float32 kernels against the float64 oracle):
  kNN indices            exact
  kNN weights            relative 2e-6
  node transforms        max |dx| / max |x|   <= 1e-5 (mixed precision), 5e-5 (plain FP32)
  ED blend positions     max abs / scene extent <= 2e-6
  Gaussian mu            max abs / scene extent <= 2e-6
  Gaussian Sigma         per-Gaussian |dS|_F / |S|_F <= 2e-5 (p99.9) and 1e-4 (max);
                         flat Gaussians (stress scene, one axis ~1e-4 in a [0,4]^3 field)
                         1e-4 / 5e-4: the float32 endpoints carry ~1e-4 relative on
                         the flat axis, which also fixes the rotation to that level
  The library rounds each ED blend once; the oracle comparisons below use the
  oracle's exact (single-rounding) blend.  The reference rounds after every
  neighbour (float accumulation), a difference of a few float32 ulps.
  quaternion             |1 - |<q, q_ref>|| <= 2e-6
  SH / features          max abs <= 5e-5 (coefficients ~N(0, 0.2))
"""
import json
import os

import numpy as np
import pytest

from tests import _helpers as H

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _t(a, dtype=None):
    t = torch.as_tensor(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def _np(t):
    return t.detach().cpu().numpy()


@pytest.fixture(scope="module", params=["bend4k", "twist20k", "stress40k"])
def scene(request):
    return H.synth.make_scene(request.param)


# ---------------------------------------------------------------- kNN ----

def test_graph_exact(dev, scene):
    from oracle import ed
    nb = _np(dev.build_graph(_t(scene.node_pos), scene.k))
    ref = ed.build_graph(scene.node_pos, scene.k)
    assert np.array_equal(nb, ref)


def test_weights_exact(dev, scene):
    from oracle import ed, skin
    pts = np.concatenate([scene.pos, skin.end_points(scene.pos, scene.rot, scene.scale).reshape(-1, 3)])
    idx, w = dev.compute_weights(_t(pts), _t(scene.node_pos), scene.k)
    ridx, rw = ed.knn_weights(pts, scene.node_pos, scene.k)
    assert np.array_equal(_np(idx).T, ridx)
    np.testing.assert_allclose(_np(w).T, rw, rtol=2e-6, atol=1e-7)


def test_weights_edge_cases(dev):
    nodes = _t(np.random.default_rng(0).random((20, 3), dtype=np.float32))
    idx, w = dev.compute_weights(_t(np.zeros((0, 3), np.float32)), nodes, 4)
    assert idx.shape == (4, 0)
    with pytest.raises(dev.ArapError) as e:
        dev.compute_weights(_t(np.zeros((5, 3), np.float32)), nodes, 13)
    assert e.value.code == 7
    with pytest.raises(dev.ArapError) as e:
        dev.compute_weights(_t(np.zeros((5, 3), np.float32)), nodes[:4], 4)
    assert e.value.code == 3
    # k = 1: weight 1 (Deform.hpp:206)
    idx, w = dev.compute_weights(nodes[:3], nodes, 1)
    assert np.allclose(_np(w), 1.0)
    # maximum k
    idx, w = dev.compute_weights(nodes, nodes, 12)
    from oracle import ed
    ridx, rw = ed.knn_weights(_np(nodes), _np(nodes), 12)
    assert np.array_equal(_np(idx).T, ridx)


def test_weights_ties_lower_index(dev):
    # four nodes at equal distance from the origin point
    nodes = np.array([[1, 0, 0], [0, 1, 0], [-1, 0, 0], [0, -1, 0], [0, 0, 3]], np.float32)
    idx, _ = dev.compute_weights(_t(np.zeros((1, 3), np.float32)), _t(nodes), 3)
    assert list(_np(idx)[:, 0]) == [0, 1, 2]
    # all k+1 nearest at the same distance: the reference's weights are 0/0;
    # the library reports it
    assert dev.device_status() == 2
    assert dev.device_status() == 0


# ------------------------------------------------------------- solver ----

def _problem(scene):
    from oracle import ed
    import importlib
    importlib.import_module("arap-deformation-of-gaussian-radiance-fields_gb300.deform").device_status()
    nb = ed.build_graph(scene.node_pos, scene.k)
    aidx, aw = ed.knn_weights(scene.pos[scene.node_vertex], scene.node_pos, scene.k)
    aims = H.oracle_aims(scene, scene.node_pos)
    return nb, aidx, aw, aims


@pytest.mark.parametrize("precision,coarse", [(0, 0), (1, 0), (1, 32)])
def test_solve_matches_oracle(dev, scene, precision, coarse):
    from oracle import ed
    nb, aidx, aw, aims = _problem(scene)
    pr = ed.EDProblem(scene.node_pos, nb, aidx, aw, scene.blocks, scene.block_type, aims)
    x_ref, st_ref = ed.gauss_newton(pr, max_iters=scene.iters, early_exit=False)
    rot_ref, tr_ref = ed.put_free_inputs(pr, x_ref)
    solver = dev.Solver(_t(nb.astype(np.int32)), _t(aidx.T.astype(np.int32)), _t(aw.T.astype(np.float32)),
                        scene.blocks, scene.block_type, max_iters=scene.iters, early_exit=0,
                        precision=precision, coarse_nodes=coarse)
    rot, tr, st = solver.solve(_t(scene.node_pos), _t(aims))
    assert st["status"] == 0
    assert st["gn_iterations"] == scene.iters
    assert st["n_rows"] == pr.n_rows
    X = np.concatenate([_np(rot), _np(tr)], axis=1)
    Xr = np.concatenate([rot_ref, tr_ref], axis=1)
    err = np.abs(X - Xr).max() / np.abs(Xr).max()
    print("solve", scene.name, precision, coarse, "rel err", err, "pcg", st["pcg_iterations"],
          "E", st["final_energy"], st_ref.final_energy)
    assert abs(st["initial_energy"] - st_ref.energies[0]) <= 1e-5 * st_ref.energies[0]
    assert err <= (1e-5 if precision == 1 else 5e-5)


@pytest.mark.parametrize("precision,centre", [(0, 0), (1, 0), (1, 1)])
def test_energy_grad(dev, scene, precision, centre):
    from oracle import ed
    nb, aidx, aw, aims = _problem(scene)
    aw32 = aw.astype(np.float32).astype(np.float64)
    pr = ed.EDProblem(scene.node_pos, nb, aidx, aw32, scene.blocks, scene.block_type, aims,
                      cons_on_center=bool(centre))
    x = ed.identity_x(pr.F) + 0.02 * np.random.default_rng(3).standard_normal(pr.F * 12)
    solver = dev.Solver(_t(nb.astype(np.int32)), _t(aidx.T.astype(np.int32)), _t(aw.T.astype(np.float32)),
                        scene.blocks, scene.block_type, precision=precision, cons_on_center=centre)
    g, e = solver.energy_grad(_t(scene.node_pos), _t(aims), _t(x))
    f = ed.residual(pr, x)
    gr = ed.gradient(pr, x)
    tol = 1e-9 if precision == 1 else 2e-6
    assert abs(e - f @ f) <= tol * (f @ f)
    assert H.rel_err(_np(g), gr) <= tol


@pytest.mark.parametrize("coarse", [0, 32])
def test_solve_centre_mode_and_weighting(dev, coarse):
    # centre mode needs non-collinear block centroids: with two blocks the
    # rotation about the line through both centroids is free and J^T J is
    # singular (for the reference's Cholesky as for any solver).  The
    # two-level solve runs at its default PCG tolerance: on this
    # ill-conditioned system a 1e-7 target is below what the FP32 PCG vectors
    # resolve (measured: 8.6e-7 at 1e-6, 1.2e-5 at 1e-7)
    from oracle import ed
    sc = H.synth.make_scene("bend4k")
    nb, aidx, aw, aims = _problem(sc)
    p = sc.node_pos
    blocks = [np.flatnonzero((p[:, 0] < 0.1) & (p[:, 1] < 0.1)), np.flatnonzero((p[:, 0] < 0.1) & (p[:, 1] >= 0.1)),
              np.flatnonzero(p[:, 0] > 0.9)]
    types = [0, 0, 1]
    for cons, wf in ((1, 1.0), (0, 3.0)):
        pr = ed.EDProblem(sc.node_pos, nb, aidx, aw, blocks, types, aims,
                          cons_on_center=bool(cons), weighting_factor=wf)
        x_ref, _ = ed.gauss_newton(pr, max_iters=5, early_exit=False)
        rot_ref, tr_ref = ed.put_free_inputs(pr, x_ref)
        solver = dev.Solver(_t(nb.astype(np.int32)), _t(aidx.T.astype(np.int32)), _t(aw.T.astype(np.float32)),
                            blocks, types, max_iters=5, early_exit=0, cons_on_center=cons,
                            weighting_factor=wf, precision=1, pcg_tol=1e-7 if coarse == 0 else 1e-6,
                            coarse_nodes=coarse)
        rot, tr, st = solver.solve(_t(sc.node_pos), _t(aims))
        X = np.concatenate([_np(rot), _np(tr)], axis=1)
        Xr = np.concatenate([rot_ref, tr_ref], axis=1)
        assert st["n_rows"] == pr.n_rows
        assert np.abs(X - Xr).max() / np.abs(Xr).max() <= 1e-5, (cons, wf, coarse)


def test_solve_early_exit(dev):
    from oracle import ed
    sc = H.synth.make_scene("bend4k")
    nb, aidx, aw, aims = _problem(sc)
    pr = ed.EDProblem(sc.node_pos, nb, aidx, aw, sc.blocks, sc.block_type, aims)
    _, st_ref = ed.gauss_newton(pr, max_iters=30, early_exit=True)
    solver = dev.Solver(_t(nb.astype(np.int32)), _t(aidx.T.astype(np.int32)), _t(aw.T.astype(np.float32)),
                        sc.blocks, sc.block_type, max_iters=30, early_exit=1, precision=1)
    _, _, st = solver.solve(_t(sc.node_pos), _t(aims))
    assert st["gn_iterations"] <= 30
    assert abs(st["gn_iterations"] - st_ref.iterations) <= 2


def test_solver_bad_input(dev):
    nb = _t(np.zeros((4, 2), np.int32))
    bad = _t(np.full((2, 4), 7, np.int32))
    with pytest.raises(dev.ArapError) as e:
        dev.Solver(nb, bad, _t(np.ones((2, 4), np.float32)), [[0]], [0])
    assert e.value.code == 3


# ----------------------------------------------------------- skinning ----

def _random_transforms(n, rng, amp=0.3):
    from oracle import skin
    q = rng.standard_normal((n, 4))
    R = skin.quat_to_matrix(skin.quat_normalize(q * np.array([4, amp, amp, amp])))
    A = R + 0.02 * rng.standard_normal((n, 3, 3))
    rot = A.transpose(0, 2, 1).reshape(n, 9).astype(np.float32)   # column-major
    trans = (0.05 * rng.standard_normal((n, 3))).astype(np.float32)
    return rot, trans


def test_skin_gaussians(dev, scene):
    from oracle import ed, skin
    rng = np.random.default_rng(7)
    rot, trans = _random_transforms(scene.n_nodes, rng)
    N = scene.n_gauss
    ends, ends_xyz = dev.end_points(_t(scene.pos), _t(scene.rot), _t(scene.scale))
    ends_ref = skin.end_points(scene.pos, scene.rot, scene.scale)
    ext = float(np.ptp(scene.pos, axis=0).max())
    np.testing.assert_allclose(_np(ends).reshape(6, 3, N).transpose(2, 0, 1), ends_ref, atol=2e-7 * ext, rtol=0)
    eidx, ew = dev.compute_weights(ends_xyz, _t(scene.node_pos), scene.k)
    table = dev.node_table(_t(rot), _t(trans), _t(scene.node_pos))
    pos = torch.empty((N, 3), device="cuda")
    q = _t(scene.rot)
    sc = torch.empty((N, 3), device="cuda")
    shs = _t(scene.shs)
    cov = torch.empty((N, 6), device="cuda")
    e_in = _np(ends).reshape(6, 3, N).transpose(2, 0, 1).copy()
    dev.skin_gaussians(ends, eidx, ew, table, _t(scene.scale), pos, q, sc, shs, cov)
    torch.cuda.synchronize()
    assert dev.device_status() == 0
    # oracle on the same weights and transforms
    # library planes [k][e*N + i] -> oracle Gaussian-major rows [i*6 + e][k]
    idx_o = _np(eidx).reshape(scene.k, 6, N).transpose(2, 1, 0).reshape(6 * N, scene.k)
    w_o = _np(ew).reshape(scene.k, 6, N).transpose(2, 1, 0).reshape(6 * N, scene.k).astype(np.float64)
    rot64 = rot.astype(np.float64)
    e_ref, p_ref, q_ref, s_ref, sh_ref = skin.skin_gaussians(
        e_in, idx_o, w_o, rot64, trans.astype(np.float64), scene.node_pos, scene.rot, scene.scale, scene.shs,
        float_accumulate=False)
    ext = float(np.ptp(scene.pos, axis=0).max())
    e_gpu = _np(ends).reshape(6, 3, N).transpose(2, 0, 1)
    assert np.abs(e_gpu - e_ref).max() / ext <= 2e-6
    assert np.abs(_np(pos) - p_ref).max() / ext <= 2e-6
    dq = np.abs(1 - np.abs((_np(q).astype(np.float64) * q_ref).sum(1)))
    assert dq.max() <= 2e-6, dq.max()
    c_ref = skin.covariance6(q_ref, s_ref)
    c = _np(cov).astype(np.float64)
    def fro(v):
        return np.sqrt(v[:, 0] ** 2 + v[:, 3] ** 2 + v[:, 5] ** 2 + 2 * (v[:, 1] ** 2 + v[:, 2] ** 2 + v[:, 4] ** 2))
    rel = fro(c - c_ref) / fro(c_ref)
    print("cov rel p99.9", np.quantile(rel, 0.999), "max", rel.max())
    flat = scene.name.startswith("stress")
    assert np.quantile(rel, 0.999) <= (1e-4 if flat else 2e-5) and rel.max() <= (5e-4 if flat else 1e-4)
    assert np.abs(_np(shs) - sh_ref).max() <= (5e-4 if flat else 5e-5)


def test_skin_samples_and_sh_golden(dev):
    from oracle import skin
    g = json.load(open(os.path.join(GOLDEN, "sh_rotation.json")))
    cases = g["cases"]
    n = len(cases)
    R = np.array([c["R"] for c in cases], np.float64)
    rot = R.transpose(0, 2, 1).reshape(n, 9).astype(np.float32)       # column-major
    trans = np.zeros((n, 3), np.float32)
    nodes = np.zeros((n, 3), np.float32)
    quat = dev.node_quaternions(_t(rot))
    table = dev.node_table(_t(rot), _t(trans), _t(nodes))
    pos = torch.zeros((n, 3), device="cuda")
    idx = _t(np.arange(n, dtype=np.int32)[None, :])
    w = _t(np.ones((1, n), np.float32))
    sh_in = np.array([c["sh_in"] for c in cases], np.float32)
    feat = _t(sh_in)
    dev.skin_samples(pos, idx, w, table, quat, feat)
    # expected: reference matrices with the odd-coefficient flip around them
    odd = np.array([1 if k % 2 else 0 for k in range(16)], bool)
    exp = []
    for c, s in zip(cases, sh_in.astype(np.float64)):
        v = s.reshape(16, 3).copy()
        v[odd] *= -1
        v[1:4] = np.array(c["sh1"]) @ v[1:4]
        v[4:9] = np.array(c["sh2"]) @ v[4:9]
        v[9:16] = np.array(c["sh3"]) @ v[9:16]
        v[odd] *= -1
        exp.append(v.reshape(-1))
    assert np.abs(_np(feat) - np.array(exp)).max() <= 2e-5


def test_skin_samples(dev, scene):
    from oracle import skin
    rng = np.random.default_rng(11)
    rot, trans = _random_transforms(scene.n_nodes, rng, amp=0.2)
    S = 20000
    lo, hi = scene.pos.min(0), scene.pos.max(0)
    sp = (lo + rng.random((S, 3)) * (hi - lo)).astype(np.float32)
    feat = (0.3 * rng.standard_normal((S, 48))).astype(np.float32)
    idx, w = dev.compute_weights(_t(sp), _t(scene.node_pos), scene.k)
    table = dev.node_table(_t(rot), _t(trans), _t(scene.node_pos))
    quat = dev.node_quaternions(_t(rot))
    p = _t(sp)
    f = _t(feat)
    dev.skin_samples(p, idx, w, table, quat, f)
    p_ref, f_ref = skin.skin_samples(sp, _np(idx).T, _np(w).T, rot.astype(np.float64),
                                     trans.astype(np.float64), scene.node_pos, feat, float_accumulate=False)
    q_ref = skin.node_quaternions(rot.astype(np.float64))
    dq = np.abs(1 - np.abs((_np(quat).astype(np.float64) * q_ref).sum(1)))
    assert dq.max() <= 2e-6
    ext = float(np.ptp(scene.pos, axis=0).max())
    assert np.abs(_np(p) - p_ref).max() / ext <= 2e-6
    assert np.abs(_np(f) - f_ref).max() <= 5e-5


def test_update_nodes_and_static(dev, scene):
    from oracle import ed
    rng = np.random.default_rng(5)
    rot, trans = _random_transforms(scene.n_nodes, rng)
    aidx, aw = ed.knn_weights(scene.pos[scene.node_vertex], scene.node_pos, scene.k)
    table = dev.node_table(_t(rot), _t(trans), _t(scene.node_pos))
    out = dev.update_nodes(_t(scene.node_pos), _t(aidx.T.astype(np.int32)), _t(aw.T.astype(np.float32)), table)
    ref = ed.ed_blend(scene.node_pos, aidx, aw, rot.astype(np.float64), trans.astype(np.float64), scene.node_pos,
                      float_accumulate=False)
    ext = float(np.ptp(scene.pos, axis=0).max())
    assert np.abs(_np(out) - ref).max() / ext <= 2e-6
    st_nodes = np.zeros(scene.n_nodes, np.uint8)
    for b, t in zip(scene.blocks, scene.block_type):
        if t < 0:
            st_nodes[b] = 1
    from oracle import skin
    m = dev.static_mask(_t(aidx.T.astype(np.int32)), _t(st_nodes), scene.n_nodes)
    assert np.array_equal(_np(m).astype(bool), skin.static_mask(aidx, np.flatnonzero(st_nodes), scene.n_nodes))


def test_aims_ops(dev, scene):
    from oracle import targets
    act = H.active_nodes(scene)
    if act.size == 0:
        pytest.skip("no active block")
    rng = np.random.default_rng(2)
    base = (scene.node_pos + 0.01 * rng.standard_normal(scene.node_pos.shape)).astype(np.float32)
    a = _t(base)
    dev.aims_translate(a, _t(act.astype(np.int32)), (0.1, -0.2, 0.3))
    assert np.abs(_np(a) - targets.translate(base, act, (0.1, -0.2, 0.3))).max() <= 1e-6
    a = _t(base)
    dev.aims_twist(a, _t(scene.node_pos), _t(act.astype(np.int32)), (0.2, 0.3, 1.0), 0.7)
    assert np.abs(_np(a) - targets.twist(base, scene.node_pos, act, (0.2, 0.3, 1.0), 0.7)).max() <= 2e-6
    a = _t(base)
    dev.aims_scale(a, _t(scene.node_pos), _t(act.astype(np.int32)), 1.5)
    assert np.abs(_np(a) - targets.scale(base, scene.node_pos, act, 1.5)).max() <= 2e-6
