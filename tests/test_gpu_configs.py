"""Parity at the benchmark's own configurations: a whole deformation frame
on the GPU against the float64 oracle.

* bend50k (50k Gaussians, 32^3 grid, ~1k nodes, k=8, 10 iterations) and
  twist300k (300k Gaussians, 64^3 grid, 4061 nodes, k=8, 20 iterations, the
  benchmarked frame), each in the chosen form (mixed precision, two-level
  PCG with 64-node aggregates), the plain form (FP32, block-Jacobi) and
  FP32 with the two-level PCG (plain2l); the chosen form also with a fresh
  coarse inverse in every Gauss-Newton iteration (chosen_fresh; the default
  keeps the previous inverse while the steps are small, which changes the
  preconditioner only).
* Node transforms against the numpy oracle's Gauss-Newton solve of the same
  scene (tests/golden/solve_<scene>.npz, made by
  tests/golden/make_solve_golden.py; exact sparse solve, Deform.cpp:95-169).
  Tolerance: max |dx| / max |x| <= 1e-5 (chosen), 5e-5 (FP32 forms).  The
  line search's halvings (Deform.cpp:144-156) must agree in every
  Gauss-Newton iteration.
* The frame's outputs (sample positions and features, Gaussian mean,
  quaternion, scale, covariance and SH, node update) against the C++
  restatement of the reference's CPU frame (oracle/cpu_frame.cpp, itself
  checked bit for bit against the numpy oracle in tests/test_cpu_frame.py)
  run on the oracle's node transforms, from the same rest state and kNN
  weights.  Tolerances:
    mu, sample and node positions   max |d| / scene extent <= 1e-5
    covariance                      max |dSigma| / max |Sigma| <= 1e-5
    quaternion                      1 - |<q, q_ref>| <= 1e-5
    SH and sample features          max abs <= 2e-4 (coefficients ~N(0, 0.2))
"""
import os

import numpy as np
import pytest

from tests import _helpers as H

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _np(t):
    return t.detach().cpu().numpy()


def _rel(a, b):
    return float(np.abs(np.asarray(a, np.float64) - b).max() / np.abs(b).max())


@pytest.fixture(scope="module", params=["bend50k", "twist300k"])
def case(request):
    from oracle import cpu_frame as cf
    sc = H.synth.make_scene(request.param)
    _, samples = cf.occupied_cell_samples(sc.pos, sc.rot, sc.scale, sc.opacity, sc.grid_num)
    rng = np.random.default_rng(5)
    feature = (0.2 * rng.standard_normal((samples.shape[0], 48))).astype(np.float32)
    g = np.load(os.path.join(GOLDEN, "solve_%s.npz" % sc.name))
    return sc, samples, feature, g


def _oracle_frame(d, sc, samples, feature, X):
    """The C++ float64 restatement of the frame on the deformer's rest state,
    kNN weights and the given node transforms X [n,12]."""
    from oracle import cpu_frame as cf
    N, k = d.N, d.k
    ends = _np(d.ends).reshape(6, 3, N).transpose(2, 0, 1)
    eidx = _np(d.ends_idx).reshape(k, 6, N).transpose(2, 1, 0)
    ew = _np(d.ends_w).reshape(k, 6, N).transpose(2, 1, 0)
    fr = cf.Frame(ends, eidx, ew, sc.node_pos, sc.rot, sc.scale, sc.shs, sample_pos=samples,
                  sample_idx=_np(d.sample_idx).T, sample_w=_np(d.sample_w).T, feature=feature)
    rot, tr = X[:, :9].astype(np.float64), X[:, 9:].astype(np.float64)
    fr.skin_samples(rot, tr)
    fr.skin_gaussians(rot, tr)
    nodes = cf.ed_blend(sc.node_pos, _np(d.anchor_idx).T, _np(d.anchor_w).T, rot, tr, sc.node_pos)
    return fr, nodes


_FORMS = {"chosen": (1, 64, 0.0), "chosen_fresh": (1, 64, -1.0), "plain": (0, 0, 0.0), "plain2l": (0, 64, 0.0)}


@pytest.mark.parametrize("form", ["chosen", "chosen_fresh", "plain", "plain2l"])
def test_frame_matches_the_oracle(dev, case, form):
    sc, samples, feature, g = case
    precision, coarse, reuse = _FORMS[form]
    cfg = dev.default_config(max_iters=sc.iters, early_exit=0, precision=precision, coarse_nodes=coarse,
                             coarse_reuse=reuse)
    d = dev.GaussianDeformer(torch.as_tensor(sc.pos), torch.as_tensor(sc.rot), torch.as_tensor(sc.scale),
                             torch.as_tensor(sc.shs), sc.node_vertex, sc.k, sc.blocks, sc.block_type,
                             sample_pos=torch.as_tensor(samples), feature=torch.as_tensor(feature), config=cfg)
    d.apply_op(sc.op)
    fr, nodes_ref = _oracle_frame(d, sc, samples, feature, g["x"])
    st = d.frame(stats=True, with_cov=True)
    torch.cuda.synchronize()
    assert st["status"] == 0 and d.status() == 0
    assert st["gn_iterations"] == int(g["iters"])
    X = np.concatenate([_np(d.rot_nodes), _np(d.trans_nodes)], 1)
    err_x = _rel(X, g["x"].astype(np.float64))
    ext = float(np.ptp(sc.pos, axis=0).max())
    err = {
        "x": err_x,
        "mu": float(np.abs(_np(d.pos) - fr.pos).max() / ext),
        "sigma": _rel(_np(d.cov), fr.cov6.astype(np.float64)),
        "q": float(np.abs(1 - np.abs((_np(d.rot).astype(np.float64) * fr.q).sum(1))).max()),
        "scale": _rel(_np(d.scale), fr.scale.astype(np.float64)),
        "shs": float(np.abs(_np(d.shs) - fr.shs).max()),
        "sample_pos": float(np.abs(_np(d.sample_pos) - fr.sample_pos).max() / ext),
        "feature": float(np.abs(_np(d.feature) - fr.feature).max()),
        "nodes": float(np.abs(_np(d.node_pos) - nodes_ref).max() / ext),
    }
    print("%s %s: pcg %d, coarse inversions %d, halvings %d (oracle %d), errors %s" % (
        sc.name, form, st["pcg_iterations"], st["coarse_inversions"], st["halvings"], int(g["halvings"].sum()),
        {k: "%.2e" % v for k, v in err.items()}))
    if coarse == 0:
        assert st["coarse_inversions"] == 0
    elif reuse < 0:
        assert st["coarse_inversions"] == st["gn_iterations"]
    else:
        assert 1 <= st["coarse_inversions"] <= st["gn_iterations"]
    if form != "plain2l":
        # the line search takes the oracle's branch in every Gauss-Newton
        # iteration.  Not so for FP32 residuals with the two-level PCG: at
        # bend50k its FP32 energy test halves one step that the float64
        # energy accepts (x error 1.2e-5), one reason the chosen form keeps
        # the residual, gradient and energy in FP64
        assert st["halvings"] == int(g["halvings"].sum())
        assert st["iteration_halvings"] == [int(v) for v in g["halvings"]]
    assert abs(st["initial_energy"] - g["energies"][0]) <= 1e-5 * g["energies"][0]
    chosen = precision == 1
    assert err_x <= (1e-5 if chosen else 5e-5)
    tol = 1e-5 if chosen else 5e-5
    assert err["mu"] <= tol and err["sample_pos"] <= tol and err["nodes"] <= tol
    assert err["sigma"] <= tol and err["q"] <= tol and err["scale"] <= tol
    assert err["shs"] <= 2e-4 and err["feature"] <= 2e-4


@pytest.mark.parametrize("form", ["chosen", "plain"])
def test_non_resident_solve_matches_the_oracle(dev, form):
    """stress200k: 7583 free nodes of 8044 (an excluded block), k = 12, more
    than the solver keeps resident in shared memory, so the chosen form runs
    the non-resident two-level PCG.  Node transforms against the float64
    C++ restatement's solve (tests/golden/solve_stress200k.npz)."""
    from oracle import cpu_frame as cf
    from oracle import ed
    sc = H.synth.make_scene("stress200k")
    g = np.load(os.path.join(GOLDEN, "solve_stress200k.npz"))
    nb = ed.build_graph(sc.node_pos, sc.k)
    aidx, aw = cf.knn_weights(sc.pos[sc.node_vertex], sc.node_pos, sc.k)
    aims = H.oracle_aims(sc, sc.node_pos)
    precision, coarse = (1, 64) if form == "chosen" else (0, 0)
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a)).cuda()  # noqa: E731
    solver = dev.Solver(t(nb.astype(np.int32)), t(aidx.T.astype(np.int32)), t(aw.T.astype(np.float32)),
                        sc.blocks, sc.block_type, max_iters=sc.iters, early_exit=0, precision=precision,
                        coarse_nodes=coarse)
    rot, tr, st = solver.solve(t(sc.node_pos), t(aims))
    assert st["status"] == 0 and st["gn_iterations"] == sc.iters
    assert st["n_free"] == 7583 and st["resident"] == 0
    X = np.concatenate([_np(rot), _np(tr)], 1)
    err = _rel(X, g["x"].astype(np.float64))
    print("stress200k %s: pcg %d, coarse %d, halvings %d (oracle %d), x error %.2e"
          % (form, st["pcg_iterations"], st["n_coarse"], st["halvings"], int(g["halvings"].sum()), err))
    assert st["halvings"] == int(g["halvings"].sum())  # the fixture keeps the total only
    assert abs(st["initial_energy"] - g["energies"][0]) <= 1e-5 * g["energies"][0]
    assert err <= (1e-5 if form == "chosen" else 5e-5)
    solver.close()
