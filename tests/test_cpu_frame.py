"""The C++/OpenMP CPU baseline (oracle/cpu_frame.cpp) against the numpy
oracle (oracle/ed.py, oracle/skin.py) on the same inputs, on CPU.

The baseline is the timed CPU leg of the benchmark and the quick float64
reference of the large GPU parity tests, so it has to restate the same
algorithm: the Gauss-Newton solve of Deform.cpp:95-169 (direct sparse solve),
the endpoint refit of GaussianView.cpp:3081-3166 and the sample skinning of
GaussianView.cpp:3060-3186."""
import importlib
import os

import numpy as np
import pytest

import _helpers as H
from oracle import cpu_frame as cf
from oracle import ed, skin

HERE = os.path.dirname(os.path.abspath(__file__))


def _solve_inputs(sc):
    nb = ed.build_graph(sc.node_pos, sc.k)
    aidx, aw = ed.knn_weights(sc.pos[sc.node_vertex], sc.node_pos, sc.k)
    return nb, aidx, aw, H.oracle_aims(sc, sc.node_pos)


def test_knn_weights_match():
    sc = H.synth.make_scene("twist20k")
    pts = sc.pos[:5000]
    i_ref, w_ref = ed.knn_weights(pts, sc.node_pos, sc.k)
    i, w = cf.knn_weights(pts, sc.node_pos, sc.k)
    np.testing.assert_array_equal(i, i_ref)
    assert np.abs(w - w_ref).max() < 1e-14


@pytest.mark.parametrize("name,ordering", [("bend4k", 0), ("twist20k", 1), ("stress40k", 0)])
def test_solve_matches_numpy_oracle(name, ordering):
    sc = H.synth.make_scene(name)
    nb, aidx, aw, aims = _solve_inputs(sc)
    pr = ed.EDProblem(sc.node_pos, nb, aidx, aw, sc.blocks, sc.block_type, aims)
    x_ref, st_ref = ed.gauss_newton(pr, max_iters=sc.iters, early_exit=False)
    rot_ref, tr_ref = ed.put_free_inputs(pr, x_ref)
    rot, tr, st = cf.solve(sc.node_pos, nb, aidx, aw, sc.blocks, sc.block_type, aims, max_iters=sc.iters,
                           ordering=ordering)
    assert st["status"] == 0 and st["gn_iterations"] == sc.iters and st["n_rows"] == pr.n_rows
    assert H.rel_err(np.concatenate([rot, tr], 1), np.concatenate([rot_ref, tr_ref], 1)) < 1e-12
    assert abs(st["initial_energy"] - st_ref.energies[0]) <= 1e-12 * st_ref.energies[0]
    assert st["halvings"] == sum(st_ref.halvings)


@pytest.mark.parametrize("cons,wf", [(1, 1.0), (0, 3.0)])
def test_solve_centre_mode_and_weighting(cons, wf):
    sc = H.synth.make_scene("bend4k")
    nb, aidx, aw, aims = _solve_inputs(sc)
    p = sc.node_pos
    blocks = [np.flatnonzero((p[:, 0] < 0.1) & (p[:, 1] < 0.1)), np.flatnonzero((p[:, 0] < 0.1) & (p[:, 1] >= 0.1)),
              np.flatnonzero(p[:, 0] > 0.9)]
    types = [0, 0, 1]
    pr = ed.EDProblem(sc.node_pos, nb, aidx, aw, blocks, types, aims, cons_on_center=bool(cons),
                      weighting_factor=wf)
    x_ref, _ = ed.gauss_newton(pr, max_iters=5, early_exit=False)
    rot_ref, tr_ref = ed.put_free_inputs(pr, x_ref)
    rot, tr, st = cf.solve(sc.node_pos, nb, aidx, aw, blocks, types, aims, cons_on_center=cons,
                           weighting_factor=wf, max_iters=5)
    assert st["n_rows"] == pr.n_rows
    assert H.rel_err(np.concatenate([rot, tr], 1), np.concatenate([rot_ref, tr_ref], 1)) < 1e-10


def test_early_exit_matches():
    sc = H.synth.make_scene("bend4k")
    nb, aidx, aw, aims = _solve_inputs(sc)
    pr = ed.EDProblem(sc.node_pos, nb, aidx, aw, sc.blocks, sc.block_type, aims)
    _, st_ref = ed.gauss_newton(pr, max_iters=30, early_exit=True)
    _, _, st = cf.solve(sc.node_pos, nb, aidx, aw, sc.blocks, sc.block_type, aims, max_iters=30, early_exit=True)
    assert st["gn_iterations"] == st_ref.iterations


def test_skinning_is_bit_identical_to_the_numpy_oracle():
    sc = H.synth.make_scene("twist20k")
    nb, aidx, aw, aims = _solve_inputs(sc)
    pr = ed.EDProblem(sc.node_pos, nb, aidx, aw, sc.blocks, sc.block_type, aims)
    x, _ = ed.gauss_newton(pr, max_iters=3, early_exit=False)
    rot, tr = ed.put_free_inputs(pr, x)
    m = 4000
    E = skin.end_points(sc.pos[:m], sc.rot[:m], sc.scale[:m])
    idx, w = ed.knn_weights(E.reshape(-1, 3), sc.node_pos, sc.k)
    w32 = w.astype(np.float32)
    e_ref, p_ref, q_ref, s_ref, sh_ref = skin.skin_gaussians(E, idx, w32.astype(np.float64), rot, tr, sc.node_pos,
                                                             sc.rot[:m], sc.scale[:m], sc.shs[:m])
    rng = np.random.default_rng(1)
    sp = (sc.pos[rng.integers(0, sc.n_gauss, 3000)] + 0.002 * rng.standard_normal((3000, 3))).astype(np.float32)
    si, sw = ed.knn_weights(sp, sc.node_pos, sc.k)
    feat = (0.2 * rng.standard_normal((3000, 48))).astype(np.float32)
    ps_ref, f_ref = skin.skin_samples(sp, si, sw.astype(np.float32), rot, tr, sc.node_pos, feat)
    fr = cf.Frame(E, idx, w32, sc.node_pos, sc.rot[:m], sc.scale[:m], sc.shs[:m], sample_pos=sp, sample_idx=si,
                  sample_w=sw.astype(np.float32), feature=feat)
    fr.skin_gaussians(rot, tr)
    fr.skin_samples(rot, tr)
    np.testing.assert_array_equal(fr.ends, e_ref)
    np.testing.assert_array_equal(fr.pos, p_ref)
    # R, K and the quaternion come from a different SVD algorithm than
    # numpy's LAPACK: equal up to the last float32 bit
    assert np.abs(fr.q - q_ref).max() <= 2e-7
    assert np.abs(fr.scale - s_ref).max() <= 2e-7 * np.abs(s_ref).max()
    assert np.abs(fr.shs - sh_ref).max() <= 2e-6
    cov_ref = skin.covariance6(q_ref, s_ref)
    assert np.abs(fr.cov6 - cov_ref).max() <= 1e-6 * np.abs(cov_ref).max()
    np.testing.assert_array_equal(fr.sample_pos, ps_ref)
    assert np.abs(fr.feature - f_ref).max() <= 2e-6
    nodes = cf.ed_blend(sc.node_pos, aidx, aw, rot, tr, sc.node_pos)
    np.testing.assert_array_equal(nodes, ed.ed_blend(sc.node_pos, aidx, aw, rot, tr, sc.node_pos))


def test_occupied_cells_match_the_oracle_csr():
    from oracle import grid as og
    sc = H.synth.make_scene("bend4k")
    valid, samples = cf.occupied_cell_samples(sc.pos, sc.rot, sc.scale, sc.opacity, sc.grid_num)
    mn, mx = og.overall_aabb(sc.pos)
    step = og.grid_step(mn, mx, sc.grid_num)
    lo, hi = og.gaussian_aabbs(sc.pos, sc.rot, sc.scale, sc.opacity)
    off, _ = og.cell_csr(lo, hi, mn, step, sc.grid_num)
    v_ref, s_ref = og.grid_samples(off, mn, step, sc.grid_num)
    np.testing.assert_array_equal(valid, v_ref)
    np.testing.assert_array_equal(samples, s_ref)


@pytest.mark.parametrize("name", ["bend50k", "twist300k"])
def test_solve_matches_the_committed_oracle_solve(name):
    """The baseline at the benchmark's sizes against the numpy oracle's
    solve of the same scene (tests/golden/make_solve_golden.py)."""
    g = np.load(os.path.join(HERE, "golden", "solve_%s.npz" % name))
    sc = H.synth.make_scene(name)
    nb, _, _, aims = (ed.build_graph(sc.node_pos, sc.k), None, None, H.oracle_aims(sc, sc.node_pos))
    aidx, aw = cf.knn_weights(sc.pos[sc.node_vertex], sc.node_pos, sc.k)
    rot, tr, st = cf.solve(sc.node_pos, nb, aidx, aw, sc.blocks, sc.block_type, aims, max_iters=int(g["iters"]))
    X = np.concatenate([rot, tr], 1)
    assert H.rel_err(X, g["x"].astype(np.float64)) < 1e-6   # the fixture is float32
    assert abs(st["initial_energy"] - g["energies"][0]) <= 1e-12 * g["energies"][0]
    assert abs(st["final_energy"] - float(g["final"])) <= 1e-9 * float(g["final"])
    assert st["halvings"] == int(g["halvings"].sum())
