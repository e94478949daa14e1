"""CPU checks of the oracle (pinned to the reference's formulas where the
reference gives something to pin to) and of the C-ABI library's exports."""
import ctypes
import json
import os
import re

import numpy as np
import pytest

from tests import _helpers as H

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def test_sh_rotation_matches_reference_formulas():
    from oracle import skin
    g = json.load(open(os.path.join(GOLDEN, "sh_rotation.json")))
    for c in g["cases"]:
        m1, m2, m3 = skin.sh_rotation_matrices(np.array(c["R"])[None])
        assert np.abs(m1[0] - np.array(c["sh1"])).max() < 1e-12
        assert np.abs(m2[0] - np.array(c["sh2"])).max() < 1e-12
        assert np.abs(m3[0] - np.array(c["sh3"])).max() < 1e-12
        out = skin.rotate_sh(np.array(c["sh_in"])[None], np.array(c["R"])[None], flip_odd=False)
        assert np.abs(out[0] - np.array(c["sh_out"])).max() < 1e-12


def test_sh_kat_test_sh_rotation():
    # helper.cpp:924-936 input through the oracle equals the reference formulas' output
    from oracle import skin
    kat = json.load(open(os.path.join(GOLDEN, "sh_rotation.json")))["kat_test_sh_rotation"]
    R = skin.quat_to_matrix(skin.quat_normalize(np.array(kat["quat_wxyz"])))
    out = skin.rotate_sh(np.array(kat["sh_in"])[None], R[None], flip_odd=False)
    assert np.abs(out[0] - np.array(kat["sh_out"])).max() < 1e-9
    assert np.abs(R - np.array(kat["R"])).max() < 1e-12


def test_sh_rotation_is_a_representation():
    from oracle import skin
    rng = np.random.default_rng(0)
    A = skin.quat_to_matrix(skin.quat_normalize(rng.standard_normal((8, 4))))
    B = skin.quat_to_matrix(skin.quat_normalize(rng.standard_normal((8, 4))))
    x = rng.standard_normal((8, 48))
    lhs = skin.rotate_sh(skin.rotate_sh(x, B), A)
    rhs = skin.rotate_sh(x, A @ B)
    assert np.abs(lhs - rhs).max() < 1e-12


def test_jacobian_matches_finite_differences():
    from oracle import ed
    sc = H.synth.make_scene("bend4k")
    nb = ed.build_graph(sc.node_pos, sc.k)
    aidx, aw = ed.knn_weights(sc.pos[sc.node_vertex], sc.node_pos, sc.k)
    aims = H.oracle_aims(sc, sc.node_pos)
    for centre in (False, True):
        pr = ed.EDProblem(sc.node_pos, nb, aidx, aw, sc.blocks, sc.block_type, aims, cons_on_center=centre)
        rng = np.random.default_rng(1)
        x = ed.identity_x(pr.F) + 0.01 * rng.standard_normal(pr.F * 12)
        v = rng.standard_normal(x.size)
        J = ed.jacobian(pr, x)
        eps = 1e-6
        fd = (ed.residual(pr, x + eps * v) - ed.residual(pr, x - eps * v)) / (2 * eps)
        # the reference's Jacobian uses float32 node differences: agreement to ~1e-7
        assert np.abs(J @ v - fd).max() <= 2e-6 * np.abs(fd).max()
        assert J.shape == (pr.n_rows, pr.n_cols)


def test_weight_scale_quirk_on_t_columns():
    # Deform.cpp:257 writes cur_weight (no weight_scale) on the t_i columns
    from oracle import ed
    sc = H.synth.make_scene("bend4k")
    nb = ed.build_graph(sc.node_pos, sc.k)
    aidx, aw = ed.knn_weights(sc.pos[sc.node_vertex], sc.node_pos, sc.k)
    pr = ed.EDProblem(sc.node_pos, nb, aidx, aw, sc.blocks, sc.block_type, sc.node_pos, weighting_factor=4.0)
    J = ed.jacobian(pr, ed.identity_x(pr.F)).tocsr()
    r = np.flatnonzero(pr.reg_scale.ravel() == 4.0)
    assert r.size > 0
    row = 6 * pr.F + 3 * r[0]
    fi = r[0] // pr.k
    assert np.isclose(J[row, 12 * fi + 9], np.sqrt(10.0))


def test_knn_ties_and_order():
    from oracle import ed
    nodes = np.array([[1, 0, 0], [0, 1, 0], [-1, 0, 0], [0, -1, 0], [0, 0, 3]], np.float32)
    idx, d = ed.knn(np.zeros((1, 3), np.float32), nodes, 4)
    assert list(idx[0]) == [0, 1, 2, 3]
    idx, w = ed.knn_weights(np.array([[0.1, 0, 0]], np.float32), nodes, 2)
    assert np.isclose(w.sum(), 1.0)


def test_refit_identity_reproduces_gaussians():
    from oracle import skin
    sc = H.synth.make_scene("bend4k")
    E = skin.end_points(sc.pos, sc.rot, sc.scale)
    pos, q, s, sh = skin.refit_gaussians(E, sc.rot, sc.scale, sc.shs)
    assert np.abs(pos - sc.pos).max() < 1e-6
    assert np.abs(np.abs((q.astype(np.float64) * sc.rot).sum(1)) - 1).max() < 1e-6
    assert (np.abs(s - sc.scale) / sc.scale).max() < 1e-4
    assert np.abs(sh - sc.shs).max() < 1e-4


def test_gauss_newton_decreases_energy():
    from oracle import ed
    sc = H.synth.make_scene("bend4k")
    nb = ed.build_graph(sc.node_pos, sc.k)
    aidx, aw = ed.knn_weights(sc.pos[sc.node_vertex], sc.node_pos, sc.k)
    aims = H.oracle_aims(sc, sc.node_pos)
    pr = ed.EDProblem(sc.node_pos, nb, aidx, aw, sc.blocks, sc.block_type, aims)
    x, st = ed.gauss_newton(pr, max_iters=6, early_exit=False)
    assert st.final_energy < 0.01 * st.energies[0]
    assert all(b <= a * (1 + 1e-12) for a, b in zip(st.energies, st.energies[1:]))


def test_point_rotate_by_axis():
    from oracle import targets
    p = targets.point_rotate_by_axis(np.array([2, 0, 0], np.float32), np.array([1, 0, 0], np.float32),
                                     (0, 0, 1), np.pi / 2)
    assert np.allclose(p, [1, 1, 0], atol=1e-6)


def _declared_functions():
    src = open(os.path.join(ROOT, "include", "arap_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(arap_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(pkg):
    from importlib import import_module
    build = import_module("arap-deformation-of-gaussian-radiance-fields_gb300.build")
    lib_path = build.build()
    lib = ctypes.CDLL(lib_path)
    names = _declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    lib.arap_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.arap_version()


def test_binding_covers_header(pkg):
    from importlib import import_module
    _lib = import_module("arap-deformation-of-gaussian-radiance-fields_gb300._lib")
    assert sorted(_lib.SIGNATURES) == _declared_functions()
