"""The stripes fixture (tests/golden/stripes_scripts.npz, the reference's
own graph.obj and deform scripts; tests/golden/make_stripes_golden.py)
against the oracle's restatements, on CPU.

The scripts name their blocks by node index in the farthest-point order of
the mesh vertices (helper.cpp:139-195), so that order is pinned by the
reference's own data: under it, each script's blocks are whole end faces of
the bar (16 nodes at y = +1.5 and 16 at y = -1.5; for script 6, 64 nodes at
x = +0.3 and 64 at x = -0.3), which no other order of the 200 vertices
would give by chance."""
import os

import numpy as np

from oracle import targets

HERE = os.path.dirname(os.path.abspath(__file__))
G = np.load(os.path.join(HERE, "golden", "stripes_scripts.npz"))


def test_farthest_point_order_matches_the_fixture():
    order = targets.farthest_point_order(G["vertices"])
    np.testing.assert_array_equal(order, G["order"])
    assert sorted(order.tolist()) == list(range(200))


def test_script_blocks_are_end_faces():
    nodes = G["vertices"][G["order"]]
    for s in range(7):
        b1, b2 = nodes[G["s%d_block1" % s]], nodes[G["s%d_block2" % s]]
        axis, v1, v2 = (0, 0.3, -0.3) if s == 6 else (1, 1.5, -1.5)
        assert np.abs(b1[:, axis] - v1).max() < 1e-5, s
        assert np.abs(b2[:, axis] - v2).max() < 1e-5, s


def test_script_aims_known_answers():
    nodes = G["vertices"][G["order"]]
    # script 0 ends half a turn about z through (0, -1.5, 0), shifted by
    # (-k/pi, 3 pi^2/k^2 * (k/pi)^2, 0) = (-5.4/pi, 3, 0): (x, y, z) -> (-x - 5.4/pi, -3 - y + 3, z)
    start = nodes[G["s0_block2"]]
    a = targets.stripes_script_aims(0, start)
    exp = np.stack([-start[:, 0] - 5.4 / targets.PI, -start[:, 1], start[:, 2]], 1)
    assert np.abs(a[-1] - exp).max() < 1e-5
    np.testing.assert_array_equal(a, G["s0_aims"])
    # script 6 pulls its block along -x by 0.01 per step
    start = nodes[G["s6_block2"]]
    a = targets.stripes_script_aims(6, start)
    assert np.abs(a[-1] - (start - [0.5, 0, 0])).max() < 1e-6
    for s in range(7):
        moved = G["s%d_block%d" % (s, targets.STRIPES_SCRIPTS[s]["moved"])]
        np.testing.assert_array_equal(targets.stripes_script_aims(s, nodes[moved]), G["s%d_aims" % s])
