"""Known answers for the grid oracle (oracle/grid.py), on CPU.

Each expected value is worked out here from the reference's own statements:
- getOverallAABB, GaussianView.cpp:3601-3631;
- the Gaussian boxes, GaussianView.cpp:3961-4019;
- GetBoxesGsGrid's cell ranges, cudakdtree.cu:425-451;
- the cell samples, GaussianView.cpp:4104-4133;
- GetAdaLpfRatio, GaussianView.cpp:4670-4751.
The GPU grid kernels are compared with this oracle in tests/test_gpu_grid.py,
so these pins carry over to them."""
import numpy as np

from oracle import grid as og

F32 = np.float32


def test_overall_aabb_known_answers():
    # [0,1]^3: mean 0.5, min -0.05 (then clamped to -0.75), max
    # (0.55 + 0.5 + 0.05) * (1 + 1/128) - 0.05, computed from the unclamped min
    mn, mx = og.overall_aabb(np.array([[0, 0, 0], [1, 1, 1], [0.3, 0.9, 0.1]], F32))
    np.testing.assert_allclose(mn, [-0.75] * 3, rtol=1e-6)
    np.testing.assert_allclose(mx, [1.1 * (1 + 1 / 128) - 0.05] * 3, rtol=1e-6)
    # [0,4]^3: min -0.2 -> -0.75; max 4.4 * (1 + 1/128) - 0.2
    mn, mx = og.overall_aabb(np.array([[0, 0, 0], [4, 4, 4]], F32))
    np.testing.assert_allclose(mn, [-0.75] * 3, rtol=1e-6)
    np.testing.assert_allclose(mx, [4.4 * (1 + 1 / 128) - 0.2] * 3, rtol=1e-6)
    # a small scene: the +-0.75 floor sets both ends
    mn, mx = og.overall_aabb(np.array([[-0.1, 0, 0.05], [0.1, 0.2, 0.1]], F32))
    np.testing.assert_array_equal(mx, [0.75] * 3)
    np.testing.assert_array_equal(mn, [-0.75] * 3)
    # [-10,10] on x only: min -11, max 22 * (1 + 1/128) - 11
    mn, mx = og.overall_aabb(np.array([[-10, 0, 0], [10, 0, 0]], F32))
    np.testing.assert_allclose(mn[0], -11, rtol=1e-6)
    np.testing.assert_allclose(mx[0], 22 * (1 + 1 / 128) - 11, rtol=1e-6)
    assert og.grid_step(np.array([-1, -2, -3], F32), np.array([1, 2, 5], F32), 4) == F32(2)


def test_gaussian_boxes_known_answers():
    a = 0.5
    f = np.sqrt(-2 * np.log((1 / 255) / a))
    pos = np.array([[1, 2, 3], [0, 0, 0], [5, 5, 5]], F32)
    c = np.cos(np.pi / 4)
    rot = np.array([[1, 0, 0, 0],
                    [c, 0, 0, c],          # 90 degrees about z: x -> y, y -> -x
                    [1, 0, 0, 0]], F32)
    scale = np.array([[0.1, 0.2, 0.3], [0.1, 0.2, 0.3], [1, 1, 1]], F32)
    opacity = np.array([a, a, 1 / 255], F32)
    lo, hi = og.gaussian_aabbs(pos, rot, scale, opacity)
    np.testing.assert_allclose(hi[0] - pos[0], f * np.array([0.1, 0.2, 0.3]), rtol=1e-5)
    np.testing.assert_allclose(pos[0] - lo[0], f * np.array([0.1, 0.2, 0.3]), rtol=1e-5)
    np.testing.assert_allclose(hi[1], f * np.array([0.2, 0.1, 0.3]), rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(lo[1], -f * np.array([0.2, 0.1, 0.3]), rtol=1e-5, atol=1e-6)
    # opacity at the cut-off: the box is the centre alone
    np.testing.assert_array_equal(lo[2], pos[2])
    np.testing.assert_array_equal(hi[2], pos[2])


def test_cell_lists_known_answer():
    g = 4
    mn = np.zeros(3, F32)
    lo = np.array([[0.2, 0.2, 0.2], [2.5, 2.5, 2.5]], F32)
    hi = np.array([[0.4, 0.4, 0.4], [2.6, 2.6, 2.6]], F32)
    off, lists = og.cell_csr(lo, hi, mn, F32(1), g, padding=1)
    counts = np.diff(off)
    # Gaussian 0: cells 0..1 on every axis (cell 0 padded, clamped at 0); Gaussian 1: cells 1..3
    assert counts.sum() == 8 + 27
    cell = lambda x, y, z: x * g * g + y * g + z  # noqa: E731
    assert list(lists[off[cell(1, 1, 1)]:off[cell(1, 1, 1) + 1]]) == [0, 1]
    assert list(lists[off[cell(0, 0, 0)]:off[cell(0, 0, 0) + 1]]) == [0]
    assert list(lists[off[cell(3, 3, 3)]:off[cell(3, 3, 3) + 1]]) == [1]
    assert counts[cell(2, 0, 0)] == 0
    off0, lists0 = og.cell_csr(lo, hi, mn, F32(1), g, padding=0)
    assert np.diff(off0).sum() == 2 and list(lists0) == [0, 1]
    assert np.flatnonzero(np.diff(off0)).tolist() == [cell(0, 0, 0), cell(2, 2, 2)]


def test_cell_samples_known_answer():
    g = 4
    mn = np.array([-1, -1, -1], F32)
    step = F32(0.5)
    off = np.zeros(g ** 3 + 1, np.int64)
    c = 1 * g * g + 2 * g + 3
    off[c + 1:] = 1
    valid, s = og.grid_samples(off, mn, step, g)
    assert valid.tolist() == [c] and s.shape == (64, 3)
    h = 0.125
    base = np.array([-1 + 1 * 0.5, -1 + 2 * 0.5, -1 + 3 * 0.5]) + h / 2
    np.testing.assert_allclose(s[0], base, rtol=1e-6)
    np.testing.assert_allclose(s[1], base + [0, 0, h], rtol=1e-6)      # z runs fastest
    np.testing.assert_allclose(s[4], base + [0, h, 0], rtol=1e-6)
    np.testing.assert_allclose(s[16], base + [h, 0, 0], rtol=1e-6)
    np.testing.assert_allclose(s[63], base + 3 * h, rtol=1e-6)


def test_adaptive_filter_known_answers():
    h = 0.125
    lattice = np.array([[i, j, k] for i in range(4) for j in range(4) for k in range(4)], np.float64) * h
    # an undeformed cell: M = h I, so the filter is 0.2 h^2 I
    got = og.ada_lpf(lattice.astype(F32)[None], lpf=0.2)[0]
    np.testing.assert_allclose(got, 0.2 * h * h * np.eye(3), rtol=1e-5, atol=1e-12)
    # a cell moved by x -> A x + b: M = h A, so the filter is 0.2 h^2 A A^T
    A = np.array([[1.2, 0.3, 0], [-0.1, 0.8, 0.2], [0.05, 0, 1.5]])
    moved = lattice @ A.T + [3, -2, 1]
    got = og.ada_lpf(moved.astype(F32)[None], lpf=0.2)[0]
    np.testing.assert_allclose(got, 0.2 * h * h * A @ A.T, rtol=1e-4, atol=1e-9)


def test_centre_cells_are_a_stable_order():
    pos = np.array([[0.5, 0.5, 0.5], [0.1, 0.1, 0.1], [0.6, 0.6, 0.6], [0.15, 0.1, 0.1]], F32)
    cell, new_index = og.center_cells(pos, np.zeros(3, F32), F32(0.5), 2)
    assert cell.tolist() == [7, 0, 7, 0]
    assert new_index.tolist() == [2, 0, 3, 1]


def test_density_of_one_gaussian():
    # sigma(x) = a exp(-|x - mu|^2 / (2 (s^2 + l))) for an isotropic Gaussian
    # and the isotropic filter l; the feature is sigma times the SH vector
    s, a, lpf = 0.1, 0.7, 0.01
    samples = np.array([[0, 0, 0], [0.1, 0, 0], [0.05, -0.2, 0.1]], F32)
    off = np.array([0, 1], np.int64)
    lists = np.array([0], np.int32)
    shs = np.arange(48, dtype=F32)[None]
    sig, feat = og.density(samples, off, lists, np.zeros(3, np.int64), np.zeros((1, 3), F32),
                           np.array([[1, 0, 0, 0]], F32), np.full((1, 3), s, F32), np.array([a], F32),
                           shs, np.float64(lpf))
    d2 = (samples.astype(np.float64) ** 2).sum(axis=1)
    expect = a * np.exp(-0.5 * d2 / (s * s + lpf))
    np.testing.assert_allclose(sig, expect, rtol=1e-6)
    np.testing.assert_allclose(feat, expect[:, None] * np.arange(48), rtol=1e-6)
