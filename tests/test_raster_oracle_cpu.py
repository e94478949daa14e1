"""Rasteriser oracle (oracle/raster.py), on CPU.

- The SH basis: its constant term is the viewer's SH0 (helper.hpp:60), and
  bands 1 and 2 have their closed forms.  Coefficients rotated by the viewer's
  SH rotation (oracle.skin.rotate_sh, pinned to the reference's formulas by
  tests/golden/sh_rotation.json) rotate the colour exactly.
- Splatting: one Gaussian straight ahead gives the analytic image.  Depth
  order, near-plane culling and the transmittance stop hold."""
import math

import numpy as np
import pytest

from oracle import raster as r
from oracle import skin

SH0_VIEWER = 0.28209479   # helper.hpp:60


def _dirs(n, seed=0):
    d = np.random.default_rng(seed).normal(size=(n, 3))
    return d / np.linalg.norm(d, axis=1, keepdims=True)


def test_sh_basis_closed_forms():
    d = _dirs(50)
    B = r.sh_basis(d)
    x, y, z = d.T
    assert abs(B[0, 0] - SH0_VIEWER) < 1e-8
    c1 = math.sqrt(3 / (4 * math.pi))
    np.testing.assert_allclose(B[:, 1:4], np.stack([-c1 * y, c1 * z, -c1 * x], 1), atol=1e-14)
    c2 = 0.5 * math.sqrt(15 / math.pi)
    c20 = 0.25 * math.sqrt(5 / math.pi)
    expect2 = np.stack([c2 * x * y, -c2 * y * z, c20 * (2 * z * z - x * x - y * y), -c2 * x * z,
                        0.5 * c2 * (x * x - y * y)], 1)
    np.testing.assert_allclose(B[:, 4:9], expect2, atol=1e-14)


def test_sh_basis_is_orthonormal():
    # Gauss-Legendre in cos(theta) x uniform phi integrates degree <= 6 exactly
    u, wu = np.polynomial.legendre.leggauss(12)
    phi = np.arange(24) * (2 * math.pi / 24)
    U, PHI = np.meshgrid(u, phi, indexing="ij")
    s = np.sqrt(1 - U * U)
    d = np.stack([s * np.cos(PHI), s * np.sin(PHI), U], -1).reshape(-1, 3)
    w = (wu[:, None] * np.full(phi.size, 2 * math.pi / phi.size)[None]).reshape(-1)
    B = r.sh_basis(d)
    np.testing.assert_allclose(B.T @ (w[:, None] * B), np.eye(16), atol=1e-12)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_rotated_coefficients_rotate_the_colour(seed):
    rng = np.random.default_rng(seed)
    q = rng.normal(size=(1, 4))
    R = skin.quat_to_matrix(skin.quat_normalize(q))[0]
    c = rng.normal(size=(1, 48))
    d = _dirs(20, seed)
    lhs = r.sh_color(np.repeat(skin.rotate_sh(c, R[None]), 20, 0), d)
    rhs = r.sh_color(np.repeat(c, 20, 0), d @ R)        # colour of the unrotated field at R^T d
    np.testing.assert_allclose(lhs, rhs, atol=1e-12)


def _camera(width, height, tan_half=0.5, near=0.01, far=100.0):
    view = np.eye(4)
    proj = np.zeros((4, 4))
    proj[0, 0] = 1 / tan_half
    proj[1, 1] = 1 / tan_half
    proj[2, 2] = far / (far - near)
    proj[2, 3] = -far * near / (far - near)
    proj[3, 2] = 1.0
    return view, proj, np.zeros(3), tan_half, tan_half


def _gaussian(pos, s, opacity, dc):
    shs = np.zeros((1, 48))
    shs[0, 0:3] = dc
    return (np.array([pos], float), shs, np.array([opacity]), np.array([[s, s, s]]),
            np.array([[1.0, 0, 0, 0]]))


def test_one_gaussian_gives_the_analytic_image():
    W = H = 32
    view, proj, cam, tx, ty = _camera(W, H)
    pos, shs, op, sc, rot = _gaussian([0, 0, 5], 0.3, 0.8, [0.4, -0.2, 1.0])
    bg = np.array([0.1, 0.2, 0.3])
    img, T, n = r.render(pos, shs, op, sc, rot, view, proj, cam, tx, ty, W, H, bg)
    f = W / (2 * tx)
    var = (f * 0.3 / 5) ** 2 + 0.3
    col = np.maximum(SH0_VIEWER * np.array([0.4, -0.2, 1.0]) + 0.5, 0)
    ys, xs = np.mgrid[0:H, 0:W]
    c = (W - 1) / 2
    alpha = np.minimum(0.99, 0.8 * np.exp(-0.5 * ((xs - c) ** 2 + (ys - c) ** 2) / var))
    alpha = np.where(alpha < 1 / 255, 0.0, alpha)
    expect = col[:, None, None] * alpha + (1 - alpha) * bg[:, None, None]
    np.testing.assert_allclose(img, expect, atol=1e-7)
    np.testing.assert_allclose(T, 1 - alpha, atol=1e-12)
    assert n.max() == 1 and n.sum() == int((alpha > 0).sum())


def test_depth_order_and_input_order():
    W = H = 16
    view, proj, cam, tx, ty = _camera(W, H)
    a = _gaussian([0, 0, 4], 0.3, 0.7, [1, 0, 0])
    b = _gaussian([0, 0, 6], 0.5, 0.9, [0, 1, 0])
    cat = [np.concatenate([u, v]) for u, v in zip(a, b)]
    rev = [np.concatenate([v, u]) for u, v in zip(a, b)]
    img1, _, _ = r.render(*cat, view, proj, cam, tx, ty, W, H)
    img2, _, _ = r.render(*rev, view, proj, cam, tx, ty, W, H)
    np.testing.assert_array_equal(img1, img2)
    g = r.preprocess(*cat, view, proj, cam, tx, ty, W, H)
    x = y = 8
    al = []
    for i in range(2):
        dx, dy = g["xy"][i, 0] - x, g["xy"][i, 1] - y
        ca, cb, cc = g["conic"][i]
        al.append(min(0.99, g["opacity"][i] * math.exp(-0.5 * (ca * dx * dx + cc * dy * dy) - cb * dx * dy)))
    expect = g["color"][0] * al[0] + g["color"][1] * al[1] * (1 - al[0])
    np.testing.assert_allclose(img1[:, y, x], expect, atol=1e-12)


def test_near_plane_culls():
    W = H = 16
    view, proj, cam, tx, ty = _camera(W, H)
    pos, shs, op, sc, rot = _gaussian([0, 0, 0.15], 0.3, 0.9, [1, 1, 1])
    img, T, n = r.render(pos, shs, op, sc, rot, view, proj, cam, tx, ty, W, H, (0.25, 0.5, 0.75))
    assert n.sum() == 0 and np.all(T == 1)
    np.testing.assert_array_equal(img[:, 3, 5], [0.25, 0.5, 0.75])


def test_compositing_stops_below_the_transmittance_floor():
    W = H = 16
    view, proj, cam, tx, ty = _camera(W, H)
    layers = [_gaussian([0, 0, 3 + i], 2.0, 0.95, [0.5 * i, 0, 0]) for i in range(5)]
    args = [np.concatenate(parts) for parts in zip(*layers)]
    img, T, n = r.render(*args, view, proj, cam, tx, ty, W, H)
    # alpha near 0.95 each: T about 0.05, 0.0025, 1.25e-4; a fourth layer would
    # leave about 6e-6 < 1e-4, so compositing stops after three
    g = r.preprocess(*args, view, proj, cam, tx, ty, W, H)
    c = 8
    al = []
    for i in range(5):
        dx, dy = g["xy"][i, 0] - c, g["xy"][i, 1] - c
        ca, cb, cc = g["conic"][i]
        al.append(min(0.99, g["opacity"][i] * math.exp(-0.5 * (ca * dx * dx + cc * dy * dy) - cb * dx * dy)))
    t3 = (1 - al[0]) * (1 - al[1]) * (1 - al[2])
    assert t3 >= 1e-4 and t3 * (1 - al[3]) < 1e-4
    assert n[c, c] == 3
    assert abs(T[c, c] - t3) < 1e-15
    expect = sum(g["color"][i] * al[i] * np.prod([1 - al[j] for j in range(i)]) for i in range(3))
    np.testing.assert_allclose(img[:, c, c], expect, atol=1e-12)
