"""Headless rasteriser (arap_render) against the oracle (oracle/raster.py)."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _camera(tan_half=0.5, near=0.01, far=100.0):
    view = np.eye(4)
    view[:3, 3] = [0.0, 0.0, 3.0]           # the scene sits in front of the camera
    proj = np.zeros((4, 4))
    proj[0, 0] = proj[1, 1] = 1 / tan_half
    proj[2, 2] = far / (far - near)
    proj[2, 3] = -far * near / (far - near)
    proj[3, 2] = 1.0
    return view, proj @ view, np.array([0.0, 0.0, -3.0]), tan_half, tan_half


def test_render_matches_the_oracle():
    import torch
    from oracle import raster as r
    rnd = importlib.import_module("arap-deformation-of-gaussian-radiance-fields_gb300.render")
    rng = np.random.default_rng(0)
    N, W, H = 200, 48, 40
    pos = rng.uniform(-1, 1, (N, 3)).astype(np.float32)
    shs = rng.normal(0, 0.3, (N, 48)).astype(np.float32)
    op = rng.uniform(0.2, 0.95, N).astype(np.float32)
    sc = np.exp(rng.normal(-2.5, 0.3, (N, 3))).astype(np.float32)
    q = rng.normal(size=(N, 4))
    rot = (q / np.linalg.norm(q, axis=1, keepdims=True)).astype(np.float32)
    view, proj, cam, tx, ty = _camera()
    bg = (0.1, 0.2, 0.3)
    img, T, n = rnd.render(*(torch.from_numpy(a).cuda() for a in (pos, shs, op, sc, rot)), view, proj, cam, tx, ty,
                           W, H, bg)
    ref, rT, rn = r.render(pos, shs, op, sc, rot, view, proj, cam, tx, ty, W, H, bg)
    got = img.cpu().numpy()
    # float32 against float64: a term at the 1/255 or 1e-4 thresholds can flip,
    # so compare the bulk tightly and bound the rest
    err = np.abs(got - ref)
    assert np.quantile(err, 0.99) < 1e-4
    assert err.max() < 2e-2
    assert np.mean(n.cpu().numpy() == rn) > 0.99
