"""The allocation-free centre order (arap_grid_center_order_noalloc) against
the allocating entry point (arap_grid_center_order), through the C ABI.

The variant keeps its scratch in a static device array that persists between
calls, so it is called twice in a row on each scene: both results must equal
the allocating entry point's exactly (an integer permutation).  This file is
collected last so that it also runs after every other GPU test."""
import importlib

import numpy as np
import pytest

from tests import _helpers as H

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _t(a):
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def mods(dev):
    lib = importlib.import_module("arap-deformation-of-gaussian-radiance-fields_gb300._lib")
    grid = importlib.import_module("arap-deformation-of-gaussian-radiance-fields_gb300.grid")
    return lib, grid


def _stream():
    return torch.cuda.current_stream().cuda_stream


@pytest.mark.parametrize("name", ["twist20k", "bend50k"])
def test_center_order_noalloc_matches_allocating(mods, name):
    lib, grid = mods
    sc = H.synth.make_scene(name)
    pos = _t(sc.pos)
    G = grid.build_grid(pos, _t(sc.rot), _t(sc.scale), _t(sc.opacity), sc.grid_num)
    N = pos.shape[0]
    ref = torch.empty((N,), dtype=torch.int32, device="cuda")
    rc = lib.load().arap_grid_center_order(G._h, N, pos.data_ptr(), ref.data_ptr(), _stream())
    assert rc == lib.OK
    for call in range(2):
        out = torch.full((N,), -1, dtype=torch.int32, device="cuda")
        rc = lib.load().arap_grid_center_order_noalloc(G._h, N, pos.data_ptr(), out.data_ptr(), _stream())
        assert rc == lib.OK, (call, rc)
        assert torch.equal(out, ref), call


def test_center_order_noalloc_rejects_oversize(mods):
    lib, grid = mods
    sc = H.synth.make_scene("bend4k")
    pos = _t(sc.pos)
    G = grid.build_grid(pos, _t(sc.rot), _t(sc.scale), _t(sc.opacity), sc.grid_num)
    # 4 bytes per Gaussian alone exceed the static scratch: rejected on the
    # host before any device work (the buffers are real and large enough)
    N = lib.CENTER_SCRATCH_BYTES // 4 + 1
    big = torch.zeros((N, 3), dtype=torch.float32, device="cuda")
    out = torch.full((N,), -1, dtype=torch.int32, device="cuda")
    rc = lib.load().arap_grid_center_order_noalloc(G._h, N, big.data_ptr(), out.data_ptr(), _stream())
    assert rc == lib.EUNSUPPORTED
    assert int((out != -1).sum()) == 0
