"""Planned Gaussian skinning (arap_skin_plan_* + arap_skin_gaussians_planned)
against arap_skin_gaussians: the same arithmetic in the same order, so every
output must be bit-identical, for spatially ordered tiles (all nodes staged in
shared memory) and for shuffled tiles (tiles over 256 distinct nodes take the
global-table path)."""
import numpy as np
import pytest

from tests import _helpers as H

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _t(a):
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


def _transforms(n, rng, amp=0.3):
    # near-rigid node transforms (column-major R), as the parity tests use
    from oracle import skin
    q = rng.standard_normal((n, 4))
    R = skin.quat_to_matrix(skin.quat_normalize(q * np.array([4, amp, amp, amp])))
    A = R + 0.02 * rng.standard_normal((n, 3, 3))
    rot = A.transpose(0, 2, 1).reshape(n, 9).astype(np.float32)
    return rot, (0.05 * rng.standard_normal((n, 3))).astype(np.float32)


@pytest.mark.parametrize("name,order", [("twist20k", "cells"), ("stress40k", "cells"), ("twist20k", "shuffled")])
def test_planned_skinning_is_bit_identical(dev, name, order):
    sc = H.synth.make_scene(name)
    rng = np.random.default_rng(11)
    if order == "cells":
        key = np.floor((sc.pos - sc.pos.min(0)) / (np.ptp(sc.pos, 0).max() / 32)).astype(np.int64)
        perm = np.lexsort((key[:, 2], key[:, 1], key[:, 0]))
    else:
        perm = rng.permutation(sc.n_gauss)
    pos0, rot0, scale0, shs0 = sc.pos[perm], sc.rot[perm], sc.scale[perm], sc.shs[perm]
    N = pos0.shape[0]
    rot_n, trans_n = _transforms(sc.n_nodes, rng)
    table = dev.node_table(_t(rot_n), _t(trans_n), _t(sc.node_pos))
    ends_a, ends_xyz = dev.end_points(_t(pos0), _t(rot0), _t(scale0))
    eidx, ew = dev.compute_weights(ends_xyz, _t(sc.node_pos), sc.k)
    plan = dev.SkinPlan(eidx, ew)
    info = plan.info()
    if order == "cells":
        assert info["overflow_tiles"] == 0 and 0 < info["max_nodes"] <= 256
    else:
        assert info["overflow_tiles"] > 0
    ends_b = ends_a.clone()
    outs = []
    for planned, ends in ((False, ends_a), (True, ends_b)):
        pos = torch.empty((N, 3), device="cuda")
        q = _t(rot0)
        s = torch.empty((N, 3), device="cuda")
        shs = _t(shs0)
        cov = torch.empty((N, 6), device="cuda")
        if planned:
            dev.skin_gaussians_planned(plan, ends, table, _t(scale0), pos, q, s, shs, cov, precision=1)
        else:
            dev.skin_gaussians(ends, eidx, ew, table, _t(scale0), pos, q, s, shs, cov, precision=1)
        outs.append((ends, pos, q, s, shs, cov))
    torch.cuda.synchronize()
    assert dev.device_status() == 0 and plan.status() == 0
    for a, b in zip(*outs):
        assert torch.equal(a, b)
    plan.close()
