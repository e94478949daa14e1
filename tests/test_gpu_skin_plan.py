"""Planned Gaussian skinning (arap_skin_plan_* + arap_skin_gaussians_planned)
against arap_skin_gaussians, for spatially ordered tiles (all nodes staged in
shared memory) and for shuffled tiles (tiles over 256 distinct nodes take the
global-table path).  The planned blend adds each endpoint's terms in node-id
order rather than kNN order, so the two agree to float32 rounding of the
sums (bit for bit on the global-table tiles), and the plan's slot assignment
keeps every staged record valid."""
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
def test_planned_skinning_matches_unplanned(dev, name, order):
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
    (e0, p0, q0, s0, h0, c0), (e1, p1, q1, s1, h1, c1) = outs
    # twice the bars of the unplanned kernel against the float64 oracle
    # (test_gpu_parity.py; 4x for 1 - |q.q'|, quadratic in the angle): the two
    # kernels differ only in the rounding of the blend sums, which nearly flat
    # Gaussians amplify in q, scale and Sigma
    ext = float(np.ptp(sc.pos, 0).max())
    flat = name.startswith("stress")
    assert (e0 - e1).abs().max().item() <= 4e-6 * ext
    assert (p0 - p1).abs().max().item() <= 4e-6 * ext
    dq = (1 - (q0.double() * q1.double()).sum(1).abs()).cpu().numpy()
    assert dq.max() <= 8e-6, dq.max()
    def fro(v):  # packed xx, xy, xz, yy, yz, zz
        return torch.sqrt(v[:, 0] ** 2 + v[:, 3] ** 2 + v[:, 5] ** 2 + 2 * (v[:, 1] ** 2 + v[:, 2] ** 2 + v[:, 4] ** 2))
    rel = (fro(c0.double() - c1.double()) / fro(c0.double()).clamp_min(1e-300)).cpu().numpy()
    assert np.quantile(rel, 0.999) <= (2e-4 if flat else 4e-5) and rel.max() <= (1e-3 if flat else 2e-4)
    assert (h0 - h1).abs().max().item() <= (1e-3 if flat else 1e-4)
    if order == "shuffled":
        # the tiles over 256 nodes take the kNN-order path: bit for bit there
        ei = eidx.cpu().numpy().reshape(-1, N)  # planes [k * 6][N]
        counts = np.array([np.unique(ei[:, t0:t0 + 128]).size for t0 in range(0, N, 128)])
        assert (counts > 256).sum() == info["overflow_tiles"]
        over = np.repeat(counts > 256, 128)[:N]
        m = torch.from_numpy(over).cuda()
        assert torch.equal(p0[m], p1[m]) and torch.equal(h0[m], h1[m])
    plan.close()
