"""The kNN kernel's CTA sizes (arap_compute_weights_ex) and its autotuner
(arap_knn_autotune): every size gives the same bits, which match the
oracle's indices, and the autotuner returns one of them with its times."""
import numpy as np
import pytest

from tests import _helpers as H

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_knn_sizes_agree_and_autotune(dev):
    from oracle import ed
    sc = H.synth.make_scene("twist20k")
    pts = torch.as_tensor(sc.pos).cuda()
    nodes = torch.as_tensor(sc.node_pos).cuda()
    outs = {t: dev.compute_weights(pts, nodes, sc.k, threads=t) for t in (128, 256, 512)}
    for t in (128, 512):
        assert torch.equal(outs[t][0], outs[256][0]) and torch.equal(outs[t][1], outs[256][1])
    ref_idx, _ = ed.knn_weights(sc.pos, sc.node_pos, sc.k)
    np.testing.assert_array_equal(outs[256][0].cpu().numpy().T, ref_idx)
    best, ms = dev.knn_autotune(pts, nodes, sc.k)
    assert best in (128, 256, 512) and all(v > 0 for v in ms.values())
    assert ms[best] == min(ms.values())
    with pytest.raises(dev.ArapError):
        dev.compute_weights(pts, nodes, sc.k, threads=64)
