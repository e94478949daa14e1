"""Stage-II alignment oracle (oracle/stage2.py), on CPU.

- Known answers for the two host routines restated from the reference:
  JudgeEmptyGrid (GaussianView.cpp:4272-4316) and ExpandOpRange
  (GaussianView.cpp:4319-4360).
- The analytic gradient of the project's definition of the L1 alignment loss,
  checked against float64 central differences.
- The Adam update: its first step and its moved-Gaussian mask.
- A few steps reducing the loss."""
import numpy as np
import pytest

from oracle import stage2 as s2


def _cell(x, y, z, g):
    return x * g * g + y * g + z


def test_judge_empty_cells_known_answer():
    g = 4
    cells = np.array([_cell(0, 1, 1, g), _cell(1, 1, 1, g), _cell(3, 3, 3, g), _cell(0, 0, 1, g),
                      _cell(2, 2, 2, g), _cell(0, 1, 3, g)])
    op = np.zeros((cells.size, 64), np.float32)
    op[0] = 1e-3                      # holds target density
    op[4, :] = np.float32(1e-8)       # 64e-8 < 1e-6: no target density
    op[5, 0] = np.float32(2e-6)       # one sample above the threshold
    empty = s2.judge_empty_cells(cells, op.reshape(-1), g)
    # (0,1,1) holds density; (1,1,1) and (0,0,1) are its face neighbours;
    # (3,3,3) and (2,2,2) are neither; (0,1,3) holds density
    assert empty.tolist() == [0, 0, 1, 0, 1, 0]
    # a diagonal neighbour is not a face neighbour
    cells2 = np.array([_cell(1, 1, 1, g), _cell(2, 2, 1, g)])
    op2 = np.zeros((2, 64), np.float32)
    op2[0] = 1.0
    assert s2.judge_empty_cells(cells2, op2.reshape(-1), g).tolist() == [0, 1]


def test_expand_converged_known_answer():
    g = 4
    cells = np.array([_cell(1, 1, 1, g), _cell(1, 1, 2, g), _cell(1, 2, 2, g), _cell(3, 3, 3, g),
                      _cell(0, 1, 1, g)])
    conv = np.array([False, True, True, True, True])
    out = s2.expand_converged(cells, conv, g)
    # the face neighbours of (1,1,1) among the cells: (1,1,2) and (0,1,1)
    assert out.tolist() == [False, False, True, True, False]
    # all converged: nothing changes
    assert s2.expand_converged(cells, np.ones(5, bool), g).tolist() == [True] * 5
    # a border cell: its clamped neighbour is itself
    c3 = np.array([_cell(3, 3, 3, g), _cell(3, 3, 2, g)])
    assert s2.expand_converged(c3, np.array([False, True]), g).tolist() == [False, False]


def _toy(seed=0, N=5, S=40, perturb=0.05):
    rng = np.random.default_rng(seed)
    true = s2.GaussianParams(
        pos=rng.uniform(0.3, 0.7, (N, 3)),
        rot=rng.normal(size=(N, 4)),
        log_scale=rng.normal(-2.0, 0.2, (N, 3)),
        logit_opacity=rng.normal(0, 1, N),
        shs=rng.normal(0, 0.3, (N, 48)))
    samples = rng.uniform(0.2, 0.8, (S, 3))
    off = np.array([0, N], np.int64)
    lists = np.arange(N, dtype=np.int32)
    ps, pg = s2.pairs_of(np.zeros(S, np.int64), off, lists)
    lpf = 0.2 * (0.6 / 16) ** 2
    aim_sig, aim_feat = s2.forward(true, samples, lpf, ps, pg)
    p = true.copy()
    p.pos = p.pos + rng.normal(0, perturb, p.pos.shape)
    p.rot = p.rot + rng.normal(0, perturb, p.rot.shape)
    p.log_scale = p.log_scale + rng.normal(0, perturb, p.log_scale.shape)
    p.logit_opacity = p.logit_opacity + rng.normal(0, perturb, p.logit_opacity.shape)
    p.shs = p.shs + rng.normal(0, perturb, p.shs.shape)
    return p, samples, lpf, ps, pg, aim_sig, aim_feat


@pytest.mark.parametrize("adaptive", [False, True])
def test_gradient_matches_finite_differences(adaptive):
    p, samples, lpf, ps, pg, aim_sig, aim_feat = _toy(seed=1)
    if adaptive:
        rng = np.random.default_rng(5)
        B = rng.normal(0, 0.01, (samples.shape[0], 3, 3))
        lpf = np.einsum("nij,nkj->nik", B, B) + 1e-4 * np.eye(3)
    _, _, gr = s2.loss_and_grad(p, samples, lpf, ps, pg, aim_sig, aim_feat, feature_weight=0.5)
    sig0, feat0 = s2.forward(p, samples, lpf, ps, pg)
    sgn_s = np.sign(sig0 - aim_sig)
    sgn_f = np.sign(feat0 - aim_feat)

    def lin_loss(q):
        # the L1 loss with its signs frozen at p: the same gradient at p
        sig, feat = s2.forward(q, samples, lpf, ps, pg)
        return float((sgn_s * (sig - aim_sig)).sum() + 0.5 * (sgn_f * (feat - aim_feat)).sum())

    eps = 1e-6
    for f in ("pos", "rot", "log_scale", "logit_opacity", "shs"):
        base = getattr(p, f)
        fd = np.zeros_like(base)
        for i in np.ndindex(base.shape):
            qp, qm = p.copy(), p.copy()
            getattr(qp, f)[i] += eps
            getattr(qm, f)[i] -= eps
            fd[i] = (lin_loss(qp) - lin_loss(qm)) / (2 * eps)
        an = getattr(gr, f)
        scale = np.abs(fd).max() + 1e-12
        assert np.abs(an - fd).max() / scale < 1e-6, f


def test_active_samples_only():
    p, samples, lpf, ps, pg, aim_sig, aim_feat = _toy(seed=2)
    act = np.zeros(samples.shape[0], bool)
    sl, fl, gr = s2.loss_and_grad(p, samples, lpf, ps, pg, aim_sig, aim_feat, active_sample=act)
    assert sl == 0 and fl == 0
    assert all(np.all(getattr(gr, f) == 0) for f in ("pos", "rot", "log_scale", "logit_opacity", "shs"))


def test_adam_first_step_and_moved_mask():
    p, samples, lpf, ps, pg, aim_sig, aim_feat = _toy(seed=3)
    _, _, gr = s2.loss_and_grad(p, samples, lpf, ps, pg, aim_sig, aim_feat)
    moved = np.array([True, False, True, True, False])
    q = p.copy()
    st = s2.AdamState()
    s2.adam_update(q, gr, st, moved=moved)
    # the first bias-corrected step is lr g / (|g| + eps)
    lr = s2.LEARNING_RATES
    exp_pos = p.pos - lr["pos"] * gr.pos / (np.abs(gr.pos) + s2.ADAM_EPS)
    np.testing.assert_allclose(q.pos[moved], exp_pos[moved], rtol=1e-12, atol=1e-15)
    np.testing.assert_array_equal(q.pos[~moved], p.pos[~moved])
    np.testing.assert_array_equal(q.shs[~moved], p.shs[~moved])
    np.testing.assert_array_equal(q.logit_opacity, p.logit_opacity)   # learning rate 0
    assert np.all(st.m["pos"][~moved] == 0)


def test_steps_reduce_the_loss():
    p, samples, lpf, ps, pg, aim_sig, aim_feat = _toy(seed=4, perturb=0.02)
    lr = {"opacity": 0.01, "shs": 0.002, "pos": 0.002, "rot": 0.01, "scale": 0.005}
    st = s2.AdamState()
    losses = []
    for _ in range(40):
        sl, fl, gr = s2.loss_and_grad(p, samples, lpf, ps, pg, aim_sig, aim_feat)
        losses.append(sl + fl)
        s2.adam_update(p, gr, st, lr=lr)
    assert losses[-1] < 0.5 * losses[0]
