"""Oracle: Stage-II alignment of the Gaussians to the deformed density field.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

The reference runs this step as ``GPUOptimize`` (GaussianView.cpp:4363-4486)
for ``_optimize_steps`` steps (101, GaussianView.hpp:420) after a deformation
(GaussianView.cpp:1695-1733).  Each step is four calls into the external
CudaRasterizer: ``forward3d_grid``, ``L1loss3d``, ``backward3d_grid`` and
``update3d``.  Their source is not in the reference tree, so this part is
**parity unpinned**: it is the project's definition of the step, built from
the visible call sites.

Two routines are restated from visible host code, and their known answers are
checked in tests:
- ``judge_empty_cells``: JudgeEmptyGrid, GaussianView.cpp:4272-4316;
- ``expand_converged``: ExpandOpRange, GaussianView.cpp:4319-4360.

The definition of one step follows.  Gaussian i has:
- mean mu_i;
- quaternion q_i (w, x, y, z), normalised when used;
- log-scale l_i, so s_i = exp(l_i);
- logit opacity o_i, so alpha_i = sigmoid(o_i);
- SH coefficients c_i [48].

For a sample x of cell c, with d = x - mu_i and the cell's low-pass filter L_c:
- G_i(x) = exp(-1/2 d^T (Sigma_i + L_c)^-1 d), with Sigma_i = R_i diag(s_i^2) R_i^T;
- density sigma(x) = sum over the cell's list of alpha_i G_i(x), as in
  ``oracle.grid.density``;
- feature F(x) = sum over the same list of alpha_i G_i(x) c_i.

The loss is sum_x |sigma(x) - sigma*(x)| + w_f sum_x |F(x) - F*(x)|_1.  It
runs over the samples of cells that are not converged, and sign(0) = 0.  The
targets sigma* and F* are the pre-deformation field carried by the sample
skinning.

The update is Adam per attribute, for the Gaussians marked moved
(CheckMovedGaussians, GaussianView.cpp:2093-2109):
- m = b1 m + (1 - b1) g, v = b2 v + (1 - b2) g^2;
- theta -= lr m_hat / (sqrt(v_hat) + eps);
- learning rates from GaussianView.hpp:418, read in update3d's argument
  order: opacity 0, SH 0.002, position 0.005, rotation 0.1, log-scale 0.0001;
- b1 = 0.9, b2 = 0.999, eps = 1e-8.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import skin as _skin

F64 = np.float64

LEARNING_RATES = {"opacity": 0.0, "shs": 0.002, "pos": 0.005, "rot": 0.1, "scale": 0.0001}
ADAM_BETA1, ADAM_BETA2, ADAM_EPS = 0.9, 0.999, 1e-8


# ----------------------------------------------------- grid-cell flags ----

def _cell_xyz(idx, g):
    return idx // (g * g), (idx // g) % g, idx % g


def _mark_with_neighbours(mark, cells, g):
    """Marks each cell and its six face neighbours, each clamped to the grid
    (the neighbour of a border cell along the outward axis is itself)."""
    x, y, z = _cell_xyz(np.asarray(cells, np.int64), g)
    mark[cells] = True
    for dx, dy, dz in ((-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)):
        xx = np.clip(x + dx, 0, g - 1)
        yy = np.clip(y + dy, 0, g - 1)
        zz = np.clip(z + dz, 0, g - 1)
        mark[xx * g * g + yy * g + zz] = True


def judge_empty_cells(valid_cells, aim_opacity, grid_num, samples_per_cell=64):
    """JudgeEmptyGrid: int32 [V], 1 for an occupied cell that neither holds
    target density (its samples' aim opacities sum to more than 1e-6) nor
    is a face neighbour of such a cell."""
    valid_cells = np.asarray(valid_cells, np.int64)
    tot = np.asarray(aim_opacity, np.float32).reshape(valid_cells.size, samples_per_cell)
    # the reference sums the 64 float opacities in order into a float
    acc = np.zeros(valid_cells.size, np.float32)
    for j in range(samples_per_cell):
        acc = (acc + tot[:, j]).astype(np.float32)
    keep = np.zeros(grid_num ** 3, bool)
    # float against the double literal 1e-6, as C++ compares them
    _mark_with_neighbours(keep, valid_cells[acc.astype(F64) > 1e-6], grid_num)
    return (~keep[valid_cells]).astype(np.int32)


def expand_converged(valid_cells, converged, grid_num):
    """ExpandOpRange: a copy of ``converged`` [V] bool in which every cell
    that is a face neighbour of a cell not converged is not converged
    either."""
    valid_cells = np.asarray(valid_cells, np.int64)
    conv = np.asarray(converged, bool)
    hot = np.zeros(grid_num ** 3, bool)
    _mark_with_neighbours(hot, valid_cells[~conv], grid_num)
    return conv & ~hot[valid_cells]


# --------------------------------------------------------- the step -----

@dataclass
class GaussianParams:
    """Float64 copies of the optimised attributes, [N,...]."""
    pos: np.ndarray
    rot: np.ndarray        # raw quaternion (w, x, y, z)
    log_scale: np.ndarray
    logit_opacity: np.ndarray
    shs: np.ndarray        # [N,48]

    def copy(self):
        return GaussianParams(*(np.array(getattr(self, f), F64) for f in _FIELDS))


_FIELDS = ("pos", "rot", "log_scale", "logit_opacity", "shs")
_LR_KEY = {"pos": "pos", "rot": "rot", "log_scale": "scale", "logit_opacity": "opacity", "shs": "shs"}


def pairs_of(samples_cell, off, lists):
    """(sample index, Gaussian index) of every pair the density sums over."""
    s_idx, g_idx = [], []
    for s, c in enumerate(np.asarray(samples_cell, np.int64)):
        ids = lists[off[c]:off[c + 1]]
        s_idx.append(np.full(ids.size, s, np.int64))
        g_idx.append(ids.astype(np.int64))
    if not s_idx:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    return np.concatenate(s_idx), np.concatenate(g_idx)


def _sigmoid(x):
    return 1.0 / (1.0 + np.exp(-x))


def _pair_terms(p: GaussianParams, samples, lpf, ps, pg):
    qn = _skin.quat_normalize(p.rot)
    R = _skin.quat_to_matrix(qn)
    s = np.exp(p.log_scale)
    Sig = np.einsum("nij,nj,nkj->nik", R, s * s, R)
    L = lpf[ps] if np.ndim(lpf) == 3 else np.eye(3) * float(lpf)
    A = np.linalg.inv(Sig[pg] + L)
    d = np.asarray(samples, F64)[ps] - p.pos[pg]
    Ad = np.einsum("nij,nj->ni", A, d)
    G = np.exp(-0.5 * np.einsum("ni,ni->n", d, Ad))
    alpha = _sigmoid(p.logit_opacity)
    return qn, R, s, A, d, Ad, G, alpha


def forward(p: GaussianParams, samples, lpf, ps, pg):
    """sigma [S] and F [S,48] of the definition above."""
    S = np.asarray(samples).shape[0]
    _, _, _, _, _, _, G, alpha = _pair_terms(p, samples, lpf, ps, pg)
    g = alpha[pg] * G
    sig = np.bincount(ps, weights=g, minlength=S)
    feat = np.zeros((S, 48))
    np.add.at(feat, ps, g[:, None] * p.shs[pg])
    return sig, feat


def _dR_dq(q):
    """d R / d q for a unit quaternion (w, x, y, z): [N,4,3,3]."""
    w, x, y, z = (q[:, i] for i in range(4))
    o = np.zeros_like(w)
    D = np.empty((q.shape[0], 4, 3, 3))
    D[:, 0] = 2 * np.stack([np.stack([o, -z, y], -1), np.stack([z, o, -x], -1), np.stack([-y, x, o], -1)], 1)
    D[:, 1] = 2 * np.stack([np.stack([o, y, z], -1), np.stack([y, -2 * x, -w], -1),
                            np.stack([z, w, -2 * x], -1)], 1)
    D[:, 2] = 2 * np.stack([np.stack([-2 * y, x, w], -1), np.stack([x, o, z], -1),
                            np.stack([-w, z, -2 * y], -1)], 1)
    D[:, 3] = 2 * np.stack([np.stack([-2 * z, -w, x], -1), np.stack([w, -2 * z, y], -1),
                            np.stack([x, y, o], -1)], 1)
    return D


def loss_and_grad(p: GaussianParams, samples, lpf, ps, pg, aim_sigma, aim_feat, active_sample=None,
                  feature_weight=1.0):
    """(shape loss, feature loss, gradient as a GaussianParams) of the L1
    loss over the active samples (all when ``active_sample`` is None)."""
    S = np.asarray(samples).shape[0]
    N = p.pos.shape[0]
    qn, R, s, A, d, Ad, G, alpha = _pair_terms(p, samples, lpf, ps, pg)
    g = alpha[pg] * G
    sig = np.bincount(ps, weights=g, minlength=S)
    feat = np.zeros((S, 48))
    np.add.at(feat, ps, g[:, None] * p.shs[pg])
    act = np.ones(S, bool) if active_sample is None else np.asarray(active_sample, bool)
    ds = np.where(act, np.sign(sig - aim_sigma), 0.0)                       # dL/dsigma
    df = np.where(act[:, None], feature_weight * np.sign(feat - aim_feat), 0.0)  # dL/dF
    shape_loss = float(np.abs(sig - aim_sigma)[act].sum())
    feature_loss = float(feature_weight * np.abs(feat - aim_feat)[act].sum())
    # per pair: dL/dg = ds + df . c_i
    c = ds[ps] + np.einsum("nk,nk->n", df[ps], p.shs[pg])
    gr = GaussianParams(np.zeros((N, 3)), np.zeros((N, 4)), np.zeros((N, 3)), np.zeros(N), np.zeros((N, 48)))
    np.add.at(gr.shs, pg, g[:, None] * df[ps])
    dalpha = np.bincount(pg, weights=c * G, minlength=N)
    gr.logit_opacity = dalpha * alpha * (1 - alpha)
    de = c * g                                   # dL/de, e = -1/2 d^T A d
    np.add.at(gr.pos, pg, de[:, None] * Ad)      # de/dmu = A d
    # de/dSigma = 1/2 (A d)(A d)^T
    GS = np.zeros((N, 3, 3))
    np.add.at(GS, pg, 0.5 * de[:, None, None] * np.einsum("ni,nj->nij", Ad, Ad))
    # Sigma = R diag(s^2) R^T
    RtGR = np.einsum("nji,njk,nkl->nil", R, GS, R)
    ds_ = 2 * s * np.einsum("nii->ni", RtGR)
    gr.log_scale = ds_ * s
    dR = 2 * np.einsum("nij,njk,nk->nik", GS, R, s * s)
    dqn = np.einsum("nij,ncij->nc", dR, _dR_dq(qn))
    nq = np.linalg.norm(p.rot, axis=1, keepdims=True)
    gr.rot = (dqn - qn * (qn * dqn).sum(1, keepdims=True)) / nq
    return shape_loss, feature_loss, gr


@dataclass
class AdamState:
    step: int = 0
    m: dict = field(default_factory=dict)
    v: dict = field(default_factory=dict)


def adam_update(p: GaussianParams, gr: GaussianParams, st: AdamState, moved=None, lr=None):
    """One Adam step of every attribute for the moved Gaussians (all when
    ``moved`` is None); ``lr`` maps attribute to rate (default
    LEARNING_RATES).  Updates ``p`` and ``st`` in place."""
    lr = dict(LEARNING_RATES if lr is None else lr)
    st.step += 1
    t = st.step
    mv = None if moved is None else np.asarray(moved, bool)
    for f in _FIELDS:
        gv = getattr(gr, f)
        if f not in st.m:
            st.m[f] = np.zeros_like(gv)
            st.v[f] = np.zeros_like(gv)
        m = ADAM_BETA1 * st.m[f] + (1 - ADAM_BETA1) * gv
        v = ADAM_BETA2 * st.v[f] + (1 - ADAM_BETA2) * gv * gv
        step = lr[_LR_KEY[f]] * (m / (1 - ADAM_BETA1 ** t)) / (np.sqrt(v / (1 - ADAM_BETA2 ** t)) + ADAM_EPS)
        val = getattr(p, f)
        if mv is None:
            st.m[f], st.v[f] = m, v
            setattr(p, f, val - step)
        else:
            sel = mv.reshape((-1,) + (1,) * (gv.ndim - 1))
            st.m[f] = np.where(sel, m, st.m[f])
            st.v[f] = np.where(sel, v, st.v[f])
            setattr(p, f, np.where(sel, val - step, val))
