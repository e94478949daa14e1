"""Oracle: density-grid construction, adaptive low-pass filter and density sampling.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  Restated from:

* ``overall_aabb``    -- GaussianView.cpp:3601-3631 (getOverallAABB), float32
* ``gaussian_aabbs``  -- GaussianView.cpp:3961-4019 / 3653-3690 (3-sigma-style
                         box from s_3d = sqrt(-2 ln(alpha_cut/alpha)) s)
* ``cell_csr``        -- cudakdtree.cu:425-451 + GaussianView.cpp:4077-4100
                         (GetBoxesGsGrid counts, serial fill: every cell's list
                         ascending by Gaussian index)
* ``grid_samples``    -- GaussianView.cpp:4104-4133 (64 samples per occupied
                         cell, in cell order)
* ``center_cells``    -- GaussianView.cpp:4136-4145 / 3918-3953 (cell of each
                         centre and the stable cell-order permutation)
* ``ada_lpf``         -- GaussianView.cpp:4670-4751 (per occupied cell the
                         least-squares linear map of the 8 corner samples,
                         M M^T * 0.2)
* ``density``         -- the project's definition of CudaRasterizer's
                         forward3d_grid (source absent; parity unpinned):
                         sigma(x) = sum_i a_i exp(-1/2 d^T (S_i + L)^-1 d),
                         F(x) = sum_i a_i exp(...) SH_i over the cell's list,
                         L = lpf * I or the cell's adaptive 3x3.
"""
from __future__ import annotations

import numpy as np

from . import skin as _skin

F32 = np.float32
ALPHA_CUT = F32(1.0) / F32(255.0)      # CUTOFF_ALPHA, helper.hpp:62
NUM_SAMPLES_PER_DIM = 128               # helper.hpp:52
SAMPLES_PER_GRID = 4                    # helper.hpp:56


def overall_aabb(pos):
    p = np.asarray(pos, F32)
    mn = p.min(axis=0)
    mx = p.max(axis=0)
    mean = ((mx + mn) / F32(2.0)).astype(F32)
    mn2 = ((mn - mean) * F32(1.1) + mean).astype(F32)
    mx2 = (((mx - mean) * F32(1.1) + mean - mn2) * F32(1.0 + 1.0 / NUM_SAMPLES_PER_DIM) + mn2).astype(F32)
    mn2 = np.minimum(mn2, F32(-0.75))
    mx2 = np.maximum(mx2, F32(0.75))
    return mn2.astype(F32), mx2.astype(F32)


def grid_step(mn, mx, grid_num):
    steps = ((mx - mn) / F32(grid_num)).astype(F32)
    return F32(steps.max())


def gaussian_aabbs(pos, rot, scale, opacity):
    """[N,3] min and max corners (float32)."""
    p = np.asarray(pos, F32)
    op = np.asarray(opacity, F32)
    s = np.asarray(scale, F32)
    with np.errstate(divide="ignore", invalid="ignore"):
        f = np.sqrt(F32(-2.0) * np.log(ALPHA_CUT / op)).astype(F32)
    f = np.where(op <= ALPHA_CUT, F32(0), f)
    s3 = (f[:, None] * s).astype(F32)
    R = _skin.quat_to_matrix(_skin.quat_normalize(np.asarray(rot, np.float64))).astype(F32)
    lo = p.copy()
    hi = p.copy()
    for d in range(3):
        e = (R[:, :, d] * s3[:, d:d + 1]).astype(F32)
        for q in ((p + e).astype(F32), (p - e).astype(F32)):
            lo = np.minimum(lo, q)
            hi = np.maximum(hi, q)
    return lo, hi


def cell_ranges(lo, hi, mn, step, grid_num, padding=1):
    a = np.floor((lo - mn) / step).astype(np.int64) - padding
    b = np.floor((hi - mn) / step).astype(np.int64) + padding
    return np.maximum(a, 0), np.minimum(b, grid_num - 1)


def cell_csr(lo, hi, mn, step, grid_num, padding=1):
    """(offsets int64 [g^3+1], lists int32) -- every cell's Gaussians ascending."""
    a, b = cell_ranges(lo, hi, mn, step, grid_num, padding)
    g = grid_num
    cells, gids = [], []
    for i in range(lo.shape[0]):
        xs = np.arange(a[i, 0], b[i, 0] + 1)
        ys = np.arange(a[i, 1], b[i, 1] + 1)
        zs = np.arange(a[i, 2], b[i, 2] + 1)
        c = (xs[:, None, None] * g * g + ys[None, :, None] * g + zs[None, None, :]).ravel()
        cells.append(c)
        gids.append(np.full(c.size, i, np.int64))
    cells = np.concatenate(cells) if cells else np.zeros(0, np.int64)
    gids = np.concatenate(gids) if gids else np.zeros(0, np.int64)
    order = np.lexsort((gids, cells))
    counts = np.bincount(cells, minlength=g ** 3)
    off = np.zeros(g ** 3 + 1, np.int64)
    off[1:] = np.cumsum(counts)
    return off, gids[order].astype(np.int32)


def grid_samples(off, mn, step, grid_num):
    """Occupied cells ascending and their 64 samples each [V*64,3] float32."""
    g = grid_num
    valid = np.flatnonzero(np.diff(off) > 0)
    interval = F32(step / F32(SAMPLES_PER_GRID))
    x = valid // (g * g)
    y = (valid - x * g * g) // g
    z = valid % g
    out = np.empty((valid.size, 64, 3), F32)
    half = 0.5 * np.float64(interval)
    for d, ci in enumerate((x, y, z)):
        # float32 products and sums (int * float is float in the reference)
        base = (mn[d] + (ci.astype(F32) * F32(step)).astype(F32)).astype(F32)
        base = (base.astype(np.float64) + half).astype(F32)
        for s in range(64):
            si = (s // 16, (s % 16) // 4, s % 4)[d]
            out[:, s, d] = (base + (F32(si) * interval).astype(F32)).astype(F32)
    return valid, out.reshape(-1, 3)


def center_cells(pos, mn, step, grid_num):
    c = np.floor((np.asarray(pos, F32) - mn) / step).astype(np.int64)
    cell = c[:, 0] * grid_num * grid_num + c[:, 1] * grid_num + c[:, 2]
    order = np.argsort(cell, kind="stable")
    new_index = np.empty_like(order)
    new_index[order] = np.arange(order.size)
    return cell, new_index


def ada_lpf(samples, lpf=0.2):
    """[V,3,3] float32: M M^T * lpf with M the least-squares map of the unit
    cube's corners to the cell's corner samples (scaled by 1/3)."""
    S = np.asarray(samples, F32).reshape(-1, 64, 3).astype(np.float64)
    corners = np.array([[(c % 2), (c // 2) % 2, (c // 4) % 2] for c in range(8)], np.float64)  # Q^T rows
    idx = (corners[:, 0] * 48 + corners[:, 1] * 12 + corners[:, 2] * 3).astype(int)
    P = (S[:, idx, :] - S[:, :1, :]) / 3.0          # [V,8,3]
    Q = corners.T                                    # [3,8]
    G = np.linalg.inv(Q @ Q.T)
    M = np.einsum("vic,ki,kj->vcj", P, Q, G)         # M = P Q^T (Q Q^T)^-1
    return (np.einsum("vij,vkj->vik", M, M) * lpf).astype(F32)


def density(samples, off, lists, cell_of_sample, pos, rot, scale, opacity, shs, lpf_mat):
    """sigma [S] and feature [S,48] (float64) by the project's definition."""
    cov = _skin.covariance6(rot, scale)
    C = np.empty((cov.shape[0], 3, 3))
    C[:, 0, 0], C[:, 0, 1], C[:, 0, 2] = cov[:, 0], cov[:, 1], cov[:, 2]
    C[:, 1, 0], C[:, 1, 1], C[:, 1, 2] = cov[:, 1], cov[:, 3], cov[:, 4]
    C[:, 2, 0], C[:, 2, 1], C[:, 2, 2] = cov[:, 2], cov[:, 4], cov[:, 5]
    S = samples.shape[0]
    sig = np.zeros(S)
    feat = np.zeros((S, 48))
    for s in range(S):
        c = cell_of_sample[s]
        ids = lists[off[c]:off[c + 1]]
        if ids.size == 0:
            continue
        L = lpf_mat[s] if lpf_mat.ndim == 3 else np.eye(3) * lpf_mat
        A = np.linalg.inv(C[ids] + L)
        d = samples[s].astype(np.float64) - pos[ids].astype(np.float64)
        g = np.asarray(opacity, np.float64)[ids] * np.exp(-0.5 * np.einsum("ni,nij,nj->n", d, A, d))
        sig[s] = g.sum()
        feat[s] = g @ np.asarray(shs, np.float64)[ids]
    return sig, feat
