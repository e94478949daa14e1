"""Oracle: kNN skinning weights, deformation graph and the Gauss-Newton ED solve.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  Parity unpinned
against executed reference code; restated from the reference source:

* ``knn`` / ``knn_weights`` / ``build_graph``  -- Deform.hpp:153-208, 84-95
* ``EDProblem`` (row bookkeeping)               -- Deform.hpp:414-455,
  Deform.cpp:6-75 (GetControlNums, BelongsToSameBlock, SelectKeyControls)
* ``residual``                                  -- Deform.cpp:378-581
* ``jacobian``                                  -- Deform.cpp:180-376
* ``gauss_newton``                              -- Deform.cpp:77-169
* ``put_free_inputs``                           -- Deform.hpp:140-151
* ``ed_blend``                                  -- Deform.hpp:230-249

Precision follows the reference: node and point positions are float32
(``Pos`` = sibr::Vector3f); distances for the kNN are float32 sqrt of a
float32 sum (Deform.hpp:164-165); the solve vector, residual and Jacobian are
float64; the blend accumulates into a float32 output (Deform.hpp:243-245).

Tie order in the kNN: the reference's selection sort breaks exact distance
ties by array position after earlier swaps; here ties go to the lower node
index.  The two differ only for exactly equal float32 distances.
"""
from __future__ import annotations

import dataclasses

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

F32 = np.float32
F64 = np.float64


# ---------------------------------------------------------------- kNN ----

def _dist_f32(p, nodes):
    """float32 distances exactly as Deform.hpp:164-165: ((dx*dx+dy*dy)+dz*dz)."""
    dx = p[:, None, 0] - nodes[None, :, 0]
    dy = p[:, None, 1] - nodes[None, :, 1]
    dz = p[:, None, 2] - nodes[None, :, 2]
    d2 = (dx * dx + dy * dy) + dz * dz
    return np.sqrt(d2)


def knn(points: np.ndarray, nodes: np.ndarray, kk: int):
    """Indices (int64 [P,kk]) and float32 distances of the kk nearest nodes,
    ascending by (distance, index).  Deform.hpp:153-185."""
    points = np.ascontiguousarray(points, F32)
    nodes = np.ascontiguousarray(nodes, F32)
    P, n = points.shape[0], nodes.shape[0]
    if kk > n:
        raise ValueError("kk=%d exceeds node count %d" % (kk, n))
    idx_out = np.empty((P, kk), np.int64)
    d_out = np.empty((P, kk), F32)
    chunk = max(1, (1 << 22) // max(n, 1))
    ar = np.arange(n)
    for s in range(0, P, chunk):
        d = _dist_f32(points[s:s + chunk], nodes)
        m = d.shape[0]
        if kk < n:
            part = np.argpartition(d, kk - 1, axis=1)[:, :kk]
        else:
            part = np.broadcast_to(ar, (m, n)).copy()
        pd = np.take_along_axis(d, part, axis=1)
        thr = pd.max(axis=1)
        # rows with ties at the threshold need an exact (d, index) order
        n_le = (d <= thr[:, None]).sum(axis=1)
        tie_rows = np.flatnonzero(n_le > kk)
        for r in tie_rows:
            o = np.lexsort((ar, d[r]))[:kk]
            part[r] = o
            pd[r] = d[r, o]
        # sort each row by (d, idx)
        order = np.lexsort((part, pd), axis=1)
        idx_out[s:s + m] = np.take_along_axis(part, order, axis=1)
        d_out[s:s + m] = np.take_along_axis(pd, order, axis=1)
    return idx_out, d_out


def knn_weights(points: np.ndarray, nodes: np.ndarray, k: int):
    """Skinning weights w_j = (1 - d_j/d_{k+1})^2 normalised (Deform.hpp:187-208).

    Returns (idx int64 [P,k], w float64 [P,k])."""
    idx, d = knn(points, nodes, k + 1)
    dmax = d[:, k].astype(F64)
    dist = d[:, :k].astype(F64)
    with np.errstate(divide="ignore", invalid="ignore"):
        w = (1.0 - dist / dmax[:, None]) ** 2
    if k == 1:
        w[:] = 1.0
    else:
        w = w / w.sum(axis=1, keepdims=True)
    return idx[:, :k], w


def build_graph(nodes: np.ndarray, k: int) -> np.ndarray:
    """Each node's k nearest other nodes (Deform.hpp:84-95: search k+1, skip the first)."""
    idx, _ = knn(nodes, nodes, k + 1)
    return idx[:, 1:]


# ------------------------------------------------------------ problem ----

@dataclasses.dataclass
class EDProblem:
    """Inputs of one ``Deform`` solve (Deform.hpp:414-455).

    node_pos   float32 [n,3]  current node positions (``DeformGraph::nodes``)
    neighbors  int [n,k]      node graph (``Node::Neighbor``)
    anchor_idx int [n,k]      kNN of each node's own vertex
                              (``cand_vertices[nodes[i].Vertex_index]``)
    anchor_w   float64 [n,k]  its weights
    blocks     list of int arrays (``indices_blocks``), block_type int [nb]
    aims       float32 [n,3]  target positions (``aim_positions``)
    """
    node_pos: np.ndarray
    neighbors: np.ndarray
    anchor_idx: np.ndarray
    anchor_w: np.ndarray
    blocks: list
    block_type: np.ndarray
    aims: np.ndarray
    cons_on_center: bool = False
    weighting_factor: float = 1.0
    w_rot: float = 1.0
    w_reg: float = 10.0
    w_con: float = 100.0

    def __post_init__(self):
        self.node_pos = np.asarray(self.node_pos, F32)
        self.aims = np.asarray(self.aims, F32)
        self.neighbors = np.asarray(self.neighbors, np.int64)
        self.anchor_idx = np.asarray(self.anchor_idx, np.int64)
        self.anchor_w = np.asarray(self.anchor_w, F64)
        self.block_type = np.asarray(self.block_type, np.int64)
        self.blocks = [np.asarray(b, np.int64) for b in self.blocks]
        n, k = self.neighbors.shape
        self.n, self.k = n, k
        # UpdateIndicies (GaussianView.cpp:2010-2035): blocks with type < 0 are static
        static = set()
        for b, t in zip(self.blocks, self.block_type):
            if t < 0:
                static.update(int(v) for v in b)
        self.static = np.array(sorted(static), np.int64)
        self.free = np.array(sorted(set(range(n)) - static), np.int64)
        self.rank = np.full(n, -1, np.int64)
        self.rank[self.free] = np.arange(self.free.size)
        self.F = int(self.free.size)
        # BelongsToSameBlock (Deform.cpp:20-32): blocks with type == -1 skipped
        memb = [np.isin(np.arange(n), b) for b, t in zip(self.blocks, self.block_type) if t != -1]

        def same_block(i, j):
            r = np.zeros(i.shape, bool)
            for m in memb:
                r |= m[i] & m[j]
            return r
        fi = np.repeat(self.free, k)
        fj = self.neighbors[self.free].reshape(-1)
        wf = F64(F32(self.weighting_factor))
        self.reg_scale = np.where(same_block(fi, fj), wf, 1.0).reshape(self.F, k)
        # control rows
        self.ctrl_blocks = [i for i, t in enumerate(self.block_type) if t != -1]
        if self.cons_on_center:
            # SelectKeyControls (Deform.cpp:34-75): the set of the first
            # min(20, |block|) ids of the block; centre = mean of their aims
            self.center_sets, self.center_aims = [], []
            for bi in self.ctrl_blocks:
                b = self.blocks[bi]
                m = min(20, b.size)
                self.center_sets.append(np.array(sorted(set(int(v) for v in b[:m])), np.int64))
                c = np.zeros(3, F32)
                for v in b[:m]:
                    c = (c + self.aims[v]).astype(F32)
                self.center_aims.append((c / F32(m)).astype(F32))
            self.n_ctrl_rows = 3 * len(self.ctrl_blocks)
        else:
            self.ctrl_nodes = (np.concatenate([self.blocks[i] for i in self.ctrl_blocks])
                               if self.ctrl_blocks else np.zeros(0, np.int64))
            self.n_ctrl_rows = 3 * self.ctrl_nodes.size
        self.sw_rot = np.sqrt(self.w_rot)
        self.sw_reg = np.sqrt(self.w_reg)
        self.sw_con = np.sqrt(self.w_con)
        self.n_rows = self.F * (6 + 3 * k) + self.static.size * 3 * k + self.n_ctrl_rows
        self.n_cols = 12 * self.F


def identity_x(F: int) -> np.ndarray:
    """Deform.cpp:83-93."""
    x = np.zeros((F, 12), F64)
    x[:, 0] = x[:, 4] = x[:, 8] = 1.0
    return x.reshape(-1)


def _rmul(X, v):
    """R v with R given column-major in X[...,0:9] (Deform.hpp:29-36)."""
    return X[..., 0:3] * v[..., 0:1] + X[..., 3:6] * v[..., 1:2] + X[..., 6:9] * v[..., 2:3]


def _blend_constraint(pr: EDProblem, X, c_nodes):
    """sum_j w_cj (R_j(v_c - g_j) + g_j + t_j) over the anchor kNN (free j),
    w_cj v_c otherwise (Deform.cpp:540-573)."""
    g = pr.node_pos.astype(F64)
    ve = g[c_nodes]                                   # [C,3]
    idx = pr.anchor_idx[c_nodes]                       # [C,k]
    wei = pr.anchor_w[c_nodes]                         # [C,k]
    rk = pr.rank[idx]
    gj = g[idx]
    Xj = X[np.maximum(rk, 0)]                          # [C,k,12]
    moved = _rmul(Xj, ve[:, None, :] - gj) + gj + Xj[..., 9:12]
    term = np.where((rk >= 0)[..., None], moved, ve[:, None, :])
    return (wei[..., None] * term).sum(axis=1)


def residual(pr: EDProblem, x: np.ndarray) -> np.ndarray:
    """CalcEnergyFunc (Deform.cpp:378-581)."""
    X = x.reshape(pr.F, 12)
    c0, c1, c2 = X[:, 0:3], X[:, 3:6], X[:, 6:9]
    rot = pr.sw_rot * np.stack([
        (c0 * c1).sum(1), (c0 * c2).sum(1), (c1 * c2).sum(1),
        (c0 * c0).sum(1) - 1.0, (c1 * c1).sum(1) - 1.0, (c2 * c2).sum(1) - 1.0], axis=1)
    g = pr.node_pos.astype(F64)
    nb = pr.neighbors[pr.free]                         # [F,k]
    rk = pr.rank[nb]
    gj = g[pr.free][:, None, :]
    gk = g[nb]
    tk = np.where((rk >= 0)[..., None], X[np.maximum(rk, 0), 9:12], 0.0)
    new_n = _rmul(X[:, None, :], gk - gj) + gj + X[:, None, 9:12] - gk - tk
    reg = pr.sw_reg * new_n * pr.reg_scale[..., None]
    nbs = pr.neighbors[pr.static]
    rks = pr.rank[nbs]
    tks = np.where((rks >= 0)[..., None], X[np.maximum(rks, 0), 9:12], 0.0)
    sta = pr.sw_reg * (-tks)
    if pr.cons_on_center:
        con = []
        for S, ca in zip(pr.center_sets, pr.center_aims):
            nv = _blend_constraint(pr, X, S)
            con.append((pr.sw_con * (nv - ca.astype(F64))).sum(axis=0))
        con = np.array(con, F64).reshape(-1)
    else:
        nv = _blend_constraint(pr, X, pr.ctrl_nodes)
        con = (pr.sw_con * (nv - pr.aims[pr.ctrl_nodes].astype(F64))).reshape(-1)
    return np.concatenate([rot.reshape(-1), reg.reshape(-1), sta.reshape(-1), con])


def jacobian(pr: EDProblem, x: np.ndarray) -> sp.csr_matrix:
    """FastCalcJacobiMat (Deform.cpp:180-376); duplicate triplets are summed
    as Eigen's setFromTriplets does."""
    F, k = pr.F, pr.k
    X = x.reshape(F, 12)
    rows, cols, vals = [], [], []
    w = pr.sw_rot
    base_r = 6 * np.arange(F)
    base_c = 12 * np.arange(F)
    # rotation rows (Deform.cpp:189-220)
    spec = [(0, [0, 1, 2], [3, 4, 5]), (0, [3, 4, 5], [0, 1, 2]),
            (1, [0, 1, 2], [6, 7, 8]), (1, [6, 7, 8], [0, 1, 2]),
            (2, [3, 4, 5], [6, 7, 8]), (2, [6, 7, 8], [3, 4, 5])]
    for r, cc, xs in spec:
        for c, xi in zip(cc, xs):
            rows.append(base_r + r)
            cols.append(base_c + c)
            vals.append(X[:, xi] * w)
    for j in range(3):
        for c in range(3):
            rows.append(base_r + 3 + j)
            cols.append(base_c + 3 * j + c)
            vals.append(2.0 * X[:, 3 * j + c] * w)
    index = 6 * F
    # regularisation rows, free side (Deform.cpp:222-266)
    wr = pr.sw_reg
    g32 = pr.node_pos
    nb = pr.neighbors[pr.free]
    rk = pr.rank[nb]
    dfl = (g32[nb] - g32[pr.free][:, None, :]).astype(F64)   # float32 difference
    s = pr.reg_scale
    rbase = index + 3 * (np.arange(F)[:, None] * k + np.arange(k)[None, :])  # [F,k]
    cbase = (12 * np.arange(F))[:, None] * np.ones((1, k), np.int64)
    for j in range(3):
        for c in range(3):
            rows.append((rbase + j).ravel())
            cols.append((cbase + j + 3 * c).ravel())
            vals.append((dfl[..., c] * wr * s).ravel())
        rows.append((rbase + j).ravel())
        cols.append((cbase + j + 9).ravel())
        vals.append(np.full(F * k, wr))
        m = rk >= 0
        rows.append((rbase + j)[m])
        cols.append((12 * rk + j + 9)[m])
        vals.append((-wr * s)[m])
    index += 3 * F * k
    # static side (Deform.cpp:268-297)
    S = pr.static.size
    if S:
        nbs = pr.neighbors[pr.static]
        rks = pr.rank[nbs]
        rbs = index + 3 * (np.arange(S)[:, None] * k + np.arange(k)[None, :])
        m = rks >= 0
        for j in range(3):
            rows.append((rbs + j)[m])
            cols.append((12 * rks + 9 + j)[m])
            vals.append(np.full(int(m.sum()), -wr))
    index += 3 * S * k
    # constraints (Deform.cpp:299-371)
    wc = pr.sw_con
    if pr.cons_on_center:
        groups = [(index + 3 * b, Sb) for b, Sb in enumerate(pr.center_sets)]
    else:
        C = pr.ctrl_nodes.size
        groups = [(index + 3 * np.arange(C), pr.ctrl_nodes)]
    for rb, cn in groups:
        cn = np.asarray(cn)
        rb = np.broadcast_to(np.asarray(rb), cn.shape)
        idx = pr.anchor_idx[cn]
        wei = pr.anchor_w[cn]
        rkc = pr.rank[idx]
        dd = (g32[cn][:, None, :] - g32[idx]).astype(F64)     # float32 difference
        m = rkc >= 0
        rr = np.broadcast_to(rb[:, None], idx.shape)
        for kk in range(3):
            for c in range(3):
                rows.append((rr + kk)[m])
                cols.append((12 * rkc + 3 * c + kk)[m])
                vals.append((wei * dd[..., c] * wc)[m])
            rows.append((rr + kk)[m])
            cols.append((12 * rkc + 9 + kk)[m])
            vals.append((wei * wc)[m])
    J = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(pr.n_rows, pr.n_cols)).tocsr()
    J.sum_duplicates()
    return J


@dataclasses.dataclass
class GNStats:
    iterations: int
    energies: list          # energy f.f at the start of each iteration
    halvings: list          # number of step halvings per iteration
    final_energy: float


def gauss_newton(pr: EDProblem, max_iters: int = 30, early_exit: bool = True,
                 x0: np.ndarray | None = None):
    """Deform::optimize (Deform.cpp:95-169) with an exact sparse solve of
    J^T J h = -J^T f standing in for SimplicialCholesky."""
    x = identity_x(pr.F) if x0 is None else x0.copy()
    energies, halvings = [], []
    it_done = 0
    f = residual(pr, x)
    for it in range(max_iters):
        J = jacobian(pr, x)
        A = (J.T @ J).tocsc()
        f = residual(pr, x)
        g = J.T @ (-f)
        h = spla.spsolve(A, g)
        normv = np.linalg.norm(x)
        old = float(f @ f)
        energies.append(old)
        alpha, nh = 1.0, 0
        while alpha > 1e-15:
            xt = x + h
            f1 = residual(pr, xt)
            if float(f1 @ f1) > old:
                h = h * 0.5
                nh += 1
            else:
                x = xt
                break
            alpha *= 0.5
        halvings.append(nh)
        it_done = it + 1
        if early_exit and np.linalg.norm(h) < (normv + 1e-6) * 1e-6:
            break
    f = residual(pr, x)
    return x, GNStats(it_done, energies, halvings, float(f @ f))


def gradient(pr: EDProblem, x: np.ndarray) -> np.ndarray:
    """J^T f, the gradient of 0.5*|f|^2 as the reference's Jacobian states it."""
    return jacobian(pr, x).T @ residual(pr, x)


def put_free_inputs(pr: EDProblem, x: np.ndarray):
    """Deform.hpp:140-151 plus resetRT for the non-free nodes: rot [n,9]
    column-major, trans [n,3] (float64)."""
    rot = np.zeros((pr.n, 9), F64)
    rot[:, 0] = rot[:, 4] = rot[:, 8] = 1.0
    trans = np.zeros((pr.n, 3), F64)
    X = x.reshape(pr.F, 12)
    rot[pr.free] = X[:, :9]
    trans[pr.free] = X[:, 9:]
    return rot, trans


def ed_blend(points: np.ndarray, idx: np.ndarray, w: np.ndarray, rot: np.ndarray,
             trans: np.ndarray, node_pos: np.ndarray, float_accumulate: bool = True) -> np.ndarray:
    """predict_mesh (Deform.hpp:230-249): w_j (R_j (p - g_j) + t_j + g_j)
    evaluated in float64.  With ``float_accumulate`` the sum is rounded to
    float32 after every neighbour, as the reference's float ``output(c) +=``
    does; without it the float64 sum is rounded once (the exact blend)."""
    p = np.asarray(points, F32)
    g = np.asarray(node_pos, F32)
    out = np.zeros(p.shape, F64)
    for j in range(idx.shape[1]):
        nj = idx[:, j]
        temp = (p - g[nj]).astype(F64)               # float32 difference
        R = rot[nj]
        moved = (R[:, 0:3] * temp[:, 0:1] + R[:, 3:6] * temp[:, 1:2]
                 + R[:, 6:9] * temp[:, 2:3]) + trans[nj] + g[nj].astype(F64)
        out = out + w[:, j:j + 1] * moved
        if float_accumulate:
            out = out.astype(F32).astype(F64)
    return out.astype(F32)
