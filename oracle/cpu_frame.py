"""ctypes wrapper of the C++/OpenMP CPU baseline (oracle/cpu_frame.cpp).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): the timed CPU
baseline of bench.py and a second oracle for the tests.  ``build()`` compiles
the library with g++ and OpenMP into ``oracle/_build/``; nothing here touches
a GPU.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cpu_frame.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libarap_cpu_frame.so")
FLAGS = ["-std=c++17", "-O3", "-fopenmp", "-fPIC", "-shared"]


def build(force: bool = False) -> str:
    """Compile the baseline (portable flags: no -march, no intrinsics)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    tmp = LIB + ".tmp"
    r = subprocess.run([cxx, *FLAGS, SRC, "-o", tmp], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("g++ failed for cpu_frame.cpp:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


class SolveStats(C.Structure):
    _fields_ = [("gn_iterations", C.c_int), ("halvings", C.c_int), ("status", C.c_int), ("n_free", C.c_int),
                ("n_rows", C.c_longlong), ("nnz_j", C.c_longlong), ("nnz_l_blocks", C.c_longlong),
                ("factor_gflop", C.c_double), ("top_columns", C.c_int), ("subtrees", C.c_int),
                ("initial_energy", C.c_double), ("final_energy", C.c_double),
                ("t_setup", C.c_double), ("t_analyse", C.c_double), ("t_jacobian", C.c_double),
                ("t_normal", C.c_double), ("t_factor", C.c_double), ("t_solve", C.c_double),
                ("t_line", C.c_double), ("t_total", C.c_double),
                ("t_phase1", C.c_double), ("t_phase2", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_lib = None
P = C.c_void_p


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(build())
        I, LL, F = C.c_int, C.c_longlong, C.c_float
        lib.ocpu_solve.restype = I
        lib.ocpu_solve.argtypes = [I, I, P, P, P, P, P, I, P, P, P, I, F, F, F, F, I, I, I, I, P, P,
                                   C.POINTER(SolveStats)]
        lib.ocpu_ed_blend.restype = None
        lib.ocpu_ed_blend.argtypes = [LL, I, P, P, P, P, P, P, P, P, I]
        lib.ocpu_skin_gaussians.restype = None
        lib.ocpu_skin_gaussians.argtypes = [LL, I, P, P, P, P, P, P, P, P, P, P, P, P, I]
        lib.ocpu_skin_samples.restype = None
        lib.ocpu_skin_samples.argtypes = [LL, I, I, P, P, P, P, P, P, P, I]
        lib.ocpu_knn_weights.restype = None
        lib.ocpu_knn_weights.argtypes = [LL, P, I, P, I, P, P, I]
        lib.ocpu_max_threads.restype = I
        lib.ocpu_max_threads.argtypes = []
        _lib = lib
    return _lib


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def max_threads() -> int:
    return load().ocpu_max_threads()


def solve(node_pos, neighbors, anchor_idx, anchor_w, blocks, block_type, aims, cons_on_center=False,
          weighting_factor=1.0, w_rot=1.0, w_reg=10.0, w_con=100.0, max_iters=30, early_exit=False,
          threads=0, ordering=0):
    """Deform::optimize restated in C++ (FP64, direct block Cholesky;
    ordering 1 = geometric nested dissection, 0 = minimum degree).
    Returns (rot [n,9] column-major float64, trans [n,3] float64, stats dict)."""
    lib = load()
    node_pos = _c(node_pos, np.float32)
    n = node_pos.shape[0]
    nb = _c(neighbors, np.int32)
    k = nb.shape[1]
    ai = _c(anchor_idx, np.int32)
    aw = _c(anchor_w, np.float64)
    aims = _c(aims, np.float32)
    bptr = np.zeros(len(blocks) + 1, np.int32)
    for i, b in enumerate(blocks):
        bptr[i + 1] = bptr[i] + len(b)
    bids = _c(np.concatenate([np.asarray(b, np.int64) for b in blocks]) if blocks else np.zeros(0), np.int32)
    bt = _c(block_type, np.int32)
    rot = np.empty((n, 9), np.float64)
    tr = np.empty((n, 3), np.float64)
    st = SolveStats()
    lib.ocpu_solve(n, k, _ptr(node_pos), _ptr(nb), _ptr(ai), _ptr(aw), _ptr(aims), len(blocks), _ptr(bptr),
                   _ptr(bids), _ptr(bt), int(bool(cons_on_center)), float(weighting_factor), float(w_rot),
                   float(w_reg), float(w_con), int(max_iters), int(bool(early_exit)), int(threads), int(ordering),
                   _ptr(rot), _ptr(tr), C.byref(st))
    return rot, tr, st.as_dict()


def knn_weights(points, nodes, k, threads=0):
    """(idx int32 [P,k], w float64 [P,k]) by brute force (Deform.hpp:187-208)."""
    lib = load()
    points = _c(points, np.float32)
    nodes = _c(nodes, np.float32)
    Pn = points.shape[0]
    idx = np.empty((Pn, k), np.int32)
    w = np.empty((Pn, k), np.float64)
    lib.ocpu_knn_weights(Pn, _ptr(points), nodes.shape[0], _ptr(nodes), int(k), _ptr(idx), _ptr(w), int(threads))
    return idx, w


def ed_blend(points, idx, w, rot, trans, node_pos, threads=0):
    lib = load()
    points = _c(points, np.float32)
    idx = _c(idx, np.int32)
    w64 = _c(w, np.float64) if np.asarray(w).dtype == np.float64 else None
    w32 = None if w64 is not None else _c(w, np.float32)
    out = np.empty_like(points)
    lib.ocpu_ed_blend(points.shape[0], idx.shape[1], _ptr(points), _ptr(idx), _ptr(w64), _ptr(w32),
                      _ptr(_c(rot, np.float64)), _ptr(_c(trans, np.float64)), _ptr(_c(node_pos, np.float32)),
                      _ptr(out), int(threads))
    return out


class Frame:
    """Buffers of one CPU frame's skinning (all host numpy, float32 weights
    as the library stores them)."""

    def __init__(self, ends, ends_idx, ends_w, node_pos, rot, scale, shs, sample_pos=None, sample_idx=None,
                 sample_w=None, feature=None):
        N = ends.shape[0]
        self.k = int(ends_idx.shape[-1])
        self.ends = _c(ends, np.float32).reshape(N, 6, 3)
        self.ends_idx = _c(ends_idx, np.int32).reshape(N, 6, self.k)
        self.ends_w = _c(ends_w, np.float32).reshape(N, 6, self.k)
        self.node_pos = _c(node_pos, np.float32)
        self.scale0 = _c(scale, np.float32)
        self.q = _c(rot, np.float32).copy()
        self.shs = _c(shs, np.float32).copy()
        self.pos = np.empty((N, 3), np.float32)
        self.scale = np.empty((N, 3), np.float32)
        self.cov6 = np.empty((N, 6), np.float32)
        self.sample_pos = None if sample_pos is None else _c(sample_pos, np.float32).copy()
        self.sample_idx = None if sample_idx is None else _c(sample_idx, np.int32)
        self.sample_w = None if sample_w is None else _c(sample_w, np.float32)
        self.feature = None if feature is None else _c(feature, np.float32).copy()

    def skin_gaussians(self, rot, trans, threads=0):
        lib = load()
        N = self.ends.shape[0]
        lib.ocpu_skin_gaussians(N, self.k, _ptr(self.ends), _ptr(self.ends_idx), _ptr(self.ends_w),
                                _ptr(_c(rot, np.float64)), _ptr(_c(trans, np.float64)), _ptr(self.node_pos),
                                _ptr(self.scale0), _ptr(self.pos), _ptr(self.q), _ptr(self.scale),
                                _ptr(self.shs), _ptr(self.cov6), int(threads))

    def skin_samples(self, rot, trans, threads=0):
        lib = load()
        S = self.sample_pos.shape[0]
        lib.ocpu_skin_samples(S, self.sample_idx.shape[1], self.node_pos.shape[0], _ptr(self.sample_pos),
                              _ptr(self.sample_idx), _ptr(self.sample_w), _ptr(_c(rot, np.float64)),
                              _ptr(_c(trans, np.float64)), _ptr(self.node_pos), _ptr(self.feature), int(threads))


# ------------------------------------------------------- timed frame ----

def occupied_cell_samples(pos, rot, scale, opacity, grid_num, padding=1):
    """The grid's occupied cells (ascending) and their 64 samples each, as
    oracle/grid.py defines them, with the per-cell Gaussian counts formed by
    a 3D difference array instead of explicit lists (only occupancy is
    needed here)."""
    from . import grid as og
    g = grid_num
    mn, mx = og.overall_aabb(pos)
    step = og.grid_step(mn, mx, g)
    lo, hi = og.gaussian_aabbs(pos, rot, scale, opacity)
    a, b = og.cell_ranges(lo, hi, mn, step, g, padding)
    D = np.zeros((g + 1, g + 1, g + 1), np.int64)
    b1 = b + 1
    for cx in (0, 1):
        for cy in (0, 1):
            for cz in (0, 1):
                sgn = -1 if (cx + cy + cz) % 2 else 1
                ix = np.where(cx, b1[:, 0], a[:, 0])
                iy = np.where(cy, b1[:, 1], a[:, 1])
                iz = np.where(cz, b1[:, 2], a[:, 2])
                np.add.at(D, (ix, iy, iz), sgn)
    cnt = D.cumsum(0).cumsum(1).cumsum(2)[:g, :g, :g].reshape(-1)
    off = np.zeros(g ** 3 + 1, np.int64)
    off[1:] = np.cumsum(cnt)
    return og.grid_samples(off, mn, step, g)


class FrameBaseline:
    """One deformation frame of a synthetic scene on the host cores: the
    Gauss-Newton solve (early exit off), sample skinning (position and SH
    feature), Gaussian skinning (6 endpoints, refit, SH, covariance) and the
    node update, in the viewer's order (GaussianView.cpp:1481-1522).  The
    set-up (graph, kNN weights of endpoints, samples and node vertices,
    samples) is done once in the constructor; ``run`` restores the rest
    state, then times one frame."""

    def __init__(self, sc, threads=0, feature_seed=5, with_samples=True):
        from . import ed, grid as og, skin, targets
        self.threads = int(threads) or max_threads()
        self.sc = sc
        # the viewer orders Gaussians by the grid cell of their centre
        # (GaussianView.cpp:3918-3953); node ids follow
        mn, mx = og.overall_aabb(sc.pos)
        step = og.grid_step(mn, mx, sc.grid_num)
        _, new_index = og.center_cells(sc.pos, mn, step, sc.grid_num)
        order = np.empty_like(new_index)
        order[new_index] = np.arange(new_index.size)
        pos, rot, scale = sc.pos[order], sc.rot[order], sc.scale[order]
        shs = sc.shs[order]
        k = sc.k
        self.node_pos = np.ascontiguousarray(sc.node_pos, np.float32)
        self.nb = ed.build_graph(self.node_pos, k).astype(np.int32)
        self.aidx, self.aw = knn_weights(self.node_pos, self.node_pos, k, self.threads)
        act = np.concatenate([b for b, t in zip(sc.blocks, sc.block_type) if t == 1]).astype(np.int64)
        aims = self.node_pos.copy()
        if sc.op[0] == "translate":
            aims = targets.translate(aims, act, sc.op[1])
        elif sc.op[0] == "twist":
            aims = targets.twist(aims, self.node_pos, act, sc.op[1], sc.op[2])
        else:
            aims = targets.scale(aims, self.node_pos, act, sc.op[1])
        self.aims = np.ascontiguousarray(aims, np.float32)
        E = skin.end_points(pos, rot, scale)
        eidx, ew = knn_weights(E.reshape(-1, 3), self.node_pos, k, self.threads)
        sample_pos = sidx = sw = feature = None
        if with_samples:
            opacity = sc.opacity[order]
            _, sample_pos = occupied_cell_samples(pos, rot, scale, opacity, sc.grid_num)
            sidx, sw = knn_weights(sample_pos, self.node_pos, k, self.threads)
            sw = sw.astype(np.float32)
            rng = np.random.default_rng(feature_seed)
            feature = (0.2 * rng.standard_normal((sample_pos.shape[0], 48))).astype(np.float32)
        self.rest = Frame(E, eidx, ew.astype(np.float32), self.node_pos, rot, scale, shs,
                          sample_pos=sample_pos, sample_idx=sidx, sample_w=sw, feature=feature)
        self.n_samples = 0 if sample_pos is None else int(sample_pos.shape[0])
        self.last = None

    def run(self):
        """Restore the rest state, then time one frame; returns
        (ms_total, parts dict in ms, solve stats)."""
        import copy
        import time
        fr = copy.copy(self.rest)
        fr.ends = self.rest.ends.copy()
        fr.q = self.rest.q.copy()
        fr.shs = self.rest.shs.copy()
        if self.rest.sample_pos is not None:
            fr.sample_pos = self.rest.sample_pos.copy()
            fr.feature = self.rest.feature.copy()
        sc = self.sc
        t0 = time.perf_counter()
        rot, tr, st = solve(self.node_pos, self.nb, self.aidx, self.aw, sc.blocks, sc.block_type, self.aims,
                            max_iters=sc.iters, early_exit=False, threads=self.threads)
        t1 = time.perf_counter()
        if fr.sample_pos is not None:
            fr.skin_samples(rot, tr, self.threads)
        t2 = time.perf_counter()
        fr.skin_gaussians(rot, tr, self.threads)
        t3 = time.perf_counter()
        nodes = ed_blend(self.node_pos, self.aidx, self.aw, rot, tr, self.node_pos, self.threads)
        t4 = time.perf_counter()
        self.last = (fr, rot, tr, nodes)
        parts = {"solve": 1e3 * (t1 - t0), "skin_samples": 1e3 * (t2 - t1), "skin_gaussians": 1e3 * (t3 - t2),
                 "update_nodes": 1e3 * (t4 - t3)}
        return 1e3 * (t4 - t0), parts, st
