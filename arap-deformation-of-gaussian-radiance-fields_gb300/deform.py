"""Host-side interface over the C ABI, mirroring the reference's deformation API.

The reference exposes the hot path as in-process C++ (no plugin ABI):

* ``DeformGraph(nodes, knn_k)`` builds the node graph (Deform.hpp:54-95) and
  ``computeWeights`` the kNN skinning weights (Deform.hpp:187-208);
* ``Deform(...)`` + ``real_time_deform()`` solves for node transforms
  (Deform.hpp:414-455, Deform.cpp:77-169) and ``putFreeInputs`` scatters them
  (Deform.hpp:140-151);
* ``GaussianView::UpdatePositionforSamples / UpdatePosition /
  UpdateAsSixPointsWithdrawBad / FastUpdateSamplesSH`` skin samples, endpoints,
  nodes and Gaussians (GaussianView.cpp:2986-3186).

Here each of those is a thin call into ``libarap_gb300.so``; torch tensors are
only device memory and streams.  Every call raises ``ArapError`` on a
non-OK status; nothing falls back to a CPU path.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from ._lib import ArapError, SolveConfig, SolveStats, check  # noqa: F401

__all__ = ["build_graph", "compute_weights", "Solver", "node_table", "end_points",
           "skin_gaussians", "skin_gaussians_backward", "node_quaternions", "skin_samples", "update_nodes",
           "static_mask", "aims_translate", "aims_twist", "aims_scale", "device_status", "StatusWord",
           "default_config", "GaussianDeformer"]


def _lib_():
    return _lib.load()


def _p(t):
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return C.c_void_p(t.data_ptr())


def _s():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _f32(t):
    return t.to(device="cuda", dtype=torch.float32).contiguous()


def _i32(t):
    return t.to(device="cuda", dtype=torch.int32).contiguous()


class StatusWord:
    """A device status word (int32) of the caller's, for the stateless calls
    that can raise a device-side error (arap_compute_weights,
    arap_skin_gaussians, arap_skin_gaussians_backward, arap_node_quaternions):
    the first ARAP_* code raised into it wins until ``read`` clears it."""

    def __init__(self):
        self.t = torch.zeros(1, dtype=torch.int32, device="cuda")

    def ptr(self):
        return _p(self.t)

    def read(self) -> int:
        """Read and clear (synchronises the current stream)."""
        return _lib_().arap_status_read(_p(self.t), _s())


_default_words = {}


def _status(status):
    """The word a stateless call records into: the caller's, or this
    process's default word of the current device (read by device_status)."""
    if status is not None:
        return status.ptr()
    dev = torch.cuda.current_device()
    w = _default_words.get(dev)
    if w is None:
        w = _default_words[dev] = StatusWord()
    return w.ptr()


def device_status() -> int:
    """Read and clear the default status word of the current device: the
    first device-side error of the stateless calls made without their own
    StatusWord (handles keep their own words: Solver.status, SkinPlan.status,
    Grid.status)."""
    dev = torch.cuda.current_device()
    w = _default_words.get(dev)
    return w.read() if w is not None else 0


def default_config(**kw) -> SolveConfig:
    cfg = SolveConfig()
    _lib_().arap_solve_config_default(C.byref(cfg))
    for k, v in kw.items():
        if not hasattr(cfg, k):
            raise KeyError(k)
        setattr(cfg, k, v)
    return cfg


# ----------------------------------------------------------------- kNN ----

def build_graph(nodes: torch.Tensor, k: int) -> torch.Tensor:
    """Node graph [n,k] int32: each node's k nearest other nodes
    (DeformGraph::setupEdges, Deform.hpp:84-95)."""
    nodes = _f32(nodes)
    n = nodes.shape[0]
    out = torch.empty((n, k), dtype=torch.int32, device="cuda")
    check("arap_build_graph", _lib_().arap_build_graph(_p(nodes), n, k, _p(out), _s()))
    return out


def compute_weights(points: torch.Tensor, nodes: torch.Tensor, k: int, status=None, threads: int = 0):
    """kNN skinning weights (DeformGraph::computeWeights, Deform.hpp:187-208).
    Returns (idx [k,P] int32, w [k,P] float32) in planes layout.  threads:
    the kernel's CTA size (0: the default; see knn_autotune)."""
    points = _f32(points)
    nodes = _f32(nodes)
    P = points.shape[0]
    idx = torch.empty((k, P), dtype=torch.int32, device="cuda")
    w = torch.empty((k, P), dtype=torch.float32, device="cuda")
    check("arap_compute_weights_ex", _lib_().arap_compute_weights_ex(
        _p(points), P, _p(nodes), nodes.shape[0], k, int(threads), _p(idx), _p(w), _status(status), _s()))
    return idx, w


def knn_autotune(points: torch.Tensor, nodes: torch.Tensor, k: int):
    """The fastest CTA size of the kNN kernel for these points and nodes
    (arap_knn_autotune): (threads, {threads: ms})."""
    points = _f32(points)
    nodes = _f32(nodes)
    t = C.c_int()
    ms = (C.c_float * 3)()
    check("arap_knn_autotune", _lib_().arap_knn_autotune(
        _p(points), points.shape[0], _p(nodes), nodes.shape[0], k, C.byref(t), C.cast(ms, C.c_void_p), _s()))
    return t.value, dict(zip((128, 256, 512), list(ms)))


# --------------------------------------------------------------- solver ----

class Solver:
    """One control-region configuration of the ED / ARAP solve
    (``Deform``, Deform.hpp:379-472).

    neighbors [n,k] int32 (graph), anchor_idx/anchor_w [k,n] (kNN of each node's
    own vertex, ``cand_vertices[Vertex_index]``), blocks: list of node-id
    sequences (``indices_blocks``), block_type: 1 active / 0 pinned /
    -1 excluded."""

    def __init__(self, neighbors, anchor_idx, anchor_w, blocks, block_type, config=None, **kw):
        lib = _lib_()
        self.neighbors = _i32(neighbors)
        self.anchor_idx = _i32(anchor_idx)
        self.anchor_w = _f32(anchor_w)
        n, k = self.neighbors.shape
        self.n, self.k = n, k
        cfg = config if config is not None else default_config(**kw)
        self.config = cfg
        offs = [0]
        flat = []
        for b in blocks:
            flat.extend(int(v) for v in b)
            offs.append(len(flat))
        types = [int(t) for t in block_type]
        nb = len(types)
        arr_i = C.c_int32 * max(1, len(offs))
        o_arr = arr_i(*offs)
        f_arr = (C.c_int32 * max(1, len(flat)))(*flat)
        t_arr = (C.c_int32 * max(1, nb))(*types)
        h = C.c_void_p()
        check("arap_solver_create", lib.arap_solver_create(
            C.byref(h), n, k, _p(self.neighbors), _p(self.anchor_idx), _p(self.anchor_w),
            C.cast(o_arr, C.c_void_p), C.cast(f_arr, C.c_void_p), C.cast(t_arr, C.c_void_p),
            nb, C.byref(cfg), _s()))
        self._h = h
        self.F = lib.arap_solver_free_count(h)
        ids = (C.c_int32 * self.F)()
        check("arap_solver_free_ids", lib.arap_solver_free_ids(h, C.cast(ids, C.c_void_p)))
        self.free_ids = torch.tensor(list(ids), dtype=torch.int64)

    def solve(self, node_pos, aims, rot_out=None, trans_out=None, stats=True):
        """Deform::real_time_deform + putFreeInputs: rot [n,9] column-major,
        trans [n,3].  With ``stats`` the stream is synchronised and the
        solve statistics are returned."""
        node_pos = _f32(node_pos)
        aims = _f32(aims)
        if rot_out is None:
            rot_out = torch.empty((self.n, 9), dtype=torch.float32, device="cuda")
        if trans_out is None:
            trans_out = torch.empty((self.n, 3), dtype=torch.float32, device="cuda")
        st = SolveStats() if stats else None
        code = _lib_().arap_solver_solve(self._h, _p(node_pos), _p(aims), _p(rot_out), _p(trans_out),
                                         C.byref(st) if st is not None else None, _s())
        check("arap_solver_solve", code)
        return rot_out, trans_out, (st.as_dict() if st is not None else None)

    def status(self) -> int:
        """Read and clear the solver's device status word (synchronises)."""
        return _lib_().arap_solver_status(self._h, _s())

    def energy_grad(self, node_pos, aims, x):
        """(J^T f at x [F*12] float64, f.f) -- the gradient of 0.5|f|^2 as the
        reference's Jacobian states it."""
        x = x.to(device="cuda", dtype=torch.float64).contiguous()
        g = torch.empty_like(x)
        e = C.c_double()
        check("arap_solver_energy_grad", _lib_().arap_solver_energy_grad(
            self._h, _p(_f32(node_pos)), _p(_f32(aims)), _p(x), _p(g), C.byref(e), _s()))
        return g, e.value

    def close(self):
        if getattr(self, "_h", None):
            _lib_().arap_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # interpreter shutdown
            pass


# ------------------------------------------------------------ skinning ----

class SolverBatch:
    """Several Solvers (one precision) solved together (arap_solver_batch_*):
    one cooperative launch per wave of instances, the grid's CTAs split among
    each wave's instances."""

    def __init__(self, solvers, balance_exponent=1.0):
        self.solvers = list(solvers)
        n = len(self.solvers)
        hs = (C.c_void_p * n)(*[s._h.value for s in self.solvers])
        h = C.c_void_p()
        check("arap_solver_batch_create", _lib_().arap_solver_batch_create(
            C.byref(h), C.cast(hs, C.c_void_p), n, float(balance_exponent), _s()))
        self._h = h

    def _ptrs(self, tensors):
        return (C.c_void_p * len(tensors))(*[t.data_ptr() for t in tensors])

    def _outputs(self, rot_out, trans_out):
        if rot_out is None:
            rot_out = [torch.empty((s.n, 9), dtype=torch.float32, device="cuda") for s in self.solvers]
        if trans_out is None:
            trans_out = [torch.empty((s.n, 3), dtype=torch.float32, device="cuda") for s in self.solvers]
        return rot_out, trans_out

    def solve(self, node_pos, aims, rot_out=None, trans_out=None, stats=True):
        """Lists of per-instance inputs and outputs; with ``stats`` the stream is
        synchronised and the per-instance statistics are returned."""
        node_pos = [_f32(x) for x in node_pos]
        aims = [_f32(x) for x in aims]
        rot_out, trans_out = self._outputs(rot_out, trans_out)
        self._keep = (node_pos, aims, rot_out, trans_out)  # pointers stay valid while queued
        n = len(self.solvers)
        st = (SolveStats * n)() if stats else None
        code = _lib_().arap_solver_batch_solve(
            self._h, C.cast(self._ptrs(node_pos), C.c_void_p), C.cast(self._ptrs(aims), C.c_void_p),
            C.cast(self._ptrs(rot_out), C.c_void_p), C.cast(self._ptrs(trans_out), C.c_void_p),
            C.cast(st, C.c_void_p) if st is not None else None, _s())
        check("arap_solver_batch_solve", code)
        return rot_out, trans_out, ([x.as_dict() for x in st] if st is not None else None)

    def autotune(self, node_pos, aims):
        node_pos = [_f32(x) for x in node_pos]
        aims = [_f32(x) for x in aims]
        rot_out, trans_out = self._outputs(None, None)
        best = C.c_float()
        check("arap_solver_batch_autotune", _lib_().arap_solver_batch_autotune(
            self._h, C.cast(self._ptrs(node_pos), C.c_void_p), C.cast(self._ptrs(aims), C.c_void_p),
            C.cast(self._ptrs(rot_out), C.c_void_p), C.cast(self._ptrs(trans_out), C.c_void_p), C.byref(best), _s()))
        return best.value

    def ctas(self):
        out = (C.c_int32 * (len(self.solvers) + 1))()
        check("arap_solver_batch_ctas", _lib_().arap_solver_batch_ctas(self._h, C.cast(out, C.c_void_p)))
        return list(out)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib_().arap_solver_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def node_table(rot, trans, node_pos):
    n = rot.shape[0]
    out = torch.empty((n, 16), dtype=torch.float32, device="cuda")
    check("arap_node_table", _lib_().arap_node_table(n, _p(rot), _p(trans), _p(_f32(node_pos)), _p(out), _s()))
    return out


def end_points(pos, rot, scale, with_xyz=True):
    """GetEndPoints: ends [18,N] planes and (optionally) [6N,3] endpoint-major."""
    pos, rot, scale = _f32(pos), _f32(rot), _f32(scale)
    N = pos.shape[0]
    ends = torch.empty((18, N), dtype=torch.float32, device="cuda")
    xyz = torch.empty((6 * N, 3), dtype=torch.float32, device="cuda") if with_xyz else None
    check("arap_end_points", _lib_().arap_end_points(N, _p(pos), _p(rot), _p(scale), _p(ends), _p(xyz), _s()))
    return ends, xyz


def skin_gaussians(ends, ends_idx, ends_w, table, scale0, pos_out, rot_inout, scale_out,
                   shs=None, cov_out=None, static=None, precision=_lib.PRECISION_PLAIN, status=None):
    N = pos_out.shape[0]
    k = ends_idx.shape[0]
    check("arap_skin_gaussians", _lib_().arap_skin_gaussians(
        N, k, _p(ends), _p(ends_idx), _p(ends_w), _p(table), _p(scale0), _p(static), _p(pos_out),
        _p(rot_inout), _p(scale_out), _p(shs), _p(cov_out), int(precision), _status(status), _s()))


class SkinPlan:
    """Set-up-time layout of the endpoint kNN for skin_gaussians_planned
    (arap_skin_plan_*): per tile of 128 Gaussians its distinct nodes and
    8-bit slot indices of its staged node records (chosen to spread shared-
    memory banks) and its weights, one contiguous block per tile."""

    def __init__(self, ends_idx, ends_w):
        self.k, self.N = int(ends_idx.shape[0]), int(ends_idx.shape[1]) // 6
        self.ends_idx, self.ends_w = ends_idx, ends_w
        h = C.c_void_p()
        check("arap_skin_plan_create", _lib_().arap_skin_plan_create(
            C.byref(h), self.N, self.k, _p(ends_idx), _p(ends_w), _s()))
        self._h = h

    def info(self):
        t, o, m = C.c_int(), C.c_int(), C.c_int()
        check("arap_skin_plan_info", _lib_().arap_skin_plan_info(self._h, C.byref(t), C.byref(o), C.byref(m)))
        return {"tiles": t.value, "overflow_tiles": o.value, "max_nodes": m.value}

    def status(self) -> int:
        """Read and clear the plan's device status word (synchronises)."""
        return _lib_().arap_skin_plan_status(self._h, _s())

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib_().arap_skin_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def skin_gaussians_planned(plan, ends, table, scale0, pos_out, rot_inout, scale_out, shs=None, cov_out=None,
                           static=None, precision=_lib.PRECISION_PLAIN):
    check("arap_skin_gaussians_planned", _lib_().arap_skin_gaussians_planned(
        plan._h, _p(ends), _p(plan.ends_idx), _p(plan.ends_w), _p(table), _p(scale0), _p(static), _p(pos_out),
        _p(rot_inout), _p(scale_out), _p(shs), _p(cov_out), int(precision), _s()))


def skin_gaussians_backward(ends_in, ends_idx, ends_w, table, scale0, grad_pos, grad_cov, n, static=None,
                            grad_node=None, status=None):
    """Adjoint of skin_gaussians' (mu, Sigma) w.r.t. the node transforms:
    returns grad_node [n,12] ([dR column-major 9 | dt 3])."""
    N = grad_pos.shape[0]
    k = ends_idx.shape[0]
    if grad_node is None:
        grad_node = torch.zeros((n, 12), dtype=torch.float32, device="cuda")
    check("arap_skin_gaussians_backward", _lib_().arap_skin_gaussians_backward(
        N, k, _p(ends_in), _p(ends_idx), _p(ends_w), _p(table), _p(scale0), _p(static), _p(grad_pos),
        _p(grad_cov), _p(grad_node), _status(status), _s()))
    return grad_node


def skin_gaussians_backward_planned(plan, ends_in, table, scale0, grad_pos, grad_cov, n, static=None,
                                    grad_node=None):
    """skin_gaussians_backward with the skinning plan of the same endpoints
    (arap_skin_gaussians_backward_planned); errors go to the plan's word."""
    if grad_node is None:
        grad_node = torch.zeros((n, 12), dtype=torch.float32, device="cuda")
    check("arap_skin_gaussians_backward_planned", _lib_().arap_skin_gaussians_backward_planned(
        plan._h, _p(ends_in), _p(plan.ends_idx), _p(plan.ends_w), _p(table), _p(scale0), _p(static),
        _p(grad_pos), _p(grad_cov), _p(grad_node), _s()))
    return grad_node


def node_quaternions(rot, precision=_lib.PRECISION_PLAIN, status=None):
    n = rot.shape[0]
    out = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    check("arap_node_quaternions", _lib_().arap_node_quaternions(n, _p(rot), _p(out), int(precision),
                                                                 _status(status), _s()))
    return out


def skin_samples(sample_pos, idx, w, table, quat=None, feature=None, static=None):
    S = sample_pos.shape[0]
    k = idx.shape[0]
    check("arap_skin_samples", _lib_().arap_skin_samples(
        S, k, _p(sample_pos), _p(idx), _p(w), _p(table), _p(quat), _p(feature), _p(static), _s()))


def update_nodes(node_pos, anchor_idx, anchor_w, table, out=None):
    n = node_pos.shape[0]
    k = anchor_idx.shape[0]
    if out is None:
        out = torch.empty_like(node_pos)
    check("arap_update_nodes", _lib_().arap_update_nodes(
        n, k, _p(node_pos), _p(anchor_idx), _p(anchor_w), _p(table), _p(out), _s()))
    return out


def static_mask(idx, node_is_static, P):
    """Items (P of them) whose every neighbour in the planes of ``idx``
    ([planes, P] int32) is a static node (CheckStaticSamples,
    GaussianView.cpp:2038-2070).  uint8 [P]."""
    planes = idx.numel() // P
    out = torch.empty((P,), dtype=torch.uint8, device="cuda")
    check("arap_static_mask", _lib_().arap_static_mask(P, planes, 1, _p(idx), _p(node_is_static), _p(out), _s()))
    return out


def aims_translate(aims, active, delta):
    check("arap_aims_translate", _lib_().arap_aims_translate(
        _p(aims), _p(active), active.numel(), float(delta[0]), float(delta[1]), float(delta[2]), _s()))


def aims_twist(aims, node_pos, active, axis, radian):
    check("arap_aims_twist", _lib_().arap_aims_twist(
        _p(aims), _p(node_pos), _p(active), active.numel(), float(axis[0]), float(axis[1]),
        float(axis[2]), float(radian), _s()))


def aims_scale(aims, node_pos, active, s):
    check("arap_aims_scale", _lib_().arap_aims_scale(
        _p(aims), _p(node_pos), _p(active), active.numel(), float(s), _s()))


# ------------------------------------------------------- frame pipeline ----

class GaussianDeformer:
    """Device-resident state of one deformable Gaussian field and its
    per-frame update, in the reference's order (GaussianView.cpp:1481-1522):
    solve, sample skinning (before nodes move), endpoint + node update,
    Gaussian refit with SH, node-quaternion SH rotation of the samples, aims
    re-anchored to the nodes."""

    def __init__(self, pos, rot, scale, shs, node_vertex, k, blocks, block_type,
                 sample_pos=None, feature=None, config=None, use_plan=True, **cfg_kw):
        dev = "cuda"
        self.word = StatusWord()   # device errors of this field's stateless calls
        self.k = int(k)
        self.pos = _f32(pos)
        self.rot = _f32(rot)
        self.scale = _f32(scale)
        self.scale0 = self.scale.clone()
        self.shs = _f32(shs) if shs is not None else None
        N = self.pos.shape[0]
        self.N = N
        nv = torch.as_tensor(node_vertex, dtype=torch.int64, device=dev)
        self.node_pos = self.pos[nv].contiguous()
        self.n = self.node_pos.shape[0]
        self.neighbors = build_graph(self.node_pos, self.k)
        gidx, gw = compute_weights(self.pos, self.node_pos, self.k, status=self.word)
        self.anchor_idx = gidx[:, nv].contiguous()
        self.anchor_w = gw[:, nv].contiguous()
        self.ends, ends_xyz = end_points(self.pos, self.rot, self.scale)
        # the kNN kernel's CTA size, tuned on the largest of its inputs here
        self.knn_threads, self.knn_tuning = knn_autotune(ends_xyz, self.node_pos, self.k)
        self.ends_idx, self.ends_w = compute_weights(ends_xyz, self.node_pos, self.k, status=self.word,
                                                     threads=self.knn_threads)
        del ends_xyz
        self.skin_plan = SkinPlan(self.ends_idx, self.ends_w) if use_plan else None
        self.sample_pos = _f32(sample_pos) if sample_pos is not None else None
        self.feature = _f32(feature) if feature is not None else None
        if self.sample_pos is not None:
            self.sample_idx, self.sample_w = compute_weights(self.sample_pos, self.node_pos, self.k,
                                                             status=self.word, threads=self.knn_threads)
        self.blocks = [torch.as_tensor(b, dtype=torch.int64) for b in blocks]
        self.block_type = [int(t) for t in block_type]
        node_static = torch.zeros(self.n, dtype=torch.uint8, device=dev)
        for b, t in zip(self.blocks, self.block_type):
            if t < 0:
                node_static[b.to(dev)] = 1
        self.node_static = node_static
        self.g_static = static_mask(self.ends_idx, node_static, N) if bool(node_static.any()) else None
        self.s_static = static_mask(self.sample_idx, node_static, self.sample_pos.shape[0]) \
            if (self.sample_pos is not None and bool(node_static.any())) else None
        self.solver = Solver(self.neighbors, self.anchor_idx, self.anchor_w, self.blocks,
                             self.block_type, config=config, **cfg_kw)
        self._cfg = (config, dict(cfg_kw))
        self.precision = self.solver.config.precision
        act = [int(v) for b, t in zip(self.blocks, self.block_type) if t == 1 for v in b]
        self.active = torch.tensor(act, dtype=torch.int32, device=dev)
        self.aims = self.node_pos.clone()
        self.rot_nodes = torch.empty((self.n, 9), dtype=torch.float32, device=dev)
        self.trans_nodes = torch.empty((self.n, 3), dtype=torch.float32, device=dev)
        self.node_pos_next = torch.empty_like(self.node_pos)
        self.cov = torch.empty((N, 6), dtype=torch.float32, device=dev)

    def _controls_key(self):
        return (tuple(tuple(int(v) for v in b.tolist()) for b in self.blocks),
                tuple(self.block_type), bool(self.solver.config.cons_on_center))

    def set_controls(self, blocks, block_type, constraints_on_center=None):
        """Replace the control blocks between frames, and optionally the
        constraint mode, as the viewer's UpdateIndicies and fresh ``Deform``
        do before a frame (GaussianView.cpp:1996-2021, 1822, 1855).  The solver
        of each configuration is created once and kept."""
        centre = bool(self.solver.config.cons_on_center) if constraints_on_center is None \
            else bool(constraints_on_center)
        key = (tuple(tuple(int(v) for v in b) for b in blocks), tuple(int(t) for t in block_type), centre)
        if len(key[0]) != len(key[1]):
            raise ValueError("set_controls: %d blocks, %d block types" % (len(key[0]), len(key[1])))
        current = self._controls_key()
        if key == current:
            return
        cache = self.__dict__.setdefault("_solvers", {})
        cache.setdefault(current, self.solver)
        solver = cache.get(key)
        if solver is None:
            config, cfg_kw = self._cfg
            cfg = SolveConfig.from_buffer_copy(config) if config is not None else default_config(**cfg_kw)
            cfg.cons_on_center = int(centre)
            solver = Solver(self.neighbors, self.anchor_idx, self.anchor_w, key[0], key[1], config=cfg)
            cache[key] = solver
        self.solver = solver
        self.blocks = [torch.as_tensor(b, dtype=torch.int64) for b in key[0]]
        self.block_type = list(key[1])
        node_static = torch.zeros(self.n, dtype=torch.uint8, device="cuda")
        for b, t in zip(self.blocks, self.block_type):
            if t < 0 and b.numel():
                node_static[b.to("cuda")] = 1
        self.node_static = node_static
        any_static = bool(node_static.any())
        self.g_static = static_mask(self.ends_idx, node_static, self.N) if any_static else None
        self.s_static = static_mask(self.sample_idx, node_static, self.sample_pos.shape[0]) \
            if (self.sample_pos is not None and any_static) else None
        act = [v for b, t in zip(key[0], key[1]) if t == 1 for v in b]
        self.active = torch.tensor(act, dtype=torch.int32, device="cuda")

    def apply_op(self, op):
        """Move the active targets (UpdateAimPosition / Twist / Scale)."""
        kind = op[0]
        if self.active.numel() == 0:
            return
        if kind == "translate":
            aims_translate(self.aims, self.active, op[1])
        elif kind == "twist":
            aims_twist(self.aims, self.node_pos, self.active, op[1], op[2])
        elif kind == "scale":
            aims_scale(self.aims, self.node_pos, self.active, op[1])
        else:
            raise ValueError(kind)

    def frame(self, stats=False, with_cov=True, skin_events=None, sample_events=None):
        rot, trans, st = self.solver.solve(self.node_pos, self.aims, self.rot_nodes, self.trans_nodes, stats=stats)
        table = node_table(rot, trans, self.node_pos)
        if self.sample_pos is not None:
            quat = node_quaternions(rot, self.precision, status=self.word) if self.feature is not None else None
            if sample_events is not None:
                sample_events[0].record()
            skin_samples(self.sample_pos, self.sample_idx, self.sample_w, table, quat, self.feature, self.s_static)
            if sample_events is not None:
                sample_events[1].record()
        if skin_events is not None:
            skin_events[0].record()
        if self.skin_plan is not None:
            skin_gaussians_planned(self.skin_plan, self.ends, table, self.scale0, self.pos, self.rot, self.scale,
                                   self.shs, self.cov if with_cov else None, self.g_static, self.precision)
        else:
            skin_gaussians(self.ends, self.ends_idx, self.ends_w, table, self.scale0, self.pos, self.rot,
                           self.scale, self.shs, self.cov if with_cov else None, self.g_static, self.precision,
                           status=self.word)
        if skin_events is not None:
            skin_events[1].record()
        update_nodes(self.node_pos, self.anchor_idx, self.anchor_w, table, self.node_pos_next)
        self.node_pos, self.node_pos_next = self.node_pos_next, self.node_pos
        self.aims.copy_(self.node_pos)
        return st

    def status(self) -> int:
        """Read and clear the device status words of this field: its solver's,
        its skinning plan's and its own (stateless calls); the first error
        found, else ARAP_OK (synchronises)."""
        codes = [self.solver.status(), self.skin_plan.status() if self.skin_plan is not None else 0,
                 self.word.read()]
        return next((c for c in codes if c), 0)
