"""Seeded synthetic Gaussian fields, deformation graphs and control regions.

The reference viewer loads a trained 3DGS PLY (GaussianView.cpp:43-339) and
samples its deformation nodes with farthest-point sampling over the Gaussian
centres (helper.cpp:139-177, GaussianView.cpp:706-719).  No PLY ships with the
reference, so these generators build fields with the published shape of the
workloads instead:

* ``bend50k``   -- 50k Gaussians in a bar [0,1]x[0,0.2]x[0,0.2], 32^3 grid,
  ~1k nodes, k=8, pinned x<0.1, active x>0.9 translated by (0,0.3,0),
  10 Gauss-Newton iterations.
* ``twist300k`` -- 300k Gaussians in [0,1]^3 (two bars and a sphere), 64^3 grid,
  ~4k nodes, k=8, pinned z<0.1, active z>0.9 twisted 90 degrees about z,
  20 iterations.
* ``stress3m``  -- 3M flat Gaussians in [0,4]^3 (one log-scale axis N(-9,0.3)),
  128^3 grid, ~30k nodes, k=12, pinned / excluded / active(x1.5 scale),
  30 iterations.
* ``stress200k`` -- the stress field at 200k Gaussians and ~8000 nodes
  (64^3 grid, 8 iterations): more free nodes than the solver keeps resident
  in shared memory, so it exercises the non-resident solve.

Every Gaussian attribute is activated the way the viewer stores it after
loading (GaussianView.cpp:140-151): scales are exp(log-scale), opacities are
sigmoid(logit), quaternions are unit (w, x, y, z), SH are 16x3 interleaved
``[coef*3 + rgb]``.

Nodes are picked by voxel downsampling: for each occupied voxel the Gaussian
nearest the voxel's member centroid becomes a node, so every node sits on a
Gaussian (its ``node_vertex``) exactly like the reference's FPS nodes
(``Node::Vertex_index``, helper.hpp:136-144).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

__all__ = ["Scene", "Instance", "make_scene", "build_scene", "batch_instances", "SCENES"]


@dataclasses.dataclass
class Scene:
    name: str
    pos: np.ndarray        # float32 [N,3]
    rot: np.ndarray        # float32 [N,4] (w,x,y,z), unit
    scale: np.ndarray      # float32 [N,3], activated
    opacity: np.ndarray    # float32 [N], activated
    shs: np.ndarray        # float32 [N,48], interleaved [coef*3+rgb]
    grid_num: int
    node_vertex: np.ndarray  # int32 [n] Gaussian index each node sits on
    node_pos: np.ndarray     # float32 [n,3]
    k: int
    blocks: list             # list of int32 arrays of node ids (block order)
    block_type: np.ndarray   # int32 [nb]: 1 active, 0 pinned, -1 excluded
    op: tuple                # ("translate", (dx,dy,dz)) | ("twist", (ax,ay,az), radian) | ("scale", s)
    iters: int

    @property
    def n_gauss(self) -> int:
        return int(self.pos.shape[0])

    @property
    def n_nodes(self) -> int:
        return int(self.node_pos.shape[0])


def _unit_quats(rng, n):
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return q.astype(np.float32)


def _sample_bar(rng, n, lo, hi):
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    return lo + rng.random((n, 3)) * (hi - lo)


def _sample_ball(rng, n, c, r):
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rad = r * rng.random(n) ** (1.0 / 3.0)
    return np.asarray(c, np.float64) + d * rad[:, None]


def voxel_nodes(pos: np.ndarray, target: int) -> np.ndarray:
    """Return the Gaussian indices chosen as nodes (about ``target`` of them).

    The voxel edge is bisected until the number of occupied voxels is within
    2% of ``target``; in each voxel the member nearest the members' centroid
    (ties: lowest index) is kept.  Output is sorted by voxel key.
    """
    p = pos.astype(np.float64)
    lo = p.min(axis=0)
    ext = float((p.max(axis=0) - lo).max())
    a, b = ext / 2000.0, ext

    def occupied(h):
        key = np.floor((p - lo) / h).astype(np.int64)
        m = int(key.max()) + 1
        flat = (key[:, 0] * m + key[:, 1]) * m + key[:, 2]
        return flat

    h = None
    for _ in range(60):
        mid = math.sqrt(a * b)
        cnt = np.unique(occupied(mid)).size
        h = mid
        if abs(cnt - target) <= 0.02 * target:
            break
        if cnt > target:
            a = mid
        else:
            b = mid
    flat = occupied(h)
    order = np.argsort(flat, kind="stable")
    fs = flat[order]
    starts = np.flatnonzero(np.r_[True, fs[1:] != fs[:-1]])
    ends = np.r_[starts[1:], fs.size]
    sums = np.add.reduceat(p[order], starts, axis=0)
    cnts = (ends - starts)[:, None]
    cent = sums / cnts
    seg = np.repeat(np.arange(starts.size), ends - starts)
    d2 = ((p[order] - cent[seg]) ** 2).sum(axis=1)
    # lexicographic (segment, d2, index) minimum per segment
    sel = np.lexsort((order, d2, seg))
    first = np.r_[True, seg[sel][1:] != seg[sel][:-1]]
    return order[sel][first].astype(np.int32)


def build_scene(name, pos, logscale_mu, logscale_sigma, grid_num, n_nodes, k,
                region_fn, op, iters, seed):
    rng = np.random.default_rng(seed + 1)
    n = pos.shape[0]
    pos = pos.astype(np.float32)
    mu = np.broadcast_to(np.asarray(logscale_mu, np.float64), (3,))
    sg = np.broadcast_to(np.asarray(logscale_sigma, np.float64), (3,))
    scale = np.exp(mu + sg * rng.standard_normal((n, 3))).astype(np.float32)
    rot = _unit_quats(rng, n)
    opacity = (1.0 / (1.0 + np.exp(-rng.standard_normal(n)))).astype(np.float32)
    shs = (0.2 * rng.standard_normal((n, 48))).astype(np.float32)
    node_vertex = voxel_nodes(pos, n_nodes)
    node_pos = pos[node_vertex].copy()
    blocks, types = region_fn(node_pos)
    return Scene(name=name, pos=pos, rot=rot, scale=scale, opacity=opacity,
                 shs=shs, grid_num=grid_num, node_vertex=node_vertex,
                 node_pos=node_pos, k=k, blocks=blocks,
                 block_type=np.asarray(types, np.int32), op=op, iters=iters)


def _regions(*specs):
    """specs: (predicate(node_pos)->mask, type) in block order."""
    def fn(node_pos):
        blocks, types = [], []
        for pred, t in specs:
            ids = np.flatnonzero(pred(node_pos)).astype(np.int32)
            if ids.size:
                blocks.append(ids)
                types.append(t)
        return blocks, types
    return fn


def _bend(n, seed, n_nodes=1000, grid_num=32, k=8, iters=10):
    rng = np.random.default_rng(seed)
    pos = _sample_bar(rng, n, (0, 0, 0), (1, 0.2, 0.2))
    reg = _regions((lambda p: p[:, 0] < 0.1, 0), (lambda p: p[:, 0] > 0.9, 1))
    return build_scene("bend%dk" % (n // 1000), pos, -5.0, 0.5, grid_num,
                       n_nodes, k, reg, ("translate", (0.0, 0.3, 0.0)), iters, seed)


def _two_bars_sphere(rng, n, s=1.0):
    n1 = n // 3
    n2 = n // 3
    n3 = n - n1 - n2
    a = _sample_bar(rng, n1, (0.15 * s, 0.15 * s, 0.0), (0.35 * s, 0.35 * s, 1.0 * s))
    b = _sample_bar(rng, n2, (0.65 * s, 0.65 * s, 0.0), (0.85 * s, 0.85 * s, 1.0 * s))
    c = _sample_ball(rng, n3, (0.5 * s, 0.5 * s, 0.5 * s), 0.2 * s)
    pos = np.concatenate([a, b, c])
    return pos[rng.permutation(n)]


def _twist(n, seed, n_nodes=4000, grid_num=64, k=8, iters=20):
    rng = np.random.default_rng(seed)
    pos = _two_bars_sphere(rng, n)
    reg = _regions((lambda p: p[:, 2] < 0.1, 0), (lambda p: p[:, 2] > 0.9, 1))
    return build_scene("twist%dk" % (n // 1000), pos, -5.0, 0.5, grid_num,
                       n_nodes, k, reg, ("twist", (0.0, 0.0, 1.0), math.pi / 2),
                       iters, seed)


def _stress(n, seed, n_nodes=30000, grid_num=128, k=12, iters=30):
    rng = np.random.default_rng(seed)
    pos = _two_bars_sphere(rng, n, 4.0)
    reg = _regions((lambda p: p[:, 2] < 0.4, 0),
                   (lambda p: (p[:, 2] > 1.2) & (p[:, 2] < 1.6) & (p[:, 0] < 2.0), -1),
                   (lambda p: p[:, 2] > 3.6, 1))
    return build_scene("stress%dk" % (n // 1000), pos, (-9.0, -4.0, -4.0),
                       (0.3, 0.5, 0.5), grid_num, n_nodes, k, reg,
                       ("scale", 1.5), iters, seed)


@dataclasses.dataclass
class Instance:
    """One deformation instance of a batch: nodes, graph degree, control
    regions and operation; with ``gaussians`` also its Gaussian field (the
    nodes sit on Gaussians, ``node_vertex``)."""
    node_pos: np.ndarray     # float32 [n,3]
    k: int
    blocks: list
    block_type: np.ndarray
    op: tuple
    iters: int
    pos: np.ndarray = None       # float32 [N,3]
    rot: np.ndarray = None       # float32 [N,4] (w,x,y,z)
    scale: np.ndarray = None     # float32 [N,3]
    shs: np.ndarray = None       # float32 [N,48]
    node_vertex: np.ndarray = None


def batch_instances(count: int = 64, seed: int = 0, nodes=(300, 8000), k: int = 8, iters: int = 20,
                    gaussians=None):
    """``count`` instances with node counts log-uniform in ``nodes``: random
    unions of bars and balls under a random scale and rotation, pinned below
    10% and active above 90% of a random axis, and an operation drawn from
    bend (translate), twist (90 degrees about the axis) and scale x U[0.5, 2].
    With ``gaussians = (lo, hi)`` every instance also gets a Gaussian field of
    a count log-uniform in [lo, hi] over the same shape (the bend workload's
    distributions: log-scale N(-5, 0.5) shifted by the instance's scale,
    uniform unit quaternions, SH N(0, 0.2)), and its nodes are picked among
    those Gaussians."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n_nodes = int(round(math.exp(rng.uniform(math.log(nodes[0]), math.log(nodes[1])))))
        npts = 12 * n_nodes
        if gaussians is not None:
            npts = max(npts, int(round(math.exp(rng.uniform(math.log(gaussians[0]), math.log(gaussians[1]))))))
        parts = []
        for _ in range(int(rng.integers(1, 4))):
            if rng.random() < 0.5:
                lo = rng.uniform(0.0, 0.5, 3)
                parts.append(_sample_bar(rng, npts, lo, lo + rng.uniform(0.15, 0.5, 3)))
            else:
                parts.append(_sample_ball(rng, npts, rng.uniform(0.3, 0.7, 3), rng.uniform(0.1, 0.3)))
        pts = np.concatenate(parts)[rng.permutation(npts * len(parts))[:npts]]
        q = _unit_quats(rng, 1)[0].astype(np.float64)
        w, x, y, z = q
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                      [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                      [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
        size = rng.uniform(0.5, 2.0)
        pts = ((pts @ R.T) * size).astype(np.float32)
        node_vertex = voxel_nodes(pts, n_nodes)
        node_pos = pts[node_vertex].astype(np.float32)
        axis = int(rng.integers(0, 3))
        c = node_pos[:, axis]
        lo, hi = np.quantile(c, 0.1), np.quantile(c, 0.9)
        blocks = [np.flatnonzero(c < lo).astype(np.int32), np.flatnonzero(c > hi).astype(np.int32)]
        kind = int(rng.integers(0, 3))
        ext = float(np.ptp(node_pos, axis=0).max())
        if kind == 0:
            d = np.zeros(3)
            d[(axis + 1) % 3] = 0.3 * ext
            op = ("translate", tuple(float(v) for v in d))
        elif kind == 1:
            a = np.zeros(3)
            a[axis] = 1.0
            op = ("twist", tuple(float(v) for v in a), math.pi / 2)
        else:
            op = ("scale", float(rng.uniform(0.5, 2.0)))
        inst = Instance(node_pos=node_pos, k=k, blocks=blocks, block_type=np.array([0, 1], np.int32), op=op,
                        iters=iters)
        if gaussians is not None:
            n = pts.shape[0]
            inst.pos = pts
            inst.rot = _unit_quats(rng, n)
            inst.scale = np.exp(-5.0 + math.log(size) + 0.5 * rng.standard_normal((n, 3))).astype(np.float32)
            inst.shs = (0.2 * rng.standard_normal((n, 48))).astype(np.float32)
            inst.node_vertex = node_vertex.astype(np.int32)
        out.append(inst)
    return out


SCENES = {
    "bend50k": lambda seed=0: _bend(50_000, seed),
    "twist300k": lambda seed=0: _twist(300_000, seed),
    "stress3m": lambda seed=0: _stress(3_000_000, seed),
    # small cases for parity tests
    "bend4k": lambda seed=0: _bend(4_000, seed, n_nodes=120, grid_num=16, iters=6),
    "twist20k": lambda seed=0: _twist(20_000, seed, n_nodes=400, grid_num=32, iters=8),
    "stress40k": lambda seed=0: _stress(40_000, seed, n_nodes=600, grid_num=32, iters=8),
    # more free nodes than the solver keeps resident in shared memory
    "stress200k": lambda seed=0: _stress(200_000, seed, n_nodes=8000, grid_num=64, iters=8),
}


def make_scene(name: str, seed: int = 0) -> Scene:
    if name not in SCENES:
        raise KeyError("unknown scene %r (have %s)" % (name, sorted(SCENES)))
    return SCENES[name](seed)
