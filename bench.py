"""Benchmark: deform ms/frame on the 300k-Gaussian / 64^3 twist workload.

One step = one deformation frame through the library, in the reference's
order (GaussianView.cpp:1481-1522): 20-iteration Gauss-Newton solve of the
node transforms (early exit off), skinning of the grid samples (position +
slerp-blended SH rotation of the 48-float features), skinning of all Gaussians
(6-endpoint ED blend, refit, SH rotation, covariance), node update and target
re-anchoring.  Every step starts from the same rest state (restored by device
copies before the step's timed region, then L2 is flushed) so each step does
identical work.

--impl ours       the CUDA library (default)
--impl reference  the reference's CPU path on the host cores, restated in
                  C++/OpenMP float64 (oracle/cpu_frame.cpp; the reference
                  itself needs Eigen/SIBR and cannot be built here), one full
                  frame per step

Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
PKG = "arap-deformation-of-gaussian-radiance-fields_gb300"
METRIC = "deform ms/frame, 300k Gaussians 64³ grid: mixed+adjoint vs plain GPU @≤1e-5"


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scene", default="twist300k")
    ap.add_argument("--form", default="chosen", choices=["plain", "chosen"],
                    help="chosen: float-float residual/gradient (FP64 iterate and sums) + two-level PCG; plain: FP32 + block-Jacobi PCG")
    ap.add_argument("--coarse-nodes", type=int, default=64)
    ap.add_argument("--other-forms", default="plain,plain2l",
                    help="forms also timed on the same state (comma list of plain, plain2l, chosen; "
                         "plain2l: FP32 residual/gradient with the two-level PCG); empty: none")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-samples", action="store_true")
    ap.add_argument("--batch", type=int, default=64,
                    help="instances of the batched-solve leg (0: skip it)")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.rows.append([v.strip() for v in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=6)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = sorted(float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit())
        mx = max((float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if len(r) > 2 + i and r[2 + i].strip() == "Active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(self.rows)}


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def reduce_max(value, ws, device="cuda"):
    """The slowest replica's value (a step ends when every GPU's replica has
    finished it).  Replicas only: this is the one cross-rank operation."""
    if ws <= 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------ workload ----

def op_text(op):
    """The control operation of a scene in words."""
    if op[0] == "twist":
        return "twist %.0f deg about (%g, %g, %g)" % ((op[2] * 180.0 / 3.141592653589793,) + tuple(op[1]))
    if op[0] == "scale":
        return "scale x%g" % op[1]
    return "translate by (%g, %g, %g)" % tuple(op[1])


def solve_config(dev, sc, form, coarse_nodes):
    """chosen: float-float residual, gradient and energy (FP64 iterate and
    grid-wide sums) with the two-level PCG;
    plain: FP32 with block-Jacobi alone (the straightforward port); plain2l:
    FP32 with the two-level PCG (what the precision choices add on their
    own)."""
    if form == "chosen":
        return dev.default_config(max_iters=sc.iters, early_exit=0, precision=1, coarse_nodes=coarse_nodes)
    if form == "plain2l":
        return dev.default_config(max_iters=sc.iters, early_exit=0, precision=0, coarse_nodes=coarse_nodes)
    return dev.default_config(max_iters=sc.iters, early_exit=0, precision=0, coarse_nodes=0)


def build_state(scene_name, form, coarse_nodes, with_samples):
    import numpy as np
    import torch
    dev = importlib.import_module(PKG + ".deform")
    synth = importlib.import_module(PKG + ".synth")
    grid = importlib.import_module(PKG + ".grid")
    sc = synth.make_scene(scene_name)
    # the reference reorders the Gaussians by the grid cell of their centre
    # before binning (GaussianView.cpp:3918-3953); node ids follow
    g0 = grid.build_grid(torch.as_tensor(sc.pos).cuda(), torch.as_tensor(sc.rot).cuda(),
                         torch.as_tensor(sc.scale).cuda(), torch.as_tensor(sc.opacity).cuda(), sc.grid_num)
    order = g0.center_order().cpu().numpy()
    g0.close()
    inv = np.empty_like(order)
    inv[order] = np.arange(order.size)
    sc.pos, sc.rot, sc.scale, sc.opacity, sc.shs = (a[order] for a in (sc.pos, sc.rot, sc.scale, sc.opacity, sc.shs))
    sc.node_vertex = inv[sc.node_vertex].astype(np.int32)
    sample_pos = feature = None
    if with_samples:
        g = grid.build_grid(torch.as_tensor(sc.pos).cuda(), torch.as_tensor(sc.rot).cuda(),
                            torch.as_tensor(sc.scale).cuda(), torch.as_tensor(sc.opacity).cuda(), sc.grid_num)
        sample_pos = g.sample_pos
        rng = np.random.default_rng(5)
        feature = torch.as_tensor((0.2 * rng.standard_normal((sample_pos.shape[0], 48))).astype(np.float32)).cuda()
    cfg = solve_config(dev, sc, form, coarse_nodes)
    st = dev.GaussianDeformer(torch.as_tensor(sc.pos), torch.as_tensor(sc.rot), torch.as_tensor(sc.scale),
                              torch.as_tensor(sc.shs), sc.node_vertex, sc.k, sc.blocks, sc.block_type,
                              sample_pos=sample_pos, feature=feature, config=cfg)
    st.apply_op(sc.op)
    torch.cuda.synchronize()
    return sc, st


def snapshot(st):
    names = ["ends", "pos", "rot", "scale", "shs", "node_pos", "aims", "sample_pos", "feature"]
    return {n: getattr(st, n).clone() for n in names if getattr(st, n, None) is not None}


def restore(st, snap):
    for n, t in snap.items():
        getattr(st, n).copy_(t)


# DRAM bytes per launch measured by ncu on the named workload
# (dram__bytes_read.sum + dram__bytes_write.sum of one launch inside the
# bench's frame), keyed by (scene, k, planned) for the Gaussian skinning and
# (scene, k) for the sample skinning.
SKIN_DRAM_BYTES = {("twist300k", 8, True): 162642432 + 44834560}
SAMPLES_DRAM_BYTES = {("twist300k", 8): 413555456 + 252287488}


def samples_roofline(st, k, ms, peak, peak_kind, traffic=None):
    """The frame's sample skinning launch (arap_skin_samples): per sample
    position read + write (24), k indices and k weights (8k), the 48-float
    feature read + write (384)."""
    if ms is None:
        return None
    S = int(st.sample_pos.shape[0])
    per = 24 + 8 * k + (384 if st.feature is not None else 0)
    gbs = per * S / (ms * 1e-3) / 1e9
    return {"kernel": "arap_skin_samples", "bound": "hbm", "samples": S, "bytes_per_sample": per,
            "bytes_per_launch": per * S, "ms_per_launch": round(ms, 5), "achieved": round(gbs, 1),
            "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": round(gbs / peak, 4),
            "traffic": traffic, "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch "
            "(profiles/skin_samples_twist300k.md)" if traffic else None}


def skin_bytes_per_gaussian(k, with_shs=True, with_cov=True, planned=True):
    """Algorithmic bytes of Gaussian skinning per Gaussian: read 6 endpoints
    (72), 6k neighbour indices (1 byte each with the skinning plan, else 4) and
    6k weights (24k), scale0 (12), previous q (16), SH (192); write endpoints
    (72), mu (12), q (16), scale (12), SH (192), Sigma (24).  The plan's node
    lists (a few hundred bytes per 128-Gaussian tile) are not counted."""
    rd = 72 + 6 * k * (1 if planned else 4) + 24 * k + 12 + 16 + (192 if with_shs else 0)
    wr = 72 + 12 + 16 + 12 + (192 if with_shs else 0) + (24 if with_cov else 0)
    return rd + wr


def batch_leg(count):
    """Batched solves: ``count`` instances (node counts log-uniform in
    [300, 8000], random shapes and operations, 20 Gauss-Newton iterations,
    chosen form) in one cooperative launch, against the same instances solved
    one after another."""
    import numpy as np
    import torch
    dev = importlib.import_module(PKG + ".deform")
    synth = importlib.import_module(PKG + ".synth")
    inst = synth.batch_instances(count)
    solvers, pos, aims = [], [], []
    for it in inst:
        p = torch.as_tensor(it.node_pos).cuda()
        nb = dev.build_graph(p, it.k)
        aidx, aw = dev.compute_weights(p, p, it.k)
        act = torch.as_tensor(it.blocks[1].astype(np.int32)).cuda()
        a = p.clone()
        if it.op[0] == "translate":
            dev.aims_translate(a, act, it.op[1])
        elif it.op[0] == "twist":
            dev.aims_twist(a, p, act, it.op[1], it.op[2])
        else:
            dev.aims_scale(a, p, act, it.op[1])
        solvers.append(dev.Solver(nb, aidx, aw, it.blocks, it.block_type, max_iters=it.iters, early_exit=0,
                                  precision=1, coarse_nodes=64))
        pos.append(p)
        aims.append(a)
    batch = dev.SolverBatch(solvers)
    best = batch.autotune(pos, aims)
    rot = [torch.empty((s.n, 9), device="cuda") for s in solvers]
    tr = [torch.empty((s.n, 3), device="cuda") for s in solvers]

    def timed(fn, reps):
        out = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            out.append(e0.elapsed_time(e1))
        return float(np.median(out))

    batch.solve(pos, aims, rot, tr, stats=False)
    ms_b = timed(lambda: batch.solve(pos, aims, rot, tr, stats=False), 3)
    _, _, st_b = batch.solve(pos, aims, rot, tr, stats=True)

    def seq():
        for s_, p_, a_, r_, t_ in zip(solvers, pos, aims, rot, tr):
            s_.solve(p_, a_, r_, t_, stats=False)
    seq()
    ms_s = timed(seq, 1)
    out = {"instances": count, "nodes_total": int(sum(s_.n for s_ in solvers)),
           "nodes_range": [int(min(s_.n for s_ in solvers)), int(max(s_.n for s_ in solvers))],
           "gn_iterations": inst[0].iters, "form": "chosen (mixed, coarse 64)",
           "ms_batched": round(ms_b, 3), "ms_sequential": round(ms_s, 3),
           "instances_per_s_batched": round(1000.0 * count / ms_b, 1),
           "batched_speedup_over_sequential": round(ms_s / ms_b, 3),
           "balance_exponent": best, "status": max(x["status"] for x in st_b)}
    batch.close()
    for s_ in solvers:
        s_.close()
    return out


def batch_frame_leg(count):
    """Batched frames with Gaussians: ``count`` instances (node counts
    log-uniform in [300, 8000], Gaussian counts log-uniform in [20k, 500k],
    random shapes and operations, 20 Gauss-Newton iterations, chosen form).
    One batched frame = the batched solve (cooperative launches in waves,
    CTA split by the autotuner) writing every instance's transforms into one
    node table, then ONE skinning launch over all instances' Gaussians (their
    endpoint kNN indices offset into the joint table, a skinning plan over the
    concatenation).  Timed directly, as a replayed CUDA graph of the same
    frame, and against the instances' frames run one after another."""
    import numpy as np
    import torch
    dev = importlib.import_module(PKG + ".deform")
    synth = importlib.import_module(PKG + ".synth")
    inst = synth.batch_instances(count, gaussians=(20_000, 500_000))
    solvers, pos, aims, seq = [], [], [], []
    node_base, gauss_base = [0], [0]
    ends_all, idx_all, w_all, s0_all, q_all, sh_all = [], [], [], [], [], []
    for it in inst:
        p = torch.as_tensor(it.node_pos).cuda()
        nb = dev.build_graph(p, it.k)
        aidx, aw = dev.compute_weights(p, p, it.k)
        act = torch.as_tensor(it.blocks[1].astype(np.int32)).cuda()
        a0 = p.clone()
        if it.op[0] == "translate":
            dev.aims_translate(a0, act, it.op[1])
        elif it.op[0] == "twist":
            dev.aims_twist(a0, p, act, it.op[1], it.op[2])
        else:
            dev.aims_scale(a0, p, act, it.op[1])
        solvers.append(dev.Solver(nb, aidx, aw, it.blocks, it.block_type, max_iters=it.iters, early_exit=0,
                                  precision=1, coarse_nodes=64))
        pos.append(p)
        aims.append(a0)
        gp = torch.as_tensor(it.pos).cuda()
        ends, exyz = dev.end_points(gp, torch.as_tensor(it.rot).cuda(), torch.as_tensor(it.scale).cuda())
        eidx, ew = dev.compute_weights(exyz, p, it.k)
        del exyz
        seq.append((ends, eidx, ew, dev.SkinPlan(eidx, ew)))
        ends_all.append(ends)
        # planes [k][6][N_i]: joined along the Gaussians of each (k, endpoint) plane
        n_i = it.pos.shape[0]
        idx_all.append((eidx + node_base[-1]).view(it.k, 6, n_i))
        w_all.append(ew.view(it.k, 6, n_i))
        s0_all.append(torch.as_tensor(it.scale).cuda())
        q_all.append(torch.as_tensor(it.rot).cuda())
        sh_all.append(torch.as_tensor(it.shs).cuda())
        node_base.append(node_base[-1] + p.shape[0])
        gauss_base.append(gauss_base[-1] + it.pos.shape[0])
    n_tot, N_tot = node_base[-1], gauss_base[-1]
    # joint buffers: per-instance solve outputs are views of one table source
    rot_all = torch.empty((n_tot, 9), device="cuda")
    tr_all = torch.empty((n_tot, 3), device="cuda")
    node_all = torch.cat(pos).contiguous()
    rot_v = [rot_all[node_base[i]:node_base[i + 1]] for i in range(count)]
    tr_v = [tr_all[node_base[i]:node_base[i + 1]] for i in range(count)]
    ends0 = torch.cat(ends_all, 1).contiguous()     # [18][N_tot]
    k = inst[0].k
    eidx_all = torch.cat(idx_all, 2).reshape(k, 6 * N_tot).contiguous()
    ew_all = torch.cat(w_all, 2).reshape(k, 6 * N_tot).contiguous()
    s0 = torch.cat(s0_all).contiguous()
    q0 = torch.cat(q_all).contiguous()
    sh0 = torch.cat(sh_all).contiguous()
    plan = dev.SkinPlan(eidx_all, ew_all)
    batch = dev.SolverBatch(solvers)
    best = batch.autotune(pos, aims)
    ends = ends0.clone()
    gpos = torch.empty((N_tot, 3), device="cuda")
    q = q0.clone()
    gsc = torch.empty((N_tot, 3), device="cuda")
    sh = sh0.clone()
    cov = torch.empty((N_tot, 6), device="cuda")

    def restore():
        ends.copy_(ends0)
        q.copy_(q0)
        sh.copy_(sh0)

    def frame():
        batch.solve(pos, aims, rot_v, tr_v, stats=False)
        table = dev.node_table(rot_all, tr_all, node_all)
        dev.skin_gaussians_planned(plan, ends, table, s0, gpos, q, gsc, sh, cov, precision=1)

    def frames_one_by_one():
        for i, (s_, (e_, ei_, ew_, pl_)) in enumerate(zip(solvers, seq)):
            a_, b_ = gauss_base[i], gauss_base[i + 1]
            r_, t_, _ = s_.solve(pos[i], aims[i], rot_v[i], tr_v[i], stats=False)
            tab = dev.node_table(r_, t_, pos[i])
            dev.skin_gaussians_planned(pl_, e_, tab, s0[a_:b_], gpos[a_:b_], q[a_:b_], gsc[a_:b_], sh[a_:b_],
                                       cov[a_:b_], precision=1)

    def timed(fn, reps):
        out = []
        for _ in range(reps):
            restore()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            out.append(e0.elapsed_time(e1))
        return float(np.median(out))

    frame()
    ms_b = timed(frame, 3)
    frames_one_by_one()
    ms_s = timed(frames_one_by_one, 2)
    # the batched frame captured once and replayed
    restore()
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        frame()   # warm the stream's allocations outside the capture
        torch.cuda.synchronize()
        with torch.cuda.graph(graph, stream=s):
            frame()
    torch.cuda.synchronize()
    ms_g = timed(graph.replay, 3)
    _, _, st_b = batch.solve(pos, aims, rot_v, tr_v, stats=True)
    out = {"instances": count, "gaussians_total": int(N_tot), "nodes_total": int(n_tot),
           "gaussians_range": [int(min(np.diff(gauss_base))), int(max(np.diff(gauss_base)))],
           "nodes_range": [int(min(np.diff(node_base))), int(max(np.diff(node_base)))],
           "gn_iterations": inst[0].iters, "form": "chosen (mixed, coarse 64)",
           "ms_batched_frame": round(ms_b, 3), "ms_batched_frame_graph_replay": round(ms_g, 3),
           "ms_frames_one_by_one": round(ms_s, 3),
           "batched_speedup_over_one_by_one": round(ms_s / ms_b, 3),
           "launches_per_batched_frame": "one cooperative solve launch per wave, one node table, one skinning",
           "balance_exponent": best, "status": max(x["status"] for x in st_b)}
    batch.close()
    plan.close()
    for s_ in solvers:
        s_.close()
    for t4 in seq:
        t4[3].close()
    return out


def _leg(fn, *args):
    """An extra block of the bench line; a failure is recorded in the block
    instead of ending the run (the frame measurement above is complete)."""
    try:
        return fn(*args)
    except Exception as e:  # noqa: BLE001
        return {"error": "%s: %s" % (type(e).__name__, e)}


def run_ours(a):
    import torch
    import numpy as np
    ws, rank = _dist()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    if ws > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
    dev = importlib.import_module(PKG + ".deform")
    sc, st = build_state(a.scene, a.form, a.coarse_nodes, not a.no_samples)
    snap = snapshot(st)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream()

    skin_ev, samp_ev = [], []

    def step(record):
        ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) if record else None
        sev = None
        if record and st.sample_pos is not None:
            sev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
        st.frame(stats=False, with_cov=True, skin_events=ev, sample_events=sev)
        if record:
            skin_ev.append(ev)
            if sev is not None:
                samp_ev.append(sev)

    for _ in range(max(3, a.warmup)):
        restore(st, snap)
        step(False)
    torch.cuda.synchronize()
    assert st.status() == 0
    step_ev = []
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with ClockSampler(torch.cuda.current_device()) as clk:
        for _ in range(a.steps):
            restore(st, snap)  # the rest state, outside the timed region
            flush.fill_(1.0)   # L2 flush between steps (256 MB > 129 MB L2)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(s)
            step(True)
            e1.record(s)
            step_ev.append((e0, e1))
        torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if ws > 1:
        torch.distributed.barrier()
    ms = [a0.elapsed_time(b0) for a0, b0 in step_ev]
    ms_step = reduce_max(float(np.mean(ms)), ws)
    skin_ms = float(np.mean([a0.elapsed_time(b0) for a0, b0 in skin_ev]))
    samp_ms = float(np.mean([a0.elapsed_time(b0) for a0, b0 in samp_ev])) if samp_ev else None
    status = st.status()

    # e2e: public API with host buffers (aims H2D, node transforms + energy D2H)
    aims_host = snap["aims"].cpu().pin_memory()
    rot_host = torch.empty((st.n, 9), dtype=torch.float32).pin_memory()
    tr_host = torch.empty((st.n, 3), dtype=torch.float32).pin_memory()
    e2e_ms = []
    for i in range(a.warmup + a.steps):
        restore(st, snap)
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        st.aims.copy_(aims_host, non_blocking=True)
        st.frame(stats=False, with_cov=True)
        rot_host.copy_(st.rot_nodes, non_blocking=True)
        tr_host.copy_(st.trans_nodes, non_blocking=True)
        torch.cuda.synchronize()
        if i >= a.warmup:
            e2e_ms.append((time.perf_counter() - t1) * 1e3)
    # stats of one frame (PCG iterations) for the record
    restore(st, snap)
    stats = st.frame(stats=True)
    torch.cuda.synchronize()
    # the other forms on the same state, same steps
    forms = {a.form: {"ms_per_frame": round(ms_step, 3), "pcg_iterations": stats["pcg_iterations"]}}
    main_solver, main_precision = st.solver, st.precision
    for other in [f for f in a.other_forms.split(",") if f and f != a.form]:
        st.solver = dev.Solver(st.neighbors, st.anchor_idx, st.anchor_w, st.blocks, st.block_type,
                               config=solve_config(dev, sc, other, a.coarse_nodes))
        st.precision = st.solver.config.precision
        for _ in range(2):
            restore(st, snap)
            st.frame(stats=False)
        o_ms = []
        for _ in range(max(2, a.steps // 2)):
            restore(st, snap)
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(s)
            st.frame(stats=False)
            e1.record(s)
            torch.cuda.synchronize()
            o_ms.append(e0.elapsed_time(e1))
        restore(st, snap)
        o_stats = st.frame(stats=True)
        torch.cuda.synchronize()
        forms[other] = {"ms_per_frame": round(float(np.mean(o_ms)), 3), "pcg_iterations": o_stats["pcg_iterations"]}
    st.solver, st.precision = main_solver, main_precision  # the adjoint block uses the benched form
    if "chosen" in forms and "plain" in forms:
        forms["chosen_speedup_over_plain"] = round(forms["plain"]["ms_per_frame"] / forms["chosen"]["ms_per_frame"], 3)
    if "chosen" in forms and "plain2l" in forms:
        forms["chosen_speedup_over_plain2l"] = round(forms["plain2l"]["ms_per_frame"] /
                                                     forms["chosen"]["ms_per_frame"], 3)

    peak, peak_kind = _peaks()
    k = sc.k
    bytes_launch = skin_bytes_per_gaussian(k, planned=st.skin_plan is not None) * sc.n_gauss
    achieved = bytes_launch / (skin_ms * 1e-3) / 1e9
    # the library's kernels per frame: the solve, the node table, the Gaussian
    # skinning and the node update, plus the sample skinning and the node
    # quaternions for the samples' features (the aims copy is a torch copy)
    launches_per_step = 4 + (1 if st.sample_pos is not None else 0) + (1 if st.feature is not None else 0)
    line = {
        "metric": METRIC,
        "value": round(ms_step, 4),
        "unit": "ms/frame",
        "n_gpus": ws,
        "steps": a.steps,
        "warmup": a.warmup,
        "ms_per_step": round(ms_step, 4),
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64" if a.form == "chosen" else "f32",
        "data": "synthetic (seeded two-bars-and-sphere field; reference datasets absent)",
        "config": {"workload": "%s: %d Gaussians, %d^3 grid, %d nodes, k=%d, %d GN iterations, "
                               "%s, form=%s" % (sc.name, sc.n_gauss, sc.grid_num, sc.n_nodes, k, sc.iters,
                                                op_text(sc.op), a.form),
                   "samples": int(st.sample_pos.shape[0]) if st.sample_pos is not None else 0,
                   "l2": "flushed between steps (256 MB write)",
                   "state": "restored to the rest pose before each step, outside the timed region",
                   "knn_threads": st.knn_threads,
                   "knn_autotune_ms": {str(t): round(v, 3) for t, v in st.knn_tuning.items()},
                   "wall_s_timed_region": round(wall, 3)},
        "e2e": {"value": round(reduce_max(float(np.mean(e2e_ms)), ws), 4), "unit": "ms/frame",
                "h2d_bytes_per_step": int(st.n * 12), "d2h_bytes_per_step": int(st.n * 48)},
        "roofline": {"kernel": "arap_skin_gaussians_planned" if st.skin_plan is not None else "arap_skin_gaussians",
                     "bound": "hbm", "achieved": round(achieved, 1),
                     "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": SKIN_DRAM_BYTES.get((sc.name, k, st.skin_plan is not None)),
                     "traffic_source": "ncu dram__bytes_read.sum + "
                     "dram__bytes_write.sum, one launch (profiles/skin_gaussians_twist300k.md)",
                     "bytes_per_launch": bytes_launch, "ms_per_launch": round(skin_ms, 5)},
        "roofline_samples": samples_roofline(st, k, samp_ms, peak, peak_kind,
                                             SAMPLES_DRAM_BYTES.get((sc.name, k))),
        "gpu_launches": launches_per_step * a.steps,
        "solve": {"bound": "latency (L2-resident persistent kernel; reported per PCG iteration)",
                  "pcg_iterations": stats["pcg_iterations"], "gn_iterations": stats["gn_iterations"],
                  "coarse_inversions": stats["coarse_inversions"],
                  "us_per_pcg_iteration": round(1000.0 * stats["phase_ms"]["pcg"] / max(1, stats["pcg_iterations"]), 2),
                  "phase_ms": {k: round(v, 3) for k, v in stats["phase_ms"].items()},
                  "final_energy": stats["final_energy"]},
        "forms": forms,
        "status": status,
        "clocks": clk.summary(),
    }
    if rank == 0 and a.batch > 0:
        line["batch"] = _leg(batch_leg, a.batch)
        line["batch_frames"] = _leg(batch_frame_leg, a.batch)
    if rank == 0:
        line["adjoint"] = _leg(adjoint_leg, st)
        line["ply_io"] = _leg(ply_leg, sc)
    if rank == 0 and not a.no_cpu_baseline:
        line["cpu_baseline"] = _leg(cpu_baseline, sc)
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()


def adjoint_leg(st, reps=10):
    """The forward/backward pair at the frame's scale: Gaussian skinning
    (arap_skin_gaussians), its adjoint (arap_skin_gaussians_backward: the
    node gradient of sum g_mu.mu + g_Sigma:Sigma for upstream gradients
    N(0,1) on every Gaussian's mu [N,3] and Sigma [N,6]) and the energy
    gradient (arap_solver_energy_grad: J^T f at the solved transforms), each
    timed with CUDA events (median of reps)."""
    import numpy as np
    import torch
    dev = importlib.import_module(PKG + ".deform")
    N, n = st.N, st.n
    rot, tr, _ = st.solver.solve(st.node_pos, st.aims, st.rot_nodes, st.trans_nodes, stats=False)
    table = dev.node_table(rot, tr, st.node_pos)
    gen = torch.Generator(device="cuda").manual_seed(3)
    g_mu = torch.randn((N, 3), device="cuda", generator=gen)
    g_cov = torch.randn((N, 6), device="cuda", generator=gen)
    grad = torch.zeros((n, 12), device="cuda")
    ends = st.ends.clone()
    pos = torch.empty((N, 3), device="cuda")
    q = st.rot.clone()
    sc = torch.empty((N, 3), device="cuda")
    cov = torch.empty((N, 6), device="cuda")
    F = st.solver.F
    free = st.solver.free_ids.to("cuda")
    x = torch.cat([rot, tr], 1)[free].to(torch.float64).reshape(-1).contiguous()

    def timed(fn):
        out = []
        for r in range(reps + 2):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            if r >= 2:
                out.append(e0.elapsed_time(e1))
        return float(np.median(out))

    def fwd():
        ends.copy_(st.ends)
        dev.skin_gaussians(ends, st.ends_idx, st.ends_w, table, st.scale0, pos, q, sc, None, cov,
                           precision=st.precision)

    def bwd_unplanned():
        grad.zero_()
        dev.skin_gaussians_backward(st.ends, st.ends_idx, st.ends_w, table, st.scale0, g_mu, g_cov, n,
                                    grad_node=grad)

    def bwd():
        grad.zero_()
        if st.skin_plan is not None:
            dev.skin_gaussians_backward_planned(st.skin_plan, st.ends, table, st.scale0, g_mu, g_cov, n,
                                                grad_node=grad)
        else:
            bwd_unplanned()

    ms_f = timed(fwd)
    ms_b = timed(bwd)
    ms_bu = timed(bwd_unplanned)
    ms_e = timed(lambda: st.solver.energy_grad(st.node_pos, st.aims, x))
    k = st.k
    bytes_b = N * (72 + 6 * k * 8 + 12 + 12 + 24)
    return {"gaussians": N, "nodes": n, "free_nodes": F, "precision": int(st.precision),
            "ms_skin_forward_with_cov": round(ms_f, 4), "ms_skin_backward": round(ms_b, 4),
            "ms_skin_backward_unplanned": round(ms_bu, 4),
            "ms_energy_grad": round(ms_e, 4),
            "backward_bytes_per_gaussian": 72 + 6 * k * 8 + 12 + 12 + 24,
            "backward_gbs": round(bytes_b / (ms_b * 1e-3) / 1e9, 1),
            "note": "backward (arap_skin_gaussians_backward_planned): the blend recomputed from the tile's staged "
                    "node records, each node's gradient summed over the plan's inverse reference lists, one "
                    "global atomic per (tile, node, component); the unplanned adjoint sums through a "
                    "shared-memory hash and atomics. Bytes per Gaussian as the unplanned reads them: endpoints, "
                    "int32 indices and float weights, scale0, upstream gradients"}


def ply_leg(sc, reps=3):
    """Host time of the 3DGS PLY round trip of the workload's Gaussians
    (arap_ply_save, then arap_ply_load with the viewer's Morton reorder),
    best of reps, through a temporary file."""
    import tempfile
    import numpy as np
    ply = importlib.import_module(PKG + ".ply")
    big = np.float32(3e38)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "scene.ply")
        t_save = t_load = float("inf")
        for _ in range(reps):
            t0 = time.perf_counter()
            ply.save_ply(path, sc.pos, sc.shs, sc.opacity, sc.scale, sc.rot, [-big] * 3, [big] * 3)
            t_save = min(t_save, time.perf_counter() - t0)
            t0 = time.perf_counter()
            out = ply.load_ply(path)
            t_load = min(t_load, time.perf_counter() - t0)
        mb = os.path.getsize(path) / 1e6
    assert out["pos"].shape[0] == sc.pos.shape[0]
    n = int(sc.pos.shape[0])
    # host threads of the load and the save encode: up to 16, one per 16k splats
    threads = min(os.cpu_count() or 1, 16, n // 16384 + 1)
    return {"splats": n, "file_mb": round(mb, 1), "save_ms": round(1e3 * t_save, 1),
            "load_ms": round(1e3 * t_load, 1), "load_mb_per_s": round(mb / t_load, 1), "threads": threads}


# ------------------------------------------------------- CPU baseline ----

def _cpu_frame(sc):
    """The C++/OpenMP FP64 restatement of the reference's CPU frame
    (oracle/cpu_frame.cpp), set up on all host threads."""
    from oracle import cpu_frame
    t0 = time.perf_counter()
    fb = cpu_frame.FrameBaseline(sc)
    return fb, time.perf_counter() - t0


def _cpu_sample_text(fb, parts, st):
    sc = fb.sc
    return ("one full frame on the host cores, no extrapolation: C++/OpenMP float64 restatement of the "
            "reference's CPU path (oracle/cpu_frame.cpp): %d-iteration Gauss-Newton solve of %d free nodes "
            "(J in CSR, J^T J, block sparse Cholesky with a minimum-degree ordering, %.1f GFLOP per "
            "factorisation, one factorisation per iteration where the reference does two), skinning of %d "
            "samples and %d Gaussians, node update; ms: solve %.0f (factorisations %.0f), samples %.0f, "
            "Gaussians %.0f, nodes %.0f" % (sc.iters, st["n_free"], st["factor_gflop"], fb.n_samples,
                                            sc.n_gauss, parts["solve"], 1e3 * st["t_factor"],
                                            parts["skin_samples"], parts["skin_gaussians"], parts["update_nodes"]))


def cpu_baseline(sc):
    fb, t_setup = _cpu_frame(sc)
    ms, parts, st = fb.run()
    return {"value": round(ms, 1), "unit": "ms/frame", "cores": fb.threads, "kind": "port",
            "sample": _cpu_sample_text(fb, parts, st), "setup_s": round(t_setup, 1)}


def run_reference(a):
    ws, rank = _dist()
    if rank != 0:
        return
    synth = importlib.import_module(PKG + ".synth")
    import numpy as np
    sc = synth.make_scene(a.scene)
    fb, t_setup = _cpu_frame(sc)
    vals = []
    t0 = time.perf_counter()
    for i in range(a.warmup + a.steps):
        if i == a.warmup:
            t0 = time.perf_counter()
        ms, parts, st = fb.run()
        if i >= a.warmup:
            vals.append(ms)
    wall = time.perf_counter() - t0
    v = float(np.mean(vals))
    line = {"metric": METRIC, "value": round(v, 1), "unit": "ms/frame", "n_gpus": ws, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": round(v, 1), "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded two-bars-and-sphere field)",
            "impl": "reference",
            "config": {"workload": "%s: %d Gaussians, %d^3 grid, %d nodes, k=%d, %d GN iterations, %s "
                                   "(reference CPU path restated in C++/OpenMP, host cores)"
                                   % (sc.name, sc.n_gauss, sc.grid_num, sc.n_nodes, sc.k, sc.iters, op_text(sc.op)),
                       "samples": fb.n_samples, "setup_s": round(t_setup, 1), "wall_s_timed_region": round(wall, 1)},
            "cpu_baseline": {"value": round(v, 1), "unit": "ms/frame", "cores": fb.threads, "kind": "port",
                             "sample": _cpu_sample_text(fb, parts, st)},
            "e2e": {"value": round(v, 1), "unit": "ms/frame", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


if __name__ == "__main__":
    a = _args()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)
