"""Shared scene setup for the parity tests (oracle on the CPU, library on the GPU)."""
import importlib
import math

import numpy as np

synth = importlib.import_module("arap-deformation-of-gaussian-radiance-fields_gb300.synth")


def active_nodes(sc):
    return np.concatenate([b for b, t in zip(sc.blocks, sc.block_type) if t == 1]).astype(np.int64) \
        if any(t == 1 for t in sc.block_type) else np.zeros(0, np.int64)


def oracle_aims(sc, node_pos):
    """Apply the scene's control operation to aims = node positions with the
    oracle's target generators."""
    from oracle import targets
    aims = node_pos.astype(np.float32).copy()
    act = active_nodes(sc)
    op = sc.op
    if op[0] == "translate":
        return targets.translate(aims, act, op[1])
    if op[0] == "twist":
        return targets.twist(aims, node_pos, act, op[1], op[2])
    return targets.scale(aims, node_pos, act, op[1])


def rel_err(a, b, floor=1e-12):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), floor))
