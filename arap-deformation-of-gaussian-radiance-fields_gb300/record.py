"""Deformation records (the viewer's ``deform.txt``) and their replay plan.

Mirrors the reference viewer's RecordDeformation / LoadDeformation
(GaussianView.cpp:4859-4935, 4960-5095) and the bookkeeping of its history
replay (GaussianView.cpp:1757-1916).  Host-side text format only.

A record is one line of whitespace-separated tokens:
``<nodes_on_mesh> Nodes: N v_1..v_N Total_Operations: T Move_Operations: M
Operation_Types: K t_1..t_K Block_Nodes: B (n_b i_1..i_n)* Mouse_Movements: S
(n_s (x y z)*)* Blocks_Types_Moves: S (n_s k_1..k_n)* Energy_on_Center: E
e_1..e_E Twist_Axis: A (x y z w)*``; every token is followed by one space and
floats are written as C++ streams write them by default (6 significant
digits, ``%g``).

Operation types (GaussianView.cpp:1758-1877): a negative value -(i+1) deletes
control block i; 0 adds the next recorded block; 1 moves the active block with
the constraints on the block centres, 2 twists it about the recorded axis, 3
scales it, 4 moves it with per-node constraints.  A move operation consumes
one entry of Mouse_Movements (one element per frame) and one of
Blocks_Types_Moves (the block types for those frames).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

OP_ADD, OP_MOVE_CENTRE, OP_TWIST, OP_SCALE, OP_MOVE = 0, 1, 2, 3, 4


@dataclass
class DeformHistory:
    nodes_on_mesh: int = 0
    node_vertices: list = field(default_factory=list)      # vertex index of every graph node
    total_operations: int = 0
    move_operations: int = 0
    operation_types: list = field(default_factory=list)
    block_nodes: list = field(default_factory=list)        # per added block: graph-node indices
    mouse_movements: list = field(default_factory=list)    # per move: [frames, 3] float32
    blocks_types_moves: list = field(default_factory=list)  # per move: the block types
    energy_on_centers: list = field(default_factory=list)
    twist_axis: list = field(default_factory=list)         # per move: (x, y, z, w) float32


def _labelled(tokens, pos, label):
    if pos >= len(tokens) or tokens[pos] != label:
        raise ValueError("deform record: expected %r at token %d" % (label, pos))
    return pos + 1


def read_deform(path) -> DeformHistory:
    """Parses a record written by the viewer (or by write_deform).  Raises
    ValueError on a malformed record, where the viewer reads garbage."""
    tokens = open(path, "r").read().split()
    h = DeformHistory()
    p = 0

    def take(n, conv):
        nonlocal p
        if p + n > len(tokens):
            raise ValueError("deform record: truncated at token %d" % p)
        vals = [conv(t) for t in tokens[p:p + n]]
        p += n
        return vals

    h.nodes_on_mesh = take(1, int)[0]
    p = _labelled(tokens, p, "Nodes:")
    h.node_vertices = take(take(1, int)[0], int)
    p = _labelled(tokens, p, "Total_Operations:")
    h.total_operations = take(1, int)[0]
    p = _labelled(tokens, p, "Move_Operations:")
    h.move_operations = take(1, int)[0]
    p = _labelled(tokens, p, "Operation_Types:")
    h.operation_types = take(take(1, int)[0], int)
    p = _labelled(tokens, p, "Block_Nodes:")
    for _ in range(take(1, int)[0]):
        h.block_nodes.append(take(take(1, int)[0], int))
    p = _labelled(tokens, p, "Mouse_Movements:")
    for _ in range(take(1, int)[0]):
        n = take(1, int)[0]
        h.mouse_movements.append(np.array(take(3 * n, float), np.float32).reshape(n, 3))
    p = _labelled(tokens, p, "Blocks_Types_Moves:")
    for _ in range(take(1, int)[0]):
        h.blocks_types_moves.append(take(take(1, int)[0], int))
    p = _labelled(tokens, p, "Energy_on_Center:")
    h.energy_on_centers = take(take(1, int)[0], int)
    p = _labelled(tokens, p, "Twist_Axis:")
    for _ in range(take(1, int)[0]):
        h.twist_axis.append(np.array(take(4, float), np.float32))
    if p != len(tokens):
        raise ValueError("deform record: %d trailing tokens" % (len(tokens) - p))
    return h


def _f(x) -> str:
    return "%g" % float(np.float32(x))


def format_deform(h: DeformHistory) -> str:
    """The record text, token for token as RecordDeformation writes it."""
    out = [str(int(h.nodes_on_mesh)), "Nodes:", str(len(h.node_vertices))]
    out += [str(int(v)) for v in h.node_vertices]
    out += ["Total_Operations:", str(int(h.total_operations)), "Move_Operations:", str(int(h.move_operations))]
    out += ["Operation_Types:", str(len(h.operation_types))] + [str(int(t)) for t in h.operation_types]
    out += ["Block_Nodes:", str(len(h.block_nodes))]
    for b in h.block_nodes:
        out += [str(len(b))] + [str(int(i)) for i in b]
    out += ["Mouse_Movements:", str(len(h.mouse_movements))]
    for m in h.mouse_movements:
        m = np.asarray(m, np.float32).reshape(-1, 3)
        out += [str(m.shape[0])] + [_f(v) for v in m.reshape(-1)]
    out += ["Blocks_Types_Moves:", str(len(h.blocks_types_moves))]
    for t in h.blocks_types_moves:
        out += [str(len(t))] + [str(int(k)) for k in t]
    out += ["Energy_on_Center:", str(len(h.energy_on_centers))] + [str(int(e)) for e in h.energy_on_centers]
    out += ["Twist_Axis:", str(len(h.twist_axis))]
    for a in h.twist_axis:
        out += [_f(v) for v in np.asarray(a, np.float32).reshape(4)]
    return "".join(t + " " for t in out)


def write_deform(path, h: DeformHistory) -> None:
    with open(path, "w") as f:
        f.write(format_deform(h))


def replay_steps(h: DeformHistory):
    """The frames a replay of the record drives, in order (the bookkeeping of
    GaussianView.cpp:1757-1916 without the viewer's geometry).  Each entry is
    a dict: ``kind`` ('delete', 'add' or 'move'), ``blocks`` (graph-node
    indices of every control block after the step) and ``types`` (their block
    types); a 'move' entry per frame also has ``op`` (OP_MOVE_CENTRE,
    OP_TWIST, OP_SCALE, OP_MOVE), ``constraints_on_center``, ``active`` (the
    active block index) and its parameter: ``translation`` (x, y, z) for
    moves, ``axis`` (x, y, z, w) and ``angle_step`` for twists,
    ``scale_step`` for scales.  A delete with no block left is skipped; the
    viewer stalls on such a step (its history never advances past it)."""
    blocks, types, steps = [], [], []
    active = 0
    add_idx = move_idx = 0
    step = 0
    while step < h.total_operations:
        op = h.operation_types[step]
        if op < 0:
            if blocks:
                cur = -(op + 1)
                del blocks[cur]
                del types[cur]
                active = cur % len(blocks) if blocks else 0
                steps.append({"kind": "delete", "blocks": [list(b) for b in blocks], "types": list(types)})
            step += 1
        elif op == OP_ADD:
            blocks.append(list(h.block_nodes[add_idx]))
            types.append(1 if len(blocks) == 1 else 0)
            if len(blocks) == 1:
                active = 0
            add_idx += 1
            step += 1
            steps.append({"kind": "add", "blocks": [list(b) for b in blocks], "types": list(types)})
        else:
            types = list(h.blocks_types_moves[move_idx])
            moves = np.asarray(h.mouse_movements[move_idx], np.float32).reshape(-1, 3)
            for f in range(moves.shape[0]):
                e = {"kind": "move", "op": op, "blocks": [list(b) for b in blocks], "types": list(types),
                     "active": active, "constraints_on_center": op == OP_MOVE_CENTRE}
                if op in (OP_MOVE_CENTRE, OP_MOVE):
                    e["translation"] = moves[f].copy()
                elif op == OP_TWIST:
                    e["axis"] = np.asarray(h.twist_axis[move_idx], np.float32).copy()
                    e["angle_step"] = int(moves[f, 0])
                elif op == OP_SCALE:
                    e["scale_step"] = int(moves[f, 0])
                steps.append(e)
            move_idx += 1
            step += 1
    return steps
