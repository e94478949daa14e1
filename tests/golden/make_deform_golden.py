"""Digest of the reference dataset's deformation record (pinocchio deform.txt),
as parsed and re-written by record.py: the record's SHA-256 and length, whether
format_deform reproduces it byte for byte, and the replay plan's shape.

    python tests/golden/make_deform_golden.py /root/reference

The record itself is not copied; the digest pins the parser and writer to the
viewer's format (GaussianView.cpp:4859-5095) on the one real record there is.
"""
import collections
import hashlib
import importlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
rec = importlib.import_module("arap-deformation-of-gaussian-radiance-fields_gb300.record")


def main(root):
    path = os.path.join(root, "datasets", "pinocchio", "point_cloud", "iteration_30000", "deform.txt")
    raw = open(path, "rb").read()
    h = rec.read_deform(path)
    steps = rec.replay_steps(h)
    moves = [s for s in steps if s["kind"] == "move"]
    digest = {
        "source": "datasets/pinocchio/point_cloud/iteration_30000/deform.txt",
        "sha256": hashlib.sha256(raw).hexdigest(),
        "bytes": len(raw),
        "round_trip_exact": rec.format_deform(h).encode() == raw,
        "nodes_on_mesh": h.nodes_on_mesh,
        "nodes": len(h.node_vertices),
        "total_operations": h.total_operations,
        "move_operations": h.move_operations,
        "operation_types": collections.Counter(h.operation_types).most_common(),
        "block_sizes": [len(b) for b in h.block_nodes],
        "frames_per_move": [int(np.asarray(m).reshape(-1, 3).shape[0]) for m in h.mouse_movements],
        "replay_frames": len(steps),
        "replay_kinds": collections.Counter(s["kind"] for s in steps).most_common(),
        "translation_sum": [float(v) for v in np.sum([m["translation"] for m in moves if "translation" in m], axis=0)],
    }
    out = os.path.join(HERE, "deform_record_pinocchio.json")
    with open(out, "w") as f:
        json.dump(digest, f, indent=1)
    print(out, digest["round_trip_exact"])


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <reference project root>" % sys.argv[0])
    main(sys.argv[1])
