"""Node transforms of the benchmark scenes' Gauss-Newton solves, computed by
the float64 numpy oracle (oracle/ed.py: Deform::optimize restated with an
exact sparse solve of J^T J h = -J^T f, Deform.cpp:95-169), for the GPU
parity tests at the benchmark's sizes.

    python tests/golden/make_solve_golden.py bend50k twist300k

Each scene writes tests/golden/solve_<scene>.npz with
  x         float32 [n,12]  node transforms [R column-major 9 | t 3] (static
                            nodes identity), the solve's output
  energies  float64 [iters] |f|^2 at the start of every iteration
  halvings  int32   [iters] line-search halvings of every iteration
  final     float64         |f|^2 after the last iteration
and the scene's name, iteration count and node count.  Early exit is off
(every iteration runs), as in the benchmark.  twist300k takes about ten
minutes (one sparse factorisation of a 48,732-column system per iteration).
"""
import importlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))
synth = importlib.import_module("arap-deformation-of-gaussian-radiance-fields_gb300.synth")


def main(names):
    from oracle import ed
    from _helpers import oracle_aims
    for name in names:
        t0 = time.time()
        sc = synth.make_scene(name)
        nb = ed.build_graph(sc.node_pos, sc.k)
        aidx, aw = ed.knn_weights(sc.pos[sc.node_vertex], sc.node_pos, sc.k)
        aims = oracle_aims(sc, sc.node_pos)
        pr = ed.EDProblem(sc.node_pos, nb, aidx, aw, sc.blocks, sc.block_type, aims)
        x, gs = ed.gauss_newton(pr, max_iters=sc.iters, early_exit=False)
        rot, tr = ed.put_free_inputs(pr, x)
        X = np.concatenate([rot, tr], 1).astype(np.float32)
        out = os.path.join(HERE, "solve_%s.npz" % name)
        np.savez_compressed(out, x=X, energies=np.asarray(gs.energies, np.float64),
                            halvings=np.asarray(gs.halvings, np.int32), final=np.float64(gs.final_energy),
                            scene=name, iters=np.int32(sc.iters), n_nodes=np.int32(sc.n_nodes))
        print("%s: %d nodes, %d iterations, final energy %.6g, %.0f s -> %s"
              % (name, sc.n_nodes, gs.iterations, gs.final_energy, time.time() - t0, out))


if __name__ == "__main__":
    main(sys.argv[1:] or ["bend50k", "twist300k"])
