"""Node transforms of the benchmark scenes' Gauss-Newton solves, computed by
the float64 numpy oracle (oracle/ed.py: Deform::optimize restated with an
exact sparse solve of J^T J h = -J^T f, Deform.cpp:95-169), for the GPU
parity tests at the benchmark's sizes.

    python tests/golden/make_solve_golden.py bend50k twist300k
    python tests/golden/make_solve_golden.py --solver=cpp stress200k

Each scene writes tests/golden/solve_<scene>.npz with
  x         float32 [n,12]  node transforms [R column-major 9 | t 3] (static
                            nodes identity), the solve's output
  energies  float64 [iters] |f|^2 at the start of every iteration
  halvings  int32   [iters] line-search halvings of every iteration
  final     float64         |f|^2 after the last iteration
and the scene's name, iteration count and node count.  Early exit is off
(every iteration runs), as in the benchmark.  twist300k takes about ten
minutes (one sparse factorisation of a 48,732-column system per iteration).
--solver=cpp uses the C++ float64 restatement instead (stress200k: 91,000
columns, about a minute on eight cores); its record keeps the first energy
and the total halvings.
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


def main(names, solver="numpy"):
    from oracle import cpu_frame, ed
    from _helpers import oracle_aims
    for name in names:
        t0 = time.time()
        sc = synth.make_scene(name)
        nb = ed.build_graph(sc.node_pos, sc.k)
        aidx, aw = ed.knn_weights(sc.pos[sc.node_vertex], sc.node_pos, sc.k)
        aims = oracle_aims(sc, sc.node_pos)
        if solver == "numpy":
            pr = ed.EDProblem(sc.node_pos, nb, aidx, aw, sc.blocks, sc.block_type, aims)
            x, gs = ed.gauss_newton(pr, max_iters=sc.iters, early_exit=False)
            rot, tr = ed.put_free_inputs(pr, x)
            energies, halvings, final = gs.energies, gs.halvings, gs.final_energy
        else:
            # the C++ restatement (oracle/cpu_frame.cpp): the same float64
            # algorithm with a block Cholesky, checked against the numpy
            # oracle in tests/test_cpu_frame.py; it records the first energy
            # and the total halvings only
            rot, tr, st = cpu_frame.solve(sc.node_pos, nb, aidx, aw, sc.blocks, sc.block_type, aims,
                                          max_iters=sc.iters, early_exit=False)
            energies, final = [st["initial_energy"]], st["final_energy"]
            halvings = [st["halvings"]]
        X = np.concatenate([rot, tr], 1).astype(np.float32)
        out = os.path.join(HERE, "solve_%s.npz" % name)
        np.savez_compressed(out, x=X, energies=np.asarray(energies, np.float64),
                            halvings=np.asarray(halvings, np.int32), final=np.float64(final),
                            scene=name, iters=np.int32(sc.iters), n_nodes=np.int32(sc.n_nodes), solver=solver)
        print("%s: %d nodes, %d iterations, final energy %.6g, %.0f s -> %s"
              % (name, sc.n_nodes, sc.iters, final, time.time() - t0, out))


if __name__ == "__main__":
    args = sys.argv[1:]
    solver = "numpy"
    if args and args[0].startswith("--solver="):
        solver = args.pop(0).split("=", 1)[1]
    main(args or ["bend50k", "twist300k"], solver)
