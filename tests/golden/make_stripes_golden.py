"""Generate tests/golden/stripes_scripts.npz: the reference's own solver
inputs, the stripes deformation graph (datasets/stripes/point_cloud/
iteration_30000/graph.obj, 200 vertices) driven by its seven deform scripts
(LoadDeformScript0..6, GaussianView.cpp:2512-2788), with the float64
oracle's frames.

    python tests/golden/make_stripes_golden.py <reference root>

What is taken from the reference tree: the graph's vertices (read as
LoadMeshPoints does, helper.cpp:264-282) and, per script, its two node
blocks, their types and its step count, parsed from the script's source.
The script's motion constants are the oracle's restatement
(oracle/targets.py STRIPES_SCRIPTS); this script checks each of them against
the source text before using it.

The graph is built on the mesh ("Build Graph on Mesh", GaussianView.cpp:
2268-2273): every vertex is a node, in farthest-point order
(oracle.targets.farthest_point_order), with k = 10 graph neighbours and
anchors (GaussianView.hpp:598).  A script runs as RunDeformScript and the
update loop do (GaussianView.cpp:1917-1993, 2790-2815): per step the moved
block's aims are the script's, the kept block's aims its nodes' positions
when the script starts; one Deform solve (Deform.cpp:95-169, at most 30
Gauss-Newton iterations with the stop test) from identity transforms; then
every node moves by the ED blend of its own vertex (predict_mesh,
Deform.hpp:230-249; rounded once, as the library's node update).

Stored per script n: ``s<n>_types``, ``s<n>_block1``, ``s<n>_block2`` (node
ids), ``s<n>_aims`` [steps, m, 3] (the moved block's aims), ``s<n>_iters``
[steps] (Gauss-Newton iterations), ``s<n>_halvings`` [steps, 30] (line-search
halvings per iteration, -1 past the last), ``s<n>_energy`` [steps] (final
energy), ``s<n>_nodes`` [len(SAVED), 200, 3] (node positions after the steps
in ``s<n>_saved``).  Also ``vertices`` (file order), ``order`` (farthest-point
order) and ``k``.
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import ed, targets  # noqa: E402

K = 10
MAX_ITERS = 30


def script_body(src, n):
    a = src.index("void sibr::GaussianView::LoadDeformScript%d()" % n)
    b = src.index("void sibr::GaussianView::", a + 10)
    return src[a:b]


def check_constants(body, n, c):
    """The oracle's motion constants of script n appear in its source."""
    def has(fragment):
        if fragment not in body:
            raise SystemExit("script %d: %r not in the reference source" % (n, fragment))
    if c["kind"] == "slide":
        has("Pos(%sf, 0.0f, 0.0f)*df_step" % c["dx"])
        return
    has("Pos center_start(%.1ff, %.1ff, %.1ff);" % c["center"])
    has("Vector4f axis(%.1ff, %.1ff, %.1ff, 0.0f);" % c["axis"])
    turn = {-1.0: "-(float)df_step*Pi/(float)inter_steps", -1.5: "-(float)df_step*1.5f*Pi/(float)inter_steps",
            -0.5: "-(float)df_step*(Pi/2.0f)/(float)inter_steps",
            0.5: "(float)df_step*(Pi/2.0f)/(float)inter_steps"}[c["turn"]]
    has("float radian = %s;" % turn)
    if c["kind"] == "bend":
        has("float k = %sf;" % c["k"])
        has({"3pi2/k2": "float a = 3.0*Pi*Pi/(k*k);", "pi/k-pi2/2k": "float a = Pi/k - Pi*Pi/(2*k);"}[c["a"]])
        has("float y = %sa*x*x;" % ("-" if c["y_sign"] < 0 else ""))
        has("float x = (float)df_step*(-k/Pi)/(float)inter_steps;")


def main(ref):
    obj = os.path.join(ref, "datasets/stripes/point_cloud/iteration_30000/graph.obj")
    src = open(os.path.join(ref, "src/projects/gaussianviewer/renderer/GaussianView.cpp")).read()
    verts = np.array([[float(t) for t in line[2:].split()[:3]] for line in open(obj) if line.startswith("v ")],
                     np.float32)
    order = targets.farthest_point_order(verts)
    nodes0 = verts[order]
    n = nodes0.shape[0]
    nb = ed.build_graph(nodes0, K)
    aidx, aw = ed.knn_weights(nodes0, nodes0, K)
    out = {"vertices": verts, "order": order.astype(np.int32), "k": np.int32(K)}
    saved = lambda steps: sorted(set(list(range(4, steps, 5)) + [0, steps - 1]))  # noqa: E731
    for s, c in targets.STRIPES_SCRIPTS.items():
        body = script_body(src, s)
        blocks = [np.array([int(v) for v in re.findall(r"\d+", m)], np.int64)
                  for m in re.findall(r"vector<unsigned int> block\d = \{([^}]*)\}", body)]
        types = tuple(int(v) for v in re.search(r"blocks_types = \{([^}]*)\}", body).group(1).split(","))
        bound = re.search(r"df_step < inter_steps([^;]*);", body).group(1).strip()
        steps = {"+1": 50, "-10": 39}[bound.replace(" ", "")]
        if types != c["types"] or steps != c["steps"] or len(blocks) != 2:
            raise SystemExit("script %d: blocks/types/steps differ from the oracle's table" % s)
        check_constants(body, s, c)
        moved = blocks[c["moved"] - 1]
        kept = blocks[2 - c["moved"]]
        aims_moved = targets.stripes_script_aims(s, nodes0[moved])
        pos = nodes0.copy()
        iters, halv, energy, snaps = [], [], [], []
        for step in range(steps):
            aims = pos.copy()
            aims[kept] = nodes0[kept]
            aims[moved] = aims_moved[step]
            pr = ed.EDProblem(pos, nb, aidx, aw, blocks, np.array(types), aims)
            x, st = ed.gauss_newton(pr, max_iters=MAX_ITERS, early_exit=True)
            rot, tr = ed.put_free_inputs(pr, x)
            pos = ed.ed_blend(pos, aidx, aw, rot, tr, pos, float_accumulate=False)
            iters.append(st.iterations)
            h = np.full(MAX_ITERS, -1, np.int32)
            h[:len(st.halvings)] = st.halvings
            halv.append(h)
            energy.append(st.final_energy)
            if step in saved(steps):
                snaps.append(pos.copy())
        print("script %d: %d steps, GN iterations %s, halvings %d" % (s, steps, iters, int(sum(
            (h[h >= 0]).sum() for h in halv))))
        out.update({"s%d_types" % s: np.array(types, np.int32), "s%d_block1" % s: blocks[0].astype(np.int32),
                    "s%d_block2" % s: blocks[1].astype(np.int32), "s%d_aims" % s: aims_moved,
                    "s%d_iters" % s: np.array(iters, np.int32), "s%d_halvings" % s: np.stack(halv),
                    "s%d_energy" % s: np.array(energy), "s%d_saved" % s: np.array(saved(steps), np.int32),
                    "s%d_nodes" % s: np.stack(snaps).astype(np.float32)})
    np.savez_compressed(os.path.join(HERE, "stripes_scripts.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(__doc__)
    main(sys.argv[1])
