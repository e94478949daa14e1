"""Generate ``sh_rotation.json``: SH band-rotation matrices computed by the
reference's own formulas.

Run in a container that has the reference checkout:

    python tests/golden/make_sh_rotation_golden.py /root/reference

The reference cannot be compiled (it needs Eigen), so this script reads the
formula text of ``Construct_SH_Rotation_MatrixCUDA``
(src/projects/gaussianviewer/renderer/cudakdtree.cu:11-111) and evaluates
each assignment ``shN.row(a)(b) = <expr>;`` in float64, in source order, for a
set of rotations.  It also reads the fixed rotation and SH input of
``Test_SH_Rotation`` (helper.cpp:924-936) and records the band-rotated output
(``SH_Rotation``, helper.cpp:938-973: no odd-coefficient flip).

Nothing of the reference is copied into the fixture except numbers it computes.
"""
from __future__ import annotations

import json
import math
import os
import re
import sys

import numpy as np

REL = "src/projects/gaussianviewer/renderer"


def _load_formulas(ref_root):
    src = open(os.path.join(ref_root, REL, "cudakdtree.cu")).read()
    start = src.index("Construct_SH_Rotation_MatrixCUDA")
    body = src[start:src.index("\n}", start)]
    stmts = []
    for m in re.finditer(r"(sh[123])\.row\((\d)\)\((\d)\)\s*=\s*(.*?);", body, re.S):
        expr = m.group(4)
        expr = re.sub(r"(sh[123])\.row\((\d)\)\((\d)\)", r"\1[\2][\3]", expr)
        expr = re.sub(r"rots\.row\((\d)\)\((\d)\)", r"R[\1][\2]", expr)
        expr = expr.replace("sqrt(", "math.sqrt(")
        stmts.append((m.group(1), int(m.group(2)), int(m.group(3)), compile(expr, "f", "eval")))
    return stmts


def _eval(stmts, R):
    env = {"math": math, "R": R,
           "sh1": [[0.0] * 3 for _ in range(3)],
           "sh2": [[0.0] * 5 for _ in range(5)],
           "sh3": [[0.0] * 7 for _ in range(7)]}
    for name, a, b, code in stmts:
        env[name][a][b] = eval(code, env)
    return env["sh1"], env["sh2"], env["sh3"]


def _quat_to_R(q):
    w, x, y, z = q / np.linalg.norm(q)
    return [[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
            [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
            [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]]


def _test_input(ref_root):
    src = open(os.path.join(ref_root, REL, "helper.cpp")).read()
    s = src[src.index("void Test_SH_Rotation"):]
    q = [float(v) for v in re.search(r"origin_q\(([^)]*)\)", s).group(1).split(",")]
    shs = [float(v) for v in re.search(r"shs_in\s*=\s*\{([^}]*)\}", s).group(1).split(",")]
    return np.array(q), np.array(shs)


def _rotate(sh, m1, m2, m3):
    s = np.array(sh, float).reshape(16, 3).copy()
    s[1:4] = np.array(m1) @ s[1:4]
    s[4:9] = np.array(m2) @ s[4:9]
    s[9:16] = np.array(m3) @ s[9:16]
    return s.reshape(-1)


def main(ref_root):
    stmts = _load_formulas(ref_root)
    assert len(stmts) == 9 + 25 + 49, len(stmts)
    rng = np.random.default_rng(1234)
    cases = []
    quats = [np.array([1.0, 0, 0, 0]), np.array([0.0, 1, 0, 0]), np.array([0.0, 0, 1, 0]),
             np.array([0.0, 0, 0, 1]), np.array([np.cos(0.3), 0, 0, np.sin(0.3)])]
    quats += [rng.standard_normal(4) for _ in range(27)]
    for q in quats:
        R = _quat_to_R(np.asarray(q, float))
        m1, m2, m3 = _eval(stmts, R)
        sh = rng.standard_normal(48) * 0.3
        cases.append({"R": R, "sh1": m1, "sh2": m2, "sh3": m3,
                      "sh_in": sh.tolist(), "sh_out": _rotate(sh, m1, m2, m3).tolist()})
    q, shs = _test_input(ref_root)
    R = _quat_to_R(q)
    m1, m2, m3 = _eval(stmts, R)
    kat = {"quat_wxyz": q.tolist(), "R": R, "sh_in": shs.tolist(),
           "sh_out": _rotate(shs, m1, m2, m3).tolist()}
    out = {"source": "reference cudakdtree.cu:11-111 formulas, helper.cpp:924-973 KAT",
           "cases": cases, "kat_test_sh_rotation": kat}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "sh_rotation.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=None, separators=(",", ":"))
    print("wrote", path, len(cases), "cases")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <reference project root>" % sys.argv[0])
    main(sys.argv[1])
