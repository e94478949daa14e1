"""Oracle: 3D Gaussian splatting binary PLY load/save.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  Restated from:

* ``load``  -- GaussianView.cpp:43-147 (loadPly_Origin) and 149-262 (loadPly):
               header read as the viewer does (the vertex count from the third
               line, the rest skipped to ``end_header``), the fixed record layout
               of helper.hpp:98-119 (RichPoint / RichPoint_Soup: pos, normal,
               SH, opacity, scale, rot[, index]), the 21-bit Morton reorder over
               the bounding box, and the activations (normalised quaternion,
               exp scale, logistic opacity; GaussianView.cpp:20-28)
* ``save``  -- GaussianView.cpp:264-339 (savePly): box and too-small filter,
               log scale, logit opacity, degree-3 SH, zero normals

The arithmetic follows the reference's float32 expressions step by step
(numpy float32 operations are IEEE single precision like the reference's).
``exp`` and ``log`` may differ from a C library's by one unit in the last
place; the tests compare those fields within 2 ulp and everything else
exactly.  Where the reference's ``std::sort`` leaves equal Morton codes in an
unspecified order, the oracle keeps file order (a stable sort).

Pinned by the known-answer file of ``tests/test_ply_cpu.py``
(``test_oracle_known_answers``), built by hand from the format's definition:
the reference ships no PLY fixture (its datasets' PLYs are missing).
"""
from __future__ import annotations

import numpy as np


def record_floats(sh_degree: int = 3, with_index: bool = False) -> int:
    k = (sh_degree + 1) ** 2
    return 3 + 3 + 3 * k + 1 + 3 + 4 + (1 if with_index else 0)


def _read_header(buf: bytes):
    # the viewer reads three lines, takes the count from the third, then skips
    # to end_header (GaussianView.cpp:57-74)
    lines, off = [], 0
    while True:
        nl = buf.index(b"\n", off)
        line = buf[off:nl].decode("ascii").rstrip("\r")
        off = nl + 1
        lines.append(line)
        if line == "end_header":
            break
    count = int(lines[2].split()[2])
    props = [ln.split()[2] for ln in lines if ln.startswith("property")]
    return count, props, off


def morton_codes(pos: np.ndarray) -> np.ndarray:
    """GaussianView.cpp:91-118: 21 bits per axis, x in bit 3i, y 3i+1, z 3i+2."""
    pos = pos.astype(np.float32)
    lo = pos.min(0)
    hi = pos.max(0)
    ext = (hi - lo).astype(np.float32)
    with np.errstate(invalid="ignore", divide="ignore"):
        rel = np.where(ext > 0, (pos - lo) / np.where(ext > 0, ext, np.float32(1)), np.float32(0)).astype(np.float32)
    scaled = (np.float32((1 << 21) - 1) * rel).astype(np.float32)
    xyz = scaled.astype(np.int64)  # truncation, as Eigen's cast<int>
    code = np.zeros(pos.shape[0], dtype=np.uint64)
    for i in range(21):
        for a in range(3):
            code |= ((xyz[:, a] >> i) & 1).astype(np.uint64) << np.uint64(3 * i + a)
    return code


def load(path: str, morton: bool = True):
    buf = open(path, "rb").read()
    count, props, off = _read_header(buf)
    nprop = len(props)
    rec = np.frombuffer(buf, dtype="<f4", count=count * nprop, offset=off).reshape(count, nprop)
    col = {p: i for i, p in enumerate(props)}
    pos = rec[:, [col["x"], col["y"], col["z"]]].astype(np.float32)
    order = np.argsort(morton_codes(pos), kind="stable") if morton and count > 1 else np.arange(count)
    rest = sum(1 for p in props if p.startswith("f_rest_"))
    k = rest // 3 + 1
    out = {}
    r = rec[order]
    out["pos"] = pos[order]
    q = r[:, [col["rot_0"], col["rot_1"], col["rot_2"], col["rot_3"]]].astype(np.float32)
    len2 = np.zeros(count, dtype=np.float32)
    for j in range(4):  # sequential float32 sum (GaussianView.cpp:128-131)
        len2 = (len2 + q[:, j] * q[:, j]).astype(np.float32)
    out["rot"] = (q / np.sqrt(len2)[:, None]).astype(np.float32)
    out["scale"] = np.exp(r[:, [col["scale_0"], col["scale_1"], col["scale_2"]]]).astype(np.float32)
    o = r[:, col["opacity"]].astype(np.float32)
    out["opacity"] = (np.float32(1) / (np.float32(1) + np.exp(-o))).astype(np.float32)
    shs = np.zeros((count, 48), dtype=np.float32)
    for c in range(3):
        shs[:, c] = r[:, col["f_dc_%d" % c]]
    for j in range(1, k):
        for c in range(3):
            shs[:, 3 * j + c] = r[:, col["f_rest_%d" % (c * (k - 1) + j - 1)]]
    out["shs"] = shs
    out["box_min"] = pos.min(0) if count else np.full(3, np.inf, np.float32)
    out["box_max"] = pos.max(0) if count else np.full(3, -np.inf, np.float32)
    if "index" in col:
        out["index"] = np.round(r[:, col["index"]].astype(np.float64)).astype(np.int32)
    return out


def save(path: str, pos, shs, opacity, scale, rot, box_min, box_max, too_small=None) -> int:
    pos = np.asarray(pos, np.float32)
    keep = np.all((pos >= np.asarray(box_min, np.float32)) & (pos <= np.asarray(box_max, np.float32)), axis=1)
    if too_small is not None:
        keep &= ~np.asarray(too_small, bool)
    idx = np.flatnonzero(keep)
    n = idx.size
    rec = np.zeros((n, 62), dtype=np.float32)
    rec[:, 0:3] = pos[idx]
    shs = np.asarray(shs, np.float32)[idx]
    rec[:, 6:9] = shs[:, 0:3]
    for j in range(1, 16):
        for c in range(3):
            rec[:, 9 + 15 * c + (j - 1)] = shs[:, 3 * j + c]
    o = np.asarray(opacity, np.float32)[idx]
    rec[:, 54] = np.log(o / (np.float32(1) - o))
    rec[:, 55:58] = np.log(np.asarray(scale, np.float32)[idx])
    rec[:, 58:62] = np.asarray(rot, np.float32)[idx]
    names = ["x", "y", "z", "nx", "ny", "nz", "f_dc_0", "f_dc_1", "f_dc_2"] + ["f_rest_%d" % i for i in range(45)] + \
        ["opacity", "scale_0", "scale_1", "scale_2", "rot_0", "rot_1", "rot_2", "rot_3"]
    head = "ply\nformat binary_little_endian 1.0\nelement vertex %d\n" % n
    head += "".join("property float %s\n" % p for p in names) + "end_header\n"
    with open(path, "wb") as f:
        f.write(head.encode("ascii"))
        f.write(rec.astype("<f4").tobytes())
    return n


def write_raw(path: str, rec: np.ndarray, props, header_extra: str = "") -> None:
    """A PLY with the given float properties and records (test fixtures)."""
    head = "ply\nformat binary_little_endian 1.0\nelement vertex %d\n" % rec.shape[0] + header_extra
    head += "".join("property float %s\n" % p for p in props) + "end_header\n"
    with open(path, "wb") as f:
        f.write(head.encode("ascii"))
        f.write(np.ascontiguousarray(rec, dtype="<f4").tobytes())


def standard_props(sh_degree: int = 3, with_index: bool = False):
    k = (sh_degree + 1) ** 2
    props = ["x", "y", "z", "nx", "ny", "nz", "f_dc_0", "f_dc_1", "f_dc_2"]
    props += ["f_rest_%d" % i for i in range(3 * (k - 1))]
    props += ["opacity", "scale_0", "scale_1", "scale_2", "rot_0", "rot_1", "rot_2", "rot_3"]
    if with_index:
        props.append("index")
    return props
