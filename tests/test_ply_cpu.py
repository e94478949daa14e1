"""3DGS PLY load/save (arap_ply_*, host only) against the oracle restatement of
the viewer's loadPly / savePly (GaussianView.cpp:43-339), on CPU.

Positions, SH, the Morton order, the box and the index property must match
exactly; exp/log-derived fields (scale, opacity) and the normalised quaternion
within 4 ulp: the C library's and numpy's float exp/log differ by up to 2 ulp,
the logistic function's add and divide can carry that to 3, and the host
compiler may fuse a multiply-add in the quaternion length."""
import importlib

import numpy as np
import pytest

from oracle import ply as oply

PKG = "arap-deformation-of-gaussian-radiance-fields_gb300"


@pytest.fixture(scope="module")
def io():
    return importlib.import_module(PKG + ".ply")


def _ulp_close(a, b, ulps=4):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    tol = ulps * np.spacing(np.maximum(np.abs(a), np.abs(b)).astype(np.float32))
    return bool(np.all(np.abs(a - b) <= tol))


def _random_records(n, sh_degree=3, with_index=False, seed=0):
    rng = np.random.default_rng(seed)
    props = oply.standard_props(sh_degree, with_index)
    rec = np.zeros((n, len(props)), np.float32)
    col = {p: i for i, p in enumerate(props)}
    rec[:, [col["x"], col["y"], col["z"]]] = rng.uniform(-3, 5, (n, 3))
    rec[:, [col["nx"], col["ny"], col["nz"]]] = rng.normal(size=(n, 3))
    for p in props:
        if p.startswith("f_"):
            rec[:, col[p]] = rng.normal(size=n)
    rec[:, col["opacity"]] = rng.normal(0, 3, n)
    rec[:, [col["scale_0"], col["scale_1"], col["scale_2"]]] = rng.uniform(-6, 0, (n, 3))
    rec[:, [col["rot_0"], col["rot_1"], col["rot_2"], col["rot_3"]]] = rng.normal(size=(n, 4))
    if with_index:
        rec[:, col["index"]] = rng.permutation(n).astype(np.float32) + rng.uniform(-0.3, 0.3, n)
    return rec, props


def test_oracle_known_answers(tmp_path):
    # three splats written by hand; the expected values follow from the
    # format's definition alone
    props = oply.standard_props(3)
    col = {p: i for i, p in enumerate(props)}
    rec = np.zeros((3, len(props)), np.float32)
    rec[0, [0, 1, 2]] = [0, 0, 0]
    rec[1, [0, 1, 2]] = [1, 1, 1]
    rec[2, [0, 1, 2]] = [0.5, 0, 0]
    rec[:, col["rot_0"]] = [2, 0, 1]
    rec[1, [col["rot_1"], col["rot_2"]]] = [3, 4]
    rec[:, col["opacity"]] = 0
    rec[:, [col["f_dc_0"], col["f_dc_1"], col["f_dc_2"]]] = [1, 2, 3]
    for i in range(45):
        rec[:, col["f_rest_%d" % i]] = 100 + i
    path = str(tmp_path / "known.ply")
    oply.write_raw(path, rec, props)
    out = oply.load(path)
    # Morton codes: (0,0,0) -> 0, (0.5,0,0) -> x = 2^20 - 1, (1,1,1) -> all bits
    np.testing.assert_array_equal(out["pos"], [[0, 0, 0], [0.5, 0, 0], [1, 1, 1]])
    np.testing.assert_array_equal(out["rot"], np.array([[1, 0, 0, 0], [1, 0, 0, 0], [0, 0.6, 0.8, 0]], np.float32))
    np.testing.assert_array_equal(out["scale"], np.ones((3, 3), np.float32))
    np.testing.assert_array_equal(out["opacity"], np.full(3, 0.5, np.float32))
    expect_sh = np.zeros(48, np.float32)
    expect_sh[0:3] = [1, 2, 3]
    for j in range(1, 16):
        for c in range(3):
            expect_sh[3 * j + c] = 100 + 15 * c + (j - 1)
    np.testing.assert_array_equal(out["shs"], np.tile(expect_sh, (3, 1)))
    np.testing.assert_array_equal(oply.morton_codes(out["pos"]),
                                  np.array([0, sum(1 << (3 * i) for i in range(20)), (1 << 63) - 1], np.uint64))


@pytest.mark.parametrize("morton", [True, False])
def test_load_matches_oracle(tmp_path, io, morton):
    rec, props = _random_records(3000, seed=1)
    path = str(tmp_path / "r.ply")
    oply.write_raw(path, rec, props)
    assert io.ply_info(path) == (3000, 3, False)
    got = io.load_ply(path, morton_order=morton)
    ref = oply.load(path, morton=morton)
    for k in ("pos", "shs", "box_min", "box_max"):
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
    for k in ("scale", "opacity", "rot"):
        assert _ulp_close(got[k], ref[k]), k


def test_morton_ties_keep_file_order(tmp_path, io):
    # duplicated positions share a Morton code: they keep their file order
    rec, props = _random_records(200, with_index=True, seed=2)
    rec[100:, :3] = rec[:100, :3]
    rec[:, props.index("index")] = np.arange(200, dtype=np.float32)
    path = str(tmp_path / "ties.ply")
    oply.write_raw(path, rec, props)
    got = io.load_ply(path, with_index=True)
    ref = oply.load(path)
    np.testing.assert_array_equal(got["index"], ref["index"])
    codes = oply.morton_codes(rec[:, :3])
    for c in np.unique(codes):
        ids = got["index"][oply.morton_codes(got["pos"]) == c]
        assert np.all(np.diff(ids) > 0)


@pytest.mark.parametrize("degree", [0, 1, 2])
def test_lower_sh_degrees(tmp_path, io, degree):
    rec, props = _random_records(500, sh_degree=degree, seed=3 + degree)
    path = str(tmp_path / ("d%d.ply" % degree))
    oply.write_raw(path, rec, props)
    assert io.ply_info(path)[1] == degree
    got = io.load_ply(path)
    ref = oply.load(path)
    np.testing.assert_array_equal(got["shs"], ref["shs"])
    k = (degree + 1) ** 2
    assert np.all(got["shs"][:, 3 * k:] == 0)


def test_index_property(tmp_path, io):
    rec, props = _random_records(700, with_index=True, seed=7)
    path = str(tmp_path / "soup.ply")
    oply.write_raw(path, rec, props)
    assert io.ply_info(path) == (700, 3, True)
    got = io.load_ply(path, with_index=True)
    ref = oply.load(path)
    np.testing.assert_array_equal(got["index"], ref["index"])
    np.testing.assert_array_equal(np.sort(got["index"]), np.arange(700))


def test_save_matches_oracle(tmp_path, io):
    rng = np.random.default_rng(11)
    n = 2500
    pos = rng.uniform(-2, 2, (n, 3)).astype(np.float32)
    shs = rng.normal(size=(n, 48)).astype(np.float32)
    opacity = rng.uniform(0.01, 0.99, n).astype(np.float32)
    scale = rng.uniform(1e-3, 1, (n, 3)).astype(np.float32)
    rot = rng.normal(size=(n, 4)).astype(np.float32)
    too_small = rng.random(n) < 0.1
    lo = np.array([-1.5, -2, -1.8], np.float32)
    hi = np.array([1.7, 1.5, 2.0], np.float32)
    pos[0] = lo  # on the box: kept
    pos[1] = hi
    a, b = str(tmp_path / "a.ply"), str(tmp_path / "b.ply")
    wa = io.save_ply(a, pos, shs, opacity, scale, rot, lo, hi, too_small)
    wb = oply.save(b, pos, shs, opacity, scale, rot, lo, hi, too_small)
    assert wa == wb
    keep = np.all((pos >= lo) & (pos <= hi), axis=1) & ~too_small
    assert wa == int(keep.sum())
    ra, rb = open(a, "rb").read(), open(b, "rb").read()
    ha, hb = ra[:ra.index(b"end_header\n") + 11], rb[:rb.index(b"end_header\n") + 11]
    assert ha == hb
    fa = np.frombuffer(ra[len(ha):], "<f4").reshape(wa, 62)
    fb = np.frombuffer(rb[len(hb):], "<f4").reshape(wb, 62)
    exact = [c for c in range(62) if c < 54 or c >= 58]
    np.testing.assert_array_equal(fa[:, exact], fb[:, exact])
    assert _ulp_close(fa[:, 54:58], fb[:, 54:58])


def test_round_trip(tmp_path, io):
    rec, props = _random_records(1000, seed=13)
    path = str(tmp_path / "in.ply")
    oply.write_raw(path, rec, props)
    first = io.load_ply(path, morton_order=False)
    out = str(tmp_path / "out.ply")
    big = np.float32(1e30)
    assert io.save_ply(out, first["pos"], first["shs"], first["opacity"], first["scale"], first["rot"],
                       [-big] * 3, [big] * 3) == 1000
    second = io.load_ply(out, morton_order=False)
    np.testing.assert_array_equal(second["pos"], first["pos"])
    np.testing.assert_array_equal(second["shs"], first["shs"])
    np.testing.assert_allclose(second["scale"], first["scale"], rtol=1e-6)
    np.testing.assert_allclose(second["opacity"], first["opacity"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(second["rot"], first["rot"], atol=1e-7)


def test_bad_files(tmp_path, io):
    lib = importlib.import_module(PKG + "._lib")
    with pytest.raises(lib.ArapError):
        io.ply_info(str(tmp_path / "missing.ply"))
    rec, props = _random_records(10, seed=17)
    p = str(tmp_path / "ascii.ply")
    with open(p, "wb") as f:
        f.write(b"ply\nformat ascii 1.0\nelement vertex 10\nproperty float x\nend_header\n")
    with pytest.raises(lib.ArapError):
        io.ply_info(p)
    p = str(tmp_path / "short.ply")
    oply.write_raw(p, rec, props)
    data = open(p, "rb").read()
    open(p, "wb").write(data[:-100])
    with pytest.raises(lib.ArapError):
        io.load_ply(p)
    p = str(tmp_path / "double.ply")
    with open(p, "wb") as f:
        f.write(b"ply\nformat binary_little_endian 1.0\nelement vertex 1\nproperty double x\nend_header\n")
    with pytest.raises(lib.ArapError):
        io.ply_info(p)
    p = str(tmp_path / "norot.ply")
    oply.write_raw(p, rec[:, :-1], props[:-1])
    with pytest.raises(lib.ArapError):
        io.ply_info(p)
