"""The reference's text caches and text scene files, read and written on
the host (no GPU): what this library reads equals what the reference's own
readers (PBDObject::ContinueSimInit, PBDObject::Init from text files) read
from the same files; what it writes equals, field for field, what the
reference's own writers (SaveMeshTopol / SaveConstraint) write; fixtures in
tests/golden/io* come from the reference's compiled code."""
import os

import numpy as np
import pytest

from positionbaseddynamicsold_gb300 import pbd

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
IO = os.path.join(GOLD, "io")


@pytest.fixture(scope="module")
def g():
    return dict(np.load(os.path.join(GOLD, "io.npz")))


def test_read_cache_matches_reference_reader(g):
    sc = pbd.read_cache(os.path.join(IO, "topol.cache"), os.path.join(IO, "constr.cache"))
    np.testing.assert_array_equal(sc["pos"].ravel(), g["cache_mesh_pos"])
    np.testing.assert_array_equal(sc["vel"].ravel(), g["cache_vel"])
    np.testing.assert_array_equal(sc["mass"], g["cache_mass"])
    prims = g["cache_mesh_prims"].reshape(-1, 2)
    tri = np.stack([g["cache_mesh_indices"][s:s + 3] for s, c in prims])
    np.testing.assert_array_equal(sc["tri_idx"], tri)
    np.testing.assert_array_equal(sc["prim_list"].ravel(), g["cache_c_prims"])
    np.testing.assert_array_equal(sc["indices"], g["cache_c_indices"])
    np.testing.assert_array_equal(sc["ctype"], g["cache_ctype"])
    np.testing.assert_array_equal(sc["rest_length"], g["cache_rest"])
    np.testing.assert_array_equal(sc["stiffness"], g["cache_stiff"])
    np.testing.assert_array_equal(sc["predicted"].ravel(), g["cache_prdp"])
    assert sc["damping"] == g["cache_damping"][0]
    np.testing.assert_array_equal(sc["gravity"], g["cache_gravity"])
    # the 6-digit text is close to the arrays the reference wrote
    np.testing.assert_allclose(sc["pos"], g["in_pos"], rtol=1e-5, atol=1e-9)


def _fields(path):
    """(name, values) of every line; the type field is left out (the
    reference's readers skip it and its spelling depends on the compiler)"""
    out = []
    for line in open(path):
        f = line.rstrip("\n").split("|")
        out.append((f[0], f[2] if len(f) > 2 else None))
    return out


def test_write_cache_matches_reference_writer(g, tmp_path):
    scene = {"pos": g["in_pos"].reshape(-1, 3), "vel": g["in_vel"], "mass": g["in_mass"],
             "tri_idx": g["in_tri"], "prim_list": g["in_prim_list"], "indices": g["in_indices"],
             "ctype": g["in_ctype"], "rest_length": g["in_rest"], "stiffness": g["in_stiff"]}
    t, c = str(tmp_path / "t.cache"), str(tmp_path / "c.cache")
    pbd.write_cache(scene, t, c, predicted=g["in_prdp"], damping=0.9, gravity=g["in_gravity"])
    assert _fields(t) == _fields(os.path.join(IO, "topol.cache"))
    assert _fields(c) == _fields(os.path.join(IO, "constr.cache"))
    # and reads back as the reference's file does
    a = pbd.read_cache(t, c)
    b = pbd.read_cache(os.path.join(IO, "topol.cache"), os.path.join(IO, "constr.cache"))
    for k in ("pos", "vel", "mass", "tri_idx", "prim_list", "indices", "ctype", "rest_length",
              "stiffness", "predicted", "gravity"):
        np.testing.assert_array_equal(a[k], b[k])
    assert a["damping"] == b["damping"]


def test_read_txt_matches_reference_reader(g):
    sc = pbd.read_txt(os.path.join(IO, "topol.txt"), os.path.join(IO, "dist.txt"), 0.75)
    np.testing.assert_array_equal(sc["pos"].ravel(), g["txt_mesh_pos"])
    np.testing.assert_array_equal(sc["tri_idx"].ravel(), g["txt_mesh_indices"])
    np.testing.assert_array_equal(sc["mass"], g["txt_mass"])
    np.testing.assert_array_equal(sc["vel"].ravel(), g["txt_vel"])
    np.testing.assert_array_equal(sc["prim_list"].ravel(), g["txt_c_prims"])
    np.testing.assert_array_equal(sc["indices"], g["txt_c_indices"])
    np.testing.assert_array_equal(sc["rest_length"], g["txt_rest"])   # powf-spelled lengths
    np.testing.assert_array_equal(sc["stiffness"], g["txt_stiff"])
    np.testing.assert_array_equal(sc["ctype"], g["txt_ctype"])


def test_windows_line_ends_and_bad_fields(tmp_path):
    src = open(os.path.join(IO, "topol.cache")).read()
    crlf = tmp_path / "crlf.cache"
    crlf.write_bytes(src.replace("\n", "\r\n").encode())
    a = pbd.read_cache(str(crlf), None)
    b = pbd.read_cache(os.path.join(IO, "topol.cache"), None)
    np.testing.assert_array_equal(a["pos"], b["pos"])
    np.testing.assert_array_equal(a["mass"], b["mass"])
    bad = tmp_path / "bad.cache"
    bad.write_text("Indices|int|0;1;x;\n")
    with pytest.raises(pbd.PBDError, match=r"bad.cache:1: not an integer"):
        pbd.read_cache(str(bad), None)
    with pytest.raises(pbd.PBDError, match="cannot open"):
        pbd.read_cache(str(tmp_path / "missing.cache"), None)
