"""Constraint sets derived from a triangle mesh on the device
(pbd_mesh_constraints / pbd_object_create_mesh) equal the host builder's
(scenes.constraints_from_mesh): the same edges and hinges in the same order,
the same float32 rest lengths bit for bit, rest angles within one float32
ulp (both take atan2 in float64; the libraries may round the last double
bit differently), and an object built on the device steps exactly like one
built from the host arrays."""
import time

import numpy as np
import pytest

from positionbaseddynamicsold_gb300 import scenes
from positionbaseddynamicsold_gb300.pbd import PBDObject, SolverPBD, mesh_constraints

pytestmark = pytest.mark.gpu

G = np.array([0.0, -9.8, 0.0], np.float32)


def random_mesh(seed):
    """a jittered grid with some triangles removed and a fan of three
    triangles on one edge (non-manifold: that edge gets no hinge)"""
    rng = np.random.default_rng(seed)
    sc = scenes.grid_cloth(21, 13, 1.0, 0.7, jitter=0.0)
    pos = sc["pos"] + rng.normal(0, 0.02, sc["pos"].shape).astype(np.float32)
    tris = sc["tri_idx"]
    keep = rng.random(len(tris)) > 0.1
    tris = tris[keep]
    a, b = tris[0, 0], tris[0, 1]
    extra = np.array([[a, b, 5], [b, a, 7]], np.int32)
    return pos.astype(np.float32), np.concatenate([tris, extra]).astype(np.int32)


def meshes():
    g = scenes.grid_cloth(33, 17, 1.0, 0.5)
    yield "grid", g["pos"], g["tri_idx"]
    sp, st = scenes.icosphere(3, 0.4)
    yield "icosphere", sp.astype(np.float32), st.astype(np.int32)
    b = scenes.batched_cloths(6, seed=2, side_lo=5, side_hi=12)
    yield "batch", b["pos"], b["tri_idx"]
    p, t = random_mesh(1)
    yield "random", p, t


def compare(got, ref):
    for k in ("prim_list", "indices", "ctype", "rest_length", "stiffness", "rest_pos"):
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
    assert got["n_distance"] == ref["n_distance"] and got["n_bending"] == ref["n_bending"]
    np.testing.assert_array_max_ulp(got["rest_angle"], ref["rest_angle"], maxulp=1)


@pytest.mark.parametrize("case", ["grid", "icosphere", "batch", "random"])
def test_device_constraints_equal_host_builder(case):
    name, pos, tris = next(m for m in meshes() if m[0] == case)
    ref = scenes.constraints_from_mesh(pos, tris, 1.0, 0.1)
    got = mesh_constraints(pos, tris, 1.0, 0.1)
    compare(got, ref)
    assert ref["n_bending"] > 0


def test_device_built_object_steps_like_host_built():
    sc = scenes.grid_cloth(40, 40, 1.0, 1.0, jitter=1e-3, seed=4, pins=[0, 39])
    a = PBDObject(sc, damping=1.0, gravity=G)
    b = PBDObject.from_mesh(sc["pos"], sc["tri_idx"], sc["mass"], rest_pos=None,
                            stiffness=(1.0, 0.1), gravity=G)
    # the host builder takes its rest shape from the un-jittered grid
    rest = scenes.grid_cloth(40, 40, 1.0, 1.0)["pos"]
    c = PBDObject.from_mesh(sc["pos"], sc["tri_idx"], sc["mass"], rest_pos=rest,
                            stiffness=(1.0, 0.1), gravity=G)
    assert a.n_prims == b.n_prims == c.n_prims
    outs = []
    for obj in (a, c):
        obj.prepare()
        s = SolverPBD(obj)
        s.step(1.0 / 600, 8, 15, None, True)
        outs.append(obj.positions())
    np.testing.assert_array_equal(outs[0], outs[1])


def test_large_mesh_build_time():
    sc = scenes.grid_cloth(512, 512, 2.0, 2.0)
    t0 = time.perf_counter()
    ref = scenes.constraints_from_mesh(sc["pos"], sc["tri_idx"], 1.0, 0.1)
    t1 = time.perf_counter()
    got = mesh_constraints(sc["pos"], sc["tri_idx"], 1.0, 0.1)
    t2 = time.perf_counter()
    compare(got, ref)
    print("512^2 constraint set: host builder %.3f s, device %.3f s" % (t1 - t0, t2 - t1))
