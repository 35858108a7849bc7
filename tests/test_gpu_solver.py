"""GPU parity of the constraint path against the oracle (pinned to the
reference by tests/test_oracle_golden.py).

Integer work (adjacency, coloring, color sort, worksets) must match exactly.
Positions after one substep must match within 1e-5 m max-abs in FP32; the
distance-only case with stiffness 1 is expected to be bit-exact because the
kernels perform the oracle's float operations in the same order.
"""
import numpy as np
import pytest

from positionbaseddynamicsold_gb300 import scenes
from positionbaseddynamicsold_gb300.pbd import (ANCHOR, DISTANCE, PBDObject, SolverPBD)

pytestmark = pytest.mark.gpu

G = np.array([0.0, -9.8, 0.0], np.float32)


def hinge_rest(sc):
    hr = np.zeros(len(sc["ctype"]), np.float32)
    b = np.nonzero(sc["ctype"] == scenes.BENDING)[0]
    for p in b:
        s = sc["prim_list"][p, 0]
        e0, e1 = sc["indices"][s], sc["indices"][s + 1]
        d = sc["pos"][e1].astype(np.float64) - sc["pos"][e0].astype(np.float64)
        hr[p] = np.sqrt((d * d).sum())
    return hr


@pytest.mark.parametrize("res,bending", [(16, True), (32, True), (12, False)])
def test_adjacency_coloring_sort(orc, res, bending):
    sc = scenes.grid_cloth(res, res, 1.0, 1.0, bending=bending, pins=[0, res - 1])
    obj = PBDObject(sc)
    sn, adj = obj.adjacency()
    osn, oadj = orc.prim2prims(sc["prim_list"], sc["indices"], len(sc["pos"]))
    np.testing.assert_array_equal(sn, osn)
    np.testing.assert_array_equal(adj, oadj)
    sweeps = obj.edge_coloring()
    col = obj.colors()
    ocol, osw = orc.edge_coloring(sc["prim_list"], sc["indices"], len(sc["pos"]), "gpu")
    np.testing.assert_array_equal(col, ocol)
    assert osw <= sweeps < osw + 16
    obj.sort_edges_colors()
    assert obj.eval_worksets() == col.max() + 1
    sc_, sp = obj.sorted()
    oc, osid, ows = orc.sort_worksets(col)
    np.testing.assert_array_equal(sc_, oc)
    np.testing.assert_array_equal(sp, osid)
    np.testing.assert_array_equal(obj.worksets(), ows)
    # every color is a set of constraints with pairwise distinct points
    for c in range(col.max() + 1):
        pts = np.concatenate([sc["indices"][sc["prim_list"][p, 0]:sc["prim_list"][p, 0] + sc["prim_list"][p, 1]]
                              for p in np.nonzero(col == c)[0]])
        assert len(np.unique(pts)) == len(pts)


def test_reference_grid_init(orc):
    """PBDObject::Init() grid (stencil + anchors) built by the library equals
    the reference layout restated in scenes.reference_grid."""
    obj = PBDObject.grid(9, 9, 1.0, 1.0, ct=DISTANCE | ANCHOR, stiffness=(1.0, 0.1, -1.0))
    ref = scenes.reference_grid(9, 9, 1.0, 1.0, anchors=True)
    np.testing.assert_array_equal(obj.positions(), ref["pos"])
    sn, adj = obj.adjacency()
    osn, oadj = orc.prim2prims(ref["prim_list"], ref["indices"], len(ref["pos"]))
    np.testing.assert_array_equal(sn, osn)
    np.testing.assert_array_equal(adj, oadj)


def gpu_substeps(sc, k, iters, dt, damping, colors=None, graph=False):
    obj = PBDObject(sc, damping=damping, gravity=G)
    if colors is None:
        obj.prepare()
    else:
        obj.set_colors(colors)
        obj.sort_edges_colors()
    s = SolverPBD(obj)
    if graph:
        s.step(dt, substeps=k, iterations=iters, use_graph=True)
    else:
        for _ in range(k):
            s.advect(dt)
            s.project_constraint(iters)
            s.integration(dt)
    return obj


def oracle_substeps(orc, sc, col, k, iters, dt, damping):
    _, sid, ws = orc.sort_worksets(col)
    st = {"pos": sc["pos"].copy(), "vel": sc["vel"].copy()}
    for _ in range(k):
        orc.substep_gpu(sc, st, sid, ws, iters, dt, damping, G)
    return st


def test_substep_hanging_cloth_32(orc):
    """32x32 hanging cloth (distance s=1 + bending s=0.1, two pinned
    corners), one substep dt=1/600 with 20 colored GS iterations."""
    sc = scenes.hanging_cloth(32, seed=1)
    obj = gpu_substeps(sc, 1, 20, 1.0 / 600, 0.9)
    st = oracle_substeps(orc, sc, obj.colors(), 1, 20, 1.0 / 600, 0.9)
    err = np.abs(obj.positions() - st["pos"]).max()
    assert err <= 1e-5, err
    assert np.abs(obj.velocities() - st["vel"]).max() <= 1e-5 * 600
    # pins stay put
    np.testing.assert_array_equal(obj.positions()[[0, 31]], sc["pos"][[0, 31]])
    r = obj.residual()
    ro, _, _ = orc.residual(sc, obj.predicted(), hinge_rest(sc))
    assert abs(r - ro) <= 1e-6 * max(ro, 1e-30)


def test_distance_only_bit_exact(orc):
    sc = scenes.grid_cloth(24, 24, 1.0, 1.0, jitter=1e-3, seed=3, pins=[0, 23], bending=False)
    sc["pos"][:, 0] *= 1.02  # pre-stretch so every constraint acts
    obj = gpu_substeps(sc, 10, 20, 1.0 / 600, 0.9)
    st = oracle_substeps(orc, sc, obj.colors(), 10, 20, 1.0 / 600, 0.9)
    np.testing.assert_array_equal(obj.positions(), st["pos"])
    np.testing.assert_array_equal(obj.velocities(), st["vel"])


def test_graph_step_equals_eager(orc):
    sc = scenes.hanging_cloth(32, seed=2)
    a = gpu_substeps(sc, 10, 20, 1.0 / 600, 0.9, graph=False)
    b = gpu_substeps(sc, 10, 20, 1.0 / 600, 0.9, colors=a.colors(), graph=True)
    np.testing.assert_array_equal(a.positions(), b.positions())


def test_anchor_constraints(orc):
    sc = scenes.reference_grid(8, 8, 1.0, 1.0, anchors=True)
    sc["pos"] = sc["pos"] + np.float32(0.01)  # move everything off the anchors' rest points
    obj = gpu_substeps(sc, 1, 5, 1.0 / 600, 1.0)
    st = oracle_substeps(orc, sc, obj.colors(), 1, 5, 1.0 / 600, 1.0)
    assert np.abs(obj.positions() - st["pos"]).max() <= 1e-6


def test_sphere_and_ground_obstacles(orc):
    """ColliWithShpGrd's sphere push and the ground plane on the GPU."""
    sc = scenes.grid_cloth(10, 10, 1.2, 1.2, origin=(-0.6, 0.95, -0.6), bending=False)
    obj = PBDObject(sc, damping=1.0, gravity=G)
    obj.prepare()
    s = SolverPBD(obj)
    s.set_sphere(True, (0.0, 0.0, 0.0), 1.0)
    s.advect(1.0 / 60)
    s.project_constraint(3)
    p = obj.predicted()
    d = np.linalg.norm(p.astype(np.float64), axis=1)
    assert (d >= 1.0 - 1e-5).all()
    s.set_sphere(False)
    s.set_ground(True, 0.9)
    s.project_constraint(1)
    assert (obj.predicted()[:, 1] >= 0.9).all()


@pytest.mark.parametrize("res", [32, 100])
def test_cluster_path_equals_per_color(orc, res):
    """The cluster-resident sweep (all points in distributed shared memory,
    colors separated by cluster barriers) gives the per-color launches'
    result bit for bit, with and without the analytic obstacles."""
    from positionbaseddynamicsold_gb300.pbd import GS_CLUSTER, GS_PER_COLOR
    sc = scenes.grid_cloth(res, res, 1.0, 1.0, origin=(-0.5, 0.9, -0.5), jitter=1e-3, seed=6,
                           pins=[0, res - 1])
    out = []
    for path in (GS_PER_COLOR, GS_CLUSTER):
        obj = PBDObject(sc, damping=0.9, gravity=G)
        obj.prepare()
        s = SolverPBD(obj)
        s.set_gs_path(path)
        assert s.gs_path() == path
        s.set_sphere(True, (0.0, 0.0, 0.0), 1.0)
        for _ in range(3):
            s.advect(1.0 / 600)
            s.project_constraint(20)
            s.integration(1.0 / 600)
        s.step(1.0 / 600, substeps=2, iterations=20, use_graph=True)
        out.append(obj.positions())
    np.testing.assert_array_equal(out[0], out[1])
    # the per-color form is checked against the oracle by the other tests
    obj = PBDObject(sc, damping=0.9, gravity=G)
    obj.prepare()
    assert SolverPBD(obj).gs_path() == GS_PER_COLOR
