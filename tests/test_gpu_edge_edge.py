"""Edge-edge CCD on the GPU against the oracle (oracle/pbd_oracle.c,
orc_ee_test / orc_ccd_ee_brute / orc_collision_resolve_jacobi_ee; the
reference declares the contact kind only, so the oracle's known answers in
test_ee_oracle.py pin the arithmetic):

* the test on random near-crossing edge pairs: hit, t, s, u and the side
  bit for bit;
* detection over two cloth patches passing through each other: the same
  contacts as testing every edge pair (so the edge hash, the low-corner
  reporting rule and the distance bound lose nothing);
* the pair count: exactly the overlapping edge boxes, within an instance
  in batches;
* one response pass over the vertex-face and edge-edge contacts together:
  bit for bit;
* two crossing strips that vertex-face CCD cannot see pass through each
  other without it and stay apart with it; graphs equal eager steps with it
  on; it is off by default.
"""
import numpy as np
import pytest

from positionbaseddynamicsold_gb300 import scenes
from positionbaseddynamicsold_gb300.pbd import (RESPONSE_MASS_WEIGHTED, CollisionSolver,
                                                PBDObject, SolverPBD, SpatialHashSystem,
                                                ee_test_batch)

pytestmark = pytest.mark.gpu

H = 1e-3
G = np.array([0.0, -9.8, 0.0], np.float32)


def random_cases(n, seed):
    rng = np.random.default_rng(seed)
    X = np.zeros((n, 4, 3), np.float32)
    P = np.zeros((n, 4, 3), np.float32)
    for i in range(n):
        c = rng.uniform(-0.5, 0.5, 3)
        da = rng.normal(size=3)
        db = rng.normal(size=3)
        la, lb = rng.uniform(0.01, 0.3, 2)
        sa, sb = rng.uniform(-0.2, 1.2, 2)
        a0 = c - sa * la * da / np.linalg.norm(da)
        a1 = a0 + la * da / np.linalg.norm(da)
        b0 = c - sb * lb * db / np.linalg.norm(db)
        b1 = b0 + lb * db / np.linalg.norm(db)
        nrm = np.cross(da, db)
        nrm /= np.linalg.norm(nrm)
        kind = i % 4
        if kind == 0:      # A passes through B's line during the step
            off, mv = rng.uniform(0.0005, 0.01), rng.uniform(0.0, 0.03)
            X[i] = [a0 + off * nrm, a1 + off * nrm, b0, b1]
            P[i] = [a0 + (off - mv) * nrm, a1 + (off - mv) * nrm, b0, b1]
        elif kind == 1:    # both move, rotating a little
            X[i] = [a0, a1, b0, b1] + rng.normal(0, 0.003, (4, 3))
            P[i] = X[i] + rng.normal(0, 0.006, (4, 3))
        elif kind == 2:    # within a few thicknesses the whole step
            off = rng.uniform(-4 * H, 4 * H)
            X[i] = [a0 + off * nrm, a1 + off * nrm, b0, b1]
            P[i] = X[i] + rng.normal(0, 0.0005, (4, 3))
        else:              # far apart
            X[i] = [a0 + 0.1 * nrm, a1 + 0.1 * nrm, b0, b1]
            P[i] = X[i] + rng.normal(0, 0.01, (4, 3))
    return X, P


def test_edge_edge_test_matches_oracle(orc):
    X, P = random_cases(2000, 1)
    hit, tsu, m0 = ee_test_batch(X, P, np.full(len(X), H, np.float32))
    nh = 0
    for i in range(len(X)):
        oh, t, s, u, om0 = orc.ee_test(X[i], P[i], H)
        assert bool(hit[i]) == oh, i
        if oh:
            nh += 1
            assert (tsu[i, 0], tsu[i, 1], tsu[i, 2]) == (np.float32(t), np.float32(s),
                                                         np.float32(u)), i
            np.testing.assert_array_equal(m0[i], om0)
    assert nh > 200


def crossing_patches(res=14, gap=0.003, travel=0.008, seed=0):
    """patch A (xz-plane) above patch B (rotated 90 degrees about y and
    jittered), one mesh; A's predicted positions go down through B"""
    rng = np.random.default_rng(seed)
    a = scenes.grid_cloth(res, res, 0.5, 0.5, origin=(-0.25, gap, -0.25))
    b = scenes.grid_cloth(res, res, 0.5, 0.5, origin=(-0.25, 0.0, -0.25))
    rot = np.array([[0, 0, 1], [0, 1, 0], [-1, 0, 0]], np.float32)
    bpos = (b["pos"] @ rot.T).astype(np.float32)
    bpos += rng.normal(0, 2e-4, bpos.shape).astype(np.float32)
    pos = np.concatenate([a["pos"], bpos]).astype(np.float32)
    tris = np.concatenate([a["tri_idx"], b["tri_idx"] + len(a["pos"])]).astype(np.int32)
    sc = scenes.constraints_from_mesh(pos, tris, 1.0, 0.1, bending=False)
    n = len(pos)
    sc.update({"pos": pos, "vel": np.zeros_like(pos), "mass": np.ones(n, np.float32),
               "tri_idx": tris})
    prd = pos.copy()
    prd[: len(a["pos"]), 1] -= travel
    prd[: len(a["pos"])] += rng.normal(0, 5e-4, (len(a["pos"]), 3)).astype(np.float32)
    return sc, prd


def detect(sc, prd, ee=True):
    obj = PBDObject(sc, damping=1.0, gravity=G)
    obj.prepare()
    obj.set_predicted(prd)
    shs = SpatialHashSystem(obj, cell_size=2.0 * scenes.mean_rest_edge(sc), log2_table=16)
    shs.init()
    cs = CollisionSolver(obj, shs, thickness=H, iterations=1, response=RESPONSE_MASS_WEIGHTED)
    cs.set_edge_edge(ee)
    cs.ccd_sh_extended()
    return obj, shs, cs


def test_detection_equals_every_pair_tested(orc):
    sc, prd = crossing_patches()
    obj, shs, cs = detect(sc, prd)
    edges = cs.ee_edges()
    ref_edges, _ = scenes.mesh_edges(sc["tri_idx"])
    np.testing.assert_array_equal(edges, ref_edges)
    pairs, ids, tsu, m0 = cs.ee_contacts()
    opairs, otsu, om0 = orc.ccd_ee_brute(edges, None, sc["pos"], prd, H)
    assert len(opairs) > 50
    np.testing.assert_array_equal(pairs, opairs)
    np.testing.assert_array_equal(tsu, otsu)
    np.testing.assert_array_equal(m0, om0)
    np.testing.assert_array_equal(ids, np.concatenate([edges[opairs[:, 0]], edges[opairs[:, 1]]], 1))
    st = cs.ee_stats()
    assert st["contacts"] == len(opairs) and st["candidates"] >= st["contacts"]


def box_pairs_brute(edges, x, p, h, point_inst=None):
    """every pair of edges without a shared point (of one instance) whose
    swept boxes, grown by 2 h * 1.001 + 4e-6 like the edge hash's, overlap"""
    f = np.float32
    grow = f(2) * f(h) * f(1.001) + f(4e-6)
    pts = np.stack([x[edges[:, 0]], x[edges[:, 1]], p[edges[:, 0]], p[edges[:, 1]]], 0)
    lo, hi = pts.min(0) - grow, pts.max(0) + grow
    i, j = np.triu_indices(len(edges), 1)
    ok = np.all((lo[i] <= hi[j]) & (lo[j] <= hi[i]), 1)
    ok &= ~((edges[i, 0] == edges[j, 0]) | (edges[i, 0] == edges[j, 1]) |
            (edges[i, 1] == edges[j, 0]) | (edges[i, 1] == edges[j, 1]))
    if point_inst is not None:
        ok &= point_inst[edges[i, 0]] == point_inst[edges[j, 0]]
    return int(ok.sum())


def test_every_overlapping_box_pair_reported_once():
    """the hash's pair count is exactly the number of overlapping edge boxes:
    nothing lost, nothing reported twice (same cell, low-corner rule)"""
    sc, prd = crossing_patches(seed=1)
    obj, shs, cs = detect(sc, prd)
    st = cs.ee_stats()
    assert st["pairs"] == box_pairs_brute(cs.ee_edges(), sc["pos"], prd, H) > 1000


def test_batch_pairs_stay_within_instances(orc):
    """two instances of crossing patches in the same place: the pairs are
    each instance's own, and the contacts those of testing every pair of one
    instance"""
    parts = [crossing_patches(seed=s) for s in (0, 5)]
    batch = scenes.concat_scenes([sc for sc, _ in parts])
    prd = np.concatenate([q for _, q in parts]).astype(np.float32)
    obj, shs, cs = detect(batch, prd)
    edges = cs.ee_edges()
    inst = batch["point_inst"]
    st = cs.ee_stats()
    assert st["pairs"] == box_pairs_brute(edges, batch["pos"], prd, H, inst)
    assert st["pairs"] < box_pairs_brute(edges, batch["pos"], prd, H)
    pairs, ids, tsu, m0 = cs.ee_contacts()
    opairs, otsu, om0 = orc.ccd_ee_brute(edges, inst, batch["pos"], prd, H)
    assert len(opairs) > 100
    assert np.all(inst[edges[opairs[:, 0], 0]] == inst[edges[opairs[:, 1], 0]])
    np.testing.assert_array_equal(pairs, opairs)
    np.testing.assert_array_equal(tsu, otsu)
    np.testing.assert_array_equal(m0, om0)


def test_response_matches_oracle(orc):
    sc, prd = crossing_patches(seed=3)
    obj, shs, cs = detect(sc, prd)
    vf = cs.contacts()
    _, ids, _, m0 = cs.ee_contacts()
    assert len(ids) > 0
    cs.collision_resolve_new()
    got = obj.predicted()
    ref = orc.resolve_jacobi_ee(vf["ids"], ids, m0, sc["pos"], prd, sc["mass"], 1, H, True)
    np.testing.assert_array_equal(got, ref)


def strips(w=1e-4):
    """strip A (long in x, narrow in z) falls through strip B (long in z,
    narrow in x, pinned): only their long edges cross"""
    a = np.array([[0, 0.01, -w], [1, 0.01, -w], [0, 0.01, w], [1, 0.01, w]], np.float32)
    b = np.array([[0.5 - w, 0, -1], [0.5 + w, 0, -1], [0.5 - w, 0, 1], [0.5 + w, 0, 1]],
                 np.float32)
    pos = np.concatenate([a - [0.5, 0, 0], b - [0.5, 0, 0]]).astype(np.float32)
    tris = np.array([[0, 2, 3], [0, 3, 1], [4, 6, 7], [4, 7, 5]], np.int32)
    sc = scenes.constraints_from_mesh(pos, tris, 1.0, 0.1, bending=False)
    mass = np.array([1, 1, 1, 1, 0, 0, 0, 0], np.float32)
    sc.update({"pos": pos, "vel": np.zeros_like(pos), "mass": mass, "tri_idx": tris})
    prd = pos.copy()
    prd[:4, 1] = -0.01
    return sc, prd


@pytest.mark.parametrize("ee", [False, True])
def test_strips_cross_only_without_edge_edge(ee):
    sc, prd = strips()
    obj = PBDObject(sc, damping=1.0, gravity=G)
    obj.prepare()
    obj.set_predicted(prd)
    shs = SpatialHashSystem(obj, cell_size=0.25, log2_table=12)
    shs.init()
    cs = CollisionSolver(obj, shs, thickness=H, iterations=1, response=RESPONSE_MASS_WEIGHTED)
    cs.set_edge_edge(ee)
    cs.ccd_sh_extended()
    assert cs.stats()["contacts"] == 0            # vertex-face CCD sees nothing
    cs.collision_resolve_new()
    p = obj.predicted()
    if ee:
        assert len(cs.ee_contacts()[0]) > 0
        # A held above B (B is pinned): each point moves by the mean of its
        # contacts' corrections, about the full 2 h + travel
        assert p[:4, 1].min() >= 0.99 * 2 * H
        np.testing.assert_array_equal(p[4:], prd[4:])
    else:
        assert p[:4, 1].max() < 0                  # passed through


def test_edge_edge_off_by_default_and_graph_equals_eager():
    sc = scenes.drape_over_sphere(res=40, seed=2, sphere_level=2)
    out = {}
    for ee in (False, True):
        for graph in (False, True):
            obj = PBDObject(sc, damping=1.0, gravity=G)
            obj.prepare()
            shs = SpatialHashSystem(obj, cell_size=sc["colli"]["cell"], log2_table=16)
            shs.init()
            cs = CollisionSolver(obj, shs, thickness=H, iterations=1,
                                 response=RESPONSE_MASS_WEIGHTED)
            if ee:
                cs.set_edge_edge(True)
            s = SolverPBD(obj)
            s.step(1.0 / 600, 150, 15, cs, graph)
            out[(ee, graph)] = obj.positions()
    np.testing.assert_array_equal(out[(True, False)], out[(True, True)])
    np.testing.assert_array_equal(out[(False, False)], out[(False, True)])
