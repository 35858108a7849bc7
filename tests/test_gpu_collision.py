"""GPU parity of the broadphase, CCD and response.

Candidate/neighbor sets and CCD hit sets are compared exactly with the
reference's own outputs (tests/golden, produced by its compiled code) and
with the oracle; positions after the response within 1e-6 m (same float
operations, same summation order), and a whole collision substep within
1e-5 m.
"""
import numpy as np
import pytest

from positionbaseddynamicsold_gb300 import scenes
from positionbaseddynamicsold_gb300.pbd import (RESPONSE_MASS_WEIGHTED, RESPONSE_REFERENCE,
                                                CollisionSolver, PBDError, PBDObject, SolverPBD,
                                                SpatialHashSystem)

pytestmark = pytest.mark.gpu


def mesh_object(pos, prdp, tri, mass=None):
    sc = {"pos": pos, "mass": np.ones(len(pos), np.float32) if mass is None else mass,
          "tri_idx": tri}
    obj = PBDObject(sc)
    obj.set_predicted(prdp)
    return obj


def test_find_neighbors_matches_reference(golden):
    g = golden("neighbors")
    obj = mesh_object(g["pos"], g["pos"], g["tri_idx"])
    shs = SpatialHashSystem(obj, g["center"], g["size"], g["cell"])
    shs.init()
    sn, nb = shs.find_neighbors_all()
    np.testing.assert_array_equal(sn, g["start_num"])
    np.testing.assert_array_equal(nb, g["nbrs"])
    np.testing.assert_array_equal(shs.find_neighbors(5), g["nbrs"][g["start_num"][5, 0]:g["start_num"][5, 0] + g["start_num"][5, 1]])


def ccd_gpu(g, hashed=False, iterations=0, response=RESPONSE_REFERENCE):
    obj = mesh_object(g["pos"], g["prdp"], g["tri_idx"])
    if hashed:
        shs = SpatialHashSystem(obj, cell_size=g["cell"], log2_table=10)
    else:
        shs = SpatialHashSystem(obj, g["center"], g["size"], g["cell"])
    shs.init()
    cs = CollisionSolver(obj, shs, thickness=float(g["thickness"]), iterations=iterations,
                         response=response)
    cs.ccd_sh_extended()
    return obj, cs


@pytest.mark.parametrize("hashed", [False, True])
def test_ccd_hit_set_matches_reference(golden, hashed):
    g = golden("ccd")
    obj, cs = ccd_gpu(g, hashed)
    ct = cs.contacts()
    assert len(ct["ids"]) == len(g["ids"])
    ref = {tuple(k): (t, tuple(w), tuple(n)) for k, t, w, n in
           zip(g["ids"].tolist(), g["t"].tolist(), g["w"].tolist(), g["n"].tolist())}
    got = {tuple(k): (t, tuple(w), tuple(n)) for k, t, w, n in
           zip(ct["ids"].tolist(), ct["t"].tolist(), ct["w"].tolist(), ct["n"].tolist())}
    assert set(got) == set(ref)
    for k in ref:
        assert got[k] == ref[k], k
    # sorted by (point, face triangle)
    key = ct["ids"][:, 0].astype(np.int64) * len(g["tri_idx"]) + ct["face"]
    assert (np.diff(key) > 0).all()


def test_vf_test_batch_matches_reference(golden):
    """ExtendedVFTest on the GPU (with its exact early exits) against the
    reference's own outputs on 1,500 random near-contact configurations:
    hit, time, barycentric weights and normal bit for bit (the reference's
    powf-spelled edge lengths only enter the inside test's epsilon)."""
    from positionbaseddynamicsold_gb300.pbd import vf_test_batch
    g = golden("vf_cases")
    hit, t, w, n = vf_test_batch(g["X"], g["P"], g["thickness"])
    np.testing.assert_array_equal(hit, g["hit"])
    h = hit.astype(bool)
    np.testing.assert_array_equal(t[h], g["t"][h])
    np.testing.assert_array_equal(w[h], g["w"][h])
    np.testing.assert_array_equal(n[h], g["n"][h])


def test_ccd_matches_oracle_pairs(orc, golden):
    g = golden("ccd")
    obj, cs = ccd_gpu(g)
    grid = orc.grid(g["center"], g["size"], g["cell"], True)
    oc, h = orc.ccd(grid, g["tri_idx"], g["pos"], g["prdp"], float(g["thickness"]))
    ct = cs.contacts()
    np.testing.assert_array_equal(ct["ids"], oc["ids"])
    np.testing.assert_array_equal(ct["face"], oc["face"])
    np.testing.assert_array_equal(ct["t"], oc["t"])
    np.testing.assert_array_equal(ct["w"], oc["w"])


@pytest.mark.parametrize("mw", [0, 1])
def test_resolve_matches_oracle(orc, golden, mw):
    g = golden("ccd")
    obj, cs = ccd_gpu(g, iterations=2, response=RESPONSE_MASS_WEIGHTED if mw else RESPONSE_REFERENCE)
    ids = cs.contacts()["ids"]
    cs.collision_resolve_new()
    want = orc.resolve_jacobi(ids, g["pos"], g["prdp"], np.ones(len(g["pos"]), np.float32), 2,
                              float(g["thickness"]), mw)
    assert np.abs(obj.predicted() - want).max() <= 1e-6


def test_resolve_reference_split_when_contacts_disjoint(orc, golden):
    """With vertex-disjoint contacts the Jacobi response is the reference's
    sequential CollisionResolveNew, up to the 2^-32 m quantisation of the
    fixed-point sums (below one float ulp of the positions here)."""
    g = golden("ccd")
    obj, cs = ccd_gpu(g, iterations=1)
    ids = cs.contacts()["ids"]
    used, keep = set(), []
    for i, row in enumerate(ids.tolist()):
        if used.isdisjoint(row):
            keep.append(i)
            used.update(row)
    sub = ids[keep]
    seq = orc.resolve_ref(sub, g["pos"], g["prdp"], 1, float(g["thickness"]))
    jac = orc.resolve_jacobi(sub, g["pos"], g["prdp"], None, 1, float(g["thickness"]), 0)
    assert len(sub) > 10
    assert np.abs(seq - jac).max() <= 1e-7


def drape_small(seed=0):
    """20x20 cloth (0.6 m) just above an icosphere (level 2, r=0.2), moving
    down at 1 m/s: contacts from the first substep."""
    cloth = scenes.grid_cloth(20, 20, 0.6, 0.6, origin=(-0.3, 0.2015, -0.3), jitter=1e-4,
                              seed=seed)
    cloth["vel"][:, 1] = -1.0
    sp, st = scenes.icosphere(2, 0.2)
    sc = scenes.add_static_mesh(cloth, sp, st)
    sc["cell"] = 2.0 * scenes.mean_rest_edge(cloth)
    return sc


def test_collision_substep_matches_oracle(orc):
    sc = drape_small()
    G = np.array([0, -9.8, 0], np.float32)
    obj = PBDObject(sc, damping=1.0, gravity=G)
    obj.prepare()
    shs = SpatialHashSystem(obj, cell_size=sc["cell"], log2_table=16)
    shs.init()
    cs = CollisionSolver(obj, shs, thickness=1e-3, iterations=1, response=RESPONSE_MASS_WEIGHTED)
    s = SolverPBD(obj)
    dt = 1.0 / 600
    s.advect(dt)
    s.project_constraint_with_colli(15, cs)
    s.integration(dt)
    _, sid, ws = orc.sort_worksets(obj.colors())
    st = {"pos": sc["pos"].copy(), "vel": sc["vel"].copy()}
    colli = {"center": (0, 0, 0), "cell": sc["cell"], "bounded": False, "thickness": 1e-3,
             "tri_idx": sc["tri_idx"], "mass_weighted": 1, "resolve_passes": 1}
    nct = orc.substep_gpu(sc, st, sid, ws, 15, dt, 1.0, G, colli=colli)
    assert nct > 0
    assert cs.stats()["contacts"] == nct
    err = np.abs(obj.positions() - st["pos"]).max()
    assert err <= 1e-5, err
    # the static sphere does not move
    ns = len(sc["pos"]) - 400
    np.testing.assert_array_equal(obj.positions()[400:], sc["pos"][400:])
    assert ns > 0


def test_collision_graph_equals_eager():
    sc = drape_small(1)
    G = np.array([0, -9.8, 0], np.float32)
    res = []
    for graph in (False, True):
        obj = PBDObject(sc, damping=1.0, gravity=G)
        obj.prepare()
        shs = SpatialHashSystem(obj, cell_size=sc["cell"], log2_table=16)
        shs.init()
        cs = CollisionSolver(obj, shs, thickness=1e-3, iterations=1, response=RESPONSE_MASS_WEIGHTED)
        s = SolverPBD(obj)
        s.step(1.0 / 600, substeps=3, iterations=15, colli=cs, use_graph=graph)
        res.append(obj.positions())
    np.testing.assert_array_equal(res[0], res[1])


@pytest.mark.parametrize("seed,h_rel", [(1, 0.2), (2, 0.5), (3, 1.0), (4, 0.5)])
def test_filters_keep_every_hit_under_deformation(orc, seed, h_rel):
    """The broadphase and distance filters drop only pairs that cannot hit:
    the GPU hit set equals the oracle's ExtendedVFTest on every pair of the
    cell neighbourhoods (no filter), with thickness comparable to the edge
    length and triangles deforming strongly during the step (corners moving
    up to ~0.4 edge lengths in random directions) on a cloth folded onto
    itself."""
    rng = np.random.default_rng(seed)
    res = 12
    cloth = scenes.grid_cloth(res, res, 1.0, 1.0, jitter=0.0, seed=seed)
    pos = cloth["pos"].astype(np.float64)
    l = 1.0 / (res - 1)
    # fold the far half back over the near half, one thickness-scale gap apart
    h = h_rel * l
    fold = pos[:, 2] > 0.5
    pos[fold, 2] = 1.0 - pos[fold, 2]
    pos[fold, 1] += 1.5 * h
    pos += rng.normal(0, 0.05 * l, pos.shape)
    prd = pos + rng.normal(0, 0.2 * l, pos.shape)
    prd[fold, 1] -= 2.0 * h      # the upper layer moves through the lower one
    pos = pos.astype(np.float32)
    prd = prd.astype(np.float32)
    tri = cloth["tri_idx"]
    cell = 2.0 * l
    obj = mesh_object(pos, prd, tri)
    shs = SpatialHashSystem(obj, cell_size=cell, log2_table=12)
    shs.init()
    cs = CollisionSolver(obj, shs, thickness=float(h), iterations=0)
    cs.ccd_sh_extended()
    got = cs.contacts()
    grid = orc.grid((0.0, 0.0, 0.0), None, cell, False)
    want, nh = orc.ccd(grid, tri, pos, prd, float(h))
    assert nh > 20
    assert len(got["ids"]) == nh
    ka = set(zip(got["ids"][:, 0].tolist(), got["face"].tolist()))
    kb = set(zip(want["ids"][:, 0].tolist(), want["face"].tolist()))
    assert ka == kb


def test_solver_retargeted_to_a_larger_object():
    """A collision solver moved to another object (other point count) sizes
    its per-point buffers for it: same contacts and response as a fresh
    solver; a response before the first detection on the new target is
    refused instead of touching stale buffers."""
    def obj_of(res, seed):
        sc = scenes.drape_over_sphere(res=res, seed=seed, sphere_level=2)
        o = PBDObject(sc, damping=1.0, gravity=np.array([0.0, -9.8, 0.0], np.float32))
        o.prepare()
        prd = sc["pos"].copy()
        prd[: sc["n_cloth_points"], 1] -= np.float32(0.12)   # through the sphere's top
        o.set_predicted(prd)
        shs = SpatialHashSystem(o, cell_size=sc["colli"]["cell"], log2_table=14)
        shs.init()
        return o, shs

    a, sa = obj_of(12, 1)
    b, sb = obj_of(40, 2)
    cs = CollisionSolver(a, sa, thickness=1e-3, iterations=1, response=RESPONSE_MASS_WEIGHTED)
    cs.ccd_sh_extended()
    cs.set_target(b)
    cs.set_acce_struct(sb)
    with pytest.raises(PBDError):
        cs.collision_resolve_new()
    cs.ccd_sh_extended()
    cs.collision_resolve_new()
    got = b.predicted()
    b2, sb2 = obj_of(40, 2)
    fresh = CollisionSolver(b2, sb2, thickness=1e-3, iterations=1,
                            response=RESPONSE_MASS_WEIGHTED)
    fresh.ccd_sh_extended()
    assert fresh.stats()["contacts"] > 0
    assert cs.stats()["contacts"] == fresh.stats()["contacts"]
    fresh.collision_resolve_new()
    np.testing.assert_array_equal(got, b2.predicted())


@pytest.mark.parametrize("graph", [False, True])
def test_overlapped_detection_equals_sequential(graph):
    """A detection run beside the following sweep (side stream, copy of the
    iteration's starting positions; the response waits for it) gives the
    sequential substeps' results bit for bit: drape with self contacts and
    a fold onto the ground plane."""
    for sc, log2 in ((scenes.drape_over_sphere(res=64, seed=4, sphere_level=3,
                                               start="contact"), 16),
                     (scenes.folding_cloth(res=64, seed=4, size=0.5), 16)):
        G = np.array([0, -9.8, 0], np.float32)
        res = []
        for overlap in (False, True):
            obj = PBDObject(sc, damping=1.0, gravity=G)
            obj.prepare()
            shs = SpatialHashSystem(obj, cell_size=sc["colli"]["cell"], log2_table=log2)
            shs.init()
            cs = CollisionSolver(obj, shs, thickness=1e-3, iterations=1,
                                 response=RESPONSE_MASS_WEIGHTED)
            cs.set_overlap(overlap)
            s = SolverPBD(obj)
            if "ground" in sc["colli"]:
                s.set_ground(True, sc["colli"]["ground"])
            s.step(1.0 / 600, substeps=30, iterations=15, colli=cs, use_graph=graph)
            res.append((obj.positions(), obj.velocities(), cs.stats()["contacts"]))
        np.testing.assert_array_equal(res[0][0], res[1][0])
        np.testing.assert_array_equal(res[0][1], res[1][1])
        assert res[0][2] == res[1][2]


@pytest.mark.parametrize("mode,key", [(1, "narrow"), (2, "vfccd"), (3, "vfdcd"), (4, "vf")])
def test_other_vf_tests_match_reference(golden, mode, key):
    """NarrowVFCCDTest, VFCCDTest, VFDCDTest and VFTest on the GPU against the
    reference's own outputs on the 1,500 near-contact cases: hit and time
    (and, where the fixture holds them, weights and normal) bit for bit,
    misses included (a miss keeps what the last evaluated time wrote)."""
    from positionbaseddynamicsold_gb300.pbd import vf_test_batch
    g = golden("vf_cases")
    hit, t, w, n = vf_test_batch(g["X"], g["P"], g["thickness"], mode)
    np.testing.assert_array_equal(hit, g[key + "_hit"])
    np.testing.assert_array_equal(t, g[key + "_t"])
    if key + "_w" in g:
        np.testing.assert_array_equal(w, g[key + "_w"])
        np.testing.assert_array_equal(n, g[key + "_n"])
    assert hit.sum() > 300


@pytest.mark.parametrize("mode", [1, 2, 3, 4])
def test_detection_with_other_vf_tests_matches_oracle(orc, mode):
    """The detection run with CCD_SH_Narrow's, VFCCDTest's, VFDCDTest's or
    CCD_SH's test in place of ExtendedVFTest: the same contacts (ids, face,
    t, w, n) as the oracle's pair driver with that test, on a cloth folded
    onto itself whose upper layer moves through the lower one."""
    rng = np.random.default_rng(40 + mode)
    res = 14
    cloth = scenes.grid_cloth(res, res, 1.0, 1.0, jitter=0.0, seed=mode)
    pos = cloth["pos"].astype(np.float64)
    l = 1.0 / (res - 1)
    h = 0.4 * l
    fold = pos[:, 2] > 0.5
    pos[fold, 2] = 1.0 - pos[fold, 2]
    pos[fold, 1] += 1.5 * h
    pos += rng.normal(0, 0.05 * l, pos.shape)
    prd = pos + rng.normal(0, 0.1 * l, pos.shape)
    prd[fold, 1] -= 2.2 * h
    pos = pos.astype(np.float32)
    prd = prd.astype(np.float32)
    tri = cloth["tri_idx"]
    cell = 2.0 * l
    obj = mesh_object(pos, prd, tri)
    shs = SpatialHashSystem(obj, cell_size=cell, log2_table=12)
    shs.init()
    cs = CollisionSolver(obj, shs, thickness=float(h), iterations=0)
    cs.set_vf_test(mode)
    cs.ccd_sh_extended()
    got = cs.contacts()
    orc.lib.orc_set_vf_test(mode)
    try:
        grid = orc.grid((0.0, 0.0, 0.0), None, cell, False)
        want, nh = orc.ccd(grid, tri, pos, prd, float(h))
    finally:
        orc.lib.orc_set_vf_test(0)
    assert nh > 10
    np.testing.assert_array_equal(got["ids"], want["ids"])
    np.testing.assert_array_equal(got["face"], want["face"])
    np.testing.assert_array_equal(got["t"], want["t"])
    np.testing.assert_array_equal(got["w"], want["w"])
    np.testing.assert_array_equal(got["n"], want["n"])


@pytest.mark.parametrize("case", ["a", "b"])
def test_old_response_matches_oracle(orc, golden, case):
    """CollisionResolve + VFResolve (the older response) on the GPU: three
    calls in a row on the detected contacts, positions and per-point
    resolve counters equal the oracle's (which is pinned to the reference's
    compiled code) run on the same contacts in the same stored order (the
    GPU's detection stores them by point, then face)."""
    g = golden("ccd")
    r = golden("resolve_old")
    obj = mesh_object(g["pos"], r[case + "_prdp0"], g["tri_idx"])
    shs = SpatialHashSystem(obj, g["center"], g["size"], g["cell"])
    shs.init()
    cs = CollisionSolver(obj, shs, thickness=float(g["thickness"]), iterations=1)
    cs.ccd_sh_extended()
    ids = cs.contacts()["ids"]
    assert len(ids) == len(r[case + "_ids"]) > 100
    assert {tuple(v) for v in ids.tolist()} == {tuple(v) for v in r[case + "_ids"].tolist()}
    prd = r[case + "_prdp0"]
    rt = np.zeros(len(g["pos"]), np.int32)
    for k in range(3):
        cs.collision_resolve_old()
        prd = orc.resolve_old(ids, g["pos"], prd, rt, float(g["thickness"]))
        np.testing.assert_array_equal(obj.predicted(), prd)
        np.testing.assert_array_equal(cs.resolve_times(), rt)
    assert rt.sum() > 0
    cs.resolve_times(reset=True)
    assert cs.resolve_times().sum() == 0
