"""The vertex-face hash search's pairs, exactly, against a brute force of its
definition: every (point, triangle) pair of the reference's candidate set
(CCD_SH_Extended, P/CCD.cpp:1541-1586: the triangle's centroid cell lies in
the 27-cell neighbourhood of a centroid cell of one of the point's incident
triangles) whose swept boxes are within 3.61 h of each other (Euclidean gap;
a sliver triangle's box unbounded) -- of one instance, the point's own
triangles left out.  Centroids, cells and boxes follow the kernels' float32
expressions.

Cases: the hashed grid; cells finer than the triangles (incident cells
spread beyond a 2 x 2 x 2 block); a sliver (the search window is then the
whole neighbourhood); a triangle that repeats a corner point; a bounded
grid (cells outside it hold nothing); a batch with a cell size per
instance.
"""
import numpy as np
import pytest

from positionbaseddynamicsold_gb300 import scenes
from positionbaseddynamicsold_gb300.pbd import (RESPONSE_MASS_WEIGHTED, CollisionSolver,
                                                PBDObject, SpatialHashSystem)

pytestmark = pytest.mark.gpu

H = 1e-3
G = np.array([0.0, -9.8, 0.0], np.float32)
f32 = np.float32


def sliver(a, b, c):
    e1, e2 = b - a, c - a
    n = np.stack([e1[:, 1] * e2[:, 2] - e1[:, 2] * e2[:, 1],
                  e1[:, 2] * e2[:, 0] - e1[:, 0] * e2[:, 2],
                  e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]], 1)
    nn = (n * n).sum(1)
    return ~(nn > f32(1e-10) * ((e1 * e1).sum(1) * (e2 * e2).sum(1)))


def brute_pairs(pos, prd, tris, cell, start, h, size=None, point_inst=None, inst_cells=None):
    tris = np.asarray(tris, np.int64)
    n, nt = len(pos), len(tris)
    a, b, c = prd[tris[:, 0]], prd[tris[:, 1]], prd[tris[:, 2]]
    cen = ((a + b) + c) / f32(3)
    tinst = point_inst[tris[:, 0]] if point_inst is not None else np.zeros(nt, np.int64)
    cl = np.broadcast_to(np.asarray(cell, f32), (nt, 3))
    if inst_cells is not None:
        cl = np.asarray(inst_cells, f32)[tinst]
    tc = np.floor((cen - np.asarray(start, f32)) / cl).astype(np.int64)
    inside = np.ones(nt, bool)
    if size is not None:
        inside = np.all((tc >= 0) & (tc < np.asarray(size)), 1)
    v6 = np.stack([a, b, c, pos[tris[:, 0]], pos[tris[:, 1]], pos[tris[:, 2]]], 0)
    tlo, thi = v6.min(0), v6.max(0)
    sl = sliver(a, b, c) | sliver(pos[tris[:, 0]], pos[tris[:, 1]], pos[tris[:, 2]])
    tlo[sl], thi[sl] = -np.inf, np.inf
    margin = f32(3.61) * f32(h) * f32(1.001) + f32(2e-6)
    m2 = margin * margin
    plo = np.minimum(pos, prd)
    phi = np.maximum(pos, prd)
    inc = [[] for _ in range(n)]
    for t, (i, j, k) in enumerate(tris):
        for v in (i, j, k):
            inc[v].append(t)
    out = []
    for v in range(n):
        cells = tc[[t for t in inc[v] if inside[t]]]
        if len(cells) == 0:
            continue
        with np.errstate(invalid="ignore"):
            g = np.maximum(f32(0), np.maximum(tlo - phi[v], plo[v] - thi))
        g = np.nan_to_num(g, nan=0.0)
        ok = inside & (((g[:, 0] * g[:, 0] + g[:, 1] * g[:, 1]) + g[:, 2] * g[:, 2]) <= m2)
        if point_inst is not None:
            ok &= tinst == point_inst[v]
        cand = np.nonzero(ok)[0]
        near = np.zeros(len(cand), bool)
        for m in cells:
            near |= np.all(np.abs(tc[cand] - m) <= 1, 1)
        for t in cand[near]:
            if v not in tris[t]:
                out.append((v, t))
    out = np.array(sorted(out), np.int32).reshape(-1, 2)
    return out


def search(sc, prd, cell, log2=16, grid_center=(0.0, 0.0, 0.0), grid_size=None,
           inst_cells=None):
    obj = PBDObject(sc, damping=1.0, gravity=G)
    obj.prepare()
    obj.set_predicted(prd)
    shs = SpatialHashSystem(obj, grid_center=grid_center, grid_size=grid_size,
                            cell_size=cell, log2_table=log2)
    if inst_cells is not None:
        shs.set_instance_cells(inst_cells)
    shs.init()
    cs = CollisionSolver(obj, shs, thickness=H, iterations=1, response=RESPONSE_MASS_WEIGHTED)
    cs.ccd_sh_extended()
    assert cs.stats()["overflow"] == 0
    return cs.pairs()


def crumpled(res=24, seed=0, amp=0.004, motion=0.003):
    """a small cloth folded over itself with jitter, and a predicted step"""
    rng = np.random.default_rng(seed)
    sc = scenes.grid_cloth(res, res, 0.1, 0.1, origin=(-0.05, 0.0, -0.05), jitter=1e-4,
                           seed=seed)
    pos = sc["pos"].astype(np.float64)
    # fold the far half back over the near half, 2 mm above it
    far = pos[:, 2] > 0.0
    pos[far, 2] = -pos[far, 2]
    pos[far, 1] += 0.002
    pos += rng.normal(0, amp / 4, pos.shape)
    sc["pos"] = pos.astype(np.float32)
    prd = (pos + rng.normal(0, motion, pos.shape)).astype(np.float32)
    return sc, prd


@pytest.mark.parametrize("cell_rel", [2.0, 0.6])
def test_pairs_hashed(cell_rel):
    sc, prd = crumpled()
    cell = f32(cell_rel * scenes.mean_rest_edge(sc))
    got = search(sc, prd, cell)
    want = brute_pairs(sc["pos"], prd, sc["tri_idx"], (cell,) * 3, (0, 0, 0), H)
    assert len(want) > 1000
    np.testing.assert_array_equal(got, want)


def test_pairs_with_a_sliver():
    sc, prd = crumpled(seed=1)
    tris = sc["tri_idx"].copy()
    # a collinear triangle: its box is unbounded, reach becomes infinite
    res = 24
    r = res // 2
    tris = np.concatenate([tris, [[r * res + 2, r * res + 3, r * res + 4]]]).astype(np.int32)
    p = sc["pos"].copy()
    p[r * res + 2: r * res + 5] = [[0.0, 0.01, 0.0], [0.001, 0.01, 0.0], [0.002, 0.01, 0.0]]
    q = prd.copy()
    q[r * res + 2: r * res + 5] = p[r * res + 2: r * res + 5]
    sc = dict(sc, pos=p, tri_idx=tris)
    cell = f32(2.0 * scenes.mean_rest_edge(sc))
    got = search(sc, q, cell)
    want = brute_pairs(p, q, tris, (cell,) * 3, (0, 0, 0), H)
    assert np.any(want[:, 1] == len(tris) - 1)
    np.testing.assert_array_equal(got, want)


def test_pairs_with_a_repeated_corner():
    """a triangle whose first two corners are one point: that point's
    incidence list holds it twice, and both of its incident-cell slots are
    written"""
    sc, prd = crumpled(seed=4)
    res = 24
    r = res // 2
    tris = np.concatenate([sc["tri_idx"], [[r * res + 5, r * res + 5, r * res + 6]]]).astype(np.int32)
    sc = dict(sc, tri_idx=tris)
    cell = f32(2.0 * scenes.mean_rest_edge(sc))
    got = search(sc, prd, cell)
    want = brute_pairs(sc["pos"], prd, tris, (cell,) * 3, (0, 0, 0), H)
    assert np.any(want[:, 1] == len(tris) - 1)
    np.testing.assert_array_equal(got, want)


def test_pairs_bounded_grid():
    sc, prd = crumpled(seed=2)
    cell = f32(2.0 * scenes.mean_rest_edge(sc))
    size = (10, 6, 10)   # smaller than the cloth: some cells fall outside
    center = np.array([0.01, 0.0, -0.01], np.float32)
    got = search(sc, prd, (cell,) * 3, grid_center=center, grid_size=size)
    shift = (np.asarray(size, np.float32) * cell) / f32(2)
    start = center - shift
    want = brute_pairs(sc["pos"], prd, sc["tri_idx"], (cell,) * 3, start, H, size=size)
    assert len(want) > 100
    np.testing.assert_array_equal(got, want)


def test_pairs_batch_instance_cells():
    parts, prds = [], []
    for k in range(3):
        sc, prd = crumpled(res=12 + 5 * k, seed=3 + k)
        parts.append(sc)
        prds.append(prd)
    batch = scenes.concat_scenes(parts)
    prd = np.concatenate(prds).astype(np.float32)
    cells = scenes.instance_cells(batch)
    got = search(batch, prd, float(cells.mean()), inst_cells=cells)
    ic = np.repeat(np.asarray(cells, np.float32).reshape(-1, 1), 3, 1) \
        if np.ndim(cells) == 1 else np.asarray(cells, np.float32)
    want = brute_pairs(batch["pos"], prd, batch["tri_idx"], None, (0, 0, 0), H,
                       point_inst=batch["point_inst"], inst_cells=ic)
    assert len(want) > 1000
    np.testing.assert_array_equal(got, want)
