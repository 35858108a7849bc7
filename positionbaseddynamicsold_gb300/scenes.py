"""Seeded synthetic cloth scenes in the reference's buffer layout.

The reference reads its cloths from text files that are not distributed
(PositionBasedDynamics.cpp:36-37 and others) or builds a grid in
PBDObject::Init (P/PBD_cuda.cu:644-869).  These generators produce the same
kind of buffers -- float3 positions, a ``massBuffer`` whose entries act as
inverse masses (0 = pinned), triangle indices (meshTopol) and a constraint
topology with ``primList`` (start, count) into ``indices`` -- for the
workloads this project measures.

Conventions:

* grid point (row i, column j) has id ``i*res_x + j`` and lies at
  ``origin + (j*dx, 0, i*dz)`` (P/PBD_cuda.cu:831-852);
* each quad is split into triangles (i, i+res_x, i+res_x+1) and
  (i, i+res_x+1, i+1) (P/PBD_cuda.cu:854-869);
* distance constraints lie on every triangle edge, ordered by (a, b);
  rest lengths come from the flat rest grid;
* a bending constraint sits on every interior edge: points (e0, e1, wA, wB)
  = hinge, then the opposite point of each adjacent triangle; its rest angle
  is the signed dihedral angle of the flat rest grid (0);
* ``mass`` holds the reference's massBuffer values: 1 for a free point and 0
  for a pinned one.  The reference uses massBuffer as an inverse mass in the
  projection (only ratios matter) and as the gravity gate in advection
  (P/PBD_cuda.cu:968), so a uniform physical mass maps to 1 everywhere.
"""
from __future__ import annotations

import numpy as np

DISTANCE, BENDING, ANCHOR = 0x001, 0x010, 0x100


def _dist32(a, b):
    d = (a.astype(np.float32) - b.astype(np.float32))
    return np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2]).astype(np.float32)


def grid_triangles(res_x, res_y):
    i = (np.arange(res_y - 1)[:, None] * res_x + np.arange(res_x - 1)[None, :]).ravel()
    t0 = np.stack([i, i + res_x, i + res_x + 1], 1)
    t1 = np.stack([i, i + res_x + 1, i + 1], 1)
    return np.stack([t0, t1], 1).reshape(-1, 3).astype(np.int32)


def mesh_edges(tris):
    """Unique undirected edges (a < b), sorted, plus the hinge table."""
    tris = np.asarray(tris, np.int64)
    n = int(tris.max()) + 1 if len(tris) else 0
    e = np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]], 0)
    opp = np.concatenate([tris[:, 2], tris[:, 0], tris[:, 1]], 0)
    a = np.minimum(e[:, 0], e[:, 1])
    b = np.maximum(e[:, 0], e[:, 1])
    key = a * n + b
    order = np.argsort(key, kind="stable")
    ks = key[order]
    uniq, first, counts = np.unique(ks, return_index=True, return_counts=True)
    edges = np.stack([uniq // n, uniq % n], 1).astype(np.int32)
    # hinges: keys with exactly two incident triangles
    two = counts == 2
    f = first[two]
    h_e = edges[two]
    wa = opp[order[f]]
    wb = opp[order[f + 1]]
    # orient the hinge so that wing A's triangle lists e0 before e1
    tri_a = order[f] % len(tris)
    ta = tris[tri_a]
    pos_e0 = np.argmax(ta == h_e[:, :1], axis=1)
    pos_e1 = np.argmax(ta == h_e[:, 1:2], axis=1)
    forward = (pos_e1 - pos_e0) % 3 == 1
    e0 = np.where(forward, h_e[:, 0], h_e[:, 1])
    e1 = np.where(forward, h_e[:, 1], h_e[:, 0])
    hinges = np.stack([e0, e1, wa, wb], 1).astype(np.int32)
    return edges, hinges


def dihedral(p, hinges):
    """Signed dihedral angle (float64) of each hinge (e0, e1, wA, wB)."""
    p = np.asarray(p, np.float64)
    e0, e1, wa, wb = (p[hinges[:, k]] for k in range(4))
    E = e1 - e0
    na = np.cross(wa - e0, wa - e1)
    nb = np.cross(wb - e1, wb - e0)
    el = np.linalg.norm(E, axis=1)
    return np.arctan2(np.einsum("ij,ij->i", np.cross(na, nb), E) / el,
                      np.einsum("ij,ij->i", na, nb))


def constraints_from_mesh(rest_pos, tris, dist_stiffness=1.0, bend_stiffness=0.1,
                          bending=True, edges=None):
    """Distance constraints on the mesh edges (or ``edges``) and bending on
    the interior edges, in the reference's primList layout."""
    e, hinges = mesh_edges(tris)
    if edges is not None:
        e = np.asarray(edges, np.int32)
    if not bending:
        hinges = np.zeros((0, 4), np.int32)
    nd, nb = len(e), len(hinges)
    prim_list = np.concatenate([
        np.stack([np.arange(nd) * 2, np.full(nd, 2)], 1),
        np.stack([2 * nd + np.arange(nb) * 4, np.full(nb, 4)], 1)], 0).astype(np.int32)
    indices = np.concatenate([e.ravel(), hinges.ravel()]).astype(np.int32)
    ctype = np.concatenate([np.full(nd, DISTANCE), np.full(nb, BENDING)]).astype(np.int32)
    rp = np.asarray(rest_pos, np.float32)
    rest_length = np.zeros(nd + nb, np.float32)
    rest_length[:nd] = _dist32(rp[e[:, 0]], rp[e[:, 1]])
    stiffness = np.concatenate([np.full(nd, dist_stiffness), np.full(nb, bend_stiffness)]).astype(np.float32)
    rest_angle = np.zeros(nd + nb, np.float32)
    hinge_rest = np.zeros(nd + nb, np.float32)
    if nb:
        rest_angle[nd:] = dihedral(rp, hinges).astype(np.float32)
        hinge_rest[nd:] = _dist32(rp[hinges[:, 0]], rp[hinges[:, 1]])
    return {
        "prim_list": prim_list, "indices": indices, "ctype": ctype,
        "rest_length": rest_length, "stiffness": stiffness, "rest_angle": rest_angle,
        "hinge_rest": hinge_rest, "rest_pos": np.zeros((nd + nb, 3), np.float32),
        "n_distance": nd, "n_bending": nb,
    }


def grid_cloth(res_x, res_y, size_x, size_y, origin=(0.0, 0.0, 0.0), jitter=0.0, seed=0,
               pins=None, dist_stiffness=1.0, bend_stiffness=0.1, bending=True):
    """A flat grid cloth in the xz-plane; ``pins`` lists pinned point ids."""
    dx = np.float32(size_x) / np.float32(res_x - 1)
    dz = np.float32(size_y) / np.float32(res_y - 1)
    jj, ii = np.meshgrid(np.arange(res_x), np.arange(res_y))
    rest = np.zeros((res_x * res_y, 3), np.float32)
    rest[:, 0] = np.float32(origin[0]) + jj.ravel().astype(np.float32) * dx
    rest[:, 1] = np.float32(origin[1])
    rest[:, 2] = np.float32(origin[2]) + ii.ravel().astype(np.float32) * dz
    tris = grid_triangles(res_x, res_y)
    scene = constraints_from_mesh(rest, tris, dist_stiffness, bend_stiffness, bending)
    pos = rest.copy()
    if jitter:
        rng = np.random.default_rng(seed)
        pos[:, 1] += rng.uniform(-jitter, jitter, len(pos)).astype(np.float32)
    mass = np.ones(len(pos), np.float32)
    if pins is not None:
        mass[np.asarray(pins, np.int64)] = 0.0
    scene.update({"pos": pos, "vel": np.zeros_like(pos), "mass": mass, "tri_idx": tris,
                  "res": (res_x, res_y), "n_cloth_points": len(pos), "n_cloth_tris": len(tris)})
    return scene


def icosphere(level, radius, center=(0.0, 0.0, 0.0)):
    """Icosahedron refined ``level`` times by edge midpoints, projected to the
    sphere: 10*4^level + 2 points, 20*4^level triangles."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
         (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
         (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
         (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, np.float64) / np.linalg.norm(p) for p in v]
    faces = f
    for _ in range(level):
        cache = {}

        def mid(a, b):
            k = (a, b) if a < b else (b, a)
            if k not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[k] = len(verts) - 1
            return cache[k]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    pos = (np.array(verts) * radius + np.asarray(center, np.float64)).astype(np.float32)
    return pos, np.array(faces, np.int32)


def add_static_mesh(scene, pos, tris, inst=None):
    """Append a static (massBuffer 0) triangle mesh to a scene's collision
    geometry; it carries no constraints."""
    n0 = len(scene["pos"])
    out = dict(scene)
    out["pos"] = np.concatenate([scene["pos"], pos]).astype(np.float32)
    out["vel"] = np.concatenate([scene["vel"], np.zeros_like(pos)]).astype(np.float32)
    out["mass"] = np.concatenate([scene["mass"], np.zeros(len(pos), np.float32)])
    out["tri_idx"] = np.concatenate([scene["tri_idx"], tris + n0]).astype(np.int32)
    if "point_inst" in scene:
        out["point_inst"] = np.concatenate([scene["point_inst"], np.full(len(pos), inst, np.int32)])
        out["tri_inst"] = np.concatenate([scene["tri_inst"], np.full(len(tris), inst, np.int32)])
    return out


def mean_rest_edge(scene):
    d = scene["ctype"] == DISTANCE
    return float(np.mean(scene["rest_length"][d].astype(np.float64)))


# ---------------------------------------------------------------------------
# the measured workloads
# ---------------------------------------------------------------------------

def instance_cells(scene, factor=2.0):
    """per-instance hash cell sizes: factor x each instance's mean rest edge
    (its distance constraints' rest lengths), float32 (n_instances,)"""
    inst = np.asarray(scene["point_inst"])
    d = np.nonzero(scene["ctype"] == DISTANCE)[0]
    k = inst[scene["indices"][scene["prim_list"][d, 0]]]
    n = int(inst.max()) + 1
    total = np.bincount(k, weights=scene["rest_length"][d].astype(np.float64), minlength=n)
    count = np.bincount(k, minlength=n)
    return (factor * total / np.maximum(count, 1)).astype(np.float32)


def hanging_cloth(res=32, seed=0):
    """32x32 grid over 1 m x 1 m in the xz-plane, distance (s=1) on every
    triangle edge, bending (s=0.1) on interior edges, corners 0 and res-1
    pinned, y jitter U(+-1e-3)."""
    return grid_cloth(res, res, 1.0, 1.0, jitter=1e-3, seed=seed, pins=[0, res - 1])


def drape_over_sphere(res=256, seed=0, sphere_level=5, start="release", gap=1.5e-3):
    """res^2 grid over 2 m x 2 m, flat at y = 0.5 above a fixed sphere of
    radius 0.4 at the origin (icosphere, 20*4^level triangles), jitter
    U(+-1e-4).  Collision: cell = 2 x mean rest edge, thickness 1e-3.

    start="contact": the released cloth fast-forwarded through its free fall
    (a rigid translation: nothing else acts on it before it touches) until
    its lowest point is `gap` above the sphere's top, every cloth point
    moved down by that fall height d and moving at sqrt(2 g d) downward
    (g = 9.8).  With the default gap of 1.5 thicknesses the sphere's top
    triangles are within the contact band from the first substep."""
    cloth = grid_cloth(res, res, 2.0, 2.0, origin=(-1.0, 0.5, -1.0), jitter=1e-4, seed=seed)
    sp, st = icosphere(sphere_level, 0.4)
    if start == "contact":
        d = float(cloth["pos"][:, 1].min()) - (float(sp[:, 1].max()) + gap)
        cloth["pos"][:, 1] -= np.float32(d)
        cloth["vel"][:, 1] = -np.float32(np.sqrt(2.0 * 9.8 * d))
    elif start != "release":
        raise ValueError("start must be 'release' or 'contact'")
    scene = add_static_mesh(cloth, sp, st)
    cell = 2.0 * mean_rest_edge(cloth)
    scene["colli"] = {"cell": cell, "thickness": 1e-3, "center": (0.0, 0.0, 0.0),
                      "bounded": False, "table_log2": 20}
    return scene


def folding_cloth(res=1024, seed=0, size=4.0):
    """res^2 grid over size x size (4 m), rotated 45 degrees about the
    vertical axis and tilted 30 degrees about x, lowest point 0.05 m above the
    ground plane y = 0, jitter U(+-1e-4).  Collision: self CCD, cell = 2 x
    mean rest edge, table 2^24, thickness 1e-3, ground plane."""
    cloth = grid_cloth(res, res, size, size, origin=(-size / 2, 0.0, -size / 2), jitter=1e-4,
                       seed=seed)
    p = cloth["pos"].astype(np.float64)
    c, s = np.cos(np.pi / 4), np.sin(np.pi / 4)
    ry = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])
    ct, st = np.cos(np.pi / 6), np.sin(np.pi / 6)
    rx = np.array([[1, 0, 0], [0, ct, -st], [0, st, ct]])
    p = p @ ry.T @ rx.T
    p[:, 1] += 0.05 - p[:, 1].min()
    cloth["pos"] = p.astype(np.float32)
    cell = 2.0 * mean_rest_edge(cloth)
    cloth["colli"] = {"cell": cell, "thickness": 1e-3, "center": (0.0, 0.0, 0.0),
                      "bounded": False, "table_log2": 24, "ground": 0.0}
    return cloth


def _batched_params(n, seed, side_lo, side_hi):
    """the per-instance draws of batched_cloths, in draw order"""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        side = int(rng.integers(side_lo, side_hi + 1))
        corners = np.array([0, side - 1, side * (side - 1), side * side - 1])
        npin = int(rng.integers(1, 5))
        pins = rng.choice(corners, npin, replace=False)
        r = float(rng.uniform(0.2, 0.6))
        sphere = (float(rng.uniform(-0.2, 0.2)), -r - float(rng.uniform(0.01, 0.3)),
                  float(rng.uniform(-0.2, 0.2)), r)
        out.append((side, pins, sphere))
    return out


def batched_cloth_points(n=512, seed=0, side_lo=16, side_hi=128):
    """points of every instance of batched_cloths(n, seed, ...)"""
    return [side * side for side, _, _ in _batched_params(n, seed, side_lo, side_hi)]


def batched_cloths(n=512, seed=0, side_lo=16, side_hi=128, subset=None):
    """n independent cloths, side U{side_lo..side_hi}, random pins (1-4
    corners) and one analytic sphere each (radius U(0.2, 0.6), centre below
    the cloth).  Instances are concatenated; point_inst/tri_inst tag them.
    subset: the instance indices to build (all by default); each instance is
    the same whichever others are built."""
    parts = []
    spheres = []
    keep = range(n) if subset is None else sorted(subset)
    params = _batched_params(n, seed, side_lo, side_hi)
    for k in keep:
        side, pins, sphere = params[k]
        c = grid_cloth(side, side, 1.0, 1.0, origin=(-0.5, 0.0, -0.5), jitter=1e-4,
                       seed=seed * 100003 + k, pins=pins)
        spheres.append(sphere)
        parts.append(c)
    return concat_scenes(parts, spheres)


def concat_scenes(parts, spheres=None):
    pos, vel, mass, tris, pl, idx, ct, rl, st, ra, hr = ([] for _ in range(11))
    pinst, tinst = [], []
    np0 = 0
    ni0 = 0
    for k, c in enumerate(parts):
        pos.append(c["pos"]); vel.append(c["vel"]); mass.append(c["mass"])
        tris.append(c["tri_idx"] + np0)
        p = c["prim_list"].copy(); p[:, 0] += ni0
        pl.append(p); idx.append(c["indices"] + np0)
        ct.append(c["ctype"]); rl.append(c["rest_length"]); st.append(c["stiffness"])
        ra.append(c["rest_angle"]); hr.append(c["hinge_rest"])
        pinst.append(np.full(len(c["pos"]), k, np.int32))
        tinst.append(np.full(len(c["tri_idx"]), k, np.int32))
        np0 += len(c["pos"])
        ni0 += len(c["indices"])
    out = {"pos": np.concatenate(pos), "vel": np.concatenate(vel), "mass": np.concatenate(mass),
           "tri_idx": np.concatenate(tris).astype(np.int32),
           "prim_list": np.concatenate(pl).astype(np.int32),
           "indices": np.concatenate(idx).astype(np.int32),
           "ctype": np.concatenate(ct), "rest_length": np.concatenate(rl),
           "stiffness": np.concatenate(st), "rest_angle": np.concatenate(ra),
           "hinge_rest": np.concatenate(hr), "point_inst": np.concatenate(pinst),
           "tri_inst": np.concatenate(tinst), "n_instances": len(parts)}
    out["rest_pos"] = np.zeros((len(out["ctype"]), 3), np.float32)
    if spheres is not None:
        out["spheres"] = np.asarray(spheres, np.float32)
    return out


def reference_grid(res_x, res_y, size_x, size_y, dist_stiffness=1.0, anchors=False):
    """The grid PBDObject::Init() builds (P/PBD_cuda.cu:19-153, 831-869):
    distance constraints from InitDistanceIndices' stencil (whose diagonal is
    (i, i+res_x-1)), rest lengths from the initial positions, and optionally
    the two anchor constraints on points 0 and res_y-1."""
    n = res_x * res_y
    pairs = []
    for i in range(n - res_x):
        if i % res_x == 0:
            pairs += [(i, i + 1), (i, i + res_x)]
        elif i % res_x == res_x - 1:
            pairs += [(i, i + res_x), (i, i + res_x - 1)]
        else:
            pairs += [(i, i + 1), (i, i + res_x), (i, i + res_x - 1)]
    for i in range(n - res_x, n - 1):
        pairs.append((i, i + 1))
    e = np.array(pairs, np.int32)
    scene = grid_cloth(res_x, res_y, size_x, size_y, bending=False)
    rest = scene["pos"]
    nd = len(e)
    prim_list = np.stack([np.arange(nd) * 2, np.full(nd, 2)], 1).astype(np.int32)
    indices = e.ravel().astype(np.int32)
    ctype = np.full(nd, DISTANCE, np.int32)
    rest_length = _dist32(rest[e[:, 0]], rest[e[:, 1]])
    stiffness = np.full(nd, dist_stiffness, np.float32)
    rest_pos = np.zeros((nd, 3), np.float32)
    if anchors:
        a_pts = [0, res_y - 1]
        a_rest = [rest[0], rest[res_x - 1]]
        prim_list = np.concatenate([prim_list, [[len(indices), 1], [len(indices) + 1, 1]]]).astype(np.int32)
        indices = np.concatenate([indices, a_pts]).astype(np.int32)
        ctype = np.concatenate([ctype, [ANCHOR, ANCHOR]]).astype(np.int32)
        rest_length = np.concatenate([rest_length, [0, 0]]).astype(np.float32)
        stiffness = np.concatenate([stiffness, [-1.0, -1.0]]).astype(np.float32)
        rest_pos = np.concatenate([rest_pos, np.array(a_rest, np.float32)]).astype(np.float32)
    m = len(ctype)
    scene.update({"prim_list": prim_list, "indices": indices, "ctype": ctype,
                  "rest_length": rest_length, "stiffness": stiffness,
                  "rest_angle": np.zeros(m, np.float32), "hinge_rest": np.zeros(m, np.float32),
                  "rest_pos": rest_pos, "n_distance": nd, "n_bending": 0})
    return scene
