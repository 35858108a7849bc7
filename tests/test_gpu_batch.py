"""Batched cloths: many instances in one object, one launch per color phase.

Every kernel sees all instances at once; constraints never cross instances,
the spatial hash mixes the instance into the bucket and the narrowphase only
pairs a point with triangles of its own instance.  So a batch must give each
instance exactly (bit for bit) what simulating that cloth alone gives, with
collisions and per-instance spheres, and must match the oracle.
"""
import numpy as np
import pytest

from positionbaseddynamicsold_gb300 import scenes
from positionbaseddynamicsold_gb300.pbd import (RESPONSE_MASS_WEIGHTED, CollisionSolver,
                                                PBDObject, SolverPBD, SpatialHashSystem)

pytestmark = pytest.mark.gpu

G = np.array([0.0, -9.8, 0.0], np.float32)
DT = 1.0 / 600


def make_batch(sides, seed=0):
    """Overlapping cloths (all centred on the origin), each pinned at one
    corner and moving down onto its own sphere."""
    rng = np.random.default_rng(seed)
    parts, spheres = [], []
    for k, side in enumerate(sides):
        c = scenes.grid_cloth(side, side, 0.3, 0.3, origin=(-0.15, 0.1, -0.15), jitter=1e-3,
                              seed=seed * 1000 + k, pins=[0])
        c["vel"][:, 1] = -float(rng.uniform(0.5, 2.0))
        parts.append(c)
        spheres.append((float(rng.uniform(-0.05, 0.05)), -0.05, float(rng.uniform(-0.05, 0.05)),
                        0.15))
    return parts, np.asarray(spheres, np.float32)


def run(sc, substeps, spheres=None, single_sphere=None, cell=None, inst_cells=None):
    obj = PBDObject(sc, damping=0.95, gravity=G)
    obj.prepare()
    shs = SpatialHashSystem(obj, cell_size=cell, log2_table=14)
    shs.init()
    if inst_cells is not None:
        shs.set_instance_cells(inst_cells)
    cs = CollisionSolver(obj, shs, thickness=2e-3, iterations=1, response=RESPONSE_MASS_WEIGHTED)
    s = SolverPBD(obj)
    if spheres is not None:
        s.set_instance_spheres(spheres)
    if single_sphere is not None:
        s.set_sphere(True, single_sphere[:3], float(single_sphere[3]))
    for _ in range(substeps):
        s.advect(DT)
        s.project_constraint_with_colli(10, cs)
        s.integration(DT)
    return obj.positions(), cs.stats()


def test_batch_equals_instances_alone():
    sides = [8, 13, 9, 16, 11]
    parts, spheres = make_batch(sides)
    batch = scenes.concat_scenes(parts)
    cell = 2.0 * scenes.mean_rest_edge(parts[0])
    got, st = run(batch, 40, spheres=spheres, cell=cell)
    assert st["contacts"] >= 0 and st["overflow"] == 0
    off = 0
    for k, c in enumerate(parts):
        alone, _ = run(c, 40, single_sphere=spheres[k], cell=cell)
        n = len(c["pos"])
        np.testing.assert_array_equal(got[off:off + n], alone)
        off += n
    # the spheres acted: some points were pushed out to the sphere surface
    d = np.linalg.norm(got[:len(parts[0]["pos"])] - spheres[0, :3], axis=1)
    assert d.min() >= spheres[0, 3] - 1e-4


def test_batch_with_per_instance_cells_equals_instances_alone():
    """Each instance hashed with its own cell size (2 x its mean rest edge)
    gives exactly what simulating it alone with that cell gives."""
    sides = [6, 15, 9, 20]
    parts, spheres = make_batch(sides, seed=5)
    batch = scenes.concat_scenes(parts)
    cells = scenes.instance_cells(batch)
    assert len(np.unique(cells)) == len(sides)
    got, st = run(batch, 40, spheres=spheres, cell=float(cells.mean()), inst_cells=cells)
    assert st["overflow"] == 0
    off = 0
    for k, c in enumerate(parts):
        alone, _ = run(c, 40, single_sphere=spheres[k], cell=float(cells[k]))
        n = len(c["pos"])
        np.testing.assert_array_equal(got[off:off + n], alone)
        off += n


def test_batch_collision_substep_matches_oracle(orc):
    """Overlapping instances with self-collision: GPU vs oracle (which pairs
    only points and triangles of the same instance)."""
    parts, _ = make_batch([10, 12, 9], seed=3)
    for c in parts:
        c["vel"][:, 1] = 0.0
        # fold each cloth onto itself so self contacts appear
        c["pos"][len(c["pos"]) // 2:, 1] += np.float32(2.5e-3)
        c["vel"][len(c["pos"]) // 2:, 1] = -1.5
    batch = scenes.concat_scenes(parts)
    cell = 2.0 * scenes.mean_rest_edge(parts[0])
    obj = PBDObject(batch, damping=1.0, gravity=G)
    obj.prepare()
    shs = SpatialHashSystem(obj, cell_size=cell, log2_table=12)
    shs.init()
    cs = CollisionSolver(obj, shs, thickness=2e-3, iterations=1, response=RESPONSE_MASS_WEIGHTED)
    s = SolverPBD(obj)
    s.advect(DT)
    s.project_constraint_with_colli(15, cs)
    s.integration(DT)
    _, sid, ws = orc.sort_worksets(obj.colors())
    st = {"pos": batch["pos"].copy(), "vel": batch["vel"].copy()}
    colli = {"center": (0, 0, 0), "cell": cell, "bounded": False, "thickness": 2e-3,
             "tri_idx": batch["tri_idx"], "mass_weighted": 1, "resolve_passes": 1,
             "tri_inst": np.ascontiguousarray(batch["tri_inst"]),
             "point_inst": np.ascontiguousarray(batch["point_inst"])}
    nct = orc.substep_gpu(batch, st, sid, ws, 15, DT, 1.0, G, colli=colli)
    assert cs.stats()["contacts"] == nct
    assert np.abs(obj.positions() - st["pos"]).max() <= 1e-5
