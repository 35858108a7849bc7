"""The resident form of the Gauss-Seidel sweep (every point in the shared
memory of one thread-block cluster of S = 1..16 blocks, colors separated by
cluster barriers, stiffness factors from a per-sweep table) gives bit for
bit the result of the per-color launches, for every cluster size that holds
the object: several sweeps per launch, one sweep per launch between
collision passes, the analytic ground and sphere inside the launch,
anchors, and stiffness values beyond the table."""
import numpy as np
import pytest

from positionbaseddynamicsold_gb300 import scenes
from positionbaseddynamicsold_gb300.pbd import (GS_CLUSTER, GS_PER_COLOR, PBDError,
                                                RESPONSE_MASS_WEIGHTED, CollisionSolver,
                                                PBDObject, SolverPBD, SpatialHashSystem)

pytestmark = pytest.mark.gpu

G = np.array([0.0, -9.8, 0.0], np.float32)
DT = 1.0 / 600


def make(sc, colli=False):
    obj = PBDObject(sc, damping=1.0, gravity=G)
    obj.prepare()
    s = SolverPBD(obj)
    cs = None
    if colli:
        shs = SpatialHashSystem(obj, cell_size=sc["colli"]["cell"], log2_table=16)
        shs.init()
        cs = CollisionSolver(obj, shs, thickness=sc["colli"]["thickness"], iterations=1,
                             response=RESPONSE_MASS_WEIGHTED)
        obj._keep = shs
        if "ground" in sc["colli"]:
            s.set_ground(True, sc["colli"]["ground"])
    return obj, s, cs


def run(sc, size, substeps, iterations, colli=False, use_graph=True):
    """size None: per-color launches; else the resident form with S = size"""
    obj, s, cs = make(sc, colli)
    if size is not None:
        s.set_gs_path(GS_CLUSTER)
        s.set_gs_cluster(size)
        assert s.gs_path() == GS_CLUSTER
        assert s.gs_cluster() == size
    s.step(DT, substeps, iterations, cs, use_graph)
    return obj.positions(), obj.velocities()


@pytest.mark.parametrize("size", [1, 2, 4, 8, 16])
def test_resident_equals_per_color_without_collisions(size):
    # every sweep of a substep in one launch
    sc = scenes.grid_cloth(90, 90, 1.0, 1.0, jitter=1e-3, seed=5, pins=[0, 89])
    ref = run(sc, None, 5, 15)
    got = run(sc, size, 5, 15)
    np.testing.assert_array_equal(got[0], ref[0])
    np.testing.assert_array_equal(got[1], ref[1])


@pytest.mark.parametrize("size", [4, 16])
def test_resident_equals_per_color_with_collisions(size):
    # one sweep per launch between CCD / response passes
    sc = scenes.drape_over_sphere(res=64, seed=1, sphere_level=3)
    ref = run(sc, None, 40, 15, colli=True)
    got = run(sc, size, 40, 15, colli=True)
    np.testing.assert_array_equal(got[0], ref[0])
    np.testing.assert_array_equal(got[1], ref[1])


@pytest.mark.parametrize("size", [1, 8])
def test_resident_equals_per_color_with_ground(size):
    sc = scenes.folding_cloth(res=96, seed=2)
    ref = run(sc, None, 30, 15, colli=True)
    got = run(sc, size, 30, 15, colli=True)
    np.testing.assert_array_equal(got[0], ref[0])


@pytest.mark.parametrize("size", [1, 16])
def test_resident_equals_per_color_with_anchors_eager(size):
    sc = scenes.reference_grid(32, 32, 1.0, 1.0, anchors=True)
    ref = run(sc, None, 10, 20, use_graph=False)
    got = run(sc, size, 10, 20, use_graph=False)
    np.testing.assert_array_equal(got[0], ref[0])


def test_resident_stiffness_values_beyond_the_table():
    # 40 distinct stiffness values: 8 from the table, the rest computed per record
    sc = scenes.grid_cloth(48, 48, 1.0, 1.0, jitter=1e-3, seed=9, pins=[0, 47])
    rng = np.random.default_rng(0)
    sc["stiffness"] = rng.choice(np.linspace(0.05, 1.0, 40).astype(np.float32),
                                 len(sc["stiffness"])).astype(np.float32)
    ref = run(sc, None, 4, 12)
    got = run(sc, 2, 4, 12)
    np.testing.assert_array_equal(got[0], ref[0])


def test_resident_sizes_that_do_not_hold_the_object_are_refused():
    sc = scenes.grid_cloth(200, 200, 1.0, 1.0, jitter=1e-3, seed=3)   # 40,000 points
    obj, s, _ = make(sc)
    s.set_gs_path(GS_CLUSTER)
    s.set_gs_cluster(1)          # one block cannot hold 640 KB of points
    with pytest.raises(PBDError):
        s.step(DT, 1, 5, None, True)
    s.set_gs_cluster(0)          # the largest size that fits
    assert s.gs_cluster() in (4, 8, 16)
    s.step(DT, 1, 5, None, True)


def test_small_object_planned_after_a_large_one_keeps_the_large_ones_launch():
    # the resident kernel's shared-memory limit is a process-wide attribute:
    # planning a small object after a large one must leave the large
    # object's launches (more shared memory per block) valid
    big = scenes.grid_cloth(120, 120, 1.0, 1.0, jitter=1e-3, seed=11, pins=[0, 119])
    small = scenes.grid_cloth(20, 20, 1.0, 1.0, jitter=1e-3, seed=12, pins=[0, 19])
    ref = run(big, None, 2, 10)
    obj_a, s_a, _ = make(big)
    s_a.set_gs_path(GS_CLUSTER)
    s_a.set_gs_cluster(4)
    s_a.step(DT, 1, 10, None, False)        # plans A: 14,400 points over 4 blocks
    obj_b, s_b, _ = make(small)
    s_b.set_gs_path(GS_CLUSTER)
    s_b.set_gs_cluster(4)
    s_b.step(DT, 1, 10, None, False)        # plans B: 400 points over 4 blocks
    s_a.step(DT, 1, 10, None, False)        # A launches again with its larger share
    np.testing.assert_array_equal(obj_a.positions(), ref[0])
