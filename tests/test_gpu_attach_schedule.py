"""Anchors as moving attachments and the stiffness schedule as a choice:

* every schedule (k = 1-(1-s)^(1/(iter+1)) of the reference's GPU kernel,
  k = 1 of its CPU path, k = s) matches the oracle in both GS launch forms:
  bit for bit on a distance-only cloth for k = 1 and k = s, within 1e-5 m
  where device and host powf may round k differently or with bending;
* a per-type stiffness change after creation equals creating the object with
  that stiffness;
* anchor targets moved every substep (an animated attachment) match the
  oracle stepping the same targets, and bad anchor arguments are refused.
"""
import numpy as np
import pytest

from positionbaseddynamicsold_gb300 import scenes
from positionbaseddynamicsold_gb300.pbd import (ANCHOR, BENDING, DISTANCE, GS_CLUSTER,
                                                SCHEDULE_DIRECT, SCHEDULE_REFERENCE,
                                                SCHEDULE_UNIT, PBDError, PBDObject, SolverPBD)

pytestmark = pytest.mark.gpu

G = np.array([0.0, -9.8, 0.0], np.float32)
DT = 1.0 / 600


def oracle_run(orc, sc, colors, k, iters, schedule, targets=None):
    _, sid, ws = orc.sort_worksets(colors)
    st = {"pos": sc["pos"].copy(), "vel": sc["vel"].copy()}
    orc.set_stiffness_schedule(schedule)
    try:
        for j in range(k):
            if targets is not None:
                sc["rest_pos"][targets[0]] = targets[1](j)
            orc.substep_gpu(sc, st, sid, ws, iters, DT, 1.0, G)
    finally:
        orc.set_stiffness_schedule(SCHEDULE_REFERENCE)
    return st


@pytest.mark.parametrize("schedule", [SCHEDULE_REFERENCE, SCHEDULE_UNIT, SCHEDULE_DIRECT])
@pytest.mark.parametrize("form", ["per-color", "resident"])
def test_schedules_match_oracle(orc, schedule, form):
    sc = scenes.grid_cloth(20, 20, 1.0, 1.0, jitter=1e-3, seed=2, pins=[0, 19], bending=False,
                           dist_stiffness=0.7)
    sc["pos"][:, 0] *= 1.02
    obj = PBDObject(sc, damping=1.0, gravity=G)
    obj.prepare()
    obj.set_stiffness_schedule(schedule)
    assert obj.stiffness_schedule() == schedule
    s = SolverPBD(obj)
    if form == "resident":
        s.set_gs_path(GS_CLUSTER)
    s.step(DT, 6, 12, None, True)
    st = oracle_run(orc, sc, obj.colors(), 6, 12, schedule)
    if schedule == SCHEDULE_REFERENCE:
        # device powf against the host's: k may differ in its last bit
        assert np.abs(obj.positions() - st["pos"]).max() <= 1e-5
    else:
        np.testing.assert_array_equal(obj.positions(), st["pos"])


@pytest.mark.parametrize("schedule", [SCHEDULE_UNIT, SCHEDULE_DIRECT])
def test_schedules_with_bending_match_oracle(orc, schedule):
    sc = scenes.hanging_cloth(24, seed=3)
    obj = PBDObject(sc, damping=1.0, gravity=G)
    obj.prepare()
    obj.set_stiffness_schedule(schedule)
    s = SolverPBD(obj)
    s.step(DT, 4, 15, None, True)
    st = oracle_run(orc, sc, obj.colors(), 4, 15, schedule)
    assert np.abs(obj.positions() - st["pos"]).max() <= 1e-5


def test_schedule_change_recaptures_the_graph():
    sc = scenes.hanging_cloth(16, seed=4)
    out = []
    for change in (False, True):
        obj = PBDObject(sc, damping=1.0, gravity=G)
        obj.prepare()
        s = SolverPBD(obj)
        if change:
            s.step(DT, 1, 10, None, True)          # captured with the default schedule
            obj.set_stiffness_schedule(SCHEDULE_UNIT)
            s.step(DT, 1, 10, None, True)
        else:
            s.step(DT, 1, 10, None, True)
            obj.set_stiffness_schedule(SCHEDULE_UNIT)
            s.step(DT, 1, 10, None, False)         # eager: no graph involved
        out.append(obj.positions())
    np.testing.assert_array_equal(out[0], out[1])


@pytest.mark.parametrize("form", ["per-color", "resident"])
def test_stiffness_change_equals_fresh_object(form):
    sc = scenes.grid_cloth(30, 30, 1.0, 1.0, jitter=1e-3, seed=5, pins=[0, 29])
    sc2 = dict(sc)
    sc2["stiffness"] = sc["stiffness"].copy()
    sc2["stiffness"][sc["ctype"] == BENDING] = 0.35
    sc2["stiffness"][sc["ctype"] == DISTANCE] = 0.8
    out = []
    for scene, change in ((sc, True), (sc2, False)):
        obj = PBDObject(scene, damping=1.0, gravity=G)
        obj.prepare()
        s = SolverPBD(obj)
        if form == "resident":
            s.set_gs_path(GS_CLUSTER)
        s.step(DT, 2, 10, None, True)
        if change:
            obj.set_stiffness(BENDING, 0.35)
            obj.set_stiffness(DISTANCE, 0.8)
        out.append(obj)
    # both stepped their first 2 substeps with their own stiffness; reset the
    # changed one to the fresh one's state and step both the same way
    a, b = out
    a.set_positions(b.positions())
    a.set_velocities(b.velocities())
    for obj in (a, b):
        s = SolverPBD(obj)
        if form == "resident":
            s.set_gs_path(GS_CLUSTER)
        s.step(DT, 5, 10, None, True)
    np.testing.assert_array_equal(a.positions(), b.positions())


def test_moving_anchor_targets_match_oracle(orc):
    sc = scenes.reference_grid(12, 12, 1.0, 1.0, anchors=True)
    anchors = np.nonzero(sc["ctype"] == ANCHOR)[0]
    base = sc["rest_pos"][anchors].copy()

    def target(j):
        a = 0.05 * (j + 1)
        return base + np.array([[0.1 * np.sin(a), 0.05 * a, 0.1 * (1 - np.cos(a))]] * len(base),
                               np.float32)

    obj = PBDObject(sc, damping=1.0, gravity=G)
    obj.prepare()
    s = SolverPBD(obj)
    for j in range(20):
        obj.set_anchor_targets(anchors, target(j))
        s.step(DT, 1, 8, None, True)
    st = oracle_run(orc, dict(sc, rest_pos=sc["rest_pos"].copy()), obj.colors(), 20, 8,
                    SCHEDULE_REFERENCE, targets=(anchors, target))
    assert np.abs(obj.positions() - st["pos"]).max() <= 1e-6
    # the attachment pulled the anchored points along
    assert np.abs(obj.positions()[[0, 11]] - sc["pos"][[0, 11]]).max() > 0.05


def test_anchor_target_arguments_are_checked():
    sc = scenes.reference_grid(6, 6, 1.0, 1.0, anchors=True)
    obj = PBDObject(sc)
    obj.prepare()
    with pytest.raises(PBDError):
        obj.set_anchor_targets([0], [[0.0, 0.0, 0.0]])          # prim 0 is a distance prim
    with pytest.raises(PBDError):
        obj.set_anchor_targets([len(sc["ctype"])], [[0.0, 0.0, 0.0]])
    a = int(np.nonzero(sc["ctype"] == ANCHOR)[0][0])
    with pytest.raises(PBDError):
        obj.set_anchor_targets([a], [[np.nan, 0.0, 0.0]])
    with pytest.raises(PBDError):
        obj.set_stiffness_schedule(7)


def test_schedule_against_reference_gpu_kernel_fixture(golden):
    """The GPU sweeps with stiffness below 1 against the reference's own
    ProjectContraintsGPUKernel (its code run on the host; the fixture of
    tests/golden/gpu_kernel_schedule.npz): the same coloring, 8 sweeps,
    within 1e-5 m (device powf against the host's)."""
    g = golden("gpu_kernel_schedule")
    sc = scenes.grid_cloth(11, 9, 1.0, 0.8, jitter=2e-2, seed=5, bending=False, pins=[0, 10])
    np.testing.assert_array_equal(sc["prim_list"], g["prim_list"])
    sc["stiffness"] = g["stiffness"].copy()
    sc["mass"] = g["mass"].copy()
    obj = PBDObject(sc, damping=1.0, gravity=np.zeros(3, np.float32))
    obj.prepare()
    _, sid = obj.sorted()
    np.testing.assert_array_equal(sid, g["sorted_prim_id"])
    np.testing.assert_array_equal(obj.worksets(), g["worksets"])
    obj.set_predicted(g["prdp"])
    SolverPBD(obj).project_constraint(8)
    assert np.abs(obj.predicted() - g["out"]).max() <= 1e-5
