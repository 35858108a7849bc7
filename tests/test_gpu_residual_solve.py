"""Substeps solved to a residual target: the device-side loop (CUDA graph
WHILE node) stops where the residual first reaches the target, its result
equals the oracle's substep with that many sweeps, and the graph and eager
forms agree bit for bit, with and without collisions.  With collisions the
loop equals the same substep composed of the public fixed-step calls, with
no chunk, one or two."""
import numpy as np
import pytest

from positionbaseddynamicsold_gb300 import scenes
from positionbaseddynamicsold_gb300.pbd import (RESPONSE_MASS_WEIGHTED, SCHEDULE_DIRECT,
                                                CollisionSolver, PBDObject, SolverPBD,
                                                SpatialHashSystem)

pytestmark = pytest.mark.gpu

G = np.array([0.0, -9.8, 0.0], np.float32)
DT = 1.0 / 600


def hanging(res=16, seed=0):
    return scenes.grid_cloth(res, res, 0.6, 0.6, jitter=1e-3, seed=seed, pins=[0, res - 1])


def test_loop_stops_at_target_and_matches_oracle(orc):
    sc = hanging()
    # residual after k sweeps from the same advected state (plain loop, one
    # chunk of 1 sweep per check)
    trace = []
    for k in range(1, 13):
        obj = PBDObject(sc, damping=1.0, gravity=G)
        obj.prepare()
        s = SolverPBD(obj)
        s.advect(DT)
        s.project_constraint(k)
        trace.append(obj.residual_stretch())
    # a target between the 6th and 7th sweep's residual stops after 7 sweeps
    target = 0.5 * (trace[5] + trace[6])
    assert trace[6] < target < trace[5]
    for graph in (False, True):
        obj = PBDObject(sc, damping=1.0, gravity=G)
        obj.prepare()
        s = SolverPBD(obj)
        s.step_to_residual(DT, 1, target=target, max_sweeps=30, chunk=1, use_graph=graph)
        st = s.solve_stats()
        assert st["last_sweeps"] == 7 and st["reached"] == 1
        # bit for bit the fixed-count substep of 7 sweeps on the GPU ...
        ref = PBDObject(sc, damping=1.0, gravity=G)
        ref.prepare()
        rs = SolverPBD(ref)
        rs.advect(DT)
        rs.project_constraint(7)
        rp = ref.predicted()
        rs.integration(DT)
        np.testing.assert_array_equal(obj.positions(), ref.positions())
        p0 = sc["pos"] + DT * (sc["vel"] + DT * G * sc["mass"][:, None])
        np.testing.assert_allclose(obj.correction(), rp - p0, rtol=0, atol=1e-6)
        # ... and the oracle's within the bending kernel's 1e-5 m parity bound
        _, sid, ws = orc.sort_worksets(obj.colors())
        ost = {"pos": sc["pos"].copy(), "vel": sc["vel"].copy()}
        orc.substep_gpu(sc, ost, sid, ws, 7, DT, 1.0, G)
        assert np.abs(obj.positions() - ost["pos"]).max() <= 1e-5


def test_max_sweeps_caps_the_loop():
    sc = hanging(seed=1)
    obj = PBDObject(sc, damping=1.0, gravity=G)
    obj.prepare()
    s = SolverPBD(obj)
    s.step_to_residual(DT, 3, target=0.0, max_sweeps=12, chunk=5)
    st = s.solve_stats()
    assert st["substeps"] == 3 and st["sweeps"] == 30 and st["reached"] == 0


def drape(seed=0):
    cloth = scenes.grid_cloth(20, 20, 0.6, 0.6, origin=(-0.3, 0.2015, -0.3), jitter=1e-4,
                              seed=seed)
    cloth["vel"][:, 1] = -1.0
    sp, st = scenes.icosphere(2, 0.2)
    sc = scenes.add_static_mesh(cloth, sp, st)
    sc["cell"] = 2.0 * scenes.mean_rest_edge(cloth)
    return sc


@pytest.mark.parametrize("colli", [False, True])
def test_graph_equals_eager(colli):
    sc = drape() if colli else hanging(seed=2)
    res = []
    for graph in (False, True):
        obj = PBDObject(sc, damping=1.0, gravity=G)
        obj.prepare()
        s = SolverPBD(obj)
        cs = None
        if colli:
            shs = SpatialHashSystem(obj, cell_size=sc["cell"], log2_table=16)
            shs.init()
            cs = CollisionSolver(obj, shs, thickness=1e-3, iterations=1,
                                 response=RESPONSE_MASS_WEIGHTED)
        s.step_to_residual(DT, 4, target=1e-5, max_sweeps=40, chunk=10 if colli else 4,
                           colli=cs, use_graph=graph)
        s.step_to_residual(DT, 4, target=1e-5, max_sweeps=40, chunk=10 if colli else 4,
                           colli=cs, use_graph=graph)
        res.append((obj.positions(), s.solve_stats()))
        if graph:
            outer, body = s.residual_graph_kernels()
            assert outer > 0 and body > 0
    np.testing.assert_array_equal(res[0][0], res[1][0])
    assert res[0][1] == res[1][1]
    assert res[0][1]["substeps"] == 8


def drape_solver(sc):
    obj = PBDObject(sc, damping=1.0, gravity=G)
    obj.prepare()
    # k = s in every sweep, so a sweep of the loop is one project_constraint(1)
    obj.set_stiffness_schedule(SCHEDULE_DIRECT)
    s = SolverPBD(obj)
    shs = SpatialHashSystem(obj, cell_size=sc["cell"], log2_table=16)
    shs.init()
    cs = CollisionSolver(obj, shs, thickness=1e-3, iterations=1, response=RESPONSE_MASS_WEIGHTED)
    return obj, s, shs, cs


@pytest.mark.parametrize("chunks", [0, 1, 2])
def test_collision_loop_equals_composed_calls(chunks):
    """advect; the contacts of the advected positions; per chunk 10 x (sweep,
    response) and the detection from the chunk's final positions; the
    response to the last contacts; integrate.  No chunk (target above the
    residual): the last contacts are those of the advected positions."""
    sc = drape(seed=3)
    got = []
    for graph in (False, True):
        obj, s, shs, cs = drape_solver(sc)
        s.step_to_residual(DT, 1, target=1.0 if chunks == 0 else 0.0,
                           max_sweeps=max(10, 10 * chunks), chunk=10, colli=cs, use_graph=graph)
        assert s.solve_stats()["last_sweeps"] == 10 * chunks
        got.append((obj.positions(), cs.stats()["contacts"]))
    obj, s, shs, cs = drape_solver(sc)
    s.advect(DT)
    cs.ccd_sh_extended()
    assert cs.stats()["contacts"] > 0
    for _ in range(chunks):
        for _ in range(10):
            s.project_constraint(1)
            cs.collision_resolve_new()
        cs.ccd_sh_extended()
    cs.collision_resolve_new()
    s.integration(DT)
    for pos, nct in got:
        np.testing.assert_array_equal(pos, obj.positions())
        assert nct == cs.stats()["contacts"]
