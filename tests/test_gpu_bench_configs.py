"""Parity at the benchmark's own configurations.

bench.py times three workloads; each is rebuilt here exactly as bench.py
builds it (its make_workload and setup: the same scene, hash table size,
thickness, response, stiffness and iteration count), driven by the GPU to
the state bench.py times, and checked against the oracle from that state:

* drape256 (256^2 cloth over the level-5 icosphere, 2^20 buckets): the CCD
  pass at the start of the first timed substep (after the 5 warm-up
  substeps of the driver's run) equals the oracle's pair test exactly
  (contact ids, time of impact, barycentric weights, normals); the whole
  substep (advect, 15 sweeps with CCD at 0/10/14 and the response,
  integrate) is within 1e-5 m of the oracle's with the same number of
  contacts in its last pass; the same again at the end of a 20-substep
  timed window;
* fold1024 (1024^2 self-colliding fold on the ground, 2^24 buckets, after
  its 120-substep pre-roll and 5 warm-up substeps): one CCD pass exactly
  equal to the oracle's, and the whole substep within 1e-5 m;
* batch512: 8 of its 512 instances (those whose spheres are closest below
  them, so they drape and fold within the pre-roll), built as in the batch
  (per-instance hash cells and spheres, 2^24 buckets), after the 120-substep
  pre-roll and 5 warm-up substeps: one substep of the batch against the
  oracle run on each instance alone with its own cell and sphere, within
  1e-5 m, contact counts equal.

Every benchmark object's coloring is also validated: no two constraints of
one color share a point (test_bench_colorings_are_valid).

The oracle runs its independent loops on every host core (the results do
not depend on the thread count).
"""
import numpy as np
import pytest

import bench
from positionbaseddynamicsold_gb300 import scenes

pytestmark = pytest.mark.gpu

G = bench.G
DT = bench.DT


@pytest.fixture(scope="module")
def orc_mt():
    from oracle.oracle import Oracle
    o = Oracle()
    o.set_threads()
    yield o
    o.set_threads(1)


def colli_of(sc, cell, **kw):
    d = {"center": (0.0, 0.0, 0.0), "cell": cell, "bounded": False,
         "thickness": sc["colli"]["thickness"], "tri_idx": sc["tri_idx"], "mass_weighted": 1,
         "resolve_passes": 1, "contact_cap": 1 << 21}
    d.update(kw)
    return d


def assert_contacts_equal(got, want):
    assert len(got["ids"]) == len(want["ids"])
    np.testing.assert_array_equal(got["ids"], want["ids"])
    np.testing.assert_array_equal(got["face"], want["face"])
    np.testing.assert_array_equal(got["t"], want["t"])
    np.testing.assert_array_equal(got["w"], want["w"])
    np.testing.assert_array_equal(got["n"], want["n"])


def ccd_pass_and_substep(orc, sc, obj, solver, cs, iters, ground=None):
    """from the object's current state: one CCD pass after advection (GPU
    vs oracle, exact), then the whole substep (GPU eager vs oracle)"""
    pos, vel = obj.get_state()
    solver.advect(DT)
    cs.ccd_sh_extended()
    got = cs.contacts()
    grid = orc.grid((0.0, 0.0, 0.0), None, sc["colli"]["cell"], False)
    want, h = orc.ccd(grid, sc["tri_idx"], pos, obj.predicted(), sc["colli"]["thickness"],
                      cap=1 << 21)
    assert h == len(want["ids"])
    assert_contacts_equal(got, want)
    solver.project_constraint_with_colli(iters, cs)
    solver.integration(DT)
    _, sid, ws = orc.sort_worksets(obj.colors())
    st = {"pos": pos.copy(), "vel": vel.copy()}
    nct = orc.substep_gpu(sc, st, sid, ws, iters, DT, 1.0, G,
                          colli=colli_of(sc, sc["colli"]["cell"]), ground=ground)
    err = float(np.abs(obj.positions() - st["pos"]).max())
    assert err <= 1e-5, err
    assert cs.stats()["contacts"] == nct
    return len(got["ids"]), nct


def test_drape256_substeps_match_oracle(orc_mt):
    sc, cfg, colli_on, tl, preroll = bench.make_workload("drape256")
    assert preroll == 0 and tl == 20 and cfg["gs_iterations"] == 15
    obj, solver, shs, cs = bench.setup(sc, colli_on, tl)
    solver.step(DT, 5, 15, cs, True)            # the driver run's warm-up substeps
    first, last = ccd_pass_and_substep(orc_mt, sc, obj, solver, cs, 15)
    assert first > 0 and last > 0
    solver.step(DT, 18, 15, cs, True)           # to the end of a 20-substep timed window
    first, last = ccd_pass_and_substep(orc_mt, sc, obj, solver, cs, 15)
    assert first > 100 and last > 100


def test_fold1024_ccd_pass_and_substep_match_oracle(orc_mt):
    sc, cfg, colli_on, tl, preroll = bench.make_workload("fold1024")
    assert tl == 24 and preroll == 120
    obj, solver, shs, cs = bench.setup(sc, colli_on, tl)
    solver.step(DT, preroll + 5, 15, cs, True)
    first, last = ccd_pass_and_substep(orc_mt, sc, obj, solver, cs, 15,
                                       ground=sc["colli"]["ground"])
    assert first > 1000 and last > 1000


def test_batch512_instances_match_oracle(orc_mt):
    ids = [21, 124, 159, 191, 217, 326, 489, 493]
    sc = scenes.batched_cloths(512, seed=0, subset=ids)
    cells = scenes.instance_cells(sc)
    sc["colli"] = {"cell": 2.0 * scenes.mean_rest_edge(sc), "thickness": 1e-3,
                   "spheres": sc["spheres"], "instance_cells": cells}
    obj, solver, shs, cs = bench.setup(sc, True, 24)
    solver.step(DT, 125, 15, cs, True)
    pos, vel = obj.get_state()
    solver.step(DT, 1, 15, cs, False)
    got = obj.positions()
    colors = obj.colors()
    p0 = q0 = 0
    total = 0
    for k, i in enumerate(ids):
        one = scenes.batched_cloths(512, seed=0, subset=[i])
        n, m = len(one["pos"]), len(one["ctype"])
        np.testing.assert_array_equal(one["pos"][:, [0, 2]], sc["pos"][p0:p0 + n][:, [0, 2]])
        _, sid, ws = orc_mt.sort_worksets(colors[q0:q0 + m])
        st = {"pos": pos[p0:p0 + n].copy(), "vel": vel[p0:p0 + n].copy()}
        one["colli"] = {"thickness": 1e-3}
        nct = orc_mt.substep_gpu(one, st, sid, ws, 15, DT, 1.0, G,
                                 colli=colli_of(one, float(cells[k])), sphere=sc["spheres"][k])
        err = float(np.abs(got[p0:p0 + n] - st["pos"]).max())
        assert err <= 1e-5, (i, err)
        total += nct
        p0 += n
        q0 += m
    assert p0 == len(got)
    assert cs.stats()["contacts"] == total
    assert total > 0


@pytest.mark.parametrize("name", ["drape256", "fold1024", "batch512"])
def test_bench_colorings_are_valid(name):
    """the device coloring of each benchmark object: every constraint has a
    color, and no two constraints of one color share a point"""
    sc, cfg, colli_on, tl, preroll = bench.make_workload(name)
    obj, solver, shs, cs = bench.setup(sc, colli_on, tl)
    colors = obj.colors().astype(np.int64)
    assert colors.min() >= 0
    pl = sc["prim_list"].astype(np.int64)
    cnt = pl[:, 1]
    owner = np.repeat(np.arange(len(pl)), cnt)
    pos = np.repeat(pl[:, 0], cnt) + (np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt))
    pts = sc["indices"].astype(np.int64)[pos]
    keys = colors[owner] * (int(pts.max()) + 1) + pts
    assert len(np.unique(keys)) == len(keys)
