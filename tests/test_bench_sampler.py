"""The bench's timing of the reference CPU path (bench.RefSampler,
bench.BatchRefSampler) on the CPU:

* the prim-range projection, run chunk after chunk, is the sequential
  projectConstraintCPU loop bit for bit;
* detection in triangle ranges against one UpdateSH table finds the
  contacts of the single pass (the union of the ranges, duplicates across
  ranges removed);
* one substep's worth of sampler steps covers 15 iterations of every prim
  and 3 detection passes over every triangle;
* the batch sampler scales the sampled instances' substep times by points.
"""
import ctypes as C

import numpy as np
import pytest

import bench
from oracle.oracle import Oracle, OrcContact, _ptr
from positionbaseddynamicsold_gb300 import scenes


@pytest.fixture(scope="module")
def orc():
    return Oracle()


def folded_cloth(res=32, seed=3):
    """a cloth folded over itself 2 mm apart, the upper half moving down
    through the lower one during the step"""
    rng = np.random.default_rng(seed)
    sc = scenes.grid_cloth(res, res, 0.1, 0.1, origin=(-0.05, 0.0, -0.05), jitter=1e-4,
                           seed=seed)
    pos = sc["pos"].astype(np.float64)
    far = pos[:, 2] > 0.0
    pos[far, 2] = -pos[far, 2]
    pos[far, 1] += 0.002
    pos = pos.astype(np.float32)
    prd = pos.copy()
    prd[far, 1] -= np.float32(0.004)
    prd += rng.normal(0, 3e-4, prd.shape).astype(np.float32)
    sc["pos"] = pos
    sc["colli"] = {"cell": 2.0 * scenes.mean_rest_edge(sc), "thickness": 1e-3}
    return sc, pos, prd


def test_projection_chunks_equal_the_sequential_loop(orc):
    sc, pos, prd = folded_cloth()
    c = orc.constraints(sc)
    mass = np.ascontiguousarray(sc["mass"])
    whole = prd.copy()
    orc.lib.orc_project_cpu(C.byref(c), 1, _ptr(mass), _ptr(whole), len(whole), None,
                            C.c_float(0.0))
    chunks = prd.copy()
    cuts = [0, 1, 517, 2048, c.n_prims - 3, c.n_prims]
    for a, b in zip(cuts[:-1], cuts[1:]):
        orc.lib.orc_project_cpu_range(C.byref(c), _ptr(mass), _ptr(chunks), a, b)
    np.testing.assert_array_equal(chunks, whole)


def test_ranges_against_one_table_find_the_pass_contacts(orc):
    sc, pos, prd = folded_cloth()
    L = orc.lib
    L.orc_sh_build.restype = C.c_void_p
    L.orc_sh_build.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    L.orc_sh_free.argtypes = [C.c_void_p]
    L.orc_ccd_sh_extended_ref_range_tab.restype = C.c_int64
    colli = orc._colli(bench.cpu_colli(sc))
    tri = np.ascontiguousarray(sc["tri_idx"], np.int32)
    nt, cap = len(tri), 1 << 18
    arr = (OrcContact * cap)()
    h = L.orc_ccd_sh_extended_ref(C.byref(colli.grid), nt, _ptr(tri), _ptr(pos), _ptr(prd),
                                  C.c_float(colli.thickness), arr, C.c_int64(cap))
    assert 0 < h < cap
    want = {(arr[i].v, arr[i].f0, arr[i].f1, arr[i].f2) for i in range(h)}
    table = L.orc_sh_build(C.byref(colli.grid), nt, _ptr(tri), _ptr(prd))
    got = set()
    for a in range(0, nt, 97):
        b = min(nt, a + 97)
        k = L.orc_ccd_sh_extended_ref_range_tab(C.byref(colli.grid), C.c_void_p(table), nt,
                                                _ptr(tri), _ptr(pos), _ptr(prd),
                                                C.c_float(colli.thickness), a, b, arr,
                                                C.c_int64(cap))
        got |= {(arr[i].v, arr[i].f0, arr[i].f1, arr[i].f2) for i in range(k)}
    L.orc_sh_free(table)
    assert got == want and len(want) > 50


@pytest.mark.parametrize("workload", ["drape256", "fold1024"])
def test_one_substep_of_steps_covers_one_substep_of_work(workload):
    sc, cfg, colli_on, _, _ = bench.make_workload(workload)
    rs = bench.RefSampler(sc, cfg, colli_on, sc["pos"], sc["vel"])
    per = rs.iters * rs.m
    assert rs.phi == pytest.approx(1.0 / per)
    # chunk sizes times steps: iterations x prims and 3 passes x triangles,
    # within one chunk of rounding
    assert abs(rs.gs_chunk * per - rs.iters * rs.n_prims) <= per
    assert abs(rs.ccd_chunk * per - 3 * rs.nt) <= per
    assert rs.ccd_chunk <= 2100
    # a pass visits every slice once, consecutive steps far apart
    assert sorted(rs.slice_order) == list(range(rs.n_slices))
    assert rs.n_slices * rs.ccd_chunk >= rs.nt > (rs.n_slices - 1) * rs.ccd_chunk
    if rs.n_slices > 10:
        assert abs(rs.slice_order[1] - rs.slice_order[0]) > rs.n_slices // 4


def test_batch_scaling_by_points():
    class Fake:
        def __init__(self, phi):
            self.phi = phi

    b = bench.BatchRefSampler.__new__(bench.BatchRefSampler)
    b.samplers = [Fake(1 / 15), Fake(1 / 30), Fake(1 / 45)]
    b.points = [256, 1024, 4096]
    b.total_points = 100000
    b.t = [0.3, 0.6, 0.0]
    b.n = [3, 6, 0]                       # the third was not stepped
    # substep times 1.5 s and 3.0 s for 1,280 points; 100,000 points in all
    want = 1280 / ((0.3 / (3 / 15) + 0.6 / (6 / 30)) * 100000)
    assert b.value() == pytest.approx(want)


def test_threaded_reference_substeps_equal_one_thread():
    """RefSubsteps with the CCD detection spread over host threads gives the
    one-thread result exactly: contact lists (stored in loop order with the
    duplicate scan) and positions, with either response; and the threaded
    contact list equals the sequential CCD_SH_Extended's."""
    from oracle.oracle import Oracle
    from positionbaseddynamicsold_gb300 import scenes
    sc = scenes.drape_over_sphere(res=40, seed=3, sphere_level=2, start="contact")
    cfg = {"gs_iterations": 15}
    for mw in (1, 0):
        out = []
        for th in (1, 4):
            rs = bench.RefSubsteps(sc, cfg, sc["pos"], sc["vel"], th, mass_weighted=mw)
            nc = []
            for _ in range(4):
                rs.step()
                nc.append(int(rs.contacts))
            out.append((rs.state["pos"].copy(), nc))
        np.testing.assert_array_equal(out[0][0], out[1][0])
        assert out[0][1] == out[1][1] and max(out[0][1]) > 0
    orc = Oracle()
    n = sc["n_cloth_points"]
    pos = sc["pos"].copy()
    prd = pos.copy()
    prd[:n, 1] -= np.float32(0.03)
    grid = orc.grid((0.0, 0.0, 0.0), None, sc["colli"]["cell"], False)
    res = []
    for th in (1, 4):
        orc.set_threads(th)
        res.append(orc.ccd(grid, sc["tri_idx"], pos, prd, 1e-3, mode="ref"))
    orc.set_threads(1)
    assert res[0][1] == res[1][1] > 20
    for k in res[0][0]:
        np.testing.assert_array_equal(res[0][0][k], res[1][0][k])


def test_reference_arm_and_gpu_arm_share_the_workload_config():
    """Both arms take the workload's config from make_workload; it holds
    only what describes the workload (no GPU-derived plan)."""
    for w in ("drape256", "hanging32"):
        sc, cfg, colli_on, tl, preroll = bench.make_workload(w)
        for k in ("colors", "autotune", "points", "parallelism"):
            assert k not in cfg
        assert cfg["preroll_substeps"] == preroll
    sc, cfg, _, _, preroll = bench.make_workload("drape256")
    assert preroll == 0 and "start" in cfg and "response" in cfg
