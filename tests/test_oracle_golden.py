"""Pin the oracle (oracle/pbd_oracle.c) to the reference's own outputs.

The fixtures in tests/golden/ were produced by the reference's code compiled
from its sources (tests/golden/make_golden.py).  Integer and index results
must match exactly; float results of identical arithmetic must match
bit-for-bit where the restatement performs the same operations, otherwise
within the stated tolerance.
"""
import ctypes as C

import numpy as np
import pytest

from oracle.oracle import _ptr


@pytest.mark.parametrize("name", ["grid", "dgrid", "refgrid"])
def test_prim2prims_and_coloring(orc_pow, golden, name):
    g = golden("coloring")
    pl, ix = g[name + "_prim_list"], g[name + "_indices"]
    n_points = int(ix.max()) + 1
    sn, adj = orc_pow.prim2prims(pl, ix, n_points)
    np.testing.assert_array_equal(sn, g[name + "_adj_sn"])
    np.testing.assert_array_equal(adj, g[name + "_adj"])
    # CPU schedule (EdgeColoringCPU), 2000 sweeps as in the fixture
    color, _ = orc_pow.edge_coloring(pl, ix, n_points, "cpu", max_iters=2000)
    np.testing.assert_array_equal(color, g[name + "_color_cpu"])
    # one speculative assignment sweep from a partial coloring
    n = len(pl)
    partial = np.ascontiguousarray(g[name + "_partial"])
    prd = np.full(n, -1, np.int32)
    orc_pow.lib.orc_assign_colors(n, _ptr(sn), _ptr(adj), _ptr(partial), _ptr(prd))
    np.testing.assert_array_equal(prd, g[name + "_prd"])


@pytest.mark.parametrize("name", ["grid", "dgrid", "refgrid"])
def test_sort_worksets(orc_pow, golden, name):
    g = golden("coloring")
    c, sid, ws = orc_pow.sort_worksets(g[name + "_gcolor"])
    np.testing.assert_array_equal(c, g[name + "_sorted_color"])
    np.testing.assert_array_equal(sid, g[name + "_sorted_id"])
    np.testing.assert_array_equal(ws, g[name + "_worksets"])


def test_gpu_schedule_coloring_is_valid(orc_pow, golden):
    g = golden("coloring")
    for name in ("grid", "dgrid", "refgrid"):
        pl, ix, col = g[name + "_prim_list"], g[name + "_indices"], g[name + "_gcolor"]
        assert (col >= 0).all()
        for c in np.unique(col):
            pts = np.concatenate([ix[pl[p, 0]:pl[p, 0] + pl[p, 1]] for p in np.nonzero(col == c)[0]])
            assert len(np.unique(pts)) == len(pts), "two constraints of one color share a point"


def test_substep_cpu_reference_path(orc_pow, golden):
    """advectCPU + projectConstraintCPU (incl. the unit-sphere push) +
    integrationCPU, 3 substeps of 5 iterations: bit-exact."""
    g = golden("substep_cpu")
    scene = {k: g[k] for k in ("mass", "prim_list", "indices", "ctype", "rest_length", "stiffness")}
    st = {"pos": g["pos0"].copy(), "vel": np.zeros_like(g["pos0"])}
    grav = np.array([0, -9.8, 0], np.float32)
    for _ in range(3):
        orc_pow.substep_cpu_ref(scene, st, 5, 1.0 / 60, grav, sphere=((0, 0, 0), 1.0))
    np.testing.assert_array_equal(st["pos"], g["pos"])
    np.testing.assert_array_equal(st["vel"], g["vel"])


def test_colored_gs_pinned_by_reference(orc_pow, golden):
    """Colored GS (the GPU kernel's semantics) equals the reference's
    sequential GS run over the constraints in color-sorted order when every
    stiffness is 1; the two differ only in how the direction is normalised
    (v/d versus v*rsqrt), so the bound is a few float ulps."""
    g = golden("substep_gpu_pin")
    scene = {k: g[k] for k in ("mass", "prim_list", "indices", "ctype", "rest_length", "stiffness")}
    _, sid, ws = orc_pow.sort_worksets(g["color"])
    st = {"pos": g["pos0"].copy(), "vel": np.zeros_like(g["pos0"])}
    orc_pow.substep_gpu(scene, st, sid, ws, 10, 1.0 / 600, 1.0, np.array([0, -9.8, 0], np.float32))
    assert np.abs(st["pos"] - g["pos"]).max() <= 2e-6


def test_find_neighbors(orc_pow, golden):
    g = golden("neighbors")
    grid = orc_pow.grid(g["center"], g["size"], g["cell"], True)
    sn, nb = orc_pow.find_neighbors_all(grid, g["tri_idx"], g["pos"])
    np.testing.assert_array_equal(sn, g["start_num"])
    np.testing.assert_array_equal(nb, g["nbrs"])


def test_ccd_sh_extended_reference_order(orc_pow, golden):
    g = golden("ccd")
    grid = orc_pow.grid(g["center"], g["size"], g["cell"], True)
    ct, h = orc_pow.ccd(grid, g["tri_idx"], g["pos"], g["prdp"], float(g["thickness"]), mode="ref")
    assert h == len(g["ids"]) and h > 50
    np.testing.assert_array_equal(ct["ids"], g["ids"])
    np.testing.assert_array_equal(ct["t"], g["t"])
    np.testing.assert_array_equal(ct["w"], g["w"])
    np.testing.assert_array_equal(ct["n"], g["n"])


def test_ccd_distinct_pairs_same_set(orc_pow, golden):
    """Evaluating each distinct (point, triangle) pair once gives the
    reference's contact set (order aside)."""
    g = golden("ccd")
    grid = orc_pow.grid(g["center"], g["size"], g["cell"], True)
    ct, h = orc_pow.ccd(grid, g["tri_idx"], g["pos"], g["prdp"], float(g["thickness"]), mode="pairs")
    a = sorted(map(tuple, ct["ids"].tolist()))
    b = sorted(map(tuple, g["ids"].tolist()))
    assert a == b
    # per contact the stored (t, w, n) are identical too
    ref_map = {tuple(k): (t, tuple(w), tuple(n)) for k, t, w, n in
               zip(g["ids"].tolist(), g["t"].tolist(), g["w"].tolist(), g["n"].tolist())}
    for k, t, w, n in zip(ct["ids"].tolist(), ct["t"].tolist(), ct["w"].tolist(), ct["n"].tolist()):
        assert ref_map[tuple(k)] == (t, tuple(w), tuple(n))


def test_collision_resolve_new(orc_pow, golden):
    g = golden("ccd")
    p = orc_pow.resolve_ref(g["ids"], g["pos"], g["prdp"], 2, float(g["thickness"]))
    np.testing.assert_array_equal(p, g["resolved"])


def test_vf_cases(orc_pow, golden):
    g = golden("vf_cases")
    n = len(g["hit"])
    for k in range(n):
        hit, t, w, nv = orc_pow.extended_vf_test(g["X"][k], g["P"][k], float(g["thickness"][k]))
        assert hit == g["hit"][k], k
        assert np.float32(t) == g["t"][k], k
        np.testing.assert_array_equal(w, g["w"][k])
        np.testing.assert_array_equal(nv, g["n"][k])
        nh, nt, _, _ = orc_pow.extended_vf_test(g["X"][k], g["P"][k], float(g["thickness"][k]), narrow=True)
        assert nh == g["narrow_hit"][k], k
        assert np.float32(nt) == g["narrow_t"][k], k
        assert orc_pow.vf_resolve_test(g["X"][k], g["P"][k], float(g["thickness"][k])) == g["resolve_test"][k]
        np.testing.assert_array_equal(orc_pow.vf_resolve_new(g["X"][k], g["P"][k], float(g["thickness"][k])),
                                      g["resolve_new"][k])


@pytest.mark.parametrize("kind", ["vfccd", "vfdcd", "vf"])
def test_vf_variants_match_reference(orc_pow, golden, kind):
    """VFCCDTest (type VF), VFDCDTest and VFTest (P/CCD.cpp:2229-2421) on the
    1,500 near-contact cases: hit, time, weights and normal equal the
    reference's own outputs (a miss leaves what the last evaluated time
    wrote, compared too)"""
    g = golden("vf_cases")
    for k in range(len(g["hit"])):
        hit, t, w, nv = orc_pow.vf_variant(kind, g["X"][k], g["P"][k], float(g["thickness"][k]))
        assert hit == g[kind + "_hit"][k], k
        assert np.float32(t) == g[kind + "_t"][k], k
        np.testing.assert_array_equal(w, g[kind + "_w"][k])
        np.testing.assert_array_equal(nv, g[kind + "_n"][k])


def test_solve_cubic(orc_pow, golden):
    g = golden("vf_cases")
    for k, (a, b, c, d) in enumerate(g["coef"]):
        x = orc_pow.solve_cubic(a, b, c, d)
        assert len(x) == g["nroot"][k]
        np.testing.assert_array_equal(x, g["roots"][k, :len(x)])
    x = orc_pow.solve_cubic(1.0, -6.0, 11.0, -6.0)
    assert np.allclose(x, [1, 2, 3], atol=1e-7)


def test_old_response_matches_reference(orc_pow, golden):
    """CollisionResolve + VFResolve (P/CCD.cpp:2423-2650), the older
    response: three calls in a row with the positions and per-point resolve
    counters carried over (the counters gate the crossing case from the
    second call on), on two contact sets; positions and counters equal the
    reference's own outputs."""
    g = golden("ccd")
    r = golden("resolve_old")
    for case in "ab":
        prd = r[case + "_prdp0"]
        rt = np.zeros(len(g["pos"]), np.int32)
        for k in range(1, 4):
            prd = orc_pow.resolve_old(r[case + "_ids"], g["pos"], prd, rt, float(g["thickness"]))
            np.testing.assert_array_equal(prd, r["%s_prdp%d" % (case, k)])
            np.testing.assert_array_equal(rt, r["%s_rt%d" % (case, k)])


def test_stiffness_schedule_pinned_to_reference_gpu_kernel(orc_pow, golden):
    """The colored projection with stiffness below 1 against the reference's
    ProjectContraintsGPUKernel itself (P/PBD_cuda.cu:1240-1306, its code
    compiled for the host by oracle/build_oracle.py and launched colour by
    colour): 8 iterations, k = 1 - (1 - s)^(1/(iter+1)), bit for bit."""
    g = golden("gpu_kernel_schedule")
    sc = {k: g[k] for k in ("prim_list", "indices", "ctype", "rest_length", "stiffness")}
    got = orc_pow.project_colored(sc, g["prdp"], g["mass"], g["sorted_prim_id"], g["worksets"],
                                  0, 8)
    np.testing.assert_array_equal(got, g["out"])
    assert np.abs(g["out"] - g["prdp"]).max() > 1e-3
