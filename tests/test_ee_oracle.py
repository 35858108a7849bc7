"""Known answers for the oracle's edge-edge CCD (the reference declares the
contact kind only, Contact::EE in P/CCD_Basic.h:14, so these hand-computed
cases pin the restatement): crossing edges hit at the coplanarity time with
the lines' closest-point parameters, parallel or separated edges and
endpoint-only contacts give no hit, the response separates a crossed pair
to 2 * thickness on its starting side, and brute-force detection reports
each pair once."""
import numpy as np
import pytest

from oracle.oracle import Oracle

H = 1e-3


@pytest.fixture(scope="module")
def orc():
    return Oracle()


def crossing(y0=0.01, y1=-0.01, s=0.5, u=0.5):
    # edge A along x at height y, moving y0 -> y1; edge B along z at y = 0,
    # placed so that the lines meet at parameter s on A and u on B
    a0, a1 = np.array([0.0, 0, 0]), np.array([1.0, 0, 0])
    b0 = np.array([s, 0.0, -u])
    b1 = np.array([s, 0.0, 1.0 - u])
    x = np.array([a0 + [0, y0, 0], a1 + [0, y0, 0], b0, b1], np.float32)
    p = np.array([a0 + [0, y1, 0], a1 + [0, y1, 0], b0, b1], np.float32)
    return x, p


def test_crossing_edges_hit_at_the_coplanar_time(orc):
    x, p = crossing()
    hit, t, s, u, m0 = orc.ee_test(x, p, H)
    assert hit
    assert t == pytest.approx(0.5, abs=1e-6)
    assert s == pytest.approx(0.5, abs=1e-6) and u == pytest.approx(0.5, abs=1e-6)
    # common normal along y, edge A starts above B
    assert abs(abs(m0[1]) - 1.0) < 1e-6 and m0[3] * m0[1] > 0


def test_asymmetric_crossing_parameters(orc):
    x, p = crossing(0.02, -0.02, s=0.25, u=0.75)
    hit, t, s, u, _ = orc.ee_test(x, p, H)
    assert hit and t == pytest.approx(0.5, abs=1e-6)
    assert s == pytest.approx(0.25, abs=1e-6) and u == pytest.approx(0.75, abs=1e-6)


def test_misses(orc):
    # passes beside B: the lines meet outside edge B
    x, p = crossing(0.01, -0.01, s=1.5, u=0.5)
    assert not orc.ee_test(x, p, H)[0]
    # stays 5 h above: never within 2 h
    x, p = crossing(0.005, 0.005)
    assert not orc.ee_test(x, p, H)[0]
    # parallel edges are left to the vertex-face tests
    x = np.array([[0, 0.01, 0], [1, 0.01, 0], [0, 0, 0.2], [1, 0, 0.2]], np.float32)
    p = x - np.array([0, 0.02, 0], np.float32) * [[1], [1], [0], [0]]
    assert not orc.ee_test(x, p, H)[0]


def test_close_start_is_a_hit_at_t0(orc):
    x, p = crossing(0.0015, 0.0015)   # 1.5 h apart the whole step
    hit, t, _, _, _ = orc.ee_test(x, p, H)
    assert hit and t == 0.0


def test_response_separates_to_two_h_on_the_start_side(orc):
    x, p = crossing()
    hit, t, s, u, m0 = orc.ee_test(x, p, H)
    ids = np.array([[0, 1, 2, 3]])
    mass = np.ones(4, np.float32)
    out = orc.resolve_jacobi_ee(np.zeros((0, 4), np.int32), ids, m0[None], x, p, mass, 1, H,
                                True)
    # A's closest point now 2 h above B's along +y (A started above)
    a_mid = 0.5 * (out[0] + out[1])
    b_mid = 0.5 * (out[2] + out[3])
    assert a_mid[1] - b_mid[1] == pytest.approx(2 * H, rel=1e-4)
    # equal masses: both edges moved by half the depth each
    assert out[0][1] == pytest.approx(-0.01 + (0.01 + 2 * H) / 2, rel=1e-3)
    # a pinned edge B (inverse mass 0) stays put; A takes all of it
    mass = np.array([1, 1, 0, 0], np.float32)
    out = orc.resolve_jacobi_ee(np.zeros((0, 4), np.int32), ids, m0[None], x, p, mass, 1, H,
                                True)
    np.testing.assert_array_equal(out[2:], p[2:])
    assert out[0][1] == pytest.approx(2 * H, rel=1e-4)


def test_brute_force_reports_each_pair_once(orc):
    x, p = crossing()
    # the two edges plus a far-away third one and one sharing a point with A
    pts_x = np.concatenate([x, [[5, 0, 0], [6, 0, 0]]]).astype(np.float32)
    pts_p = np.concatenate([p, [[5, 0, 0], [6, 0, 0]]]).astype(np.float32)
    edges = np.array([[0, 1], [2, 3], [4, 5], [1, 4]], np.int32)
    pairs, tsu, m0 = orc.ccd_ee_brute(edges, None, pts_x, pts_p, H)
    np.testing.assert_array_equal(pairs, [[0, 1]])
    # instances: B in another instance -> no pair
    inst = np.array([0, 0, 1, 1, 0, 0], np.int32)
    pairs, _, _ = orc.ccd_ee_brute(edges, inst, pts_x, pts_p, H)
    assert len(pairs) == 0
