"""The arithmetic behind the narrowphase's exact shortcuts, restated in numpy
float32 (no fused multiply-add, IEEE division and square root, as the
kernels compile) and checked against float64 on the CPU.  The kernels
themselves are checked on the GPU against the reference's compiled
ExtendedVFTest (test_gpu_collision.py) and at the benchmark's states
(test_gpu_bench_configs.py); these tests state why the shortcuts cannot
change a decision:

* the plane test |d| - 2h < -1e-6, taken in double by the reference, is
  decided in float only when the float difference is clear of the bound,
  and every such decision equals the double one, also for d drawn right at
  the bound;
* the no-root test's Bernstein coefficients in float: "no root" (all four
  clear of 1e-5 sum |a| with one sign) and "both signs" (one clear above,
  one below) agree with the double test on every random cubic, including
  cubics with roots placed at the interval's ends;
* the outside-over-the-step bound (vf_outside_all_step): on random point /
  triangle steps (coplanar neighbours, layers a thickness apart, fast and
  slow motion, near-slivers), whenever it reports the point outside, the
  barycentric weights of the point's projection, sampled densely over the
  step in float64, keep one weight below -eps(t) at every sample.
"""
import numpy as np

f32 = np.float32


def plane_close_float(d, th2):
    """(decided, value) of the kernels' plane_close before its double branch"""
    fd = np.abs(d.astype(f32)) - th2.astype(f32)
    yes = fd < f32(-1.000001e-6)
    no = fd > f32(-0.999999e-6)
    return yes | no, yes


def test_plane_test_float_decisions_equal_double():
    rng = np.random.default_rng(0)
    n = 400_000
    th2 = (2.0 * rng.uniform(1e-4, 1e-2, n)).astype(f32)
    # distances spread widely, and drawn right at the bound |d| = 2h - 1e-6
    d = np.concatenate([rng.normal(0, 1e-2, n // 2),
                        (th2[n // 2:].astype(np.float64) - 1e-6) *
                        (1 + rng.normal(0, 1e-6, n - n // 2)) * rng.choice([-1, 1], n - n // 2)])
    d = d.astype(f32)
    want = np.abs(d.astype(np.float64)) - th2.astype(np.float64) < -1e-6
    decided, val = plane_close_float(d, th2)
    assert decided.mean() > 0.9
    np.testing.assert_array_equal(val[decided], want[decided])


def bernstein_f32(a0, a1, a2, a3):
    u, L = f32(-1e-3), f32(1.002)
    c0 = ((a3 * u + a2) * u + a1) * u + a0
    c1 = L * ((f32(3) * a3 * u + f32(2) * a2) * u + a1)
    c2 = L * L * (f32(3) * a3 * u + a2)
    c3 = L * L * L * a3
    third = f32(1) / f32(3)
    b = np.stack([c0, c0 + c1 * third, c0 + f32(2) * c1 * third + c2 * third,
                  c0 + c1 + c2 + c3], 1)
    tol = f32(1e-5) * (np.abs(a0) + np.abs(a1) + np.abs(a2) + np.abs(a3))
    return b, tol


def bernstein_f64(a0, a1, a2, a3):
    a0, a1, a2, a3 = (np.asarray(v, np.float64) for v in (a0, a1, a2, a3))
    u, L = -1e-3, 1.002
    c0 = ((a3 * u + a2) * u + a1) * u + a0
    c1 = L * ((3.0 * a3 * u + 2.0 * a2) * u + a1)
    c2 = L * L * (3.0 * a3 * u + a2)
    c3 = L * L * L * a3
    third = 1.0 / 3.0
    b = np.stack([c0, c0 + c1 * third, c0 + 2.0 * c1 * third + c2 * third, c0 + c1 + c2 + c3], 1)
    tol = 1e-9 * (np.abs(a0) + np.abs(a1) + np.abs(a2) + np.abs(a3))
    return (b > tol[:, None]).all(1) | (b < -tol[:, None]).all(1)


def test_no_root_float_decisions_equal_double():
    rng = np.random.default_rng(1)
    n = 300_000
    scale = 10.0 ** rng.uniform(-12, -3, (n, 1))
    a = (rng.normal(0, 1, (n, 4)) * scale)
    # a third with a root placed near 0, 1 or inside: a0 from a3, a2, a1
    k = n // 3
    r = rng.choice([-1e-3, 0.0, 0.5, 1.0, 1.001], k) + rng.normal(0, 1e-7, k)
    a[:k, 0] = -(a[:k, 1] * r + a[:k, 2] * r ** 2 + a[:k, 3] * r ** 3)
    a = a.astype(f32)
    a0, a1, a2, a3 = a[:, 0], a[:, 1], a[:, 2], a[:, 3]
    b, tol = bernstein_f32(a0, a1, a2, a3)
    ok = (tol > 0) & np.isfinite(tol)
    no_root = ok & ((b > tol[:, None]).all(1) | (b < -tol[:, None]).all(1))
    both = ok & ~no_root & (b > tol[:, None]).any(1) & (b < -tol[:, None]).any(1)
    want = bernstein_f64(a0, a1, a2, a3)
    assert no_root.sum() > 1000 and both.sum() > 1000
    assert want[no_root].all()
    assert not want[both].any()


# ---- vf_outside_all_step --------------------------------------------------
def dot(a, b):
    return (a * b).sum(-1)


def bern_cross(a0, a1, b0, b1):
    return [np.cross(a0, b0), (np.cross(a0, b1) + np.cross(a1, b0)) * f32(0.5),
            np.cross(a1, b1)]


def bern_dot(u, v):
    return [dot(u[0], v[0]), f32(0.5) * (dot(u[0], v[1]) + dot(u[1], v[0])),
            (dot(u[0], v[2]) + f32(4) * dot(u[1], v[1]) + dot(u[2], v[0])) * f32(1.0 / 6.0),
            f32(0.5) * (dot(u[1], v[2]) + dot(u[2], v[1])), dot(u[2], v[2])]


def seg_origin_dist(a, b):
    d = b - a
    dd = dot(d, d)
    with np.errstate(invalid="ignore", divide="ignore"):
        t = np.where(dd > 0, np.clip(-dot(a, d) / dd, f32(0), f32(1)), f32(0)).astype(f32)
    q = a + d * t[:, None]
    return np.sqrt(dot(q, q))


def outside_all_step(X, P, th):
    """numpy float32 restatement of vf_outside_all_step; X, P: (4, n, 3)"""
    a0, a1 = X[2] - X[1], P[2] - P[1]
    b0, b1 = X[3] - X[1], P[3] - P[1]
    c0, c1 = X[3] - X[2], P[3] - P[2]
    es = seg_origin_dist(a0, a1) + seg_origin_dist(b0, b1) + seg_origin_dist(c0, c1)
    big = np.maximum(np.abs(X).max((0, 2)), np.abs(P).max((0, 2)))
    ok = (es > 0) & (big <= f32(1000) * (es / f32(3)))
    n = bern_cross(a0, a1, b0, b1)
    D = bern_dot(n, n)
    ok &= (D[0] >= f32(1e-4) * (dot(a0, a0) * dot(b0, b0))) & \
          (D[4] >= f32(1e-4) * (dot(a1, a1) * dot(b1, b1)))
    dmin = f32(0.25) * np.minimum(D[0], D[4])
    ok &= (D[1] >= dmin) & (D[2] >= dmin) & (D[3] >= dmin)
    with np.errstate(divide="ignore", invalid="ignore"):
        e = f32(3) * f32(th) / es * f32(1.0001) + f32(0.01)
    nmag = sum(np.sqrt(dot(v, v)) for v in n)
    r0 = [X[k] - X[0] for k in (1, 2, 3)]
    r1 = [P[k] - P[0] for k in (1, 2, 3)]
    out = np.zeros(len(es), bool)
    for i in range(3):
        j, k = (i + 1) % 3, (i + 2) % 3
        m = bern_cross(r0[j], r1[j], r0[k], r1[k])
        C = bern_dot(m, n)
        tol = f32(1e-4) * (sum(np.sqrt(dot(v, v)) for v in m) * nmag + e * nmag * nmag)
        out |= np.all(np.stack([C[q] + e * D[q] < -tol for q in range(5)]), 0)
    return out & ok


def fails_inside_everywhere(X, P, th, ts):
    """float64: at every t of ts, some barycentric weight of the point's
    projection lies below -eps(t), eps = th / (mean edge length at t)"""
    X = X.astype(np.float64)
    P = P.astype(np.float64)
    fail = np.ones(X.shape[1], bool)
    for t in ts:
        c = X + t * (P - X)
        nrm = np.cross(c[2] - c[1], c[3] - c[1])
        D = dot(nrm, nrm)
        r = [c[k] - c[0] for k in (1, 2, 3)]
        w = np.stack([dot(np.cross(r[(i + 1) % 3], r[(i + 2) % 3]), nrm) / D for i in range(3)], 1)
        es = (np.linalg.norm(c[1] - c[2], axis=1) + np.linalg.norm(c[1] - c[3], axis=1) +
              np.linalg.norm(c[2] - c[3], axis=1))
        eps = th / (es / 3.0)
        fail &= (w < -eps[:, None]).any(1)
    return fail


def random_steps(rng, n, edge, motion, spread=3.0, layer=0.0):
    base = rng.uniform(-0.5, 0.5, (n, 3))
    tri = np.stack([np.zeros((n, 3)), np.tile([edge, 0, 0], (n, 1)), np.tile([0, edge, 0], (n, 1))])
    tri = tri + rng.normal(0, 0.2 * edge, (3, n, 3))
    pt = rng.uniform(-spread * edge, (1 + spread) * edge, (n, 3))
    pt[:, 2] = layer + rng.normal(0, 0.5 * edge, n)
    X = np.concatenate([pt[None], tri]) + base
    P = X + rng.normal(0, 1, (4, n, 3)) * motion
    return X.astype(f32), P.astype(f32)


def test_outside_all_step_never_rejects_a_possible_hit():
    rng = np.random.default_rng(2)
    th = 1e-3
    ts = np.linspace(0.0, 1.0, 257)
    n_out = 0
    for edge, motion, layer in [(1e-3, 1e-5, 0.0), (1e-3, 1e-4, 0.0), (1e-3, 1e-3, 0.0),
                                (1e-3, 1e-5, 2e-3), (8e-3, 2e-3, 0.0), (3e-2, 5e-3, 1e-3)]:
        X, P = random_steps(rng, 40_000, edge, motion, layer=layer)
        out = outside_all_step(X, P, th)
        n_out += out.sum()
        assert fails_inside_everywhere(X[:, out], P[:, out], th, ts).all()
    assert n_out > 50_000


def test_outside_all_step_declines_slivers():
    rng = np.random.default_rng(3)
    X, P = random_steps(rng, 5_000, 1e-3, 1e-5)
    # flatten the triangles into slivers: the third corner onto the first edge
    X[3] = X[1] + f32(0.3) * (X[2] - X[1])
    P[3] = P[1] + f32(0.3) * (P[2] - P[1])
    assert not outside_all_step(X, P, 1e-3).any()
