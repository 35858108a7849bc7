"""The CPU oracle of the learned warm start: BF16 rounding, the float64
network's backward pass against central finite differences, Adam against
its defining recurrences, and the feature stencil on a small grid."""
import numpy as np

from oracle import mlp_oracle as M
from positionbaseddynamicsold_gb300 import scenes


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -7, -2.5, 3.0e-5],
                 np.float32)
    r = M.bf16(x)
    # 1 + 2^-8 is a tie: to even (1.0); 1 + 3*2^-8 ties to 1 + 2^-6
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == 1.0 + 2 ** -7
    assert r[4] == -2.5
    assert abs(r[5] - 3.0e-5) <= 3.0e-5 * 2 ** -8


def test_float64_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = M.init_params(3).astype(np.float64)
    p[M.OFF_W3:M.OFF_B3] *= 10.0          # a non-trivial output layer
    p[M.OFF_B2:M.OFF_W3] = rng.normal(0, 0.3, M.N_HID)
    X = rng.normal(0, 1, (40, 16))
    T = rng.normal(0, 0.5, (40, 3))
    mask = (rng.uniform(size=40) > 0.2).astype(np.float64)
    loss, g = M.loss_and_grad(p, X, T, mask, bf16_ops=False)
    idx = rng.choice(M.N_PARAMS, 120, replace=False)
    idx = np.concatenate([idx, [M.OFF_W1 + 15, M.OFF_B2 + 3, M.OFF_B3, M.OFF_B3 + 2]])
    h = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += h
        lp, _ = M.loss_and_grad(q, X, T, mask, bf16_ops=False)
        q[i] -= 2 * h
        lm, _ = M.loss_and_grad(q, X, T, mask, bf16_ops=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_adam_recurrence():
    p = np.array([1.0, -2.0, 0.5])
    g = np.array([0.1, -0.3, 0.0])
    m = np.zeros(3)
    v = np.zeros(3)
    p1, m1, v1 = M.adam(p, m, v, g, 1, lr=1e-2)
    # first bias-corrected step moves each parameter by lr * sign(g)
    np.testing.assert_allclose(p1, p - 1e-2 * np.sign(g) * (np.abs(g) / (np.abs(g) + 1e-8)),
                               rtol=0, atol=1e-12)
    np.testing.assert_allclose(m1, 0.1 * g)
    np.testing.assert_allclose(v1, 0.001 * g * g)


def test_feature_stencil_on_a_grid():
    sc = scenes.grid_cloth(5, 4, 0.4, 0.3, pins=[0])
    st = M.stencil(sc)
    # an interior point of a triangulated grid has six incident edges
    i = 1 * 5 + 2
    assert (st["nb"][i] >= 0).all()
    assert st["lbar"][i] > 0
    # the pinned corner: pinned flag, inverse-mass share 0
    F = M.features(sc, sc["pos"])
    assert F[0, 10] == 1.0 and F[0, 9] == 0.0
    assert (F[:, 15] == 1.0).all()
    # the rest state has no strain and no dihedral deviation
    assert np.abs(F[:, :6]).max() < 1e-6
    assert np.abs(F[:, 11:15]).max() < 1e-6
