"""The learned warm start on the GPU against its CPU oracle: the tensor-core
forward pass, the gradients of the tensor-core backward pass, Adam, the
feature kernel, the prediction applied to an object, and the guard that
falls back to the plain sweeps when a prediction raises the residual."""
import numpy as np
import pytest

from oracle import mlp_oracle as M
from positionbaseddynamicsold_gb300 import scenes
from positionbaseddynamicsold_gb300.pbd import PBDObject, SolverPBD, WarmStart

pytestmark = pytest.mark.gpu

G = np.array([0.0, -9.8, 0.0], np.float32)
DT = 1.0 / 600


def random_params(seed, out_scale=3.0):
    rng = np.random.default_rng(seed)
    p = M.init_params(seed).astype(np.float64)
    p[M.OFF_W3:M.OFF_B3] *= out_scale
    p[M.OFF_B2:M.OFF_W3] = rng.normal(0, 0.2, M.N_HID)
    p[M.OFF_B3:] = rng.normal(0, 0.05, 3)
    return p.astype(np.float32)


@pytest.mark.parametrize("n", [1, 127, 128, 1000, 5000])
def test_forward_matches_oracle(n):
    p = random_params(1)
    ws = WarmStart(p)
    x = np.random.default_rng(n).normal(0, 1, (n, 16)).astype(np.float32)
    y = ws.forward(x)
    want, _ = M.forward(p, x)
    scale = max(1.0, np.abs(want).max())
    assert np.abs(y - want).max() <= 2e-3 * scale


def test_gradients_match_oracle():
    p = random_params(2)
    ws = WarmStart(p)
    rng = np.random.default_rng(7)
    n = 3000
    x = rng.normal(0, 1, (n, 16)).astype(np.float32)
    t = rng.normal(0, 0.3, (n, 3)).astype(np.float32)
    mask = (rng.uniform(size=n) > 0.1).astype(np.float32)
    g, loss = ws.gradients(x, t, mask)
    want_loss, want = M.loss_and_grad(p, x, t, mask)
    assert abs(loss - want_loss) <= 1e-4 * want_loss
    err = np.linalg.norm(g - want) / np.linalg.norm(want)
    assert err <= 5e-3, err
    # every parameter block, separately
    for a, b in [(M.OFF_W1, M.OFF_W2), (M.OFF_W2, M.OFF_B2), (M.OFF_B2, M.OFF_W3),
                 (M.OFF_W3, M.OFF_B3), (M.OFF_B3, M.N_PARAMS)]:
        e = np.linalg.norm(g[a:b] - want[a:b]) / max(np.linalg.norm(want[a:b]), 1e-12)
        assert e <= 1e-2, (a, b, e)
    # and the exact float64 network agrees to BF16 accuracy
    _, exact = M.loss_and_grad(p, x, t, mask, bf16_ops=False)
    assert np.linalg.norm(g - exact) / np.linalg.norm(exact) <= 3e-2


def test_adam_matches_oracle():
    p = random_params(3)
    ws = WarmStart(p)
    rng = np.random.default_rng(4)
    m = np.zeros(M.N_PARAMS)
    v = np.zeros(M.N_PARAMS)
    q = p.astype(np.float64)
    for t in range(1, 4):
        g = rng.normal(0, 1e-2, M.N_PARAMS).astype(np.float32)
        ws.set_gradient(g)
        ws.adam(1e-3)
        q, m, v = M.adam(q, m, v, g.astype(np.float64), t, 1e-3)
    np.testing.assert_allclose(ws.params(), q, rtol=0, atol=2e-6)


def small_scene(seed=0, res=12):
    sc = scenes.grid_cloth(res, res, 0.5, 0.5, jitter=1e-3, seed=seed, pins=[0, res - 1])
    return sc


def test_features_match_oracle():
    sc = small_scene()
    obj = PBDObject(sc, damping=1.0, gravity=G)
    obj.prepare()
    rng = np.random.default_rng(5)
    pos = sc["pos"] + rng.normal(0, 2e-3, sc["pos"].shape).astype(np.float32)
    obj.set_predicted(pos)
    ws = WarmStart()
    x = ws.features(obj)
    want = M.features(sc, pos)
    # GPU features are FP32 rounded to BF16; allow one BF16 ulp
    tol = 2.0 ** -7 * np.maximum(np.abs(want), 1e-30) + 1e-6
    assert (np.abs(x - want) <= tol).all()


def test_predict_moves_free_points_by_lbar_times_output():
    sc = small_scene(1)
    obj = PBDObject(sc, damping=1.0, gravity=G)
    obj.prepare()
    p = random_params(6, out_scale=1.0)
    ws = WarmStart(p)
    pos = sc["pos"].copy()
    obj.set_predicted(pos)
    x = ws.features(obj)
    y = ws.forward(x)
    ws.predict(obj)
    got = obj.predicted()
    st = M.stencil(sc)
    free = (st["w"] != 0) & (st["lbar"] > 0)
    want = pos.astype(np.float64).copy()
    want[free] += y[free] * st["lbar"][free, None]
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-6)
    np.testing.assert_array_equal(got[~free], pos[~free])


def test_guard_reverts_a_bad_prediction_to_the_plain_solve():
    """a network whose output is a large constant raises the residual; the
    substep then equals the plain solve bit for bit"""
    sc = small_scene(2)
    p = np.zeros(M.N_PARAMS, np.float32)
    p[M.OFF_B3:] = [0.3, -0.2, 0.25]
    res = []
    for learned in (False, True):
        obj = PBDObject(sc, damping=1.0, gravity=G)
        obj.prepare()
        s = SolverPBD(obj)
        if learned:
            ws = WarmStart(p)
            s.set_warmstart(ws)
        s.step_to_residual(DT, substeps=4, target=1e-9, max_sweeps=20, chunk=5)
        st = s.solve_stats()
        res.append((obj.positions(), st))
    np.testing.assert_array_equal(res[0][0], res[1][0])
    assert res[1][1]["reverts"] == 4 and res[0][1]["reverts"] == 0
    assert res[1][1]["sweeps"] == res[0][1]["sweeps"] == 80
