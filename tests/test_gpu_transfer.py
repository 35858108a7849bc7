"""Host transfers of the object state: pageable arrays (through the object's
page-locked staging) and page-locked arrays (copied directly) round-trip
exactly; set_state has read the caller's arrays when it returns; the mass
column stays on the positions; a step between upload and download sees the
uploaded state."""
import numpy as np
import pytest
import torch

from positionbaseddynamicsold_gb300 import scenes
from positionbaseddynamicsold_gb300.pbd import PBDObject, SolverPBD

pytestmark = pytest.mark.gpu

G = np.array([0.0, -9.8, 0.0], np.float32)


def pinned(shape):
    return torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()


@pytest.mark.parametrize("kind", ["pageable", "page-locked"])
def test_state_round_trip(kind):
    sc = scenes.grid_cloth(37, 29, 1.0, 1.0, jitter=1e-3, seed=1, pins=[0])
    obj = PBDObject(sc, damping=1.0, gravity=G)
    obj.prepare()
    n = obj.n_points
    rng = np.random.default_rng(0)
    x = rng.normal(size=(n, 3)).astype(np.float32)
    v = rng.normal(size=(n, 3)).astype(np.float32)
    if kind == "page-locked":
        xs, vs = pinned((n, 3)), pinned((n, 3))
        xs[:], vs[:] = x, v
    else:
        xs, vs = x.copy(), v.copy()
    obj.set_state(xs, vs)
    xs[:] = 7.0          # the call has read the arrays already
    vs[:] = 7.0
    if kind == "page-locked":
        xo, vo = pinned((n, 3)), pinned((n, 3))
        obj.get_state(xo, vo)
    else:
        xo, vo = obj.get_state()
    np.testing.assert_array_equal(xo, x)
    np.testing.assert_array_equal(vo, v)
    np.testing.assert_array_equal(obj.positions(), x)
    np.testing.assert_array_equal(obj.velocities(), v)


def test_step_between_transfers_equals_resident_steps():
    sc = scenes.grid_cloth(30, 30, 1.0, 1.0, jitter=1e-3, seed=2, pins=[0, 29])
    a = PBDObject(sc, damping=1.0, gravity=G)
    b = PBDObject(sc, damping=1.0, gravity=G)
    for o in (a, b):
        o.prepare()
    sa, sb = SolverPBD(a), SolverPBD(b)
    xh, vh = pinned((a.n_points, 3)), pinned((a.n_points, 3))
    a.get_state(xh, vh)
    for _ in range(10):
        a.set_state(xh, vh)
        sa.step(1.0 / 600, 1, 15, None, True)
        a.get_state(xh, vh)
        sb.step(1.0 / 600, 1, 15, None, True)
    np.testing.assert_array_equal(xh, b.positions())
    np.testing.assert_array_equal(vh, b.velocities())
    # pinned points kept their inverse mass 0 through the uploads
    np.testing.assert_array_equal(xh[[0, 29]], sc["pos"][[0, 29]])
