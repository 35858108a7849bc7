"""What the trained warm start gains over the plain sweeps, on held-out
cloths of its training family (hanging, 1-4 pinned corners, wind), at the
stretch-residual target it was trained for (1e-3): from identical states it
needs at most half the sweeps of the plain solve while reaching the target
at least as often, and along its own trajectories it needs fewer sweeps over
the first substeps, where the target is reachable."""
import os

import pytest

from positionbaseddynamicsold_gb300 import warmstart_train as wt

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained():
    assert os.path.exists(wt.DEFAULT_WEIGHTS), "trained weights missing"
    params, scales, meta = wt.load_params()
    return params, scales, float(meta["target"])


def test_same_state_sweeps(trained):
    params, scales, tgt = trained
    r = wt.evaluate_same_state(params, scales, n_traj=2, substeps=15, target=tgt,
                               side_lo=64, side_hi=128, seed=11)
    assert r["both_reached"] >= 20
    assert r["learned_reached"] >= r["plain_reached"] - 1
    assert 2 * r["learned_sweeps"] <= r["plain_sweeps"], r


def test_closed_loop_sweeps_while_reachable(trained):
    params, scales, tgt = trained
    r = wt.evaluate(params, scales, n_traj=2, substeps=10, target=tgt, side_lo=64,
                    side_hi=128, seed=11, early=10)
    p, l = r["plain"], r["learned"]
    assert p["early_reached"] == p["early_substeps"] == 20
    assert l["early_reached"] >= 19
    assert l["early_sweeps"] < p["early_sweeps"], r
