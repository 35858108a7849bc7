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


def test_contact_weights_cut_the_sweeps_of_a_held_out_fold():
    """The network trained on contact states (folds on the ground, drapes
    over a sphere) on a fold it was not trained on (seed outside the
    training range): from identical states, the warm-started solve reaches
    the residual of 60 plain sweeps with at most 3/4 of their sweeps in
    total, on at least 5 of 6 substeps, and its device time is lower."""
    from positionbaseddynamicsold_gb300 import scenes
    assert os.path.exists(wt.CONTACT_WEIGHTS), "trained contact weights missing"
    params, scales, meta = wt.load_params(wt.CONTACT_WEIGHTS)
    sc = scenes.folding_cloth(res=160, seed=987_654, size=160 * 4.0 / 1024)
    r = wt.evaluate_contact_same_state(params, scales, sc, 18, preroll=120, substeps=6,
                                       sweeps=60, chunk=10)
    assert r["learned_reached"] >= 5, r
    assert r["learned_sweeps"] <= 0.75 * r["plain_sweeps"], r
    assert r["learned_ms"] < r["plain_ms"], r
    # the plain residual levels off: 200 sweeps take it little below 60
    curve = {c["sweeps"]: c["stretch_residual"] for c in r["residual_curve_first_state"]}
    assert curve[200] > 0.5 * curve[60] > 0.0


def test_hanging_weights_cut_the_sweeps_of_a_held_out_drape():
    """The network trained on pinned hanging cloths on a scene family it was
    not trained on, a drape over a sphere (a 128² cloth in contact from its
    first substep): from identical states the warm-started solve reaches the
    residual of 60 plain sweeps with at most 3/4 of their sweeps in total,
    on at least 5 of 6 substeps, and its device time is lower."""
    from positionbaseddynamicsold_gb300 import scenes
    assert os.path.exists(wt.DEFAULT_WEIGHTS), "trained hanging-cloth weights missing"
    params, scales, meta = wt.load_params(wt.DEFAULT_WEIGHTS)
    sc = scenes.drape_over_sphere(res=128, seed=765_432, start="contact")
    r = wt.evaluate_contact_same_state(params, scales, sc, 18, preroll=0, substeps=6,
                                       sweeps=60, chunk=10)
    assert r["learned_reached"] >= 5, r
    assert r["learned_sweeps"] <= 0.75 * r["plain_sweeps"], r
    assert r["learned_ms"] < r["plain_ms"], r
