"""The autotuner times every GS launch form that applies and keeps the
fastest; the choice changes speed only, never the result."""
import numpy as np
import pytest

from positionbaseddynamicsold_gb300 import scenes
from positionbaseddynamicsold_gb300.pbd import GS_CLUSTER, GS_PER_COLOR, PBDObject, SolverPBD

pytestmark = pytest.mark.gpu

G = np.array([0.0, -9.8, 0.0], np.float32)


@pytest.mark.parametrize("res", [24, 200])
def test_autotune_keeps_results(res):
    sc = scenes.grid_cloth(res, res, 1.0, 1.0, jitter=1e-3, seed=3, pins=[0, res - 1])
    out = []
    for tune in (False, True):
        obj = PBDObject(sc, damping=1.0, gravity=G)
        obj.prepare()
        s = SolverPBD(obj)
        if tune:
            pre = obj.predicted()
            t = s.autotune(iterations=5, reps=3)
            np.testing.assert_array_equal(obj.predicted(), pre)   # state restored
            assert len(t["candidates"]) >= 4
            blocks = [c["block"] for c in t["candidates"]]
            assert blocks[:4] == [64, 128, 256, 512]
            assert all(c["us_per_sweep"] > 0 for c in t["candidates"])
            best = t["candidates"][t["best"]]
            assert s.gs_path() == best["path"]
            if best["path"] == GS_PER_COLOR:
                assert s.gs_block() == best["block"]
            if res == 24:
                # small enough for the cluster form
                assert any(c["path"] == GS_CLUSTER for c in t["candidates"])
        s.step(1.0 / 600, substeps=6, iterations=15, use_graph=True)
        out.append(obj.positions())
    np.testing.assert_array_equal(out[0], out[1])
