"""Resuming from the reference's caches on the GPU: an object created from
the two cache files equals one created from the same arrays (substeps bit
for bit), and an object's saved state reads back as that state."""
import os

import numpy as np
import pytest

from positionbaseddynamicsold_gb300 import pbd
from positionbaseddynamicsold_gb300.pbd import PBDObject, SolverPBD

pytestmark = pytest.mark.gpu

IO = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "io")


def test_object_from_cache_equals_object_from_arrays(tmp_path):
    t, c = os.path.join(IO, "topol.cache"), os.path.join(IO, "constr.cache")
    sc = pbd.read_cache(t, c)
    a = PBDObject.from_cache(t, c)
    b = PBDObject(sc, damping=sc["damping"], gravity=sc["gravity"])
    b.set_predicted(sc["predicted"])
    np.testing.assert_array_equal(a.predicted(), b.predicted())
    out = []
    for o in (a, b):
        o.prepare()
        s = SolverPBD(o)
        s.step(1.0 / 600, substeps=5, iterations=10, use_graph=False)
        out.append(o.positions())
    np.testing.assert_array_equal(out[0], out[1])
    # the state after the substeps, saved and read back (6 significant digits)
    a.save_cache(str(tmp_path / "t.cache"), str(tmp_path / "c.cache"))
    back = pbd.read_cache(str(tmp_path / "t.cache"), str(tmp_path / "c.cache"))
    np.testing.assert_allclose(back["pos"], out[0], rtol=1e-5, atol=1e-8)
    np.testing.assert_allclose(back["vel"], a.velocities(), rtol=1e-5, atol=1e-6)
    np.testing.assert_array_equal(back["prim_list"], sc["prim_list"])
    np.testing.assert_array_equal(back["ctype"], sc["ctype"])
    assert back["damping"] == pytest.approx(sc["damping"])
