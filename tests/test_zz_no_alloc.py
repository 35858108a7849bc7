"""pbd_residual_noalloc: the residual for callers that cannot allocate device
memory, checked against pbd_constraints_residual.

The caller here owns every device buffer (allocated with torch, as an engine
would from its own arena) and hands the library only pointers; the library
computes the residual with its fixed file-scope scratch and allocates
nothing.  Two calls in a row must both agree with the allocating entry point
within the residual tolerance of the other parity tests (1e-6 relative) and
with each other exactly.  The other cases: distance-only and bending-only
calls (their sums add up to the full call's, and the distance-only residual
is the stretch residual), a point id out of range (NaN, and the next clean
call is right again: the flag is cleared), and a constraint count above the
array's maximum (refused on the host before any launch).  Collected last so
a failure here leaves the rest of the suite already run.
"""
import numpy as np
import pytest

from positionbaseddynamicsold_gb300 import scenes
from positionbaseddynamicsold_gb300.pbd import (PBDError, PBDObject, SolverPBD,
                                                residual_noalloc)

pytestmark = pytest.mark.gpu

MAX_CONSTRAINTS = 1 << 24


@pytest.fixture(scope="module")
def case():
    torch = pytest.importorskip("torch")
    sc = scenes.hanging_cloth(32, seed=4)
    obj = PBDObject(sc, damping=0.9, gravity=(0.0, -9.8, 0.0))
    obj.prepare()
    s = SolverPBD(obj)
    s.advect(1.0 / 600)
    s.project_constraint(5)
    want = obj.residual()
    want_stretch = obj.residual_stretch()
    assert want > 0.0 and want_stretch > 0.0

    dist = np.nonzero(sc["ctype"] == scenes.DISTANCE)[0]
    bend = np.nonzero(sc["ctype"] == scenes.BENDING)[0]
    pl, ix = sc["prim_list"], sc["indices"]
    didx = np.stack([ix[pl[dist, 0]], ix[pl[dist, 0] + 1]], 1).astype(np.int32)
    bidx = np.stack([ix[pl[bend, 0] + k] for k in range(4)], 1).astype(np.int32)
    x0 = sc["pos"].astype(np.float64)
    hinge = np.linalg.norm(x0[bidx[:, 1]] - x0[bidx[:, 0]], axis=1).astype(np.float32)
    p = obj.predicted()
    pos4 = np.concatenate([p, sc["mass"][:, None]], 1).astype(np.float32)

    dev = torch.device("cuda", 0)
    t = {"pos": torch.from_numpy(pos4).to(dev),
         "didx": torch.from_numpy(didx).to(dev),
         "rest": torch.from_numpy(sc["rest_length"][dist].copy()).to(dev),
         "bidx": torch.from_numpy(bidx).to(dev),
         "ang": torch.from_numpy(sc["rest_angle"][bend].copy()).to(dev),
         "hinge": torch.from_numpy(hinge).to(dev)}
    return {"torch": torch, "dev": dev, "t": t, "n": len(pos4), "nd": len(dist),
            "nb": len(bend), "want": want, "want_stretch": want_stretch, "obj": obj}


def call(c, nd=None, nb=None, didx=None):
    """one call on the case's buffers; nd / nb: constraint counts passed
    (0 leaves that kind's buffers out); returns [residual, sum C^2, sum L^2]"""
    torch, dev, t = c["torch"], c["dev"], c["t"]
    nd = c["nd"] if nd is None else nd
    nb = c["nb"] if nb is None else nb
    didx = t["didx"] if didx is None else didx
    out = torch.full((3,), -1.0, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    residual_noalloc(t["pos"].data_ptr(), c["n"],
                     didx.data_ptr() if nd else 0, t["rest"].data_ptr() if nd else 0, nd,
                     t["bidx"].data_ptr() if nb else 0, t["ang"].data_ptr() if nb else 0,
                     t["hinge"].data_ptr() if nb else 0, nb, out.data_ptr(),
                     stream.cuda_stream)
    torch.cuda.synchronize(dev)
    return out.cpu().numpy()


def test_residual_noalloc_matches_allocating_entry_point(case):
    want = case["want"]
    got = [call(case), call(case)]
    for g in got:
        assert abs(g[0] - want) <= 1e-6 * want, (g[0], want)
    assert got[0][0] == got[1][0]
    assert got[0][1] > 0.0 and got[0][2] > 0.0


def test_residual_noalloc_distance_only_and_bending_only(case):
    full = call(case)
    d = call(case, nb=0)
    b = call(case, nd=0)
    # distance constraints alone: the stretch residual of the allocating path
    ws = case["want_stretch"]
    assert abs(d[0] - ws) <= 1e-6 * ws, (d[0], ws)
    # the two kinds' sums make up the full call's (same terms, other order)
    np.testing.assert_allclose(d[1] + b[1], full[1], rtol=1e-12)
    np.testing.assert_allclose(d[2] + b[2], full[2], rtol=1e-12)
    assert b[0] > 0.0 and np.isfinite(b[0])


def test_residual_noalloc_point_id_out_of_range_gives_nan_then_recovers(case):
    bad = case["t"]["didx"].clone()
    bad[0, 1] = case["n"]          # one past the last point: skipped by the kernel
    got = call(case, didx=bad)
    assert np.isnan(got[0])
    # the next clean call clears the flag and is right again
    ok = call(case)
    assert abs(ok[0] - case["want"]) <= 1e-6 * case["want"]


def test_residual_noalloc_refuses_more_constraints_than_the_array_holds(case):
    # rejected on the host before any launch: nothing is read
    with pytest.raises(PBDError) as e:
        call(case, nd=MAX_CONSTRAINTS - case["nb"] + 1)
    assert "exceed the maximum" in str(e.value)
    with pytest.raises(PBDError):
        call(case, nd=MAX_CONSTRAINTS + 1, nb=0)
    ok = call(case)
    assert abs(ok[0] - case["want"]) <= 1e-6 * case["want"]
