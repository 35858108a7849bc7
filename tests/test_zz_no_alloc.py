"""pbd_residual_noalloc: the residual for callers that cannot allocate device
memory, checked against pbd_constraints_residual.

The caller here owns every device buffer (allocated with torch, as an engine
would from its own arena) and hands the library only pointers; the library
computes the residual with its fixed file-scope scratch and allocates
nothing.  Two calls in a row must both agree with the allocating entry point
within the residual tolerance of the other parity tests (1e-6 relative) and
with each other exactly.  Collected last so a failure here leaves the rest of
the suite already run.
"""
import numpy as np
import pytest

from positionbaseddynamicsold_gb300 import scenes
from positionbaseddynamicsold_gb300.pbd import PBDObject, SolverPBD, residual_noalloc

pytestmark = pytest.mark.gpu


def test_residual_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    sc = scenes.hanging_cloth(32, seed=4)
    obj = PBDObject(sc, damping=0.9, gravity=(0.0, -9.8, 0.0))
    obj.prepare()
    s = SolverPBD(obj)
    s.advect(1.0 / 600)
    s.project_constraint(5)
    want = obj.residual()
    assert want > 0.0

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
    t_pos = torch.from_numpy(pos4).to(dev)
    t_didx = torch.from_numpy(didx).to(dev)
    t_rest = torch.from_numpy(sc["rest_length"][dist].copy()).to(dev)
    t_bidx = torch.from_numpy(bidx).to(dev)
    t_ang = torch.from_numpy(sc["rest_angle"][bend].copy()).to(dev)
    t_hinge = torch.from_numpy(hinge).to(dev)
    stream = torch.cuda.current_stream(dev)
    got = []
    for _ in range(2):
        out = torch.full((3,), -1.0, dtype=torch.float64, device=dev)
        residual_noalloc(t_pos.data_ptr(), len(pos4), t_didx.data_ptr(), t_rest.data_ptr(),
                         len(dist), t_bidx.data_ptr(), t_ang.data_ptr(), t_hinge.data_ptr(),
                         len(bend), out.data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize(dev)
        got.append(out.cpu().numpy())
    for g in got:
        assert abs(g[0] - want) <= 1e-6 * want, (g[0], want)
    assert got[0][0] == got[1][0]
    assert got[0][1] > 0.0 and got[0][2] > 0.0
