"""Small, self-contained GPU cases for kernel profiling (ncu captures).

    python -m positionbaseddynamicsold_gb300.profile_cases mlp
    python -m positionbaseddynamicsold_gb300.profile_cases ccd

mlp: a 1024 x 1024 hanging cloth (1,048,576 points, inputs far larger than
     L2), the trained warm start applied once to the advected positions
     (k_eval_hinges, k_mlp_infer) and one training pass over the same points'
     features (k_mlp_train).
ccd: the drape256 scene after 160 substeps (the cloth lies on the sphere),
     one CCD pass (k_point_pairs, k_dist_filter, k_narrow).
ccd_fold: the fold1024 scene (1,048,576 points, ground plane) after 120
     substeps, one CCD pass.
ccd_fold_ee: the fold scene at 512 x 512 over 2 m x 2 m (262,144 points,
     fold1024's spacing) after 120 substeps, one CCD pass with edge-edge CCD on (k_ee_entries, k_ee_gather,
     k_ee_pairs, k_ee_filter, k_ee_narrow: about 4.6 M edge-cell entries).
Each case runs its kernels once after one warm-up call, so `-c` small
captures the steady-state launch.
"""
from __future__ import annotations

import sys

import numpy as np

from . import scenes
from .pbd import (RESPONSE_MASS_WEIGHTED, CollisionSolver, PBDObject, SolverPBD,
                  SpatialHashSystem, WarmStart)

DT = 1.0 / 600
G = np.array([0.0, -9.8, 0.0], np.float32)


def case_mlp():
    from . import warmstart_train as wt
    params, scales, _ = wt.load_params()
    sc = scenes.grid_cloth(1024, 1024, 4.0, 4.0, jitter=1e-4, seed=1, pins=[0, 1023])
    obj = PBDObject(sc, damping=1.0, gravity=G)
    obj.prepare()
    s = SolverPBD(obj)
    ws = WarmStart(params, scales)
    for _ in range(2):           # warm-up + profiled
        s.advect(DT)
        ws.predict(obj)
    x = ws.features(obj)
    rng = np.random.default_rng(0)
    t = rng.normal(0, 1, (len(x), 3)).astype(np.float32)
    for _ in range(2):
        ws.gradients(x, t)
    obj.sync()
    print("mlp case done: %d points" % obj.n_points)


def _ccd(sc, log2, substeps, edge_edge=False):
    obj = PBDObject(sc, damping=1.0, gravity=G)
    obj.prepare()
    shs = SpatialHashSystem(obj, cell_size=sc["colli"]["cell"], log2_table=log2)
    shs.init()
    cs = CollisionSolver(obj, shs, thickness=sc["colli"]["thickness"], iterations=1,
                         response=RESPONSE_MASS_WEIGHTED)
    n = obj.n_points
    cs.set_capacity(max(1 << 22, 64 * n), max(1 << 20, 4 * n))
    s = SolverPBD(obj)
    if "ground" in sc["colli"]:
        s.set_ground(True, sc["colli"]["ground"])
    s.step(DT, substeps=substeps, iterations=15, colli=cs, use_graph=True)
    s.advect(DT)
    cs.set_edge_edge(edge_edge)
    for _ in range(2):           # warm-up + profiled
        cs.ccd_sh_extended()
    obj.sync()
    print("ccd case done: %s%s" % (cs.stats(), " ee %s" % cs.ee_stats() if edge_edge else ""))


def case_ccd():
    _ccd(scenes.drape_over_sphere(res=256, seed=0), 20, 160)


def case_ccd_fold():
    _ccd(scenes.folding_cloth(res=1024, seed=0), 24, 120)


def case_ccd_fold_ee():
    _ccd(scenes.folding_cloth(res=512, seed=0, size=2.0), 22, 120, edge_edge=True)


if __name__ == "__main__":
    {"mlp": case_mlp, "ccd": case_ccd, "ccd_fold": case_ccd_fold,
     "ccd_fold_ee": case_ccd_fold_ee}[sys.argv[1]]()
