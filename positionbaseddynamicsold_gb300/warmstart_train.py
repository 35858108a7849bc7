"""Training and evaluation of the learned warm start on solver trajectories.

Trajectories (the hanging-cloth family): a square cloth of 1 m x 1 m with
side U{side_lo..side_hi} points, 1-4 random corners pinned, y jitter
U(+-1e-3), gravity -9.8 plus a constant wind acceleration U(0, 5) m/s^2 in a
random horizontal direction, substeps of 1/600 s.

Training: every substep is advected, its features recorded
(pbd_warmstart_record), solved by the plain colored sweeps to the residual
target (pbd_solver_project_to_residual), and the network takes one Adam step
on the (features, correction) pairs of all the cloth's points
(pbd_warmstart_train_step); the forward and backward passes run on the
tensor cores.

Evaluation: held-out seeds, each trajectory run twice through
pbd_solver_step_to_residual, plain and warm-started; reported per path: GS
sweeps, substeps that reached the target, rejected predictions, time.

    python -m positionbaseddynamicsold_gb300.warmstart_train --trajectories 2000 \\
        --out positionbaseddynamicsold_gb300/data/warmstart.npz
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import scenes
from .pbd import (RESPONSE_MASS_WEIGHTED, CollisionSolver, PBDObject, SolverPBD,
                  SpatialHashSystem, WarmStart)

DT = 1.0 / 600
PKG = os.path.dirname(os.path.abspath(__file__))
DEFAULT_WEIGHTS = os.path.join(PKG, "data", "warmstart.npz")
# trained on the contact families (folds on the ground, drapes over a sphere)
CONTACT_WEIGHTS = os.path.join(PKG, "data", "warmstart_contact.npz")

N_IN, N_HID, N_OUT = 16, 64, 3
N_PARAMS = N_HID * N_IN + N_HID * N_HID + N_HID + N_OUT * N_HID + N_OUT


def init_params(seed=0):
    """uniform fan-in initialisation; small output layer, zero biases"""
    rng = np.random.default_rng(seed)
    W1 = rng.uniform(-1, 1, (N_HID, N_IN)) * np.sqrt(3.0 / N_IN)
    W2 = rng.uniform(-1, 1, (N_HID, N_HID)) * np.sqrt(3.0 / N_HID)
    W3 = rng.uniform(-1, 1, (N_OUT, N_HID)) * 0.1 * np.sqrt(3.0 / N_HID)
    return np.concatenate([W1.ravel(), W2.ravel(), np.zeros(N_HID), W3.ravel(),
                           np.zeros(N_OUT)]).astype(np.float32)


def trajectory(seed, side_lo=64, side_hi=256):
    """one scene of the family, with its gravity (+ wind) vector"""
    rng = np.random.default_rng(seed)
    side = int(rng.integers(side_lo, side_hi + 1))
    corners = np.array([0, side - 1, side * (side - 1), side * side - 1])
    pins = rng.choice(corners, int(rng.integers(1, 5)), replace=False)
    sc = scenes.grid_cloth(side, side, 1.0, 1.0, jitter=1e-3, seed=seed, pins=pins)
    ang = rng.uniform(0, 2 * np.pi)
    wind = rng.uniform(0, 5)
    g = np.array([wind * np.cos(ang), -9.8, wind * np.sin(ang)], np.float32)
    return sc, g


def fit_scales(seed=0, n_traj=4, substeps=40, target=1e-3, max_sweeps=200, chunk=5,
               side_lo=64, side_hi=256):
    """input / output scales from plain-solver trajectories: 1/std of the
    strains, of the corrections / lbar and of the dihedral deviations; the
    output scale is the corrections' std (so the network's targets are O(1))"""
    ws = WarmStart()
    rows = []
    for k in range(n_traj):
        sc, g = trajectory(50_000 + seed * 100_003 + k, side_lo, side_hi)
        obj = PBDObject(sc, damping=1.0, gravity=g)
        obj.prepare()
        s = SolverPBD(obj)
        for j in range(substeps):
            s.advect(DT)
            if j > 0:
                rows.append(ws.features(obj))
            s.project_to_residual(target, max_sweeps, chunk)
            s.integration(DT)
        s.close()
        obj.close()
    X = np.concatenate(rows).astype(np.float64)

    def inv_std(cols):
        sd = float(np.sqrt(np.mean(X[:, cols] ** 2)))
        return 1.0 / sd if sd > 1e-12 else 1.0

    sc_ = np.ones(17, np.float32)
    sc_[0:6] = inv_std(slice(0, 6))
    sd_corr = 1.0 / inv_std(slice(6, 9))
    sc_[6:9] = 1.0 / sd_corr
    sc_[11:15] = inv_std(slice(11, 15))
    sc_[16] = sd_corr
    return sc_


def train(n_traj=2000, substeps=40, target=1e-3, max_sweeps=200, chunk=5, lr=1e-3, seed=0,
          side_lo=64, side_hi=256, log=print, params=None, scales=None, on_policy=False,
          traj_offset=10_000):
    """on_policy = False: trajectories of the plain solver; True: the
    trajectory follows the warm-started solve while the targets stay the
    plain solve's corrections of the same states"""
    ws = WarmStart(init_params(seed) if params is None else params, scales)
    hist = []
    t0 = time.time()
    for k in range(n_traj):
        sc, g = trajectory(traj_offset + seed * 100_003 + k, side_lo, side_hi)
        obj = PBDObject(sc, damping=1.0, gravity=g)
        obj.prepare()
        s = SolverPBD(obj)
        losses = []
        for j in range(substeps):
            losses.append(s.train_substep(ws, DT, target, max_sweeps, chunk, lr, on_policy,
                                          want_loss=(j % 10 == 9)))
        ls = [x for x in losses if x is not None]
        hist.append(float(np.mean(ls)) if ls else float("nan"))
        if log and (k % 50 == 49 or k == n_traj - 1):
            log(f"trajectory {k + 1}/{n_traj}: loss {np.mean(hist[-50:]):.4e}  "
                f"{time.time() - t0:.0f}s")
        s.close()
        obj.close()
    return ws.params(), hist


def evaluate(params, scales, n_traj=20, substeps=40, target=1e-3, max_sweeps=200, chunk=5,
             seed=7, side_lo=64, side_hi=256, min_sweeps=0, early=15):
    """closed loop: plain and warm-started pbd_solver_step_to_residual, each
    on its own trajectory of the held-out scenes; sweeps and substeps that
    reached the target, over all substeps and over the first `early` ones
    (where the target is reachable for both), and host wall time"""
    keys = ("sweeps", "reached", "substeps", "reverts")
    out = {}
    for name in ("plain", "learned"):
        out[name] = {k: 0 for k in keys}
        out[name].update({"seconds": 0.0, "early_sweeps": 0, "early_reached": 0,
                          "early_substeps": 0})
    ws = WarmStart(params, scales)
    for k in range(n_traj):
        sc, g = trajectory(900_000 + seed * 100_003 + k, side_lo, side_hi)
        for name in ("plain", "learned"):
            obj = PBDObject(sc, damping=1.0, gravity=g)
            obj.prepare()
            s = SolverPBD(obj)
            if name == "learned":
                s.set_warmstart(ws, min_sweeps)
            o = out[name]
            for j in range(substeps):
                t0 = time.perf_counter()
                s.step_to_residual(DT, 1, target, max_sweeps, chunk)
                st = s.solve_stats(reset=True)   # synchronises
                if j:                             # the first substep builds the graph
                    o["seconds"] += time.perf_counter() - t0
                for key in keys:
                    o[key] += st[key]
                if j < early:
                    o["early_sweeps"] += st["sweeps"]
                    o["early_reached"] += st["reached"]
                    o["early_substeps"] += st["substeps"]
            s.close()
            obj.close()
    return out


def evaluate_same_state(params, scales, n_traj=8, substeps=40, target=1e-3, max_sweeps=200,
                        chunk=5, seed=7, side_lo=64, side_hi=256):
    """per-solve comparison from identical states: along plain-solver
    trajectories, every advected state is solved twice -- from the advected
    positions (plain) and from the guarded prediction (learned); sweeps are
    summed over the substeps where both reach the target"""
    ws = WarmStart(params, scales)
    out = {"substeps": 0, "both_reached": 0, "plain_sweeps": 0, "learned_sweeps": 0,
           "plain_reached": 0, "learned_reached": 0, "reverts": 0}
    for k in range(n_traj):
        sc, g = trajectory(900_000 + seed * 100_003 + k, side_lo, side_hi)
        obj = PBDObject(sc, damping=1.0, gravity=g)
        obj.prepare()
        s = SolverPBD(obj)
        for j in range(substeps):
            s.advect(DT)
            p0 = obj.predicted()
            dp = obj.correction() if j > 0 else np.zeros_like(p0)
            r0 = obj.residual_stretch()
            ws.predict(obj)
            rev = obj.residual_stretch() > r0
            if rev:
                obj.set_predicted(p0)
            swl, rl = s.project_to_residual(target, max_sweeps, chunk)
            obj.set_predicted(p0)
            obj.set_correction(dp)
            swp, rp = s.project_to_residual(target, max_sweeps, chunk)
            s.integration(DT)
            out["substeps"] += 1
            out["reverts"] += int(rev)
            out["plain_reached"] += int(rp <= target)
            out["learned_reached"] += int(rl <= target)
            if rp <= target and rl <= target:
                out["both_reached"] += 1
                out["plain_sweeps"] += swp
                out["learned_sweeps"] += swl
        s.close()
        obj.close()
    return out


# ---- contact families: cloths on the ground and over a sphere ------------

G0 = np.array([0.0, -9.8, 0.0], np.float32)


def contact_scene(seed, family):
    """one scene of a contact family, with its hash table size.
    fold: a square cloth of side U{96..256} points at fold1024's spacing
    (4 m / 1024), rotated, tilted and dropped onto the ground plane y = 0
    so it folds onto itself; drape: a cloth of side U{64..192} over 2 m
    whose free fall is fast-forwarded to just above an icosphere (level 4,
    r = 0.4)."""
    rng = np.random.default_rng(seed)
    if family == "fold":
        res = int(rng.integers(96, 257))
        sc = scenes.folding_cloth(res=res, seed=seed, size=res * 4.0 / 1024)
        return sc, 18
    if family == "drape":
        res = int(rng.integers(64, 193))
        sc = scenes.drape_over_sphere(res=res, seed=seed, sphere_level=4, start="contact")
        return sc, 18
    raise ValueError("family must be 'fold' or 'drape'")


def contact_solver(sc, log2):
    """object, solver, hash and collision solver as the benchmark sets them up
    (mass-weighted response, thickness and cell from the scene)"""
    obj = PBDObject(sc, damping=1.0, gravity=G0)
    obj.prepare()
    s = SolverPBD(obj)
    shs = SpatialHashSystem(obj, cell_size=sc["colli"]["cell"], log2_table=log2)
    shs.init()
    cs = CollisionSolver(obj, shs, thickness=sc["colli"]["thickness"], iterations=1,
                         response=RESPONSE_MASS_WEIGHTED)
    n = obj.n_points
    cs.set_capacity(max(1 << 22, 64 * n), max(1 << 20, 4 * n))
    if "ground" in sc["colli"]:
        s.set_ground(True, sc["colli"]["ground"])
    if "spheres" in sc["colli"]:
        s.set_instance_spheres(sc["colli"]["spheres"])
    if "instance_cells" in sc["colli"]:
        shs.set_instance_cells(sc["colli"]["instance_cells"])
    obj._keep = shs
    return obj, s, cs


def fit_contact_scales(seed=0, n_traj=6, families=("fold", "drape"), preroll=90, lead=3,
                       substeps=6, sweeps=60, chunk=10):
    """input / output scales (as fit_scales) from plain solves of contact
    states of the families"""
    ws = WarmStart()
    rows = []
    for k in range(n_traj):
        fam = families[k % len(families)]
        sc, log2 = contact_scene(60_000 + seed * 100_003 + k, fam)
        obj, s, cs = contact_solver(sc, log2)
        s.step(DT, preroll, 15, cs, True)
        s.step_to_residual(DT, lead, 0.0, sweeps, chunk, cs, True)
        for _ in range(substeps):
            s.advect(DT)
            rows.append(ws.features(obj))
            s.project_to_residual(0.0, sweeps, chunk, cs)
            s.integration(DT)
        cs.close()
        s.close()
        obj.close()
    X = np.concatenate(rows).astype(np.float64)

    def inv_std(cols):
        sd = float(np.sqrt(np.mean(X[:, cols] ** 2)))
        return 1.0 / sd if sd > 1e-12 else 1.0

    sc_ = np.ones(17, np.float32)
    sc_[0:6] = inv_std(slice(0, 6))
    sd_corr = 1.0 / inv_std(slice(6, 9))
    sc_[6:9] = 1.0 / sd_corr
    sc_[11:15] = inv_std(slice(11, 15))
    sc_[16] = sd_corr
    return sc_


def train_contact(ws, n_traj, families=("fold", "drape"), preroll=(30, 150), substeps=30,
                  sweeps=60, chunk=10, lr=1e-3, seed=0, on_policy=False, log=print,
                  traj_offset=20_000):
    """Training on contact states: each trajectory runs a random number of
    plain fixed-15-iteration substeps (in `preroll`) to reach contacts, then
    `substeps` training substeps: the advected state is solved by `sweeps`
    plain sweeps (chunks of `chunk`, a detection per chunk, the response
    after every sweep) and the network takes one Adam step on its points'
    (features, correction) pairs."""
    hist = []
    t0 = time.time()
    for k in range(n_traj):
        fam = families[k % len(families)]
        sd = traj_offset + seed * 100_003 + k
        sc, log2 = contact_scene(sd, fam)
        obj, s, cs = contact_solver(sc, log2)
        rng = np.random.default_rng(sd)
        s.step(DT, int(rng.integers(preroll[0], preroll[1] + 1)), 15, cs, True)
        losses = []
        for j in range(substeps):
            losses.append(s.train_substep(ws, DT, 0.0, sweeps, chunk, lr, on_policy, colli=cs,
                                          want_loss=(j % 10 == 9)))
        ls = [x for x in losses if x is not None]
        hist.append(float(np.mean(ls)) if ls else float("nan"))
        if log and (k % 20 == 19 or k == n_traj - 1):
            log(f"contact trajectory {k + 1}/{n_traj}: loss {np.mean(hist[-20:]):.4e}  "
                f"{time.time() - t0:.0f}s")
        cs.close()
        s.close()
        obj.close()
    return hist


def timed_solve(s, obj, cs, state, dprev, target, max_sweeps, chunk):
    """one substep solved to `target` from `state` (positions, velocities)
    with the solver's current warm start, through the CUDA graph of
    pbd_solver_step_to_residual; the graph is built by a first untimed run
    from the same state.  Returns (device ms, solve stats)."""
    import torch
    stream = torch.cuda.ExternalStream(obj.stream())
    out = None
    for rep in range(2):
        obj.set_state(*state)
        obj.set_correction(dprev)
        obj.sync()
        s.solve_stats(reset=True)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.step_to_residual(DT, 1, target, max_sweeps, chunk, cs, True)
        e1.record(stream)
        e1.synchronize()
        out = (e0.elapsed_time(e1), s.solve_stats(reset=True))
    return out


def residual_curve(s, obj, cs, state, dprev, ks, chunk=10):
    """stretch residual after k plain sweeps (chunks of `chunk`, a detection
    per chunk, the response after every sweep) of one advected state, for
    every k in ks"""
    out = []
    for k in ks:
        obj.set_state(*state)
        obj.set_correction(dprev)
        s.advect(DT)
        sw, r = s.project_to_residual(0.0, int(k), min(chunk, max(1, int(k))), cs)
        out.append({"sweeps": int(sw), "stretch_residual": float(r)})
    return out


def evaluate_contact_same_state(params, scales, sc, log2, preroll, substeps=8, sweeps=60,
                                chunk=10, lead=5, curve_ks=(0, 5, 10, 15, 30, 60, 120, 200)):
    """The warm start against the plain sweeps on a contact workload, from
    identical states along a plain trajectory: after `preroll` fixed
    15-iteration substeps and `lead` plain solved substeps (so the previous
    correction exists), each of `substeps` states is solved (a) plain with
    `sweeps` sweeps, whose final stretch residual r_K becomes the target,
    and (b) warm-started until the residual is at or below r_K (at most
    `sweeps`).  Both solves detect their first contacts from the same
    advected positions.  Reported: sweeps and device time of each solve
    (CUDA graph of pbd_solver_step_to_residual, graph built beforehand),
    the guard's rejections, and the plain residual curve of the first
    state."""
    obj, s, cs = contact_solver(sc, log2)
    ws = WarmStart(params, scales)
    s.step(DT, preroll, 15, cs, True)
    s.step_to_residual(DT, lead, 0.0, sweeps, chunk, cs, True)
    rows = []
    curve = None
    for j in range(substeps):
        state = obj.get_state()
        dprev = obj.correction()
        if curve is None:
            curve = residual_curve(s, obj, cs, state, dprev, curve_ks, chunk)
        s.set_warmstart(None)
        tp, stp = timed_solve(s, obj, cs, state, dprev, 0.0, sweeps, chunk)
        rk = stp["last_residual"]
        s.set_warmstart(ws)
        tl, stl = timed_solve(s, obj, cs, state, dprev, rk * (1.0 + 1e-9), sweeps, chunk)
        # the same state started from the previous substep's correction
        # (p0 + dprev, kept only if it lowers the residual): the warm start
        # without a network, for comparison (sweeps only)
        s.set_warmstart(None)
        obj.set_state(*state)
        obj.set_correction(dprev)
        s.advect(DT)
        p0 = obj.predicted()
        r0 = obj.residual_stretch()
        obj.set_predicted(p0 + dprev)
        if obj.residual_stretch() > r0:
            obj.set_predicted(p0)
        swd, rd = s.project_to_residual(rk * (1.0 + 1e-9), sweeps, chunk, cs)
        rows.append({"plain_sweeps": stp["sweeps"], "plain_ms": tp, "target": rk,
                     "learned_sweeps": stl["sweeps"], "learned_ms": tl,
                     "learned_reached": int(stl["reached"]), "reverted": int(stl["reverts"]),
                     "r_advected": stl["last_r0"], "r_predicted": stl["last_r1"],
                     "previous_correction_sweeps": int(swd),
                     "previous_correction_reached": int(rd <= rk * (1.0 + 1e-9))})
        # the trajectory goes on with the plain solve
        s.set_warmstart(None)
        obj.set_state(*state)
        obj.set_correction(dprev)
        s.step_to_residual(DT, 1, 0.0, sweeps, chunk, cs, True)
    s.set_warmstart(None)
    cs.close()
    s.close()
    obj.close()
    tp = sum(r["plain_ms"] for r in rows)
    tl = sum(r["learned_ms"] for r in rows)
    return {"substeps": len(rows), "sweeps_plain": sweeps, "chunk": chunk,
            "plain_ms": tp, "learned_ms": tl, "speedup": tp / tl if tl else None,
            "learned_reached": sum(r["learned_reached"] for r in rows),
            "reverted": sum(r["reverted"] for r in rows),
            "plain_sweeps": sum(r["plain_sweeps"] for r in rows),
            "learned_sweeps": sum(r["learned_sweeps"] for r in rows),
            "previous_correction_sweeps": sum(r["previous_correction_sweeps"] for r in rows),
            "previous_correction_reached": sum(r["previous_correction_reached"] for r in rows),
            "residual_curve_first_state": curve, "per_substep": rows}


def save(path, params, scales, meta):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez(path, params=np.asarray(params, np.float32), scales=np.asarray(scales, np.float32),
             meta=json.dumps(meta))


def load_params(path=DEFAULT_WEIGHTS):
    """(params, scales, meta) of a trained network"""
    d = np.load(path)
    return (d["params"].astype(np.float32), d["scales"].astype(np.float32),
            json.loads(str(d["meta"])))


def apply_once(params, scales, side=1024, repeats=3, sweeps=15, seed=0):
    """the network on one side^2 hanging cloth with eager launches (no
    graph): per repeat one substep's advection, the features and inference
    with the prediction applied (pbd_warmstart_predict), the recording, a
    plain solve of `sweeps` sweeps and one training step
    (pbd_warmstart_train_step); host-timed milliseconds per call, each call
    synchronised"""
    sc = scenes.grid_cloth(side, side, 1.0, 1.0, jitter=1e-3, seed=seed,
                           pins=np.array([0, side - 1]))
    obj = PBDObject(sc, damping=1.0, gravity=(0.0, -9.8, 0.0))
    obj.prepare()
    s = SolverPBD(obj)
    ws = WarmStart(params, scales)
    t = {"predict": [], "train_step": []}
    for _ in range(repeats):
        s.advect(DT)
        obj.sync()
        t0 = time.perf_counter()
        ws.predict(obj)
        obj.sync()
        t["predict"].append(1e3 * (time.perf_counter() - t0))
        ws.record(obj)
        s.project_constraint(sweeps)
        obj.sync()
        t0 = time.perf_counter()
        ws.train_step(obj, want_loss=True)
        t["train_step"].append(1e3 * (time.perf_counter() - t0))
        s.integration(DT)
    out = {"points": obj.n_points, "repeats": repeats,
           "predict_ms": t["predict"], "train_step_ms": t["train_step"]}
    ws.close()
    s.close()
    obj.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--trajectories", type=int, default=2000)
    ap.add_argument("--substeps", type=int, default=40)
    ap.add_argument("--target", type=float, default=1e-3)
    ap.add_argument("--max-sweeps", type=int, default=200)
    ap.add_argument("--chunk", type=int, default=5)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--side-lo", type=int, default=64)
    ap.add_argument("--side-hi", type=int, default=256)
    ap.add_argument("--eval-trajectories", type=int, default=20)
    ap.add_argument("--on-policy-trajectories", type=int, default=0,
                    help="then continue training on trajectories of the warm-started solver")
    ap.add_argument("--init", default=None, help="start from these weights (and scales)")
    ap.add_argument("--contact-trajectories", type=int, default=0,
                    help="train on contact states (folds on the ground, drapes over a sphere) "
                         "instead of hanging cloths")
    ap.add_argument("--contact-on-policy", type=int, default=0,
                    help="then contact trajectories that follow the warm-started solve")
    ap.add_argument("--families", default="fold,drape",
                    help="contact families to train on (fold, drape)")
    ap.add_argument("--contact-substeps", type=int, default=30)
    ap.add_argument("--contact-sweeps", type=int, default=60)
    ap.add_argument("--eval-only", default=None,
                    help="evaluate these weights on the contact workloads and exit")
    ap.add_argument("--apply-once", type=int, default=0, metavar="SIDE",
                    help="apply the network (weights from --init, else the contact-trained "
                         "ones) to a SIDE^2 hanging cloth with eager launches and exit")
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    a = ap.parse_args()
    t0 = time.time()
    if a.apply_once:
        params, scales, _ = load_params(a.init or CONTACT_WEIGHTS)
        print(json.dumps(apply_once(params, scales, a.apply_once)))
        return
    if a.contact_trajectories or a.contact_on_policy or a.eval_only:
        return main_contact(a, t0)
    params = None
    if a.init:
        params, scales, _ = load_params(a.init)
    else:
        scales = fit_scales(a.seed, 4, a.substeps, a.target, a.max_sweeps, a.chunk, a.side_lo,
                            a.side_hi)
    hist = []
    if a.trajectories:
        params, hist = train(a.trajectories, a.substeps, a.target, a.max_sweeps, a.chunk, a.lr,
                             a.seed, a.side_lo, a.side_hi, scales=scales, params=params)
    if a.on_policy_trajectories:
        params, h2 = train(a.on_policy_trajectories, a.substeps, a.target, a.max_sweeps, a.chunk,
                           a.lr, a.seed, a.side_lo, a.side_hi, scales=scales, params=params,
                           on_policy=True, traj_offset=400_000)
        hist += h2
    meta = {k: getattr(a, k) for k in ("trajectories", "on_policy_trajectories", "substeps",
                                       "target", "max_sweeps", "chunk", "lr", "seed", "side_lo",
                                       "side_hi", "init")}
    meta["train_seconds"] = time.time() - t0
    meta["final_loss"] = float(np.mean(hist[-50:])) if hist else None
    ev = evaluate(params, scales, a.eval_trajectories, a.substeps, a.target, a.max_sweeps,
                  a.chunk, side_lo=a.side_lo, side_hi=a.side_hi)
    meta["eval"] = ev
    meta["eval_same_state"] = evaluate_same_state(params, scales, 8, a.substeps, a.target,
                                                  a.max_sweeps, a.chunk, side_lo=a.side_lo,
                                                  side_hi=a.side_hi)
    meta["scales"] = [float(x) for x in scales]
    save(a.out, params, scales, meta)
    print(json.dumps(meta, indent=1))


def main_contact(a, t0):
    """training on the contact families, evaluation on the fold1024 and
    drape256 workloads (same-state, targets r_plain(K))"""
    if a.eval_only:
        params, scales, _ = load_params(a.eval_only)
        print(json.dumps(evaluate_workloads(params, scales, a.contact_sweeps), indent=1))
        return
    fams = tuple(f for f in a.families.split(",") if f)
    if a.init:
        params, scales, _ = load_params(a.init)
    else:
        scales = fit_contact_scales(a.seed, families=fams)
        params = init_params(a.seed)
    ws = WarmStart(params, scales)
    hist = []
    if a.contact_trajectories:
        hist += train_contact(ws, a.contact_trajectories, families=fams,
                              substeps=a.contact_substeps, sweeps=a.contact_sweeps, lr=a.lr,
                              seed=a.seed)
    if a.contact_on_policy:
        hist += train_contact(ws, a.contact_on_policy, families=fams, substeps=a.contact_substeps,
                              sweeps=a.contact_sweeps, lr=a.lr, seed=a.seed, on_policy=True,
                              traj_offset=420_000)
    params = ws.params()
    meta = {k: getattr(a, k) for k in ("contact_trajectories", "contact_on_policy",
                                       "contact_substeps", "contact_sweeps", "lr", "seed",
                                       "init")}
    meta["families"] = list(fams)
    meta["train_seconds"] = time.time() - t0
    meta["final_loss"] = float(np.mean(hist[-20:])) if hist else None
    meta["scales"] = [float(x) for x in scales]
    meta["eval_contact"] = evaluate_workloads(params, scales, a.contact_sweeps)
    save(a.out, params, scales, meta)
    print(json.dumps(meta, indent=1))


def workload_scene(name):
    """the benchmark's contact workloads: (scene, log2 buckets, pre-roll)"""
    if name == "fold1024":
        return scenes.folding_cloth(res=1024, seed=0), 24, 120
    if name == "drape256":
        return scenes.drape_over_sphere(res=256, seed=0, start="contact"), 20, 0
    if name == "batch512":
        # 512 cloths in one object, each hashed with its own cell and kept
        # off its own sphere (the batch the benchmark times)
        sc = scenes.batched_cloths(512, seed=0)
        sc["colli"] = {"cell": 2.0 * scenes.mean_rest_edge(sc), "thickness": 1e-3,
                       "spheres": sc["spheres"], "instance_cells": scenes.instance_cells(sc)}
        return sc, 24, 120
    raise ValueError(name)


def evaluate_workloads(params, scales, sweeps=60, substeps=16, names=("fold1024", "drape256")):
    out = {}
    for name in names:
        sc, log2, pre = workload_scene(name)
        r = evaluate_contact_same_state(params, scales, sc, log2, pre, substeps=substeps,
                                        sweeps=sweeps)
        r.pop("per_substep")
        out[name] = r
    return out


if __name__ == "__main__":
    main()
