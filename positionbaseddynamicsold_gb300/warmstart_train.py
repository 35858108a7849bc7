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
from .pbd import PBDObject, SolverPBD, WarmStart

DT = 1.0 / 600
PKG = os.path.dirname(os.path.abspath(__file__))
DEFAULT_WEIGHTS = os.path.join(PKG, "data", "warmstart.npz")

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


def save(path, params, scales, meta):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez(path, params=np.asarray(params, np.float32), scales=np.asarray(scales, np.float32),
             meta=json.dumps(meta))


def load_params(path=DEFAULT_WEIGHTS):
    """(params, scales, meta) of a trained network"""
    d = np.load(path)
    return (d["params"].astype(np.float32), d["scales"].astype(np.float32),
            json.loads(str(d["meta"])))


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
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    a = ap.parse_args()
    t0 = time.time()
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


if __name__ == "__main__":
    main()
