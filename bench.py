"""Throughput of the PBD cloth step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload drape256|fold1024|batch512|hanging32]
                    [--sub-workloads fold1024,batch512]

Headline workload (drape256): a 256x256 cloth (2 m x 2 m, 130,050 triangles,
195,585 distance + 194,565 bending constraints) over a fixed icosphere
(r = 0.4, 20,480 triangles); spatial hash with cell = 2 x mean rest edge and
2^20 buckets, vertex-face CCD with thickness 1e-3 (cloth-sphere and self
collision), FP32 positions, FP64 cubic; dt = 1/600 (10 substeps per 1/60
frame), 15 colored Gauss-Seidel iterations, CCD at iterations 0, 10 and 14.
One step = one substep: advect, 15 x (CCD when due, one sweep over all
colors, one response pass), integrate.  The cloth is released flat at
y = 0.5; its free fall (a rigid translation) is fast-forwarded to 1.5 mm
above the sphere's top, so contacts start at the first substep, and both
bench arms start from that state and run the same W warm-up and K timed
substeps.  L2 is flushed (a 256 MiB write) before every timed substep; each
substep is timed with CUDA events on the object's stream.

After the headline, the other workloads of --sub-workloads (default
fold1024: the 1024x1024 self-colliding fold, and batch512: 512 cloths in
one launch per color phase) are measured the same way, after their
120-substep pre-roll, and reported under "workloads".

Metric: cloth substeps/s.  `e2e` is the same step through the C ABI with
the state in page-locked host memory: upload positions and velocities, step,
read them back, every step, replaying the first min(K, 100) timed substeps
from the state they started from.  `cpu_baseline` times the reference's CPU
path (the oracle's restatement: sequential GS, triangle-ordered CCD with
de-duplication by scan, sequential response) from the timed start state:
whole substeps with the CCD detection on every host core for drape256,
bounded RefSampler steps on one thread for fold1024 and batch512.
`--impl reference` times the reference CPU path on the headline's start
state and substeps (whole substeps, every host core for the CCD detection),
with the GPU arm's response, and the reference's own response as a second
number.

Other modes: --solve residual runs every substep to a stretch-residual
target (--target, at most --max-sweeps sweeps in chunks of --chunk, the loop
on the device in a CUDA graph), --learned adds the trained warm start,
the autotuner picks the GS launch form after the pre-roll (--no-autotune
keeps the default form).  `learned_warm_start` in the line compares both
trained networks (contact states, pinned hanging cloths) with the plain
sweeps on fold1024, drape256 and batch512, solve by solve from identical
states, at the residual the plain solve reaches with 60 sweeps; each
workload's record is the network that measured faster there, with the
other's result beside it (see learned_eval).

Multi-GPU: a single cloth does not shard; N GPUs run N independent replicas
(value = replicas x substeps / slowest replica's time).  batch512 shards its
instances over the ranks, balanced by points, with no exchange on the data
path.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cloth substeps/s"
# DRAM bytes per launch of the dominant kernel (the per-color GS launch),
# dram__bytes_read.sum + dram__bytes_write.sum averaged over one ncu capture
# of 40-60 launches of the workload on the current kernel (the profile
# named beside each)
TRAFFIC_BYTES = {"drape256": 1355614.0, "fold1024": 21407981.0, "batch512": 64789632.0}
TRAFFIC_SOURCE = {w: "profiles/k_project_color_traffic.md" for w in TRAFFIC_BYTES}
G = np.array([0.0, -9.8, 0.0], np.float32)
DT = 1.0 / 600.0
ITERS = 15


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


RESPONSE_NOTE = ("mass-weighted: CollisionResolveNew's separation split by inverse mass with a "
                 "scale-free degeneracy guard (the reference's |n|^2 <= 1e-6 guard rejects every "
                 "triangle of this cloth and sphere, so its own response moves nothing here)")


def make_workload(name, rank=0, world=1):
    """(scene, config, collisions on, log2 hash buckets, pre-roll substeps).
    The config describes the workload only and is the same in both bench
    arms.  batch512 with world > 1: this rank's share of the instances
    (balanced by points, no exchange); every other workload is one object
    per rank (replicas)."""
    from positionbaseddynamicsold_gb300 import scenes
    from positionbaseddynamicsold_gb300.dist import shard_instances
    l2 = "flushed (256 MiB write) before every timed GPU substep"
    if name == "drape256":
        sc = scenes.drape_over_sphere(res=256, seed=0, start="contact")
        cfg = {"workload": "drape256: 256x256 cloth over a fixed icosphere (20,480 tris), "
                           "vertex-face CCD + self collision",
               "grid": 256, "substep_dt": DT, "gs_iterations": ITERS, "ccd_passes_per_substep": 3,
               "hash_buckets": 2 ** 20, "thickness": 1e-3, "cell": sc["colli"]["cell"],
               "start": "released flat at y = 0.5, free fall fast-forwarded to 1.5 mm above the "
                        "sphere's top (every point moving down at 1.389 m/s)",
               "preroll_substeps": 0, "response": RESPONSE_NOTE, "l2": l2}
        return sc, cfg, True, 20, 0
    if name == "fold1024":
        sc = scenes.folding_cloth(res=1024, seed=0)
        cfg = {"workload": "fold1024: 1024x1024 cloth dropped onto a ground plane, self CCD",
               "grid": 1024, "substep_dt": DT, "gs_iterations": ITERS,
               "ccd_passes_per_substep": 3, "hash_buckets": 2 ** 24, "thickness": 1e-3,
               "cell": sc["colli"]["cell"], "preroll_substeps": 120, "response": RESPONSE_NOTE,
               "l2": l2}
        return sc, cfg, True, 24, 120
    if name == "batch512":
        subset = None
        if world > 1:
            subset = shard_instances(scenes.batched_cloth_points(512, seed=0), world, rank)
        sc = scenes.batched_cloths(512, seed=0, subset=subset)
        sc["colli"] = {"cell": 2.0 * scenes.mean_rest_edge(sc), "thickness": 1e-3,
                       "spheres": sc["spheres"], "instance_cells": scenes.instance_cells(sc)}
        cfg = {"workload": "batch512: 512 cloths, side U{16..128}, random pins, one sphere each, "
                           "self CCD per instance (hash cell 2 x each cloth's mean rest edge), "
                           "all in one launch per color phase",
               "instances": 512, "instances_this_rank": 512 if subset is None else len(subset),
               "substep_dt": DT, "gs_iterations": ITERS,
               "ccd_passes_per_substep": 3, "hash_buckets": 2 ** 24, "thickness": 1e-3,
               "cell_per_instance": [float(sc["colli"]["instance_cells"].min()),
                                     float(sc["colli"]["instance_cells"].max())],
               "preroll_substeps": 120, "response": RESPONSE_NOTE, "l2": l2}
        return sc, cfg, True, 24, 120
    if name == "hanging32":
        sc = scenes.hanging_cloth(32, seed=0)
        cfg = {"workload": "hanging32: 32x32 hanging cloth, no collisions", "grid": 32,
               "substep_dt": DT, "gs_iterations": 20, "preroll_substeps": 0, "l2": l2}
        return sc, cfg, False, 0, 0
    raise SystemExit("unknown workload " + name)


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 6:
                self.samples.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if s[2 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def setup(sc, colli_on, table_log2, overlap=True):
    from positionbaseddynamicsold_gb300.pbd import (RESPONSE_MASS_WEIGHTED, CollisionSolver,
                                                    PBDObject, SolverPBD, SpatialHashSystem)
    obj = PBDObject(sc, damping=1.0, gravity=G)
    obj.prepare()
    solver = SolverPBD(obj)
    shs = cs = None
    if colli_on:
        shs = SpatialHashSystem(obj, cell_size=sc["colli"]["cell"], log2_table=table_log2)
        shs.init()
        cs = CollisionSolver(obj, shs, thickness=sc["colli"]["thickness"], iterations=1,
                             response=RESPONSE_MASS_WEIGHTED)
        n = obj.n_points
        cs.set_capacity(max(1 << 22, 64 * n), max(1 << 20, 4 * n))
        cs.set_overlap(overlap)
        if "ground" in sc["colli"]:
            solver.set_ground(True, sc["colli"]["ground"])
        if "spheres" in sc["colli"]:
            solver.set_instance_spheres(sc["colli"]["spheres"])
        if "instance_cells" in sc["colli"]:
            shs.set_instance_cells(sc["colli"]["instance_cells"])
    return obj, solver, shs, cs


def measure(name, args, rank, world, headline=True):
    """One workload on the GPU: pre-roll, autotune, W warm-up and K timed
    substeps (CUDA events on the object's stream, L2 flushed before each),
    the GS kernel's roofline, e2e through the C ABI and the CPU baseline.
    Returns the workload's record (the full contract line for the
    headline)."""
    import torch
    from positionbaseddynamicsold_gb300 import scenes
    from positionbaseddynamicsold_gb300.dist import max_over_ranks

    sc, cfg, colli_on, tl, preroll = make_workload(name, rank, world)
    if args.preroll is not None:
        preroll = args.preroll
        cfg["preroll_substeps"] = preroll
    # batch512 shards its instances over the ranks (the job's substeps are
    # done when the slowest rank is); the other workloads run replicas
    sharded = name == "batch512" and world > 1
    units = 1 if sharded else world
    obj, solver, shs, cs = setup(sc, colli_on, tl, overlap=not args.no_overlap)
    plan = {}
    if colli_on:
        plan["detection_overlaps_sweep"] = not args.no_overlap
    solver.set_gs_path({"auto": 0, "per-color": 1, "cluster": 2}[args.gs_path])
    if args.gs_block:
        solver.set_gs_block(args.gs_block)
    if args.gs_cluster:
        solver.set_gs_cluster(args.gs_cluster)
    if args.edge_edge:
        if cs is None:
            raise SystemExit("--edge-edge needs a workload with collisions")
        cs.set_edge_edge(True)
        cfg["edge_edge_ccd"] = True
    stream = torch.cuda.ExternalStream(obj.stream())
    nd = int((sc["ctype"] == scenes.DISTANCE).sum())
    nb = int((sc["ctype"] == scenes.BENDING).sum())
    n_colors = obj.eval_worksets()
    iters = cfg["gs_iterations"]
    plan.update({"colors": n_colors, "points": obj.n_points, "triangles": obj.n_tris,
            "distance_constraints": nd, "bending_constraints": nb})

    if args.solve == "residual":
        cfg["solve"] = {"target_stretch_residual": args.target, "max_sweeps": args.max_sweeps,
                        "chunk": args.chunk, "warm_start": bool(args.learned)}
        if args.learned:
            from positionbaseddynamicsold_gb300 import warmstart_train as wt
            from positionbaseddynamicsold_gb300.pbd import WarmStart
            params, scales, _ = wt.load_params(wt.DEFAULT_WEIGHTS if name == "hanging32"
                                               else wt.CONTACT_WEIGHTS)
            ws_net = WarmStart(params, scales)
            solver.set_warmstart(ws_net)

        def step():
            solver.step_to_residual(DT, 1, args.target, args.max_sweeps, args.chunk, cs, True)
    else:
        def step():
            solver.step(DT, 1, iters, cs, True)

    for _ in range(preroll):
        step()
    if not args.no_autotune and args.gs_path == "auto":
        # the GS launch form picked on the workload's own state; the choice
        # changes speed, never results (the autotuner puts the predicted
        # positions it sweeps back afterwards)
        plan["autotune"] = solver.autotune(iterations=iters, reps=3)
    for _ in range(args.warmup):
        step()
    obj.sync()
    if args.solve == "residual":
        solver.solve_stats(reset=True)
    # the state the timed substeps start from; the e2e loop replays the same
    # substeps from it
    state0 = obj.get_state()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    t_wall = time.perf_counter()
    if args.profile_range and headline:
        torch.cuda.profiler.start()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.fill_(k & 255)
            ev[k][0].record(stream)
            step()
            ev[k][1].record(stream)
    torch.cuda.synchronize()
    if args.profile_range and headline:
        torch.cuda.profiler.stop()
    t_wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in ev))
    value = units * args.steps / (ms / 1e3)
    stats = cs.stats() if cs is not None else {}
    residual = obj.residual()
    state_end = obj.get_state()
    if args.solve == "residual":
        sst = solver.solve_stats()
        cfg["solve"]["timed_substeps"] = sst
        outer, body = solver.residual_graph_kernels()
        # solve_stats was reset before the timed substeps
        chunks = sst["sweeps"] / max(1, sst["substeps"]) / args.chunk
        launches_total = int(round(args.steps * (outer + body * chunks)))
    else:
        launches_total = solver.graph_kernels() * args.steps

    # roofline of the dominant kernel (the GS sweep): eager projections on
    # the same state, timed with events on the object's stream, launched as
    # the timed substeps launch them (per-color: one launch per color phase;
    # resident form: one launch per sweep between collision passes, one for
    # all sweeps without collisions); algorithmic bytes per sweep =
    # 84*nd + 164*nb
    pos_save = obj.positions()
    prd_save = obj.predicted()
    bytes_sweep = 84.0 * nd + 164.0 * nb
    gs_form = solver.gs_path()
    gs_kernel = {1: "k_project_color", 2: "k_gs_resident"}[gs_form]
    per_sweep = gs_form == 2 and colli_on

    def sweeps():
        if per_sweep:
            for _ in range(iters):
                solver.project_constraint(1)
        else:
            solver.project_constraint(iters)

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sweeps()
    obj.sync()
    reps = 3
    with torch.cuda.stream(stream):
        e0.record(stream)
        for _ in range(reps):
            sweeps()
        e1.record(stream)
    torch.cuda.synchronize()
    gs_ms = e0.elapsed_time(e1)
    n_launch = reps * (iters * n_colors if gs_form == 1 else iters if per_sweep else 1)
    achieved = reps * iters * bytes_sweep / (gs_ms / 1e3) / 1e9
    obj.set_positions(pos_save)
    obj.set_predicted(prd_save)
    peak, peak_kind = load_peaks()

    # end to end through the C ABI with host buffers: the state lives in
    # page-locked host arrays, uploaded before and read back after every step
    n_pts = obj.n_points
    x_h = torch.empty((n_pts, 3), dtype=torch.float32, pin_memory=True).numpy()
    v_h = torch.empty((n_pts, 3), dtype=torch.float32, pin_memory=True).numpy()
    x_h[:], v_h[:] = state0
    e2e_steps = max(1, min(args.steps, 100))
    obj.sync()
    ph = [0.0, 0.0, 0.0]   # host clock: uploads, step (launch + wait), downloads
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ta = time.perf_counter()
        obj.set_state(x_h, v_h)
        tb = time.perf_counter()
        step()
        obj.sync()
        tc = time.perf_counter()
        obj.get_state(x_h, v_h)
        td = time.perf_counter()
        ph[0] += tb - ta
        ph[1] += tc - tb
        ph[2] += td - tc
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s)
    e2e = {"value": units * e2e_steps / e2e_s, "unit": "substeps/s",
           "h2d_bytes_per_step": 2 * 12 * obj.n_points, "d2h_bytes_per_step": 2 * 12 * obj.n_points,
           "phases_us": {"upload": 1e6 * ph[0] / e2e_steps, "step": 1e6 * ph[1] / e2e_steps,
                         "download": 1e6 * ph[2] / e2e_steps}}
    traffic = args.traffic if (args.traffic is not None and headline) else (
        TRAFFIC_BYTES.get(name) if gs_form == 1 else None)
    out = {
        "metric": METRIC, "value": value, "unit": "substeps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "strong" if sharded else "weak", "vs_baseline": None,
        "dtype": "f32+f64(ccd cubic)",
        "data": "synthetic (seeded scene generators)",
        "config": cfg,
        "parallelism": ("instances sharded over %d ranks" % world if sharded else
                        "replicas only" if world > 1 else "single GPU"),
        "plan": plan,
        "e2e": e2e,
        "gpu_launches": launches_total,
        "roofline": {"bound": "hbm", "kernel": gs_kernel, "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": traffic,
                     "traffic_source": TRAFFIC_SOURCE.get(name) if traffic is not None else None,
                     "launches_timed": n_launch, "avg_launch_us": gs_ms * 1e3 / n_launch,
                     "bytes_per_sweep": bytes_sweep,
                     "cluster_size": solver.gs_cluster() if gs_form == 2 else None},
        "clocks": clk,
        "wall_s_timed_region": t_wall,
        "last_step": {"candidates": stats.get("candidates"), "contacts": stats.get("contacts"),
                      "edge_edge": cs.ee_stats() if args.edge_edge else None,
                      "overflow": stats.get("overflow"), "relative_residual": residual},
    }
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(name, sc, cfg, colli_on, state0, args)
    del state_end
    for h in (cs, shs, solver, obj):
        if h is not None:
            h.close()
    del flush
    torch.cuda.empty_cache()
    return out


def run_ours(args, rank, world):
    import torch
    torch.cuda.set_device(0 if world == 1 else int(os.environ.get("LOCAL_RANK", rank)))
    out = measure(args.workload, args, rank, world, headline=True)
    subs = [w for w in args.sub_workloads.split(",") if w and w != args.workload]
    if subs:
        out["workloads"] = {}
        for w in subs:
            rec = measure(w, args, rank, world, headline=False)
            out["workloads"][w] = {k: rec[k] for k in
                                   ("value", "unit", "ms_per_step", "steps", "warmup", "config",
                                    "plan", "e2e", "gpu_launches", "roofline", "clocks",
                                    "last_step", "cpu_baseline") if k in rec}
    if rank == 0 and not args.no_learned_eval:
        out["learned_warm_start"] = learned_eval()
    return out


def learned_eval(substeps=12, sweeps=60):
    """The learned warm start against the plain sweeps on fold1024, drape256
    and batch512 (config 4 with and without the warm start).  Both trained
    networks are evaluated on every workload: the contact-state network
    (folds on the ground, drapes over a sphere) and the hanging-cloth network
    (square cloths with pinned corners).  Each workload's record is the
    network that measured faster there (contact states on fold1024, hanging
    cloths on drape256 and batch512), with the other's result beside it
    under `other_weights`.  From identical states along a plain trajectory
    after each workload's pre-roll, the plain solve runs `sweeps` sweeps
    (chunks of 10, a CCD detection per chunk, the response after every
    sweep) and its final stretch residual r_K is the target the
    warm-started solve must reach.  Both solves detect their first contacts
    from the same advected positions.  Device time of each solve from the
    CUDA graph of pbd_solver_step_to_residual; `residual_curve_first_state`
    is the plain residual after 0..200 sweeps of the first state (it levels
    off: the contact response and the pins keep a floor far above 1e-4)."""
    from positionbaseddynamicsold_gb300 import warmstart_train as wt
    out = {"target": "r_plain(%d sweeps)" % sweeps}
    nets = {}
    for path in (wt.CONTACT_WEIGHTS, wt.DEFAULT_WEIGHTS):
        try:
            params, scales, meta = wt.load_params(path)
        except FileNotFoundError:
            continue
        nets[path] = (params, scales, meta.get("families") or ["hanging"])
    pick = {"fold1024": wt.CONTACT_WEIGHTS, "drape256": wt.DEFAULT_WEIGHTS,
            "batch512": wt.DEFAULT_WEIGHTS}
    keep = ("weights", "trained_on", "speedup", "learned_ms", "learned_sweeps", "reverted",
            "learned_reached")
    for name, first in pick.items():
        res = {}
        for path, (params, scales, fam) in nets.items():
            r = wt.evaluate_workloads(params, scales, sweeps, substeps, names=(name,))[name]
            r["weights"] = os.path.relpath(path, ROOT)
            r["trained_on"] = fam
            res[path] = r
        if not res:
            out[name] = {"unavailable": "no trained weights"}
            continue
        main = res.get(first) or next(iter(res.values()))
        for path, r in res.items():
            if r is not main:
                main["other_weights"] = {k: r[k] for k in keep}
        out[name] = main
    return out


def cpu_colli(sc):
    return {"center": (0.0, 0.0, 0.0), "cell": sc["colli"]["cell"], "bounded": False,
            "thickness": sc["colli"]["thickness"], "tri_idx": sc["tri_idx"], "mass_weighted": 0,
            "resolve_passes": 1, "contact_cap": 1 << 21}


class RefSampler:
    """The reference's CPU path (the oracle's restatement of it) in bounded
    steps, each a fraction phi = 1 / (iterations * m) of a substep, in the
    reference's order:

    * GS: the next phi * iterations * n_prims prims of projectConstraintCPU's
      sequential loop (one full iteration per step when m = 1);
    * CCD: a slice of phi * 3 * n_tris consecutive triangles of
      CCD_SH_Extended's loop (three detection passes per substep), against
      the table UpdateSH built at the pass's first slice; a pass's slices
      are taken in a stride order that spreads a short run over the mesh;
    * response: the contacts that slice found, resolved five times (fifteen
      response passes per substep over one pass's contacts);
    * advection at the first step of a substep, integration at the last;
      with a sphere, ColliWithShpGrd after each full GS iteration.

    m keeps a step near 2,000 triangle queries so a step stays a bounded
    sample on every workload; the substep rate is phi * steps / time."""

    def __init__(self, sc, cfg, colli_on, pos, vel, sphere=None):
        import ctypes as C
        from oracle.oracle import Oracle, OrcContact, _ptr
        self.C, self.ptr = C, _ptr
        self.orc = Oracle()
        self.L = self.orc.lib
        self.L.orc_ccd_sh_extended_ref_range_tab.restype = C.c_int64
        self.L.orc_sh_build.restype = C.c_void_p
        self.L.orc_sh_build.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        self.L.orc_sh_free.argtypes = [C.c_void_p]
        self.table = None
        self.c = self.orc.constraints(sc)
        self.colli_on = colli_on
        self.pos = np.ascontiguousarray(pos, np.float32).copy()
        self.vel = np.ascontiguousarray(vel, np.float32).copy()
        self.prdp = self.pos.copy()
        self.n = len(self.pos)
        self.nt = len(sc["tri_idx"])
        self.n_prims = int(self.c.n_prims)
        self.iters = cfg["gs_iterations"]
        self.m = max(1, -(-3 * self.nt // (self.iters * 2000))) if colli_on else 1
        self.phi = 1.0 / (self.iters * self.m)
        self.gs_chunk = max(1, round(self.phi * self.iters * self.n_prims))
        self.ccd_chunk = max(1, round(self.phi * 3 * self.nt))
        # a pass's triangle slices, visited in a stride order coprime to
        # their count so that a short run samples the whole mesh
        self.n_slices = max(1, -(-self.nt // self.ccd_chunk))
        stride = max(1, int(self.n_slices * 0.618))
        while np.gcd(stride, self.n_slices) != 1:
            stride += 1
        self.slice_order = [(j * stride) % self.n_slices for j in range(self.n_slices)]
        self.gp = self.sk = 0
        self.colli = self.orc._colli(cpu_colli(sc)) if colli_on else None
        self.cap = 1 << 21
        self.arr = (OrcContact * self.cap)()
        self.tri = np.ascontiguousarray(sc["tri_idx"], np.int32)
        self.g = np.ascontiguousarray(G)
        self.mass = np.ascontiguousarray(sc["mass"])
        self.sphere = None if sphere is None else np.ascontiguousarray(sphere[:3], np.float32)
        self.radius = 0.0 if sphere is None else float(sphere[3])
        self.k = 0

    def step(self):
        C, P, L = self.C, self.ptr, self.L
        per = self.iters * self.m
        s = self.k % per
        if s == 0:
            L.orc_advect_cpu(self.n, C.c_float(DT), P(self.g), P(self.vel), P(self.prdp),
                             P(self.pos))
        left = self.gs_chunk
        while left:
            a = self.gp
            b = min(self.n_prims, a + left)
            L.orc_project_cpu_range(C.byref(self.c), P(self.mass), P(self.prdp), a, b)
            left -= b - a
            self.gp = b % self.n_prims
            if b == self.n_prims and self.sphere is not None:  # ColliWithShpGrd per iteration
                L.orc_colli_sphere(self.n, P(self.prdp), P(self.sphere), C.c_float(self.radius))
        if self.colli_on:
            t0 = self.slice_order[self.sk] * self.ccd_chunk
            t1 = min(self.nt, t0 + self.ccd_chunk)
            if self.sk == 0:  # a detection pass starts: UpdateSH bins every triangle once
                if self.table:
                    L.orc_sh_free(self.table)
                self.table = L.orc_sh_build(C.byref(self.colli.grid), self.nt, P(self.tri),
                                            P(self.prdp))
            h = L.orc_ccd_sh_extended_ref_range_tab(
                C.byref(self.colli.grid), C.c_void_p(self.table), self.nt, P(self.tri),
                P(self.pos), P(self.prdp), C.c_float(self.colli.thickness), t0, t1, self.arr,
                C.c_int64(self.cap))
            self.sk = (self.sk + 1) % self.n_slices
            L.orc_collision_resolve_ref(int(min(h, self.cap)), self.arr, P(self.pos),
                                        P(self.prdp), 5, C.c_float(self.colli.thickness))
        if s == per - 1:
            L.orc_integrate(self.n, C.c_float(DT), P(self.vel), P(self.prdp), P(self.pos))
        self.k += 1

    def sample(self):
        return ("each step = 1/%d substep: %d of %d prims of one sequential GS iteration%s; "
                "1 host thread" % (self.iters * self.m, self.gs_chunk, self.n_prims,
                                   ", %d of %d triangles of a CCD pass, its contacts resolved 5 "
                                   "times" % (self.ccd_chunk, self.nt) if self.colli_on else ""))


class BatchRefSampler:
    """batch512 on the reference, which has no batches: each cloth is its own
    simulation with its own spatial hash (cell 2 x its mean rest edge) and
    sphere, run one after another.  A sample of every `every`-th instance,
    each built exactly as in the batch, advances in RefSampler steps taken
    round-robin; the batch's substep time is the sampled instances' substep
    times summed and scaled by the points of all instances over theirs."""

    def __init__(self, cfg, n_inst=512, seed=0, every=32):
        from positionbaseddynamicsold_gb300 import scenes
        sizes = scenes.batched_cloth_points(n_inst, seed=seed)
        self.ids = list(range(0, n_inst, every))
        self.points = [sizes[i] for i in self.ids]
        self.total_points = int(sum(sizes))
        self.samplers = []
        for i in self.ids:
            sc = scenes.batched_cloths(n_inst, seed=seed, subset=[i])
            sc["colli"] = {"cell": 2.0 * scenes.mean_rest_edge(sc), "thickness": 1e-3}
            self.samplers.append(RefSampler(sc, cfg, True, sc["pos"], sc["vel"],
                                            sphere=sc["spheres"][0]))
        self.reset()

    def reset(self):
        self.t = [0.0] * len(self.samplers)
        self.n = [0] * len(self.samplers)
        self.k = 0

    def step(self):
        j = self.k % len(self.samplers)
        t0 = time.perf_counter()
        self.samplers[j].step()
        self.t[j] += time.perf_counter() - t0
        self.n[j] += 1
        self.k += 1

    def value(self):
        done = [j for j in range(len(self.samplers)) if self.n[j]]
        tsub = sum(self.t[j] / (self.n[j] * self.samplers[j].phi) for j in done)
        pts = sum(self.points[j] for j in done)
        return pts / (tsub * self.total_points)

    def sample(self):
        return ("instances %s of 512 (%d of %d points) simulated separately, round-robin "
                "RefSampler steps (1/15 to 1/%d substep each: a GS iteration share, a CCD "
                "pass share, its contacts resolved 5 times, the sphere per iteration), "
                "scaled to all instances by points; 1 host thread"
                % (",".join(map(str, self.ids)), sum(self.points), self.total_points,
                   max(s.iters * s.m for s in self.samplers)))


class RefSubsteps:
    """The reference's CPU path in whole substeps (advectCPU,
    projectConstraintWithColliCPU, integrationCPU: P/PBD_cuda.cu:997-1210,
    the oracle's restatement): per iteration [UpdateSH + CCD_SH_Extended at
    iterations 0, 10 and 14], one sequential GS pass over every prim in id
    order, one CollisionResolveNew pass over the stored contacts in order.
    CCD_SH_Extended's triangle loop runs on `threads` host threads over
    consecutive triangle slices whose hits are stored in loop order with the
    reference's duplicate scan, so the contact list, and with it the whole
    step, is the one-thread result; everything else is sequential as in the
    reference.  mass_weighted = 1 gives the response the GPU arm runs
    (inverse-mass split, scale-free guard); 0 the reference's own."""

    def __init__(self, sc, cfg, pos, vel, threads, mass_weighted=1):
        from oracle.oracle import Oracle
        self.orc = Oracle()
        self.threads = threads
        self.sc = sc
        self.iters = cfg["gs_iterations"]
        self.colli = None
        if "colli" in sc:
            self.colli = dict(cpu_colli(sc), mass_weighted=int(mass_weighted))
        self.state = {"pos": np.ascontiguousarray(pos, np.float32).copy(),
                      "vel": np.ascontiguousarray(vel, np.float32).copy()}
        self.contacts = 0

    def step(self):
        self.orc.set_threads(self.threads)
        self.contacts = self.orc.substep_cpu_ref(self.sc, self.state, self.iters, DT, G,
                                                 colli=self.colli)

    def sample(self, n):
        return ("%d whole substeps (advect, %d iterations of sequential GS + CCD at 0/10/14 + "
                "sequential response, integrate); CCD detection on %d host threads, "
                "everything else on one" % (n, self.iters, self.threads))


def cpu_baseline(name, sc, cfg, colli_on, state0, args, budget_s=10.0):
    """The reference CPU path (oracle restatement) from the timed start
    state.  drape256 / hanging32: whole substeps on every host core for
    about budget_s seconds (RefSubsteps).  fold1024 (a whole substep takes
    about half a minute there) and batch512 (512 separate simulations):
    RefSampler steps on one thread."""
    if name == "batch512":
        rs = BatchRefSampler(cfg)
        for _ in range(len(rs.samplers)):
            rs.step()  # warm-up
        rs.reset()
        t0 = time.perf_counter()
        while rs.k < 2 * len(rs.samplers) or time.perf_counter() - t0 < budget_s:
            rs.step()
        dt = time.perf_counter() - t0
        return {"value": rs.value(), "unit": "substeps/s", "cores": 1, "kind": "port",
                "sample": "%d steps in %.1f s; %s" % (rs.k, dt, rs.sample()),
                "host_cores_available": os.cpu_count()}
    if name == "fold1024":
        rs = RefSampler(sc, cfg, colli_on, state0[0], state0[1])
        rs.step()  # warm-up
        steps, t0 = 0, time.perf_counter()
        while steps < 3 or time.perf_counter() - t0 < budget_s:
            rs.step()
            steps += 1
        dt = time.perf_counter() - t0
        return {"value": steps * rs.phi / dt, "unit": "substeps/s", "cores": 1, "kind": "port",
                "sample": "%d steps in %.1f s; %s" % (steps, dt, rs.sample()),
                "host_cores_available": os.cpu_count()}
    threads = os.cpu_count() or 1
    rs = RefSubsteps(sc, cfg, state0[0], state0[1], threads)
    n, t0 = 0, time.perf_counter()
    while n < 2 or time.perf_counter() - t0 < budget_s:
        rs.step()
        n += 1
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "substeps/s", "cores": threads, "kind": "port",
            "sample": "from the timed start state: " + rs.sample(n),
            "host_cores_available": os.cpu_count()}


def run_reference(args):
    """The reference's CPU implementation of the path (the oracle's
    restatement of it: the reference sources are not present on the GPU
    host) on the GPU arm's workload, config and start state.  drape256 /
    hanging32: the same W warm-up and K timed whole substeps as the GPU arm
    (RefSubsteps, every host core), with the GPU arm's response; then
    min(K, 5) substeps from the same state with the reference's own response
    as a second number.  fold1024 / batch512: bounded RefSampler steps from
    the workload's start state."""
    sc, cfg, colli_on, tl, preroll = make_workload(args.workload)
    if args.workload in ("drape256", "hanging32"):
        threads = os.cpu_count() or 1
        rs = RefSubsteps(sc, cfg, sc["pos"], sc["vel"], threads)
        for _ in range(args.warmup):
            rs.step()
        start = (rs.state["pos"].copy(), rs.state["vel"].copy())
        t0 = time.perf_counter()
        for _ in range(args.steps):
            rs.step()
        dt = time.perf_counter() - t0
        value = args.steps / dt
        sample = ("the GPU arm's start state and substeps: %d warm-up + %s"
                  % (args.warmup, rs.sample(args.steps)))
        cores = threads
        extra = {"last_step": {"contacts": int(rs.contacts)}}
        if colli_on:
            n2 = max(1, min(args.steps, 5))
            r2 = RefSubsteps(sc, cfg, start[0], start[1], threads, mass_weighted=0)
            t1 = time.perf_counter()
            for _ in range(n2):
                r2.step()
            d2 = time.perf_counter() - t1
            extra["reference_response"] = {
                "value": n2 / d2, "unit": "substeps/s", "substeps": n2,
                "note": "the same start state with the reference's own response "
                        "(|n|^2 <= 1e-6 guard: no corrections on this cloth)",
                "last_step_contacts": int(r2.contacts)}
    else:
        extra = {}
        cores = 1
        if args.workload == "batch512":
            rs = BatchRefSampler(cfg)
            for _ in range(args.warmup):
                rs.step()
            rs.reset()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                rs.step()
            dt = time.perf_counter() - t0
            value = rs.value()
        else:
            rs = RefSampler(sc, cfg, colli_on, sc["pos"], sc["vel"])
            for _ in range(args.warmup):
                rs.step()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                rs.step()
            dt = time.perf_counter() - t0
            value = args.steps * rs.phi / dt
        sample = rs.sample()
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": "substeps/s",
           "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32+f64(ccd cubic)",
           "data": "synthetic (seeded scene generators)", "config": cfg,
           "cpu_baseline": {"value": value, "unit": "substeps/s", "cores": cores, "kind": "port",
                            "sample": sample, "host_cores_available": os.cpu_count()},
           "e2e": {"value": value, "unit": "substeps/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    out.update(extra)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="drape256", choices=["drape256", "fold1024", "batch512",
                                                          "hanging32"])
    ap.add_argument("--preroll", type=int, default=None,
                    help="untimed substeps before the warm-up (default: the workload's own)")
    ap.add_argument("--sub-workloads", default="fold1024,batch512",
                    help="comma-separated workloads measured after the headline one and "
                         "reported under 'workloads' (empty: none)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--gs-path", default="auto", choices=["auto", "per-color", "cluster"])
    ap.add_argument("--gs-cluster", type=int, default=0,
                    help="cluster size of the resident form (with --gs-path cluster)")
    ap.add_argument("--gs-block", type=int, default=0,
                    help="threads per block of the per-color launches (with --gs-path "
                         "per-color; profiles pin the autotuned form this way: under ncu "
                         "every launch is serialised and the autotuner's timings are not "
                         "representative)")
    ap.add_argument("--profile-range", action="store_true",
                    help="cudaProfilerStart/Stop around the timed substeps (for ncu "
                         "--profile-from-start off)")
    ap.add_argument("--traffic", type=float, default=None,
                    help="ncu dram bytes per launch of the dominant kernel (overrides the "
                         "measured default)")
    ap.add_argument("--solve", default="fixed", choices=["fixed", "residual"],
                    help="fixed: gs_iterations sweeps per substep (the reference's step); "
                         "residual: sweeps until the stretch residual <= --target")
    ap.add_argument("--target", type=float, default=1e-3)
    ap.add_argument("--max-sweeps", type=int, default=200)
    ap.add_argument("--chunk", type=int, default=10)
    ap.add_argument("--learned", action="store_true",
                    help="with --solve residual: warm start from the trained network")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default GS launch form (per-color, 256 threads) instead of "
                         "the autotuner's pick")
    ap.add_argument("--no-overlap", action="store_true",
                    help="run each CCD detection before its sweep on the object's stream "
                         "instead of beside it (same results)")
    ap.add_argument("--edge-edge", action="store_true",
                    help="also run edge-edge CCD (not in the reference's step; off by default)")
    ap.add_argument("--no-learned-eval", action="store_true",
                    help="skip the learned-vs-plain evaluation on the contact workloads")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)))
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    out = run_ours(args, rank, world)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
