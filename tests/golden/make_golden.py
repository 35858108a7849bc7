"""Regenerate the golden fixtures in this directory from the reference's own
compiled code (oracle/_ref/libpbdref.so, built from the reference sources by
oracle/build_oracle.py, which finds the reference checkout: PBD_REFERENCE_ROOT
first, then the checkout's mount point on the development machine).  Run it
on the development machine:

    python tests/golden/make_golden.py        # all fixtures
    python tests/golden/make_golden.py io     # the text-cache fixtures only

Every fixture is a small .npz of seeded synthetic inputs and the reference's
outputs for them.  tests/test_oracle_golden.py checks the oracle against them.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.oracle import Oracle, RefLib, _ptr  # noqa: E402
from positionbaseddynamicsold_gb300 import scenes  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def coloring(ref, orc):
    """Mixed distance+bending grid (the reference's CPU schedule deadlocks
    there: its resolve sweep stops at the first conflict and prim 0 loses to
    a 4-point neighbour every time), a distance-only grid, and the grid
    PBDObject::Init builds with its two anchors."""
    out = {}
    for name, sc in (("grid", scenes.grid_cloth(9, 7, 1.0, 1.0)),
                     ("dgrid", scenes.grid_cloth(9, 7, 1.0, 1.0, bending=False)),
                     ("refgrid", scenes.reference_grid(8, 8, 1.0, 1.0, anchors=True))):
        pl = np.ascontiguousarray(sc["prim_list"], np.int32)
        ix = np.ascontiguousarray(sc["indices"], np.int32)
        n = len(pl)
        sn = np.zeros((n, 2), np.int32)
        tot = ref.lib.ref_prim2prims(n, _ptr(pl), _ptr(ix), _ptr(sn), None)
        adj = np.zeros(tot, np.int32)
        ref.lib.ref_prim2prims(n, _ptr(pl), _ptr(ix), _ptr(sn), _ptr(adj))
        color = np.zeros(n, np.int32)
        ref.lib.ref_edge_coloring_cpu(n, _ptr(pl), _ptr(ix), 2000, _ptr(color))
        gcol, _ = orc.edge_coloring(pl, ix, int(ix.max()) + 1, "gpu")
        # one assign sweep from a partial coloring
        rng = np.random.default_rng(7)
        partial = np.where(rng.random(n) < 0.5, gcol, -1).astype(np.int32)
        prd = np.full(n, -1, np.int32)
        ref.lib.ref_assign_colors_cpu(n, _ptr(pl), _ptr(ix), _ptr(partial), _ptr(prd))
        # sort + worksets of the oracle's GPU-schedule coloring
        sc_col = gcol.copy()
        sid = np.arange(n, dtype=np.int32)
        ws = np.zeros((n, 2), np.int32)
        nw = ref.lib.ref_sort_worksets(n, _ptr(sc_col), _ptr(sid), _ptr(ws))
        out.update({name + "_prim_list": pl, name + "_indices": ix, name + "_adj_sn": sn,
                    name + "_adj": adj, name + "_color_cpu": color,
                    name + "_partial": partial, name + "_prd": prd,
                    name + "_gcolor": gcol, name + "_sorted_color": sc_col,
                    name + "_sorted_id": sid, name + "_worksets": ws[:nw]})
    np.savez_compressed(os.path.join(OUT, "coloring.npz"), **out)


def substep_cpu(ref):
    """projectConstraintCPU path incl. the unit-sphere push (pins, 2 constraints
    per pinned point only where the partner is free)."""
    sc = scenes.grid_cloth(10, 10, 1.2, 1.2, origin=(-0.6, 0.95, -0.6), jitter=1e-3, seed=3,
                           pins=[0, 9], bending=False)
    pos = sc["pos"].copy()
    vel = np.zeros_like(pos)
    g = np.array([0, -9.8, 0], np.float32)
    ref.lib.ref_substeps_cpu(len(pos), _ptr(pos), _ptr(vel), _ptr(sc["mass"]), len(sc["ctype"]),
                             _ptr(sc["prim_list"]), _ptr(sc["indices"]), _ptr(sc["rest_length"]),
                             _ptr(sc["stiffness"]), _ptr(sc["ctype"]), C.c_float(0.9),
                             _ptr(g), C.c_float(1.0 / 60), 5, 3)
    np.savez_compressed(os.path.join(OUT, "substep_cpu.npz"), pos0=sc["pos"], mass=sc["mass"],
                        prim_list=sc["prim_list"], indices=sc["indices"], ctype=sc["ctype"],
                        rest_length=sc["rest_length"], stiffness=sc["stiffness"],
                        pos=pos, vel=vel)


def substep_gpu_pin(ref, orc):
    """The colored-GS semantics pinned through the reference's sequential GS:
    with every stiffness 1, unit masses, no damping and the sphere out of
    reach, projectConstraintCPU over the constraints permuted into
    color-sorted order is the colored GS up to float rounding of the
    normalisation."""
    sc = scenes.grid_cloth(12, 12, 1.0, 1.0, origin=(0.0, 5.0, 0.0), jitter=1e-3, seed=5,
                           bending=False)
    # stretch so the constraints act
    pos = sc["pos"].copy()
    pos[:, 0] *= 1.05
    n = len(sc["ctype"])
    color, _ = orc.edge_coloring(sc["prim_list"], sc["indices"], len(pos), "gpu")
    _, sid, ws = orc.sort_worksets(color)
    pl = np.stack([np.arange(n) * 2, np.full(n, 2)], 1).astype(np.int32)
    ix = sc["indices"].reshape(-1, 2)[sid].ravel().astype(np.int32)
    rl = sc["rest_length"][sid].copy()
    st = sc["stiffness"][sid].copy()
    ct = sc["ctype"][sid].copy()
    p = pos.copy()
    vel = np.zeros_like(p)
    g = np.array([0, -9.8, 0], np.float32)
    ref.lib.ref_substeps_cpu(len(p), _ptr(p), _ptr(vel), _ptr(sc["mass"]), n, _ptr(pl), _ptr(ix),
                             _ptr(rl), _ptr(st), _ptr(ct), C.c_float(1.0), _ptr(g),
                             C.c_float(1.0 / 600), 10, 1)
    np.savez_compressed(os.path.join(OUT, "substep_gpu_pin.npz"), pos0=pos, mass=sc["mass"],
                        prim_list=sc["prim_list"], indices=sc["indices"], ctype=sc["ctype"],
                        rest_length=sc["rest_length"], stiffness=sc["stiffness"],
                        color=color, pos=p, vel=vel)


def crumpled(res, seed, amp):
    sc = scenes.grid_cloth(res, res, 1.0, 1.0, origin=(-0.5, 0.0, -0.5), bending=False)
    rng = np.random.default_rng(seed)
    p = sc["pos"] + rng.uniform(-amp, amp, sc["pos"].shape).astype(np.float32)
    return sc, p.astype(np.float32)


def neighbors(ref):
    sc, p = crumpled(12, 11, 0.04)
    center = np.array([0.0, 0.0, 0.0], np.float32)
    size = np.array([12, 6, 12], np.int32)
    cell = np.array([0.1, 0.1, 0.1], np.float32)
    tri = sc["tri_idx"]
    sn = np.zeros((len(tri), 2), np.int32)
    tot = ref.lib.ref_find_neighbors_all(_ptr(center), _ptr(size), _ptr(cell), len(tri), _ptr(tri),
                                         len(p), _ptr(p), _ptr(sn), None)
    out = np.zeros(tot, np.int32)
    ref.lib.ref_find_neighbors_all(_ptr(center), _ptr(size), _ptr(cell), len(tri), _ptr(tri),
                                   len(p), _ptr(p), _ptr(sn), _ptr(out))
    np.savez_compressed(os.path.join(OUT, "neighbors.npz"), pos=p, tri_idx=tri, center=center,
                        size=size, cell=cell, start_num=sn, nbrs=out)


def two_sheets(seed=13):
    """Sheet A static at y=0; sheet B (offset in x,z) moving from y=+0.02 to
    y=-0.015, so B's points sweep through A's faces and A's points are
    swept by B's faces."""
    a = scenes.grid_cloth(10, 10, 1.0, 1.0, origin=(-0.5, 0.0, -0.5), bending=False)
    b = scenes.grid_cloth(10, 10, 1.0, 1.0, origin=(-0.47, 0.02, -0.46), bending=False)
    rng = np.random.default_rng(seed)
    pos = np.concatenate([a["pos"], b["pos"]]).astype(np.float32)
    tri = np.concatenate([a["tri_idx"], b["tri_idx"] + len(a["pos"])]).astype(np.int32)
    prd = pos.copy()
    nb = len(b["pos"])
    prd[len(a["pos"]):, 1] = -0.015 + rng.uniform(-0.003, 0.003, nb).astype(np.float32)
    prd[len(a["pos"]):, 0] += rng.uniform(-0.004, 0.004, nb).astype(np.float32)
    prd[:len(a["pos"]), 1] += rng.uniform(-0.002, 0.002, len(a["pos"])).astype(np.float32)
    return pos, prd, tri


def ccd(ref):
    pos, prd, tri = two_sheets()
    center = np.array([0.0, 0.0, 0.0], np.float32)
    size = np.array([12, 4, 12], np.int32)
    cell = np.array([0.1, 0.1, 0.1], np.float32)
    thickness = 0.004
    cap = 200000
    ids = np.zeros((cap, 4), np.int32)
    t = np.zeros(cap, np.float32)
    w = np.zeros((cap, 4), np.float64)
    nn = np.zeros((cap, 3), np.float32)
    h = ref.lib.ref_ccd_sh_extended(_ptr(center), _ptr(size), _ptr(cell), len(tri), _ptr(tri),
                                    len(pos), _ptr(pos), _ptr(prd), C.c_float(thickness),
                                    C.c_longlong(cap), _ptr(ids), _ptr(t), _ptr(w), _ptr(nn))
    ids, t, w, nn = ids[:h], t[:h], w[:h], nn[:h]
    resolved = prd.copy()
    ref.lib.ref_collision_resolve_new(len(pos), _ptr(pos), _ptr(resolved), int(h), _ptr(ids), 2,
                                      C.c_float(thickness))
    np.savez_compressed(os.path.join(OUT, "ccd.npz"), pos=pos, prdp=prd, tri_idx=tri,
                        center=center, size=size, cell=cell, thickness=np.float32(thickness),
                        ids=ids, t=t, w=w, n=nn, resolved=resolved)


def gpu_kernel_schedule(ref, orc):
    """ProjectContraintsGPUKernel (P/PBD_cuda.cu:1240-1306), compiled for the
    host from the reference's own file, run colour by colour for 8
    iterations on a jittered grid with distance stiffness below 1 (mixed
    0.15 / 0.5 / 0.85), so the factor k = 1 - (1 - s)^(1/(iter+1)) is
    exercised at every iteration count; pins and unequal masses included."""
    sc = scenes.grid_cloth(11, 9, 1.0, 0.8, jitter=2e-2, seed=5, bending=False, pins=[0, 10])
    rng = np.random.default_rng(5)
    n = len(sc["pos"])
    sc["stiffness"] = rng.choice(np.array([0.15, 0.5, 0.85], np.float32),
                                 len(sc["stiffness"])).astype(np.float32)
    mass = np.where(sc["mass"] > 0, rng.uniform(0.5, 2.0, n), 0.0).astype(np.float32)
    color, _ = orc.edge_coloring(sc["prim_list"], sc["indices"], n)
    _, sid, ws = orc.sort_worksets(color)
    prd = (sc["pos"] + rng.normal(0, 0.03, sc["pos"].shape)).astype(np.float32)
    out = prd.copy()
    rest = np.zeros((2, 3), np.float32)
    keep = [np.ascontiguousarray(a) for a in (sid, sc["indices"], sc["ctype"], mass,
                                              sc["rest_length"], sc["stiffness"],
                                              sc["prim_list"])]
    ref.lib.ref_project_colored_gpu_kernel(11, len(ws), _ptr(np.ascontiguousarray(ws)), 0, 8,
                                           *[_ptr(a) for a in keep], _ptr(out), _ptr(rest))
    np.savez_compressed(os.path.join(OUT, "gpu_kernel_schedule.npz"), prim_list=sc["prim_list"],
                        indices=sc["indices"], ctype=sc["ctype"], rest_length=sc["rest_length"],
                        stiffness=sc["stiffness"], mass=mass, sorted_prim_id=sid, worksets=ws,
                        prdp=prd, out=out)


def resolve_old(ref):
    """The older response CollisionResolve (three calls in a row on the ccd
    fixture's contacts, positions and resolve counters carried over), with
    a second contact set of sheets pushed further through each other."""
    g = dict(np.load(os.path.join(OUT, "ccd.npz")))
    out = {}
    for case, push in (("a", 0.0), ("b", 0.012)):
        prd = g["prdp"].copy()
        prd[prd[:, 1] > np.median(prd[:, 1]), 1] -= np.float32(push)
        ids = g["ids"] if push == 0.0 else None
        if ids is None:
            cap = 200000
            ids = np.zeros((cap, 4), np.int32)
            t = np.zeros(cap, np.float32)
            w = np.zeros((cap, 4), np.float64)
            nn = np.zeros((cap, 3), np.float32)
            h = ref.lib.ref_ccd_sh_extended(_ptr(g["center"]), _ptr(g["size"]), _ptr(g["cell"]),
                                            len(g["tri_idx"]), _ptr(g["tri_idx"]), len(g["pos"]),
                                            _ptr(g["pos"]), _ptr(prd), C.c_float(g["thickness"]),
                                            C.c_longlong(cap), _ptr(ids), _ptr(t), _ptr(w),
                                            _ptr(nn))
            ids = ids[:h].copy()
        rt = np.zeros(len(g["pos"]), np.int32)
        out[case + "_prdp0"] = prd.copy()
        out[case + "_ids"] = ids
        for k in range(3):
            ref.lib.ref_collision_resolve_old(len(g["pos"]), _ptr(g["pos"]), _ptr(prd), len(ids),
                                              _ptr(np.ascontiguousarray(ids)),
                                              C.c_float(g["thickness"]), _ptr(rt))
            out["%s_prdp%d" % (case, k + 1)] = prd.copy()
            out["%s_rt%d" % (case, k + 1)] = rt.copy()
    np.savez_compressed(os.path.join(OUT, "resolve_old.npz"), **out)


def vf_cases(ref, n=1500, seed=17):
    """Random vertex/face motions close to contact, plus cubic roots."""
    rng = np.random.default_rng(seed)
    X = np.zeros((n, 4, 3), np.float32)
    P = np.zeros((n, 4, 3), np.float32)
    th = np.zeros(n, np.float32)
    for k in range(n):
        s = 10 ** rng.uniform(-2, 0)
        tri = rng.normal(size=(3, 3)) * s
        nrm = np.cross(tri[1] - tri[0], tri[2] - tri[0])
        nrm /= np.linalg.norm(nrm) + 1e-30
        wts = rng.dirichlet([1, 1, 1]) * 1.2 - 0.066
        v0 = wts @ tri + nrm * rng.uniform(-0.05, 0.05) * s
        vel = -nrm * rng.uniform(-0.1, 0.1) * s + rng.normal(size=3) * 0.01 * s
        fvel = rng.normal(size=(3, 3)) * 0.01 * s * rng.integers(0, 2)
        X[k, 0] = v0
        X[k, 1:] = tri
        P[k, 0] = v0 + vel
        P[k, 1:] = tri + fvel
        th[k] = s * 10 ** rng.uniform(-3, -1)
    hit = np.zeros(n, np.int32)
    tt = np.zeros(n, np.float32)
    ww = np.zeros((n, 4), np.float64)
    nn = np.zeros((n, 3), np.float32)
    nhit = np.zeros(n, np.int32)
    ntt = np.zeros(n, np.float32)
    rtest = np.zeros(n, np.int32)
    rnew = np.zeros((n, 4, 3), np.float32)
    for k in range(n):
        x = np.ascontiguousarray(X[k].ravel())
        p = np.ascontiguousarray(P[k].ravel())
        t = C.c_float()
        w = np.zeros(4, np.float64)
        nv = np.zeros(3, np.float32)
        hit[k] = ref.lib.ref_extended_vf_test(_ptr(x), _ptr(p), C.c_float(th[k]), 0, 1, 2, 3,
                                              C.byref(t), _ptr(w), _ptr(nv))
        tt[k] = t.value
        ww[k] = w
        nn[k] = nv
        nhit[k] = ref.lib.ref_narrow_vf_ccd_test(_ptr(x), _ptr(p), C.c_float(th[k]), 0, 1, 2, 3,
                                                 C.byref(t), _ptr(w), _ptr(nv))
        ntt[k] = t.value
        rtest[k] = ref.lib.ref_vf_resolve_test(_ptr(x), _ptr(p), C.c_float(th[k]))
        q = p.copy()
        ref.lib.ref_vf_resolve_new(_ptr(x), _ptr(q), C.c_float(th[k]))
        rnew[k] = q.reshape(4, 3)
    # VFCCDTest (type VF), VFDCDTest and VFTest on the same cases
    extra = {}
    for key, fn in (("vfccd", ref.lib.ref_vf_ccd_test), ("vfdcd", ref.lib.ref_vf_dcd_test),
                    ("vf", ref.lib.ref_vf_test)):
        eh = np.zeros(n, np.int32)
        et = np.zeros(n, np.float32)
        ew = np.zeros((n, 4), np.float64)
        en = np.zeros((n, 3), np.float32)
        for k in range(n):
            x = np.ascontiguousarray(X[k].ravel())
            p = np.ascontiguousarray(P[k].ravel())
            t = C.c_float()
            w = np.zeros(4, np.float64)
            nv = np.zeros(3, np.float32)
            eh[k] = fn(_ptr(x), _ptr(p), C.c_float(th[k]), 0, 1, 2, 3, C.byref(t), _ptr(w),
                       _ptr(nv))
            et[k] = t.value
            ew[k] = w
            en[k] = nv
        extra.update({key + "_hit": eh, key + "_t": et, key + "_w": ew, key + "_n": en})
    coef = rng.normal(size=(500, 4))
    coef[:50, 0] = 0.0  # quadratic cases
    coef = np.concatenate([coef, [[1.0, -6.0, 11.0, -6.0]]])
    roots = np.full((len(coef), 3), np.nan)
    nroot = np.zeros(len(coef), np.int32)
    for k, (a, b, c, d) in enumerate(coef):
        x = np.zeros(3, np.float64)
        m = ref.lib.ref_solve_cubic(a, b, c, d, x)
        nroot[k] = m
        roots[k, :m] = x[:m]
    np.savez_compressed(os.path.join(OUT, "vf_cases.npz"), X=X, P=P, thickness=th, hit=hit, t=tt,
                        w=ww, n=nn, narrow_hit=nhit, narrow_t=ntt, resolve_test=rtest,
                        resolve_new=rnew, coef=coef, roots=roots, nroot=nroot, **extra)


def _ref_read(ref, fn, args, cap=1 << 16):
    """run a reference reader; its 14 output arrays trimmed to their sizes"""
    kinds = ["f", "i", "i", "f", "f", "i", "f", "i", "f", "f", "f", "i", "f", "f"]
    outs = [np.zeros(cap, np.float32 if k == "f" else np.int32) for k in kinds]
    ptrs = (C.c_void_p * 14)(*[o.ctypes.data for o in outs])
    sizes = np.zeros(14, np.int64)
    r = fn(*args, ptrs, C.c_longlong(cap), _ptr(sizes))
    assert r == 0
    names = ["mesh_pos", "mesh_indices", "mesh_prims", "vel", "mass", "c_indices", "c_pos",
             "c_prims", "prdp", "rest", "stiff", "ctype", "damping", "gravity"]
    res = {}
    for k, nm in enumerate(names):
        m = 1 if nm == "damping" else 3 if nm == "gravity" else int(sizes[k])
        res[nm] = outs[k][:m].copy()
    return res


def io_files(ref):
    """The reference's text caches (PBDObject::SaveMeshTopol / SaveConstraint
    of a small pinned, jittered grid with bending prims, random velocities,
    masses and predicted positions) and what its readers
    (PBDObject::ContinueSimInit) read back; text scene files in the format
    IO::ReadTopolFromTxt / ReadDistConstrFromTxt read, and what they read."""
    d = os.path.join(OUT, "io")
    os.makedirs(d, exist_ok=True)
    rng = np.random.default_rng(21)
    sc = scenes.grid_cloth(6, 5, 0.5, 0.4, jitter=1e-3, seed=4, pins=[0, 5])
    n = len(sc["pos"])
    pos = np.ascontiguousarray(sc["pos"], np.float32)
    vel = rng.normal(0, 0.3, (n, 3)).astype(np.float32)
    mass = rng.uniform(0.5, 2.0, n).astype(np.float32)
    mass[[0, 5]] = 0.0
    prdp = (pos + rng.normal(0, 1e-3, (n, 3))).astype(np.float32)
    tri = np.ascontiguousarray(sc["tri_idx"], np.int32)
    g = np.array([0.25, -9.8, -0.125], np.float32)
    pl = np.ascontiguousarray(sc["prim_list"], np.int32)
    ix = np.ascontiguousarray(sc["indices"], np.int32)
    ct = np.ascontiguousarray(sc["ctype"], np.int32)
    rl = np.ascontiguousarray(sc["rest_length"], np.float32)
    st = np.ascontiguousarray(sc["stiffness"], np.float32)
    tpath, cpath = os.path.join(d, "topol.cache"), os.path.join(d, "constr.cache")
    L = ref.lib
    L.ref_save_caches(tpath.encode(), cpath.encode(), n, _ptr(pos), _ptr(vel), _ptr(mass),
                      len(tri), _ptr(tri), C.c_float(0.9), _ptr(g), len(pl), _ptr(pl), _ptr(ix),
                      _ptr(ct), _ptr(rl), _ptr(st), _ptr(prdp))
    got = _ref_read(ref, L.ref_read_caches, (tpath.encode(), cpath.encode()))
    # text scene files: positions with six decimals, one line of triangles,
    # one header line then one line of distance pairs
    pairs = ix[: 2 * int((ct == scenes.DISTANCE).sum())]
    with open(os.path.join(d, "topol.txt"), "w") as f:
        f.write("P:" + ",".join("%.6f" % v for v in pos.ravel()) + "\n")
        f.write("Tri:" + ",".join(str(v) for v in tri.ravel()) + "\n")
    with open(os.path.join(d, "dist.txt"), "w") as f:
        f.write("NumConstr:%d\n" % (len(pairs) // 2))
        f.write("Dist:" + ",".join(str(v) for v in pairs) + "\n")
    txt = _ref_read(ref, L.ref_read_txt, (os.path.join(d, "topol.txt").encode(),
                                          os.path.join(d, "dist.txt").encode(), C.c_float(0.75)))
    out = {"in_pos": pos, "in_vel": vel, "in_mass": mass, "in_prdp": prdp, "in_tri": tri,
           "in_gravity": g, "in_prim_list": pl, "in_indices": ix, "in_ctype": ct,
           "in_rest": rl, "in_stiff": st}
    out.update({"cache_" + k: v for k, v in got.items()})
    out.update({"txt_" + k: v for k, v in txt.items()})
    np.savez_compressed(os.path.join(OUT, "io.npz"), **out)


def main():
    ref = RefLib()
    if sys.argv[1:] == ["io"]:
        io_files(ref)
        return
    orc = Oracle()
    coloring(ref, orc)
    substep_cpu(ref)
    substep_gpu_pin(ref, orc)
    neighbors(ref)
    ccd(ref)
    resolve_old(ref)
    gpu_kernel_schedule(ref, orc)
    vf_cases(ref)
    io_files(ref)
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)))


if __name__ == "__main__":
    main()
