"""ctypes front end of the oracle libraries (test infrastructure only).

``Oracle`` wraps ``oracle/_build/liboracle.so`` (the C restatement of the
reference, see pbd_oracle.h); ``RefLib`` wraps ``oracle/_ref/libpbdref.so``
(the reference's own code, available only where its sources were present at
build time).  Only tests/, __graft_entry__.smoke() and bench.py's
cpu_baseline leg import this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle as _b

DISTANCE, BENDING, ANCHOR = 0x001, 0x010, 0x100

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


class OrcConstraints(C.Structure):
    _fields_ = [("n_prims", C.c_int), ("prim_list", C.c_void_p), ("indices", C.c_void_p),
                ("ctype", C.c_void_p), ("rest_length", C.c_void_p), ("stiffness", C.c_void_p),
                ("rest_angle", C.c_void_p), ("rest_pos", C.c_void_p)]


class OrcGrid(C.Structure):
    _fields_ = [("start", C.c_float * 3), ("cell", C.c_float * 3), ("size", C.c_int * 3),
                ("bounded", C.c_int)]


class OrcContact(C.Structure):
    _fields_ = [("v", C.c_int), ("f0", C.c_int), ("f1", C.c_int), ("f2", C.c_int),
                ("face", C.c_int), ("t", C.c_float), ("w", C.c_double * 4), ("n", C.c_float * 3)]


class OrcEEHit(C.Structure):
    _fields_ = [("t", C.c_float), ("s", C.c_float), ("u", C.c_float), ("m0", C.c_float * 4)]


class OrcColliParams(C.Structure):
    _fields_ = [("enabled", C.c_int), ("grid", OrcGrid), ("thickness", C.c_float),
                ("resolve_passes", C.c_int), ("mass_weighted", C.c_int), ("ccd_every", C.c_int),
                ("n_tris", C.c_int), ("tri_idx", C.c_void_p), ("tri_inst", C.c_void_p),
                ("point_inst", C.c_void_p), ("contact_cap", C.c_int64)]


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def contacts_to_numpy(arr, n):
    """Structured arrays of a ctypes OrcContact array."""
    n = int(n)
    ids = np.array([[arr[i].v, arr[i].f0, arr[i].f1, arr[i].f2] for i in range(n)],
                   dtype=np.int32).reshape(n, 4)
    face = np.array([arr[i].face for i in range(n)], dtype=np.int32)
    t = np.array([arr[i].t for i in range(n)], dtype=np.float32)
    w = np.array([list(arr[i].w) for i in range(n)], dtype=np.float64).reshape(n, 4)
    nn = np.array([list(arr[i].n) for i in range(n)], dtype=np.float32).reshape(n, 3)
    return {"ids": ids, "face": face, "t": t, "w": w, "n": nn}


class Oracle:
    """The C restatement; every method mirrors one pbd_oracle.h entry."""

    def __init__(self, path: str | None = None):
        self.lib = C.CDLL(path or _b.build_oracle())
        L = self.lib
        L.orc_prim2prims.restype = C.c_int64
        L.orc_edge_coloring_gpu.restype = C.c_int
        L.orc_edge_coloring_cpu.restype = C.c_int
        L.orc_eval_worksets.restype = C.c_int
        L.orc_residual.restype = C.c_double
        L.orc_ccd_ee_brute.restype = C.c_int64
        L.orc_solve_cubic.restype = C.c_int
        L.orc_solve_cubic.argtypes = [C.c_double] * 4 + [_f64p]
        L.orc_extended_vf_test.restype = C.c_int
        L.orc_narrow_vf_ccd_test.restype = C.c_int
        L.orc_find_neighbors_all.restype = C.c_int64
        L.orc_ccd_sh_extended_ref.restype = C.c_int64
        L.orc_get_threads.restype = C.c_int
        L.orc_ccd_vf_pairs.restype = C.c_int64
        L.orc_vf_resolve_test.restype = C.c_int
        L.orc_vf_resolve_deltas.restype = C.c_int
        L.orc_substep_gpu.restype = C.c_int64
        L.orc_substep_gpu_obst.restype = C.c_int64
        L.orc_substep_cpu_ref.restype = C.c_int64
        L.orc_dihedral_angle.restype = C.c_double
        L.orc_bending_project_f64.restype = C.c_int
        L.orc_bending_project_f32.restype = C.c_int

    def set_threads(self, n=None):
        """host threads for the oracle's independent loops (process-wide;
        None: every core); results do not depend on the count"""
        self.lib.orc_set_threads(int(n if n is not None else (os.cpu_count() or 1)))
        return self.lib.orc_get_threads()

    # -- constraints -----------------------------------------------------
    @staticmethod
    def constraints(scene):
        keep = [np.ascontiguousarray(scene[k]) for k in
                ("prim_list", "indices", "ctype", "rest_length", "stiffness")]
        ra = scene.get("rest_angle")
        rp = scene.get("rest_pos")
        ra = None if ra is None else np.ascontiguousarray(ra, dtype=np.float32)
        rp = None if rp is None else np.ascontiguousarray(rp, dtype=np.float32)
        c = OrcConstraints(len(scene["ctype"]), *[_ptr(a) for a in keep], _ptr(ra), _ptr(rp))
        c._keep = (keep, ra, rp)
        return c

    def prim2prims(self, prim_list, indices, n_points):
        n = len(prim_list)
        pl = np.ascontiguousarray(prim_list, dtype=np.int32)
        ix = np.ascontiguousarray(indices, dtype=np.int32)
        sn = np.zeros((n, 2), np.int32)
        tot = self.lib.orc_prim2prims(n, _ptr(pl), _ptr(ix), n_points, _ptr(sn), None)
        adj = np.zeros(max(tot, 1), np.int32)
        self.lib.orc_prim2prims(n, _ptr(pl), _ptr(ix), n_points, _ptr(sn), _ptr(adj))
        return sn, adj[:tot]

    def edge_coloring(self, prim_list, indices, n_points, schedule="gpu", max_iters=1 << 30):
        sn, adj = self.prim2prims(prim_list, indices, n_points)
        n = len(prim_list)
        color = np.full(n, -1, np.int32)
        prd = np.full(n, -1, np.int32)
        pl = np.ascontiguousarray(prim_list, dtype=np.int32)
        fn = self.lib.orc_edge_coloring_gpu if schedule == "gpu" else self.lib.orc_edge_coloring_cpu
        sweeps = fn(n, _ptr(pl), _ptr(sn), _ptr(adj), _ptr(color), _ptr(prd), max_iters)
        return color, sweeps

    def sort_worksets(self, color):
        n = len(color)
        c = np.ascontiguousarray(color, dtype=np.int32).copy()
        sid = np.arange(n, dtype=np.int32)
        self.lib.orc_sort_edges_colors(n, _ptr(c), _ptr(sid))
        ws = np.zeros((max(n, 1), 2), np.int32)
        nw = self.lib.orc_eval_worksets(n, _ptr(c), _ptr(ws))
        return c, sid, ws[:nw].copy()

    # -- solver ----------------------------------------------------------
    def set_stiffness_schedule(self, mode):
        """0: k = 1-(1-s)^(1/(iter+1)); 1: k = 1; 2: k = s (process-wide)"""
        self.lib.orc_set_stiffness_schedule(int(mode))

    def project_colored(self, scene, prdp, mass, sorted_prim_id, worksets, it0, it1):
        """the colored sweeps it0..it1-1 alone (orc_project_colored); returns
        the new predicted positions"""
        c = self.constraints(scene)
        p = np.ascontiguousarray(prdp, dtype=np.float32).copy()
        sid = np.ascontiguousarray(sorted_prim_id, dtype=np.int32)
        ws = np.ascontiguousarray(worksets, dtype=np.int32)
        m = np.ascontiguousarray(mass, dtype=np.float32)
        self.lib.orc_project_colored(C.byref(c), _ptr(sid), len(ws), _ptr(ws), int(it0), int(it1),
                                     _ptr(m), _ptr(p), 0)
        return p

    def substep_gpu(self, scene, state, sorted_prim_id, worksets, iterations, dt, damping,
                    gravity, bending_fp64=False, colli=None, sphere=None, ground=None):
        """state: dict pos, vel (float32 (N,3)); modified in place.  sphere:
        (cx, cy, cz, r) pushed out after every sweep; ground: plane height."""
        c = self.constraints(scene)
        n = state["pos"].shape[0]
        prdp = state["pos"].copy()
        g = np.ascontiguousarray(gravity, dtype=np.float32)
        sid = np.ascontiguousarray(sorted_prim_id, dtype=np.int32)
        ws = np.ascontiguousarray(worksets, dtype=np.int32)
        cp = self._colli(colli)
        sp4 = None if sphere is None else np.ascontiguousarray(sphere, dtype=np.float32)
        nct = self.lib.orc_substep_gpu_obst(
            n, C.byref(c), _ptr(sid), len(ws), _ptr(ws), iterations, C.c_float(dt),
            C.c_float(damping), _ptr(g), _ptr(scene["mass"]), _ptr(state["pos"]),
            _ptr(state["vel"]), _ptr(prdp), int(bending_fp64),
            C.byref(cp) if cp is not None else None, _ptr(sp4), int(ground is not None),
            C.c_float(0.0 if ground is None else ground))
        state["prdp"] = prdp
        return nct

    def substep_cpu_ref(self, scene, state, iterations, dt, gravity, colli=None,
                        sphere=None):
        c = self.constraints(scene)
        n = state["pos"].shape[0]
        prdp = state["pos"].copy()
        g = np.ascontiguousarray(gravity, dtype=np.float32)
        cp = self._colli(colli)
        sc = None if sphere is None else np.ascontiguousarray(sphere[0], dtype=np.float32)
        sr = 0.0 if sphere is None else float(sphere[1])
        return self.lib.orc_substep_cpu_ref(
            n, C.byref(c), iterations, C.c_float(dt), _ptr(g), _ptr(scene["mass"]),
            _ptr(state["pos"]), _ptr(state["vel"]), _ptr(prdp),
            C.byref(cp) if cp is not None else None, _ptr(sc), C.c_float(sr))

    def _colli(self, colli):
        if colli is None:
            return None
        g = self.grid(colli["center"], colli.get("size"), colli["cell"], colli.get("bounded", False))
        tri = np.ascontiguousarray(colli["tri_idx"], dtype=np.int32)
        ti = colli.get("tri_inst")
        pi = colli.get("point_inst")
        cp = OrcColliParams(1, g, colli["thickness"], colli.get("resolve_passes", 1),
                            int(colli.get("mass_weighted", 0)), colli.get("ccd_every", 10),
                            len(tri), _ptr(tri), _ptr(ti), _ptr(pi),
                            colli.get("contact_cap", 1 << 20))
        cp._keep = (tri, ti, pi)
        return cp

    def residual(self, scene, prdp, hinge_rest=None):
        c = self.constraints(scene)
        num = C.c_double()
        den = C.c_double()
        p = np.ascontiguousarray(prdp, dtype=np.float32)
        hr = None if hinge_rest is None else np.ascontiguousarray(hinge_rest, dtype=np.float32)
        r = self.lib.orc_residual(C.byref(c), _ptr(p), _ptr(hr), C.byref(num), C.byref(den))
        return r, num.value, den.value

    # -- collision -------------------------------------------------------
    def grid(self, center, size, cell, bounded):
        g = OrcGrid()
        ce = np.ascontiguousarray(center, dtype=np.float32)
        cl = np.ascontiguousarray(np.broadcast_to(np.float32(cell), (3,)) if np.ndim(cell) == 0 else cell,
                                  dtype=np.float32)
        sz = None if size is None else np.ascontiguousarray(size, dtype=np.int32)
        self.lib.orc_grid_init(C.byref(g), _ptr(ce), _ptr(sz), _ptr(cl), int(bool(bounded)))
        return g

    def find_neighbors_all(self, grid, tri_idx, pos):
        tri = np.ascontiguousarray(tri_idx, dtype=np.int32)
        p = np.ascontiguousarray(pos, dtype=np.float32)
        nt = len(tri)
        sn = np.zeros((nt, 2), np.int32)
        tot = self.lib.orc_find_neighbors_all(C.byref(grid), nt, _ptr(tri), _ptr(p), _ptr(sn), None)
        out = np.zeros(max(tot, 1), np.int32)
        self.lib.orc_find_neighbors_all(C.byref(grid), nt, _ptr(tri), _ptr(p), _ptr(sn), _ptr(out))
        return sn, out[:tot]

    def solve_cubic(self, a, b, c, d):
        x = np.zeros(3, np.float64)
        n = self.lib.orc_solve_cubic(a, b, c, d, x)
        return x[:n]

    def vf_variant(self, kind, x, p, thickness, ids=(0, 1, 2, 3)):
        """kind: 'vfccd' (VFCCDTest, type VF), 'vfdcd' (VFDCDTest) or 'vf'
        (VFTest) -> (hit, t, w, n)"""
        fn = {"vfccd": self.lib.orc_vf_ccd_test, "vfdcd": self.lib.orc_vf_dcd_test,
              "vf": self.lib.orc_vf_test}[kind]
        xs = np.ascontiguousarray(x, dtype=np.float32).reshape(12)
        ps = np.ascontiguousarray(p, dtype=np.float32).reshape(12)
        ct = OrcContact()
        hit = fn(_ptr(xs), _ptr(ps), C.c_float(thickness), *[int(i) for i in ids], C.byref(ct))
        return hit, ct.t, np.array(ct.w), np.array(ct.n, dtype=np.float32)

    def extended_vf_test(self, x, p, thickness, ids=(0, 1, 2, 3), narrow=False, fp64=False):
        """fp64: the all-double yardstick (orc_extended_vf_test_f64)"""
        xs = np.ascontiguousarray(x, dtype=np.float32).reshape(12)
        ps = np.ascontiguousarray(p, dtype=np.float32).reshape(12)
        ct = OrcContact()
        fn = (self.lib.orc_extended_vf_test_f64 if fp64 else
              self.lib.orc_narrow_vf_ccd_test if narrow else self.lib.orc_extended_vf_test)
        hit = fn(_ptr(xs), _ptr(ps), C.c_float(thickness), *[int(i) for i in ids], C.byref(ct))
        return hit, ct.t, np.array(ct.w), np.array(ct.n, dtype=np.float32)

    def ccd(self, grid, tri_idx, pos, prdp, thickness, mode="pairs", tri_inst=None,
            point_inst=None, cap=1 << 20):
        tri = np.ascontiguousarray(tri_idx, dtype=np.int32)
        x = np.ascontiguousarray(pos, dtype=np.float32)
        p = np.ascontiguousarray(prdp, dtype=np.float32)
        arr = (OrcContact * cap)()
        if mode == "ref":
            h = self.lib.orc_ccd_sh_extended_ref(C.byref(grid), len(tri), _ptr(tri), _ptr(x),
                                                 _ptr(p), C.c_float(thickness), arr, C.c_int64(cap))
        else:
            h = self.lib.orc_ccd_vf_pairs(C.byref(grid), len(x), len(tri), _ptr(tri),
                                          _ptr(tri_inst), _ptr(point_inst), _ptr(x), _ptr(p),
                                          C.c_float(thickness), arr, C.c_int64(cap))
        return contacts_to_numpy(arr, min(h, cap)), h

    def _contacts_struct(self, ids, face=None):
        n = len(ids)
        arr = (OrcContact * max(n, 1))()
        for i in range(n):
            arr[i].v, arr[i].f0, arr[i].f1, arr[i].f2 = [int(v) for v in ids[i]]
            arr[i].face = -1 if face is None else int(face[i])
        return arr

    def resolve_ref(self, ids, pos, prdp, iterations, thickness):
        p = np.ascontiguousarray(prdp, dtype=np.float32).copy()
        x = np.ascontiguousarray(pos, dtype=np.float32)
        arr = self._contacts_struct(ids)
        self.lib.orc_collision_resolve_ref(len(ids), arr, _ptr(x), _ptr(p), iterations,
                                           C.c_float(thickness))
        return p

    def resolve_old(self, ids, pos, prdp, resolve_times, thickness):
        """CollisionResolve + VFResolve (the older response); resolve_times
        (int32 per point) is updated in place; returns the new positions"""
        p = np.ascontiguousarray(prdp, dtype=np.float32).copy()
        x = np.ascontiguousarray(pos, dtype=np.float32)
        assert resolve_times.dtype == np.int32 and resolve_times.flags.c_contiguous
        arr = self._contacts_struct(ids)
        self.lib.orc_collision_resolve_old(len(ids), arr, _ptr(x), _ptr(p), _ptr(resolve_times),
                                           C.c_float(thickness))
        return p

    def resolve_jacobi(self, ids, pos, prdp, mass, iterations, thickness, mass_weighted):
        p = np.ascontiguousarray(prdp, dtype=np.float32).copy()
        x = np.ascontiguousarray(pos, dtype=np.float32)
        m = None if mass is None else np.ascontiguousarray(mass, dtype=np.float32)
        arr = self._contacts_struct(ids)
        self.lib.orc_collision_resolve_jacobi(len(x), len(ids), arr, _ptr(x), _ptr(p), _ptr(m),
                                              iterations, C.c_float(thickness), int(mass_weighted))
        return p

    # -- edge-edge CCD (no reference arithmetic; see pbd_oracle.h) ----------
    def ee_test(self, x, p, thickness):
        """x, p: (4, 3) start / predicted a0, a1, b0, b1 -> (hit, t, s, u, m0[4])"""
        xs = np.ascontiguousarray(x, dtype=np.float32).reshape(12)
        ps = np.ascontiguousarray(p, dtype=np.float32).reshape(12)
        h = OrcEEHit()
        hit = self.lib.orc_ee_test(_ptr(xs), _ptr(ps), C.c_float(thickness), C.byref(h))
        return bool(hit), h.t, h.s, h.u, np.array(h.m0[:], np.float32)

    def ccd_ee_brute(self, edges, point_inst, x, p, thickness, cap=1 << 20):
        """all edge pairs tested: (pairs (n, 2), tsu (n, 3), m0 (n, 4))"""
        e = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 2)
        xs = np.ascontiguousarray(x, dtype=np.float32)
        ps = np.ascontiguousarray(p, dtype=np.float32)
        pi = None if point_inst is None else np.ascontiguousarray(point_inst, dtype=np.int32)
        pairs = np.zeros((cap, 2), np.int32)
        hits = (OrcEEHit * cap)()
        n = self.lib.orc_ccd_ee_brute(len(e), _ptr(e), _ptr(pi), _ptr(xs), _ptr(ps),
                                      C.c_float(thickness), _ptr(pairs), hits, C.c_int64(cap))
        assert n <= cap
        tsu = np.array([[hits[i].t, hits[i].s, hits[i].u] for i in range(n)], np.float32).reshape(-1, 3)
        m0 = np.array([hits[i].m0[:] for i in range(n)], np.float32).reshape(-1, 4)
        return pairs[:n].copy(), tsu, m0

    def resolve_jacobi_ee(self, vf_ids, ee_ids, ee_m0, pos, prdp, mass, iterations, thickness,
                          mass_weighted):
        """one Jacobi scheme over vertex-face (v, f0, f1, f2) and edge-edge
        (a0, a1, b0, b1; side info m0) contacts together"""
        p = np.ascontiguousarray(prdp, dtype=np.float32).copy()
        x = np.ascontiguousarray(pos, dtype=np.float32)
        m = None if mass is None else np.ascontiguousarray(mass, dtype=np.float32)
        vf = self._contacts_struct(vf_ids)
        ee = np.ascontiguousarray(ee_ids, dtype=np.int32).reshape(-1, 4)
        m0 = np.ascontiguousarray(ee_m0, dtype=np.float32).reshape(-1, 4)
        self.lib.orc_collision_resolve_jacobi_ee(len(x), len(vf_ids), vf, len(ee), _ptr(ee),
                                                 _ptr(m0), _ptr(x), _ptr(p), _ptr(m), iterations,
                                                 C.c_float(thickness), int(mass_weighted))
        return p

    def vf_resolve_test(self, x, p, thickness):
        xs = np.ascontiguousarray(x, dtype=np.float32).reshape(12)
        ps = np.ascontiguousarray(p, dtype=np.float32).reshape(12)
        return self.lib.orc_vf_resolve_test(_ptr(xs), _ptr(ps), C.c_float(thickness))

    def vf_resolve_new(self, x, p, thickness):
        xs = np.ascontiguousarray(x, dtype=np.float32).reshape(12)
        ps = np.ascontiguousarray(p, dtype=np.float32).reshape(12).copy()
        self.lib.orc_vf_resolve_new(_ptr(xs), _ptr(ps), C.c_float(thickness))
        return ps.reshape(4, 3)


class RefLib:
    """The reference's own compiled CPU code (development machine only)."""

    def __init__(self, path: str | None = None):
        path = path or _b.build_ref()
        if path is None or not os.path.exists(path):
            raise FileNotFoundError("reference library not built (reference sources absent)")
        self.lib = C.CDLL(path)
        L = self.lib
        L.ref_prim2prims.restype = C.c_longlong
        L.ref_find_neighbors_all.restype = C.c_longlong
        L.ref_ccd_sh_extended.restype = C.c_longlong
        L.ref_sort_worksets.restype = C.c_int
        L.ref_solve_cubic.restype = C.c_int
        L.ref_solve_cubic.argtypes = [C.c_double] * 4 + [_f64p]
        L.ref_extended_vf_test.restype = C.c_int
        L.ref_narrow_vf_ccd_test.restype = C.c_int
        L.ref_vf_resolve_test.restype = C.c_int
