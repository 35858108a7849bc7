"""Python mirror of the reference's cloth-step classes over the C ABI.

``PBDObject``, ``SolverPBD``, ``SpatialHashSystem`` and ``CollisionSolver``
keep the reference's names and method meanings (P/PBD_Basic.cuh:145-259,
P/SpatialHashSystem.h:10-96, P/CCD_Basic.h:33-135; P/ =
PositionBasedDynamicsCUDA/PositionBasedDynamicsCUDA/).  Every method is one
call into libpbd_gb300.so (include/pbd_c.h); there is no Python or CPU
fallback: if the library cannot be loaded, or a call fails, PBDError is
raised.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

DISTANCE, BENDING, ANCHOR = 0x001, 0x010, 0x100
JACOBI, GAUSSSEIDEL = 0, 1
RESPONSE_REFERENCE, RESPONSE_MASS_WEIGHTED = 0, 1
GS_AUTO, GS_PER_COLOR, GS_CLUSTER = 0, 1, 2
SCHEDULE_REFERENCE, SCHEDULE_UNIT, SCHEDULE_DIRECT = 0, 1, 2
_ERRS = {1: "ARG", 2: "OOM", 3: "CUDA", 4: "TIMEOUT", 5: "OVERFLOW", 6: "STATE"}


class PBDError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("PBD_ERR_%s: %s" % (_ERRS.get(code, code), msg))
        self.code = code


class _MeshDesc(C.Structure):
    _fields_ = [("n_points", C.c_int), ("pos", C.c_void_p), ("vel", C.c_void_p),
                ("mass", C.c_void_p), ("rest_pos", C.c_void_p), ("n_tris", C.c_int),
                ("tri_idx", C.c_void_p), ("ct_mask", C.c_uint), ("stiffness", C.c_float * 2),
                ("point_inst", C.c_void_p), ("tri_inst", C.c_void_p),
                ("damping_rate", C.c_float), ("gravity", C.c_float * 3)]


class _Desc(C.Structure):
    _fields_ = [("n_points", C.c_int), ("pos", C.c_void_p), ("vel", C.c_void_p),
                ("mass", C.c_void_p), ("n_tris", C.c_int), ("tri_idx", C.c_void_p),
                ("n_prims", C.c_int), ("prim_list", C.c_void_p), ("indices", C.c_void_p),
                ("constraint_type", C.c_void_p), ("rest_length", C.c_void_p),
                ("stiffness", C.c_void_p), ("rest_angle", C.c_void_p), ("rest_pos", C.c_void_p),
                ("point_inst", C.c_void_p), ("tri_inst", C.c_void_p),
                ("damping_rate", C.c_float), ("gravity", C.c_float * 3)]


_LIB = None

# every symbol include/pbd_c.h declares
EXPORTS = [
    "pbd_last_error", "pbd_version", "pbd_object_create", "pbd_object_create_grid",
    "pbd_object_destroy", "pbd_object_sizes", "pbd_object_get_positions",
    "pbd_object_get_velocities", "pbd_object_get_predicted", "pbd_object_set_positions",
    "pbd_object_set_velocities", "pbd_object_set_predicted", "pbd_object_stream",
    "pbd_object_sync", "pbd_constraints_edge_coloring", "pbd_constraints_sort_edges_colors",
    "pbd_constraints_eval_worksets", "pbd_constraints_set_colors", "pbd_constraints_get_colors",
    "pbd_constraints_get_sorted", "pbd_constraints_get_worksets",
    "pbd_constraints_get_adjacency", "pbd_constraints_residual", "pbd_solver_create",
    "pbd_solver_destroy", "pbd_solver_set_target", "pbd_solver_advect",
    "pbd_solver_project_constraint", "pbd_solver_project_constraint_with_colli",
    "pbd_solver_integration", "pbd_solver_set_sphere", "pbd_solver_set_ground",
    "pbd_solver_set_instance_spheres",
    "pbd_solver_step", "pbd_solver_set_gs_path", "pbd_solver_get_gs_path",
    "pbd_solver_graph_kernels", "pbd_shs_create", "pbd_shs_create_hashed", "pbd_shs_destroy",
    "pbd_shs_set_grid_center", "pbd_shs_set_grid_size", "pbd_shs_set_division", "pbd_shs_init",
    "pbd_shs_update", "pbd_shs_find_neighbors", "pbd_shs_find_neighbors_all",
    "pbd_colli_create", "pbd_colli_destroy", "pbd_colli_set_target",
    "pbd_colli_set_acce_struct", "pbd_colli_set_thickness", "pbd_colli_set_iterations",
    "pbd_colli_set_response", "pbd_colli_set_capacity", "pbd_colli_set_overlap",
    "pbd_colli_ccd_sh_extended",
    "pbd_colli_collision_resolve_new", "pbd_colli_collision_resolve_old",
    "pbd_colli_resolve_times", "pbd_colli_get_contacts", "pbd_colli_stats",
    "pbd_colli_get_pairs",
    "pbd_ccd_vf_test_batch", "pbd_ccd_vf_test_batch_mode", "pbd_colli_set_vf_test",
    "pbd_residual_noalloc",
    "pbd_scene_read_cache", "pbd_scene_read_txt", "pbd_scene_desc", "pbd_scene_destroy",
    "pbd_scene_write_cache", "pbd_object_create_from_cache", "pbd_object_save_cache",
    "pbd_constraints_residual_stretch", "pbd_solver_step_to_residual", "pbd_solver_solve_stats",
    "pbd_solver_residual_graph_kernels", "pbd_object_get_correction",
    "pbd_object_set_correction",
    "pbd_warmstart_num_params", "pbd_warmstart_create", "pbd_warmstart_destroy",
    "pbd_warmstart_set_params", "pbd_warmstart_get_params", "pbd_warmstart_forward",
    "pbd_warmstart_set_scales", "pbd_warmstart_get_scales",
    "pbd_warmstart_gradients", "pbd_warmstart_set_gradient", "pbd_warmstart_adam",
    "pbd_warmstart_record", "pbd_warmstart_train_step", "pbd_warmstart_features",
    "pbd_warmstart_predict", "pbd_solver_set_warmstart", "pbd_solver_project_to_residual",
    "pbd_solver_autotune", "pbd_solver_get_gs_block",
    "pbd_solver_set_gs_block", "pbd_solver_train_substep", "pbd_solver_set_gs_cluster",
    "pbd_solver_get_gs_cluster", "pbd_mesh_constraints", "pbd_object_create_mesh",
    "pbd_object_set_stiffness_schedule", "pbd_object_get_stiffness_schedule",
    "pbd_object_set_stiffness", "pbd_object_set_anchor_targets",
    "pbd_colli_set_edge_edge", "pbd_colli_ee_edges", "pbd_colli_get_ee_contacts",
    "pbd_colli_ee_stats", "pbd_ee_test_batch", "pbd_object_get_state", "pbd_object_set_state",
    "pbd_shs_set_instance_cells",
]


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libpbd_gb300.so (building it with nvcc if absent)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise PBDError(3, "libpbd_gb300.so not built: run python -m positionbaseddynamicsold_gb300.build")
        path = _build.build()
    L = C.CDLL(path)
    for name in EXPORTS:
        f = getattr(L, name)
        f.restype = C.c_int
    L.pbd_last_error.restype = C.c_char_p
    L.pbd_solver_advect.argtypes = [C.c_void_p, C.c_float]
    L.pbd_solver_integration.argtypes = [C.c_void_p, C.c_float]
    L.pbd_solver_project_constraint.argtypes = [C.c_void_p, C.c_int, C.c_int]
    L.pbd_solver_project_constraint_with_colli.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    L.pbd_solver_step.argtypes = [C.c_void_p, C.c_float, C.c_int, C.c_int, C.c_void_p, C.c_int]
    L.pbd_solver_set_sphere.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_float]
    L.pbd_solver_set_ground.argtypes = [C.c_void_p, C.c_int, C.c_float]
    L.pbd_colli_set_thickness.argtypes = [C.c_void_p, C.c_float]
    L.pbd_colli_set_capacity.argtypes = [C.c_void_p, C.c_longlong, C.c_longlong]
    L.pbd_object_create_grid.argtypes = [C.c_float, C.c_void_p, C.c_int, C.c_int, C.c_float,
                                         C.c_float, C.c_uint, C.c_void_p, C.c_void_p]
    L.pbd_constraints_get_adjacency.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_longlong, C.c_void_p]
    L.pbd_shs_find_neighbors_all.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong,
                                             C.c_void_p]
    L.pbd_colli_get_contacts.argtypes = [C.c_void_p] + [C.c_void_p] * 5 + [C.c_longlong, C.c_void_p]
    L.pbd_residual_noalloc.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                       C.c_void_p]
    L.pbd_solver_step_to_residual.argtypes = [C.c_void_p, C.c_float, C.c_int, C.c_void_p,
                                              C.c_double, C.c_int, C.c_int, C.c_int]
    L.pbd_solver_project_to_residual.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_int,
                                                 C.c_int, C.c_void_p, C.c_void_p]
    L.pbd_solver_train_substep.argtypes = [C.c_void_p, C.c_void_p, C.c_float, C.c_void_p,
                                           C.c_double, C.c_int, C.c_int, C.c_float, C.c_int,
                                           C.c_void_p]
    L.pbd_scene_read_txt.argtypes = [C.c_char_p, C.c_char_p, C.c_float, C.c_void_p]
    L.pbd_scene_read_cache.argtypes = [C.c_char_p, C.c_char_p, C.c_void_p]
    L.pbd_scene_write_cache.argtypes = [C.c_void_p, C.c_void_p, C.c_char_p, C.c_char_p]
    L.pbd_object_create_from_cache.argtypes = [C.c_char_p, C.c_char_p, C.c_void_p]
    L.pbd_object_save_cache.argtypes = [C.c_void_p, C.c_char_p, C.c_char_p]
    L.pbd_mesh_constraints.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_longlong,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p]
    L.pbd_object_set_stiffness.argtypes = [C.c_void_p, C.c_uint, C.c_float]
    L.pbd_colli_ee_edges.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p]
    L.pbd_colli_get_ee_contacts.argtypes = [C.c_void_p] + [C.c_void_p] * 4 + [C.c_longlong,
                                                                              C.c_void_p]
    L.pbd_warmstart_adam.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_float]
    L.pbd_warmstart_train_step.argtypes = [C.c_void_p, C.c_void_p, C.c_float, C.c_void_p]
    _LIB = L
    return L


def _check(rc):
    if rc != 0:
        raise PBDError(rc, _LIB.pbd_last_error().decode(errors="replace"))


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a if shape is None else a.reshape(shape)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class PBDObject:
    """PBDObject + ConstraintPBD (P/PBD_Basic.cuh:97-211) resident on the GPU."""

    def __init__(self, scene=None, damping=1.0, gravity=(0.0, -9.8, 0.0), _handle=None):
        self.L = load()
        self.h = C.c_void_p()
        if _handle is not None:
            self.h = _handle
        else:
            self._create(scene, damping, gravity)
        n, nt, np_ = C.c_int(), C.c_int(), C.c_int()
        _check(self.L.pbd_object_sizes(self.h, C.byref(n), C.byref(nt), C.byref(np_)))
        self.n_points, self.n_tris, self.n_prims = n.value, nt.value, np_.value

    def _create(self, s, damping, gravity):
        keep = []

        def k(a):
            keep.append(a)
            return _p(a)

        d = _Desc()
        pos = _f32(s["pos"]).reshape(-1)
        d.n_points = len(pos) // 3
        d.pos = k(pos)
        d.vel = k(_f32(s["vel"]).reshape(-1)) if s.get("vel") is not None else None
        d.mass = k(_f32(s["mass"]))
        tri = _i32(s.get("tri_idx", np.zeros((0, 3), np.int32))).reshape(-1)
        d.n_tris = len(tri) // 3
        d.tri_idx = k(tri) if len(tri) else None
        ct = _i32(s.get("ctype", np.zeros(0, np.int32)))
        d.n_prims = len(ct)
        if len(ct):
            d.prim_list = k(_i32(s["prim_list"]).reshape(-1))
            d.indices = k(_i32(s["indices"]))
            d.constraint_type = k(ct)
            d.rest_length = k(_f32(s["rest_length"]))
            d.stiffness = k(_f32(s["stiffness"]))
            if s.get("rest_angle") is not None:
                d.rest_angle = k(_f32(s["rest_angle"]))
            if s.get("rest_pos") is not None:
                d.rest_pos = k(_f32(s["rest_pos"]).reshape(-1))
        if s.get("point_inst") is not None:
            d.point_inst = k(_i32(s["point_inst"]))
            d.tri_inst = k(_i32(s["tri_inst"]))
        d.damping_rate = damping
        for i in range(3):
            d.gravity[i] = gravity[i]
        _check(self.L.pbd_object_create(C.byref(d), C.byref(self.h)))

    @classmethod
    def from_mesh(cls, pos, tris, mass, vel=None, rest_pos=None, stiffness=(1.0, 0.1),
                  bending=True, point_inst=None, tri_inst=None, damping=1.0,
                  gravity=(0.0, -9.8, 0.0)):
        """an object whose constraints the device derives from the triangle
        mesh (pbd_object_create_mesh): distance on every edge, bending on
        every interior edge"""
        L = load()
        keep = []

        def k(a):
            keep.append(a)
            return _p(a)

        d = _MeshDesc()
        p = _f32(pos).reshape(-1)
        t = _i32(tris).reshape(-1)
        d.n_points = len(p) // 3
        d.pos = k(p)
        d.vel = k(_f32(vel).reshape(-1)) if vel is not None else None
        d.mass = k(_f32(mass))
        d.rest_pos = k(_f32(rest_pos).reshape(-1)) if rest_pos is not None else None
        d.n_tris = len(t) // 3
        d.tri_idx = k(t)
        d.ct_mask = DISTANCE | (BENDING if bending else 0)
        d.stiffness[0], d.stiffness[1] = float(stiffness[0]), float(stiffness[1])
        if point_inst is not None:
            d.point_inst = k(_i32(point_inst))
            d.tri_inst = k(_i32(tri_inst))
        d.damping_rate = damping
        for i in range(3):
            d.gravity[i] = gravity[i]
        h = C.c_void_p()
        _check(L.pbd_object_create_mesh(C.byref(d), C.byref(h)))
        return cls(_handle=h)

    @classmethod
    def from_cache(cls, topol_path, constr_path):
        """PBDObject::ContinueSimInit: an object from the reference's two caches"""
        L = load()
        h = C.c_void_p()
        _check(L.pbd_object_create_from_cache(_enc(topol_path), _enc(constr_path), C.byref(h)))
        return cls(_handle=h)

    def set_stiffness_schedule(self, mode):
        """SCHEDULE_REFERENCE (k = 1-(1-s)^(1/(iter+1))), SCHEDULE_UNIT (k = 1)
        or SCHEDULE_DIRECT (k = s)"""
        _check(self.L.pbd_object_set_stiffness_schedule(self.h, int(mode)))

    def stiffness_schedule(self):
        v = C.c_int()
        _check(self.L.pbd_object_get_stiffness_schedule(self.h, C.byref(v)))
        return v.value

    def set_stiffness(self, ct_mask, value):
        """stiffness of every constraint of the types in ct_mask"""
        _check(self.L.pbd_object_set_stiffness(self.h, int(ct_mask), float(value)))

    def set_anchor_targets(self, prims, targets):
        """move the rest positions (targets, (n, 3)) of the ANCHOR prims"""
        p = _i32(prims).reshape(-1)
        t = _f32(targets).reshape(-1)
        assert len(t) == 3 * len(p)
        _check(self.L.pbd_object_set_anchor_targets(self.h, len(p), _p(p), _p(t)))

    def save_cache(self, topol_path, constr_path):
        """the current state as the reference's two caches"""
        _check(self.L.pbd_object_save_cache(self.h, _enc(topol_path), _enc(constr_path)))

    @classmethod
    def grid(cls, res_x, res_y, size_x, size_y, ct=DISTANCE, stiffness=(1.0, 0.1, -1.0),
             damping=1.0, gravity=(0.0, -9.8, 0.0)):
        """PBDObject(damping, gravity, resX, resY, sizeX, sizeY) + SetConstrOption + Init()."""
        L = load()
        h = C.c_void_p()
        g = np.asarray(gravity, np.float32)
        st = np.asarray(stiffness, np.float32)
        _check(L.pbd_object_create_grid(damping, _p(g), res_x, res_y, size_x, size_y, ct, _p(st),
                                        C.byref(h)))
        return cls(_handle=h)

    def close(self):
        if self.h:
            self.L.pbd_object_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _get3(self, fn):
        out = np.empty((self.n_points, 3), np.float32)
        _check(fn(self.h, _p(out)))
        return out

    def positions(self):
        return self._get3(self.L.pbd_object_get_positions)

    def velocities(self):
        return self._get3(self.L.pbd_object_get_velocities)

    def predicted(self):
        return self._get3(self.L.pbd_object_get_predicted)

    def get_state(self, pos=None, vel=None):
        """positions and velocities in one call; pos / vel: optional (n, 3)
        float32 arrays to fill (page-locked ones are copied directly)"""
        pos = np.empty((self.n_points, 3), np.float32) if pos is None else pos
        vel = np.empty((self.n_points, 3), np.float32) if vel is None else vel
        assert pos.dtype == np.float32 and vel.dtype == np.float32
        assert pos.flags.c_contiguous and vel.flags.c_contiguous
        _check(self.L.pbd_object_get_state(self.h, _p(pos), _p(vel)))
        return pos, vel

    def set_state(self, pos, vel):
        _check(self.L.pbd_object_set_state(self.h, _p(_f32(pos, (-1,))), _p(_f32(vel, (-1,)))))

    def set_positions(self, a):
        _check(self.L.pbd_object_set_positions(self.h, _p(_f32(a, (-1,)))))

    def set_velocities(self, a):
        _check(self.L.pbd_object_set_velocities(self.h, _p(_f32(a, (-1,)))))

    def set_predicted(self, a):
        _check(self.L.pbd_object_set_predicted(self.h, _p(_f32(a, (-1,)))))

    def stream(self) -> int:
        s = C.c_void_p()
        _check(self.L.pbd_object_stream(self.h, C.byref(s)))
        return s.value or 0

    def sync(self):
        _check(self.L.pbd_object_sync(self.h))

    # ConstraintPBD
    def edge_coloring(self, iterations=20000):
        sw = C.c_int()
        _check(self.L.pbd_constraints_edge_coloring(self.h, iterations, C.byref(sw)))
        return sw.value

    def sort_edges_colors(self):
        _check(self.L.pbd_constraints_sort_edges_colors(self.h))

    def eval_worksets(self):
        n = C.c_int()
        _check(self.L.pbd_constraints_eval_worksets(self.h, C.byref(n)))
        return n.value

    def set_colors(self, color):
        _check(self.L.pbd_constraints_set_colors(self.h, _p(_i32(color))))

    def colors(self):
        out = np.empty(self.n_prims, np.int32)
        _check(self.L.pbd_constraints_get_colors(self.h, _p(out)))
        return out

    def sorted(self):
        sc = np.empty(self.n_prims, np.int32)
        sp = np.empty(self.n_prims, np.int32)
        _check(self.L.pbd_constraints_get_sorted(self.h, _p(sc), _p(sp)))
        return sc, sp

    def worksets(self):
        n = C.c_int()
        _check(self.L.pbd_constraints_get_worksets(self.h, None, 0, C.byref(n)))
        out = np.empty((max(n.value, 1), 2), np.int32)
        _check(self.L.pbd_constraints_get_worksets(self.h, _p(out), n.value, C.byref(n)))
        return out[:n.value]

    def adjacency(self):
        tot = C.c_longlong()
        sn = np.empty((self.n_prims, 2), np.int32)
        _check(self.L.pbd_constraints_get_adjacency(self.h, _p(sn), None, 0, C.byref(tot)))
        adj = np.empty(max(tot.value, 1), np.int32)
        _check(self.L.pbd_constraints_get_adjacency(self.h, None, _p(adj), tot.value, C.byref(tot)))
        return sn, adj[:tot.value]

    def residual(self):
        r = C.c_double()
        _check(self.L.pbd_constraints_residual(self.h, C.byref(r)))
        return r.value

    def residual_stretch(self):
        """relative stretch residual of the predicted positions (distance
        constraints only), the stopping test of step_to_residual"""
        r = C.c_double()
        _check(self.L.pbd_constraints_residual_stretch(self.h, C.byref(r)))
        return r.value

    def correction(self):
        """p_final - p_advected of the last substep solved to a residual"""
        return self._get3(self.L.pbd_object_get_correction)

    def set_correction(self, d):
        d = _f32(d).reshape(-1)
        _check(self.L.pbd_object_set_correction(self.h, _p(d)))

    def prepare(self, iterations=20000):
        """EdgeColoring + SortEdgesColors + EvalWorksets; returns sweeps."""
        sw = self.edge_coloring(iterations)
        self.sort_edges_colors()
        self.eval_worksets()
        return sw


def mesh_constraints(rest_pos, tris, dist_stiffness=1.0, bend_stiffness=0.1, bending=True):
    """The constraint set of a triangle mesh derived on the device
    (pbd_mesh_constraints), in the layout of scenes.constraints_from_mesh:
    distance prims on the edges, then bending prims on the interior edges."""
    L = load()
    rp = _f32(rest_pos).reshape(-1)
    t = _i32(tris).reshape(-1)
    n, nt = len(rp) // 3, len(t) // 3
    ne, nh = C.c_int(), C.c_int()
    _check(L.pbd_mesh_constraints(n, _p(rp), nt, _p(t), 0, C.byref(ne), C.byref(nh),
                                  None, None, None, None))
    cap = max(ne.value, nh.value, 1)
    e = np.zeros((cap, 2), np.int32)
    el = np.zeros(cap, np.float32)
    h = np.zeros((cap, 4), np.int32)
    ha = np.zeros(cap, np.float32)
    _check(L.pbd_mesh_constraints(n, _p(rp), nt, _p(t), cap, C.byref(ne), C.byref(nh),
                                  _p(e), _p(el), _p(h), _p(ha)))
    nd, nb = ne.value, (nh.value if bending else 0)
    e, el, h, ha = e[:nd], el[:nd], h[:nb], ha[:nb]
    prim_list = np.concatenate([
        np.stack([np.arange(nd) * 2, np.full(nd, 2)], 1),
        np.stack([2 * nd + np.arange(nb) * 4, np.full(nb, 4)], 1)], 0).astype(np.int32)
    rest_length = np.zeros(nd + nb, np.float32)
    rest_length[:nd] = el
    rest_angle = np.zeros(nd + nb, np.float32)
    rest_angle[nd:] = ha
    return {
        "prim_list": prim_list,
        "indices": np.concatenate([e.ravel(), h.ravel()]).astype(np.int32),
        "ctype": np.concatenate([np.full(nd, DISTANCE), np.full(nb, BENDING)]).astype(np.int32),
        "rest_length": rest_length,
        "stiffness": np.concatenate([np.full(nd, dist_stiffness),
                                     np.full(nb, bend_stiffness)]).astype(np.float32),
        "rest_angle": rest_angle, "rest_pos": np.zeros((nd + nb, 3), np.float32),
        "n_distance": nd, "n_bending": nb,
    }


class SpatialHashSystem:
    """SpatialHashSystem (P/SpatialHashSystem.h:10-96) over an object's triangles."""

    def __init__(self, obj: PBDObject, grid_center=(0.0, 0.0, 0.0), grid_size=None,
                 cell_size=(1.0, 1.0, 1.0), log2_table=None):
        self.L = load()
        self.obj = obj
        self.h = C.c_void_p()
        cell = np.broadcast_to(np.asarray(cell_size, np.float32), (3,)).copy()
        if grid_size is None:
            _check(self.L.pbd_shs_create_hashed(obj.h, _p(cell), int(log2_table or 20), C.byref(self.h)))
            if any(grid_center):
                _check(self.L.pbd_shs_set_grid_center(self.h, _p(np.asarray(grid_center, np.float32))))
        else:
            _check(self.L.pbd_shs_create(obj.h, _p(np.asarray(grid_center, np.float32)),
                                         _p(np.asarray(grid_size, np.int32)), _p(cell),
                                         C.byref(self.h)))

    def set_instance_cells(self, cells):
        """cell size per instance ((n_instances, 3) or (n_instances,)); None
        or empty: one cell size for all"""
        if cells is None or len(cells) == 0:
            _check(self.L.pbd_shs_set_instance_cells(self.h, 0, None))
            return
        c = np.asarray(cells, np.float32)
        if c.ndim == 1:
            c = np.repeat(c[:, None], 3, 1)
        c = np.ascontiguousarray(c.reshape(-1, 3))
        _check(self.L.pbd_shs_set_instance_cells(self.h, len(c), _p(c)))

    def close(self):
        if self.h:
            self.L.pbd_shs_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init(self):
        _check(self.L.pbd_shs_init(self.h))

    def update(self):
        _check(self.L.pbd_shs_update(self.h))

    def find_neighbors_all(self):
        tot = C.c_longlong()
        sn = np.empty((self.obj.n_tris, 2), np.int32)
        _check(self.L.pbd_shs_find_neighbors_all(self.h, _p(sn), None, 0, C.byref(tot)))
        out = np.empty(max(tot.value, 1), np.int32)
        _check(self.L.pbd_shs_find_neighbors_all(self.h, None, _p(out), tot.value, C.byref(tot)))
        return sn, out[:tot.value]

    def find_neighbors(self, tri):
        n = C.c_int()
        _check(self.L.pbd_shs_find_neighbors(self.h, tri, None, 0, C.byref(n)))
        out = np.empty(max(n.value, 1), np.int32)
        _check(self.L.pbd_shs_find_neighbors(self.h, tri, _p(out), n.value, C.byref(n)))
        return out[:n.value]


class CollisionSolver:
    """CollisionSolver (P/CCD_Basic.h:33-135)."""

    def __init__(self, obj: PBDObject = None, shs: SpatialHashSystem = None, thickness=0.0,
                 iterations=1, response=RESPONSE_REFERENCE):
        self.L = load()
        self.h = C.c_void_p()
        _check(self.L.pbd_colli_create(C.byref(self.h)))
        if obj is not None:
            self.set_target(obj)
        if shs is not None:
            self.set_acce_struct(shs)
        self.set_thickness(thickness)
        self.set_iterations(iterations)
        self.set_response(response)

    def close(self):
        if self.h:
            self.L.pbd_colli_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_target(self, obj):
        self.obj = obj
        _check(self.L.pbd_colli_set_target(self.h, obj.h))

    def set_acce_struct(self, shs):
        self.shs = shs
        _check(self.L.pbd_colli_set_acce_struct(self.h, shs.h))

    def set_thickness(self, t):
        _check(self.L.pbd_colli_set_thickness(self.h, float(t)))

    def set_iterations(self, it):
        _check(self.L.pbd_colli_set_iterations(self.h, int(it)))

    def set_response(self, mode):
        _check(self.L.pbd_colli_set_response(self.h, int(mode)))

    def set_capacity(self, candidates, contacts):
        _check(self.L.pbd_colli_set_capacity(self.h, int(candidates), int(contacts)))

    def collision_resolve_old(self):
        """CollisionResolve + VFResolve, the reference's older response"""
        _check(self.L.pbd_colli_collision_resolve_old(self.h))

    def resolve_times(self, reset=False):
        """the older response's per-point resolve counters (int32)"""
        n = self.obj.n_points
        out = np.zeros(n, np.int32)
        _check(self.L.pbd_colli_resolve_times(self.h, _p(out), int(bool(reset))))
        return out

    def set_vf_test(self, mode):
        """narrowphase test of the detection (VFTEST_EXTENDED: CCD_SH_Extended,
        VFTEST_NARROW: CCD_SH_Narrow, VFTEST_VF: CCD_SH)"""
        _check(self.L.pbd_colli_set_vf_test(self.h, int(mode)))

    def set_overlap(self, on=True):
        """detections inside step / project_constraint_with_colli run beside
        the following sweep on a side stream (same results either way)"""
        _check(self.L.pbd_colli_set_overlap(self.h, int(bool(on))))

    def ccd_sh_extended(self):
        _check(self.L.pbd_colli_ccd_sh_extended(self.h))

    def collision_resolve_new(self):
        _check(self.L.pbd_colli_collision_resolve_new(self.h))

    def contacts(self):
        cnt = C.c_longlong()
        _check(self.L.pbd_colli_get_contacts(self.h, None, None, None, None, None, 0, C.byref(cnt)))
        h = cnt.value
        ids = np.empty((max(h, 1), 4), np.int32)
        face = np.empty(max(h, 1), np.int32)
        t = np.empty(max(h, 1), np.float32)
        w = np.empty((max(h, 1), 4), np.float64)
        n = np.empty((max(h, 1), 3), np.float32)
        _check(self.L.pbd_colli_get_contacts(self.h, _p(ids), _p(face), _p(t), _p(w), _p(n), h,
                                             C.byref(cnt)))
        return {"ids": ids[:h], "face": face[:h], "t": t[:h], "w": w[:h], "n": n[:h]}

    def pairs(self):
        """the hash search's (point, triangle) pairs of the last CCD call,
        sorted"""
        n = C.c_longlong()
        _check(self.L.pbd_colli_get_pairs(self.h, None, 0, C.byref(n)))
        out = np.zeros((max(n.value, 1), 2), np.int32)
        _check(self.L.pbd_colli_get_pairs(self.h, _p(out), n.value, C.byref(n)))
        out = out[: n.value]
        return out[np.lexsort((out[:, 1], out[:, 0]))]

    def stats(self):
        a, b, c = C.c_longlong(), C.c_longlong(), C.c_int()
        _check(self.L.pbd_colli_stats(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return {"candidates": a.value, "contacts": b.value, "overflow": c.value}

    # edge-edge CCD (no reference arithmetic; off by default)
    def set_edge_edge(self, on=True):
        _check(self.L.pbd_colli_set_edge_edge(self.h, int(bool(on))))

    def ee_edges(self):
        n = C.c_int()
        _check(self.L.pbd_colli_ee_edges(self.h, None, 0, C.byref(n)))
        e = np.zeros((max(n.value, 1), 2), np.int32)
        _check(self.L.pbd_colli_ee_edges(self.h, _p(e), len(e), C.byref(n)))
        return e[:n.value]

    def ee_contacts(self):
        """(pairs (n, 2), ids (n, 4), tsu (n, 3), m0 (n, 4)) sorted by edge pair"""
        n = C.c_longlong()
        _check(self.L.pbd_colli_get_ee_contacts(self.h, None, None, None, None, 0, C.byref(n)))
        k = max(n.value, 1)
        pairs = np.zeros((k, 2), np.int32)
        ids = np.zeros((k, 4), np.int32)
        tsu = np.zeros((k, 3), np.float32)
        m0 = np.zeros((k, 4), np.float32)
        _check(self.L.pbd_colli_get_ee_contacts(self.h, _p(pairs), _p(ids), _p(tsu), _p(m0), k,
                                                C.byref(n)))
        m = n.value
        return pairs[:m], ids[:m], tsu[:m], m0[:m]

    def ee_stats(self):
        v = [C.c_longlong() for _ in range(4)]
        _check(self.L.pbd_colli_ee_stats(self.h, *[C.byref(x) for x in v]))
        return dict(zip(("entries", "pairs", "candidates", "contacts"), [x.value for x in v]))


class SolverPBD:
    """SolverPBD (P/PBD_Basic.cuh:213-259)."""

    def __init__(self, obj: PBDObject = None):
        self.L = load()
        self.h = C.c_void_p()
        _check(self.L.pbd_solver_create(C.byref(self.h)))
        if obj is not None:
            self.set_target(obj)

    def close(self):
        if self.h:
            self.L.pbd_solver_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_target(self, obj):
        self.obj = obj
        _check(self.L.pbd_solver_set_target(self.h, obj.h))

    def advect(self, dt):
        _check(self.L.pbd_solver_advect(self.h, dt))

    def project_constraint(self, iterations, solver_type=GAUSSSEIDEL):
        _check(self.L.pbd_solver_project_constraint(self.h, solver_type, iterations))

    def project_constraint_with_colli(self, iterations, colli, solver_type=GAUSSSEIDEL):
        _check(self.L.pbd_solver_project_constraint_with_colli(self.h, solver_type, iterations,
                                                               colli.h if colli else None))

    def integration(self, dt):
        _check(self.L.pbd_solver_integration(self.h, dt))

    def set_sphere(self, enable, center=(0.0, 0.0, 0.0), radius=1.0):
        c = np.asarray(center, np.float32)
        _check(self.L.pbd_solver_set_sphere(self.h, int(enable), _p(c), radius))

    def set_ground(self, enable, height=0.0):
        _check(self.L.pbd_solver_set_ground(self.h, int(enable), height))

    def set_instance_spheres(self, spheres):
        """spheres: (n_instances, 4) centre xyz + radius, or None."""
        if spheres is None or len(spheres) == 0:
            _check(self.L.pbd_solver_set_instance_spheres(self.h, 0, None))
            return
        a = np.ascontiguousarray(spheres, np.float32).reshape(-1, 4)
        _check(self.L.pbd_solver_set_instance_spheres(self.h, len(a), _p(a)))

    def set_gs_path(self, path):
        _check(self.L.pbd_solver_set_gs_path(self.h, int(path)))

    def gs_path(self):
        v = C.c_int()
        _check(self.L.pbd_solver_get_gs_path(self.h, C.byref(v)))
        return v.value

    def graph_kernels(self):
        n = C.c_longlong()
        _check(self.L.pbd_solver_graph_kernels(self.h, C.byref(n)))
        return n.value

    def step(self, dt, substeps=1, iterations=20, colli=None, use_graph=True):
        _check(self.L.pbd_solver_step(self.h, dt, substeps, iterations,
                                      colli.h if colli else None, int(use_graph)))

    def set_warmstart(self, ws, min_sweeps=0):
        self.ws = ws
        _check(self.L.pbd_solver_set_warmstart(self.h, ws.h if ws is not None else None,
                                               int(min_sweeps)))

    def step_to_residual(self, dt, substeps=1, target=1e-4, max_sweeps=60, chunk=5, colli=None,
                         use_graph=True):
        """substeps solved until the stretch residual <= target (in chunks
        of `chunk` sweeps, at most max_sweeps)"""
        _check(self.L.pbd_solver_step_to_residual(self.h, dt, substeps,
                                                  colli.h if colli else None, float(target),
                                                  int(max_sweeps), int(chunk), int(use_graph)))

    def project_to_residual(self, target=1e-4, max_sweeps=60, chunk=5, colli=None):
        """the solve alone (no advect / integration); returns (sweeps, residual)"""
        sw = C.c_int()
        r = C.c_double()
        _check(self.L.pbd_solver_project_to_residual(self.h, colli.h if colli else None,
                                                     float(target), int(max_sweeps), int(chunk),
                                                     C.byref(sw), C.byref(r)))
        return sw.value, r.value

    def autotune(self, iterations=15, reps=5):
        """time the GS launch forms and keep the fastest; returns the table"""
        r = _AutotuneResult()
        _check(self.L.pbd_solver_autotune(self.h, int(iterations), int(reps), C.byref(r)))
        rows = [{"path": r.path[k], "block": r.block[k], "us_per_sweep": r.us_per_sweep[k]}
                for k in range(r.n)]
        return {"candidates": rows, "best": r.best}

    def set_gs_block(self, block):
        _check(self.L.pbd_solver_set_gs_block(self.h, int(block)))

    def gs_block(self):
        v = C.c_int()
        _check(self.L.pbd_solver_get_gs_block(self.h, C.byref(v)))
        return v.value

    def set_gs_cluster(self, size):
        """cluster size of the resident form (0: the largest that fits)"""
        _check(self.L.pbd_solver_set_gs_cluster(self.h, int(size)))

    def gs_cluster(self):
        v = C.c_int()
        _check(self.L.pbd_solver_get_gs_cluster(self.h, C.byref(v)))
        return v.value

    def train_substep(self, ws, dt, target=1e-3, max_sweeps=200, chunk=5, lr=1e-3,
                      on_policy=True, colli=None, want_loss=False):
        """one training substep of the warm start (see pbd_solver_train_substep)"""
        loss = C.c_double()
        _check(self.L.pbd_solver_train_substep(self.h, ws.h, dt, colli.h if colli else None,
                                               float(target), int(max_sweeps), int(chunk),
                                               float(lr), int(on_policy),
                                               C.byref(loss) if want_loss else None))
        return loss.value if want_loss else None

    def solve_stats(self, reset=False):
        st = _SolveStats()
        _check(self.L.pbd_solver_solve_stats(self.h, C.byref(st), int(reset)))
        return {k: getattr(st, k) for k, _ in _SolveStats._fields_}

    def residual_graph_kernels(self):
        """(kernels outside the WHILE bodies, kernels in one body)"""
        a, b = C.c_longlong(), C.c_longlong()
        _check(self.L.pbd_solver_residual_graph_kernels(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value


class _SolveStats(C.Structure):
    _fields_ = [("substeps", C.c_longlong), ("sweeps", C.c_longlong), ("reached", C.c_longlong),
                ("reverts", C.c_longlong), ("last_residual", C.c_double),
                ("last_sweeps", C.c_int), ("last_r0", C.c_double), ("last_r1", C.c_double)]


class _AutotuneResult(C.Structure):
    _fields_ = [("n", C.c_int), ("best", C.c_int), ("path", C.c_int * 12),
                ("block", C.c_int * 12), ("us_per_sweep", C.c_double * 12)]


class WarmStart:
    """Learned warm start: per-point MLP 16 -> 64 -> 64 -> 3 on the tensor
    cores (no reference counterpart).  Parameters: W1[64][16], W2[64][64],
    b2[64], W3[3][64], b3[3] flattened in that order."""

    def __init__(self, params=None, scales=None):
        self.L = load()
        self.h = C.c_void_p()
        _check(self.L.pbd_warmstart_create(C.byref(self.h)))
        self.n_params = self.L.pbd_warmstart_num_params()
        if params is not None:
            self.set_params(params)
        if scales is not None:
            self.set_scales(scales)

    def close(self):
        if self.h:
            self.L.pbd_warmstart_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params):
        a = _f32(params).ravel()
        _check(self.L.pbd_warmstart_set_params(self.h, _p(a), len(a)))

    def set_scales(self, scales):
        """17 scales: features 0..14 (15 unused), then the output"""
        a = _f32(scales).ravel()
        _check(self.L.pbd_warmstart_set_scales(self.h, _p(a), len(a)))

    def scales(self):
        a = np.zeros(17, np.float32)
        _check(self.L.pbd_warmstart_get_scales(self.h, _p(a), 17))
        return a

    def params(self):
        a = np.zeros(self.n_params, np.float32)
        _check(self.L.pbd_warmstart_get_params(self.h, _p(a), len(a)))
        return a

    def forward(self, x):
        x = _f32(x, (-1, 16))
        y = np.zeros((len(x), 3), np.float32)
        _check(self.L.pbd_warmstart_forward(self.h, _p(x), len(x), _p(y)))
        return y

    def gradients(self, x, t, mask=None):
        x = _f32(x, (-1, 16))
        t = _f32(t, (-1, 3))
        m = None if mask is None else _f32(mask)
        g = np.zeros(self.n_params, np.float32)
        loss = C.c_double()
        _check(self.L.pbd_warmstart_gradients(self.h, _p(x), _p(t), _p(m), len(x), _p(g),
                                              C.byref(loss)))
        return g, loss.value

    def set_gradient(self, g):
        g = _f32(g).ravel()
        _check(self.L.pbd_warmstart_set_gradient(self.h, _p(g), len(g)))

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        _check(self.L.pbd_warmstart_adam(self.h, lr, beta1, beta2, eps))

    def record(self, obj):
        _check(self.L.pbd_warmstart_record(self.h, obj.h))

    def train_step(self, obj, lr=1e-3, want_loss=True):
        loss = C.c_double()
        _check(self.L.pbd_warmstart_train_step(self.h, obj.h, lr,
                                               C.byref(loss) if want_loss else None))
        return loss.value if want_loss else None

    def features(self, obj):
        n = obj.n_points
        x = np.zeros((n, 16), np.float32)
        _check(self.L.pbd_warmstart_features(self.h, obj.h, _p(x)))
        return x

    def predict(self, obj):
        _check(self.L.pbd_warmstart_predict(self.h, obj.h))


def _enc(path):
    return None if path is None else os.fsencode(path)


def _scene_dict(h):
    """copy a pbd_scene's arrays out (scene dict as scenes.py builds them)"""
    L = load()
    d = _Desc()
    prd = C.c_void_p()
    hd, hg = C.c_int(), C.c_int()
    _check(L.pbd_scene_desc(h, C.byref(d), C.byref(prd), C.byref(hd), C.byref(hg)))

    def arr(ptr, n, ct, dt):
        if not ptr or n == 0:
            return np.zeros(0, dt)
        return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ct)), shape=(n,)).astype(dt).copy()

    n, nt, np_ = d.n_points, d.n_tris, d.n_prims
    pl = arr(d.prim_list, 2 * np_, C.c_int, np.int32).reshape(-1, 2)
    n_idx = int((pl[:, 0] + pl[:, 1]).max()) if np_ else 0
    sc = {
        "pos": arr(d.pos, 3 * n, C.c_float, np.float32).reshape(-1, 3),
        "vel": (arr(d.vel, 3 * n, C.c_float, np.float32).reshape(-1, 3) if d.vel
                else np.zeros((n, 3), np.float32)),
        "mass": arr(d.mass, n, C.c_float, np.float32),
        "tri_idx": arr(d.tri_idx, 3 * nt, C.c_int, np.int32).reshape(-1, 3),
        "prim_list": pl,
        "indices": arr(d.indices, n_idx, C.c_int, np.int32),
        "ctype": arr(d.constraint_type, np_, C.c_int, np.int32),
        "rest_length": arr(d.rest_length, np_, C.c_float, np.float32),
        "stiffness": arr(d.stiffness, np_, C.c_float, np.float32),
        "predicted": (arr(prd.value, 3 * n, C.c_float, np.float32).reshape(-1, 3)
                      if prd.value else None),
        "damping": float(d.damping_rate) if hd.value else None,
        "gravity": np.array(list(d.gravity), np.float32) if hg.value else None,
    }
    L.pbd_scene_destroy(h)
    return sc


def read_cache(topol_path, constr_path):
    """the reference's topology / constraint caches (either may be None)"""
    L = load()
    h = C.c_void_p()
    _check(L.pbd_scene_read_cache(_enc(topol_path), _enc(constr_path), C.byref(h)))
    return _scene_dict(h)


def read_txt(topol_path, dist_constr_path, stiffness):
    """the reference's text scene files (topology; distance constraints)"""
    L = load()
    h = C.c_void_p()
    _check(L.pbd_scene_read_txt(_enc(topol_path), _enc(dist_constr_path), float(stiffness),
                                C.byref(h)))
    return _scene_dict(h)


def write_cache(scene, topol_path, constr_path, predicted=None, damping=1.0,
                gravity=(0.0, 0.0, 0.0)):
    """a scene dict written as the reference's two caches"""
    L = load()
    keep = []

    def k(a):
        keep.append(a)
        return _p(a)

    d = _Desc()
    pos = _f32(scene["pos"]).reshape(-1)
    d.n_points = len(pos) // 3
    d.pos = k(pos)
    d.vel = k(_f32(scene["vel"]).reshape(-1)) if scene.get("vel") is not None else None
    d.mass = k(_f32(scene["mass"]))
    tri = _i32(scene.get("tri_idx", np.zeros((0, 3), np.int32))).reshape(-1)
    d.n_tris = len(tri) // 3
    d.tri_idx = k(tri) if len(tri) else None
    ct = _i32(scene.get("ctype", np.zeros(0, np.int32)))
    d.n_prims = len(ct)
    if len(ct):
        d.prim_list = k(_i32(scene["prim_list"]).reshape(-1))
        d.indices = k(_i32(scene["indices"]))
        d.constraint_type = k(ct)
        d.rest_length = k(_f32(scene["rest_length"]))
        d.stiffness = k(_f32(scene["stiffness"]))
    d.damping_rate = damping
    for i in range(3):
        d.gravity[i] = gravity[i]
    prd = None if predicted is None else _f32(predicted).reshape(-1)
    _check(L.pbd_scene_write_cache(C.byref(d), _p(prd), _enc(topol_path), _enc(constr_path)))


def residual_noalloc(d_pos4, n_points, d_dist_idx, d_rest_length, n_dist, d_bend_idx,
                     d_rest_angle, d_hinge_rest, n_bend, d_out, stream=0):
    """pbd_residual_noalloc on caller-owned device pointers (ints)."""
    L = load()
    _check(L.pbd_residual_noalloc(d_pos4, n_points, d_dist_idx or None, d_rest_length or None,
                                  n_dist, d_bend_idx or None, d_rest_angle or None,
                                  d_hinge_rest or None, n_bend, d_out, stream or None))


def ee_test_batch(X, P, thickness):
    """pbd_ee_test_batch: the edge-edge test on n (edge a, edge b) cases.
    X, P: (n, 4, 3) start / predicted a0, a1, b0, b1; thickness: (n,)."""
    L = load()
    X = np.ascontiguousarray(X, np.float32).reshape(-1, 12)
    P = np.ascontiguousarray(P, np.float32).reshape(-1, 12)
    th = np.ascontiguousarray(thickness, np.float32)
    n = len(X)
    hit = np.zeros(n, np.int32)
    tsu = np.zeros((n, 3), np.float32)
    m0 = np.zeros((n, 4), np.float32)
    _check(L.pbd_ee_test_batch(_p(X), _p(P), _p(th), n, _p(hit), _p(tsu), _p(m0)))
    return hit, tsu, m0


VFTEST_EXTENDED, VFTEST_NARROW, VFTEST_CCD, VFTEST_DCD, VFTEST_VF = range(5)


def vf_test_batch(X, P, thickness, mode=VFTEST_EXTENDED):
    """pbd_ccd_vf_test_batch_mode: a vertex-face test (VFTEST_*; default
    ExtendedVFTest) on n (point, triangle) cases.  X, P: (n, 4, 3) start /
    predicted positions; thickness: (n,)."""
    L = load()
    X = np.ascontiguousarray(X, np.float32).reshape(-1, 12)
    P = np.ascontiguousarray(P, np.float32).reshape(-1, 12)
    th = np.ascontiguousarray(thickness, np.float32)
    n = len(X)
    hit = np.zeros(n, np.int32)
    t = np.zeros(n, np.float32)
    w = np.zeros((n, 4), np.float64)
    nrm = np.zeros((n, 3), np.float32)
    _check(L.pbd_ccd_vf_test_batch_mode(_p(X), _p(P), _p(th), n, int(mode), _p(hit), _p(t),
                                        _p(w), _p(nrm)))
    return hit, t, w, nrm
