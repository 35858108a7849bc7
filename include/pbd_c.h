/*
 * pbd_c.h -- C ABI of the GB300 PBD cloth step (libpbd_gb300.so).
 *
 * Drop-in boundary for the reference's cloth-step path
 * (vivienldy/PositionBasedDynamicsOld; paths relative to
 * PositionBasedDynamicsCUDA/PositionBasedDynamicsCUDA/).  The reference is a
 * set of C++ classes linked into one executable; each entry point below
 * replaces the method cited beside it.  Plain pointers and sizes only.
 *
 * Conventions
 *  - Every call returns PBD_OK (0) or a PBD_ERR_* code; pbd_last_error()
 *    gives a one-line message for the calling thread's last failure.
 *  - The library owns device memory.  Host arrays are copied in and out
 *    explicitly; float3 data is 3 floats per point (the reference's AoS).
 *  - Each object owns one CUDA stream; solver, hash and collision calls on an
 *    object are asynchronous on that stream.  Copy-out calls synchronise it.
 *    Handles are not thread-safe.
 *  - massBuffer semantics follow the reference: the value is the inverse
 *    mass in the projection and the gravity gate in advection; 0 pins.
 */
#ifndef PBD_C_H
#define PBD_C_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
    PBD_OK = 0,
    PBD_ERR_ARG = 1,      /* bad argument or size                        */
    PBD_ERR_OOM = 2,      /* device allocation failed                    */
    PBD_ERR_CUDA = 3,     /* CUDA runtime error                          */
    PBD_ERR_TIMEOUT = 4,  /* coloring did not converge in max sweeps     */
    PBD_ERR_OVERFLOW = 5, /* candidate / contact capacity exceeded       */
    PBD_ERR_STATE = 6     /* call out of order (e.g. no coloring yet)    */
};

/* ConstraintType, P/PBD_Basic.cuh:38-43 */
enum { PBD_DISTANCE = 0x001, PBD_BENDING = 0x010, PBD_ANCHOR = 0x100 };
/* SolverType, P/PBD_Basic.cuh:46-51 (only Gauss-Seidel is implemented by the
 * reference and here) */
enum { PBD_JACOBI = 0, PBD_GAUSSSEIDEL = 1 };
/* contact response variants */
enum {
    PBD_RESPONSE_REFERENCE = 0,    /* VFResolveTest/VFResolveNew arithmetic (P/CCD.cpp:1996-2090) */
    PBD_RESPONSE_MASS_WEIGHTED = 1 /* same split, weighted by massBuffer; scale-free degeneracy guard */
};

typedef struct pbd_object pbd_object;
typedef struct pbd_solver pbd_solver;
typedef struct pbd_shs pbd_shs;
typedef struct pbd_colli pbd_colli;

/* Scene description: the buffers of PBDObject and ConstraintPBD
 * (P/PBD_Basic.cuh:89-211). */
typedef struct pbd_object_desc {
    int n_points;
    const float *pos;             /* meshTopol.posBuffer, 3*n_points            */
    const float *vel;             /* velBuffer, 3*n_points (NULL = zero)         */
    const float *mass;            /* massBuffer, n_points                        */
    int n_tris;
    const int *tri_idx;           /* meshTopol.indices, 3*n_tris (may be 0/NULL) */
    int n_prims;
    const int *prim_list;         /* constrPBDBuffer.topol.primList, 2*n_prims   */
    const int *indices;           /* constrPBDBuffer.topol.indices               */
    const int *constraint_type;   /* constraintType, n_prims                     */
    const float *rest_length;     /* restLengthBuffer, n_prims                   */
    const float *stiffness;       /* stiffnessBuffer, n_prims                    */
    const float *rest_angle;      /* bending rest angles, n_prims (NULL = 0)     */
    const float *rest_pos;        /* anchor rest positions, 3*n_prims (NULL)     */
    const int *point_inst;        /* instance id per point (NULL = one cloth)    */
    const int *tri_inst;          /* instance id per triangle (NULL)             */
    float damping_rate;           /* PBDObject::dampingRate                      */
    float gravity[3];             /* PBDObject::gravity                          */
} pbd_object_desc;

const char *pbd_last_error(void);
int pbd_version(void);

/* ---- PBDObject ----------------------------------------------------------- */
/* PBDObject(damping, gravity, ht) + Init(topol, constr) (P/PBD_cuda.cu:650-658):
 * uploads the scene, builds Point2PrimsMap/Prim2PrimsMap on the device. */
int pbd_object_create(const pbd_object_desc *desc, pbd_object **out);
/* PBDObject(damping, gravity, resX, resY, sizeX, sizeY, ht) + SetConstrOption
 * + Init() (P/PBD_cuda.cu:644-869): the reference's own grid, distance
 * stencil and anchors.  stiffness[3] = {distance, bending, anchor}. */
int pbd_object_create_grid(float damping, const float *gravity, int res_x, int res_y,
                           float size_x, float size_y, unsigned ct_mask,
                           const float *stiffness, pbd_object **out);
/* A triangle mesh whose constraints are derived on the device (no reference
 * counterpart: the reference builds its grid stencil on the host,
 * P/PBD_cuda.cu:19-123, or reads Houdini caches). */
typedef struct pbd_mesh_desc {
    int n_points;
    const float *pos;             /* 3*n_points                                  */
    const float *vel;             /* 3*n_points (NULL = zero)                    */
    const float *mass;            /* massBuffer, n_points                        */
    const float *rest_pos;        /* rest shape, 3*n_points (NULL = pos)         */
    int n_tris;
    const int *tri_idx;           /* 3*n_tris                                    */
    unsigned ct_mask;             /* PBD_DISTANCE and/or PBD_BENDING             */
    float stiffness[2];           /* {distance, bending}                         */
    const int *point_inst;        /* instance id per point (NULL = one cloth)    */
    const int *tri_inst;          /* instance id per triangle (NULL)             */
    float damping_rate;
    float gravity[3];
} pbd_mesh_desc;
/* Constraint set of a triangle mesh, derived on the device: a distance
 * constraint on every edge (rest length |p_a - p_b| in float32 from
 * rest_pos) and a dihedral bending constraint (e0, e1, wA, wB) on every edge
 * shared by exactly two triangles (rest angle: the signed dihedral angle of
 * rest_pos in float64, stored as float32).  Edges (a < b) and hinges come
 * out in the order of the key a * n_points + b; a hinge's wA / wB are the
 * vertices opposite the edge in the first / second of its triangles in
 * (slot, triangle) order, e0 -> e1 following wing A's triangle.  With all
 * output pointers NULL only the counts are written; otherwise every
 * non-NULL output gets its values (edges 2 ints, hinges 4 ints each) and
 * both counts must be <= capacity. */
int pbd_mesh_constraints(int n_points, const float *rest_pos, int n_tris, const int *tri_idx,
                         long long capacity, int *n_edges, int *n_hinges, int *edges,
                         float *edge_rest, int *hinges, float *hinge_angle);
/* pbd_mesh_constraints + pbd_object_create: distance prims first (edge
 * order), then bending prims (hinge order), stiffness per type. */
int pbd_object_create_mesh(const pbd_mesh_desc *desc, pbd_object **out);
/* ~PBDObject / freeGPUBuffers (P/PBD_cuda.cu:752-794) */
int pbd_object_destroy(pbd_object *obj);
int pbd_object_sizes(const pbd_object *obj, int *n_points, int *n_tris, int *n_prims);
/* meshTopol.posBuffer / velBuffer / constrPBDBuffer.prdPBuffer copy-out and
 * copy-in (Buffer::LoadToHost / LoadToDevice, P/Buffer.cuh:123-165), 3 floats
 * per point.  Page-locked caller arrays (cudaHostAlloc / cudaHostRegister)
 * are copied directly, others through the object's page-locked staging.
 * get_* blocks until the values are in the caller's array; set_* returns
 * once the caller's array has been read, and the copy is ordered before
 * later work on the object's stream. */
int pbd_object_get_positions(pbd_object *obj, float *pos3);
int pbd_object_get_velocities(pbd_object *obj, float *vel3);
int pbd_object_get_predicted(pbd_object *obj, float *prdp3);
int pbd_object_set_positions(pbd_object *obj, const float *pos3);
int pbd_object_set_velocities(pbd_object *obj, const float *vel3);
int pbd_object_set_predicted(pbd_object *obj, const float *prdp3);
/* positions and velocities together, one synchronisation (the per-frame
 * LoadToHost / LoadToDevice of posBuffer and velBuffer) */
int pbd_object_get_state(pbd_object *obj, float *pos3, float *vel3);
int pbd_object_set_state(pbd_object *obj, const float *pos3, const float *vel3);

/* Stiffness schedule: the factor k a projection applies for stiffness s in
 * sweep iter (0-based) of a projection call.  PBD_SCHEDULE_REFERENCE (the
 * default): k = 1 - (1 - s)^(1/(iter+1)), ProjectContraintsGPUKernel
 * (P/PBD_cuda.cu:1282); PBD_SCHEDULE_UNIT: k = 1, projectConstraintCPU
 * (P/PBD_cuda.cu:1119); PBD_SCHEDULE_DIRECT: k = s.  Solver graphs are
 * recaptured when it changes. */
enum { PBD_SCHEDULE_REFERENCE = 0, PBD_SCHEDULE_UNIT = 1, PBD_SCHEDULE_DIRECT = 2 };
int pbd_object_set_stiffness_schedule(pbd_object *obj, int schedule);
int pbd_object_get_stiffness_schedule(pbd_object *obj, int *schedule);
/* stiffnessBuffer of every prim whose constraintType is in ct_mask set to
 * value (PBDObject::SetConstrOption's per-type stiffness, P/PBD_cuda.cu:
 * 669-673, changed after Init); stream-ordered. */
int pbd_object_set_stiffness(pbd_object *obj, unsigned ct_mask, float value);
/* Attachments: the rest positions of the ANCHOR prims `prims` (the points
 * InitAnchorConstr pins, P/PBD_cuda.cu:125-153, snapped to by the ANCHOR
 * branch, :1298-1305) moved to targets (3 floats each), e.g. every substep
 * for an animated attachment; stream-ordered, the caller's arrays are read
 * before the call returns. */
int pbd_object_set_anchor_targets(pbd_object *obj, int n, const int *prims, const float *targets);
/* the object's CUDA stream (cudaStream_t) */
int pbd_object_stream(pbd_object *obj, void **stream);
int pbd_object_sync(pbd_object *obj);

/* ---- ConstraintPBD ------------------------------------------------------- */
/* EdgeColoring / EdgeColoringGPU (P/PBD_cuda.cu:433-544): speculative greedy
 * coloring on the device, run until every constraint is coloured (the
 * reference runs a fixed count and never reads its flag).  Returns
 * PBD_ERR_TIMEOUT if max_iterations sweeps do not suffice. */
int pbd_constraints_edge_coloring(pbd_object *obj, int max_iterations, int *sweeps);
/* SortEdgesColors (P/PBD_cuda.cu:546-587): stable device sort of prim ids by
 * color; also builds the per-color constraint records the solver reads. */
int pbd_constraints_sort_edges_colors(pbd_object *obj);
/* EvalWorksets (P/PBD_cuda.cu:589-625): (start, count) per color. */
int pbd_constraints_eval_worksets(pbd_object *obj, int *n_worksets);
/* install an externally computed coloring (color per prim id, >= 0) */
int pbd_constraints_set_colors(pbd_object *obj, const int *color);
int pbd_constraints_get_colors(pbd_object *obj, int *color);
int pbd_constraints_get_sorted(pbd_object *obj, int *sorted_color, int *sorted_prim_id);
int pbd_constraints_get_worksets(pbd_object *obj, int *worksets, int cap, int *n);
/* Prim2PrimsMap (P/PBD_cuda.cu:170-202): startNumList (2 per prim) and
 * indices; pass adj NULL to query the total. */
int pbd_constraints_get_adjacency(pbd_object *obj, int *start_num, int *adj,
                                  long long cap, long long *total);
/* relative residual sqrt(sum C^2)/sqrt(sum L^2) of the predicted positions
 * (distance: C=|pa-pb|-l, L=l; bending: C=(theta-theta0)|hinge|,
 * L=rest hinge length).  No reference counterpart (the reference has no
 * convergence measure). */
int pbd_constraints_residual(pbd_object *obj, double *residual);

/* ---- SolverPBD (P/PBD_Basic.cuh:213-259) --------------------------------- */
int pbd_solver_create(pbd_solver **out);
int pbd_solver_destroy(pbd_solver *s);
/* SolverPBD::SetTarget */
int pbd_solver_set_target(pbd_solver *s, pbd_object *obj);
/* SolverPBD::Advect / AdvectGPUKernel (P/PBD_cuda.cu:949-1052) */
int pbd_solver_advect(pbd_solver *s, float dt);
/* SolverPBD::ProjectConstraint / projectConstraintGPU (P/PBD_cuda.cu:1054-1070,
 * 1240-1435): `iterations` colored Gauss-Seidel sweeps over every color
 * (distance, bending and anchor constraints).  Iteration numbering for the
 * stiffness schedule starts at 0 on each call. */
int pbd_solver_project_constraint(pbd_solver *s, int solver_type, int iterations);
/* SolverPBD::ProjectConstraintWithColli (P/PBD_cuda.cu:1072-1088, CPU form
 * 1130-1210): per iteration ii, CCD when ii % 10 == 0 or last, one GS sweep,
 * the collision response, the analytic obstacles. */
int pbd_solver_project_constraint_with_colli(pbd_solver *s, int solver_type, int iterations,
                                             pbd_colli *colli);
/* SolverPBD::Integration / IntegrationGPUKernel (P/PBD_cuda.cu:1437-1518) */
int pbd_solver_integration(pbd_solver *s, float dt);
/* analytic obstacles of ColliWithShpGrd (P/PBD_cuda.cu:1519-1573), applied
 * after every GS iteration when enabled: sphere push-out (the reference's
 * fixed unit sphere, tolerance 0.001) and the ground plane CollideGround. */
int pbd_solver_set_sphere(pbd_solver *s, int enable, const float *center, float radius);
int pbd_solver_set_ground(pbd_solver *s, int enable, float height);
/* one analytic sphere per instance of a batched object (n spheres, 4 floats
 * each: centre xyz, radius), applied like the sphere above to every point of
 * the instance after each GS iteration; n = 0 removes them.  No reference
 * counterpart (the reference simulates one object). */
int pbd_solver_set_instance_spheres(pbd_solver *s, int n, const float *spheres4);
/* whole substeps: Advect, ProjectConstraint[WithColli], Integration, repeated
 * `substeps` times; recorded into a CUDA graph on first use (use_graph=1)
 * and replayed.  colli may be NULL. */
int pbd_solver_step(pbd_solver *s, float dt, int substeps, int iterations, pbd_colli *colli,
                    int use_graph);

/* How a Gauss-Seidel sweep runs: PBD_GS_PER_COLOR launches one kernel per
 * color (any size); PBD_GS_CLUSTER (the resident form) keeps every point in
 * the shared memory of one thread-block cluster of S = 1, 2, 4, 8 or 16
 * blocks (about 14,000 points per block on GB300) for whole sweeps, color
 * phases separated by cluster barriers; PBD_GS_AUTO (default) takes the
 * per-color form.  All give identical results; pbd_solver_autotune picks the
 * fastest form, block size and cluster size for an object.
 * No reference counterpart (the reference launches one kernel per color). */
enum { PBD_GS_AUTO = 0, PBD_GS_PER_COLOR = 1, PBD_GS_CLUSTER = 2 };
int pbd_solver_set_gs_path(pbd_solver *s, int path);
/* the form the next sweep will use (PBD_GS_PER_COLOR or PBD_GS_CLUSTER) */
int pbd_solver_get_gs_path(pbd_solver *s, int *path);

/* Autotuner (no reference counterpart): times `iterations` sweeps (one
 * launch sequence per sweep) replayed `reps` times from a CUDA graph for each
 * launch form that applies -- the per-color launches with 64, 128, 256 and
 * 512 threads per block, and the resident form with every cluster size that
 * holds the object (block = S in the result) -- and keeps the
 * fastest for this solver and object.  The predicted positions are restored;
 * all forms give identical results. */
typedef struct pbd_autotune_result {
    int n;                  /* candidates timed                       */
    int best;               /* index of the one kept                  */
    int path[12];            /* PBD_GS_PER_COLOR / PBD_GS_CLUSTER     */
    int block[12];           /* threads per block; cluster size S     */
    double us_per_sweep[12]; /* GPU time per sweep, microseconds      */
} pbd_autotune_result;
int pbd_solver_autotune(pbd_solver *s, int iterations, int reps, pbd_autotune_result *result);
/* threads per block of the per-color launches (256 until autotuned or set;
 * a multiple of 32 in [32, 512]) */
int pbd_solver_set_gs_block(pbd_solver *s, int block);
int pbd_solver_get_gs_block(pbd_solver *s, int *block);
/* cluster size S of the resident form (0: the largest that holds the object;
 * else 1, 2, 4, 8 or 16); get reports the size a sweep would use, 0 when
 * none holds the object */
int pbd_solver_set_gs_cluster(pbd_solver *s, int size);
int pbd_solver_get_gs_cluster(pbd_solver *s, int *size);

/* kernel launches recorded in the cached pbd_solver_step graph (no
 * reference counterpart; used to report launches per step) */
int pbd_solver_graph_kernels(pbd_solver *s, long long *n);

/* ---- SpatialHashSystem (P/SpatialHashSystem.h:10-96) ---------------------- */
/* SpatialHashSystem(posBuffer, triIdxBuffer, ht, gridCenter, gridSize,
 * cellSize): bounded uniform grid over triangle centroids. */
int pbd_shs_create(pbd_object *obj, const float *grid_center, const int *grid_size,
                   const float *cell_size, pbd_shs **out);
/* Unbounded grid hashed into 2^log2_table buckets; a bucket entry is used
 * only for its own cell, so results equal an unbounded uniform grid. */
int pbd_shs_create_hashed(pbd_object *obj, const float *cell_size, int log2_table,
                          pbd_shs **out);
int pbd_shs_destroy(pbd_shs *shs);
/* Hashed grid only (no reference counterpart; the reference hashes one
 * object): a cell size per instance (3 floats each, n = number of
 * instances), so every batched cloth is binned with the cells it would get
 * alone -- the per-instance hash tables of a batch; n = 0 returns to the one
 * cell size. */
int pbd_shs_set_instance_cells(pbd_shs *shs, int n, const float *cells3);
int pbd_shs_set_grid_center(pbd_shs *shs, const float *center);
int pbd_shs_set_grid_size(pbd_shs *shs, const int *size);
int pbd_shs_set_division(pbd_shs *shs, const float *cell_size);
/* InitSH / UpdateSH (P/SpatialHashSystem.cpp:88-121): bin the triangles by
 * the centroids of the object's predicted positions. */
int pbd_shs_init(pbd_shs *shs);
int pbd_shs_update(pbd_shs *shs);
/* FindNeighbors (P/SpatialHashSystem.cpp:134-187) for one triangle / all
 * triangles (start_num: 2 per triangle). */
int pbd_shs_find_neighbors(pbd_shs *shs, int tri, int *out, int cap, int *n);
int pbd_shs_find_neighbors_all(pbd_shs *shs, int *start_num, int *out, long long cap,
                               long long *total);

/* ---- CollisionSolver (P/CCD_Basic.h:33-135) ------------------------------- */
int pbd_colli_create(pbd_colli **out);
int pbd_colli_destroy(pbd_colli *c);
int pbd_colli_set_target(pbd_colli *c, pbd_object *obj);       /* SetTarget      */
int pbd_colli_set_acce_struct(pbd_colli *c, pbd_shs *shs);     /* SetAcceStruct  */
int pbd_colli_set_thickness(pbd_colli *c, float thickness);    /* SetThickness   */
int pbd_colli_set_iterations(pbd_colli *c, int iterations);    /* SetIterations: response passes */
int pbd_colli_set_response(pbd_colli *c, int mode);            /* PBD_RESPONSE_* */
int pbd_colli_set_capacity(pbd_colli *c, long long candidates, long long contacts);
/* No counterpart in the reference (its detection and projection share one
 * host thread).  on = 1 (default): inside pbd_solver_step and
 * pbd_solver_project_constraint_with_colli, a due detection runs on a
 * low-priority side stream from a copy of the iteration's starting
 * positions, beside that iteration's sweep; the response waits for it.
 * The contacts, and every result, are those of on = 0 (detection, then
 * sweep, on the object's stream). */
int pbd_colli_set_overlap(pbd_colli *c, int on);
/* CCD_SH_Extended (P/CCD.cpp:210-274, 1522-1587): UpdateSH on the predicted
 * positions, then the vertex-face ExtendedVFTest over every distinct
 * (point, neighbour triangle) pair; contacts kept on the device, sorted by
 * (point, face triangle). */
int pbd_colli_ccd_sh_extended(pbd_colli *c);
/* CollisionResolveNew (P/CCD.cpp:372-484, 1874-1994): `iterations` passes of
 * the response over the current contacts; within a pass every contact
 * reads the pass-start positions and each point moves by the mean of its
 * active contacts' corrections. */
int pbd_colli_collision_resolve_new(pbd_colli *c);
/* The older response, CollisionResolve + VFResolve (P/CCD.cpp:2423-2650), on
 * the current contacts: two passes over the contacts in stored order, each
 * applied in place before the next is tested (one GPU thread walks the
 * order, which decides the result); a contact is skipped while its point
 * stays on its starting side at least 2 thickness from the predicted plane;
 * a point closer than that on its side is pushed out by (2h - depth)/2, one
 * that crossed by (depth + 2h)/2 when one of the four points was never
 * resolved or VFCCDTest still finds the crossing.  The per-point resolve
 * counters persist across calls, as the reference's resolveTimes buffer
 * does.  The reference's debug output and cache saves are not reproduced. */
int pbd_colli_collision_resolve_old(pbd_colli *c);
/* copy out (out may be NULL) and optionally zero the resolve counters of
 * pbd_colli_collision_resolve_old, one int per point of the target */
int pbd_colli_resolve_times(pbd_colli *c, int *out, int reset);
/* contactData (P/CCD_Basic.h:12-31) copy-out: ids 4 per contact (i0..i3),
 * face triangle, t, w (4 doubles), n (3 floats); any output may be NULL. */
int pbd_colli_get_contacts(pbd_colli *c, int *ids, int *face, float *t, double *w, float *n,
                           long long cap, long long *count);
/* The free ExtendedVFTest (P/CCD.cpp:1733-1808) on n independent
 * configurations, host arrays in and out: x12/p12 = start / predicted
 * positions of point, f0, f1, f2 (12 floats each per case), thickness per
 * case; outputs hit (0/1), t, w (4 doubles), n (3 floats) per case. */
int pbd_ccd_vf_test_batch(const float *x12, const float *p12, const float *thickness, int n,
                          int *hit, float *t, double *w, float *nrm);
/* The vertex-face tests of the reference's detection drivers: */
enum {
    PBD_VFTEST_EXTENDED = 0, /* ExtendedVFTest (P/CCD.cpp:1733-1808), CCD_SH_Extended  */
    PBD_VFTEST_NARROW = 1,   /* NarrowVFCCDTest (P/CCD.cpp:1810-1872), CCD_SH_Narrow   */
    PBD_VFTEST_CCD = 2,      /* VFCCDTest, type VF (P/CCD.cpp:2308-2421)               */
    PBD_VFTEST_DCD = 3,      /* VFDCDTest (P/CCD.cpp:2265-2306)                        */
    PBD_VFTEST_VF = 4        /* VFTest = VFCCDTest || VFDCDTest (P/CCD.cpp:2229-2263),
                                CCD_SH (P/CCD.cpp:2168-2227)                           */
};
/* pbd_ccd_vf_test_batch with the test chosen by mode (PBD_VFTEST_*).  A
 * miss leaves in t, w and n what the test's last evaluated time wrote, as
 * the reference leaves its Contact. */
int pbd_ccd_vf_test_batch_mode(const float *x12, const float *p12, const float *thickness,
                               int n, int mode, int *hit, float *t, double *w, float *nrm);
/* the narrowphase test of a collision solver's detection (default
 * PBD_VFTEST_EXTENDED, CCD_SH_Extended's): NARROW makes the detection
 * CCD_SH_Narrow (P/CCD.cpp:1588-1731), VF makes it CCD_SH
 * (P/CCD.cpp:2168-2227); the candidate pairs are the same in every mode */
int pbd_colli_set_vf_test(pbd_colli *c, int mode);
/* number of broadphase candidate pairs that reached the narrow phase in
 * the last CCD call, and the overflow word: 1 candidates, 2 contacts, 4 a
 * point with more than 16 incident triangles, 16 hash-search pairs,
 * 32/64/128/256 edge-edge entries / pairs / candidates / contacts, 512 a
 * radix-sort wait that ran out (never expected) */
int pbd_colli_stats(pbd_colli *c, long long *candidates, long long *contacts, int *overflow);
/* The (point, triangle) pairs the last CCD call's hash search handed to
 * the distance filter, in device order: pairs of the reference's candidate
 * set (CCD_SH_Extended, P/CCD.cpp:1541-1586) whose swept boxes lie within
 * 3.61 thicknesses of each other (Euclidean gap between the boxes), the
 * point's own triangles left out.  *n = their count; min(*n, cap) pairs
 * (point, triangle) are written to pairs when it is not NULL. */
int pbd_colli_get_pairs(pbd_colli *c, int *pairs, long long cap, long long *n);

/* ---- edge-edge CCD (declared only by the reference: Contact::EE,
 * P/CCD_Basic.h:14; EEResolve commented out, P/CCD.cpp:925-928) -------------- */
/* Off by default (the reference's step).  On: every CCD pass also finds
 * edge-edge contacts among the target's unique mesh edges -- the coplanarity
 * cubic of ExtendedVFTest in FP64, times 0, its roots in [0, 1] and 1 in
 * ascending order, a hit at the first time the lines of the two edges meet
 * strictly inside both edges closer than 2 * thickness -- and every response
 * pass separates them along their common normal to 2 * thickness on the
 * side they started on, in the same Jacobi sums as the vertex-face
 * contacts.  Solver graphs are recaptured when this changes. */
int pbd_colli_set_edge_edge(pbd_colli *c, int on);
/* the target's unique edges (a < b, 2 ints each) the edge-edge pass uses;
 * edges NULL: count only */
int pbd_colli_ee_edges(pbd_colli *c, int *edges, long long cap, int *n);
/* edge-edge contacts of the last CCD pass, sorted by edge pair: pairs (edge
 * ids, 2 per), ids (a0 a1 b0 b1), tsu (t and the closest-point parameters
 * s on edge a, u on edge b), m0 (unit common normal at t = 0 and the side
 * +1/-1 edge a starts on); any output may be NULL; PBD_ERR_OVERFLOW when a
 * buffer of the pass overflowed. */
int pbd_colli_get_ee_contacts(pbd_colli *c, int *pairs, int *ids, float *tsu, float *m0,
                              long long cap, long long *count);
/* counts of the last edge-edge pass: edge-cell entries, box-overlapping
 * pairs, candidates after the distance bound, contacts */
int pbd_colli_ee_stats(pbd_colli *c, long long *entries, long long *pairs, long long *candidates,
                       long long *contacts);
/* the edge-edge test on n independent configurations (x12 / p12: start /
 * predicted a0, a1, b0, b1, 12 floats per case): hit, tsu (3 floats), m0 (4
 * floats) per case */
int pbd_ee_test_batch(const float *x12, const float *p12, const float *thickness, int n,
                      int *hit, float *tsu, float *m0);

/* ---- the reference's text caches and text scene files ----------------------- */
/* Host-side scene read from the reference's files (no GPU needed). */
typedef struct pbd_scene pbd_scene;
/* IO::ReadTopolFromCache + IO::ReadConstraintFromCache, i.e. what
 * PBDObject::ContinueSimInit reads (P/PBD_Basic.cuh:326-530,
 * P/PBD_cuda.cu:660-667).  Either path may be NULL.  Lines split at '|' with
 * exactly three fields are read by name (Indices, P, primList, velBuffer,
 * massBuffer, dampingRate, gravity; Indices, P, primList, prdPBuffer,
 * restPosBuffer, restLengthBuffer, stiffnessBuffer, constraintType), values
 * converted like stoi / stof; other lines are skipped.  Differences: a
 * trailing '\r' is removed (files written on Windows); a field that does not
 * convert returns PBD_ERR_ARG naming the file and line (the reference
 * throws); a mesh primList entry must be a triangle; a topology without
 * massBuffer gets 1 per point. */
int pbd_scene_read_cache(const char *topol_path, const char *constr_path, pbd_scene **out);
/* IO::ReadTopolFromTxt + IO::ReadDistConstrFromTxt (P/PBD_Basic.cuh:532-660):
 * positions and triangles from the topology file (massBuffer 1, zero
 * velocity), distance constraints with `stiffness` and the reference's powf
 * rest lengths from the constraint file (dist_constr_path may be NULL).
 * Constraints of a second data line follow those of the first (the
 * reference restarts their primList offsets at 0 on every line). */
int pbd_scene_read_txt(const char *topol_path, const char *dist_constr_path, float stiffness,
                       pbd_scene **out);
/* the scene as a pbd_object_desc (pointers into the scene, valid until
 * pbd_scene_destroy); *predicted = the cache's prdPBuffer or NULL; whether
 * the cache held dampingRate / gravity */
int pbd_scene_desc(pbd_scene *s, pbd_object_desc *desc, const float **predicted,
                   int *has_damping, int *has_gravity);
int pbd_scene_destroy(pbd_scene *s);
/* PBDObject::SaveMeshTopol / SaveConstraint (P/PBD_cuda.cu:907-938): the
 * reference's line format, values with 6 significant digits as its output
 * streams print them; predicted may be NULL (positions written); either
 * path may be NULL.  The type field is written as the reference's Windows
 * builds spell it; no reader uses it. */
int pbd_scene_write_cache(const pbd_object_desc *desc, const float *predicted,
                          const char *topol_path, const char *constr_path);
/* PBDObject::ContinueSimInit (P/PBD_cuda.cu:660-667): an object from the two
 * caches, predicted positions from prdPBuffer when present */
int pbd_object_create_from_cache(const char *topol_path, const char *constr_path,
                                 pbd_object **out);
/* the object's current state written as the two caches (SaveMeshTopol and
 * SaveConstraint), so the reference can continue from it */
int pbd_object_save_cache(pbd_object *obj, const char *topol_path, const char *constr_path);

/* ---- allocation-free residual --------------------------------------------- */
/* No counterpart in the reference.  The relative residual of
 * pbd_constraints_residual computed from device buffers the caller owns,
 * without allocating device memory: for callers that cannot let a library
 * call cudaMalloc (an engine that sub-allocates everything from its own
 * arena, code between its allocation phase and a graph capture, a process
 * under a fixed device-memory budget).  Partial sums live in a 1 MiB
 * file-scope device array that every GPU loading the library keeps until
 * exit; calls whose work overlaps on the GPU race on it.  The first call on a
 * device looks the array's address up (make it before any stream capture);
 * a later call looks it up again when the device's context changed (after
 * cudaDeviceReset the library's module, and the array, can be reloaded at
 * another address).
 *   d_pos4       float4 per point (xyz used), 16-byte aligned
 *   d_dist_idx   int2 per distance constraint, d_rest_length float each
 *   d_bend_idx   int4 {e0, e1, wA, wB} per bending constraint, with
 *                d_rest_angle and d_hinge_rest (rest hinge length) each
 *   d_out        3 doubles on the device, 8-byte aligned: residual, sum C^2,
 *                sum L^2
 *   stream       cudaStream_t (NULL = legacy default stream)
 * At most 16,777,216 constraints in total (PBD_ERR_ARG beyond).  A point id
 * outside [0, n_points) is skipped and the residual written as NaN. */
int pbd_residual_noalloc(const float *d_pos4, int n_points, const int *d_dist_idx,
                         const float *d_rest_length, int n_dist, const int *d_bend_idx,
                         const float *d_rest_angle, const float *d_hinge_rest, int n_bend,
                         double *d_out, void *stream);

/* ---- substeps solved to a residual target --------------------------------- */
/* No counterpart in the reference (its substeps run a fixed iteration count,
 * P/PBD_cuda.cu:1308-1435).  The stopping test uses the relative stretch
 * residual sqrt(sum C^2)/sqrt(sum l^2) over the distance constraints
 * (C = |p_a - p_b| - l), FP64. */
int pbd_constraints_residual_stretch(pbd_object *obj, double *residual);

typedef struct pbd_solve_stats {
    long long substeps;     /* substeps solved since the last reset            */
    long long sweeps;       /* GS sweeps they ran                              */
    long long reached;      /* substeps that ended at or below the target      */
    long long reverts;      /* warm starts rejected because the residual rose  */
    double last_residual;   /* residual at the end of the last substep's loop  */
    int last_sweeps;        /* sweeps of the last substep                      */
    double last_r0, last_r1;/* warm start guard of the last substep: residual
                               of the advected positions / after prediction   */
} pbd_solve_stats;

/* `substeps` substeps, each: Advect; [warm start]; colored GS sweeps in
 * chunks of `chunk` (1..32) until the stretch residual is <= target or
 * another chunk would exceed max_sweeps; with colli, a CCD detection starts
 * every chunk, every sweep is followed by the contact response and the
 * analytic obstacles, and the loop ends with one more detection + response;
 * the correction p - p_advected is kept (the warm start's feature);
 * Integration.  Sweep i uses the stiffness exponent 1/(i+1)
 * (P/PBD_cuda.cu:1282).  use_graph = 1 captures the substeps in a CUDA
 * graph whose WHILE nodes run the loop on the device (no host round trip);
 * use_graph = 0 runs the same kernels and reads the loop condition on the
 * host after each chunk. */
int pbd_solver_step_to_residual(pbd_solver *s, float dt, int substeps, pbd_colli *colli,
                                double target, int max_sweeps, int chunk, int use_graph);
int pbd_solver_solve_stats(pbd_solver *s, pbd_solve_stats *stats, int reset);
/* the solve alone on the current predicted positions (no Advect, no
 * Integration, no warm start), host-driven: sweeps in chunks until the
 * stretch residual <= target or max_sweeps; with colli as above.  Records
 * the correction p - p_before; returns the sweeps run and the residual.
 * Used to generate the warm start's training targets. */
int pbd_solver_project_to_residual(pbd_solver *s, pbd_colli *colli, double target,
                                   int max_sweeps, int chunk, int *sweeps, double *residual);
/* kernel nodes of the cached pbd_solver_step_to_residual graph: outside the
 * WHILE bodies (all substeps) and inside one body (one chunk) */
int pbd_solver_residual_graph_kernels(pbd_solver *s, long long *n_outer, long long *n_body);
/* the correction p_final - p_advected of the last solved substep, 3 per point */
int pbd_object_get_correction(pbd_object *obj, float *corr3);
/* overwrite it (e.g. to resume a run: the warm start reads it as a feature) */
int pbd_object_set_correction(pbd_object *obj, const float *corr3);

/* ---- learned warm start ---------------------------------------------------- */
/* No counterpart in the reference.  A per-point MLP 16 -> 64 -> 64 -> 3 (SiLU)
 * predicts the correction the sweeps will apply to the advected positions,
 * in units of the point's mean incident rest length, from 16 features:
 * strains of the first six incident distance constraints, the previous
 * substep's correction, an inverse-mass share, a pinned flag, the dihedral
 * deviations of the first four incident bending constraints and a constant 1.
 * BF16 operands on the tensor cores, FP32 accumulation, FP32 master
 * parameters trained with Adam.  Parameter vector (pbd_warmstart_num_params
 * floats): W1[64][16] (column 15 acts on the constant feature), W2[64][64],
 * b2[64], W3[3][64], b3[3]. */
typedef struct pbd_warmstart pbd_warmstart;
int pbd_warmstart_num_params(void);
int pbd_warmstart_create(pbd_warmstart **out);          /* parameters zero    */
int pbd_warmstart_destroy(pbd_warmstart *w);
int pbd_warmstart_set_params(pbd_warmstart *w, const float *params, int n);  /* resets Adam */
int pbd_warmstart_get_params(pbd_warmstart *w, float *params, int n);
/* 17 positive scales: features 0..14 are multiplied by scales[0..14] before
 * the network (scales[15] is unused: feature 15 is the constant 1) and the
 * network's output is multiplied by scales[16] * lbar; all 1 by default */
int pbd_warmstart_set_scales(pbd_warmstart *w, const float *scales, int n);
int pbd_warmstart_get_scales(pbd_warmstart *w, float *scales, int n);
/* network outputs y (3 per row) of n feature rows x (16 floats each, rounded
 * to BF16; column 15 taken as 1) */
int pbd_warmstart_forward(pbd_warmstart *w, const float *x, int n, float *y);
/* gradient of L = 1/(2 m) sum_{rows with mask != 0} |y - t|^2 (m = rows with
 * mask != 0; mask NULL = all rows) with respect to the parameter vector, and L */
int pbd_warmstart_gradients(pbd_warmstart *w, const float *x, const float *t, const float *mask,
                            int n, float *grad, double *loss);
/* load a gradient (for checking the optimizer) / one Adam step on the
 * current gradient, which is then cleared */
int pbd_warmstart_set_gradient(pbd_warmstart *w, const float *grad, int n);
int pbd_warmstart_adam(pbd_warmstart *w, float lr, float beta1, float beta2, float eps);
/* training on solver trajectories: call pbd_warmstart_record right after
 * Advect (features of the advected positions), solve the substep, then
 * pbd_warmstart_train_step: targets = (p - p_advected)/lbar for the free
 * points, one forward/backward pass over every point of the object and one
 * Adam step (beta 0.9 / 0.999, eps 1e-8); loss may be NULL (no sync). */
int pbd_warmstart_record(pbd_warmstart *w, pbd_object *obj);
int pbd_warmstart_train_step(pbd_warmstart *w, pbd_object *obj, float lr, double *loss);
/* One training substep on the solver's object, all on the device except the
 * loop conditions: Advect; features of the advected state; the plain solve
 * to the residual target (as pbd_solver_step_to_residual, collisions
 * included); one forward/backward pass + Adam step on (features, plain
 * correction).  on_policy = 0: the trajectory continues from the plain
 * solve.  on_policy = 1: the advected state is solved again from the
 * (just updated) network's prediction, guard included, and the trajectory
 * continues from that solve, so later substeps are drawn from the states the
 * warm-started solver visits.  Then the correction record and Integration.
 * loss may be NULL. */
int pbd_solver_train_substep(pbd_solver *s, pbd_warmstart *w, float dt, pbd_colli *colli,
                             double target, int max_sweeps, int chunk, float lr, int on_policy,
                             double *loss);
/* features (16 floats per point, BF16 values) of the object's predicted positions */
int pbd_warmstart_features(pbd_warmstart *w, pbd_object *obj, float *x);
/* apply the prediction to the object's predicted positions (test hook) */
int pbd_warmstart_predict(pbd_warmstart *w, pbd_object *obj);
/* use the network in pbd_solver_step_to_residual (NULL = plain sweeps);
 * an accepted prediction is followed by at least min_sweeps sweeps (they
 * remove the prediction's small-scale error before it reaches the
 * velocities) */
int pbd_solver_set_warmstart(pbd_solver *s, pbd_warmstart *w, int min_sweeps);

#ifdef __cplusplus
}
#endif
#endif
