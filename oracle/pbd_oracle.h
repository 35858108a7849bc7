/*
 * pbd_oracle.h -- CPU restatement of the reference PBD cloth step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA
 * implementation in positionbaseddynamicsold_gb300/: only tests/, the smoke
 * check in __graft_entry__.py and the cpu_baseline leg of bench.py may load it.
 * Nothing on the product path links or calls it.
 *
 * Every routine restates one function of the reference
 * (vivienldy/PositionBasedDynamicsOld, paths relative to
 * PositionBasedDynamicsCUDA/PositionBasedDynamicsCUDA/) and cites it.
 * Parity pin: tests/test_oracle_golden.py checks these routines against
 * fixtures produced by the reference's own code compiled from its sources
 * (tests/golden/make_golden.py drives oracle/ref_adapter.cpp).
 *
 * Layout conventions follow the reference: positions/velocities are float3
 * AoS (3 floats per point), primList is int2 (start, count) into `indices`,
 * colorWorksets is int2 (start, count) into sortedPrimId.
 *
 * Compile with -ffp-contract=off: the reference's host code performs
 * plain IEEE float operations (no fused multiply-add).
 */
#ifndef PBD_ORACLE_H
#define PBD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Distance() spelled as powf like the reference (1) or as sqrtf of the
 * squared sum like the CUDA kernels (0, default). */
void orc_set_pow_distance(int on);
/* host threads for the loops whose iterations are independent (default 1;
 * results do not depend on the count); orc_get_threads returns 1 when the
 * library was built without OpenMP */
void orc_set_threads(int n);
int orc_get_threads(void);

/* constraint type bits, P/PBD_Basic.cuh:38-43 */
#define ORC_DISTANCE 0x001
#define ORC_BENDING 0x010
#define ORC_ANCHOR 0x100

/* ------------------------------------------------------------------ */
/* constraint graph and coloring                                        */
/* ------------------------------------------------------------------ */

/* GenePoint2PrimsMap + GenePrim2PrimsMap (P/PBD_cuda.cu:155-202).
 * adj_start_num: int2 per prim (start, count); adj_idx: neighbor prim ids.
 * Pass adj_idx == NULL to only count; returns total neighbor entries. */
int64_t orc_prim2prims(int n_prims, const int *prim_list, const int *indices,
                       int n_points, int *adj_start_num, int *adj_idx);

/* AssignColorsGPU (P/PBD_cuda.cu:313-372), one sweep over all prims. */
void orc_assign_colors(int n_prims, const int *adj_start_num, const int *adj_idx,
                       const int *color, int *prd_color);

/* ResolveConflictsGPU (P/PBD_cuda.cu:374-431), one sweep; returns the
 * conflict flag (non-zero if any prim kept its speculative color rejected). */
int orc_resolve_conflicts_gpu(int n_prims, const int *prim_list,
                              const int *adj_start_num, const int *adj_idx,
                              int *color, const int *prd_color);

/* ResolveConflictsCPU (P/PBD_cuda.cu:256-310): stops the sweep at the first
 * conflict. */
int orc_resolve_conflicts_cpu(int n_prims, const int *prim_list,
                              const int *adj_start_num, const int *adj_idx,
                              int *color, const int *prd_color);

/* EdgeColoringGPU schedule (P/PBD_cuda.cu:487-544): assign+resolve sweeps
 * until no conflict or max_iters.  color/prd_color must be initialised
 * (-1 = uncoloured).  Returns the number of sweeps run. */
int orc_edge_coloring_gpu(int n_prims, const int *prim_list,
                          const int *adj_start_num, const int *adj_idx,
                          int *color, int *prd_color, int max_iters);

/* EdgeColoringCPU schedule (P/PBD_cuda.cu:448-485) with an early exit once
 * a sweep accepts every prim.  Returns sweeps run. */
int orc_edge_coloring_cpu(int n_prims, const int *prim_list,
                          const int *adj_start_num, const int *adj_idx,
                          int *color, int *prd_color, int max_iters);

/* SortEdgesColors (P/PBD_cuda.cu:546-587): stable sort of (color, prim id),
 * in place on both arrays. */
void orc_sort_edges_colors(int n, int *color, int *sorted_prim_id);

/* EvalWorksets (P/PBD_cuda.cu:589-625) as run-length encoding of the sorted
 * colors; worksets gets 2 ints per run.  Returns the number of runs. */
int orc_eval_worksets(int n, const int *sorted_color, int *worksets);

/* ------------------------------------------------------------------ */
/* solver step                                                          */
/* ------------------------------------------------------------------ */

typedef struct orc_constraints {
    int n_prims;
    const int *prim_list;     /* 2 per prim: start, count            */
    const int *indices;       /* point ids                            */
    const int *ctype;         /* ORC_DISTANCE / ORC_BENDING / ORC_ANCHOR */
    const float *rest_length; /* per prim (distance)                  */
    const float *stiffness;   /* per prim                             */
    const float *rest_angle;  /* per prim (bending), may be NULL      */
    const float *rest_pos;    /* 3 per prim (anchor), may be NULL     */
} orc_constraints;

/* AdvectGPUKernel (P/PBD_cuda.cu:949-979).  damp_pow = powf(dampingRate, dt)
 * evaluated once by the caller. */
void orc_advect_gpu(int n, float dt, float damp_pow, const float *gravity,
                    const float *mass, float *vel, float *prdp, const float *pos);

/* advectCPU (P/PBD_cuda.cu:997-1009): ignores mass and damping. */
void orc_advect_cpu(int n, float dt, const float *gravity, float *vel,
                    float *prdp, const float *pos);

/* IntegrationGPUKernel / integrationCPU (P/PBD_cuda.cu:1453-1482). */
void orc_integrate(int n, float dt, float *vel, const float *prdp, float *pos);

/* projectConstraintGPU (P/PBD_cuda.cu:1240-1435): for each iteration, for
 * each workset (colour) in order, apply every constraint of the workset.
 * Every constraint of a workset is processed (the reference's integer
 * division launch shortfall at P/PBD_cuda.cu:1336-1337 is not reproduced).
 * Distance: ProjectContraintsGPUKernel arithmetic.  Bending: dihedral
 * constraint (no reference code; see orc_bending_project).  Anchor: snap to
 * rest_pos.  A distance constraint whose two inverse masses sum to zero is
 * skipped (the reference divides by zero there). */
void orc_project_colored(const orc_constraints *c, const int *sorted_prim_id,
                         int n_worksets, const int *worksets, int iter_begin,
                         int iter_end, const float *mass, float *prdp,
                         int bending_fp64);

/* Stiffness schedule of the colored GS: 0 = k = 1 - (1-s)^(1/(iter+1))
 * (P/PBD_cuda.cu:1282, the default), 1 = k = 1 (P/PBD_cuda.cu:1119),
 * 2 = k = s.  Process-wide. */
void orc_set_stiffness_schedule(int mode);

/* One constraint of the colored GS, iteration `iter` (stiffness schedule
 * above). */
void orc_project_one(const orc_constraints *c, int prim, int iter,
                     const float *mass, float *prdp, int bending_fp64);

/* projectConstraintCPU (P/PBD_cuda.cu:1090-1127): sequential GS over every
 * 2-point prim in id order, k = 1, then ColliWithShpGrd per iteration. */
void orc_project_cpu(const orc_constraints *c, int iterations,
                     const float *mass, float *prdp, int n_points,
                     const float *sphere_center, float sphere_radius);
/* one sequential pass of projectConstraintCPU's loop over prims [p0, p1) */
void orc_project_cpu_range(const orc_constraints *c, const float *mass, float *prdp,
                           int p0, int p1);

/* ColliWithShpGrd (P/PBD_cuda.cu:1519-1573). */
void orc_colli_sphere(int n, float *prdp, const float *center, float radius);

/* Dihedral bending projection of the four points p[0..3]
 * (p0,p1 = hinge edge, p2,p3 = opposite points), signed angle with
 * gradients of Bridson, Marino & Fedkiw 2003 inside the PBD projection of
 * Mueller et al. 2007.  Float version: same operation order as the CUDA
 * kernel.  Returns 1 if a correction was applied. */
int orc_bending_project_f32(float *p0, float *p1, float *p2, float *p3,
                            const float *w, float rest_angle, float k);
int orc_bending_project_f64(double *p0, double *p1, double *p2, double *p3,
                            const double *w, double rest_angle, double k);
/* Signed dihedral angle of the hinge (p0,p1) with wings p2, p3. */
double orc_dihedral_angle(const double *p0, const double *p1, const double *p2,
                          const double *p3);

/* Relative constraint residual sqrt(sum C^2)/sqrt(sum L^2): distance
 * C = |pa-pb| - l, L = l; bending C = (theta - theta0)*|hinge|,
 * L = rest hinge length (hinge_rest per prim, may be NULL -> current).
 * FP64 accumulation. */
double orc_residual(const orc_constraints *c, const float *prdp,
                    const float *hinge_rest, double *num_out, double *den_out);

/* ------------------------------------------------------------------ */
/* broadphase (SpatialHashSystem)                                       */
/* ------------------------------------------------------------------ */

typedef struct orc_grid {
    float start[3];   /* m_girdStartPos                                  */
    float cell[3];    /* m_cellSize                                      */
    int size[3];      /* m_gridSize (bounded mode)                       */
    int bounded;      /* 1: reference bounded grid; 0: unbounded grid      */
} orc_grid;

/* InitSH (P/SpatialHashSystem.cpp:88-98): start = center - size*cell/2. */
void orc_grid_init(orc_grid *g, const float *center, const int *size,
                   const float *cell, int bounded);

/* evalTriCentroids + calcGridPosCPU (P/SpatialHashSystem.cpp:276-298,
 * 391-399): cell coordinates of each triangle centroid. */
void orc_tri_cells(const orc_grid *g, int n_tris, const int *tri_idx,
                   const float *pos, int *cell_xyz);

/* calcGridHashCPU (P/SpatialHashSystem.cpp:401-413): -1 outside. */
int orc_cell_hash(const orc_grid *g, const int *cell_xyz);

/* UpdateSH + FindNeighbors for every triangle (P/SpatialHashSystem.cpp:
 * 100-121, 134-187, 326-389) on a fresh grid: neighbor lists in the
 * reference's order (27 cells z,y,x; within a cell the stable sort order).
 * out_start_num: 2 ints per triangle.  Pass out_idx NULL to count. */
int64_t orc_find_neighbors_all(const orc_grid *g, int n_tris, const int *tri_idx,
                               const float *pos, int *out_start_num, int *out_idx);

/* ------------------------------------------------------------------ */
/* narrowphase (CCD)                                                    */
/* ------------------------------------------------------------------ */

typedef struct orc_contact {
    int v, f0, f1, f2;  /* ctxIndices i0..i3                 */
    int face;           /* triangle id of the face           */
    float t;            /* Contact::t                        */
    double w[4];        /* Contact::w                        */
    float n[3];         /* Contact::n                        */
} orc_contact;

/* solve_cubic / newtons_method / solve_quadratic (P/CCD.cpp:48-113). */
int orc_solve_cubic(double a, double b, double c, double d, double x[3]);
int orc_solve_quadratic(double a, double b, double c, double x[2]);
double orc_newtons_method(double a, double b, double c, double d, double x0,
                          int init_dir);

/* free ExtendedVFTest (P/CCD.cpp:1733-1808).  x[12] = start positions of
 * vertex, p1, p2, p3; p[12] = predicted positions.  Returns 1 on hit and
 * fills t, w, n. */
int orc_extended_vf_test(const float *x, const float *p, float thickness,
                         int i0, int i1, int i2, int i3, orc_contact *ct);

/* free NarrowVFCCDTest (P/CCD.cpp:1810-1872). */
int orc_narrow_vf_ccd_test(const float *x, const float *p, float thickness,
                           int i0, int i1, int i2, int i3, orc_contact *ct);
/* free VFCCDTest with type VF (P/CCD.cpp:2308-2421), VFDCDTest
 * (P/CCD.cpp:2265-2306) and VFTest = VFCCDTest || VFDCDTest
 * (P/CCD.cpp:2229-2263) */
int orc_vf_ccd_test(const float *x, const float *p, float thickness, int i0, int i1, int i2,
                    int i3, orc_contact *ct);
int orc_vf_dcd_test(const float *x, const float *p, float thickness, int i0, int i1, int i2,
                    int i3, orc_contact *ct);
int orc_vf_test(const float *x, const float *p, float thickness, int i0, int i1, int i2, int i3,
                orc_contact *ct);

/* free CCD_SH_Extended (P/CCD.cpp:1522-1587) restated loop for loop:
 * triangles in id order, their points, neighbor triangles, IsDuplicated
 * de-duplication (P/CCD.cpp:132-147).  Contacts come out in the
 * reference's order.  Returns the number of contacts (<= cap written). */
int64_t orc_ccd_sh_extended_ref(const orc_grid *g, int n_tris, const int *tri_idx,
                                const float *pos, const float *prdp,
                                float thickness, orc_contact *out, int64_t cap);

/* The same loop restricted to triangles [tri_begin, tri_end) of the outer
 * loop (the neighbour search still bins every triangle): a slice of one
 * CCD pass, used to time the reference path in bounded pieces. */
/* UpdateSH's table over every triangle (binned by prdp), and the ranged
 * detection below run against it (a detection pass = one build, then its
 * triangle ranges). */
typedef struct orc_sh_table orc_sh_table;
orc_sh_table *orc_sh_build(const orc_grid *g, int n_tris, const int *tri_idx, const float *prdp);
void orc_sh_free(orc_sh_table *t);
int64_t orc_ccd_sh_extended_ref_range_tab(const orc_grid *g, const orc_sh_table *t, int n_tris,
                                          const int *tri_idx, const float *pos,
                                          const float *prdp, float thickness, int tri_begin,
                                          int tri_end, orc_contact *out, int64_t cap);
/* the same on orc_get_threads() threads: consecutive triangle slices
 * detected in parallel, then stored in loop order with the duplicate scan
 * (the contact list equals the sequential one) */
int64_t orc_ccd_sh_extended_ref_range_tab_mt(const orc_grid *g, const orc_sh_table *t,
                                             int n_tris, const int *tri_idx, const float *pos,
                                             const float *prdp, float thickness, int tri_begin,
                                             int tri_end, orc_contact *out, int64_t cap);
int64_t orc_ccd_sh_extended_ref_range(const orc_grid *g, int n_tris, const int *tri_idx,
                                      const float *pos, const float *prdp, float thickness,
                                      int tri_begin, int tri_end, orc_contact *out, int64_t cap);

/* Same contact set, computed once per distinct (point, triangle) pair
 * using point -> incident triangle lists (the evaluation order the CUDA
 * path uses); contacts sorted by (point, face triangle).  inst (may be
 * NULL) restricts pairs to points and triangles of the same instance. */
/* the test orc_ccd_vf_pairs runs on each pair (0 ExtendedVFTest, default;
 * 1 NarrowVFCCDTest; 2 VFCCDTest; 3 VFDCDTest; 4 VFTest), process-wide */
void orc_set_vf_test(int mode);
int64_t orc_ccd_vf_pairs(const orc_grid *g, int n_points, int n_tris,
                         const int *tri_idx, const int *tri_inst,
                         const int *point_inst, const float *pos,
                         const float *prdp, float thickness, orc_contact *out,
                         int64_t cap);

/* free VFResolveTest (P/CCD.cpp:1996-2032). */
int orc_vf_resolve_test(const float *x, const float *p, float thickness);

/* free VFResolveNew (P/CCD.cpp:2034-2090), in place on p[12]. */
void orc_vf_resolve_new(const float *x, float *p, float thickness);

/* free CollisionResolveNew (P/CCD.cpp:1874-1994): `iterations` sequential
 * passes over the contacts in order. */
void orc_collision_resolve_ref(int n_contacts, const orc_contact *cts,
                               const float *pos, float *prdp, int iterations,
                               float thickness);

/* Contact response as the CUDA path runs it: per pass every contact
 * evaluates VFResolveTest on the pass-start positions and, if active,
 * computes its four corrections; each point then moves by the mean of the
 * corrections of its active contacts, summed in 2^-32 m fixed point so the
 * result does not depend on contact order.  mass_weighted=0 uses the
 * reference split (VFResolveNew); 1 uses the inverse-mass split (see the
 * CUDA kernel for the formula). */
/* CollisionResolveNew's sequential in-place pass with the correction of
 * orc_vf_resolve_deltas (mass_weighted 0: the reference's; 1: inverse-mass
 * split, scale-free guard) */
void orc_collision_resolve_seq(int n_contacts, const orc_contact *cts, const float *pos,
                               float *prdp, const float *mass, int iterations,
                               float thickness, int mass_weighted);
/* the older response CollisionResolve + VFResolve (P/CCD.cpp:2423-2650):
 * two sequential in-place passes; resolve_times (one counter per point,
 * kept by the caller between calls) gates the crossing case */
void orc_collision_resolve_old(int n_contacts, const orc_contact *cts, const float *pos,
                               float *prdp, int *resolve_times, float thickness);
void orc_collision_resolve_jacobi(int n_points, int n_contacts,
                                  const orc_contact *cts, const float *pos,
                                  float *prdp, const float *mass, int iterations,
                                  float thickness, int mass_weighted);

/* The four corrections of one contact (Jacobi form); returns 1 if active. */
int orc_vf_resolve_deltas(const float *x, const float *p, const float *w_mass,
                          float thickness, int mass_weighted, float *delta);

/* ------------------------------------------------------------------ */
/* whole substeps                                                        */
/* ------------------------------------------------------------------ */

typedef struct orc_colli_params {
    int enabled;
    orc_grid grid;
    float thickness;
    int resolve_passes;     /* passes of the response per GS iteration   */
    int mass_weighted;
    int ccd_every;          /* CCD when ii % ccd_every == 0 or last (10)  */
    int n_tris;
    const int *tri_idx;
    const int *tri_inst;    /* may be NULL */
    const int *point_inst;  /* may be NULL */
    int64_t contact_cap;
} orc_colli_params;

/* ExtendedVFTest entirely in FP64 with roots polished to 1e-14: the
 * accuracy yardstick the reference-arithmetic results are measured
 * against (t, w and the hit decision). */
int orc_extended_vf_test_f64(const float *x, const float *p, float thickness, int i0, int i1,
                             int i2, int i3, orc_contact *ct);

/* Edge-edge CCD (no reference arithmetic: Contact::EE is declared in
 * P/CCD_Basic.h:14, EEResolve is commented out in P/CCD.cpp:925-928).
 * x, p: start / predicted positions of a0, a1, b0, b1.  Times 0, the
 * coplanarity cubic's roots in [0, 1] and 1 in ascending order (as
 * ExtendedVFTest); a hit is the first time the lines of the two edges meet
 * strictly inside both edges closer than 2 * thickness.  m0 = the unit
 * common normal of the edges at t = 0, m0[3] = the side (+1/-1) edge A
 * starts on along it.  Edges parallel at t = 0 give no hit. */
typedef struct orc_ee_hit {
    float t, s, u;
    float m0[4];
} orc_ee_hit;
int orc_ee_test(const float *x, const float *p, float thickness, orc_ee_hit *hit);
/* every pair i < j of edges (2 point ids each) that share no point and lie
 * in one instance, tested with orc_ee_test; returns the number of hits
 * (stored up to cap, in (i, j) order) */
int64_t orc_ccd_ee_brute(int n_edges, const int *edges, const int *point_inst, const float *x,
                         const float *p, float thickness, int *pairs, orc_ee_hit *hits,
                         int64_t cap);
/* corrections of one edge-edge contact at the predicted positions p (a0,
 * a1, b0, b1), inverse masses wm: the segments' closest points are pushed
 * apart along the predicted common normal (oriented like m0) until they
 * are 2 * thickness apart on the m0[3] side, split by wm and the closest-
 * point weights.  Returns 0 when the pair needs no correction. */
int orc_ee_resolve_deltas(const float *p, const float *wm, const float *m0s, float thickness,
                          float *delta);
/* orc_collision_resolve_jacobi over vertex-face and edge-edge contacts
 * together (one set of fixed-point sums per pass) */
void orc_collision_resolve_jacobi_ee(int n_points, int n_vf, const orc_contact *vf,
                                     int n_ee, const int *ee_ids, const float *ee_m0,
                                     const float *pos, float *prdp, const float *mass,
                                     int iterations, float thickness, int mass_weighted);

/* GPU-semantics substep: advect, iterations x (optional CCD, colored GS
 * sweep, optional response), integrate.  Returns contacts found in the
 * last CCD pass (or 0). */
int64_t orc_substep_gpu(int n_points, const orc_constraints *c,
                        const int *sorted_prim_id, int n_worksets,
                        const int *worksets, int iterations, float dt,
                        float damping, const float *gravity, const float *mass,
                        float *pos, float *vel, float *prdp, int bending_fp64,
                        const orc_colli_params *colli);
/* orc_substep_gpu with the GPU path's analytic obstacles after every sweep
 * (and its response): sphere4 = {centre xyz, radius} or NULL (the sphere
 * push of ColliWithShpGrd), the ground plane y = ground_h when ground_on */
int64_t orc_substep_gpu_obst(int n_points, const orc_constraints *c,
                             const int *sorted_prim_id, int n_worksets,
                             const int *worksets, int iterations, float dt,
                             float damping, const float *gravity, const float *mass,
                             float *pos, float *vel, float *prdp, int bending_fp64,
                             const orc_colli_params *colli, const float *sphere4,
                             int ground_on, float ground_h);
void orc_ground(int n, float *prdp, float h);

/* Reference CPU substep (P/PBD_cuda.cu:997-1009 advectCPU,
 * 1130-1210 projectConstraintWithColliCPU or 1090-1127 projectConstraintCPU,
 * 1453-1465 integrationCPU) with the reference's triangle-ordered CCD
 * (P/CCD.cpp:210-274) and one sequential response pass per iteration
 * (P/CCD.cpp:372-484).  Used as the CPU baseline. */
int64_t orc_substep_cpu_ref(int n_points, const orc_constraints *c, int iterations,
                            float dt, const float *gravity, const float *mass,
                            float *pos, float *vel, float *prdp,
                            const orc_colli_params *colli,
                            const float *sphere_center, float sphere_radius);

#ifdef __cplusplus
}
#endif
#endif
