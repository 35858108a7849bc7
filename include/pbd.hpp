// pbd.hpp -- header-only C++ classes over the C ABI of libpbd_gb300.so.
//
// Named like the reference's classes (vivienldy/PositionBasedDynamicsOld,
// PositionBasedDynamicsCUDA/PositionBasedDynamicsCUDA/PBD_Basic.cuh:145-259,
// SpatialHashSystem.h:10-96, CCD_Basic.h:33-135) so that a driver written
// against the reference ports by renaming the include.  Every method is one C
// ABI call; failures throw pbd::Error with the library's message.
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "pbd_c.h"

namespace pbd {

struct Error : std::runtime_error {
    int code;
    Error(int c, const char *m) : std::runtime_error(m ? m : "pbd error"), code(c) {}
};

inline void check(int rc) {
    if (rc != PBD_OK) throw Error(rc, pbd_last_error());
}

// PBDObject + ConstraintPBD (PBD_Basic.cuh:97-211)
class PBDObject {
public:
    explicit PBDObject(const pbd_object_desc &d) { check(pbd_object_create(&d, &h_)); }
    // PBDObject(dampingRate, gravity, resX, resY, sizeX, sizeY, ht) +
    // SetConstrOption(ct, stiffness) + Init()
    PBDObject(float damping, const float gravity[3], int res_x, int res_y, float size_x,
              float size_y, unsigned ct, const float stiffness[3]) {
        check(pbd_object_create_grid(damping, gravity, res_x, res_y, size_x, size_y, ct,
                                     stiffness, &h_));
    }
    ~PBDObject() { pbd_object_destroy(h_); }
    PBDObject(const PBDObject &) = delete;
    PBDObject &operator=(const PBDObject &) = delete;

    pbd_object *handle() const { return h_; }
    int points() const {
        int n = 0;
        check(pbd_object_sizes(h_, &n, nullptr, nullptr));
        return n;
    }
    // ConstraintPBD::EdgeColoring / SortEdgesColors / EvalWorksets
    int EdgeColoring(int iterations) {
        int sweeps = 0;
        check(pbd_constraints_edge_coloring(h_, iterations, &sweeps));
        return sweeps;
    }
    void SortEdgesColors() { check(pbd_constraints_sort_edges_colors(h_)); }
    int EvalWorksets() {
        int n = 0;
        check(pbd_constraints_eval_worksets(h_, &n));
        return n;
    }
    // Buffer::LoadToHost of meshTopol.posBuffer / velBuffer / prdPBuffer
    std::vector<float> Positions() { return get(pbd_object_get_positions); }
    std::vector<float> Velocities() { return get(pbd_object_get_velocities); }
    std::vector<float> Predicted() { return get(pbd_object_get_predicted); }
    void SetPositions(const std::vector<float> &v) { check(pbd_object_set_positions(h_, v.data())); }
    double Residual() {
        double r = 0;
        check(pbd_constraints_residual(h_, &r));
        return r;
    }

private:
    std::vector<float> get(int (*fn)(pbd_object *, float *)) {
        std::vector<float> out(3 * (size_t)points());
        check(fn(h_, out.data()));
        return out;
    }
    pbd_object *h_ = nullptr;
};

// SpatialHashSystem (SpatialHashSystem.h:10-96)
class SpatialHashSystem {
public:
    SpatialHashSystem(PBDObject &obj, const float center[3], const int size[3],
                      const float cell[3]) {
        check(pbd_shs_create(obj.handle(), center, size, cell, &h_));
    }
    SpatialHashSystem(PBDObject &obj, const float cell[3], int log2_table) {
        check(pbd_shs_create_hashed(obj.handle(), cell, log2_table, &h_));
    }
    ~SpatialHashSystem() { pbd_shs_destroy(h_); }
    SpatialHashSystem(const SpatialHashSystem &) = delete;
    SpatialHashSystem &operator=(const SpatialHashSystem &) = delete;
    void SetGridCenter(const float c[3]) { check(pbd_shs_set_grid_center(h_, c)); }
    void SetGridSize(const int s[3]) { check(pbd_shs_set_grid_size(h_, s)); }
    void SetDivision(const float c[3]) { check(pbd_shs_set_division(h_, c)); }
    void InitSH() { check(pbd_shs_init(h_)); }
    void UpdateSH() { check(pbd_shs_update(h_)); }
    std::vector<int> FindNeighbors(int tri) {
        int n = 0;
        check(pbd_shs_find_neighbors(h_, tri, nullptr, 0, &n));
        std::vector<int> out(n);
        check(pbd_shs_find_neighbors(h_, tri, out.data(), n, &n));
        return out;
    }
    pbd_shs *handle() const { return h_; }

private:
    pbd_shs *h_ = nullptr;
};

// CollisionSolver (CCD_Basic.h:33-135)
class CollisionSolver {
public:
    CollisionSolver() { check(pbd_colli_create(&h_)); }
    ~CollisionSolver() { pbd_colli_destroy(h_); }
    CollisionSolver(const CollisionSolver &) = delete;
    CollisionSolver &operator=(const CollisionSolver &) = delete;
    void SetTarget(PBDObject &o) { check(pbd_colli_set_target(h_, o.handle())); }
    void SetAcceStruct(SpatialHashSystem &s) { check(pbd_colli_set_acce_struct(h_, s.handle())); }
    void SetThickness(float t) { check(pbd_colli_set_thickness(h_, t)); }
    void SetIterations(int i) { check(pbd_colli_set_iterations(h_, i)); }
    void SetResponse(int mode) { check(pbd_colli_set_response(h_, mode)); }
    void SetOverlap(bool on) { check(pbd_colli_set_overlap(h_, on ? 1 : 0)); }
    // CollisionResolve (the older response), counters kept across calls
    void CollisionResolve() { check(pbd_colli_collision_resolve_old(h_)); }
    // PBD_VFTEST_*: which driver's narrowphase test the detection runs
    void SetVFTest(int mode) { check(pbd_colli_set_vf_test(h_, mode)); }
    void CCD_SH_Extended() { check(pbd_colli_ccd_sh_extended(h_)); }
    void CollisionResolveNew() { check(pbd_colli_collision_resolve_new(h_)); }
    long long ContactCount() {
        long long n = 0;
        check(pbd_colli_get_contacts(h_, nullptr, nullptr, nullptr, nullptr, nullptr, 0, &n));
        return n;
    }
    pbd_colli *handle() const { return h_; }

private:
    pbd_colli *h_ = nullptr;
};

// SolverPBD (PBD_Basic.cuh:213-259)
class SolverPBD {
public:
    SolverPBD() { check(pbd_solver_create(&h_)); }
    ~SolverPBD() { pbd_solver_destroy(h_); }
    SolverPBD(const SolverPBD &) = delete;
    SolverPBD &operator=(const SolverPBD &) = delete;
    void SetTarget(PBDObject &o) { check(pbd_solver_set_target(h_, o.handle())); }
    void Advect(float dt) { check(pbd_solver_advect(h_, dt)); }
    void ProjectConstraint(int solver_type, int iterations) {
        check(pbd_solver_project_constraint(h_, solver_type, iterations));
    }
    void ProjectConstraintWithColli(int solver_type, int iterations, CollisionSolver &c) {
        check(pbd_solver_project_constraint_with_colli(h_, solver_type, iterations, c.handle()));
    }
    void Integration(float dt) { check(pbd_solver_integration(h_, dt)); }
    void Step(float dt, int substeps, int iterations, CollisionSolver *c, bool graph = true) {
        check(pbd_solver_step(h_, dt, substeps, iterations, c ? c->handle() : nullptr, graph));
    }
    // no reference counterparts below: substeps solved to a stretch-residual
    // target (device-side loop in a CUDA graph), the learned warm start and
    // the launch-form autotuner
    void StepToResidual(float dt, int substeps, CollisionSolver *c, double target,
                        int max_sweeps, int chunk, bool graph = true) {
        check(pbd_solver_step_to_residual(h_, dt, substeps, c ? c->handle() : nullptr, target,
                                          max_sweeps, chunk, graph));
    }
    pbd_solve_stats SolveStats(bool reset = false) {
        pbd_solve_stats st;
        check(pbd_solver_solve_stats(h_, &st, reset));
        return st;
    }
    void SetWarmStart(pbd_warmstart *w, int min_sweeps = 0) {
        check(pbd_solver_set_warmstart(h_, w, min_sweeps));
    }
    pbd_autotune_result Autotune(int iterations = 15, int reps = 5) {
        pbd_autotune_result r;
        check(pbd_solver_autotune(h_, iterations, reps, &r));
        return r;
    }
    void SetGSPath(int path) { check(pbd_solver_set_gs_path(h_, path)); }
    pbd_solver *handle() const { return h_; }

private:
    pbd_solver *h_ = nullptr;
};

// learned warm start: per-point MLP on the tensor cores
class WarmStart {
public:
    WarmStart() { check(pbd_warmstart_create(&h_)); }
    ~WarmStart() { pbd_warmstart_destroy(h_); }
    WarmStart(const WarmStart &) = delete;
    WarmStart &operator=(const WarmStart &) = delete;
    void SetParams(const std::vector<float> &p) {
        check(pbd_warmstart_set_params(h_, p.data(), (int)p.size()));
    }
    void SetScales(const std::vector<float> &s) {
        check(pbd_warmstart_set_scales(h_, s.data(), (int)s.size()));
    }
    std::vector<float> Params() {
        std::vector<float> p(pbd_warmstart_num_params());
        check(pbd_warmstart_get_params(h_, p.data(), (int)p.size()));
        return p;
    }
    double TrainSubstep(SolverPBD &s, float dt, CollisionSolver *c, double target,
                        int max_sweeps, int chunk, float lr, bool on_policy) {
        double loss = 0.0;
        check(pbd_solver_train_substep(s.handle(), h_, dt, c ? c->handle() : nullptr, target,
                                       max_sweeps, chunk, lr, on_policy, &loss));
        return loss;
    }
    pbd_warmstart *handle() const { return h_; }

private:
    pbd_warmstart *h_ = nullptr;
};

}  // namespace pbd
