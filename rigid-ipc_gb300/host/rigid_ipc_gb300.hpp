// C++17 host layer over the rigc C ABI, mirroring the reference's interface
// for the narrow phase so a caller of the CPU path can switch by name:
//
//   RigidBodyAssembler              src/physics/rigid_body_assembler.hpp
//   detect_collision_candidates_rigid  src/ccd/rigid/broad_phase.hpp:52-59
//   DistanceBarrierConstraint       src/opt/distance_barrier_constraint.hpp:17-101
//     ::construct_constraint_set    (:51)
//     ::compute_earliest_toi        (:41)
//     ::has_active_collisions       (:36)
//   DistanceBarrierRBProblem        src/problems/distance_barrier_rb_problem.hpp:36-367
//     ::compute_barrier_term        (:267-273)
//     ::compute_earliest_toi        (:86-87)
//     ::has_collisions              (:82)
//
// Eigen types become std::vector<double> (dofs: 6 per body, [p, theta]) and
// a block-sparse matrix of 6x6 blocks; errors throw rigc::gb300::Error with
// the C ABI's status.  All device work is on the GPU; this header only moves
// host arrays through rigc_narrow_phase-style calls.
#pragma once

#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/rigc.h"

namespace ipc::rigid::gb300 {

struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string& where)
        : std::runtime_error(where + ": " + rigc_status_string(s)), status(s)
    {
    }
};

inline void check(int s, const char* where, bool allow_conservative = false)
{
    if (s == RIGC_OK) return;
    if (allow_conservative && (s == RIGC_ERR_QUEUE_OVERFLOW || s == RIGC_ERR_ITER_LIMIT)) return;
    throw Error(s, where);
}

// Device buffer owned by the host layer (only the pose uploads need one).
// Uploads go through rigc_copy, on the context's stream: queued after the
// context's earlier work (which may still read the previous poses when the
// context runs on a caller stream) and finished when upload returns.
class DeviceArray {
public:
    DeviceArray() = default;
    DeviceArray(const DeviceArray&) = delete;
    DeviceArray& operator=(const DeviceArray&) = delete;
    ~DeviceArray()
    {
        if (ptr_) cudaFree(ptr_);
    }
    double* upload(rigc_ctx* ctx, const std::vector<double>& v)
    {
        size_t bytes = v.size() * sizeof(double);
        if (bytes > cap_) {
            // the old buffer may still be read by queued work: free it only
            // after the context's stream has drained
            if (ptr_) {
                check(rigc_copy(ctx, nullptr, nullptr, 0), "rigc_copy");
                cudaFree(ptr_);
            }
            ptr_ = nullptr;
            if (cudaMalloc(&ptr_, bytes) != cudaSuccess) throw Error(RIGC_ERR_OOM, "DeviceArray");
            cap_ = bytes;
        }
        check(rigc_copy(ctx, ptr_, v.data(), bytes), "DeviceArray::upload");
        return static_cast<double*>(ptr_);
    }

private:
    void* ptr_ = nullptr;
    size_t cap_ = 0;
};

// Flattened bodies (what RigidBodyAssembler::init produces).
struct SceneArrays {
    std::vector<double> rest_vertices;   // nv x 3, body frame
    std::vector<int32_t> edges;          // ne x 2
    std::vector<int32_t> faces;          // nf x 3
    std::vector<int32_t> faces_to_edges; // nf x 3
    std::vector<int32_t> body_vertex_start, body_edge_start, body_face_start;
    std::vector<int32_t> group_ids, body_types;
    std::vector<double> r_max;
    double average_edge_length = 0;
};

class RigidBodyAssembler {
public:
    explicit RigidBodyAssembler(const SceneArrays& s) : arrays_(s)
    {
        rigc_scene_desc d {};
        d.num_bodies = (int32_t)s.group_ids.size();
        d.num_vertices = (int32_t)(s.rest_vertices.size() / 3);
        d.num_edges = (int32_t)(s.edges.size() / 2);
        d.num_faces = (int32_t)(s.faces.size() / 3);
        d.rest_vertices = s.rest_vertices.data();
        d.edges = s.edges.data();
        d.faces = s.faces.data();
        d.faces_to_edges = s.faces_to_edges.data();
        d.body_vertex_start = s.body_vertex_start.data();
        d.body_edge_start = s.body_edge_start.data();
        d.body_face_start = s.body_face_start.data();
        d.group_ids = s.group_ids.data();
        d.body_types = s.body_types.data();
        d.r_max = s.r_max.data();
        d.average_edge_length = s.average_edge_length;
        check(rigc_ctx_create(&d, &ctx_), "rigc_ctx_create");
    }
    RigidBodyAssembler(const RigidBodyAssembler&) = delete;
    RigidBodyAssembler& operator=(const RigidBodyAssembler&) = delete;
    ~RigidBodyAssembler()
    {
        if (ctx_) rigc_ctx_destroy(ctx_);
    }

    size_t num_bodies() const { return arrays_.group_ids.size(); }
    size_t num_vertices() const { return arrays_.rest_vertices.size() / 3; }
    rigc_ctx* ctx() const { return ctx_; }
    const SceneArrays& arrays() const { return arrays_; }

    // world_vertices(poses): nv x 3, row-major
    std::vector<double> world_vertices(const std::vector<double>& dofs) const
    {
        double* x = x0_.upload(ctx_, dofs);
        double* V = nullptr;
        size_t bytes = 3 * num_vertices() * sizeof(double);
        if (cudaMalloc(&V, bytes) != cudaSuccess) throw Error(RIGC_ERR_OOM, "world_vertices");
        int s = rigc_world_vertices(ctx_, x, V);
        std::vector<double> out(3 * num_vertices());
        if (s == RIGC_OK) s = rigc_copy(ctx_, out.data(), V, bytes);
        cudaFree(V);
        check(s, "rigc_world_vertices");
        return out;
    }

    // uploads used by the classes below
    mutable DeviceArray x0_, x1_;

private:
    SceneArrays arrays_;
    rigc_ctx* ctx_ = nullptr;
};

struct Candidates {
    std::vector<int32_t> ee;  // pairs (edge0 < edge1)
    std::vector<int32_t> fv;  // pairs (face, vertex)
    size_t size() const { return ee.size() / 2 + fv.size() / 2; }
};

enum class DetectionMethod { HASH_GRID };

// TrajectoryType (src/ccd/ccd.hpp:31-47) of the narrow phase: the rigid
// interval trajectory or the piecewise-linear one (the JSON default)
enum class TrajectoryType { RIGID, PIECEWISE_LINEAR };

// detect_collision_candidates_rigid (continuous when poses differ)
inline void detect_collision_candidates_rigid(
    const RigidBodyAssembler& bodies, const std::vector<double>& poses_t0,
    const std::vector<double>& poses_t1, Candidates& candidates,
    DetectionMethod = DetectionMethod::HASH_GRID, double inflation_radius = 0.0,
    bool continuous = true)
{
    double* x0 = bodies.x0_.upload(bodies.ctx(), poses_t0);
    double* x1 = bodies.x1_.upload(bodies.ctx(), poses_t1);
    rigc_candidates c {};
    check(rigc_detect_candidates(bodies.ctx(), x0, x1, continuous ? 1 : 0, inflation_radius, &c),
          "rigc_detect_candidates");
    candidates.ee.resize(2 * c.num_ee);
    candidates.fv.resize(2 * c.num_fv);
    check(rigc_copy(bodies.ctx(), candidates.ee.data(), c.ee, candidates.ee.size() * 4), "rigc_copy");
    check(rigc_copy(bodies.ctx(), candidates.fv.data(), c.fv, candidates.fv.size() * 4), "rigc_copy");
}

struct Constraints {
    std::vector<int32_t> type, verts, prims, bodies;
    std::vector<double> weight, eps_x;
    size_t size() const { return type.size(); }
};

// 6x6 block-sparse rows (row_ptr over bodies, sorted columns, row-major blocks)
struct BlockSparse {
    std::vector<int32_t> row_ptr, col;
    std::vector<double> val;
    size_t nnz_blocks() const { return col.size(); }
};

class DistanceBarrierConstraint {
public:
    double initial_barrier_activation_distance = 1e-3;
    double minimum_separation_distance = 0.0;
    // CollisionConstraint's default (src/opt/collision_constraint.cpp:7)
    TrajectoryType trajectory_type = TrajectoryType::RIGID;
    double barrier_activation_distance() const { return initial_barrier_activation_distance; }

    void construct_constraint_set(
        const RigidBodyAssembler& bodies, const std::vector<double>& poses,
        Constraints& out) const
    {
        double* x = bodies.x0_.upload(bodies.ctx(), poses);
        rigc_constraints c {};
        check(rigc_construct_constraint_set(bodies.ctx(), x, barrier_activation_distance(),
                                            minimum_separation_distance, &c),
              "rigc_construct_constraint_set");
        out.type.resize(c.num);
        out.verts.resize(4 * c.num);
        out.prims.resize(2 * c.num);
        out.bodies.resize(2 * c.num);
        out.weight.resize(c.num);
        out.eps_x.resize(c.num);
        rigc_ctx* k = bodies.ctx();
        check(rigc_copy(k, out.type.data(), c.type, c.num * 4), "rigc_copy");
        check(rigc_copy(k, out.verts.data(), c.verts, c.num * 16), "rigc_copy");
        check(rigc_copy(k, out.prims.data(), c.prims, c.num * 8), "rigc_copy");
        check(rigc_copy(k, out.bodies.data(), c.bodies, c.num * 8), "rigc_copy");
        check(rigc_copy(k, out.weight.data(), c.weight, c.num * 8), "rigc_copy");
        check(rigc_copy(k, out.eps_x.data(), c.eps_x, c.num * 8), "rigc_copy");
    }

    // earliest time of impact in (0, 1], or +infinity when nothing collides
    double compute_earliest_toi(
        const RigidBodyAssembler& bodies, const std::vector<double>& poses_t0,
        const std::vector<double>& poses_t1) const
    {
        return earliest_toi(bodies, poses_t0, poses_t1, trajectory_type);
    }

    // has_active_collisions_narrow_phase runs the rigid CCD for the
    // piecewise-linear trajectory too (src/opt/distance_barrier_constraint.cpp:91-95)
    bool has_active_collisions(
        const RigidBodyAssembler& bodies, const std::vector<double>& poses_t0,
        const std::vector<double>& poses_t1) const
    {
        return std::isfinite(earliest_toi(bodies, poses_t0, poses_t1, TrajectoryType::RIGID));
    }

private:
    double earliest_toi(const RigidBodyAssembler& bodies, const std::vector<double>& poses_t0,
                        const std::vector<double>& poses_t1, TrajectoryType trajectory) const
    {
        double* x0 = bodies.x0_.upload(bodies.ctx(), poses_t0);
        double* x1 = bodies.x1_.upload(bodies.ctx(), poses_t1);
        double toi = INFINITY;
        if (trajectory == TrajectoryType::PIECEWISE_LINEAR)
            check(rigc_compute_earliest_toi_piecewise_linear(bodies.ctx(), x0, x1,
                                                             minimum_separation_distance, &toi),
                  "rigc_compute_earliest_toi_piecewise_linear", true);
        else
            check(rigc_compute_earliest_toi(bodies.ctx(), x0, x1, minimum_separation_distance, &toi),
                  "rigc_compute_earliest_toi", true);
        return toi;
    }
};

class DistanceBarrierRBProblem {
public:
    explicit DistanceBarrierRBProblem(const SceneArrays& s) : assembler_(s) {}

    DistanceBarrierConstraint& constraint() { return constraint_; }
    const RigidBodyAssembler& assembler() const { return assembler_; }

    // compute_barrier_term(x, grad, hess, compute_grad, compute_hess) over
    // the constraint set at x (rebuilt here, as compute_objective does)
    double compute_barrier_term(
        const std::vector<double>& x, std::vector<double>& grad, BlockSparse& hess,
        bool compute_grad = true, bool compute_hess = true)
    {
        double* xd = assembler_.x0_.upload(assembler_.ctx(), x);
        rigc_ctx* k = assembler_.ctx();
        check(rigc_construct_constraint_set(k, xd, constraint_.barrier_activation_distance(),
                                            constraint_.minimum_separation_distance, nullptr),
              "rigc_construct_constraint_set");
        int flags = (compute_grad ? RIGC_GRAD : 0) | (compute_hess ? RIGC_HESS | RIGC_PROJECT_PSD : 0);
        rigc_barrier_out o {};
        check(rigc_barrier_term(k, xd, constraint_.barrier_activation_distance(),
                                constraint_.minimum_separation_distance, flags, &o),
              "rigc_barrier_term");
        const size_t nb = assembler_.num_bodies();
        if (compute_grad || compute_hess) {
            grad.resize(6 * nb);
            check(rigc_copy(k, grad.data(), o.grad, grad.size() * 8), "rigc_copy");
        }
        if (compute_hess) {
            hess.row_ptr.resize(nb + 1);
            hess.col.resize(o.nnzb);
            hess.val.resize(36 * o.nnzb);
            check(rigc_copy(k, hess.row_ptr.data(), o.row_ptr, (nb + 1) * 4), "rigc_copy");
            check(rigc_copy(k, hess.col.data(), o.col, o.nnzb * 4), "rigc_copy");
            check(rigc_copy(k, hess.val.data(), o.val, o.nnzb * 36 * 8), "rigc_copy");
        }
        return o.energy;
    }

    double compute_earliest_toi(const std::vector<double>& x_i, const std::vector<double>& x_j)
    {
        return constraint_.compute_earliest_toi(assembler_, x_i, x_j);
    }

    bool has_collisions(const std::vector<double>& x_i, const std::vector<double>& x_j)
    {
        return constraint_.has_active_collisions(assembler_, x_i, x_j);
    }

    // compute_min_distance(x) (distance_barrier_rb_problem.cpp:1583-1589):
    // the smallest constraint distance at x, -1 when the set is empty
    double compute_min_distance(const std::vector<double>& x)
    {
        double* xd = assembler_.x0_.upload(assembler_.ctx(), x);
        double d = -1;
        check(rigc_min_distance(assembler_.ctx(), xd, constraint_.barrier_activation_distance(),
                                constraint_.minimum_separation_distance, &d),
              "rigc_min_distance");
        return d;
    }

    // detect_intersections(poses) (rigid_body_problem.cpp:289-360)
    bool detect_intersections(const std::vector<double>& x)
    {
        double* xd = assembler_.x0_.upload(assembler_.ctx(), x);
        int64_t n = 0;
        check(rigc_detect_intersections(assembler_.ctx(), xd, &n), "rigc_detect_intersections");
        return n > 0;
    }

private:
    RigidBodyAssembler assembler_;
    DistanceBarrierConstraint constraint_;
};

} // namespace ipc::rigid::gb300
