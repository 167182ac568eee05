// CPU oracle for the Rigid IPC narrow phase (test infrastructure only).
//
// This library restates the reference's CPU algorithm for the hot path so the
// CUDA path can be checked against it.  It is linked only by the tests, by the
// smoke check and by the CPU-baseline leg of the benchmark; the product path
// never calls it.  Each function cites the reference file:line it follows
// (paths relative to the rigid-ipc source tree).  Third-party arithmetic the
// reference takes from ipc-toolkit (distances, distance types, barrier,
// constraint-set construction, PSD projection, hash-grid pairing) is restated
// from the published IPC formulation; filib/Boost.Interval semantics are
// restated from their documented definitions.  Derivatives here come from
// forward-mode second-order autodiff, independent of the closed forms the
// CUDA kernels use.
#pragma once

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

namespace orc {

// fn(i) for i in [0, n) over the host's threads, chunk items at a time; the
// work of each i may not depend on another's (results that are summed are
// summed afterwards, in index order, by the caller)
template <class F> void parallel_for(long long n, long long chunk, F fn)
{
    const int nt = std::max(1, (int)std::thread::hardware_concurrency());
    if (nt == 1 || n <= chunk) {
        for (long long i = 0; i < n; i++) fn(i);
        return;
    }
    std::atomic<long long> next(0);
    auto work = [&]() {
        for (;;) {
            const long long i0 = next.fetch_add(chunk);
            if (i0 >= n) break;
            for (long long i = i0; i < std::min(n, i0 + chunk); i++) fn(i);
        }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < nt; t++) th.emplace_back(work);
    for (auto& t : th) t.join();
}


// ---------------------------------------------------------------------------
// Second-order forward-mode autodiff scalar with N variables (value, gradient,
// Hessian), the role of DScalar2 in src/autodiff/autodiff.h.
template <int N> struct D2 {
    double v = 0;
    double g[N] = {};
    double h[N][N] = {};
    D2() = default;
    D2(double x) : v(x) {}
    static D2 var(double x, int i)
    {
        D2 r(x);
        r.g[i] = 1;
        return r;
    }
};

template <int N> inline D2<N> operator+(const D2<N>& a, const D2<N>& b)
{
    D2<N> r;
    r.v = a.v + b.v;
    for (int i = 0; i < N; i++) r.g[i] = a.g[i] + b.g[i];
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++) r.h[i][j] = a.h[i][j] + b.h[i][j];
    return r;
}
template <int N> inline D2<N> operator-(const D2<N>& a, const D2<N>& b)
{
    D2<N> r;
    r.v = a.v - b.v;
    for (int i = 0; i < N; i++) r.g[i] = a.g[i] - b.g[i];
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++) r.h[i][j] = a.h[i][j] - b.h[i][j];
    return r;
}
template <int N> inline D2<N> operator-(const D2<N>& a)
{
    D2<N> r;
    r.v = -a.v;
    for (int i = 0; i < N; i++) r.g[i] = -a.g[i];
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++) r.h[i][j] = -a.h[i][j];
    return r;
}
template <int N> inline D2<N> operator*(const D2<N>& a, const D2<N>& b)
{
    D2<N> r;
    r.v = a.v * b.v;
    for (int i = 0; i < N; i++) r.g[i] = a.v * b.g[i] + b.v * a.g[i];
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++)
            r.h[i][j] = a.v * b.h[i][j] + b.v * a.h[i][j] + a.g[i] * b.g[j]
                + b.g[i] * a.g[j];
    return r;
}
template <int N> inline D2<N> operator*(double s, const D2<N>& a)
{
    D2<N> r;
    r.v = s * a.v;
    for (int i = 0; i < N; i++) r.g[i] = s * a.g[i];
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++) r.h[i][j] = s * a.h[i][j];
    return r;
}
template <int N> inline D2<N> operator*(const D2<N>& a, double s) { return s * a; }
template <int N> inline D2<N> operator+(const D2<N>& a, double s)
{
    D2<N> r = a;
    r.v += s;
    return r;
}
template <int N> inline D2<N> operator+(double s, const D2<N>& a) { return a + s; }
template <int N> inline D2<N> operator-(const D2<N>& a, double s) { return a + (-s); }
template <int N> inline D2<N> operator-(double s, const D2<N>& a) { return (-a) + s; }

// unary chain rule with f(a), f'(a), f''(a)
template <int N>
inline D2<N> chain(const D2<N>& a, double f, double df, double ddf)
{
    D2<N> r;
    r.v = f;
    for (int i = 0; i < N; i++) r.g[i] = df * a.g[i];
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++)
            r.h[i][j] = df * a.h[i][j] + ddf * a.g[i] * a.g[j];
    return r;
}
template <int N> inline D2<N> inv(const D2<N>& a)
{
    double x = a.v;
    return chain(a, 1 / x, -1 / (x * x), 2 / (x * x * x));
}
template <int N> inline D2<N> operator/(const D2<N>& a, const D2<N>& b)
{
    return a * inv(b);
}
template <int N> inline D2<N> operator/(const D2<N>& a, double s)
{
    return (1.0 / s) * a;
}
template <int N> inline D2<N> log(const D2<N>& a)
{
    double x = a.v;
    return chain(a, std::log(x), 1 / x, -1 / (x * x));
}
template <int N> inline D2<N> sqrt(const D2<N>& a)
{
    double s = std::sqrt(a.v);
    return chain(a, s, 0.5 / s, -0.25 / (s * a.v));
}

inline double val(double x) { return x; }
template <int N> inline double val(const D2<N>& x) { return x.v; }

// ---------------------------------------------------------------------------
// Scene view: borrowed flat arrays, the same layout the C-ABI takes
// (RigidBodyAssembler::init, src/physics/rigid_body_assembler.cpp:19-118).
struct Scene {
    int nb = 0, nv = 0, ne = 0, nf = 0;
    const double* rest = nullptr;   // nv x 3, body frame
    const int* edges = nullptr;     // ne x 2
    const int* faces = nullptr;     // nf x 3
    const int* f2e = nullptr;       // nf x 3
    const int* bvs = nullptr;       // nb + 1
    const int* bes = nullptr;       // nb + 1
    const int* bfs = nullptr;       // nb + 1
    const int* group = nullptr;     // nb
    const int* type = nullptr;      // nb (0 static, 1 kinematic, 2 dynamic)
    const double* rmax = nullptr;   // nb
    double avg_edge_len = 0;
    std::vector<int> vbody, ebody, fbody;
    std::vector<double> edge_len;   // rest edge lengths
    void finalize();
};

// Constraint types in the order the reference concatenates them
// (vv, ev, ee, fv; rigid_body_collision_constraint.hpp:186-240).
enum { C_VV = 0, C_EV = 1, C_EE = 2, C_FV = 3 };

struct Constraint {
    int type;
    int v[4];       // vertex ids in ipc-toolkit vertex_indices order
    int prim[2];    // primitive ids: VV (v0,v1) EV (edge,vertex) EE (ea,eb) FV (face,vertex)
    int body[2];    // local body 0 / 1
    double weight;  // multiplicity (VV, EV), 1 otherwise
    double eps_x;   // EE mollifier threshold
    int nverts() const { return type == C_VV ? 2 : (type == C_EV ? 3 : 4); }
};

// local body of each constraint vertex (rigid_body_collision_constraint.hpp:51,94,140,180)
inline int local_body(int type, int i)
{
    switch (type) {
    case C_VV: return i == 0 ? 0 : 1;
    case C_EV: return i == 0 ? 0 : 1;
    case C_EE: return i < 2 ? 0 : 1;
    default: return i == 0 ? 0 : 1;
    }
}

// ---------------------------------------------------------------------------
// rotation and world vertices (src/physics/pose.tpp:203-218, rigid_body.tpp)
void rotation_matrix(const double* theta, double R[9]);
// V, dV/dtheta (3x3 per vertex: [coord][k]), d2V/dtheta2 (3x3x3: [coord][k][l])
void world_vertices_diff(
    const Scene& s, const double* x, std::vector<double>& V,
    std::vector<double>& dV, std::vector<double>& d2V);
void world_vertices(const Scene& s, const double* x, std::vector<double>& V);

// distances (squared) and types
enum {
    PT_P_T0 = 0, PT_P_T1, PT_P_T2, PT_P_E0, PT_P_E1, PT_P_E2, PT_P_T
};
enum {
    EE_EA0_EB0 = 0, EE_EA0_EB1, EE_EA1_EB0, EE_EA1_EB1,
    EE_EA_EB0, EE_EA_EB1, EE_EA0_EB, EE_EA1_EB, EE_EA_EB
};
int point_triangle_distance_type(const double* p, const double* t0, const double* t1, const double* t2);
int edge_edge_distance_type(const double* ea0, const double* ea1, const double* eb0, const double* eb1);
double point_point_sqdist(const double* p, const double* q);
double point_line_sqdist(const double* p, const double* e0, const double* e1);
// segment-segment squared distance by the closest features (the distance of
// an EE constraint)
double edge_edge_sqdist(const double* a0, const double* a1, const double* b0, const double* b1);
double point_plane_sqdist(const double* p, const double* t0, const double* t1, const double* t2);
double line_line_sqdist(const double* ea0, const double* ea1, const double* eb0, const double* eb1);
double ee_cross_sqnorm(const double* ea0, const double* ea1, const double* eb0, const double* eb1);

// barrier b(d; s) of ipc-toolkit (log barrier of the squared distance)
double barrier(double d, double s);
// squared distance of one constraint (the distance its barrier uses)
double constraint_sqdist(const Constraint& c, const std::vector<double>& V);

// candidates (ipc-toolkit Candidates)
struct Candidates {
    std::vector<std::array<int, 2>> ev, ee, fv;  // (edge,vertex) (edge,edge) (face,vertex)
};

// constraint set from candidates (ipc::construct_constraint_set)
void construct_constraint_set(
    const Scene& s, const Candidates& cand, const std::vector<double>& V,
    double dhat, double dmin, std::vector<Constraint>& out);

// symmetric PSD projection (ipc-toolkit project_to_psd: eigen-clamp)
void project_to_psd(int n, const double* A, double* out);

// per-constraint local energy, 12-gradient and 12x12 Hessian in body space
struct LocalTerm {
    double energy;
    double grad[12];
    double hess[144];
};
void constraint_local_term(
    const Scene& s, const Constraint& c, const std::vector<double>& V,
    const std::vector<double>& dV, const std::vector<double>& d2V,
    double dhat, double dmin, bool project, LocalTerm& out);

// barrier term assembled (compute_barrier_term,
// src/problems/distance_barrier_rb_problem.cpp:1299-1399).  Hessian returned
// as BSR with 6x6 blocks, columns sorted per row.
struct BSR {
    std::vector<int> row_ptr, col;
    std::vector<double> val;  // nnzb x 36 (row-major blocks)
};
double barrier_term(
    const Scene& s, const double* x, const std::vector<Constraint>& cs,
    double dhat, double dmin, std::vector<double>& grad, BSR& hess,
    bool project);

double barrier_energy(const Scene& s, const double* x, const std::vector<Constraint>& cs,
                      double dhat, double dmin);

// body energy (compute_body_energy, distance_barrier_rb_problem.cpp:847-944)
struct BodyState {
    double mass;
    double moment[3];
    double pose_t0[6];
    double vel_t0[6];      // v (world), omega (body frame)
    double Qdot[9];        // row-major
    bool fixed[6];
    int type;
    // kinematic bodies: the pose the step drives the body to (the front of
    // its kinematic pose list, init_augmented_lagrangian); without one,
    // x0 + h v
    bool has_target = false;
    double kin_target[6] = { 0, 0, 0, 0, 0, 0 };
};
double body_energy(
    const BodyState& b, const double* x6, const double gravity[3], double h,
    double grad[6], double hess[36]);

// one simulation time step (DistanceBarrierRBProblem::simulation_step with
// the IPC Newton solver); bodies' pose_t0 / vel_t0 (linear) / Qdot advance,
// kappa is the barrier stiffness carried from step to step (1 before the
// first step)
struct SimParams {
    double h, gravity[3], dhat, dmin, mu, epsv;
    int max_newton_iterations;
    double velocity_conv_tol;
    int velocity_conv_tol_abs;
    double line_search_lower_bound, dhat_epsilon, min_barrier_stiffness_scale;
    double bbox_diagonal, average_mass;
    int newton_polish = 0;  // full Newton steps after convergence (0: the reference's solver)
    double ccd_rescale = 1; // step bound s * toi when the CCD limits the step (1: the reference)
    int trajectory = 0;     // line-search CCD: 0 RIGID, 1 PIECEWISE_LINEAR (minimum separation dmin)
};
struct SimStats {
    long long newton_iterations = 0, newton_steps = 0, objective_evals = 0, ccd_calls = 0;
};
// what the adjoint of a step needs besides the start-of-step state: the
// solution x (6 nb), the final barrier stiffness, and d kappa / d kappa0
// (kappa0 = -gE.gB / gB.gB at the start of the step: 2^doublings while
// kappa0 lies inside its clamp and no doubling reached the cap, else 0)
struct StepRecord {
    std::vector<double> x;
    double kappa = 0, dkappa_dk0 = 0;
};
void simulation_step(const Scene& s, std::vector<BodyState>& bodies, const SimParams& p,
                     double& kappa, SimStats* st, StepRecord* rec = nullptr);

// body energy over (x6, pose_t0, linear velocity, Qdot): gradient and Hessian
// over these 24 variables
void body_energy_state_derivs(
    const BodyState& b, const double* x6, const double gravity[3], double h,
    double grad[24], double hess[576]);
// dR / dtheta_a (a = 0..2), each row-major 3 x 3
void rotation_matrix_jacobian(const double* theta, double dR[27]);
// d2R / dtheta_a dtheta_c, [a][c] each row-major 3 x 3
void rotation_matrix_hessian(const double* theta, double d2R[81]);

// Adjoint of one time step (implicit differentiation of the converged
// Newton solve): given dL / d(state after the step) in `in` (poses 6 nb,
// velocities 6 nb, Qdot 9 nb), accumulate dL / d(state before) into `out`.
// Returns false when the Hessian of the free dofs cannot be factorised, or
// when the scene has kinematic bodies (their targets are not differentiated).
struct AdjointState {
    std::vector<double> pose, vel, Qdot;
};
bool adjoint_step(const Scene& s, const std::vector<BodyState>& pre, const SimParams& p,
                  const StepRecord& rec, const AdjointState& in, AdjointState& out);

// lagged friction constraints and their local terms
struct FrictionConstraint {
    Constraint c;
    double lambda;   // normal force magnitude at the start of the step
    double p0, p1;   // closest-point parameters (EV alpha; EE alpha, beta; FV b1, b2)
    double T[6];     // tangent basis, columns t1 = T[0..2], t2 = T[3..5]
};
void construct_friction_constraints(
    const Scene& s, const std::vector<Constraint>& cs, const std::vector<double>& V0,
    double dhat, double dmin, double kappa, std::vector<FrictionConstraint>& out);
void friction_local_term(
    const Scene& s, const FrictionConstraint& f, const std::vector<double>& V,
    const std::vector<double>& V0, const std::vector<double>& dV,
    const std::vector<double>& d2V, double mu, double epsvh, bool project, LocalTerm& out);
double friction_term(
    const Scene& s, const double* x, const double* x0, const std::vector<FrictionConstraint>& fcs,
    double mu, double epsvh, std::vector<double>& grad, BSR& hess, bool project);

// ---------------------------------------------------------------------------
// broad phase
struct AABB {
    double lo[3], hi[3];
};
// the reference's AABB overlap test (center / half-extent form)
bool aabb_overlap(const AABB& a, const AABB& b);
// body boxes (RigidBody::compute_bounding_box, rigid_body.cpp:246-272)
void body_bounding_box(
    const Scene& s, int b, const double* x0, const double* x1, double lo[3],
    double hi[3]);
// close body pairs (close_bodies_bvh, rigid_body_assembler.cpp:307-356)
// (face, edge) pairs of different groups whose boxes at x overlap
void edge_face_candidates(const Scene& s, const double* x, std::vector<std::array<int, 2>>& out);

std::vector<std::array<int, 2>> close_bodies(
    const Scene& s, const double* x0, const double* x1, double inflation);
// element boxes; included flags per vertex/edge/face
void element_aabbs(
    const Scene& s, const double* x0, const double* x1, bool continuous,
    double inflation, const std::vector<std::array<int, 2>>& body_pairs,
    std::vector<AABB>& vbox, std::vector<AABB>& ebox, std::vector<AABB>& fbox,
    std::vector<char>& vin, std::vector<char>& ein, std::vector<char>& fin);
// candidate detection (detect_collision_candidates_rigid, hash-grid pairing)
void detect_candidates(
    const Scene& s, const double* x0, const double* x1, bool continuous,
    double inflation, bool brute_force, Candidates& out);

// ---------------------------------------------------------------------------
// rigid interval CCD
// box counter, optional per-candidate box budget (0 = none, as the
// reference) and the worst status (5 = budget exhausted, with the smallest
// unexplored t.lo reported as a conservative time of impact)
struct CCDStats {
    long long boxes = 0;
    long long max_boxes = 0;
    int status = 0;
    // optional running minimum over all candidates (bits of a non-negative
    // double): boxes starting at or after it are skipped, which keeps the
    // earliest time of impact (it does not depend on the visiting order)
    std::atomic<unsigned long long>* gmin = nullptr;
};
bool edge_edge_toi(
    const Scene& s, const double* x0, const double* x1, int ea, int eb,
    double earliest, double toi_tol, double& toi, CCDStats* st);
bool face_vertex_toi(
    const Scene& s, const double* x0, const double* x1, int f, int v,
    double earliest, double toi_tol, double& toi, CCDStats* st);
double earliest_toi(
    const Scene& s, const double* x0, const double* x1, const Candidates& c,
    double toi_tol, int nthreads, std::vector<double>* per_candidate,
    CCDStats* st);

// piecewise-linear trajectory CCD (pl_ccd.cpp)
struct PLStats {
    long long boxes = 0;   // boxes of the linear CCDs
    long long pieces = 0;  // pieces (including halvings)
    int status = 0;        // 5: a linear CCD ran out of boxes; 4: a piece
                           // could not be halved further (conservative start)
};
// the linear CCD alone: points p0 -> p1 (4 x 3 each; EE a0 a1 b0 b1, FV v
// f0 f1 f2) moving on straight lines over t in [0, 1], minimum separation ms
bool linear_ccd(bool fv, const double* p0, const double* p1, double ms, double& toi,
                long long& boxes, int& status);
bool pl_edge_edge_toi(const Scene& s, const double* x0, const double* x1, int ea, int eb,
                      double earliest_bound, double dmin, double& toi, PLStats* st);
bool pl_face_vertex_toi(const Scene& s, const double* x0, const double* x1, int f, int v,
                        double earliest_bound, double dmin, double& toi, PLStats* st);
double pl_earliest_toi(const Scene& s, const double* x0, const double* x1, const Candidates& c,
                       double dmin, int nthreads, std::vector<double>* per, PLStats* st);

} // namespace orc
