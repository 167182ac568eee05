/*
 * rigc.h -- C ABI of the GB300 (sm_103a) Rigid IPC narrow phase.
 *
 * Every entry point is plain C: pointers, sizes and an int status.  Device
 * pointers are CUDA global-memory addresses on the context's device; "host"
 * in a name means host memory.  All work is ordered on the context's stream
 * (rigc_set_stream); an entry point synchronises only when it returns a value
 * in host memory.  No exception crosses this boundary.
 *
 * Paths below are relative to the rigid-ipc source tree (ipc-sim/rigid-ipc).
 * Each entry point names the reference interface it replaces.
 */
#ifndef RIGC_H
#define RIGC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (the reference returns bool / infinity / throws; see
 * src/opt/distance_barrier_constraint.cpp:263-264, src/ccd/ccd.cpp:217) */
#define RIGC_OK 0
#define RIGC_ERR_ARG 1            /* invalid argument                         */
#define RIGC_ERR_CUDA 2           /* CUDA runtime error                       */
#define RIGC_ERR_OOM 3            /* device allocation failed                 */
#define RIGC_ERR_QUEUE_OVERFLOW 4 /* CCD box stack overflowed (result kept
                                     conservative)                            */
#define RIGC_ERR_ITER_LIMIT 5     /* CCD box budget exhausted (result kept
                                     conservative)                            */
#define RIGC_ERR_NAN 6            /* non-finite pose input                    */
#define RIGC_ERR_TOO_LARGE 7      /* input larger than a fixed-capacity entry
                                     point accepts                            */
#define RIGC_ERR_SOLVE 8          /* the Hessian of the free dofs could not be
                                     factorised (adjoint)                     */

/* body types (src/physics/rigid_body.hpp RigidBodyType) */
#define RIGC_BODY_STATIC 0
#define RIGC_BODY_KINEMATIC 1
#define RIGC_BODY_DYNAMIC 2

/* rigc_barrier_term flags (compute_grad / compute_hess of
 * DistanceBarrierRBProblem::compute_barrier_term) */
#define RIGC_GRAD 1
#define RIGC_HESS 2
#define RIGC_PROJECT_PSD 4 /* project each 12x12 pair Hessian to PSD       */

/* rigc_sim_params.trajectory_type (TrajectoryType, src/ccd/ccd.hpp:31-47) */
#define RIGC_TRAJECTORY_RIGID 0
#define RIGC_TRAJECTORY_PIECEWISE_LINEAR 1

/* rigc_earliest_toi flags */
#define RIGC_TOI_NO_PRUNE 1 /* search every candidate in full (per-candidate
                               times of impact become exact, slower)         */

typedef struct rigc_ctx rigc_ctx;

/* Flattened rigid bodies, as RigidBodyAssembler::init builds them
 * (src/physics/rigid_body_assembler.cpp:19-118).  Host pointers; copied. */
typedef struct rigc_scene_desc {
    int32_t num_bodies;
    int32_t num_vertices;
    int32_t num_edges;
    int32_t num_faces;
    const double* rest_vertices;     /* num_vertices x 3, body frame         */
    const int32_t* edges;            /* num_edges x 2, global vertex ids     */
    const int32_t* faces;            /* num_faces x 3, global vertex ids     */
    const int32_t* faces_to_edges;   /* num_faces x 3, edge (j, j+1 mod 3)   */
    const int32_t* body_vertex_start;/* num_bodies + 1                       */
    const int32_t* body_edge_start;  /* num_bodies + 1                       */
    const int32_t* body_face_start;  /* num_bodies + 1                       */
    const int32_t* group_ids;        /* num_bodies                           */
    const int32_t* body_types;       /* num_bodies, RIGC_BODY_*              */
    const double* r_max;             /* num_bodies, max rest vertex norm     */
    double average_edge_length;
} rigc_scene_desc;

/* Candidate pairs (ipc-toolkit Candidates as filled by
 * src/ccd/rigid/broad_phase.cpp:166-204).  Device pointers owned by the
 * context, valid until the next call that writes candidates.  Pairs are
 * sorted and unique: ee = (edge0 < edge1), fv = (face, vertex). */
typedef struct rigc_candidates {
    int64_t num_ee;
    int64_t num_fv;
    const int32_t* ee; /* num_ee x 2 */
    const int32_t* fv; /* num_fv x 2 */
} rigc_candidates;

/* Constraint set (ipc-toolkit Constraints: vv | ev | ee | fv, built by
 * DistanceBarrierConstraint::construct_constraint_set,
 * src/opt/distance_barrier_constraint.cpp:267-306).  Device pointers owned by
 * the context. type: 0 VV, 1 EV, 2 EE, 3 FV; verts in ipc-toolkit
 * vertex_indices order (-1 unused); prims = VV (v0, v1), EV (edge, vertex),
 * EE (edge0, edge1), FV (face, vertex); bodies = (local body 0, 1). */
typedef struct rigc_constraints {
    int64_t num;
    int64_t num_vv, num_ev, num_ee, num_fv;
    const int32_t* type;   /* num          */
    const int32_t* verts;  /* num x 4      */
    const int32_t* prims;  /* num x 2      */
    const int32_t* bodies; /* num x 2      */
    const double* weight;  /* num, multiplicity */
    const double* eps_x;   /* num, EE mollifier threshold */
} rigc_constraints;

/* Barrier term: energy (host), gradient (device, 6 per body) and the Hessian
 * as block-sparse rows of 6x6 row-major blocks (device). */
typedef struct rigc_barrier_out {
    double energy;
    int64_t nnzb;
    const double* grad;      /* 6 * num_bodies         */
    const int32_t* row_ptr;  /* num_bodies + 1         */
    const int32_t* col;      /* nnzb, sorted per row   */
    const double* val;       /* nnzb x 36              */
} rigc_barrier_out;

/* Counters of the last calls (for measurement). */
typedef struct rigc_stats {
    int64_t ccd_boxes;        /* boxes evaluated by the last earliest-toi    */
    int64_t ccd_candidates;   /* candidates of the last earliest-toi         */
    int64_t ccd_collisions;   /* candidates with an impact                   */
    int64_t grid_items;       /* hash-grid (cell, element) items             */
    int64_t large_elements;   /* elements tested outside the grid            */
    int64_t cand_ee;          /* current candidates (last broad phase)       */
    int64_t cand_fv;
    int64_t kernel_launches;  /* kernels launched by this library so far     */
    int32_t last_status;
    int32_t ccd_launches;     /* search launches of the last earliest-toi    */
    int64_t ccd_pieces;       /* search pieces those launches took up        */
} rigc_stats;

/* ---- context (replaces the RigidBodyAssembler set-up,
 *      src/physics/rigid_body_assembler.cpp:19-118) ---- */
int rigc_ctx_create(const rigc_scene_desc* desc, rigc_ctx** out);
int rigc_ctx_destroy(rigc_ctx* ctx);

/* ---- batched form (no counterpart in the reference, which simulates one
 * scene per process): many independent scenes in one context, so that every
 * call processes all of them in the same launches.  body_scene (host,
 * num_bodies) gives each body's scene, non-decreasing, in [0, num_scenes).
 * Element pairs are only formed within a scene (the scene is part of the
 * hash-grid cell key); the CCD prunes each scene by its own running minimum;
 * constraint sets, gradients and the block-sparse Hessian are those of the
 * scenes side by side.  Per-scene results of the last call: */
int rigc_ctx_create_batched(const rigc_scene_desc* desc, int32_t num_scenes,
                            const int32_t* body_scene, rigc_ctx** out);
int rigc_num_scenes(const rigc_ctx* ctx);
/* earliest time of impact of each scene (host, num_scenes; INFINITY when a
 * scene has no impact), after rigc_earliest_toi / rigc_compute_earliest_toi */
int rigc_scene_tois(rigc_ctx* ctx, double* toi_host);
/* barrier energy of each scene (host, num_scenes), after rigc_barrier_term */
int rigc_scene_barrier_energies(rigc_ctx* ctx, double* energy_host);
int rigc_set_stream(rigc_ctx* ctx, void* cuda_stream);
const char* rigc_status_string(int status);
int rigc_get_stats(const rigc_ctx* ctx, rigc_stats* out);

/* Copy bytes between any two addresses the device can see (host, pinned or
 * device; cudaMemcpyDefault) on the context's stream, then synchronise
 * (bytes 0: only wait for the context's stream).  For FFI callers without
 * CUDA bindings. */
int rigc_copy(rigc_ctx* ctx, void* dst, const void* src, size_t bytes);

/* World vertices V = R(theta) v + p for all vertices (device in/out).
 * Replaces RigidBodyAssembler::world_vertices
 * (src/physics/rigid_body_assembler.cpp:191-202). */
int rigc_world_vertices(rigc_ctx* ctx, const double* x, double* V);

/* ---- broad phase: detect_collision_candidates_rigid with
 * DetectionMethod::HASH_GRID (src/ccd/rigid/broad_phase.hpp:52-59,
 * broad_phase.cpp:19-91 discrete, :127-204 continuous).  x0, x1: device,
 * 6 * num_bodies doubles [p, theta] per body.  continuous = 0 ignores x1. */
int rigc_detect_candidates(rigc_ctx* ctx, const double* x0, const double* x1,
                           int continuous, double inflation_radius,
                           rigc_candidates* out);

/* Candidates given by the caller instead of the broad phase (host arrays,
 * ee: num_ee (edge, edge) pairs, fv: num_fv (face, vertex) pairs), the
 * Candidates argument of compute_earliest_toi_narrow_phase
 * (src/opt/distance_barrier_constraint.cpp:151-156).  Indices are checked;
 * RIGC_ERR_ARG when one is out of range. */
int rigc_set_candidates(rigc_ctx* ctx, int64_t num_ee, const int32_t* ee,
                        int64_t num_fv, const int32_t* fv);

/* Per-candidate cap on the boxes one CCD search may evaluate (default
 * 2^22; the reference has none).  A search that reaches it reports the
 * smallest t.lo still unexplored, a conservative time of impact, and
 * RIGC_ERR_ITER_LIMIT. */
int rigc_set_ccd_budget(rigc_ctx* ctx, int64_t max_boxes_per_candidate);

/* ---- narrow phase CCD: compute_earliest_toi_narrow_phase
 * (src/opt/distance_barrier_constraint.cpp:151-265) over the candidates of
 * the last rigc_detect_candidates / rigc_set_candidates call, trajectory RIGID
 * (src/ccd/rigid/time_of_impact.cpp:158-310).  Every candidate searches
 * t in [0, 1]; *toi_host = INFINITY when nothing collides.  per_candidate
 * (device, optional, num_ee + num_fv doubles, ee first). */
int rigc_earliest_toi(rigc_ctx* ctx, const double* x0, const double* x1,
                      double toi_tolerance, int flags, double* toi_host,
                      double* per_candidate);

/* DistanceBarrierConstraint::compute_earliest_toi
 * (src/opt/distance_barrier_constraint.cpp:130-149): continuous broad phase
 * with inflation dmin / 2, then the narrow phase. */
int rigc_compute_earliest_toi(rigc_ctx* ctx, const double* x0,
                              const double* x1, double dmin,
                              double* toi_host);

/* ---- narrow phase CCD, trajectory PIECEWISE_LINEAR (the reference's JSON
 * default): compute_earliest_toi_narrow_phase over the candidates of the
 * last rigc_detect_candidates / rigc_set_candidates call with
 * compute_piecewise_linear_edge_edge_time_of_impact /
 * compute_piecewise_linear_face_vertex_time_of_impact
 * (src/ccd/piecewise_linear/time_of_impact.cpp:326-651), minimum separation
 * dmin.  Each body's pose moves linearly over pieces of [0, 1] halved until
 * the rigid trajectory's deviation from the straight line is below half the
 * features' distance; a linear CCD (the inclusion-based method of
 * Tight-Inclusion, with the deviation + dmin as minimum separation and a
 * co-domain tolerance of 1e-6) finds each piece's first impact.  Every
 * candidate searches t in [0, 1]; *toi_host = INFINITY when nothing
 * collides; per_candidate (device, optional, num_ee + num_fv doubles, ee
 * first).  RIGC_ERR_ITER_LIMIT when a linear CCD used its 10^6 boxes,
 * RIGC_ERR_QUEUE_OVERFLOW when a piece or box could not be halved further
 * (results kept: the earliest unexplored time, conservative). */
int rigc_earliest_toi_piecewise_linear(rigc_ctx* ctx, const double* x0,
                                       const double* x1, double dmin,
                                       double* toi_host, double* per_candidate);

/* How the piecewise-linear CCD spreads its searches: 0 one candidate per
 * warp (the warp evaluates each box's corners together; the default, also
 * for -1), 1 one per lane.  The results are the same bits. */
int rigc_set_pl_search(rigc_ctx* ctx, int32_t per_lane);

/* Time windows of the rigid CCD's pruned searches (the earliest time of
 * impact; no counterpart in the reference, whose candidates run in any
 * order under one running minimum, compute_earliest_toi in
 * src/ccd/rigid/time_of_impact.cpp): the first launch searches only the boxes
 * that start before 2^-window_log2 and defers the others, each later launch
 * doubles the window, so the boxes of all candidates are searched roughly in
 * time order and the running minimum, once found, skips every later box.
 * -1 the built-in choice (2^-6 from 65,536 candidates on, else none), 0 no
 * windows.  The earliest time of impact
 * is the same bits either way; only the work differs. */
int rigc_set_ccd_window(rigc_ctx* ctx, int32_t window_log2);

/* DistanceBarrierConstraint::compute_earliest_toi
 * (src/opt/distance_barrier_constraint.cpp:130-149) with trajectory
 * PIECEWISE_LINEAR: continuous broad phase with inflation dmin / 2, then the
 * piecewise-linear narrow phase. */
int rigc_compute_earliest_toi_piecewise_linear(rigc_ctx* ctx, const double* x0,
                                               const double* x1, double dmin,
                                               double* toi_host);

/* ---- constraint set: DistanceBarrierConstraint::construct_constraint_set
 * (src/opt/distance_barrier_constraint.cpp:267-306): discrete broad phase
 * with inflation (dhat + dmin) / 2, then ipc::construct_constraint_set. */
int rigc_construct_constraint_set(rigc_ctx* ctx, const double* x, double dhat,
                                  double dmin, rigc_constraints* out);

/* ---- minimum distance: DistanceBarrierRBProblem::compute_min_distance(x)
 * (src/problems/distance_barrier_rb_problem.cpp:1583-1589) over
 * DistanceBarrierConstraint::compute_minimum_distance
 * (src/opt/distance_barrier_constraint.cpp:308-323), called by
 * IPCSolver::init_solve / post_step_update (src/solvers/ipc_solver.cpp:36-89):
 * the constraint set at x (device poses), the smallest constraint distance
 * over it; -1 when the set is empty, as the reference returns for an
 * infinite minimum.  Leaves that constraint set in the context. */
int rigc_min_distance(rigc_ctx* ctx, const double* x, double dhat, double dmin,
                      double* min_distance);

/* ---- intersection check: RigidBodyProblem::detect_intersections
 * (src/physics/rigid_body_problem.cpp:289-360), run at the end of every
 * time step (SimState::simulation_step, src/SimState.cpp:374-395, logs
 * has_intersections): edge-face candidates of the bodies
 * at x (device poses; close bodies and element boxes with no inflation) and
 * a segment-triangle crossing test on each.  Writes the number of crossing
 * (edge, face) pairs; the poses are intersection-free when it is 0.  The
 * segment-triangle test is the orientation-based one: the edge's endpoints
 * on different sides of the face's plane (coplanar pairs do not count) and
 * the edge's line inside the face. */
int rigc_detect_intersections(rigc_ctx* ctx, const double* x, int64_t* num_crossings);

/* Replace the context's constraint set with host arrays (same layout as
 * rigc_constraints). */
int rigc_set_constraints(rigc_ctx* ctx, int64_t num, const int32_t* type,
                         const int32_t* verts, const int32_t* prims,
                         const int32_t* bodies, const double* weight,
                         const double* eps_x);

/* ---- barrier term: DistanceBarrierRBProblem::compute_barrier_term
 * (src/problems/distance_barrier_rb_problem.hpp:267-273, .cpp:1299-1399)
 * over the context's constraint set. */
int rigc_barrier_term(rigc_ctx* ctx, const double* x, double dhat, double dmin,
                      int flags, rigc_barrier_out* out);

/* Per-constraint energy, body-space gradient (12) and 12x12 Hessian before
 * assembly (apply_chain_rule, distance_barrier_rb_problem.cpp:1182-1248).
 * Device outputs; any may be NULL. */
int rigc_barrier_local_terms(rigc_ctx* ctx, const double* x, double dhat,
                             double dmin, int flags, double* energy,
                             double* grad, double* hess);

/* Per-body state at the start of the time step (device pointers). */
typedef struct rigc_body_state {
    const double* mass;        /* num_bodies                                 */
    const double* moment;      /* num_bodies x 3, principal moments          */
    const double* x_t0;        /* num_bodies x 6, pose [p, theta]            */
    const double* v_t0;        /* num_bodies x 6, [v world, omega body]      */
    const double* Qdot_t0;     /* num_bodies x 9, dR/dt row-major            */
    const int32_t* dof_fixed;  /* num_bodies, bit k set when dof k is fixed  */
} rigc_body_state;

/* ---- inertial energy: DistanceBarrierRBProblem::compute_energy_term with
 * implicit Euler (src/problems/distance_barrier_rb_problem.cpp:706-944).
 * Per dynamic body E = 1/2 m q.q - m q.(q0 + h (v0 + h g))
 * + 1/2 tr(Q J Q^T) - tr(Q J (Q0 + h Qdot0)^T).  Outputs: energy (host,
 * summed), grad (device, 6 per body), hess (device, 36 per body, the
 * body's diagonal 6x6 block, row-major); grad / hess may be NULL. */
int rigc_body_energy(rigc_ctx* ctx, const rigc_body_state* state,
                     const double* x, const double gravity[3], double h,
                     double* energy_host, double* grad, double* hess);

/* ---- lagged friction.
 * rigc_friction_setup replaces
 * DistanceBarrierRBProblem::update_friction_constraints
 * (src/problems/distance_barrier_rb_problem.cpp:168-188): from the context's
 * current collision constraint set (built by rigc_construct_constraint_set
 * at the start-of-step poses x_t0, device) it builds the friction constraints
 * of ipc-toolkit's construct_friction_constraint_set: per constraint the
 * normal force magnitude lambda = -kappa w b'(d) 2 sqrt(d) (dhat the barrier
 * activation distance, w the multiplicity), the closest-point parameters and
 * an orthonormal tangent basis at x_t0; coefficient_friction (mu) is kept
 * with them.  The set stays fixed until the next setup, as the reference
 * keeps it through a lagging iteration.  num_out (host, may be NULL). */
int rigc_friction_setup(rigc_ctx* ctx, const double* x_t0, double dhat,
                        double barrier_stiffness, double coefficient_friction,
                        int64_t* num_out);

/* Friction constraints as built (device pointers, valid until the next
 * setup): type / verts x 4 / bodies x 2 as rigc_constraints; coef x 9 per
 * constraint = lambda, closest-point parameters (EV alpha; EE alpha, beta;
 * FV b1, b2; 0 otherwise), tangent basis t1 (3), t2 (3). */
typedef struct rigc_friction_view {
    int64_t num;
    double mu;
    const int32_t* type;
    const int32_t* verts;
    const int32_t* bodies;
    const double* coef;
} rigc_friction_view;
int rigc_get_friction(rigc_ctx* ctx, rigc_friction_view* out);

/* Friction potential D(x) = sum mu lambda f0(|T^T Gamma (V(x) - V(x_t0))|)
 * with its body gradient and PSD-projected block-sparse Hessian:
 * DistanceBarrierRBProblem::compute_friction_term
 * (src/problems/distance_barrier_rb_problem.cpp:1469-1572) with
 * epsv_times_h = static_friction_speed_bound * timestep (:1436).  Outputs
 * as rigc_barrier_term (own buffers: a friction term and a barrier term can
 * be held at the same time). */
int rigc_friction_term(rigc_ctx* ctx, const double* x, double epsv_times_h,
                       int flags, rigc_barrier_out* out);

/* Per-constraint friction energy, body gradient (12) and 12x12 Hessian
 * before assembly (compute_friction_potential, :1411-1467).  Device outputs;
 * any may be NULL. */
int rigc_friction_local_terms(rigc_ctx* ctx, const double* x,
                              double epsv_times_h, int flags, double* energy,
                              double* grad, double* hess);

/* ---- time stepping.  DistanceBarrierRBProblem::simulation_step
 * (src/problems/distance_barrier_rb_problem.cpp:118-143) with the IPC Newton
 * solver (src/solvers/ipc_solver.cpp, src/solvers/newton_solver.cpp) for the
 * default settings: implicit Euler, velocity convergence, one friction
 * lagging iteration, kinematic bodies through the augmented Lagrangian
 * (their schedules: rigc_sim_set_kinematic).  Every term, the CCD
 * line-search filter and the Newton linear solve (a dense LDL^T for at most
 * 768 free dofs, else block-Jacobi preconditioned conjugate gradients on the
 * block-sparse Hessian, relative residual 1e-12, and when those do not
 * converge within 300 iterations the dense LDL^T for the rest of the step,
 * up to 8192 free dofs) run on the device; the solver's scalar decisions run
 * on the host.  Field names follow
 * the reference's JSON settings; average_mass and world_bbox_diagonal are the
 * values the problem computes at start-up (RigidBodyAssembler::average_mass,
 * rigid_body_assembler.cpp:104-118; the world bounding-box diagonal,
 * rigid_body_problem.cpp:91-94). */
typedef struct rigc_sim_params {
    double timestep;
    double gravity[3];
    double dhat;                        /* barrier activation distance      */
    double dmin;                        /* minimum separation distance      */
    double coefficient_friction;        /* mu; 0 disables friction          */
    double static_friction_speed_bound; /* eps_v                            */
    int32_t max_newton_iterations;      /* 3000                             */
    double velocity_conv_tol;           /* 1e-2                             */
    int32_t velocity_conv_tol_abs;      /* 0: relative to the bbox diagonal */
    double line_search_lower_bound;     /* 1e-12                            */
    double dhat_epsilon;                /* 1e-9                             */
    double min_barrier_stiffness_scale; /* 1e11                             */
    double average_mass;
    double world_bbox_diagonal;
    /* Full Newton steps (unprojected Hessian) after the solver converges,
     * while they keep contracting and the CCD admits them; 0 (the
     * reference's solver) by default.  The line search accepts a step only
     * when the objective decreases, which stalls at |dx| ~ sqrt(eps); the
     * differentiable rollout needs the solution to the rounding of the
     * gradient instead. */
    int32_t newton_polish;
    /* Bound of the line search's step when the CCD limits it: s * toi with
     * s in (0, 1] (1: the reference's solver).  s < 1 keeps the first step
     * into a contact from ending closer than (1 - s) of the gap, below the
     * rigid CCD's spatial resolution (1e-4 m), where the CCD's conservative
     * time of impact shrinks every following step. */
    double ccd_rescale;
    /* The line search's CCD: RIGC_TRAJECTORY_RIGID (0, the interval rigid
     * trajectory) or RIGC_TRAJECTORY_PIECEWISE_LINEAR (1, the reference's
     * JSON default; minimum separation dmin).  Plain contexts only. */
    int32_t trajectory_type;
} rigc_sim_params;

/* Bodies' state (host pointers, copied by rigc_sim_init). */
typedef struct rigc_sim_state {
    const double* mass;        /* num_bodies                                */
    const double* moment;      /* num_bodies x 3, principal moments         */
    const int32_t* dof_fixed;  /* num_bodies, bit k set when dof k is fixed */
    const double* poses;       /* num_bodies x 6 [p, theta]                 */
    const double* velocities;  /* num_bodies x 6 [v world, omega body]      */
    const double* Qdot;        /* num_bodies x 9, dR/dt row-major           */
} rigc_sim_state;

typedef struct rigc_step_stats {
    int64_t newton_iterations, newton_steps, objective_evals, ccd_calls, cg_iterations;
    double barrier_stiffness;  /* kappa after the last step               */
} rigc_step_stats;

/* Start a simulation on the context (barrier stiffness 1, as the reference
 * starts), advance it by num_steps steps (stats accumulated, may be NULL),
 * and read the state back (host outputs, any may be NULL).  The linear
 * velocities and Qdot advance; the angular velocities are left as given
 * (the implicit-Euler energy uses Qdot). */
int rigc_sim_init(rigc_ctx* ctx, const rigc_sim_params* params,
                  const rigc_sim_state* state);
int rigc_sim_step(rigc_ctx* ctx, int32_t num_steps, rigc_step_stats* stats);
int rigc_sim_get_state(rigc_ctx* ctx, double* poses, double* velocities,
                       double* Qdot, double* barrier_stiffness);

/* Batched contexts (rigc_ctx_create_batched): rigc_sim_step advances every
 * scene as its own problem -- the reference's simulation_step per scene,
 * with its own barrier stiffness, regularisation, CCD step bound, line
 * search, convergence and stiffness updates -- while each kernel runs over
 * all scenes at once; the per-scene linear solves are block-Jacobi PCG.
 * Friction and newton_polish are not supported there (RIGC_ERR_ARG).  Each
 * scene's average mass and world bounding-box diagonal (host arrays,
 * num_scenes values; NULL keeps rigc_sim_params' value) set after
 * rigc_sim_init. */
int rigc_sim_scene_params(rigc_ctx* ctx, const double* average_mass,
                          const double* bbox_diagonal);

/* A kinematic body's schedule (RigidBody::kinematic_max_time and
 * kinematic_poses, src/physics/rigid_body.hpp:260-261, read by
 * src/io/read_rb_scene.cpp:94-101,233-245), set after rigc_sim_init: each
 * time step drives the body to the next of the num_poses poses (host,
 * num_poses x 6: position, rotation vector; init_augmented_lagrangian,
 * src/problems/distance_barrier_rb_problem.cpp:204-226), then to x0 + h v
 * once they are used up; once max_time has run out (a negative max_time is
 * no limit) the body becomes static: every dof fixed, its velocity zero
 * (step_kinematic_bodies, :237-251).  Plain contexts; RIGC_ERR_ARG for a
 * body that is not kinematic. */
int rigc_sim_set_kinematic(rigc_ctx* ctx, int32_t body, double max_time, int64_t num_poses,
                           const double* poses);

/* ---- autotuner (new).  Times the narrow phase's launch shapes on the
 * context's own workload -- k_ccd's resident blocks per SM, the CCD frame
 * cache's slots per body, the CCD searches per candidate,
 * k_barrier_local's constraints per warp, the CCD boxes a search piece
 * evaluates before handing its pending boxes to the next launch, one CCD
 * search per lane, per warp or per half-warp -- one
 * after the other (median of three runs each), over the continuous
 * candidates of x0 -> x1 and the constraint set at x0 (device poses), and
 * keeps the fastest in the context for every later call.  rigc_set_tune
 * sets them directly: for ccd_blocks_per_sm, cache_slots_per_body and
 * barrier_per_warp 0 is the built-in choice; for ccd_seeds_log2,
 * ccd_hand_off and ccd_warp the built-in choice is -1 (0 means something
 * else there: one seed, never hand off, one search per lane). */
typedef struct rigc_tune_report {
    int32_t ccd_blocks_per_sm, cache_slots_per_body, barrier_per_warp;
    double ccd_ms_default, ccd_ms, barrier_ms_default, barrier_ms;
    int32_t ccd_seeds_log2;
    int32_t ccd_hand_off;
    int32_t ccd_warp;
    int32_t ccd_window_log2;  /* rigc_set_ccd_window's choice (-1: built-in) */
} rigc_tune_report;
int rigc_autotune(rigc_ctx* ctx, const double* x0, const double* x1, double dhat, double dmin,
                  rigc_tune_report* report);
/* ccd_seeds_log2: each candidate's search split into 2^k searches from the
 * nodes of its subdivision tree at depth k (0 .. 5; -1: chosen by the
 * candidate count).  ccd_hand_off: a search piece that has evaluated this
 * many boxes hands its pending boxes to a further k_ccd launch, so that deep
 * searches spread over the whole GPU (0: never; -1: the built-in 64).  The
 * earliest time of impact depends on neither.  ccd_warp: 0 searches one
 * candidate per lane (k_ccd), 1 one per warp with the lanes
 * evaluating each box together (k_ccd_group<32>: a tenth of the FP64 chain
 * per box; the built-in choice, -1), 2 / 3 the same fitted to 4 / 5 blocks
 * per SM (fewer registers, more warps to hide latency), 4 one per half-warp
 * (k_ccd_group<16>: two searches share each instruction of the warp), 5 the
 * same fitted to 4 blocks per SM.
 * The results are the same bits either way. */
int rigc_set_tune(rigc_ctx* ctx, int32_t ccd_blocks_per_sm, int32_t cache_slots_per_body,
                  int32_t barrier_per_warp, int32_t ccd_seeds_log2, int32_t ccd_hand_off,
                  int32_t ccd_warp);

/* ---- differentiation (new: the reference has no adjoint).
 * rigc_sim_rollout advances the simulation by num_steps steps like
 * rigc_sim_step and keeps the state before every checkpoint_every-th step on
 * the device.  rigc_sim_backward then takes the gradient of a loss with
 * respect to the state after the rollout (host arrays: poses num_bodies x 6,
 * velocities num_bodies x 6, Qdot num_bodies x 9; velocities and Qdot may be
 * NULL for zero) and writes its gradient with respect to the state before
 * it (host outputs of the same shapes).  Each step is differentiated
 * implicitly at its converged solution x*: H lambda = dL/dx* on the free
 * dofs with H the unprojected Hessian of E/m + kappa/m B assembled on the
 * device, then dL/ds = dL/ds|direct - (1/m) (d2E/dx ds)^T lambda, including
 * the dependence of the step's initial barrier stiffness on the state.
 * Steps between checkpoints are recomputed (bit-identical) from the
 * checkpoint, segment by segment from the last.  Friction is not
 * differentiated (RIGC_ERR_ARG when coefficient_friction > 0); use
 * newton_polish > 0 so that each step's gradient vanishes to rounding.
 * The simulation state is left as it was after the rollout. */
int rigc_sim_rollout(rigc_ctx* ctx, int32_t num_steps, int32_t checkpoint_every,
                     rigc_step_stats* stats);
int rigc_sim_backward(rigc_ctx* ctx, const double* d_poses, const double* d_velocities,
                      const double* d_Qdot, double* g_poses, double* g_velocities,
                      double* g_Qdot);

/* ---- one narrow-phase pass from host memory (the call a host Newton loop
 * makes per iteration): copies x0/x1 in, runs compute_earliest_toi(x0, x1)
 * and construct_constraint_set + compute_barrier_term at x0, copies the
 * gradient and the block-sparse Hessian out.  Host buffers: grad_host
 * (6 * num_bodies), row_ptr_host (num_bodies + 1), col_host / val_host of
 * capacity nnzb_cap blocks (nnzb always written). */
int rigc_narrow_phase_host(rigc_ctx* ctx, const double* x0_host,
                           const double* x1_host, double dhat, double dmin,
                           double* toi_host, double* energy_host,
                           double* grad_host, int32_t* row_ptr_host,
                           int32_t* col_host, double* val_host,
                           int64_t nnzb_cap, int64_t* nnzb_host);

/* ---- FP64 issue throughput (new: a measurement of the part, for the
 * rooflines of the FP64-bound kernels).  Runs independent chains of DFMA
 * (op 0) or DADD (op 1) on every resident warp of the device, with only
 * active_lanes lanes of each warp working, iters x 8 instructions per
 * thread, timed with CUDA events on the legacy default stream (one warm-up
 * launch first).  Outputs: elapsed ms, warp-level FP64 instructions issued
 * and lane-level FLOPs (2 per DFMA).  Allocates and frees a small device
 * buffer; synchronises the device. */
int rigc_fp64_throughput(int32_t op, int32_t active_lanes, int32_t iters, double* ms,
                         double* warp_instructions, double* lane_flops);

/* ---- per-constraint barrier terms without any device allocation.
 * No counterpart in the reference: the reference allocates freely on the
 * host.  This entry point is for callers that must not allocate device
 * memory at call time -- code that runs inside another framework's memory
 * pool or a fixed memory budget, or latency-critical loops where a
 * cudaMalloc / cudaFree would synchronise the device -- and that therefore
 * cannot create a rigc_ctx.  The caller passes every input and output as
 * device memory it already owns; the only working memory is a file-scope
 * device array inside the library (the per-body rotation frames) that holds
 * RIGC_NOALLOC_MAX_BODIES bodies, 3 MiB, and stays resident on every GPU that
 * loads the library until the process exits.
 *
 * Same results as rigc_barrier_local_terms for the same constraints.
 * Inputs (device): rest_vertices (num_vertices x 3, body frame), x (6 per
 * body), the constraint arrays in rigc_constraints layout (type, verts x 4,
 * bodies x 2, weight, eps_x).  Outputs (device, any may be NULL): energy
 * (num_constraints), grad (x 12), hess (x 144).  flags as rigc_barrier_term.
 * Returns RIGC_ERR_TOO_LARGE when num_bodies > RIGC_NOALLOC_MAX_BODIES.
 * Preconditions: 0 <= type <= 3, every body index in [0, num_bodies), every
 * vertex index the type uses in [0, num_vertices).  The arrays are on the
 * device, so the kernel checks them: a constraint that breaks one gets NaN
 * energy, gradient and Hessian and reads nothing out of range; the status
 * returned cannot report it (that would need a synchronisation).
 *
 * The first call on a device looks up the device address of the working
 * array (a one-time set-up per device); make that first call before any
 * stream capture.  Every call shares the one working array, so calls that
 * overlap on the GPU (different streams, or different host threads) race:
 * serialise them on one stream.  The array keeps the last call's contents;
 * each call overwrites every frame it reads. */
#define RIGC_NOALLOC_MAX_BODIES 4096
int rigc_barrier_local_terms_noalloc(
    const double* rest_vertices, int64_t num_vertices, int32_t num_bodies, const double* x,
    int64_t num_constraints, const int32_t* type, const int32_t* verts,
    const int32_t* bodies, const double* weight, const double* eps_x,
    double dhat, double dmin, int flags, double* energy, double* grad,
    double* hess, void* cuda_stream);

#ifdef __cplusplus
}
#endif

#endif /* RIGC_H */
