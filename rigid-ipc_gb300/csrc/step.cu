// Time stepping on the device: the rigid IPC problem's simulation step with
// the IPC Newton solver, every term, the collision filtering and the linear
// solve on the GPU, the solver's scalar decisions on the host.
//
// Replaces DistanceBarrierRBProblem::simulation_step
// (src/problems/distance_barrier_rb_problem.cpp:118-143) for the default
// settings (implicit Euler, IPC solver with velocity convergence, one friction
// lagging iteration, no kinematic bodies):
//  * update_constraints (:145-166): lagged friction constraints at the
//    start-of-step poses x0 with the current barrier stiffness;
//  * IPCSolver::init_solve (src/solvers/ipc_solver.cpp:36-65): initial
//    stiffness from the energy and barrier gradients at x0 (ipc-toolkit's
//    initial_barrier_stiffness: argmin |grad E + kappa grad B| clamped to
//    [kappa_min, 100 kappa_min], kappa_min = scale m / (4 d0 b''(d0)),
//    d0 = (1e-8 bbox + dmin)^2) and the initial minimum distance;
//  * NewtonSolver::solve (src/solvers/newton_solver.cpp:158-300): objective
//    E/m + kappa/m B + D/m (compute_objective, :633-703) on the free degrees
//    of freedom, regularised Newton direction (:421-478; H + c I with c
//    doubling from 1e-8 while the solve fails or is not a descent direction,
//    halving after a success), velocity convergence (:95-140), line search
//    over [0, min(toi(x, x + d), 1)] halving until the objective decreases
//    (:302-418), the gradient fallback, and the adaptive stiffness update
//    (ipc_solver.cpp:67-89: kappa doubles, up to 100 kappa_min, while the
//    minimum distance keeps shrinking below dhat_epsilon (bbox + dmin));
//  * take_step (:488-626): implicit-Euler v and Qdot.
// The Newton system on the free dofs is factorised densely (blocked LDL^T
// without pivoting) when it has at most kDenseMax unknowns, else solved by
// preconditioned conjugate gradients on the block-sparse Hessian (6x6 blocks:
// body energy + barrier + friction) with a block-Jacobi preconditioner, to a
// relative residual of 1e-12.  A failed solve (zero pivot, non-positive
// curvature, no convergence) counts as a failed factorisation in the
// reference and raises the regularisation.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <array>
#include <deque>
#include <vector>

#include "common.cuh"
#include "geometry_rn.cuh"
#include "rotation.cuh"
#include "sort.cuh"

namespace rigc {

int construct_constraints(Ctx& c, const double* x, double dhat, double dmin);
int detect_and_count(Ctx& c, const double* x0, const double* x1, bool continuous, double infl);
int compute_world_vertices_rn(Ctx& c, const double* x, double* V, DevBuf& rotbuf);
int body_energy(Ctx& c, const rigc_body_state& s, const double* x, const double gravity[3],
                double h, double* energy_host, double* grad, double* hess);
int friction_setup(Ctx& c, const double* x0, double dhat, double kappa, double mu, double dmin);
int friction_term(Ctx& c, const double* x, double epsvh, int flags, rigc_barrier_out* out);
int barrier_term_impl(Ctx& c, const double* x, double dhat, double dmin, int flags,
                      rigc_barrier_out* out);
int run_ccd(Ctx& c, const double* x0, const double* x1, double toi_tol, int flags,
            double* toi_host, double* per);
int run_pl_ccd(Ctx& c, const double* x0, const double* x1, double dmin, double* toi_host, double* per);

// the line search's CCD over the candidates just found: the rigid interval
// trajectory (time tolerance 1e-4) or the piecewise-linear one with minimum
// separation dmin (DistanceBarrierConstraint::compute_earliest_toi with the
// scene's trajectory_type)
static int line_search_ccd(Ctx& c, const rigc_sim_params& p, const double* x, const double* xt,
                           double* toi)
{
    if (p.trajectory_type == RIGC_TRAJECTORY_PIECEWISE_LINEAR)
        return run_pl_ccd(c, x, xt, p.dmin, toi, nullptr);
    return run_ccd(c, x, xt, 1e-4, 0, toi, nullptr);
}

namespace {

// ---------------------------------------------------------------------------
// kernels

__global__ void k_axpy(int64_t n, double a, const double* __restrict__ x,
                       const double* __restrict__ y, double* __restrict__ out)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = y[i] + a * x[i];
}

// g = gE / m + (kappa / m) gB + gD / m, zero on fixed degrees of freedom
__global__ void k_combine_grad(int nb, const double* __restrict__ gE, const double* __restrict__ gB,
                               const double* __restrict__ gD, double sE, double sB, double sD,
                               const int* __restrict__ fixed, double* __restrict__ g)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 6 * nb) return;
    double v = sE * gE[i];
    if (gB) v += sB * gB[i];
    if (gD) v += sD * gD[i];
    g[i] = ((fixed[i / 6] >> (i % 6)) & 1) ? 0.0 : v;
}

struct HessView {
    const double* body;      // nb x 36 (scale sE)
    const int* brp;          // barrier BSR (scale sB)
    const int* bcol;
    const double* bval;
    const int* frp;          // friction BSR (scale sD)
    const int* fcol;
    const double* fval;
    double sE, sB, sD, reg;  // scales and the regularisation c (H + c I)
    const int* fixed;
    int nb;
    // batched contexts: per-scene scales and regularisation, by body scene
    // (used instead of sE, sB, sD, reg when bscene is set)
    const int* bscene = nullptr;
    const double* scE = nullptr;
    const double* scB = nullptr;
    const double* scReg = nullptr;
};

// the scales of body b's rows: (sE, sB, sD, reg)
__device__ __forceinline__ void row_scales(const HessView& H, int b, double& sE, double& sB,
                                           double& sD, double& reg)
{
    if (H.bscene) {
        const int sc = H.bscene[b];
        sE = H.scE[sc];
        sB = H.scB[sc];
        sD = sE;
        reg = H.scReg[sc];
    } else {
        sE = H.sE;
        sB = H.sB;
        sD = H.sD;
        reg = H.reg;
    }
}

// row i of y = H x on the free degrees of freedom (fixed rows and columns
// removed)
__device__ __forceinline__ void hess_row(const HessView& H, int i, const double* __restrict__ x,
                                         double* __restrict__ y)
{
    const int b = i / 6, r = i % 6;
    if ((H.fixed[b] >> r) & 1) {
        y[i] = 0;
        return;
    }
    double sE, sB, sD, reg;
    row_scales(H, b, sE, sB, sD, reg);
    double acc = 0;
    const double* Bb = H.body + 36 * (size_t)b + 6 * r;
    for (int c = 0; c < 6; c++) acc += sE * Bb[c] * x[6 * b + c];
    if (H.brp)
        for (int k = H.brp[b]; k < H.brp[b + 1]; k++) {
            const double* V = H.bval + 36 * (size_t)k + 6 * r;
            const int cb = H.bcol[k];
            for (int c = 0; c < 6; c++) acc += sB * V[c] * x[6 * cb + c];
        }
    if (H.frp)
        for (int k = H.frp[b]; k < H.frp[b + 1]; k++) {
            const double* V = H.fval + 36 * (size_t)k + 6 * r;
            const int cb = H.fcol[k];
            for (int c = 0; c < 6; c++) acc += sD * V[c] * x[6 * cb + c];
        }
    y[i] = acc + reg * x[i];
}

__global__ void k_hess_matvec(HessView H, const double* __restrict__ x, double* __restrict__ y)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 6 * H.nb) hess_row(H, i, x, y);
}

// the same with the view read from device memory (the CG graphs keep their
// arguments fixed; the view's scales change between solves)
__global__ void k_hess_matvec_dev(const HessView* __restrict__ Hp, const double* __restrict__ x,
                                  double* __restrict__ y)
{
    const HessView H = *Hp;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 6 * H.nb) hess_row(H, i, x, y);
}

// inverse of each body's diagonal 6x6 block (free part; fixed rows and
// columns become the identity), by Cholesky; a block that is not positive
// definite falls back to the inverse of its absolute diagonal
__global__ void k_block_jacobi(HessView H, double* __restrict__ Minv)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= H.nb) return;
    double sE, sB, sD, reg;
    row_scales(H, b, sE, sB, sD, reg);
    double A[36];
    for (int k = 0; k < 36; k++) A[k] = sE * H.body[36 * (size_t)b + k];
    if (H.brp)
        for (int k = H.brp[b]; k < H.brp[b + 1]; k++)
            if (H.bcol[k] == b)
                for (int e = 0; e < 36; e++) A[e] += sB * H.bval[36 * (size_t)k + e];
    if (H.frp)
        for (int k = H.frp[b]; k < H.frp[b + 1]; k++)
            if (H.fcol[k] == b)
                for (int e = 0; e < 36; e++) A[e] += sD * H.fval[36 * (size_t)k + e];
    const int fx = H.fixed[b];
    for (int r = 0; r < 6; r++) {
        A[7 * r] += reg;
        for (int c = 0; c < 6; c++)
            if (((fx >> r) & 1) || ((fx >> c) & 1)) A[6 * r + c] = r == c ? 1.0 : 0.0;
    }
    // Cholesky A = L L^T
    double L[36];
    bool pd = true;
    for (int k = 0; k < 36; k++) L[k] = 0;
    for (int j = 0; j < 6 && pd; j++) {
        double d = A[7 * j];
        for (int k = 0; k < j; k++) d -= L[6 * j + k] * L[6 * j + k];
        if (!(d > 0)) {
            pd = false;
            break;
        }
        double ljj = sqrt(d);
        L[7 * j] = ljj;
        for (int i = j + 1; i < 6; i++) {
            double s = 0.5 * (A[6 * i + j] + A[6 * j + i]);
            for (int k = 0; k < j; k++) s -= L[6 * i + k] * L[6 * j + k];
            L[6 * i + j] = s / ljj;
        }
    }
    double* M = Minv + 36 * (size_t)b;
    if (!pd) {
        for (int r = 0; r < 6; r++)
            for (int c = 0; c < 6; c++) {
                double a = fabs(A[7 * r]);
                M[6 * r + c] = r == c ? (a > 0 ? 1.0 / a : 1.0) : 0.0;
            }
        return;
    }
    // columns of A^-1 by two triangular solves
    for (int c = 0; c < 6; c++) {
        double y[6];
        for (int i = 0; i < 6; i++) {
            double s = i == c ? 1.0 : 0.0;
            for (int k = 0; k < i; k++) s -= L[6 * i + k] * y[k];
            y[i] = s / L[7 * i];
        }
        for (int i = 5; i >= 0; i--) {
            double s = y[i];
            for (int k = i + 1; k < 6; k++) s -= L[6 * k + i] * y[k];
            y[i] = s / L[7 * i];
        }
        for (int i = 0; i < 6; i++) M[6 * i + c] = y[i];
    }
}

__global__ void k_block_apply(int nb, const double* __restrict__ Minv, const double* __restrict__ r,
                              const int* __restrict__ fixed, double* __restrict__ z)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 6 * nb) return;
    const int b = i / 6, row = i % 6;
    double acc = 0;
    const double* M = Minv + 36 * (size_t)b + 6 * row;
    for (int c = 0; c < 6; c++) acc += M[c] * r[6 * b + c];
    z[i] = ((fixed[b] >> row) & 1) ? 0.0 : acc;
}

// deterministic dot product: 256 partial sums, then one block
__global__ void k_dot_partial(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                              double* __restrict__ part)
{
    __shared__ double sh[256];
    double s = 0;
    for (int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256)
        s += a[i] * b[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_dot_final(const double* __restrict__ part, int m, double* __restrict__ out)
{
    __shared__ double sh[256];
    sh[threadIdx.x] = threadIdx.x < m ? part[threadIdx.x] : 0.0;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

// CG step length on the device: alpha = rz / pAp, or 0 once the residual
// is within the tolerance (then the iteration has converged, and a zero
// direction is not a breakdown)
__global__ void k_cg_alpha(const double* __restrict__ rz, const double* __restrict__ pAp,
                           const double* __restrict__ rr, const double* __restrict__ tol2,
                           double* __restrict__ alpha, int* __restrict__ flags)
{
    if (flags[1] || *rr <= *tol2) {
        flags[1] = 1;  // converged
        *alpha = 0;
        return;
    }
    const double d = *pAp;
    if (!(d > 0) || !isfinite(d)) {
        flags[0] = 1;  // breakdown: not positive definite
        *alpha = 0;
    } else {
        *alpha = *rz / d;
    }
}

// x += alpha p; r -= alpha Ap
__global__ void k_cg_update(int64_t n, const double* __restrict__ alpha, const double* __restrict__ p,
                            const double* __restrict__ Ap, double* __restrict__ x,
                            double* __restrict__ r)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double a = *alpha;
    x[i] += a * p[i];
    r[i] -= a * Ap[i];
}

// p = z + (rz_new / rz_old) p (unchanged once converged)
__global__ void k_cg_direction(int64_t n, const double* __restrict__ rz_new,
                               const double* __restrict__ rz_old, const double* __restrict__ z,
                               const int* __restrict__ flags, double* __restrict__ p)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || flags[0] || flags[1]) return;
    p[i] = z[i] + (*rz_new / *rz_old) * p[i];
}

// Last node of the CG graph's loop body: counts the iteration and ends the
// loop once the solve converged (flag or residual within tolerance), broke
// down (flag or a non-finite residual) or ran max_it iterations.
__global__ void k_cg_continue(const int* __restrict__ flags, const double* __restrict__ rr,
                              const double* __restrict__ tol2, long long* __restrict__ iters,
                              long long max_it, cudaGraphConditionalHandle loop)
{
    const long long it = ++*iters;
    const double v = *rr;
    const bool end = flags[0] || flags[1] || v <= *tol2 || !isfinite(v) || it >= max_it;
    cudaGraphSetConditional(loop, end ? 0u : 1u);
}

// largest |V(x1) - V(x0)| coordinate over all vertices (max of non-negative
// doubles through their bit patterns)
__global__ void k_max_vertex_move(int nv, const double* __restrict__ V0, const double* __restrict__ V1,
                                  unsigned long long* __restrict__ out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double m = 0;
    if (i < 3 * nv) m = fabs(V1[i] - V0[i]);
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// smallest squared distance of the constraint set (the distance each barrier
// uses, in the round-to-nearest order of the constraint set)
__global__ void k_min_constraint_distance(int64_t n, const int* __restrict__ type,
                                          const int* __restrict__ verts, const double* __restrict__ V,
                                          unsigned long long* __restrict__ out)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double d = INFINITY;
    if (i < n) {
        const int t = type[i];
        const double* P[4];
        for (int k = 0; k < 4; k++) {
            int v = verts[4 * i + k];
            P[k] = V + 3 * (size_t)(v < 0 ? 0 : v);
        }
        if (t == 0) d = pp_sqdist_rn(P[0], P[1]);
        else if (t == 1) d = pl_sqdist_rn(P[0], P[1], P[2]);
        else if (t == 2) d = ee_sqdist_rn(P[0], P[1], P[2], P[3]);
        else d = ptplane_sqdist_rn(P[0], P[1], P[2], P[3]);
    }
    for (int o = 16; o > 0; o >>= 1) d = fmin(d, __shfl_xor_sync(0xffffffffu, d, o));
    if ((threadIdx.x & 31) == 0) atomicMin(out, (unsigned long long)__double_as_longlong(d));
}

// implicit-Euler update of the dynamic bodies: v = (q - q0) / h,
// Qdot = (R(theta) - R(theta0)) / h, then the poses
__global__ void k_take_step(int nb, const int* __restrict__ type, const int* __restrict__ fixed,
                            const double* __restrict__ x, double* __restrict__ x0,
                            double* __restrict__ v, double* __restrict__ Qdot, double h)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    if (type[b] == RIGC_BODY_DYNAMIC) {
        double Q[9], Q0[9];
        const double t[3] = { x[6 * b + 3], x[6 * b + 4], x[6 * b + 5] };
        const double t0[3] = { x0[6 * b + 3], x0[6 * b + 4], x0[6 * b + 5] };
        rot_rn(t, Q);
        rot_rn(t0, Q0);
        for (int k = 0; k < 3; k++)
            v[6 * b + k] = ((fixed[b] >> k) & 1) ? 0.0 : (x[6 * b + k] - x0[6 * b + k]) / h;
        for (int k = 0; k < 9; k++) Qdot[9 * b + k] = (Q[k] - Q0[k]) / h;
    }
    for (int k = 0; k < 6; k++) x0[6 * b + k] = x[6 * b + k];
}

// DistanceBarrierConstraint::construct_constraint_set: discrete candidates
// with inflation (dhat + dmin) / 2, then the constraint set
int build_constraints(Ctx& c, const double* x, double dhat, double dmin)
{
    if (c.s.nb <= 1) {
        c.cons.num = c.cons.num_vv = c.cons.num_ev = c.cons.num_ee = c.cons.num_fv = 0;
        return RIGC_OK;
    }
    RIGC_TRY(detect_and_count(c, x, x, false, (dhat + dmin) / 2.0));
    return construct_constraints(c, x, dhat, dmin);
}

// dense copy of the free part of H + reg I: one thread per (body, row)
__global__ void k_dense_fill(HessView H, const int* __restrict__ free_idx, int nfree,
                             double* __restrict__ A)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 6 * H.nb) return;
    const int b = i / 6, r = i % 6;
    const int fi = free_idx[i];
    if (fi < 0) return;
    double* row = A + (size_t)fi * nfree;
    for (int c = 0; c < 6; c++) {
        const int fj = free_idx[6 * b + c];
        if (fj >= 0) row[fj] += H.sE * H.body[36 * (size_t)b + 6 * r + c];
    }
    if (H.brp)
        for (int k = H.brp[b]; k < H.brp[b + 1]; k++) {
            const int cb = H.bcol[k];
            for (int c = 0; c < 6; c++) {
                const int fj = free_idx[6 * cb + c];
                if (fj >= 0) row[fj] += H.sB * H.bval[36 * (size_t)k + 6 * r + c];
            }
        }
    if (H.frp)
        for (int k = H.frp[b]; k < H.frp[b + 1]; k++) {
            const int cb = H.fcol[k];
            for (int c = 0; c < 6; c++) {
                const int fj = free_idx[6 * cb + c];
                if (fj >= 0) row[fj] += H.sD * H.fval[36 * (size_t)k + 6 * r + c];
            }
        }
    row[fi] += H.reg;
}

// Dense LDL^T (no pivoting) of the free part of the Hessian, blocked: for
// each panel of kPanel columns, k_ldlt_panel factorises the panel (rows
// j0..n-1) in shared memory, one column at a time (d_c = a_cc,
// l_rc = a_rc / d_c, then a_rc' -= l_rc d_c l_c'c within the panel), and
// k_ldlt_update applies the panel to the trailing lower triangle
// (A22 -= L21 D L21^T) in 32 x 32 tiles over many CTAs.  k_ldlt_solve then
// solves L D L^T x = b with blocked forward and backward substitution in one
// CTA.  flags[0] = 1 on a zero or non-finite pivot or a non-finite solution.
// A's lower triangle is overwritten by L (unit diagonal implied), D by the
// pivots.
constexpr int kPanel = 32;
constexpr int kPanelStride = kPanel + 1;  // shared-memory row stride (no bank conflicts down a column)

__global__ void __launch_bounds__(512) k_ldlt_panel(double* __restrict__ A, int n, int j0, int rows,
                                                    double* __restrict__ D, int* __restrict__ flags)
{
    extern __shared__ double P[];  // rows x kPanel, row stride kPanelStride
    const int m = min(rows, n - j0), w = min(kPanel, n - j0);
    if (flags[0]) return;
    for (int e = threadIdx.x; e < m * w; e += blockDim.x) {
        const int r = e / w, c = e % w;
        P[r * kPanelStride + c] = r >= c ? A[(size_t)(j0 + r) * n + j0 + c] : 0.0;
    }
    __syncthreads();
    bool bad = false;
    for (int c = 0; c < w; c++) {
        const double d = P[c * kPanelStride + c];
        if (!(fabs(d) > 0) || !isfinite(d)) {
            bad = true;
            break;
        }
        for (int r = c + 1 + threadIdx.x; r < m; r += blockDim.x) P[r * kPanelStride + c] /= d;
        __syncthreads();
        // a_rc' -= l_rc d l_c'c for c < c' <= r
        const int cols = w - c - 1;
        for (int e = threadIdx.x; e < (m - c - 1) * cols; e += blockDim.x) {
            const int r = c + 1 + e / cols, cc = c + 1 + e % cols;
            if (cc <= r) P[r * kPanelStride + cc] -= P[r * kPanelStride + c] * d * P[cc * kPanelStride + c];
        }
        __syncthreads();
    }
    if (bad) {
        if (threadIdx.x == 0) flags[0] = 1;
        return;
    }
    for (int e = threadIdx.x; e < m * w; e += blockDim.x) {
        const int r = e / w, c = e % w;
        if (r > c) A[(size_t)(j0 + r) * n + j0 + c] = P[r * kPanelStride + c];
        else if (r == c) D[j0 + c] = P[r * kPanelStride + c];
    }
}

// Systems too large for a panel in shared memory: after k_ldlt_panel has
// factorised the panel's w x w diagonal block, each row r below it takes its
// panel entries through the same column-by-column elimination as
// k_ldlt_panel's (divide by the pivot, then subtract l_rc d_c l_c'c from the
// later columns), one thread per row
__global__ void __launch_bounds__(128) k_ldlt_trsm(double* __restrict__ A, int n, int j0, int w,
                                                   const double* __restrict__ D,
                                                   const int* __restrict__ flags)
{
    if (flags[0]) return;
    __shared__ double L[kPanel][kPanel + 1], d[kPanel];
    for (int e = threadIdx.x; e < kPanel * kPanel; e += blockDim.x) {
        const int r = e / kPanel, c = e % kPanel;
        L[r][c] = (r < w && c < r) ? A[(size_t)(j0 + r) * n + j0 + c] : 0.0;
    }
    if (threadIdx.x < kPanel) d[threadIdx.x] = threadIdx.x < w ? D[j0 + threadIdx.x] : 1.0;
    __syncthreads();
    const int r = j0 + w + blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double x[kPanel];
#pragma unroll
    for (int c = 0; c < kPanel; c++) x[c] = c < w ? A[(size_t)r * n + j0 + c] : 0.0;
#pragma unroll
    for (int c = 0; c < kPanel; c++) {
        if (c >= w) break;
        x[c] /= d[c];
#pragma unroll
        for (int cc = c + 1; cc < kPanel; cc++)
            if (cc < w) x[cc] -= x[c] * d[c] * L[cc][c];
    }
#pragma unroll
    for (int c = 0; c < kPanel; c++)
        if (c < w) A[(size_t)r * n + j0 + c] = x[c];
}

// A[i][k] -= sum_c L[i][c] D[c] L[k][c] over the panel columns c, for the
// trailing lower triangle i >= k >= j0 + w; one 32 x 32 tile per CTA
__global__ void __launch_bounds__(256) k_ldlt_update(double* __restrict__ A, int n, int j0, int w,
                                                     const double* __restrict__ D,
                                                     const int* __restrict__ flags)
{
    if (flags[0]) return;
    // tile (bi, bk), bi >= bk, from the linear block index
    const int t = blockIdx.x;
    int bi = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
    while ((bi + 1) * (bi + 2) / 2 <= t) bi++;
    while (bi * (bi + 1) / 2 > t) bi--;
    const int bk = t - bi * (bi + 1) / 2;
    const int base = j0 + w;
    const int i0 = base + 32 * bi, k0 = base + 32 * bk;
    __shared__ double Li[32][kPanel + 1], Lk[32][kPanel + 1], d[kPanel];
    for (int e = threadIdx.x; e < 32 * kPanel; e += blockDim.x) {
        const int r = e / kPanel, c = e % kPanel;
        Li[r][c] = (i0 + r < n && c < w) ? A[(size_t)(i0 + r) * n + j0 + c] : 0.0;
        Lk[r][c] = (k0 + r < n && c < w) ? A[(size_t)(k0 + r) * n + j0 + c] : 0.0;
    }
    if (threadIdx.x < kPanel) d[threadIdx.x] = threadIdx.x < w ? D[j0 + threadIdx.x] : 0.0;
    __syncthreads();
    for (int e = threadIdx.x; e < 32 * 32; e += blockDim.x) {
        const int r = e / 32, q = e % 32;
        const int i = i0 + r, k = k0 + q;
        if (i >= n || k >= n || k > i) continue;
        double acc = 0;
        for (int c = 0; c < w; c++) acc += Li[r][c] * d[c] * Lk[q][c];
        A[(size_t)i * n + k] -= acc;
    }
}

// L D L^T x = b by blocks of 32: y = L^-1 b, y /= D, x = L^-T y
__global__ void __launch_bounds__(256) k_ldlt_solve(const double* __restrict__ A, int n,
                                                    const double* __restrict__ D,
                                                    const double* __restrict__ b,
                                                    double* __restrict__ x, int* __restrict__ flags)
{
    if (flags[0]) return;
    __shared__ double Lb[32][33];  // the diagonal block of the current block row
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = b[i];
    __syncthreads();
    // forward: rows of block [b0, b0 + 32) minus the solved columns [0, b0)
    for (int b0 = 0; b0 < n; b0 += 32) {
        const int nb = min(32, n - b0);
        for (int r = warp; r < nb; r += 8) {
            double acc = 0;
            for (int k = lane; k < b0; k += 32) acc += A[(size_t)(b0 + r) * n + k] * x[k];
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0) x[b0 + r] -= acc;
        }
        for (int e = threadIdx.x; e < nb * 32; e += blockDim.x) {
            const int r = e / 32, q = e % 32;
            Lb[r][q] = q < nb ? A[(size_t)(b0 + r) * n + b0 + q] : 0.0;
        }
        __syncthreads();
        if (warp == 0) {
            double y = lane < nb ? x[b0 + lane] : 0.0;
            for (int r = 1; r < nb; r++) {
                const double yr = __shfl_sync(0xffffffffu, y, r - 1);
                // lanes >= r subtract column r - 1
                if (lane >= r && lane < nb) y -= Lb[lane][r - 1] * yr;
            }
            if (lane < nb) x[b0 + lane] = y;
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] /= D[i];
    __syncthreads();
    // backward: block [b0, b0 + 32) minus the solved rows [b0 + 32, n)
    for (int b0 = ((n - 1) / 32) * 32; b0 >= 0; b0 -= 32) {
        const int nb = min(32, n - b0);
        for (int r = warp; r < nb; r += 8) {
            double acc = 0;
            for (int k = b0 + 32 + lane; k < n; k += 32) acc += A[(size_t)k * n + b0 + r] * x[k];
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0) x[b0 + r] -= acc;
        }
        for (int e = threadIdx.x; e < nb * 32; e += blockDim.x) {
            const int r = e / 32, q = e % 32;
            Lb[r][q] = q < nb ? A[(size_t)(b0 + r) * n + b0 + q] : 0.0;
        }
        __syncthreads();
        if (warp == 0) {
            double y = lane < nb ? x[b0 + lane] : 0.0;
            for (int r = nb - 1; r > 0; r--) {
                const double yr = __shfl_sync(0xffffffffu, y, r);
                // lanes < r subtract row r's entry in their column
                if (lane < r) y -= Lb[r][lane] * yr;
            }
            if (lane < nb) x[b0 + lane] = y;
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        if (!isfinite(x[i])) flags[0] = 1;
}

// ---------------------------------------------------------------------------
// augmented Lagrangian of kinematic bodies
// (DistanceBarrierRBProblem::compute_augmented_lagrangian,
// src/problems/distance_barrier_rb_problem.cpp:946-1109): for a kinematic
// body with target x_pred = x0 + h v (init_augmented_lagrangian, :190-235)
//   kq/2 m |q - q_pred|^2 - sqrt(m) lam.(q - q_pred)
//   + kQ/2 tr((Q - Q_pred) J (Q - Q_pred)^T) - tr(Lam^T (Q - Q_pred) Js)
// with J = diag(1/2 (-I0 + I1 + I2), ...) and Js = sqrt(J).

__device__ __forceinline__ void al_J(const double* I, double J[3], double Js[3])
{
    J[0] = 0.5 * (-I[0] + I[1] + I[2]);
    J[1] = 0.5 * (I[0] - I[1] + I[2]);
    J[2] = 0.5 * (I[0] + I[1] - I[2]);
    for (int k = 0; k < 3; k++) Js[k] = sqrt(fmax(J[k], 0.0));
}

__global__ void k_al_init(int nb, const int* __restrict__ type, const double* __restrict__ x0,
                          const double* __restrict__ v, double h, const double* __restrict__ target,
                          double* __restrict__ xpred, double* __restrict__ lam, double* __restrict__ Lam)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    // a kinematic body's target: its scheduled pose, else x0 + h v
    const bool to_pose = type[b] == RIGC_BODY_KINEMATIC && target && !isnan(target[6 * b]);
    for (int k = 0; k < 6; k++)
        xpred[6 * b + k] = to_pose ? target[6 * b + k]
                                   : x0[6 * b + k] + (type[b] == RIGC_BODY_KINEMATIC ? h * v[6 * b + k] : 0.0);
    for (int k = 0; k < 3; k++) lam[3 * b + k] = 0;
    for (int k = 0; k < 9; k++) Lam[9 * b + k] = 0;
}

// energies (per body, 0 for the others) and, when asked, gradient and
// Hessian blocks added into the body-energy arrays
__global__ void k_al_terms(int nb, const int* __restrict__ type, const double* __restrict__ x,
                           const double* __restrict__ xpred, const double* __restrict__ mass,
                           const double* __restrict__ moment, const double* __restrict__ lam,
                           const double* __restrict__ Lam, double kq, double kQ,
                           double* __restrict__ energy, double* __restrict__ grad,
                           double* __restrict__ hess)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    if (type[b] != RIGC_BODY_KINEMATIC) {
        energy[b] = 0;
        return;
    }
    const double m = mass[b], sm = sqrt(m);
    const double* q = x + 6 * b;
    const double* qp = xpred + 6 * b;
    double e = 0;
    for (int i = 0; i < 3; i++) {
        const double d = q[i] - qp[i];
        e += kq / 2 * m * d * d - sm * lam[3 * b + i] * d;
        if (grad) grad[6 * b + i] += kq * m * d - sm * lam[3 * b + i];
        if (hess) hess[36 * (size_t)b + 7 * i] += kq * m;
    }
    double J[3], Js[3];
    al_J(moment + 3 * b, J, Js);
    double F[kFrameDoubles], Qp[9];
    const double t[3] = { q[3], q[4], q[5] };
    const double tp[3] = { qp[3], qp[4], qp[5] };
    body_frame(t, F);
    rot_rn(tp, Qp);
    double c[9];
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) {
            const double d = F[3 * i + k] - Qp[3 * i + k];
            const double L = Lam[9 * b + 3 * i + k];
            e += kQ / 2 * J[k] * d * d - L * d * Js[k];
            c[3 * i + k] = kQ * J[k] * d - L * Js[k];
        }
    energy[b] = e;
    if (grad)
        for (int a = 0; a < 3; a++) {
            double acc = 0;
            for (int r = 0; r < 9; r++) acc += c[r] * F[9 + 9 * a + r];
            grad[6 * b + 3 + a] += acc;
        }
    if (hess)
        for (int a = 0; a < 3; a++)
            for (int cc = 0; cc < 3; cc++) {
                const double* d2 = F + 36 + 9 * sym_index(a, cc);
                double acc = 0;
                for (int i = 0; i < 3; i++)
                    for (int k = 0; k < 3; k++)
                        acc += kQ * J[k] * F[9 + 9 * a + 3 * i + k] * F[9 + 9 * cc + 3 * i + k]
                            + c[3 * i + k] * d2[3 * i + k];
                hess[36 * (size_t)b + 6 * (3 + a) + 3 + cc] += acc;
            }
}

// progress sums (compute_{linear,angular}_augment_lagrangian_progress,
// :265-337): out = (|q_pred - q|^2, |q_pred - q0|^2, |Q - Q_pred|^2,
// |Q0 - Q_pred|^2) over the kinematic bodies, one block
__global__ void __launch_bounds__(256) k_al_progress(int nb, const int* __restrict__ type,
                                                     const double* __restrict__ x,
                                                     const double* __restrict__ xpred,
                                                     const double* __restrict__ x0,
                                                     double* __restrict__ out)
{
    __shared__ double sh[4][256];
    double a[4] = { 0, 0, 0, 0 };
    for (int b = threadIdx.x; b < nb; b += 256) {
        if (type[b] != RIGC_BODY_KINEMATIC) continue;
        for (int i = 0; i < 3; i++) {
            const double d = xpred[6 * b + i] - x[6 * b + i], d0 = xpred[6 * b + i] - x0[6 * b + i];
            a[0] += d * d;
            a[1] += d0 * d0;
        }
        double Q[9], Qp[9], Q0[9];
        const double t[3] = { x[6 * b + 3], x[6 * b + 4], x[6 * b + 5] };
        const double tp[3] = { xpred[6 * b + 3], xpred[6 * b + 4], xpred[6 * b + 5] };
        const double t0[3] = { x0[6 * b + 3], x0[6 * b + 4], x0[6 * b + 5] };
        rot_rn(t, Q);
        rot_rn(tp, Qp);
        rot_rn(t0, Q0);
        for (int k = 0; k < 9; k++) {
            a[2] += (Q[k] - Qp[k]) * (Q[k] - Qp[k]);
            a[3] += (Q0[k] - Qp[k]) * (Q0[k] - Qp[k]);
        }
    }
    for (int j = 0; j < 4; j++) sh[j][threadIdx.x] = a[j];
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int j = 0; j < 4; j++) sh[j][threadIdx.x] += sh[j][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x < 4) out[threadIdx.x] = sh[threadIdx.x][0];
}

// multiplier updates of update_augmented_lagrangian (:339-423)
__global__ void k_al_update(int nb, const int* __restrict__ type, const double* __restrict__ x,
                            const double* __restrict__ xpred, const double* __restrict__ mass,
                            const double* __restrict__ moment, int upd_q, int upd_Q, double kq,
                            double kQ, double* __restrict__ lam, double* __restrict__ Lam)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb || type[b] != RIGC_BODY_KINEMATIC) return;
    if (upd_q)
        for (int i = 0; i < 3; i++)
            lam[3 * b + i] -= kq * sqrt(mass[b]) * (x[6 * b + i] - xpred[6 * b + i]);
    if (upd_Q) {
        double J[3], Js[3], Q[9], Qp[9];
        al_J(moment + 3 * b, J, Js);
        const double t[3] = { x[6 * b + 3], x[6 * b + 4], x[6 * b + 5] };
        const double tp[3] = { xpred[6 * b + 3], xpred[6 * b + 4], xpred[6 * b + 5] };
        rot_rn(t, Q);
        rot_rn(tp, Qp);
        for (int i = 0; i < 3; i++)
            for (int k = 0; k < 3; k++) Lam[9 * b + 3 * i + k] -= kQ * (Q[3 * i + k] - Qp[3 * i + k]) * Js[k];
    }
}

// ---------------------------------------------------------------------------
// per-scene kernels of batched contexts (bodies ordered by scene)

// out[s] = sum over scene s's dofs of a[i] b[i] (b null: sum of a), one block
// per scene, in a fixed order
__global__ void __launch_bounds__(256) k_seg_dot(const int* __restrict__ scene_bstart, int per_body,
                                                 const double* __restrict__ a,
                                                 const double* __restrict__ b,
                                                 double* __restrict__ out)
{
    __shared__ double sh[256];
    const int sc = blockIdx.x;
    const int64_t lo = (int64_t)scene_bstart[sc] * per_body, hi = (int64_t)scene_bstart[sc + 1] * per_body;
    double acc = 0;
    for (int64_t i = lo + threadIdx.x; i < hi; i += 256) acc += b ? a[i] * b[i] : a[i];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[sc] = sh[0];
}

// g = gE / m_s + (kappa_s / m_s) gB, zero on fixed dofs
__global__ void k_combine_grad_sc(int nb, const double* __restrict__ gE, const double* __restrict__ gB,
                                  const int* __restrict__ bscene, const double* __restrict__ scE,
                                  const double* __restrict__ scB, const int* __restrict__ fixed,
                                  double* __restrict__ g)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 6 * nb) return;
    const int b = i / 6, sc = bscene[b];
    double v = scE[sc] * gE[i];
    if (gB) v += scB[sc] * gB[i];
    g[i] = ((fixed[b] >> (i % 6)) & 1) ? 0.0 : v;
}

// out = y + alpha_s x (per-scene alpha)
__global__ void k_axpy_sc(int nb, const int* __restrict__ bscene, const double* __restrict__ alpha,
                          const double* __restrict__ x, const double* __restrict__ y,
                          double* __restrict__ out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 6 * nb) out[i] = y[i] + alpha[bscene[i / 6]] * x[i];
}

// CG per scene: flags[2 s] breakdown, flags[2 s + 1] converged (scenes that
// are not solved start converged and keep alpha = 0)
__global__ void k_cg_alpha_sc(int ns, const double* __restrict__ rz, const double* __restrict__ pAp,
                              const double* __restrict__ rr, const double* __restrict__ tol2,
                              double* __restrict__ alpha, int* __restrict__ flags)
{
    int sc = blockIdx.x * blockDim.x + threadIdx.x;
    if (sc >= ns) return;
    int* f = flags + 2 * sc;
    if (f[0] || f[1] || rr[sc] <= tol2[sc]) {
        if (!f[0]) f[1] = 1;
        alpha[sc] = 0;
        return;
    }
    const double d = pAp[sc];
    if (!(d > 0) || !isfinite(d)) {
        f[0] = 1;
        alpha[sc] = 0;
    } else {
        alpha[sc] = rz[sc] / d;
    }
}

__global__ void k_cg_update_sc(int nb, const int* __restrict__ bscene, const double* __restrict__ alpha,
                               const double* __restrict__ p, const double* __restrict__ Ap,
                               double* __restrict__ x, double* __restrict__ r)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 6 * nb) return;
    const double a = alpha[bscene[i / 6]];
    if (a == 0) return;
    x[i] += a * p[i];
    r[i] -= a * Ap[i];
}

__global__ void k_cg_direction_sc(int nb, const int* __restrict__ bscene,
                                  const double* __restrict__ rz_new, const double* __restrict__ rz_old,
                                  const double* __restrict__ z, const int* __restrict__ flags,
                                  double* __restrict__ p)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 6 * nb) return;
    const int sc = bscene[i / 6];
    if (flags[2 * sc] || flags[2 * sc + 1]) return;
    p[i] = z[i] + (rz_new[sc] / rz_old[sc]) * p[i];
}

// Last node of the per-scene CG graph's loop body (one block): the loop
// ends once every solved scene (mask) has converged or broken down, or after
// max_it iterations.
__global__ void __launch_bounds__(256) k_cg_continue_sc(int ns, const int* __restrict__ mask,
                                                        const int* __restrict__ flags,
                                                        const double* __restrict__ rr,
                                                        const double* __restrict__ tol2,
                                                        long long* __restrict__ iters,
                                                        long long max_it,
                                                        cudaGraphConditionalHandle loop)
{
    int open = 0;
    for (int k = threadIdx.x; k < ns; k += blockDim.x) {
        if (!mask[k]) continue;
        const double v = rr[k];
        if (!(flags[2 * k] || flags[2 * k + 1] || v <= tol2[k] || !isfinite(v))) open = 1;
    }
    open = __syncthreads_or(open);
    if (threadIdx.x == 0) {
        const long long it = ++*iters;
        cudaGraphSetConditional(loop, (open && it < max_it) ? 1u : 0u);
    }
}

// v[i] = 0 on the dofs of scenes whose mask differs from keep
__global__ void k_mask_scenes(int nb, const int* __restrict__ bscene, const int* __restrict__ mask,
                              int keep, double* __restrict__ v)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 6 * nb && (mask[bscene[i / 6]] != 0) != (keep != 0)) v[i] = 0;
}

// largest |V1 - V0| coordinate per scene (one block per scene's vertex range)
__global__ void __launch_bounds__(256) k_max_vertex_move_sc(const int* __restrict__ vstart,
                                                            const double* __restrict__ V0,
                                                            const double* __restrict__ V1,
                                                            double* __restrict__ out)
{
    __shared__ double sh[256];
    const int sc = blockIdx.x;
    double m = 0;
    for (int64_t i = 3 * (int64_t)vstart[sc] + threadIdx.x; i < 3 * (int64_t)vstart[sc + 1]; i += 256)
        m = fmax(m, fabs(V1[i] - V0[i]));
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[sc] = sh[0];
}

// smallest squared constraint distance per scene (bits of a non-negative double)
__global__ void k_min_constraint_distance_sc(int64_t n, const int* __restrict__ type,
                                             const int* __restrict__ verts,
                                             const int* __restrict__ bodies,
                                             const int* __restrict__ bscene,
                                             const double* __restrict__ V,
                                             unsigned long long* __restrict__ out)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int t = type[i];
    const double* P[4];
    for (int k = 0; k < 4; k++) {
        int v = verts[4 * i + k];
        P[k] = V + 3 * (size_t)(v < 0 ? 0 : v);
    }
    double d;
    if (t == 0) d = pp_sqdist_rn(P[0], P[1]);
    else if (t == 1) d = pl_sqdist_rn(P[0], P[1], P[2]);
    else if (t == 2) d = ee_sqdist_rn(P[0], P[1], P[2], P[3]);
    else d = ptplane_sqdist_rn(P[0], P[1], P[2], P[3]);
    atomicMin(out + bscene[bodies[2 * i]], (unsigned long long)__double_as_longlong(d));
}

// rhs of the free dofs (-g) and the scatter of the solution back
__global__ void k_gather_neg(int n6, const int* __restrict__ free_idx, const double* __restrict__ g,
                             double* __restrict__ out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n6 && free_idx[i] >= 0) out[free_idx[i]] = -g[i];
}
__global__ void k_scatter_free(int n6, const int* __restrict__ free_idx, const double* __restrict__ xf,
                               double* __restrict__ x)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n6) x[i] = free_idx[i] >= 0 ? xf[free_idx[i]] : 0.0;
}

// max |v_i| over the vector, as the bits of a non-negative double
__global__ void k_max_abs(int64_t n, const double* __restrict__ v, unsigned long long* __restrict__ out)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double a = i < n ? fabs(v[i]) : 0.0;
    for (int o = 16; o > 0; o >>= 1) a = fmax(a, __shfl_xor_sync(0xffffffffu, a, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(a));
}

// y = H x over every row and column (no fixed-dof masking)
__global__ void k_hess_rows(HessView H, const double* __restrict__ x, double* __restrict__ y)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 6 * H.nb) return;
    const int b = i / 6, r = i % 6;
    double acc = 0;
    if (H.sE != 0) {
        const double* Bb = H.body + 36 * (size_t)b + 6 * r;
        for (int c = 0; c < 6; c++) acc += H.sE * Bb[c] * x[6 * b + c];
    }
    if (H.brp)
        for (int k = H.brp[b]; k < H.brp[b + 1]; k++) {
            const double* V = H.bval + 36 * (size_t)k + 6 * r;
            const int cb = H.bcol[k];
            for (int c = 0; c < 6; c++) acc += H.sB * V[c] * x[6 * cb + c];
        }
    y[i] = acc + H.reg * x[i];
}

// ---------------------------------------------------------------------------
// adjoint of one time step.  State layout per body: pose [p, theta] (6),
// velocities [v, omega] (6), Qdot (9); the three arrays are stored one after
// the other (6 nb, 6 nb, 9 nb).

// the update s' = (x*, (p* - p0) / h, (R(theta*) - R(theta0)) / h) of a
// dynamic body (the others keep their velocities and Qdot; omega is kept):
// dL/dx* (xbar) and the direct part of dL/ds (out, overwritten)
__global__ void k_adj_direct(int nb, const int* __restrict__ type, const int* __restrict__ fixed,
                             const double* __restrict__ xs, const double* __restrict__ x0,
                             const double* __restrict__ in, double h, double* __restrict__ xbar,
                             double* __restrict__ out)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const double* ap = in;
    const double* av = in + 6 * (size_t)nb;
    const double* aq = in + 12 * (size_t)nb;
    double* op = out;
    double* ov = out + 6 * (size_t)nb;
    double* oq = out + 12 * (size_t)nb;
    for (int k = 0; k < 6; k++) {
        xbar[6 * b + k] = ap[6 * b + k];
        op[6 * b + k] = 0;
        ov[6 * b + k] = 0;
    }
    if (type[b] != RIGC_BODY_DYNAMIC) {
        for (int k = 0; k < 6; k++) ov[6 * b + k] = av[6 * b + k];
        for (int k = 0; k < 9; k++) oq[9 * b + k] = aq[9 * b + k];
        return;
    }
    for (int k = 0; k < 9; k++) oq[9 * b + k] = 0;
    const int fx = fixed[b];
    for (int k = 0; k < 3; k++) {
        if (!((fx >> k) & 1)) {
            xbar[6 * b + k] += av[6 * b + k] / h;
            op[6 * b + k] = -av[6 * b + k] / h;
        }
        ov[6 * b + 3 + k] = av[6 * b + 3 + k];
    }
    double F1[kFrameDoubles], F0[kFrameDoubles];
    const double t1[3] = { xs[6 * b + 3], xs[6 * b + 4], xs[6 * b + 5] };
    const double t0[3] = { x0[6 * b + 3], x0[6 * b + 4], x0[6 * b + 5] };
    body_frame(t1, F1);
    body_frame(t0, F0);
    for (int a = 0; a < 3; a++) {
        double s1 = 0, s0 = 0;
        for (int k = 0; k < 9; k++) {
            s1 += aq[9 * b + k] * F1[9 + 9 * a + k];
            s0 += aq[9 * b + k] * F0[9 + 9 * a + k];
        }
        xbar[6 * b + 3 + a] += s1 / h;
        op[6 * b + 3 + a] = -s0 / h;
    }
}

// out += alpha (d2E / dx ds)^T w with E the body energy at pose xe and
// start-of-step state (x0, v0, Qdot0):
//   d2E/dp dp0 = -m I, d2E/dp dv0 = -m h I,
//   d2E/dtheta_a dT_ik = -J_k dQ_ik/dtheta_a with T = R(theta0) + h Qdot0
__global__ void k_adj_exs(int nb, const int* __restrict__ type, const int* __restrict__ fixed,
                          const double* __restrict__ mass, const double* __restrict__ moment,
                          const double* __restrict__ xe, const double* __restrict__ x0,
                          const double* __restrict__ w, double alpha, double h,
                          double* __restrict__ out)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb || type[b] != RIGC_BODY_DYNAMIC) return;
    double* op = out;
    double* ov = out + 6 * (size_t)nb;
    double* oq = out + 12 * (size_t)nb;
    const int fx = fixed[b];
    const double m = mass[b];
    if ((fx & 7) != 7)
        for (int k = 0; k < 3; k++) {
            op[6 * b + k] -= alpha * m * w[6 * b + k];
            ov[6 * b + k] -= alpha * m * h * w[6 * b + k];
        }
    if ((fx & 56) != 56) {
        const double* I = moment + 3 * b;
        const double J[3] = { 0.5 * (-I[0] + I[1] + I[2]), 0.5 * (I[0] - I[1] + I[2]),
                              0.5 * (I[0] + I[1] - I[2]) };
        double F[kFrameDoubles], F0[kFrameDoubles];
        const double te[3] = { xe[6 * b + 3], xe[6 * b + 4], xe[6 * b + 5] };
        const double t0[3] = { x0[6 * b + 3], x0[6 * b + 4], x0[6 * b + 5] };
        body_frame(te, F);
        body_frame(t0, F0);
        double Tb[9];
        for (int i = 0; i < 3; i++)
            for (int k = 0; k < 3; k++) {
                double acc = 0;
                for (int a = 0; a < 3; a++) acc += w[6 * b + 3 + a] * F[9 + 9 * a + 3 * i + k];
                Tb[3 * i + k] = -alpha * J[k] * acc;
            }
        for (int e = 0; e < 9; e++) oq[9 * b + e] += h * Tb[e];
        for (int cc = 0; cc < 3; cc++) {
            double acc = 0;
            for (int e = 0; e < 9; e++) acc += Tb[e] * F0[9 + 9 * cc + e];
            op[6 * b + 3 + cc] += acc;
        }
    }
}

// fixed dofs keep x0: dL/dx0_C += dL/dx*_C - (H lambda)_C
__global__ void k_adj_fixed(int nb, const int* __restrict__ fixed, const double* __restrict__ xbar,
                            const double* __restrict__ Hl, double* __restrict__ op)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 6 * nb) return;
    if ((fixed[i / 6] >> (i % 6)) & 1) op[i] += xbar[i] - Hl[i];
}

// op += s (u1 + u2) over the poses
__global__ void k_adj_pose_add(int64_t n, double s, const double* __restrict__ u1,
                               const double* __restrict__ u2, double* __restrict__ op)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) op[i] += s * (u1[i] + u2[i]);
}

double barrier_hessian_d(double d, double s)
{
    if (d <= 0.0 || d >= s) return 0.0;
    double sd = s / d;
    return (sd + 2) * sd - 2 * std::log(d / s) - 3;
}

} // namespace

// ---------------------------------------------------------------------------

// systems with at most this many free dofs are factorised densely
constexpr int kDenseMax = 768;
// above kDenseMax free dofs: PCG for at most kCGTry iterations, then (up to
// kDenseLimit free dofs, n^2 doubles) the dense LDL^T for the rest of the step
constexpr int kDenseLimit = 8192;
constexpr long long kCGTry = 300;

struct Sim {
    rigc_sim_params p {};
    int nb = 0, nv = 0, nfree = 0;
    DevBuf free_idx, dense, dense_b, dense_x, dense_d;  // dense LDL^T path
    DevBuf mass, moment, fixed, x0, vel, Qdot;          // body state
    DevBuf x, xt, dir, g, gE, hE, gtmp;                 // Newton vectors
    DevBuf r, z, pp, Ap, Minv, sol, part, scal;         // CG
    DevBuf V0, V1;                                      // world vertices
    double kappa = 1, kappa_max = 0;
    double dk = 0;  // d kappa / d kappa0 of the current step (0 when kappa0 is clamped)
    std::vector<int> h_fixed;
    bool dense_step = false;  // this step's PCG did not converge: dense LDL^T from then on
    // rollout tape: checkpoints (21 nb doubles each: poses, velocities, Qdot),
    // the state after the rollout, and one recomputed segment
    int tape_steps = 0, tape_every = 0;
    DevBuf ckpt, final_state, seg_pre, seg_x;
    std::vector<double> seg_kappa, seg_dk;
    // adjoint vectors: dL/d(state) in and out, dL/dx*, scratch
    DevBuf adj, adj_out, xbar, u1, u2;
    // batched contexts: every scene is its own problem (own average mass,
    // bounding-box diagonal, stiffness, regularisation, step length and
    // convergence); per-scene device scalars and reduction outputs
    std::vector<double> sc_mass, sc_bbox;
    DevBuf sc_dev, sc_red, sc_vstart;
    // augmented Lagrangian of kinematic bodies (per step)
    bool has_kinematic = false, al_sat_q = false, al_sat_Q = false;
    double al_kq = 1e3, al_kQ = 1e3;
    DevBuf al_xpred, al_lam, al_Lam, al_e;
    // kinematic schedules (rigid_body.hpp:260-261): per body the time it
    // keeps moving and the poses each step drives it to; the step's targets
    // (6 per body, NaN first for none)
    std::vector<double> kin_max_time;
    std::vector<std::deque<std::array<double, 6>>> kin_poses;
    DevBuf kin_target;
    // CUDA graphs of the CG solvers' iteration loops (single problem, per
    // scene): one while node whose body is one CG iteration ending in its
    // continuation test.  Rebuilt when an argument (a buffer address or a
    // size, the key) changes; the Hessian view they read is hview.
    struct LoopGraph {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        std::vector<unsigned long long> key;
        int kernels = 0;  // kernel nodes per iteration
        void release()
        {
            if (exec) cudaGraphExecDestroy(exec);
            if (graph) cudaGraphDestroy(graph);
            exec = nullptr;
            graph = nullptr;
            key.clear();
        }
    };
    LoopGraph cg_one, cg_sc;
    DevBuf hview;
    cudaStream_t cap = nullptr;  // the stream graphs are captured on
};

namespace {

struct Objective {
    double f;
    bool grad_hess;
    rigc_barrier_out bo, fo;
};

rigc_body_state state_of(Sim& S)
{
    rigc_body_state s;
    s.mass = S.mass.as<double>();
    s.moment = S.moment.as<double>();
    s.x_t0 = S.x0.as<double>();
    s.v_t0 = S.vel.as<double>();
    s.Qdot_t0 = S.Qdot.as<double>();
    s.dof_fixed = S.fixed.as<int32_t>();
    return s;
}

int dot_dev(Ctx& c, Sim& S, int64_t n, const double* a, const double* b, double* out_dev)
{
    RIGC_COUNT_LAUNCH();
    k_dot_partial<<<64, 256, 0, c.stream>>>(n, a, b, S.part.as<double>());
    RIGC_COUNT_LAUNCH();
    k_dot_final<<<1, 256, 0, c.stream>>>(S.part.as<double>(), 64, out_dev);
    return RIGC_OK;
}

int read_scalars(Ctx& c, const double* dev, double* host, int n)
{
    RIGC_CUDA(cudaMemcpyAsync(host, dev, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    RIGC_CUDA(cudaStreamSynchronize(c.stream));
    return RIGC_OK;
}

std::vector<unsigned long long> graph_key(std::initializer_list<const void*> ptrs,
                                          std::initializer_list<long long> sizes)
{
    std::vector<unsigned long long> k;
    for (const void* p : ptrs) k.push_back((unsigned long long)(uintptr_t)p);
    for (long long s : sizes) k.push_back((unsigned long long)s);
    return k;
}

// G holds (or is given) an executable graph whose only node is a while loop
// around the launches body(stream, loop handle) issues; a graph built for the
// same key is reused.  Its launches are captured, not run: nothing executes
// until the graph is launched.  The handle's default value is 1, so every
// launch runs the body at least once; the body's last kernel decides whether
// it runs again.
template <class Body>
int loop_graph(Sim& S, Sim::LoopGraph& G, const std::vector<unsigned long long>& key, int kernels,
               Body body)
{
    if (G.exec && G.key == key) return RIGC_OK;
    G.release();
    if (!S.cap) RIGC_CUDA(cudaStreamCreateWithFlags(&S.cap, cudaStreamNonBlocking));
    RIGC_CUDA(cudaGraphCreate(&G.graph, 0));
    cudaGraphConditionalHandle loop;
    RIGC_CUDA(cudaGraphConditionalHandleCreate(&loop, G.graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = loop;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    RIGC_CUDA(cudaGraphAddNode(&node, G.graph, nullptr, nullptr, 0, &cp));
    cudaGraph_t bodyg = cp.conditional.phGraph_out[0];
    RIGC_CUDA(cudaStreamBeginCaptureToGraph(S.cap, bodyg, nullptr, nullptr, 0,
                                            cudaStreamCaptureModeThreadLocal));
    body(S.cap, loop);
    cudaGraph_t captured = nullptr;
    const cudaError_t e = cudaStreamEndCapture(S.cap, &captured);
    if (e != cudaSuccess) {
        G.release();
        RIGC_CUDA(e);
    }
    RIGC_CUDA(cudaGraphInstantiate(&G.exec, G.graph, 0));
    G.key = key;
    G.kernels = kernels;
    return RIGC_OK;
}

// objective (and optionally its gradient in S.g and the Hessian pieces)
int objective(Ctx& c, Sim& S, const double* x, bool grad_hess, Objective& O, bool project = true)
{
    const rigc_sim_params& p = S.p;
    const double m = p.average_mass;
    rigc_body_state bs = state_of(S);
    double E;
    RIGC_TRY(body_energy(c, bs, x, p.gravity, p.timestep, &E, grad_hess ? S.gE.as<double>() : nullptr,
                         grad_hess ? S.hE.as<double>() : nullptr));
    if (S.has_kinematic && !(S.al_sat_q && S.al_sat_Q)) {
        RIGC_COUNT_LAUNCH();
        k_al_terms<<<grid_for(S.nb, 128), 128, 0, c.stream>>>(
            S.nb, c.s.type, x, S.al_xpred.as<double>(), S.mass.as<double>(), S.moment.as<double>(),
            S.al_lam.as<double>(), S.al_Lam.as<double>(), S.al_kq, S.al_kQ, S.al_e.as<double>(),
            grad_hess ? S.gE.as<double>() : nullptr, grad_hess ? S.hE.as<double>() : nullptr);
        double* e_dev = reinterpret_cast<double*>(c.d_scalars.as<char>() + 2568);
        RIGC_TRY(sum_f64(S.al_e.as<double>(), S.nb, e_dev, c.scratch[1], c.stream));
        double al;
        RIGC_TRY(read_scalars(c, e_dev, &al, 1));
        E += al;
    }
    RIGC_TRY(build_constraints(c, x, p.dhat, p.dmin));
    const int flags = grad_hess ? (RIGC_GRAD | RIGC_HESS | (project ? RIGC_PROJECT_PSD : 0)) : 0;
    RIGC_TRY(barrier_term_impl(c, x, p.dhat, p.dmin, flags, &O.bo));
    double D = 0;
    O.fo = rigc_barrier_out {};
    if (p.coefficient_friction > 0 && c.fric.num > 0) {
        RIGC_TRY(friction_term(c, x, p.static_friction_speed_bound * p.timestep, flags, &O.fo));
        D = O.fo.energy;
    }
    O.f = E / m + S.kappa / m * O.bo.energy + D / m;
    O.grad_hess = grad_hess;
    if (grad_hess) {
        RIGC_COUNT_LAUNCH();
        k_combine_grad<<<grid_for(6 * S.nb, 256), 256, 0, c.stream>>>(
            S.nb, S.gE.as<double>(), O.bo.grad, O.fo.grad, 1.0 / m, S.kappa / m, 1.0 / m,
            S.fixed.as<int>(), S.g.as<double>());
        RIGC_CUDA(cudaGetLastError());
    }
    return RIGC_OK;
}

HessView hess_view(Sim& S, const Objective& O, double reg)
{
    const double m = S.p.average_mass;
    HessView H;
    H.body = S.hE.as<double>();
    H.brp = O.bo.nnzb > 0 ? O.bo.row_ptr : nullptr;
    H.bcol = O.bo.col;
    H.bval = O.bo.val;
    H.frp = O.fo.nnzb > 0 ? O.fo.row_ptr : nullptr;
    H.fcol = O.fo.col;
    H.fval = O.fo.val;
    H.sE = 1.0 / m;
    H.sB = S.kappa / m;
    H.sD = 1.0 / m;
    H.reg = reg;
    H.fixed = S.fixed.as<int>();
    H.nb = S.nb;
    return H;
}

// PCG for (H + reg I) d = -g on the free dofs; false when it breaks down
// or does not reach the tolerance
int pcg(Ctx& c, Sim& S, const HessView& H, bool& ok, int64_t& iters, long long cap = 0)
{
    const int64_t n = 6 * (int64_t)S.nb;
    cudaStream_t st = c.stream;
    const unsigned gn = grid_for(n, 256);
    double* d = S.sol.as<double>();
    double* r = S.r.as<double>();
    double* z = S.z.as<double>();
    double* pp = S.pp.as<double>();
    double* Ap = S.Ap.as<double>();
    double* sc = S.scal.as<double>();  // [0] rz, [1] rz_new, [2] pAp, [3] alpha, [4] rr, [5] bb
    int* flags = reinterpret_cast<int*>(sc + 8);  // [0] breakdown, [1] converged
    RIGC_CUDA(cudaMemsetAsync(d, 0, n * sizeof(double), st));
    RIGC_CUDA(cudaMemsetAsync(flags, 0, 2 * sizeof(int), st));
    // r = -g
    RIGC_COUNT_LAUNCH();
    k_axpy<<<gn, 256, 0, st>>>(n, -2.0, S.g.as<double>(), S.g.as<double>(), r);
    RIGC_COUNT_LAUNCH();
    k_block_jacobi<<<grid_for(S.nb, 64), 64, 0, st>>>(H, S.Minv.as<double>());
    RIGC_COUNT_LAUNCH();
    k_block_apply<<<gn, 256, 0, st>>>(S.nb, S.Minv.as<double>(), r, H.fixed, z);
    RIGC_CUDA(cudaMemcpyAsync(pp, z, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    RIGC_TRY(dot_dev(c, S, n, r, z, sc + 0));
    RIGC_TRY(dot_dev(c, S, n, r, r, sc + 5));
    RIGC_CUDA(cudaMemcpyAsync(sc + 4, sc + 5, sizeof(double), cudaMemcpyDeviceToDevice, st));
    double h5[2];
    RIGC_TRY(read_scalars(c, sc + 5, h5, 1));
    const double bnorm2 = h5[0];
    ok = true;
    iters = 0;
    if (bnorm2 == 0) return RIGC_OK;
    const double tol2 = 1e-24 * bnorm2;  // relative residual 1e-12
    const long long max_it = cap > 0 ? cap : std::max<long long>(1000, 4 * n);
    // the iteration loop runs on the device as one graph launch: its
    // arguments are fixed, so the view, the tolerance and the iteration
    // count live in device memory (sc[7] tolerance, sc[20] iterations)
    double* tol2_dev = sc + 7;
    long long* it_dev = reinterpret_cast<long long*>(sc + 20);
    RIGC_TRY(S.hview.reserve(sizeof(HessView)));
    HessView* Hd = S.hview.as<HessView>();
    const double* Minv = S.Minv.as<double>();
    const int nb = S.nb;
    const int* fixed = H.fixed;
    double* part = S.part.as<double>();
    const std::vector<unsigned long long> key = graph_key(
        { (const void*)Hd, d, r, z, pp, Ap, sc, Minv, fixed, part }, { n, max_it });
    auto body = [&](cudaStream_t cs, cudaGraphConditionalHandle loop) {
        k_hess_matvec_dev<<<gn, 256, 0, cs>>>(Hd, pp, Ap);
        k_dot_partial<<<64, 256, 0, cs>>>(n, pp, Ap, part);
        k_dot_final<<<1, 256, 0, cs>>>(part, 64, sc + 2);
        k_cg_alpha<<<1, 1, 0, cs>>>(sc + 0, sc + 2, sc + 4, tol2_dev, sc + 3, flags);
        k_cg_update<<<gn, 256, 0, cs>>>(n, sc + 3, pp, Ap, d, r);
        k_block_apply<<<gn, 256, 0, cs>>>(nb, Minv, r, fixed, z);
        k_dot_partial<<<64, 256, 0, cs>>>(n, r, z, part);
        k_dot_final<<<1, 256, 0, cs>>>(part, 64, sc + 1);
        k_dot_partial<<<64, 256, 0, cs>>>(n, r, r, part);
        k_dot_final<<<1, 256, 0, cs>>>(part, 64, sc + 4);
        k_cg_direction<<<gn, 256, 0, cs>>>(n, sc + 1, sc + 0, z, flags, pp);
        cudaMemcpyAsync(sc + 0, sc + 1, sizeof(double), cudaMemcpyDeviceToDevice, cs);
        k_cg_continue<<<1, 1, 0, cs>>>(flags, sc + 4, tol2_dev, it_dev, max_it, loop);
    };
    RIGC_TRY(loop_graph(S, S.cg_one, key, 12, body));
    RIGC_CUDA(cudaMemcpyAsync(Hd, &H, sizeof(HessView), cudaMemcpyHostToDevice, st));
    RIGC_CUDA(cudaMemcpyAsync(tol2_dev, &tol2, sizeof(double), cudaMemcpyHostToDevice, st));
    RIGC_CUDA(cudaMemsetAsync(it_dev, 0, sizeof(long long), st));
    RIGC_CUDA(cudaGraphLaunch(S.cg_one.exec, st));
    double rr;
    int fl[2];
    long long its;
    RIGC_CUDA(cudaMemcpyAsync(&rr, sc + 4, sizeof(double), cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaMemcpyAsync(fl, flags, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaMemcpyAsync(&its, it_dev, sizeof(long long), cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaStreamSynchronize(st));
    iters = its;
    count_launches(its * S.cg_one.kernels);
    ok = fl[1] || rr <= tol2;
    return RIGC_OK;
}

int dense_ldlt(Ctx& c, double* A, int n, double* D, int* flags)
{
    static bool attr = false;
    const size_t smem = (size_t)kDenseMax * kPanelStride * sizeof(double);
    if (!attr) {
        RIGC_CUDA(cudaFuncSetAttribute(k_ldlt_panel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
        attr = true;
    }
    // up to kDenseMax unknowns the whole panel column is factorised in shared
    // memory; above, its diagonal block there and the rows below by k_ldlt_trsm
    const bool big = n > kDenseMax;
    for (int j0 = 0; j0 < n; j0 += kPanel) {
        const int w = std::min(kPanel, n - j0);
        const int rows = big ? w : n - j0;
        RIGC_COUNT_LAUNCH();
        k_ldlt_panel<<<1, 512, (size_t)rows * kPanelStride * sizeof(double), c.stream>>>(
            A, n, j0, rows, D, flags);
        const int rest = n - j0 - w;
        if (big && rest > 0) {
            RIGC_COUNT_LAUNCH();
            k_ldlt_trsm<<<grid_for(rest, 128), 128, 0, c.stream>>>(A, n, j0, w, D, flags);
        }
        if (rest > 0) {
            const int tiles = (rest + 31) / 32;
            RIGC_COUNT_LAUNCH();
            k_ldlt_update<<<tiles * (tiles + 1) / 2, 256, 0, c.stream>>>(A, n, j0, w, D, flags);
        }
    }
    RIGC_CUDA(cudaGetLastError());
    return RIGC_OK;
}

// dense LDL^T solve of (H + reg I) d = -g on the free dofs into S.sol
int dense_solve(Ctx& c, Sim& S, const HessView& H, bool& ok)
{
    const int n = S.nfree;
    const int n6 = 6 * S.nb;
    cudaStream_t st = c.stream;
    if (n > kDenseMax) {
        RIGC_TRY(S.dense.reserve((size_t)n * n * sizeof(double) + 8));
        RIGC_TRY(S.dense_b.reserve((size_t)n * sizeof(double) + 8));
        RIGC_TRY(S.dense_x.reserve((size_t)n * sizeof(double) + 8));
        RIGC_TRY(S.dense_d.reserve((size_t)n * sizeof(double) + 8));
    }
    int* flags = reinterpret_cast<int*>(S.scal.as<double>() + 8);
    RIGC_CUDA(cudaMemsetAsync(flags, 0, 2 * sizeof(int), st));
    RIGC_CUDA(cudaMemsetAsync(S.dense.ptr, 0, (size_t)n * n * sizeof(double), st));
    RIGC_COUNT_LAUNCH();
    k_dense_fill<<<grid_for(n6, 128), 128, 0, st>>>(H, S.free_idx.as<int>(), n, S.dense.as<double>());
    RIGC_COUNT_LAUNCH();
    k_gather_neg<<<grid_for(n6, 256), 256, 0, st>>>(n6, S.free_idx.as<int>(), S.g.as<double>(),
                                                    S.dense_b.as<double>());
    RIGC_TRY(dense_ldlt(c, S.dense.as<double>(), n, S.dense_d.as<double>(), flags));
    RIGC_COUNT_LAUNCH();
    k_ldlt_solve<<<1, 256, 0, st>>>(S.dense.as<double>(), n, S.dense_d.as<double>(),
                                    S.dense_b.as<double>(), S.dense_x.as<double>(), flags);
    RIGC_COUNT_LAUNCH();
    k_scatter_free<<<grid_for(n6, 256), 256, 0, st>>>(n6, S.free_idx.as<int>(), S.dense_x.as<double>(),
                                                      S.sol.as<double>());
    RIGC_CUDA(cudaGetLastError());
    int fl = 0;
    RIGC_CUDA(cudaMemcpyAsync(&fl, flags, sizeof(int), cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaStreamSynchronize(st));
    ok = fl == 0;
    return RIGC_OK;
}

// The Newton system on the free dofs: the dense LDL^T up to kDenseMax
// unknowns; above, PCG, and when it does not converge within kCGTry
// iterations (the stiff couplings of a contact pile) the dense LDL^T up to
// kDenseLimit unknowns, for the rest of the time step
int newton_solve(Ctx& c, Sim& S, const HessView& H, bool& solved, int64_t& cgit)
{
    cgit = 0;
    if (S.nfree <= kDenseMax || S.dense_step) return dense_solve(c, S, H, solved);
    const bool can_dense = S.nfree <= kDenseLimit;
    RIGC_TRY(pcg(c, S, H, solved, cgit, can_dense ? kCGTry : 0));
    if (!solved && can_dense) {
        S.dense_step = true;
        RIGC_TRY(dense_solve(c, S, H, solved));
    }
    return RIGC_OK;
}

double host_dot(Ctx& c, Sim& S, const double* a, const double* b)
{
    double v = 0;
    if (dot_dev(c, S, 6 * (int64_t)S.nb, a, b, S.scal.as<double>() + 6) != RIGC_OK) return NAN;
    if (read_scalars(c, S.scal.as<double>() + 6, &v, 1) != RIGC_OK) return NAN;
    return v;
}

int min_distance(Ctx& c, Sim& S, const double* x, double* md)
{
    RIGC_TRY(build_constraints(c, x, S.p.dhat, S.p.dmin));
    const int64_t n = c.cons.num;
    if (n == 0) {
        *md = -1;
        return RIGC_OK;
    }
    RIGC_TRY(compute_world_vertices_rn(c, x, S.V0.as<double>(), c.scratch[5]));
    unsigned long long* out = reinterpret_cast<unsigned long long*>(S.scal.as<double>() + 12);
    const unsigned long long inf = 0x7ff0000000000000ull;
    RIGC_CUDA(cudaMemcpyAsync(out, &inf, sizeof(inf), cudaMemcpyHostToDevice, c.stream));
    RIGC_COUNT_LAUNCH();
    k_min_constraint_distance<<<grid_for(n, 256), 256, 0, c.stream>>>(
        n, c.cons.type.as<int>(), c.cons.verts.as<int>(), S.V0.as<double>(), out);
    double d2;
    RIGC_TRY(read_scalars(c, reinterpret_cast<double*>(out), &d2, 1));
    *md = std::isfinite(d2) ? std::sqrt(d2) : -1;
    return RIGC_OK;
}

// max over vertices and coordinates of |V(x + d) - V(x)|
int max_vertex_move(Ctx& c, Sim& S, const double* x, const double* x1, double* m)
{
    RIGC_TRY(compute_world_vertices_rn(c, x, S.V0.as<double>(), c.scratch[5]));
    RIGC_TRY(compute_world_vertices_rn(c, x1, S.V1.as<double>(), c.scratch[5]));
    unsigned long long* out = reinterpret_cast<unsigned long long*>(S.scal.as<double>() + 13);
    RIGC_CUDA(cudaMemsetAsync(out, 0, sizeof(unsigned long long), c.stream));
    RIGC_COUNT_LAUNCH();
    k_max_vertex_move<<<grid_for(3 * (int64_t)S.nv, 256), 256, 0, c.stream>>>(
        S.nv, S.V0.as<double>(), S.V1.as<double>(), out);
    RIGC_TRY(read_scalars(c, reinterpret_cast<double*>(out), m, 1));
    return RIGC_OK;
}

int al_progress(Ctx& c, Sim& S, const double* x, double& eq, double& eQ)
{
    double* out = S.scal.as<double>() + 16;
    RIGC_COUNT_LAUNCH();
    k_al_progress<<<1, 256, 0, c.stream>>>(S.nb, c.s.type, x, S.al_xpred.as<double>(),
                                           S.x0.as<double>(), out);
    double a[4];
    RIGC_TRY(read_scalars(c, out, a, 4));
    eq = (a[0] == 0 && a[1] == 0) ? 1.0 : 1 - std::sqrt(a[0] / (a[1] == 0 ? 1 : a[1]));
    eQ = (a[2] == 0 && a[3] == 0) ? 1.0 : 1 - std::sqrt(a[2] / (a[3] == 0 ? 1 : a[3]));
    return RIGC_OK;
}

// are_equality_constraints_satisfied (:425-431)
int al_satisfied(Ctx& c, Sim& S, const double* x, bool& sat)
{
    sat = true;
    if (!S.has_kinematic) return RIGC_OK;
    double eq, eQ;
    RIGC_TRY(al_progress(c, S, x, eq, eQ));
    sat = eq >= 0.999 && eQ >= 0.999;
    return RIGC_OK;
}

// update_augmented_lagrangian (:339-423)
int al_update(Ctx& c, Sim& S, const double* x)
{
    double eq, eQ;
    RIGC_TRY(al_progress(c, S, x, eq, eQ));
    int upd_q = 0, upd_Q = 0;
    const double kq = S.al_kq, kQ = S.al_kQ;
    if (eq >= 0.999) S.al_sat_q = true;
    else if (eq < 0.99 && S.al_kq < 1e8) S.al_kq *= 2;
    else upd_q = 1;
    if (eQ >= 0.999) S.al_sat_Q = true;
    else if (eQ < 0.99 && S.al_kQ < 1e8) S.al_kQ *= 2;
    else upd_Q = 1;
    if (upd_q || upd_Q) {
        RIGC_COUNT_LAUNCH();
        k_al_update<<<grid_for(S.nb, 128), 128, 0, c.stream>>>(
            S.nb, c.s.type, x, S.al_xpred.as<double>(), S.mass.as<double>(), S.moment.as<double>(),
            upd_q, upd_Q, kq, kQ, S.al_lam.as<double>(), S.al_Lam.as<double>());
        RIGC_CUDA(cudaGetLastError());
    }
    return RIGC_OK;
}

int max_abs(Ctx& c, Sim& S, const double* v, double* m)
{
    const int64_t n = 6 * (int64_t)S.nb;
    unsigned long long* out = reinterpret_cast<unsigned long long*>(S.scal.as<double>() + 14);
    RIGC_CUDA(cudaMemsetAsync(out, 0, sizeof(unsigned long long), c.stream));
    RIGC_COUNT_LAUNCH();
    k_max_abs<<<grid_for(n, 256), 256, 0, c.stream>>>(n, v, out);
    RIGC_TRY(read_scalars(c, reinterpret_cast<double*>(out), m, 1));
    return RIGC_OK;
}

// ---- batched contexts: per-scene pieces of the driver

// device layout of S.sc_dev (ns doubles each): 0 scE = 1/m, 1 scB = kappa/m,
// 2 reg, 3 alpha, 4 rz, 5 rz_new, 6 pAp, 7 rr, 8 tol2, 9 cg alpha; then
// 2 ns ints of CG flags and ns ints of masks
struct ScenePtrs {
    double *scE, *scB, *reg, *alpha, *rz, *rz_new, *pAp, *rr, *tol2, *cga;
    int *flags, *mask, *on;
};

ScenePtrs scene_ptrs(Sim& S, int ns)
{
    double* d = S.sc_dev.as<double>();
    ScenePtrs P;
    P.scE = d;
    P.scB = d + ns;
    P.reg = d + 2 * ns;
    P.alpha = d + 3 * ns;
    P.rz = d + 4 * ns;
    P.rz_new = d + 5 * ns;
    P.pAp = d + 6 * ns;
    P.rr = d + 7 * ns;
    P.tol2 = d + 8 * ns;
    P.cga = d + 9 * ns;
    P.flags = reinterpret_cast<int*>(d + 10 * ns);
    P.mask = P.flags + 2 * ns;
    P.on = reinterpret_cast<int*>(d + 12 * ns);
    return P;
}

// restrict the broad phase (hence constraints, energies and the CCD) to the
// scenes in on (a host mask); restored by scene_all
int scene_only(Ctx& c, Sim& S, const std::vector<int>& on)
{
    ScenePtrs P = scene_ptrs(S, c.s.nscenes);
    RIGC_CUDA(cudaMemcpyAsync(P.on, on.data(), on.size() * sizeof(int), cudaMemcpyHostToDevice,
                              c.stream));
    c.scene_on = P.on;
    return RIGC_OK;
}
void scene_all(Ctx& c) { c.scene_on = nullptr; }

int upload(Ctx& c, double* dst, const std::vector<double>& v)
{
    RIGC_CUDA(cudaMemcpyAsync(dst, v.data(), v.size() * 8, cudaMemcpyHostToDevice, c.stream));
    return RIGC_OK;
}

// per-scene dot products of two dof vectors into host out (ns values)
int seg_dot(Ctx& c, Sim& S, const double* a, const double* b, std::vector<double>& out)
{
    const int ns = c.s.nscenes;
    RIGC_COUNT_LAUNCH();
    k_seg_dot<<<ns, 256, 0, c.stream>>>(c.s.scene_bstart, 6, a, b, S.sc_red.as<double>());
    out.resize(ns);
    RIGC_CUDA(cudaMemcpyAsync(out.data(), S.sc_red.ptr, (size_t)ns * 8, cudaMemcpyDeviceToHost, c.stream));
    RIGC_CUDA(cudaStreamSynchronize(c.stream));
    return RIGC_OK;
}

// per-scene objective E_s / m_s + kappa_s / m_s B_s (host f), with the
// gradient in S.g and the Hessian pieces when asked
int objective_scenes(Ctx& c, Sim& S, const double* x, bool grad_hess, const std::vector<double>& kappa,
                     std::vector<double>& f, Objective& O)
{
    const rigc_sim_params& p = S.p;
    const int ns = c.s.nscenes;
    rigc_body_state bs = state_of(S);
    double E;
    RIGC_TRY(body_energy(c, bs, x, p.gravity, p.timestep, &E, grad_hess ? S.gE.as<double>() : nullptr,
                         grad_hess ? S.hE.as<double>() : nullptr));
    std::vector<double> Es;
    RIGC_COUNT_LAUNCH();
    k_seg_dot<<<ns, 256, 0, c.stream>>>(c.s.scene_bstart, 1, c.scratch[0].as<double>(), nullptr,
                                        S.sc_red.as<double>());
    Es.resize(ns);
    RIGC_CUDA(cudaMemcpyAsync(Es.data(), S.sc_red.ptr, (size_t)ns * 8, cudaMemcpyDeviceToHost, c.stream));
    RIGC_TRY(build_constraints(c, x, p.dhat, p.dmin));
    const int flags = grad_hess ? (RIGC_GRAD | RIGC_HESS | RIGC_PROJECT_PSD) : 0;
    RIGC_TRY(barrier_term_impl(c, x, p.dhat, p.dmin, flags, &O.bo));  // syncs the stream
    O.fo = rigc_barrier_out {};
    f.resize(ns);
    for (int k = 0; k < ns; k++) {
        const double m = S.sc_mass[k];
        const double B = k < (int)c.h_scene_energy.size() ? c.h_scene_energy[k] : 0.0;
        f[k] = Es[k] / m + kappa[k] / m * B;
    }
    O.grad_hess = grad_hess;
    if (grad_hess) {
        ScenePtrs P = scene_ptrs(S, ns);
        RIGC_COUNT_LAUNCH();
        k_combine_grad_sc<<<grid_for(6 * S.nb, 256), 256, 0, c.stream>>>(
            S.nb, S.gE.as<double>(), O.bo.grad, c.s.bscene, P.scE, P.scB, S.fixed.as<int>(),
            S.g.as<double>());
        RIGC_CUDA(cudaGetLastError());
    }
    return RIGC_OK;
}

HessView hess_view_scenes(Sim& S, const Ctx& c, const Objective& O)
{
    const int ns = c.s.nscenes;
    ScenePtrs P = scene_ptrs(S, ns);
    HessView H {};
    H.body = S.hE.as<double>();
    H.brp = O.bo.nnzb > 0 ? O.bo.row_ptr : nullptr;
    H.bcol = O.bo.col;
    H.bval = O.bo.val;
    H.frp = nullptr;
    H.fixed = S.fixed.as<int>();
    H.nb = S.nb;
    H.bscene = c.s.bscene;
    H.scE = P.scE;
    H.scB = P.scB;
    H.scReg = P.reg;
    return H;
}

// block-Jacobi PCG per scene for (H + reg_s I) d = -g on the scenes with
// solve[s] set (the others keep S.sol); solved[s] on return
int pcg_scenes(Ctx& c, Sim& S, const HessView& H, const std::vector<int>& solve,
               std::vector<int>& solved, int64_t& iters)
{
    const int ns = c.s.nscenes;
    const int nb = S.nb;
    const int64_t n = 6 * (int64_t)nb;
    cudaStream_t st = c.stream;
    const unsigned gn = grid_for(n, 256), gs = grid_for(ns, 128);
    ScenePtrs P = scene_ptrs(S, ns);
    double* d = S.sol.as<double>();
    double* r = S.r.as<double>();
    double* z = S.z.as<double>();
    double* pp = S.pp.as<double>();
    double* Ap = S.Ap.as<double>();
    // flags: scenes not solved start converged
    std::vector<int> fl(2 * ns, 0);
    for (int k = 0; k < ns; k++) fl[2 * k + 1] = solve[k] ? 0 : 1;
    RIGC_CUDA(cudaMemcpyAsync(P.flags, fl.data(), fl.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    RIGC_CUDA(cudaMemcpyAsync(P.mask, solve.data(), ns * sizeof(int), cudaMemcpyHostToDevice, st));
    // r = -g on the solved scenes (0 elsewhere); d = 0 there (the other
    // scenes keep their solution)
    RIGC_COUNT_LAUNCH();
    k_axpy<<<gn, 256, 0, st>>>(n, -2.0, S.g.as<double>(), S.g.as<double>(), r);
    RIGC_COUNT_LAUNCH();
    k_mask_scenes<<<gn, 256, 0, st>>>(nb, c.s.bscene, P.mask, 1, r);
    RIGC_COUNT_LAUNCH();
    k_mask_scenes<<<gn, 256, 0, st>>>(nb, c.s.bscene, P.mask, 0, d);
    RIGC_COUNT_LAUNCH();
    k_block_jacobi<<<grid_for(nb, 64), 64, 0, st>>>(H, S.Minv.as<double>());
    RIGC_COUNT_LAUNCH();
    k_block_apply<<<gn, 256, 0, st>>>(nb, S.Minv.as<double>(), r, H.fixed, z);
    RIGC_CUDA(cudaMemcpyAsync(pp, z, n * 8, cudaMemcpyDeviceToDevice, st));
    RIGC_COUNT_LAUNCH();
    k_seg_dot<<<ns, 256, 0, st>>>(c.s.scene_bstart, 6, r, z, P.rz);
    RIGC_COUNT_LAUNCH();
    k_seg_dot<<<ns, 256, 0, st>>>(c.s.scene_bstart, 6, r, r, P.rr);
    std::vector<double> bb(ns);
    RIGC_CUDA(cudaMemcpyAsync(bb.data(), P.rr, ns * 8, cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaStreamSynchronize(st));
    std::vector<double> tol2(ns);
    for (int k = 0; k < ns; k++) tol2[k] = 1e-24 * bb[k];  // relative residual 1e-12
    RIGC_TRY(upload(c, P.tol2, tol2));
    solved.assign(ns, 0);
    for (int k = 0; k < ns; k++)
        if (solve[k] && bb[k] == 0) solved[k] = 1;
    iters = 0;
    const long long max_it = std::max<long long>(1000, 4 * n);
    // the iteration loop is one graph launch (a while node): the view and
    // the iteration count live in device memory (sc[20] iterations)
    long long* it_dev = reinterpret_cast<long long*>(S.scal.as<double>() + 20);
    RIGC_TRY(S.hview.reserve(sizeof(HessView)));
    HessView* Hd = S.hview.as<HessView>();
    const double* Minv = S.Minv.as<double>();
    const int* fixed = H.fixed;
    const int* bscene = c.s.bscene;
    const int* sbs = c.s.scene_bstart;
    const std::vector<unsigned long long> key = graph_key(
        { (const void*)Hd, d, r, z, pp, Ap, Minv, fixed, bscene, sbs, P.rz, P.flags, it_dev },
        { n, ns, max_it });
    auto body = [&](cudaStream_t cs, cudaGraphConditionalHandle loop) {
        k_hess_matvec_dev<<<gn, 256, 0, cs>>>(Hd, pp, Ap);
        k_seg_dot<<<ns, 256, 0, cs>>>(sbs, 6, pp, Ap, P.pAp);
        k_cg_alpha_sc<<<gs, 128, 0, cs>>>(ns, P.rz, P.pAp, P.rr, P.tol2, P.cga, P.flags);
        k_cg_update_sc<<<gn, 256, 0, cs>>>(nb, bscene, P.cga, pp, Ap, d, r);
        k_block_apply<<<gn, 256, 0, cs>>>(nb, Minv, r, fixed, z);
        k_seg_dot<<<ns, 256, 0, cs>>>(sbs, 6, r, z, P.rz_new);
        k_seg_dot<<<ns, 256, 0, cs>>>(sbs, 6, r, r, P.rr);
        k_cg_direction_sc<<<gn, 256, 0, cs>>>(nb, bscene, P.rz_new, P.rz, z, P.flags, pp);
        cudaMemcpyAsync(P.rz, P.rz_new, ns * 8, cudaMemcpyDeviceToDevice, cs);
        k_cg_continue_sc<<<1, 256, 0, cs>>>(ns, P.mask, P.flags, P.rr, P.tol2, it_dev, max_it, loop);
    };
    RIGC_TRY(loop_graph(S, S.cg_sc, key, 9, body));
    RIGC_CUDA(cudaMemcpyAsync(Hd, &H, sizeof(HessView), cudaMemcpyHostToDevice, st));
    RIGC_CUDA(cudaMemsetAsync(it_dev, 0, sizeof(long long), st));
    RIGC_CUDA(cudaGraphLaunch(S.cg_sc.exec, st));
    std::vector<double> rr(ns);
    long long its = 0;
    RIGC_CUDA(cudaMemcpyAsync(fl.data(), P.flags, 2 * ns * sizeof(int), cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaMemcpyAsync(rr.data(), P.rr, ns * 8, cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaMemcpyAsync(&its, it_dev, sizeof(long long), cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaStreamSynchronize(st));
    iters = its;
    count_launches(its * S.cg_sc.kernels);
    for (int k = 0; k < ns; k++) {
        if (!solve[k]) continue;
        if (fl[2 * k] || !std::isfinite(rr[k])) continue;  // broken down: not solved
        if (fl[2 * k + 1] || rr[k] <= tol2[k]) solved[k] = 1;
    }
    return RIGC_OK;
}

// per-scene minimum constraint distance at x (-1 without constraints)
int min_distance_scenes(Ctx& c, Sim& S, const double* x, std::vector<double>& md)
{
    const int ns = c.s.nscenes;
    RIGC_TRY(build_constraints(c, x, S.p.dhat, S.p.dmin));
    md.assign(ns, -1.0);
    const int64_t n = c.cons.num;
    if (n == 0) return RIGC_OK;
    RIGC_TRY(compute_world_vertices_rn(c, x, S.V0.as<double>(), c.scratch[5]));
    unsigned long long* out = reinterpret_cast<unsigned long long*>(S.sc_red.as<double>());
    std::vector<unsigned long long> inf(ns, 0x7ff0000000000000ull);
    RIGC_CUDA(cudaMemcpyAsync(out, inf.data(), ns * 8, cudaMemcpyHostToDevice, c.stream));
    RIGC_COUNT_LAUNCH();
    k_min_constraint_distance_sc<<<grid_for(n, 256), 256, 0, c.stream>>>(
        n, c.cons.type.as<int>(), c.cons.verts.as<int>(), c.cons.bodies.as<int>(), c.s.bscene,
        S.V0.as<double>(), out);
    std::vector<double> d2(ns);
    RIGC_CUDA(cudaMemcpyAsync(d2.data(), out, ns * 8, cudaMemcpyDeviceToHost, c.stream));
    RIGC_CUDA(cudaStreamSynchronize(c.stream));
    for (int k = 0; k < ns; k++) md[k] = std::isfinite(d2[k]) ? std::sqrt(d2[k]) : -1;
    return RIGC_OK;
}

int max_vertex_move_scenes(Ctx& c, Sim& S, const double* x, const double* x1, std::vector<double>& m)
{
    const int ns = c.s.nscenes;
    RIGC_TRY(compute_world_vertices_rn(c, x, S.V0.as<double>(), c.scratch[5]));
    RIGC_TRY(compute_world_vertices_rn(c, x1, S.V1.as<double>(), c.scratch[5]));
    RIGC_COUNT_LAUNCH();
    k_max_vertex_move_sc<<<ns, 256, 0, c.stream>>>(S.sc_vstart.as<int>(), S.V0.as<double>(),
                                                   S.V1.as<double>(), S.sc_red.as<double>());
    m.resize(ns);
    RIGC_CUDA(cudaMemcpyAsync(m.data(), S.sc_red.ptr, ns * 8, cudaMemcpyDeviceToHost, c.stream));
    RIGC_CUDA(cudaStreamSynchronize(c.stream));
    return RIGC_OK;
}

// One time step of every scene of a batched context, each scene as its own
// problem: the same solver as sim_step with per-scene stiffness (from the
// scene's average mass and bounding-box diagonal), regularisation, CCD
// step bound, line search, convergence and stiffness updates; the kernels
// run over all scenes at once.  Friction and the polish are not supported
// here (RIGC_ERR_ARG).  Per-scene linear solves by block-Jacobi PCG.
// The free dofs' compact indices from the bodies' fixed flags (the
// reference's free_dof slicing) and the dense solver's buffers for them.
int set_free_dofs(Ctx& c, Sim& S)
{
    const int nb = S.nb;
    std::vector<int> fidx(6 * (size_t)nb, -1);
    int nf = 0;
    for (int b = 0; b < nb; b++)
        for (int k = 0; k < 6; k++)
            if (!((S.h_fixed[b] >> k) & 1)) fidx[6 * b + k] = nf++;
    S.nfree = nf;
    RIGC_TRY(S.free_idx.reserve(fidx.size() * sizeof(int) + 8));
    RIGC_CUDA(cudaMemcpyAsync(S.free_idx.ptr, fidx.data(), fidx.size() * sizeof(int),
                              cudaMemcpyHostToDevice, c.stream));
    if (nf <= kDenseMax) {
        RIGC_TRY(S.dense.reserve((size_t)nf * nf * sizeof(double) + 8));
        RIGC_TRY(S.dense_b.reserve((size_t)nf * sizeof(double) + 8));
        RIGC_TRY(S.dense_x.reserve((size_t)nf * sizeof(double) + 8));
        RIGC_TRY(S.dense_d.reserve((size_t)nf * sizeof(double) + 8));
    }
    RIGC_CUDA(cudaStreamSynchronize(c.stream));
    return RIGC_OK;
}

// RigidBody::convert_to_static (rigid_body.hpp:186-193): the body static,
// every dof fixed, its velocity zero
int convert_to_static(Ctx& c, Sim& S, int b)
{
    const int stat = RIGC_BODY_STATIC, all = 0x3f;
    c.s.h_type[b] = stat;
    S.h_fixed[b] = all;
    RIGC_CUDA(cudaMemcpyAsync(c.s.type + b, &stat, sizeof(int), cudaMemcpyHostToDevice, c.stream));
    RIGC_CUDA(cudaMemcpyAsync(S.fixed.as<int>() + b, &all, sizeof(int), cudaMemcpyHostToDevice, c.stream));
    RIGC_CUDA(cudaMemsetAsync(S.vel.as<double>() + 6 * (size_t)b, 0, 6 * sizeof(double), c.stream));
    RIGC_CUDA(cudaStreamSynchronize(c.stream));
    return RIGC_OK;
}

// init_augmented_lagrangian's part of the schedules
// (distance_barrier_rb_problem.cpp:204-226): *target the step's targets, or
// null without any scheduled pose
int kinematic_targets(Ctx& c, Sim& S, const double** target)
{
    *target = nullptr;
    if (S.kin_max_time.empty()) return RIGC_OK;
    const int nb = S.nb;
    bool changed = false, any = false;
    std::vector<double> t(6 * (size_t)nb, NAN);
    for (int b = 0; b < nb; b++) {
        if (c.s.h_type[b] != RIGC_BODY_KINEMATIC) continue;
        if (S.kin_max_time[b] < 0) {
            RIGC_TRY(convert_to_static(c, S, b));
            changed = true;
        } else if (!S.kin_poses[b].empty()) {
            for (int k = 0; k < 6; k++) t[6 * (size_t)b + k] = S.kin_poses[b].front()[k];
            any = true;
        }
    }
    if (changed) {
        RIGC_TRY(set_free_dofs(c, S));
        S.has_kinematic = false;
        for (int b = 0; b < nb; b++) S.has_kinematic |= c.s.h_type[b] == RIGC_BODY_KINEMATIC;
    }
    if (!any) return RIGC_OK;
    RIGC_TRY(S.kin_target.reserve(t.size() * sizeof(double)));
    RIGC_CUDA(cudaMemcpyAsync(S.kin_target.ptr, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice,
                              c.stream));
    RIGC_CUDA(cudaStreamSynchronize(c.stream));
    *target = S.kin_target.as<double>();
    return RIGC_OK;
}

// step_kinematic_bodies (distance_barrier_rb_problem.cpp:237-251)
int advance_kinematic(Ctx& c, Sim& S)
{
    if (S.kin_max_time.empty()) return RIGC_OK;
    bool changed = false;
    for (int b = 0; b < S.nb; b++) {
        if (c.s.h_type[b] != RIGC_BODY_KINEMATIC) continue;
        if (S.kin_max_time[b] < 0) {
            RIGC_TRY(convert_to_static(c, S, b));
            changed = true;
        } else {
            S.kin_max_time[b] -= S.p.timestep;
            if (!S.kin_poses[b].empty()) S.kin_poses[b].pop_front();
        }
    }
    if (changed) {
        RIGC_TRY(set_free_dofs(c, S));
        S.has_kinematic = false;
        for (int b = 0; b < S.nb; b++) S.has_kinematic |= c.s.h_type[b] == RIGC_BODY_KINEMATIC;
    }
    return RIGC_OK;
}

int sim_step_scenes(Ctx& c, rigc_step_stats* stats)
{
    Sim& S = *c.sim;
    const rigc_sim_params& p = S.p;
    if (p.coefficient_friction > 0 || p.newton_polish > 0 || S.has_kinematic) return RIGC_ERR_ARG;
    const int ns = c.s.nscenes, nb = S.nb;
    const int64_t n = 6 * (int64_t)nb;
    cudaStream_t st = c.stream;
    const unsigned gn = grid_for(n, 256);
    ScenePtrs P = scene_ptrs(S, ns);
    double* x0 = S.x0.as<double>();
    double* x = S.x.as<double>();
    double* xt = S.xt.as<double>();
    double* dir = S.dir.as<double>();
    rigc_step_stats local {};
    struct AllScenesOnExit {
        Ctx& c;
        ~AllScenesOnExit() { scene_all(c); }
    } guard { c };
    scene_all(c);
    std::vector<double> kappa(ns), kmax(ns), prev_md(ns), coeff(ns, 0.0), alpha(ns), lb(ns), f, ft;
    std::vector<double> scE(ns), scB(ns), reg(ns, 0.0);
    auto upload_scales = [&]() -> int {
        for (int k = 0; k < ns; k++) {
            scE[k] = 1.0 / S.sc_mass[k];
            scB[k] = kappa[k] / S.sc_mass[k];
        }
        RIGC_TRY(upload(c, P.scE, scE));
        RIGC_TRY(upload(c, P.scB, scB));
        return RIGC_OK;
    };

    // IPCSolver::init_solve per scene
    {
        rigc_body_state bs = state_of(S);
        double E;
        RIGC_TRY(body_energy(c, bs, x0, p.gravity, p.timestep, &E, S.gE.as<double>(), nullptr));
        RIGC_TRY(build_constraints(c, x0, p.dhat, p.dmin));
        rigc_barrier_out bo;
        RIGC_TRY(barrier_term_impl(c, x0, p.dhat, p.dmin, RIGC_GRAD, &bo));
        RIGC_CUDA(cudaMemcpyAsync(S.gtmp.ptr, bo.grad, n * 8, cudaMemcpyDeviceToDevice, st));
        std::vector<double> gg, ge;
        RIGC_TRY(seg_dot(c, S, S.gtmp.as<double>(), S.gtmp.as<double>(), gg));
        RIGC_TRY(seg_dot(c, S, S.gtmp.as<double>(), S.gE.as<double>(), ge));
        const double dmin = p.dmin;
        for (int k = 0; k < ns; k++) {
            double d0 = 1e-8 * S.sc_bbox[k] + dmin;
            d0 *= d0;
            const double sb = 2 * dmin * p.dhat + p.dhat * p.dhat;
            if (d0 - dmin * dmin >= sb) d0 = dmin * p.dhat + 0.5 * p.dhat * p.dhat;
            double kmin = 4 * d0 * barrier_hessian_d(d0 - dmin * dmin, sb);
            kmin = p.min_barrier_stiffness_scale * S.sc_mass[k] / kmin;
            kmax[k] = 100 * kmin;
            const double k0 = gg[k] > 0 ? -ge[k] / gg[k] : 1.0;
            kappa[k] = std::min(kmax[k], std::max(kmin, k0));
        }
    }
    RIGC_TRY(min_distance_scenes(c, S, x0, prev_md));

    RIGC_CUDA(cudaMemcpyAsync(x, x0, n * 8, cudaMemcpyDeviceToDevice, st));
    // state per scene: 0 iterating, 1 done
    std::vector<int> done(ns, 0), solve(ns), solved, mask(ns);
    std::vector<double> gdv;
    int it = 0;
    for (; it < p.max_newton_iterations; it++) {
        int active = 0;
        for (int k = 0; k < ns; k++) active += !done[k];
        if (!active) break;
        RIGC_TRY(upload_scales());
        Objective O;
        std::vector<int> on(ns);
        for (int k = 0; k < ns; k++) on[k] = !done[k];
        RIGC_TRY(scene_only(c, S, on));
        RIGC_TRY(objective_scenes(c, S, x, true, kappa, f, O));
        local.objective_evals++;
        // compute_regularized_direction per scene
        for (int k = 0; k < ns; k++) solve[k] = !done[k];
        std::vector<int> ok(ns, 0);
        for (;;) {
            int any = 0;
            for (int k = 0; k < ns; k++) any |= solve[k];
            if (!any) break;
            for (int k = 0; k < ns; k++) reg[k] = coeff[k];
            RIGC_TRY(upload(c, P.reg, reg));
            HessView H = hess_view_scenes(S, c, O);
            int64_t cgit;
            RIGC_TRY(pcg_scenes(c, S, H, solve, solved, cgit));
            local.cg_iterations += cgit;
            RIGC_TRY(seg_dot(c, S, S.g.as<double>(), S.sol.as<double>(), gdv));
            for (int k = 0; k < ns; k++) {
                if (!solve[k]) continue;
                const bool good = solved[k] && gdv[k] <= 0;
                if (good) {
                    coeff[k] /= 2;
                    if (coeff[k] < 1e-8) coeff[k] = 0;
                    ok[k] = 1;
                    solve[k] = 0;
                } else {
                    coeff[k] = std::max(2 * coeff[k], 1e-8);
                    if (!std::isfinite(coeff[k])) {
                        solve[k] = 0;  // regularisation failed: the scene stops
                        done[k] = 1;
                    }
                }
            }
        }
        for (int k = 0; k < ns; k++) mask[k] = !done[k] && ok[k];
        RIGC_CUDA(cudaMemcpyAsync(P.mask, mask.data(), ns * sizeof(int), cudaMemcpyHostToDevice, st));
        RIGC_CUDA(cudaMemcpyAsync(dir, S.sol.ptr, n * 8, cudaMemcpyDeviceToDevice, st));
        RIGC_COUNT_LAUNCH();
        k_mask_scenes<<<gn, 256, 0, st>>>(nb, c.s.bscene, P.mask, 1, dir);
        // velocity convergence
        if (it > 0) {
            RIGC_COUNT_LAUNCH();
            k_axpy<<<gn, 256, 0, st>>>(n, 1.0, dir, x, xt);
            std::vector<double> mv;
            RIGC_TRY(max_vertex_move_scenes(c, S, x, xt, mv));
            for (int k = 0; k < ns; k++) {
                if (!mask[k]) continue;
                const double tol = p.velocity_conv_tol * (p.velocity_conv_tol_abs ? 1.0 : S.sc_bbox[k]);
                if (mv[k] / p.timestep <= tol) {
                    done[k] = 1;
                    mask[k] = 0;
                }
            }
        }
        // line search per scene over the scenes in mask (the gradient on the
        // free dofs is S.g); found[k] and alpha[k] on return
        std::vector<int> found(ns, 0);
        auto line_search = [&](std::vector<int>& search) -> int {
            RIGC_TRY(seg_dot(c, S, S.g.as<double>(), dir, gdv));
            RIGC_COUNT_LAUNCH();
            k_axpy<<<gn, 256, 0, st>>>(n, 1.0, dir, x, xt);
            double toi;
            RIGC_TRY(scene_only(c, S, search));
            RIGC_TRY(detect_and_count(c, x, xt, true, p.dmin / 2.0));
            int s2 = run_ccd(c, x, xt, 1e-4, 0, &toi, nullptr);
            if (s2 != RIGC_OK && s2 != RIGC_ERR_QUEUE_OVERFLOW && s2 != RIGC_ERR_ITER_LIMIT) return s2;
            local.ccd_calls++;
            for (int k = 0; k < ns; k++) {
                if (!search[k]) continue;
                lb[k] = std::min(p.line_search_lower_bound / std::sqrt(std::fabs(gdv[k])), 1e-1);
                const double tk = k < (int)c.h_scene_toi.size() ? c.h_scene_toi[k] : toi;
                alpha[k] = std::min(1.0, tk < 1.0 ? p.ccd_rescale * tk : tk);
            }
            for (;;) {
                std::vector<double> a(ns, 0.0);
                int any = 0;
                for (int k = 0; k < ns; k++)
                    if (search[k] && !found[k] && std::isfinite(lb[k]) && alpha[k] >= lb[k]) {
                        a[k] = alpha[k];
                        any = 1;
                    }
                if (!any) break;
                RIGC_TRY(upload(c, P.alpha, a));
                RIGC_COUNT_LAUNCH();
                k_axpy_sc<<<gn, 256, 0, st>>>(nb, c.s.bscene, P.alpha, dir, x, xt);
                std::vector<int> on_t(ns);
                for (int k = 0; k < ns; k++) on_t[k] = a[k] != 0;
                RIGC_TRY(scene_only(c, S, on_t));
                Objective Oi;
                RIGC_TRY(objective_scenes(c, S, xt, false, kappa, ft, Oi));
                local.objective_evals++;
                for (int k = 0; k < ns; k++) {
                    if (a[k] == 0) continue;
                    if (ft[k] < f[k]) found[k] = 1;
                    else alpha[k] /= 2.0;
                }
            }
            return RIGC_OK;
        };
        std::vector<int> search = mask;
        RIGC_TRY(line_search(search));
        // gradient fallback: d = -g on the scenes without a step
        std::vector<int> retry(ns, 0);
        int any_retry = 0;
        for (int k = 0; k < ns; k++) {
            retry[k] = mask[k] && !found[k];
            any_retry |= retry[k];
        }
        if (any_retry) {
            RIGC_CUDA(cudaMemcpyAsync(P.mask, retry.data(), ns * sizeof(int), cudaMemcpyHostToDevice, st));
            RIGC_COUNT_LAUNCH();
            k_axpy<<<gn, 256, 0, st>>>(n, -2.0, S.g.as<double>(), S.g.as<double>(), xt);
            // dir = -g on the retried scenes, unchanged elsewhere
            RIGC_COUNT_LAUNCH();
            k_mask_scenes<<<gn, 256, 0, st>>>(nb, c.s.bscene, P.mask, 1, xt);
            RIGC_COUNT_LAUNCH();
            k_mask_scenes<<<gn, 256, 0, st>>>(nb, c.s.bscene, P.mask, 0, dir);
            RIGC_COUNT_LAUNCH();
            k_axpy<<<gn, 256, 0, st>>>(n, 1.0, xt, dir, dir);
            RIGC_TRY(line_search(retry));
            for (int k = 0; k < ns; k++)
                if (retry[k] && !found[k]) done[k] = 1;  // line search failed: the scene stops
        }
        // x += alpha_s d on the scenes with a step
        std::vector<double> a(ns, 0.0);
        // (an iteration counts once it takes its step, as in sim_step)
        for (int k = 0; k < ns; k++)
            if (found[k]) {
                a[k] = alpha[k];
                local.newton_steps++;
                local.newton_iterations++;
            }
        RIGC_TRY(upload(c, P.alpha, a));
        RIGC_COUNT_LAUNCH();
        k_axpy_sc<<<gn, 256, 0, st>>>(nb, c.s.bscene, P.alpha, dir, x, x);
        // adaptive stiffness per scene
        std::vector<double> md;
        RIGC_TRY(scene_only(c, S, found));
        RIGC_TRY(min_distance_scenes(c, S, x, md));
        scene_all(c);
        for (int k = 0; k < ns; k++) {
            if (!found[k]) continue;
            const double eps = p.dhat_epsilon * (S.sc_bbox[k] + p.dmin);
            if (prev_md[k] < eps && md[k] < eps && md[k] < prev_md[k])
                kappa[k] = std::min(kmax[k], 2 * kappa[k]);
            prev_md[k] = md[k];
        }
    }

    // take_step
    scene_all(c);
    RIGC_COUNT_LAUNCH();
    k_take_step<<<grid_for(nb, 128), 128, 0, st>>>(nb, c.s.type, S.fixed.as<int>(), x, x0,
                                                   S.vel.as<double>(), S.Qdot.as<double>(),
                                                   p.timestep);
    RIGC_CUDA(cudaGetLastError());
    RIGC_CUDA(cudaStreamSynchronize(st));
    S.kappa = *std::max_element(kappa.begin(), kappa.end());
    if (stats) {
        stats->newton_iterations += local.newton_iterations;
        stats->newton_steps += local.newton_steps;
        stats->objective_evals += local.objective_evals;
        stats->ccd_calls += local.ccd_calls;
        stats->cg_iterations += local.cg_iterations;
        stats->barrier_stiffness = S.kappa;
    }
    return RIGC_OK;
}

} // namespace

int sim_init(Ctx& c, const rigc_sim_params& p, const rigc_sim_state& s)
{
    if (!c.sim) c.sim = new Sim;
    Sim& S = *c.sim;
    S.p = p;
    S.nb = c.s.nb;
    S.nv = c.s.nv;
    const int nb = S.nb;
    const size_t v6 = (size_t)6 * nb * sizeof(double) + 64;
    DevBuf* vecs[] = { &S.x0, &S.vel, &S.x, &S.xt, &S.dir, &S.g, &S.gE, &S.gtmp,
                       &S.r, &S.z, &S.pp, &S.Ap, &S.sol };
    for (DevBuf* b : vecs) RIGC_TRY(b->reserve(v6));
    RIGC_TRY(S.mass.reserve((size_t)nb * 8 + 8));
    RIGC_TRY(S.moment.reserve((size_t)nb * 24 + 8));
    RIGC_TRY(S.fixed.reserve((size_t)nb * 4 + 8));
    RIGC_TRY(S.Qdot.reserve((size_t)nb * 72 + 8));
    RIGC_TRY(S.hE.reserve((size_t)nb * 36 * 8 + 8));
    RIGC_TRY(S.Minv.reserve((size_t)nb * 36 * 8 + 8));
    RIGC_TRY(S.part.reserve(64 * 8));
    RIGC_TRY(S.scal.reserve(32 * 8));
    RIGC_TRY(S.V0.reserve((size_t)S.nv * 24 + 8));
    RIGC_TRY(S.V1.reserve((size_t)S.nv * 24 + 8));
    cudaStream_t st = c.stream;
    RIGC_CUDA(cudaMemcpyAsync(S.mass.ptr, s.mass, (size_t)nb * 8, cudaMemcpyHostToDevice, st));
    RIGC_CUDA(cudaMemcpyAsync(S.moment.ptr, s.moment, (size_t)nb * 24, cudaMemcpyHostToDevice, st));
    RIGC_CUDA(cudaMemcpyAsync(S.fixed.ptr, s.dof_fixed, (size_t)nb * 4, cudaMemcpyHostToDevice, st));
    RIGC_CUDA(cudaMemcpyAsync(S.x0.ptr, s.poses, (size_t)nb * 48, cudaMemcpyHostToDevice, st));
    RIGC_CUDA(cudaMemcpyAsync(S.vel.ptr, s.velocities, (size_t)nb * 48, cudaMemcpyHostToDevice, st));
    RIGC_CUDA(cudaMemcpyAsync(S.Qdot.ptr, s.Qdot, (size_t)nb * 72, cudaMemcpyHostToDevice, st));
    RIGC_CUDA(cudaStreamSynchronize(st));
    S.h_fixed.assign(s.dof_fixed, s.dof_fixed + nb);
    RIGC_TRY(set_free_dofs(c, S));
    S.kin_max_time.clear();
    S.kin_poses.clear();
    // per-scene set-up of batched contexts (average mass and bounding-box
    // diagonal default to the global ones; rigc_sim_scene_params sets them)
    const int ns = c.s.nscenes;
    S.sc_mass.assign(ns, p.average_mass);
    S.sc_bbox.assign(ns, p.world_bbox_diagonal);
    RIGC_TRY(S.sc_dev.reserve((size_t)ns * 13 * 8 + 64));
    RIGC_TRY(S.sc_red.reserve((size_t)ns * 8 + 64));
    {
        std::vector<int> vs(ns + 1);
        for (int k = 0; k <= ns; k++) vs[k] = c.s.h_bvs[c.s.h_scene_bstart[k]];
        RIGC_TRY(S.sc_vstart.reserve((size_t)(ns + 1) * sizeof(int) + 8));
        RIGC_CUDA(cudaMemcpyAsync(S.sc_vstart.ptr, vs.data(), vs.size() * sizeof(int),
                                  cudaMemcpyHostToDevice, st));
        RIGC_CUDA(cudaStreamSynchronize(st));
    }
    S.has_kinematic = false;
    for (int b = 0; b < nb; b++) S.has_kinematic |= c.s.h_type[b] == RIGC_BODY_KINEMATIC;
    RIGC_TRY(S.al_xpred.reserve((size_t)nb * 48 + 64));
    RIGC_TRY(S.al_lam.reserve((size_t)nb * 24 + 64));
    RIGC_TRY(S.al_Lam.reserve((size_t)nb * 72 + 64));
    RIGC_TRY(S.al_e.reserve((size_t)nb * 8 + 64));
    S.kappa = 1;  // m_barrier_stiffness before the first solve
    S.tape_steps = 0;
    S.tape_every = 0;
    return RIGC_OK;
}

int sim_step(Ctx& c, rigc_step_stats* stats)
{
    if (!c.sim) return RIGC_ERR_ARG;
    if (c.s.nscenes > 1) return sim_step_scenes(c, stats);
    Sim& S = *c.sim;
    const rigc_sim_params& p = S.p;
    const int nb = S.nb;
    const int64_t n = 6 * (int64_t)nb;
    cudaStream_t st = c.stream;
    double* x0 = S.x0.as<double>();
    double* x = S.x.as<double>();
    double* xt = S.xt.as<double>();
    double* dir = S.dir.as<double>();
    rigc_step_stats local {};
    S.dense_step = false;

    // update_constraints: lagged friction at x0 with the current stiffness
    if (p.coefficient_friction > 0) {
        RIGC_TRY(build_constraints(c, x0, p.dhat, p.dmin));
        RIGC_TRY(friction_setup(c, x0, p.dhat, S.kappa, p.coefficient_friction, 0.0));
    }
    // init_augmented_lagrangian: kinematic bodies whose time has run out
    // become static, the others' targets are their scheduled poses or
    // x0 + h v
    S.al_kq = S.al_kQ = 1e3;
    S.al_sat_q = S.al_sat_Q = false;
    const double* kin_target = nullptr;
    RIGC_TRY(kinematic_targets(c, S, &kin_target));
    if (S.has_kinematic) {
        RIGC_COUNT_LAUNCH();
        k_al_init<<<grid_for(nb, 128), 128, 0, st>>>(nb, c.s.type, x0, S.vel.as<double>(), p.timestep,
                                                     kin_target, S.al_xpred.as<double>(),
                                                     S.al_lam.as<double>(), S.al_Lam.as<double>());
    }

    // IPCSolver::init_solve
    {
        rigc_body_state bs = state_of(S);
        double E;
        RIGC_TRY(body_energy(c, bs, x0, p.gravity, p.timestep, &E, S.gE.as<double>(), nullptr));
        RIGC_TRY(build_constraints(c, x0, p.dhat, p.dmin));
        rigc_barrier_out bo;
        RIGC_TRY(barrier_term_impl(c, x0, p.dhat, p.dmin, RIGC_GRAD, &bo));
        RIGC_CUDA(cudaMemcpyAsync(S.gtmp.ptr, bo.grad, n * 8, cudaMemcpyDeviceToDevice, st));
        const double gg = host_dot(c, S, S.gtmp.as<double>(), S.gtmp.as<double>());
        const double ge = host_dot(c, S, S.gtmp.as<double>(), S.gE.as<double>());
        const double dmin = p.dmin;
        double d0 = 1e-8 * p.world_bbox_diagonal + dmin;
        d0 *= d0;
        const double sb = 2 * dmin * p.dhat + p.dhat * p.dhat;
        if (d0 - dmin * dmin >= sb) d0 = dmin * p.dhat + 0.5 * p.dhat * p.dhat;
        double kmin = 4 * d0 * barrier_hessian_d(d0 - dmin * dmin, sb);
        kmin = p.min_barrier_stiffness_scale * p.average_mass / kmin;
        S.kappa_max = 100 * kmin;
        const double k0 = gg > 0 ? -ge / gg : 1.0;
        S.kappa = std::min(S.kappa_max, std::max(kmin, k0));
        S.dk = (gg > 0 && k0 > kmin && k0 < S.kappa_max) ? 1.0 : 0.0;
    }
    double prev_min_distance;
    RIGC_TRY(min_distance(c, S, x0, &prev_min_distance));

    RIGC_CUDA(cudaMemcpyAsync(x, x0, n * 8, cudaMemcpyDeviceToDevice, st));
    double coeff = 0;
    bool energy_converged = false;
    int it = 0;
    for (; it < p.max_newton_iterations; it++) {
        Objective O;
        RIGC_TRY(objective(c, S, x, true, O));
        local.objective_evals++;
        const double fx = O.f;
        // compute_regularized_direction
        bool ok = false;
        while (!ok) {
            bool solved;
            int64_t cgit;
            HessView H = hess_view(S, O, coeff);
            RIGC_TRY(newton_solve(c, S, H, solved, cgit));
            local.cg_iterations += cgit;
            double gd = solved ? host_dot(c, S, S.g.as<double>(), S.sol.as<double>()) : 0;
            ok = solved && gd <= 0;
            if (ok) {
                coeff /= 2;
                if (coeff < 1e-8) coeff = 0;
            } else {
                coeff = std::max(2 * coeff, 1e-8);
                if (!std::isfinite(coeff)) break;
            }
        }
        if (!ok) break;
        RIGC_CUDA(cudaMemcpyAsync(dir, S.sol.ptr, n * 8, cudaMemcpyDeviceToDevice, st));
        // velocity convergence
        if (it > 0) {
            RIGC_COUNT_LAUNCH();
            k_axpy<<<grid_for(n, 256), 256, 0, st>>>(n, 1.0, dir, x, xt);
            double mv;
            RIGC_TRY(max_vertex_move(c, S, x, xt, &mv));
            const double tol = p.velocity_conv_tol * (p.velocity_conv_tol_abs ? 1.0 : p.world_bbox_diagonal);
            energy_converged = mv / p.timestep <= tol;
            bool sat;
            RIGC_TRY(al_satisfied(c, S, x, sat));
            if (energy_converged && sat) break;
        }
        // line search (the gradient on the free dofs is S.g)
        auto line_search = [&](double& alpha, bool& found) -> int {
            found = false;
            const double gdv = host_dot(c, S, S.g.as<double>(), dir);
            const double lb = std::min(p.line_search_lower_bound / std::sqrt(std::fabs(gdv)), 1e-1);
            RIGC_COUNT_LAUNCH();
            k_axpy<<<grid_for(n, 256), 256, 0, st>>>(n, 1.0, dir, x, xt);
            double toi;
            RIGC_TRY(detect_and_count(c, x, xt, true, p.dmin / 2.0));
            int s2 = line_search_ccd(c, p, x, xt, &toi);
            if (s2 != RIGC_OK && s2 != RIGC_ERR_QUEUE_OVERFLOW && s2 != RIGC_ERR_ITER_LIMIT) return s2;
            local.ccd_calls++;
            alpha = std::min(1.0, toi < 1.0 ? p.ccd_rescale * toi : toi);
            while (std::isfinite(lb) && alpha >= lb) {
                RIGC_COUNT_LAUNCH();
                k_axpy<<<grid_for(n, 256), 256, 0, st>>>(n, alpha, dir, x, xt);
                Objective Oi;
                RIGC_TRY(objective(c, S, xt, false, Oi));
                local.objective_evals++;
                if (Oi.f < fx) {
                    found = true;
                    return RIGC_OK;
                }
                alpha /= 2.0;
            }
            return RIGC_OK;
        };
        double alpha = 1;
        bool found;
        RIGC_TRY(line_search(alpha, found));
        if (!found) {
            // gradient fallback: d = -g
            RIGC_COUNT_LAUNCH();
            k_axpy<<<grid_for(n, 256), 256, 0, st>>>(n, -2.0, S.g.as<double>(), S.g.as<double>(), dir);
            alpha = 1;
            RIGC_TRY(line_search(alpha, found));
            if (!found) break;
        }
        RIGC_COUNT_LAUNCH();
        k_axpy<<<grid_for(n, 256), 256, 0, st>>>(n, alpha, dir, x, x);
        local.newton_steps++;
        // NewtonSolver::post_step_update: augmented Lagrangian
        if (energy_converged && S.has_kinematic) {
            bool sat;
            RIGC_TRY(al_satisfied(c, S, x, sat));
            if (!sat) RIGC_TRY(al_update(c, S, x));
        }
        // adaptive stiffness
        double md;
        RIGC_TRY(min_distance(c, S, x, &md));
        const double eps = p.dhat_epsilon * (p.world_bbox_diagonal + p.dmin);
        if (prev_min_distance < eps && md < eps && md < prev_min_distance) {
            S.dk = 2 * S.kappa < S.kappa_max ? 2 * S.dk : 0.0;
            S.kappa = std::min(S.kappa_max, 2 * S.kappa);
        }
        prev_min_distance = md;
    }
    local.newton_iterations = it;

    // optional polish: full Newton steps with the unprojected Hessian while
    // they keep contracting and the CCD admits the full step (the line
    // search's decrease test stalls at |dx| ~ sqrt(eps))
    double prev_step = INFINITY;
    for (int k = 0; k < p.newton_polish; k++) {
        Objective O;
        RIGC_TRY(objective(c, S, x, true, O, false));
        local.objective_evals++;
        bool solved;
        int64_t cgit = 0;
        HessView H = hess_view(S, O, 0.0);
        RIGC_TRY(newton_solve(c, S, H, solved, cgit));
        local.cg_iterations += cgit;
        if (!solved) break;
        const double gd = host_dot(c, S, S.g.as<double>(), S.sol.as<double>());
        double step;
        RIGC_TRY(max_abs(c, S, S.sol.as<double>(), &step));
        if (!(step > 0) || gd > 0 || step >= 0.5 * prev_step) break;
        RIGC_COUNT_LAUNCH();
        k_axpy<<<grid_for(n, 256), 256, 0, st>>>(n, 1.0, S.sol.as<double>(), x, xt);
        double toi;
        RIGC_TRY(detect_and_count(c, x, xt, true, p.dmin / 2.0));
        int s2 = line_search_ccd(c, p, x, xt, &toi);
        if (s2 != RIGC_OK && s2 != RIGC_ERR_QUEUE_OVERFLOW && s2 != RIGC_ERR_ITER_LIMIT) return s2;
        local.ccd_calls++;
        if (toi < 1.0) break;
        RIGC_CUDA(cudaMemcpyAsync(x, xt, n * 8, cudaMemcpyDeviceToDevice, st));
        prev_step = step;
        local.newton_steps++;
    }

    // take_step
    RIGC_COUNT_LAUNCH();
    k_take_step<<<grid_for(nb, 128), 128, 0, st>>>(nb, c.s.type, S.fixed.as<int>(), x, x0,
                                                   S.vel.as<double>(), S.Qdot.as<double>(),
                                                   p.timestep);
    RIGC_CUDA(cudaGetLastError());
    RIGC_CUDA(cudaStreamSynchronize(st));
    RIGC_TRY(advance_kinematic(c, S));
    local.barrier_stiffness = S.kappa;
    if (stats) {
        stats->newton_iterations += local.newton_iterations;
        stats->newton_steps += local.newton_steps;
        stats->objective_evals += local.objective_evals;
        stats->ccd_calls += local.ccd_calls;
        stats->cg_iterations += local.cg_iterations;
        stats->barrier_stiffness = local.barrier_stiffness;
    }
    return RIGC_OK;
}

int sim_set_kinematic(Ctx& c, int body, double max_time, int64_t num_poses, const double* poses)
{
    if (!c.sim || c.s.nscenes > 1 || body < 0 || body >= c.s.nb || num_poses < 0 || (num_poses && !poses))
        return RIGC_ERR_ARG;
    if (c.s.h_type[body] != RIGC_BODY_KINEMATIC) return RIGC_ERR_ARG;
    Sim& S = *c.sim;
    if (S.kin_max_time.empty()) {
        S.kin_max_time.assign(S.nb, INFINITY);
        S.kin_poses.assign(S.nb, {});
    }
    // read_rb_scene.cpp:99-101: a negative time is no limit
    S.kin_max_time[body] = max_time < 0 ? INFINITY : max_time;
    S.kin_poses[body].clear();
    for (int64_t i = 0; i < num_poses; i++) {
        std::array<double, 6> q;
        for (int k = 0; k < 6; k++) q[k] = poses[6 * i + k];
        S.kin_poses[body].push_back(q);
    }
    return RIGC_OK;
}

int sim_scene_params(Ctx& c, const double* average_mass, const double* bbox_diagonal)
{
    if (!c.sim) return RIGC_ERR_ARG;
    Sim& S = *c.sim;
    for (int k = 0; k < c.s.nscenes; k++) {
        if (average_mass && !(average_mass[k] > 0)) return RIGC_ERR_ARG;
        if (bbox_diagonal && !(bbox_diagonal[k] > 0)) return RIGC_ERR_ARG;
    }
    for (int k = 0; k < c.s.nscenes; k++) {
        if (average_mass) S.sc_mass[k] = average_mass[k];
        if (bbox_diagonal) S.sc_bbox[k] = bbox_diagonal[k];
    }
    return RIGC_OK;
}

int sim_get_state(Ctx& c, double* poses, double* velocities, double* Qdot, double* kappa)
{
    if (!c.sim) return RIGC_ERR_ARG;
    Sim& S = *c.sim;
    const int nb = S.nb;
    cudaStream_t st = c.stream;
    if (poses) RIGC_CUDA(cudaMemcpyAsync(poses, S.x0.ptr, (size_t)nb * 48, cudaMemcpyDeviceToHost, st));
    if (velocities)
        RIGC_CUDA(cudaMemcpyAsync(velocities, S.vel.ptr, (size_t)nb * 48, cudaMemcpyDeviceToHost, st));
    if (Qdot) RIGC_CUDA(cudaMemcpyAsync(Qdot, S.Qdot.ptr, (size_t)nb * 72, cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaStreamSynchronize(st));
    if (kappa) *kappa = S.kappa;
    return RIGC_OK;
}

// ---------------------------------------------------------------------------
// rollout with checkpoints and its adjoint

namespace {

int save_state(Ctx& c, Sim& S, double* dst)
{
    const size_t nb = S.nb;
    cudaStream_t st = c.stream;
    RIGC_CUDA(cudaMemcpyAsync(dst, S.x0.ptr, 48 * nb, cudaMemcpyDeviceToDevice, st));
    RIGC_CUDA(cudaMemcpyAsync(dst + 6 * nb, S.vel.ptr, 48 * nb, cudaMemcpyDeviceToDevice, st));
    RIGC_CUDA(cudaMemcpyAsync(dst + 12 * nb, S.Qdot.ptr, 72 * nb, cudaMemcpyDeviceToDevice, st));
    return RIGC_OK;
}

int load_state(Ctx& c, Sim& S, const double* src)
{
    const size_t nb = S.nb;
    cudaStream_t st = c.stream;
    RIGC_CUDA(cudaMemcpyAsync(S.x0.ptr, src, 48 * nb, cudaMemcpyDeviceToDevice, st));
    RIGC_CUDA(cudaMemcpyAsync(S.vel.ptr, src + 6 * nb, 48 * nb, cudaMemcpyDeviceToDevice, st));
    RIGC_CUDA(cudaMemcpyAsync(S.Qdot.ptr, src + 12 * nb, 72 * nb, cudaMemcpyDeviceToDevice, st));
    return RIGC_OK;
}

// S.adj holds dL/d(state after the step); on return it holds dL/d(state
// before).  pre: the state before the step (21 nb doubles), xs: its
// solution, kappa / dk: the step's final stiffness and d kappa / d kappa0.
int adjoint_step(Ctx& c, Sim& S, const double* pre, const double* xs, double kappa, double dk)
{
    const rigc_sim_params& p = S.p;
    const int nb = S.nb;
    const int64_t n = 6 * (int64_t)nb;
    const double M = p.average_mass, h = p.timestep;
    cudaStream_t st = c.stream;
    const unsigned gb = grid_for(nb, 128), gn = grid_for(n, 256);
    double* out = S.adj_out.as<double>();
    double* xbar = S.xbar.as<double>();
    double* lam = S.sol.as<double>();
    RIGC_TRY(load_state(c, S, pre));
    const double* x0 = S.x0.as<double>();
    RIGC_COUNT_LAUNCH();
    k_adj_direct<<<gb, 128, 0, st>>>(nb, c.s.type, S.fixed.as<int>(), xs, x0, S.adj.as<double>(), h,
                                     xbar, out);
    // unprojected Hessian of E/m + kappa/m B at x*, then H_FF lambda = xbar_F
    S.kappa = kappa;
    Objective O;
    RIGC_TRY(objective(c, S, xs, true, O, false));
    RIGC_COUNT_LAUNCH();
    k_axpy<<<gn, 256, 0, st>>>(n, -2.0, xbar, xbar, S.g.as<double>());  // g = -xbar
    HessView H = hess_view(S, O, 0.0);
    bool solved;
    int64_t cgit = 0;
    if (S.nfree <= kDenseMax) RIGC_TRY(dense_solve(c, S, H, solved));
    else RIGC_TRY(pcg(c, S, H, solved, cgit));
    if (!solved) return RIGC_ERR_SOLVE;
    RIGC_COUNT_LAUNCH();
    k_hess_rows<<<gn, 256, 0, st>>>(H, lam, S.u1.as<double>());
    RIGC_COUNT_LAUNCH();
    k_adj_fixed<<<gn, 256, 0, st>>>(nb, S.fixed.as<int>(), xbar, S.u1.as<double>(), out);
    RIGC_COUNT_LAUNCH();
    k_adj_exs<<<gb, 128, 0, st>>>(nb, c.s.type, S.fixed.as<int>(), S.mass.as<double>(),
                                  S.moment.as<double>(), xs, x0, lam, -1.0 / M, h, out);
    // the initial stiffness kappa0 = -gE.gB / gB.gB at x0
    if (dk != 0) {
        const double kbar = -dk / M * host_dot(c, S, lam, O.bo.grad);
        if (kbar != 0) {
            rigc_body_state bs = state_of(S);
            double E;
            RIGC_TRY(body_energy(c, bs, x0, p.gravity, h, &E, S.gE.as<double>(), S.hE.as<double>()));
            RIGC_TRY(build_constraints(c, x0, p.dhat, p.dmin));
            rigc_barrier_out bo;
            RIGC_TRY(barrier_term_impl(c, x0, p.dhat, p.dmin, RIGC_GRAD | RIGC_HESS, &bo));
            double* gB = S.gtmp.as<double>();
            RIGC_CUDA(cudaMemcpyAsync(gB, bo.grad, n * 8, cudaMemcpyDeviceToDevice, st));
            const double gg = host_dot(c, S, gB, gB);
            const double ge = host_dot(c, S, gB, S.gE.as<double>());
            const double k0 = -ge / gg;
            const double sc = -kbar / gg;
            double* w = S.r.as<double>();
            RIGC_COUNT_LAUNCH();
            k_axpy<<<gn, 256, 0, st>>>(n, 2 * k0, gB, S.gE.as<double>(), w);
            HessView HB {};
            HB.body = S.hE.as<double>();
            HB.brp = bo.nnzb > 0 ? bo.row_ptr : nullptr;
            HB.bcol = bo.col;
            HB.bval = bo.val;
            HB.sB = 1.0;
            HB.fixed = S.fixed.as<int>();
            HB.nb = nb;
            HessView HE = HB;
            HE.brp = nullptr;
            HE.sE = 1.0;
            RIGC_COUNT_LAUNCH();
            k_hess_rows<<<gn, 256, 0, st>>>(HB, w, S.u1.as<double>());
            RIGC_COUNT_LAUNCH();
            k_hess_rows<<<gn, 256, 0, st>>>(HE, gB, S.u2.as<double>());
            RIGC_COUNT_LAUNCH();
            k_adj_pose_add<<<gn, 256, 0, st>>>(n, sc, S.u1.as<double>(), S.u2.as<double>(), out);
            RIGC_COUNT_LAUNCH();
            k_adj_exs<<<gb, 128, 0, st>>>(nb, c.s.type, S.fixed.as<int>(), S.mass.as<double>(),
                                          S.moment.as<double>(), x0, x0, gB, sc, h, out);
        }
    }
    RIGC_CUDA(cudaGetLastError());
    std::swap(S.adj, S.adj_out);
    return RIGC_OK;
}

} // namespace

int sim_rollout(Ctx& c, int steps, int every, rigc_step_stats* stats)
{
    if (!c.sim || steps < 0 || every < 1) return RIGC_ERR_ARG;
    Sim& S = *c.sim;
    const size_t w = 21 * (size_t)S.nb;
    const int nck = (steps + every - 1) / every;
    RIGC_TRY(S.ckpt.reserve((size_t)std::max(nck, 1) * w * sizeof(double)));
    RIGC_TRY(S.final_state.reserve(w * sizeof(double)));
    S.tape_steps = 0;
    for (int k = 0; k < steps; k++) {
        if (k % every == 0) RIGC_TRY(save_state(c, S, S.ckpt.as<double>() + (size_t)(k / every) * w));
        RIGC_TRY(sim_step(c, stats));
    }
    RIGC_TRY(save_state(c, S, S.final_state.as<double>()));
    RIGC_CUDA(cudaStreamSynchronize(c.stream));
    S.tape_steps = steps;
    S.tape_every = every;
    return RIGC_OK;
}

int sim_backward(Ctx& c, const double* dp, const double* dv, const double* dq, double* gp,
                 double* gv, double* gq)
{
    if (!c.sim || !dp || !gp || !gv || !gq) return RIGC_ERR_ARG;
    Sim& S = *c.sim;
    if (S.tape_every < 1 || S.p.coefficient_friction > 0 || S.has_kinematic) return RIGC_ERR_ARG;
    const int nb = S.nb, K = S.tape_every, steps = S.tape_steps;
    const size_t w = 21 * (size_t)nb;
    cudaStream_t st = c.stream;
    const size_t vb = w * sizeof(double) + 64;
    DevBuf* vecs[] = { &S.adj, &S.adj_out, &S.xbar, &S.u1, &S.u2 };
    for (DevBuf* b : vecs) RIGC_TRY(b->reserve(vb));
    RIGC_TRY(S.seg_pre.reserve((size_t)K * w * sizeof(double)));
    RIGC_TRY(S.seg_x.reserve((size_t)K * 6 * nb * sizeof(double)));
    S.seg_kappa.assign(K, 0.0);
    S.seg_dk.assign(K, 0.0);
    double* a = S.adj.as<double>();
    RIGC_CUDA(cudaMemcpyAsync(a, dp, 48 * (size_t)nb, cudaMemcpyHostToDevice, st));
    if (dv) RIGC_CUDA(cudaMemcpyAsync(a + 6 * nb, dv, 48 * (size_t)nb, cudaMemcpyHostToDevice, st));
    else RIGC_CUDA(cudaMemsetAsync(a + 6 * nb, 0, 48 * (size_t)nb, st));
    if (dq) RIGC_CUDA(cudaMemcpyAsync(a + 12 * nb, dq, 72 * (size_t)nb, cudaMemcpyHostToDevice, st));
    else RIGC_CUDA(cudaMemsetAsync(a + 12 * nb, 0, 72 * (size_t)nb, st));
    const double kappa_after = S.kappa;
    int status = RIGC_OK;
    for (int seg = (steps + K - 1) / K - 1; seg >= 0 && status == RIGC_OK; seg--) {
        const int s0 = seg * K, s1 = std::min(steps, s0 + K);
        // recompute the segment from its checkpoint
        RIGC_TRY(load_state(c, S, S.ckpt.as<double>() + (size_t)seg * w));
        for (int j = s0; j < s1; j++) {
            RIGC_TRY(save_state(c, S, S.seg_pre.as<double>() + (size_t)(j - s0) * w));
            RIGC_TRY(sim_step(c, nullptr));
            RIGC_CUDA(cudaMemcpyAsync(S.seg_x.as<double>() + (size_t)(j - s0) * 6 * nb, S.x0.ptr,
                                      48 * (size_t)nb, cudaMemcpyDeviceToDevice, st));
            S.seg_kappa[j - s0] = S.kappa;
            S.seg_dk[j - s0] = S.dk;
        }
        for (int j = s1 - 1; j >= s0; j--) {
            status = adjoint_step(c, S, S.seg_pre.as<double>() + (size_t)(j - s0) * w,
                                  S.seg_x.as<double>() + (size_t)(j - s0) * 6 * nb,
                                  S.seg_kappa[j - s0], S.seg_dk[j - s0]);
            if (status != RIGC_OK) break;
        }
    }
    if (status == RIGC_OK) {
        a = S.adj.as<double>();
        RIGC_CUDA(cudaMemcpyAsync(gp, a, 48 * (size_t)nb, cudaMemcpyDeviceToHost, st));
        RIGC_CUDA(cudaMemcpyAsync(gv, a + 6 * nb, 48 * (size_t)nb, cudaMemcpyDeviceToHost, st));
        RIGC_CUDA(cudaMemcpyAsync(gq, a + 12 * nb, 72 * (size_t)nb, cudaMemcpyDeviceToHost, st));
    }
    // leave the simulation where the rollout ended
    RIGC_TRY(load_state(c, S, S.final_state.as<double>()));
    RIGC_CUDA(cudaStreamSynchronize(st));
    S.kappa = kappa_after;
    return status;
}

void sim_release(Ctx& c)
{
    if (!c.sim) return;
    Sim& S = *c.sim;
    DevBuf* bufs[] = { &S.mass, &S.moment, &S.fixed, &S.x0, &S.vel, &S.Qdot, &S.x, &S.xt,
                       &S.dir, &S.g, &S.gE, &S.hE, &S.gtmp, &S.r, &S.z, &S.pp, &S.Ap,
                       &S.Minv, &S.sol, &S.part, &S.scal, &S.V0, &S.V1, &S.free_idx,
                       &S.dense, &S.dense_b, &S.dense_x, &S.dense_d, &S.ckpt,
                       &S.final_state, &S.seg_pre, &S.seg_x, &S.adj, &S.adj_out, &S.xbar,
                       &S.u1, &S.u2, &S.sc_dev, &S.sc_red, &S.sc_vstart, &S.al_xpred,
                       &S.al_lam, &S.al_Lam, &S.al_e, &S.hview };
    for (DevBuf* b : bufs) b->release();
    S.cg_one.release();
    S.cg_sc.release();
    if (S.cap) cudaStreamDestroy(S.cap);
    delete c.sim;
    c.sim = nullptr;
}

} // namespace rigc

// DistanceBarrierRBProblem::compute_min_distance(x)
// (src/problems/distance_barrier_rb_problem.cpp:1583-1589) over
// DistanceBarrierConstraint::compute_minimum_distance
// (src/opt/distance_barrier_constraint.cpp:308-323): the constraint set at x,
// the smallest squared distance over it, its square root, -1 when the set is
// empty (an infinite minimum).
extern "C" int rigc_min_distance(rigc_ctx* ctx, const double* x, double dhat, double dmin,
                                 double* min_distance)
{
    using namespace rigc;
    if (!ctx || !x || !min_distance || !(dhat > 0) || !(dmin >= 0)) return RIGC_ERR_ARG;
    Ctx& c = *ctx_of(ctx);
    RIGC_TRY(build_constraints(c, x, dhat, dmin));
    const int64_t n = c.cons.num;
    if (n == 0) {
        *min_distance = -1;
        return RIGC_OK;
    }
    RIGC_TRY(c.md_V.reserve((size_t)3 * c.s.nv * sizeof(double) + 8));
    RIGC_TRY(c.md_out.reserve(sizeof(unsigned long long)));
    RIGC_TRY(compute_world_vertices_rn(c, x, c.md_V.as<double>(), c.md_rot));
    unsigned long long* out = c.md_out.as<unsigned long long>();
    const unsigned long long inf = 0x7ff0000000000000ull;
    RIGC_CUDA(cudaMemcpyAsync(out, &inf, sizeof(inf), cudaMemcpyHostToDevice, c.stream));
    RIGC_COUNT_LAUNCH();
    k_min_constraint_distance<<<grid_for(n, 256), 256, 0, c.stream>>>(
        n, c.cons.type.as<int>(), c.cons.verts.as<int>(), c.md_V.as<double>(), out);
    RIGC_CUDA(cudaGetLastError());
    double d2;
    RIGC_CUDA(cudaMemcpyAsync(&d2, out, sizeof(d2), cudaMemcpyDeviceToHost, c.stream));
    RIGC_CUDA(cudaStreamSynchronize(c.stream));
    *min_distance = std::isfinite(d2) ? std::sqrt(d2) : -1;
    return RIGC_OK;
}
