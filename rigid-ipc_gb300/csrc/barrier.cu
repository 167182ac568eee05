// Barrier energy, body-space gradient and 12x12 pair Hessian per constraint,
// with the rigid-pose chain rule folded in, and their deterministic assembly
// into a per-body gradient and a 6x6 block-sparse Hessian.
//
// Replaces DistanceBarrierRBProblem::compute_barrier_term
// (src/problems/distance_barrier_rb_problem.cpp:1299-1399): the ipc-toolkit
// constraint potentials (log barrier of the squared distance shifted by
// dmin^2, src/opt/distance_barrier_constraint.tpp:11-17; EE mollifier),
// apply_chain_rule (:1182-1248, including project_to_psd of the 12x12),
// local_hessian_to_global_triplets (:1157-1179) and merge_derivative_storage
// (:1260-1297).
//
// Derivation used by k_barrier_local.  With X the constraint's vertex
// positions and x the two bodies' 6-dof poses, X_i = R_b v_i + p_b and
// J_i = dX_i/dx_b = [I | D_i], D_i[:, k] = (dR/dtheta_k) v_i.
//  * PT / EE: d = u^2 / D with u = (A x B).w and D = |A x B|^2, where
//    A, B, w are signed sums of the vertices (coefficients alpha, beta,
//    gamma).  grad u = {alpha_i (B x w) + beta_i (w x A) + gamma_i n},
//    grad D = {2 alpha_i (B x n) + 2 beta_i (n x A)}; the Hessians are
//    Gram(dn) terms and skew bilinear blocks [s_ij]x between vertices i != j.
//  * PE: d = |a x b|^2 / |e|^2, the same pieces with a Gram(de) term.
//  * PP: d = |w|^2.
// f = weight * m(D) * b(d - dmin^2) (m = 1 except mollified EE), so the body
// Hessian is  sum of outer products of the body-space gradients of the basic
// scalars + Gram terms + skew pair blocks + the curvature term
// sum_i grad_Xi f . d2X_i/dtheta2.  It is then projected to the PSD cone by
// a warp-parallel Jacobi eigensolver (a matrix with no negative eigenvalue is
// returned unchanged, as project_to_psd does), V max(L, 0) V^T otherwise.
#include <algorithm>

#include "common.cuh"
#include "geometry_rn.cuh"
#include "local_terms.cuh"
#include "rotation.cuh"
#include "sort.cuh"

namespace rigc {

// ---------------------------------------------------------------------------
// per-body frames (R, dR, d2R) and positions

__global__ void k_body_frames(const double* __restrict__ x, int nb, double* __restrict__ frames)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    double t[3] = { x[6 * b + 3], x[6 * b + 4], x[6 * b + 5] };
    double F[kFrameDoubles];
    body_frame(t, F);
    double* out = frames + (size_t)b * 96;
#pragma unroll
    for (int i = 0; i < kFrameDoubles; i++) out[i] = F[i];
    out[90] = x[6 * b];
    out[91] = x[6 * b + 1];
    out[92] = x[6 * b + 2];
}

// ---------------------------------------------------------------------------

struct BarrierArgs {
    const double* rest;
    const double* frames;
    const int* ctype;
    const int* cverts;
    const int* cbodies;
    const double* cweight;
    const double* ceps;
    int64_t n;
    double dhat, dmin;
    int flags;
    double* energy;   // n
    double* grad;     // n x 12
    double* blocks;   // n x 4 x 36 (blocks (0,0) (0,1) (1,0) (1,1))
    double* hess;     // optional n x 144 (full local Hessian)
    // index limits checked on the device when check_nv >= 0 (callers whose
    // constraint arrays were not validated on the host): a constraint with a
    // type, vertex or body index out of range reads nothing and gets NaN
    // outputs
    int check_nb = 0;
    int64_t check_nv = -1;
};

// the index check of a constraint (see BarrierArgs::check_nv)
static __device__ bool constraint_in_range(const BarrierArgs& a, int64_t ci)
{
    const int type = a.ctype[ci];
    if (type < 0 || type > 3) return false;
    const int nvc = type == 0 ? 2 : (type == 1 ? 3 : 4);
    for (int i = 0; i < 2; i++) {
        const int b = a.cbodies[2 * ci + i];
        if (b < 0 || b >= a.check_nb) return false;
    }
    for (int i = 0; i < nvc; i++) {
        const int v = a.cverts[4 * ci + i];
        if (v < 0 || (int64_t)v >= a.check_nv) return false;
    }
    return true;
}

__device__ __forceinline__ int local_body_of(int type, int i)
{
    if (type == 2) return i < 2 ? 0 : 1;
    return i == 0 ? 0 : 1;
}

// H += J_i^T Hb J_j (+ its transpose when i and j are different vertices),
// J_i = [I | D_i], on the upper triangle
__device__ __forceinline__ void add_vertex_block(SMat H, const Vtx& Vi, int oi, const Vtx& Vj, int oj,
                                                 const double (*Hb)[3], bool same_vertex)
{
    double HD[3][3], DH[3][3], DHD[3][3];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            HD[r][c] = Hb[r][0] * Vj.D[0][c] + Hb[r][1] * Vj.D[1][c] + Hb[r][2] * Vj.D[2][c];
            DH[r][c] = Vi.D[0][r] * Hb[0][c] + Vi.D[1][r] * Hb[1][c] + Vi.D[2][r] * Hb[2][c];
        }
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
            DHD[r][c] = Vi.D[0][r] * HD[0][c] + Vi.D[1][r] * HD[1][c] + Vi.D[2][r] * HD[2][c];
    for (int r = 0; r < 6; r++)
        for (int c = 0; c < 6; c++) {
            double v = r < 3 ? (c < 3 ? Hb[r][c] : HD[r][c - 3])
                             : (c < 3 ? DH[r - 3][c] : DHD[r - 3][c - 3]);
            int R = oi + r, C = oj + c;
            if (same_vertex) {
                if (R <= C) H.at(R, C) += v;
            } else {
                if (R <= C) H.at(R, C) += v;
                if (C <= R) H.at(C, R) += v;
            }
        }
}

// A mollified EE constraint whose closest features are endpoints (kept as EE
// by the constraint set because the edges are nearly parallel): f = w m(D)
// b(d - dmin^2) with D = |A x B|^2 of the two edges and d the point-point or
// point-edge squared distance of the closest features.  Vertex-space
// gradients and 3x3 Hessian blocks in closed form:
//   grad D_i = 2 M_i^T n, M_i = alpha_i (-[B]x) + beta_i [A]x,
//   hess D_ij = 2 M_i^T M_j + 2 (beta_i alpha_j - alpha_i beta_j) [n]x,
// and the same for N = |a x b|^2 of a point-edge distance d = N / |e|^2;
// then J^T (.) J and the curvature term into body space.
static __device__ __noinline__ bool ee_endpoint_build(const BarrierArgs& a, int64_t ci, SMat H,
                                                      const Vtx* V, const double (*vrest)[3],
                                                      const int* lbody, const double* const* fr,
                                                      int dtype)
{
    const double weight = a.cweight[ci];
    int kind = 1, p = 0, q = 0, e0 = 0, e1 = 0;
    switch (dtype) {
    case EE_EA0_EB0: kind = 0; p = 0; q = 2; break;
    case EE_EA0_EB1: kind = 0; p = 0; q = 3; break;
    case EE_EA1_EB0: kind = 0; p = 1; q = 2; break;
    case EE_EA1_EB1: kind = 0; p = 1; q = 3; break;
    case EE_EA_EB0: p = 2; e0 = 0; e1 = 1; break;
    case EE_EA_EB1: p = 3; e0 = 0; e1 = 1; break;
    case EE_EA0_EB: p = 0; e0 = 2; e1 = 3; break;
    default: p = 1; e0 = 2; e1 = 3; break;
    }
    const double alD[4] = { -1, 1, 0, 0 }, beD[4] = { 0, 0, -1, 1 };
    double A[3], B[3], n[3];
    for (int j = 0; j < 3; j++) {
        A[j] = V[1].X[j] - V[0].X[j];
        B[j] = V[3].X[j] - V[2].X[j];
    }
    cross(A, B, n);
    const double Dm = dot(n, n);
    double gD[4][3], gd[4][3];
    {
        double Bn[3], nA[3];
        cross(B, n, Bn);
        cross(n, A, nA);
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 3; j++) {
                gD[i][j] = 2 * (alD[i] * Bn[j] + beD[i] * nA[j]);
                gd[i][j] = 0;
            }
    }
    double d, N = 0, De = 1;
    double pa[3], pb[3], c[3], e[3];
    double alE[4] = { 0, 0, 0, 0 }, beE[4] = { 0, 0, 0, 0 }, gaE[4] = { 0, 0, 0, 0 };
    double gN[4][3], gE[4][3];
    if (kind == 0) {
        double w[3];
        for (int j = 0; j < 3; j++) w[j] = V[p].X[j] - V[q].X[j];
        d = dot(w, w);
        for (int j = 0; j < 3; j++) {
            gd[p][j] = 2 * w[j];
            gd[q][j] = -2 * w[j];
        }
    } else {
        alE[p] = -1; alE[e0] = 1; beE[p] = -1; beE[e1] = 1; gaE[e0] = -1; gaE[e1] = 1;
        for (int j = 0; j < 3; j++) {
            pa[j] = V[e0].X[j] - V[p].X[j];
            pb[j] = V[e1].X[j] - V[p].X[j];
            e[j] = V[e1].X[j] - V[e0].X[j];
        }
        cross(pa, pb, c);
        N = dot(c, c);
        De = dot(e, e);
        d = N / De;
        double bc[3], ca[3];
        cross(pb, c, bc);
        cross(c, pa, ca);
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 3; j++) {
                gN[i][j] = 2 * (alE[i] * bc[j] + beE[i] * ca[j]);
                gE[i][j] = 2 * gaE[i] * e[j];
                gd[i][j] = gN[i][j] / De - N / (De * De) * gE[i][j];
            }
    }
    // barrier of the shifted squared distance and the mollifier
    const double s = 2 * a.dmin * a.dhat + a.dhat * a.dhat;
    const double dd = d - a.dmin * a.dmin;
    double bv = 0, b1 = 0, b2 = 0;
    bool active = dd < s;
    if (dd <= 0.0) {
        bv = INFINITY;
        active = false;
    } else if (active) {
        double lg = log(dd / s);
        double dm = dd - s;
        bv = -dm * dm * lg;
        b1 = (s - dd) * (2 * lg - s / dd + 1);
        double sd = s / dd;
        b2 = (sd + 2) * sd - 2 * lg - 3;
    }
    double m = 1, m1 = 0, m2 = 0;
    if (Dm < a.ceps[ci]) {
        double ie = 1.0 / a.ceps[ci];
        double xe = Dm * ie;
        m = (2 - xe) * xe;
        m1 = (2 - 2 * xe) * ie;
        m2 = -2 * ie * ie;
    }
    if (a.energy) a.energy[ci] = weight * m * bv;
    const bool want_g = (a.flags & (RIGC_GRAD | RIGC_HESS)) != 0;
    const bool want_h = (a.flags & RIGC_HESS) != 0;
    if (!active) {
        if (a.grad)
            for (int k = 0; k < 12; k++) a.grad[ci * 12 + k] = 0;
        if (a.blocks && want_h)
            for (int k = 0; k < 144; k++) a.blocks[ci * 144 + k] = 0;
        if (a.hess && want_h)
            for (int k = 0; k < 144; k++) a.hess[ci * 144 + k] = 0;
        return false;
    }
    if (!want_g) return false;
    double gv[4][3];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 3; j++) gv[i][j] = weight * (m * b1 * gd[i][j] + bv * m1 * gD[i][j]);
    double G[12];
    to_body(V, lbody, 4, gv, G);
    if (a.grad)
        for (int k = 0; k < 12; k++) a.grad[ci * 12 + k] = G[k];
    if (!want_h) return false;

    for (int r = 0; r < 12; r++)
        for (int cc = r; cc < 12; cc++) H.at(r, cc) = 0;
    // M_i = alpha_i (-[B]x) + beta_i [A]x (dn/dX_i), C_i likewise for c = a x b
    auto skew_of = [](double sa, const double* Bv, double sb, const double* Av, double (*M)[3]) {
        double v0 = -sa * Bv[0] + sb * Av[0], v1 = -sa * Bv[1] + sb * Av[1],
               v2 = -sa * Bv[2] + sb * Av[2];
        M[0][0] = 0; M[0][1] = -v2; M[0][2] = v1;
        M[1][0] = v2; M[1][1] = 0; M[1][2] = -v0;
        M[2][0] = -v1; M[2][1] = v0; M[2][2] = 0;
    };
    for (int i = 0; i < 4; i++)
        for (int j = i; j < 4; j++) {
            double Mi[3][3], Mj[3][3], Hb[3][3];
            skew_of(alD[i], B, beD[i], A, Mi);
            skew_of(alD[j], B, beD[j], A, Mj);
            const double kD = 2 * (beD[i] * alD[j] - alD[i] * beD[j]);
            const double nx[3][3] = { { 0, -n[2], n[1] }, { n[2], 0, -n[0] }, { -n[1], n[0], 0 } };
            double Ci[3][3], Cj[3][3], kN = 0;
            const double cx[3][3] = { { 0, -c[2], c[1] }, { c[2], 0, -c[0] }, { -c[1], c[0], 0 } };
            if (kind == 1) {
                skew_of(alE[i], pb, beE[i], pa, Ci);
                skew_of(alE[j], pb, beE[j], pa, Cj);
                kN = 2 * (beE[i] * alE[j] - alE[i] * beE[j]);
            }
            for (int r = 0; r < 3; r++)
                for (int q2 = 0; q2 < 3; q2++) {
                    // hess D block
                    double hD = kD * nx[r][q2];
                    for (int k = 0; k < 3; k++) hD += 2 * Mi[k][r] * Mj[k][q2];
                    // hess d block
                    double hd;
                    if (kind == 0) {
                        double si = i == p ? 1.0 : (i == q ? -1.0 : 0.0);
                        double sj = j == p ? 1.0 : (j == q ? -1.0 : 0.0);
                        hd = r == q2 ? 2 * si * sj : 0.0;
                    } else {
                        double hN = kN * cx[r][q2];
                        for (int k = 0; k < 3; k++) hN += 2 * Ci[k][r] * Cj[k][q2];
                        double hE = r == q2 ? 2 * gaE[i] * gaE[j] : 0.0;
                        hd = hN / De - (gN[i][r] * gE[j][q2] + gE[i][r] * gN[j][q2]) / (De * De)
                            + 2 * N / (De * De * De) * gE[i][r] * gE[j][q2] - N / (De * De) * hE;
                    }
                    Hb[r][q2] = weight * (m * b2 * gd[i][r] * gd[j][q2] + m * b1 * hd
                                          + m1 * b1 * (gd[i][r] * gD[j][q2] + gD[i][r] * gd[j][q2])
                                          + bv * m2 * gD[i][r] * gD[j][q2] + bv * m1 * hD);
                }
            add_vertex_block(H, V[i], 6 * lbody[i], V[j], 6 * lbody[j], Hb, i == j);
        }
    for (int i = 0; i < 4; i++) add_curvature(H, fr[lbody[i]], lbody[i], vrest[i], gv[i]);
    return true;
}

// Energy, gradient and (upper triangle of the) unprojected body Hessian of
// constraint ci into H; returns true when H holds a Hessian to project and
// write, false when every output of the constraint is already written.
static __device__ __noinline__ bool barrier_build(const BarrierArgs& a, int64_t ci, SMat H)
{
    if (a.check_nv >= 0 && !constraint_in_range(a, ci)) {
        const double nan = __longlong_as_double(0x7ff8000000000000ll);
        if (a.energy) a.energy[ci] = nan;
        if (a.grad)
            for (int k = 0; k < 12; k++) a.grad[ci * 12 + k] = nan;
        if (a.flags & RIGC_HESS) {
            if (a.blocks)
                for (int k = 0; k < 144; k++) a.blocks[ci * 144 + k] = nan;
            if (a.hess)
                for (int k = 0; k < 144; k++) a.hess[ci * 144 + k] = nan;
        }
        return false;
    }
    const int type = a.ctype[ci];
    const int nvc = type == 0 ? 2 : (type == 1 ? 3 : 4);
    const double weight = a.cweight[ci];
    int lbody[4];
    const double* fr[2];
    int bod[2] = { a.cbodies[2 * ci], a.cbodies[2 * ci + 1] };
    fr[0] = a.frames + (size_t)bod[0] * 96;
    fr[1] = a.frames + (size_t)bod[1] * 96;
    Vtx V[4];
    double vrest[4][3];
    for (int i = 0; i < nvc; i++) {
        lbody[i] = local_body_of(type, i);
        int vi = a.cverts[4 * ci + i];
        const double* f = fr[lbody[i]];
        for (int j = 0; j < 3; j++) vrest[i][j] = a.rest[3 * (size_t)vi + j];
        const double* v = vrest[i];
        for (int j = 0; j < 3; j++) {
            V[i].X[j] = f[3 * j] * v[0] + f[3 * j + 1] * v[1] + f[3 * j + 2] * v[2] + f[90 + j];
            for (int k = 0; k < 3; k++) {
                const double* dR = f + 9 + 9 * k;
                V[i].D[j][k] = dR[3 * j] * v[0] + dR[3 * j + 1] * v[1] + dR[3 * j + 2] * v[2];
            }
        }
    }

    if (type == 2) {
        const int dt = ee_type_rn(V[0].X, V[1].X, V[2].X, V[3].X);
        if (dt != EE_EA_EB) return ee_endpoint_build(a, ci, H, V, vrest, lbody, fr, dt);
    }

    // coefficient patterns: A = sum alpha_i X_i, B = sum beta_i X_i, w = sum gamma_i X_i
    double al[4] = { 0, 0, 0, 0 }, be[4] = { 0, 0, 0, 0 }, ga[4] = { 0, 0, 0, 0 };
    double A[3], B[3], W[3], n[3];
    double d, u = 0, Dn = 0;
    if (type == 2) {        // EE: A = X1 - X0, B = X3 - X2, w = X2 - X0
        al[0] = -1; al[1] = 1; be[2] = -1; be[3] = 1; ga[0] = -1; ga[2] = 1;
    } else if (type == 3) { // FV: A = X2 - X1, B = X3 - X1, w = X0 - X1
        al[1] = -1; al[2] = 1; be[1] = -1; be[3] = 1; ga[0] = 1; ga[1] = -1;
    } else if (type == 1) { // EV: a = X1 - X0, b = X2 - X0 ; e = X2 - X1 (gamma)
        al[0] = -1; al[1] = 1; be[0] = -1; be[2] = 1; ga[1] = -1; ga[2] = 1;
    } else {                // VV: w = X0 - X1
        ga[0] = 1; ga[1] = -1;
    }
    for (int j = 0; j < 3; j++) {
        A[j] = 0; B[j] = 0; W[j] = 0;
        for (int i = 0; i < nvc; i++) {
            A[j] += al[i] * V[i].X[j];
            B[j] += be[i] * V[i].X[j];
            W[j] += ga[i] * V[i].X[j];
        }
    }
    double De = 0;
    if (type >= 2) {
        cross(A, B, n);
        u = dot(n, W);
        Dn = dot(n, n);
        d = u * u / Dn;
    } else if (type == 1) {
        cross(A, B, n);  // c = a x b
        Dn = dot(n, n);  // N = |c|^2
        De = dot(W, W);  // |e|^2
        d = Dn / De;
    } else {
        d = dot(W, W);
        n[0] = n[1] = n[2] = 0;
    }

    // barrier of the shifted squared distance
    const double s = 2 * a.dmin * a.dhat + a.dhat * a.dhat;
    const double dd = d - a.dmin * a.dmin;
    double bv = 0, b1 = 0, b2 = 0;
    bool active = dd < s;
    if (dd <= 0.0) {
        bv = INFINITY;
        active = false;
    } else if (active) {
        double lg = log(dd / s);
        double dm = dd - s;
        bv = -dm * dm * lg;
        b1 = (s - dd) * (2 * lg - s / dd + 1);
        double sd = s / dd;
        b2 = (sd + 2) * sd - 2 * lg - 3;
    }
    // EE mollifier m(D), D = |A x B|^2
    double m = 1, m1 = 0, m2 = 0;
    if (type == 2 && Dn < a.ceps[ci]) {
        double ie = 1.0 / a.ceps[ci];
        double xe = Dn * ie;
        m = (2 - xe) * xe;
        m1 = (2 - 2 * xe) * ie;
        m2 = -2 * ie * ie;
    }
    if (a.energy) a.energy[ci] = weight * m * bv;
    const bool want_g = (a.flags & (RIGC_GRAD | RIGC_HESS)) != 0;
    const bool want_h = (a.flags & RIGC_HESS) != 0;
    if (!active) {
        if (a.grad)
            for (int k = 0; k < 12; k++) a.grad[ci * 12 + k] = 0;
        if (a.blocks && want_h)
            for (int k = 0; k < 144; k++) a.blocks[ci * 144 + k] = 0;
        if (a.hess && want_h)
            for (int k = 0; k < 144; k++) a.hess[ci * 144 + k] = 0;
        return false;
    }
    if (!want_g) return false;

    // ---- basic scalars and their vertex-space gradients
    // g1: gradient of the first scalar (u, N or d), g2: of the second (D, |e|^2)
    double g1v[4][3], g2v[4][3];
    double c1, c2;  // grad d = c1 g1 + c2 g2
    if (type >= 2) {
        double Bw[3], wA[3], Bn[3], nA[3];
        cross(B, W, Bw);
        cross(W, A, wA);
        cross(B, n, Bn);
        cross(n, A, nA);
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 3; j++) {
                g1v[i][j] = al[i] * Bw[j] + be[i] * wA[j] + ga[i] * n[j];
                g2v[i][j] = 2 * (al[i] * Bn[j] + be[i] * nA[j]);
            }
        c1 = 2 * u / Dn;
        c2 = -u * u / (Dn * Dn);
    } else if (type == 1) {
        double bc[3], ca[3];
        cross(B, n, bc);
        cross(n, A, ca);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                g1v[i][j] = 2 * (al[i] * bc[j] + be[i] * ca[j]);
                g2v[i][j] = 2 * ga[i] * W[j];
            }
        c1 = 1 / De;
        c2 = -Dn / (De * De);
    } else {
        for (int j = 0; j < 3; j++) {
            g1v[0][j] = 2 * W[j];
            g1v[1][j] = -2 * W[j];
            g2v[0][j] = g2v[1][j] = 0;
        }
        c1 = 1;
        c2 = 0;
    }
    // f = weight * m * b(d):  grad f = P_g1 g1 + P_g2 g2
    const double wm = weight * m;
    // (the mollifier's gradient lies along grad D = g2, EE only)
    const double Pg1 = wm * b1 * c1;
    const double Pg2 = wm * b1 * c2 + (type == 2 ? weight * bv * m1 : 0.0);
    double gv[4][3];
    for (int i = 0; i < nvc; i++)
        for (int j = 0; j < 3; j++) gv[i][j] = Pg1 * g1v[i][j] + Pg2 * g2v[i][j];
    double G[12];
    to_body(V, lbody, nvc, gv, G);
    if (a.grad)
        for (int k = 0; k < 12; k++) a.grad[ci * 12 + k] = G[k];
    if (!want_h) return false;

    // ---- Hessian
    for (int r = 0; r < 12; r++)
        for (int c = r; c < 12; c++) H.at(r, c) = 0;
    double G1[12], G2[12];
    to_body(V, lbody, nvc, g1v, G1);
    to_body(V, lbody, nvc, g2v, G2);
    // second-derivative coefficients of d in terms of (g1, g2) and the
    // Hessians of the basic scalars:
    //  PT/EE: hess d = (2/D) g1g1 + c1 H_u - (2u/D^2)(g1g2 + g2g1) + (2u^2/D^3) g2g2 + c2 H_D
    //  PE:    hess d = (1/De) H_N - (1/De^2)(g1g2 + g2g1) + (2N/De^3) g2g2 + c2 H_e
    //  PP:    hess d = H_w (Gram of dw)
    double duu, duD, dDD;
    if (type >= 2) {
        duu = 2 / Dn;
        duD = -2 * u / (Dn * Dn);
        dDD = 2 * u * u / (Dn * Dn * Dn);
    } else if (type == 1) {
        duu = 0;
        duD = -1 / (De * De);
        dDD = 2 * Dn / (De * De * De);
    } else {
        duu = duD = dDD = 0;
    }
    // f Hessian = P1 gd gd^T + P2 hess d + [EE] P3 g2g2 + P4 H_D + P5 (g2 gd^T + gd g2^T)
    const double P1 = wm * b2, P2 = wm * b1;
    const double P3 = type == 2 ? weight * bv * m2 : 0.0;
    const double P4 = type == 2 ? weight * bv * m1 : 0.0;
    const double P5 = type == 2 ? weight * m1 * b1 : 0.0;
    const double a11 = P1 * c1 * c1 + P2 * duu;
    const double a12 = P1 * c1 * c2 + P2 * duD + P5 * c1;
    const double a22 = P1 * c2 * c2 + P2 * dDD + P3 + 2 * P5 * c2;
    add_outer(H, a11, G1);
    add_sym_outer(H, a12, G1, G2);
    add_outer(H, a22, G2);

    // coefficients of the scalar Hessians
    const double bu = P2 * c1;            // on H_u (PT/EE) or H_N (PE)
    const double bD = P2 * c2 + P4;       // on H_D (PT/EE) or H_e (PE)
    double M[4][9];
    if (type >= 2) {
        // H_D Gram part: 2 (dn)^T(dn), dn/dX_i = alpha_i(-[B]x) + beta_i [A]x
        for (int i = 0; i < 4; i++) {
            double* Mi = M[i];
            double sa = al[i], sb = be[i];
            // -[B]x * sa + [A]x * sb
            double v0 = -sa * B[0] + sb * A[0], v1 = -sa * B[1] + sb * A[1], v2 = -sa * B[2] + sb * A[2];
            Mi[0] = 0; Mi[1] = -v2; Mi[2] = v1;
            Mi[3] = v2; Mi[4] = 0; Mi[5] = -v0;
            Mi[6] = -v1; Mi[7] = v0; Mi[8] = 0;
        }
        add_gram(H, 2 * bD, V, lbody, 4, M);
        // skew pair blocks: s_ij = bu * s_ij(u) + bD * s_ij(D)
        for (int i = 0; i < 4; i++)
            for (int j = i + 1; j < 4; j++) {
                double sv[3];
                for (int k = 0; k < 3; k++) {
                    double su = -al[i] * be[j] * W[k] + al[j] * be[i] * W[k]
                        + al[i] * ga[j] * B[k] - al[j] * ga[i] * B[k]
                        - be[i] * ga[j] * A[k] + be[j] * ga[i] * A[k];
                    double sD = 2 * (-al[i] * be[j] * n[k] + al[j] * be[i] * n[k]);
                    sv[k] = bu * su + bD * sD;
                }
                if (sv[0] == 0 && sv[1] == 0 && sv[2] == 0) continue;
                add_skew_pair(H, V[i], 6 * lbody[i], V[j], 6 * lbody[j], sv);
            }
    } else if (type == 1) {
        // H_N = 2 (dc)^T(dc) + skew(c); H_e = 2 (de)^T(de)
        for (int i = 0; i < 3; i++) {
            double* Mi = M[i];
            double sa = al[i], sb = be[i];
            double v0 = -sa * B[0] + sb * A[0], v1 = -sa * B[1] + sb * A[1], v2 = -sa * B[2] + sb * A[2];
            Mi[0] = 0; Mi[1] = -v2; Mi[2] = v1;
            Mi[3] = v2; Mi[4] = 0; Mi[5] = -v0;
            Mi[6] = -v1; Mi[7] = v0; Mi[8] = 0;
        }
        add_gram(H, 2 * bu, V, lbody, 3, M);
        for (int i = 0; i < 3; i++) {
            double* Mi = M[i];
            for (int k = 0; k < 9; k++) Mi[k] = 0;
            Mi[0] = Mi[4] = Mi[8] = ga[i];
        }
        add_gram(H, 2 * bD, V, lbody, 3, M);
        for (int i = 0; i < 3; i++)
            for (int j = i + 1; j < 3; j++) {
                double sv[3];
                for (int k = 0; k < 3; k++)
                    sv[k] = bu * 2 * (-al[i] * be[j] * n[k] + al[j] * be[i] * n[k]);
                if (sv[0] == 0 && sv[1] == 0 && sv[2] == 0) continue;
                add_skew_pair(H, V[i], 6 * lbody[i], V[j], 6 * lbody[j], sv);
            }
    } else {
        // d = |w|^2: hess = 2 (dw)^T (dw), coefficient P2 (c1 = 1)
        for (int i = 0; i < 2; i++) {
            double* Mi = M[i];
            for (int k = 0; k < 9; k++) Mi[k] = 0;
            Mi[0] = Mi[4] = Mi[8] = ga[i];
        }
        add_gram(H, 2 * P2, V, lbody, 2, M);
    }
    // curvature of the rigid maps
    for (int i = 0; i < nvc; i++) add_curvature(H, fr[lbody[i]], lbody[i], vrest[i], gv[i]);
    return true;
}


// One warp per block.  Lanes 0 .. per_warp-1 each build one constraint's
// terms (a thread per constraint); then the whole warp projects the built
// Hessians one after another.  per_warp is chosen by the host so that small
// constraint sets still spread over the SMs.
__global__ void __launch_bounds__(kBarrierTPB)
k_barrier_local(BarrierArgs a, int per_warp)
{
    extern __shared__ double smem[];
    const int lane = threadIdx.x;
    const int64_t ci = (int64_t)blockIdx.x * per_warp + lane;
    const bool mine = lane < per_warp && ci < a.n;
    SMat H { smem + lane };
    bool built = mine && barrier_build(a, ci, H);
    if (!(a.flags & RIGC_HESS)) return;  // uniform over the block
    if (a.flags & RIGC_PROJECT_PSD) {
        double* work = smem + kSymEntries * kBarrierTPB;
        unsigned todo = __ballot_sync(0xffffffffu, built);
        while (todo) {
            int t = __ffs(todo) - 1;
            todo &= todo - 1;
            warp_psd_project(SMat { smem + t }, work, lane);
        }
    }
    if (built) write_local_hessian(H, ci, a.hess, a.blocks);
}

size_t local_terms_smem_bytes()
{
    return (size_t)(kSymEntries * kBarrierTPB + kWorkDoubles) * sizeof(double);
}

// constraints per warp: a thread per constraint once there are enough of
// them to fill the GPU, fewer (down to one) for small sets
int local_terms_per_warp(int64_t n)
{
    int64_t w = (n + kNumSMs * 8 - 1) / (kNumSMs * 8);
    return (int)std::max<int64_t>(1, std::min<int64_t>(kBarrierTPB, w));
}

int launch_body_frames(Ctx& c, const double* x)
{
    RIGC_TRY(c.frames.reserve((size_t)c.s.nb * 96 * sizeof(double)));
    RIGC_COUNT_LAUNCH();
    k_body_frames<<<grid_for(c.s.nb, 128), 128, 0, c.stream>>>(x, c.s.nb, c.frames.as<double>());
    RIGC_CUDA(cudaGetLastError());
    return RIGC_OK;
}

int launch_barrier_local(Ctx& c, const double* x, double dhat, double dmin, int flags,
                         double* energy, double* grad, double* blocks, double* hess)
{
    RIGC_TRY(launch_body_frames(c, x));
    if (c.cons.num == 0) return RIGC_OK;
    static bool attr = false;
    if (!attr) {
        RIGC_CUDA(cudaFuncSetAttribute(k_barrier_local, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)local_terms_smem_bytes()));
        attr = true;
    }
    BarrierArgs a;
    a.rest = c.s.rest;
    a.frames = c.frames.as<double>();
    a.ctype = c.cons.type.as<int>();
    a.cverts = c.cons.verts.as<int>();
    a.cbodies = c.cons.bodies.as<int>();
    a.cweight = c.cons.weight.as<double>();
    a.ceps = c.cons.eps.as<double>();
    a.n = c.cons.num;
    a.dhat = dhat;
    a.dmin = dmin;
    a.flags = flags;
    a.energy = energy;
    a.grad = grad;
    a.blocks = blocks;
    a.hess = hess;
    const int pw = c.tune.barrier_per_warp > 0 ? std::min(c.tune.barrier_per_warp, kBarrierTPB)
                                               : local_terms_per_warp(c.cons.num);
    RIGC_COUNT_LAUNCH();
    k_barrier_local<<<grid_for(c.cons.num, pw), kBarrierTPB, local_terms_smem_bytes(), c.stream>>>(a, pw);
    RIGC_CUDA(cudaGetLastError());
    return RIGC_OK;
}

// Frames and per-constraint terms with every buffer supplied by the caller
// (the frames array holds 96 doubles per body); used by the entry point that
// allocates nothing.
int launch_barrier_local_raw(const double* rest, int64_t nv, int nb, const double* x, int64_t n,
                             const int* ctype, const int* cverts, const int* cbodies,
                             const double* cweight, const double* ceps, double dhat, double dmin,
                             int flags, double* frames, double* energy, double* grad,
                             double* hess, cudaStream_t stream)
{
    RIGC_COUNT_LAUNCH();
    k_body_frames<<<grid_for(nb, 128), 128, 0, stream>>>(x, nb, frames);
    RIGC_CUDA(cudaGetLastError());
    if (n == 0) return RIGC_OK;
    RIGC_CUDA(cudaFuncSetAttribute(k_barrier_local, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)local_terms_smem_bytes()));
    BarrierArgs a;
    a.rest = rest;
    a.frames = frames;
    a.ctype = ctype;
    a.cverts = cverts;
    a.cbodies = cbodies;
    a.cweight = cweight;
    a.ceps = ceps;
    a.n = n;
    a.dhat = dhat;
    a.dmin = dmin;
    a.flags = flags;
    a.energy = energy;
    a.grad = grad;
    a.blocks = nullptr;
    a.hess = hess;
    a.check_nb = nb;
    a.check_nv = nv;
    const int pw = local_terms_per_warp(n);
    RIGC_COUNT_LAUNCH();
    k_barrier_local<<<grid_for(n, pw), kBarrierTPB, local_terms_smem_bytes(), stream>>>(a, pw);
    RIGC_CUDA(cudaGetLastError());
    return RIGC_OK;
}

// ---------------------------------------------------------------------------
// deterministic assembly: sort block keys, sum equal keys in constraint order

__global__ void k_block_keys(const int* __restrict__ bodies, int64_t n, int nb,
                             uint64_t* __restrict__ keys, uint32_t* __restrict__ vals)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 4 * n) return;
    int64_t c = i >> 2;
    int blk = (int)(i & 3);
    int bi = bodies[2 * c + (blk >> 1)], bj = bodies[2 * c + (blk & 1)];
    keys[i] = (uint64_t)bi * (uint64_t)nb + (uint64_t)bj;
    vals[i] = (uint32_t)i;
}

__global__ void k_grad_keys(const int* __restrict__ bodies, int64_t n,
                            uint32_t* __restrict__ keys, uint32_t* __restrict__ vals)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 2 * n) return;
    keys[i] = (uint32_t)bodies[i];
    vals[i] = (uint32_t)i;
}

template <class Key>
__global__ void k_heads(const Key* __restrict__ keys, int64_t m, int32_t* __restrict__ head)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    head[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

// segment starts: seg_start[segid] = i for heads
__global__ void k_seg_starts(const int32_t* __restrict__ head, const int32_t* __restrict__ segid,
                             int64_t m, int32_t* __restrict__ seg_start)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    if (head[i]) seg_start[segid[i]] = (int32_t)i;
}

// one thread per (unique block, entry): sequential sum in slot order
__global__ void k_block_sums(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ slots,
                             const int32_t* __restrict__ seg_start,
                             const int32_t* __restrict__ nseg_ptr, int64_t m,
                             const double* __restrict__ blocks, int nb,
                             int32_t* __restrict__ col, double* __restrict__ val,
                             int32_t* __restrict__ row_count)
{
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t nseg = *nseg_ptr;
    if (t >= (int64_t)nseg * 36) return;
    int32_t sgi = (int32_t)(t / 36);
    int e = (int)(t % 36);
    int64_t s0 = seg_start[sgi];
    int64_t s1 = sgi + 1 < nseg ? seg_start[sgi + 1] : m;
    double acc = 0;
    for (int64_t i = s0; i < s1; i++) acc += blocks[(size_t)slots[i] * 36 + e];
    val[(size_t)sgi * 36 + e] = acc;
    if (e == 0) {
        uint64_t k = keys[s0];
        int32_t r = (int32_t)(k / (uint64_t)nb);
        col[sgi] = (int32_t)(k % (uint64_t)nb);
        atomicAdd(&row_count[r], 1);
    }
}

__global__ void k_grad_sums(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ slots,
                            const int32_t* __restrict__ seg_start,
                            const int32_t* __restrict__ nseg_ptr, int64_t m,
                            const double* __restrict__ cgrad, double* __restrict__ grad)
{
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t nseg = *nseg_ptr;
    if (t >= (int64_t)nseg * 6) return;
    int32_t sgi = (int32_t)(t / 6);
    int e = (int)(t % 6);
    int64_t s0 = seg_start[sgi];
    int64_t s1 = sgi + 1 < nseg ? seg_start[sgi + 1] : m;
    double acc = 0;
    for (int64_t i = s0; i < s1; i++) {
        uint32_t slot = slots[i];  // = 2 c + side
        acc += cgrad[(size_t)(slot >> 1) * 12 + 6 * (slot & 1) + e];
    }
    grad[(size_t)keys[s0] * 6 + e] = acc;
}

int assemble_terms(Ctx& c, const int* bodies, int64_t n, const double* cgrad,
                   const double* cblocks, DevBuf& grad, DevBuf& row_ptr, DevBuf& col,
                   DevBuf& val, int32_t* nseg_dev_pair, bool with_hess)
{
    const int nb = c.s.nb;
    cudaStream_t st = c.stream;
    RIGC_TRY(grad.reserve((size_t)6 * nb * sizeof(double)));
    RIGC_TRY(row_ptr.reserve((size_t)(nb + 1) * sizeof(int32_t)));
    RIGC_CUDA(cudaMemsetAsync(grad.ptr, 0, (size_t)6 * nb * sizeof(double), st));
    RIGC_CUDA(cudaMemsetAsync(row_ptr.ptr, 0, (size_t)(nb + 1) * sizeof(int32_t), st));
    if (n == 0) return RIGC_OK;
    // scratch usage: 0 keys_in, 1 vals_in, 2 keys_out, 3 vals_out, 4/5 sort tmp,
    // 6 hist/scan tmp, 7 head/segid/seg_start
    DevBuf* S = c.scratch;
    // ---- gradient
    {
        int64_t m = 2 * n;
        RIGC_TRY(S[0].reserve(m * 4));
        RIGC_TRY(S[1].reserve(m * 4));
        RIGC_TRY(S[2].reserve(m * 4));
        RIGC_TRY(S[3].reserve(m * 4));
        RIGC_TRY(S[7].reserve(m * 12 + 16));
        RIGC_COUNT_LAUNCH();
        k_grad_keys<<<grid_for(m, 256), 256, 0, st>>>(bodies, n, S[0].as<uint32_t>(),
                                                     S[1].as<uint32_t>());
        RIGC_TRY(radix_sort_pairs<uint32_t>(S[0].as<uint32_t>(), S[1].as<uint32_t>(),
                                            S[2].as<uint32_t>(), S[3].as<uint32_t>(), m,
                                            bits_for((uint64_t)nb), S[4], S[5], S[6], st));
        int32_t* head = S[7].as<int32_t>();
        int32_t* segid = head + m;
        int32_t* segst = segid + m;
        RIGC_COUNT_LAUNCH();
        k_heads<uint32_t><<<grid_for(m, 256), 256, 0, st>>>(S[2].as<uint32_t>(), m, head);
        int32_t* nseg_dev = nseg_dev_pair;
        RIGC_TRY(exclusive_scan_i32(head, segid, m, nseg_dev, S[6], st));
        RIGC_COUNT_LAUNCH();
        k_seg_starts<<<grid_for(m, 256), 256, 0, st>>>(head, segid, m, segst);
        // at most m segments; the kernel reads the true count on the device
        RIGC_COUNT_LAUNCH();
        k_grad_sums<<<grid_for(m * 6, 256), 256, 0, st>>>(
            S[2].as<uint32_t>(), S[3].as<uint32_t>(), segst, nseg_dev, m, cgrad,
            grad.as<double>());
    }
    if (!with_hess) return RIGC_OK;
    // ---- Hessian blocks
    {
        int64_t m = 4 * n;
        RIGC_TRY(S[0].reserve(m * 8));
        RIGC_TRY(S[1].reserve(m * 4));
        RIGC_TRY(S[2].reserve(m * 8));
        RIGC_TRY(S[3].reserve(m * 4));
        RIGC_TRY(S[7].reserve(m * 12 + 16));
        RIGC_COUNT_LAUNCH();
        k_block_keys<<<grid_for(m, 256), 256, 0, st>>>(bodies, n, nb,
                                                      S[0].as<uint64_t>(), S[1].as<uint32_t>());
        RIGC_TRY(radix_sort_pairs<uint64_t>(S[0].as<uint64_t>(), S[1].as<uint32_t>(),
                                            S[2].as<uint64_t>(), S[3].as<uint32_t>(), m,
                                            bits_for((uint64_t)nb * nb), S[4], S[5], S[6], st));
        int32_t* head = S[7].as<int32_t>();
        int32_t* segid = head + m;
        int32_t* segst = segid + m;
        RIGC_COUNT_LAUNCH();
        k_heads<uint64_t><<<grid_for(m, 256), 256, 0, st>>>(S[2].as<uint64_t>(), m, head);
        int32_t* nseg_dev = nseg_dev_pair + 1;  // read back by the caller
        RIGC_TRY(exclusive_scan_i32(head, segid, m, nseg_dev, S[6], st));
        RIGC_COUNT_LAUNCH();
        k_seg_starts<<<grid_for(m, 256), 256, 0, st>>>(head, segid, m, segst);
        // capacity for the upper bound m blocks: no host round trip here
        RIGC_TRY(col.reserve((size_t)m * sizeof(int32_t)));
        RIGC_TRY(val.reserve((size_t)m * 36 * sizeof(double)));
        RIGC_COUNT_LAUNCH();
        k_block_sums<<<grid_for(m * 36, 256), 256, 0, st>>>(
            S[2].as<uint64_t>(), S[3].as<uint32_t>(), segst, nseg_dev, m, cblocks, nb,
            col.as<int32_t>(), val.as<double>(), row_ptr.as<int32_t>() + 1);
        // row counts -> row_ptr (exclusive scan of counts shifted by one)
        int32_t* rp = row_ptr.as<int32_t>();
        RIGC_TRY(S[4].reserve((size_t)(nb + 1) * sizeof(int32_t)));
        RIGC_CUDA(cudaMemcpyAsync(S[4].ptr, rp + 1, (size_t)nb * sizeof(int32_t),
                                  cudaMemcpyDeviceToDevice, st));
        RIGC_TRY(exclusive_scan_i32(S[4].as<int32_t>(), rp, nb, rp + nb, S[6], st));
    }
    return RIGC_OK;
}

// Per-scene sums of per-constraint values in constraint order.  Within each
// type segment the constraints are ordered by their first primitive, hence
// by body and by scene; each thread binary-searches its scene's range in the
// four segments.
__global__ void k_scene_sums(const double* __restrict__ val, const int* __restrict__ bodies,
                             const int* __restrict__ bscene, int4 seg_start, int64_t n,
                             int nscenes, double* __restrict__ out)
{
    int sc = blockIdx.x * blockDim.x + threadIdx.x;
    if (sc >= nscenes) return;
    const int64_t starts[5] = { seg_start.x, seg_start.y, seg_start.z, seg_start.w, n };
    double acc = 0;
    for (int t = 0; t < 4; t++) {
        int64_t lo = starts[t], hi = starts[t + 1];
        // first constraint of the segment with scene >= sc
        int64_t a = lo, b = hi;
        while (a < b) {
            int64_t m = (a + b) / 2;
            if (bscene[bodies[2 * m]] < sc) a = m + 1;
            else b = m;
        }
        for (int64_t i = a; i < hi && bscene[bodies[2 * i]] == sc; i++) acc += val[i];
    }
    out[sc] = acc;
}

int scene_sums(Ctx& c, const double* val, const int* bodies, int64_t n, const int64_t seg[4],
               std::vector<double>& out)
{
    const int ns = c.s.nscenes;
    out.assign(ns, 0.0);
    if (n == 0) return RIGC_OK;
    RIGC_TRY(c.scene_energy.reserve((size_t)ns * 8 + 8));
    int4 st4 = make_int4((int)seg[0], (int)seg[1], (int)seg[2], (int)seg[3]);
    RIGC_COUNT_LAUNCH();
    k_scene_sums<<<grid_for(ns, 128), 128, 0, c.stream>>>(val, bodies, c.s.bscene, st4, n, ns,
                                                          c.scene_energy.as<double>());
    RIGC_CUDA(cudaMemcpyAsync(out.data(), c.scene_energy.ptr, (size_t)ns * 8, cudaMemcpyDeviceToHost,
                              c.stream));
    RIGC_CUDA(cudaStreamSynchronize(c.stream));
    return RIGC_OK;
}

int assemble_barrier(Ctx& c, bool with_hess)
{
    // on the device (d_scalars int 1) until the caller syncs
    c.nnzb = (with_hess && c.cons.num > 0) ? -1 : 0;
    return assemble_terms(c, c.cons.bodies.as<int>(), c.cons.num, c.c_grad.as<double>(),
                          c.c_blocks.as<double>(), c.grad, c.row_ptr, c.col, c.val,
                          c.d_scalars.as<int32_t>(), with_hess);
}

} // namespace rigc
