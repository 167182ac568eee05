// Lagged friction: constraint set at the start of the step and the friction
// potential's energy, body-space gradient and PSD-projected 12x12 Hessian per
// constraint, assembled like the barrier term.
//
// Replaces DistanceBarrierRBProblem::update_friction_constraints
// (src/problems/distance_barrier_rb_problem.cpp:168-188, ipc-toolkit
// construct_friction_constraint_set) and compute_friction_term /
// compute_friction_potential (:1411-1572): for each collision constraint at
// the start-of-step vertices V0,
//   lambda = -kappa * w * b'(d) * 2 sqrt(d)       (normal force magnitude,
//            b' the barrier derivative in the squared distance d, w the
//            constraint multiplicity),
//   closest-point weights g_i (point minus closest point on the other
//            primitive: VV (1, -1); EV (1, -(1 - a), -a); EE (1 - a, a,
//            -(1 - b), -b); FV (1, -(1 - b1 - b2), -b1, -b2)), line / plane
//            closest points as in the IPC formulation,
//   T = an orthonormal basis (t1, t2) of the contact's tangent plane;
// and with U = V(x) - V0, u = T^T sum_i g_i U_i and eps = eps_v h,
//   D = mu lambda f0(|u|),  f0(x) = x (x >= eps),
//                           -x^3 / (3 eps^2) + x^2 / eps + eps / 3 otherwise,
//   grad_Xi D = mu lambda f1(|u|)/|u| g_i T u,
//   hess_X D  = mu lambda A^T H_u A,  A = T^T Gamma (2 x 3n),
//   H_u = I/|u| - u u^T/|u|^3 (|u| >= eps), (2/eps - |u|/eps^2) I -
//         u u^T / (eps^2 |u|) (0 < |u| < eps), 2/eps I (u = 0);
// the rigid chain rule (apply_chain_rule, :1182-1248) maps A's rows and the
// vertex gradient to body space and adds the rotation curvature; the 12x12 is
// projected to the PSD cone.
#include <cstring>

#include "common.cuh"
#include "geometry_rn.cuh"
#include "local_terms.cuh"
#include "sort.cuh"

namespace rigc {

int compute_world_vertices_rn(Ctx& c, const double* x, double* V, DevBuf& rotbuf);

constexpr int kFricCoef = 9;  // lambda, closest (2), t1 (3), t2 (3)

__device__ __forceinline__ void normalize3_rn(double* v)
{
    double n = __dsqrt_rn(dot3_rn(v, v));
    v[0] = RDIV(v[0], n);
    v[1] = RDIV(v[1], n);
    v[2] = RDIV(v[2], n);
}

// derivative of the log barrier in the squared distance
__device__ __forceinline__ double barrier_d1(double d, double s)
{
    if (d <= 0.0 || d >= s) return 0.0;
    return (s - d) * (2 * log(d / s) - s / d + 1);
}

struct FrictionSetupArgs {
    const int* ctype;
    const int* cverts;
    const double* cweight;
    const double* V0;  // nv x 3 world vertices at the start of the step
    int64_t n;
    double dhat, dmin, kappa;
    double* coef;      // n x kFricCoef
    double* v0c;       // n x 12: the constraint's start-of-step vertices
};

// Start-of-step set-up, one thread per constraint, in the explicit
// round-to-nearest operation order of geometry_rn.cuh (the distance the
// constraint set classified with, closest points by 2x2 normal equations,
// bases by cross products).
__global__ void k_friction_setup(FrictionSetupArgs a)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int type = a.ctype[i];
    const int nvc = type == 0 ? 2 : (type == 1 ? 3 : 4);
    double P[4][3];
    for (int k = 0; k < 4; k++)
        for (int j = 0; j < 3; j++) {
            P[k][j] = k < nvc ? a.V0[3 * (size_t)a.cverts[4 * i + k] + j] : 0.0;
            a.v0c[i * 12 + 3 * k + j] = P[k][j];
        }
    double d = 0, p0 = 0, p1 = 0, t1[3], t2[3], n[3];
    if (type == 0) {
        // any orthonormal basis of the plane orthogonal to p0 - p1
        sub3_rn(P[0], P[1], n);
        d = dot3_rn(n, n);
        normalize3_rn(n);
        double ax[3] = { 1, 0, 0 };
        if (fabs(n[0]) > 0.9) {
            ax[0] = 0;
            ax[1] = 1;
        }
        cross3_rn(n, ax, t1);
        normalize3_rn(t1);
        cross3_rn(n, t1, t2);
    } else if (type == 1) {
        double e[3], w[3], c[3];
        sub3_rn(P[2], P[1], e);
        sub3_rn(P[0], P[1], w);
        p0 = RDIV(dot3_rn(e, w), dot3_rn(e, e));
        d = pl_sqdist_rn(P[0], P[1], P[2]);
        for (int j = 0; j < 3; j++) n[j] = RSUB(w[j], RMUL(p0, e[j]));
        for (int j = 0; j < 3; j++) t1[j] = e[j];
        normalize3_rn(t1);
        cross3_rn(e, n, c);
        for (int j = 0; j < 3; j++) t2[j] = c[j];
        normalize3_rn(t2);
    } else if (type == 2) {
        double ea[3], eb[3], w[3];
        sub3_rn(P[1], P[0], ea);
        sub3_rn(P[3], P[2], eb);
        sub3_rn(P[2], P[0], w);
        double aa = dot3_rn(ea, ea), ab = dot3_rn(ea, eb), bb = dot3_rn(eb, eb);
        double aw = dot3_rn(ea, w), bw = dot3_rn(eb, w);
        double det = RSUB(RMUL(aa, bb), RMUL(ab, ab));
        p0 = RDIV(RSUB(RMUL(aw, bb), RMUL(ab, bw)), det);
        p1 = RDIV(RSUB(RMUL(aw, ab), RMUL(aa, bw)), det);
        d = ee_sqdist_rn(P[0], P[1], P[2], P[3]);
        cross3_rn(ea, eb, n);
        for (int j = 0; j < 3; j++) t1[j] = ea[j];
        normalize3_rn(t1);
        normalize3_rn(n);
        cross3_rn(n, t1, t2);
    } else {
        double e1[3], e2[3], w[3];
        sub3_rn(P[2], P[1], e1);
        sub3_rn(P[3], P[1], e2);
        sub3_rn(P[0], P[1], w);
        double a11 = dot3_rn(e1, e1), a12 = dot3_rn(e1, e2), a22 = dot3_rn(e2, e2);
        double r1 = dot3_rn(e1, w), r2 = dot3_rn(e2, w);
        double det = RSUB(RMUL(a11, a22), RMUL(a12, a12));
        p0 = RDIV(RSUB(RMUL(a22, r1), RMUL(a12, r2)), det);
        p1 = RDIV(RSUB(RMUL(a11, r2), RMUL(a12, r1)), det);
        d = ptplane_sqdist_rn(P[0], P[1], P[2], P[3]);
        cross3_rn(e1, e2, n);
        for (int j = 0; j < 3; j++) t1[j] = e1[j];
        normalize3_rn(t1);
        normalize3_rn(n);
        cross3_rn(n, t1, t2);
    }
    const double s = 2 * a.dmin * a.dhat + a.dhat * a.dhat;
    double* o = a.coef + i * kFricCoef;
    o[0] = -a.kappa * a.cweight[i] * barrier_d1(d - a.dmin * a.dmin, s) * 2 * sqrt(d);
    o[1] = p0;
    o[2] = p1;
    for (int j = 0; j < 3; j++) {
        o[3 + j] = t1[j];
        o[6 + j] = t2[j];
    }
}

struct FrictionArgs {
    const double* rest;
    const double* frames;
    const int* ctype;
    const int* cverts;
    const int* cbodies;
    const double* coef;
    const double* v0c;
    int64_t n;
    double mu, epsvh;
    int flags;
    double* energy;
    double* grad;
    double* blocks;
    double* hess;
};

__device__ __forceinline__ int fric_local_body(int type, int i)
{
    if (type == 2) return i < 2 ? 0 : 1;
    return i == 0 ? 0 : 1;
}

static __device__ __noinline__ bool friction_build(const FrictionArgs& a, int64_t ci, SMat H)
{
    const int type = a.ctype[ci];
    const int nvc = type == 0 ? 2 : (type == 1 ? 3 : 4);
    const double* cf = a.coef + ci * kFricCoef;
    const double lambda = cf[0], p0 = cf[1], p1 = cf[2];
    const double t1[3] = { cf[3], cf[4], cf[5] }, t2[3] = { cf[6], cf[7], cf[8] };
    double g[4];
    if (type == 0) {
        g[0] = 1; g[1] = -1; g[2] = g[3] = 0;
    } else if (type == 1) {
        g[0] = 1; g[1] = -(1 - p0); g[2] = -p0; g[3] = 0;
    } else if (type == 2) {
        g[0] = 1 - p0; g[1] = p0; g[2] = -(1 - p1); g[3] = -p1;
    } else {
        g[0] = 1; g[1] = -(1 - p0 - p1); g[2] = -p0; g[3] = -p1;
    }
    const int bod[2] = { a.cbodies[2 * ci], a.cbodies[2 * ci + 1] };
    const double* fr[2] = { a.frames + (size_t)bod[0] * 96, a.frames + (size_t)bod[1] * 96 };
    int lbody[4];
    Vtx V[4];
    double vrest[4][3];
    double u0 = 0, u1 = 0;
    for (int i = 0; i < nvc; i++) {
        lbody[i] = fric_local_body(type, i);
        int vi = a.cverts[4 * ci + i];
        const double* f = fr[lbody[i]];
        for (int j = 0; j < 3; j++) vrest[i][j] = a.rest[3 * (size_t)vi + j];
        const double* v = vrest[i];
        double U[3];
        for (int j = 0; j < 3; j++) {
            V[i].X[j] = f[3 * j] * v[0] + f[3 * j + 1] * v[1] + f[3 * j + 2] * v[2] + f[90 + j];
            for (int k = 0; k < 3; k++) {
                const double* dR = f + 9 + 9 * k;
                V[i].D[j][k] = dR[3 * j] * v[0] + dR[3 * j + 1] * v[1] + dR[3 * j + 2] * v[2];
            }
            U[j] = V[i].X[j] - a.v0c[ci * 12 + 3 * i + j];
        }
        u0 += g[i] * dot(t1, U);
        u1 += g[i] * dot(t2, U);
    }
    const double x = sqrt(u0 * u0 + u1 * u1);
    const double eps = a.epsvh;
    const double ml = a.mu * lambda;
    double f0, f1x, h00, h01, h11;
    if (x >= eps) {
        f0 = x;
        f1x = 1 / x;
        double x3 = x * x * x;
        h00 = f1x - u0 * u0 / x3;
        h01 = -u0 * u1 / x3;
        h11 = f1x - u1 * u1 / x3;
    } else {
        f0 = -x * x * x / (3 * eps * eps) + x * x / eps + eps / 3;
        f1x = 2 / eps - x / (eps * eps);
        double k = x > 0 ? -1 / (eps * eps * x) : 0.0;
        h00 = f1x + k * u0 * u0;
        h01 = k * u0 * u1;
        h11 = f1x + k * u1 * u1;
    }
    if (a.energy) a.energy[ci] = ml * f0;
    const bool want_g = (a.flags & (RIGC_GRAD | RIGC_HESS)) != 0;
    const bool want_h = (a.flags & RIGC_HESS) != 0;
    if (!want_g) return false;
    double gX[4][3];
    for (int i = 0; i < nvc; i++)
        for (int j = 0; j < 3; j++) gX[i][j] = ml * f1x * g[i] * (t1[j] * u0 + t2[j] * u1);
    double G[12];
    to_body(V, lbody, nvc, gX, G);
    if (a.grad)
        for (int k = 0; k < 12; k++) a.grad[ci * 12 + k] = G[k];
    if (!want_h) return false;
    for (int r = 0; r < 12; r++)
        for (int c = r; c < 12; c++) H.at(r, c) = 0;
    double A0[4][3], A1[4][3], G0[12], G1[12];
    for (int i = 0; i < nvc; i++)
        for (int j = 0; j < 3; j++) {
            A0[i][j] = g[i] * t1[j];
            A1[i][j] = g[i] * t2[j];
        }
    to_body(V, lbody, nvc, A0, G0);
    to_body(V, lbody, nvc, A1, G1);
    add_outer(H, ml * h00, G0);
    add_sym_outer(H, ml * h01, G0, G1);
    add_outer(H, ml * h11, G1);
    for (int i = 0; i < nvc; i++) add_curvature(H, fr[lbody[i]], lbody[i], vrest[i], gX[i]);
    return true;
}

// one warp per block, per_warp constraints built by lanes, then projected
// by the warp (the layout of the barrier kernel)
__global__ void __launch_bounds__(kBarrierTPB)
k_friction_local(FrictionArgs a, int per_warp)
{
    extern __shared__ double smem[];
    const int lane = threadIdx.x;
    const int64_t ci = (int64_t)blockIdx.x * per_warp + lane;
    const bool mine = lane < per_warp && ci < a.n;
    SMat H { smem + lane };
    bool built = mine && friction_build(a, ci, H);
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

// ---------------------------------------------------------------------------

int friction_setup(Ctx& c, const double* x0, double dhat, double kappa, double mu, double dmin)
{
    Friction& F = c.fric;
    const int64_t n = c.cons.num;
    cudaStream_t st = c.stream;
    RIGC_TRY(F.type.reserve((size_t)n * 4 + 8));
    RIGC_TRY(F.verts.reserve((size_t)n * 16 + 8));
    RIGC_TRY(F.bodies.reserve((size_t)n * 8 + 8));
    RIGC_TRY(F.coef.reserve((size_t)n * kFricCoef * 8 + 8));
    RIGC_TRY(F.v0c.reserve((size_t)n * 12 * 8 + 8));
    F.num = 0;
    F.mu = mu;
    if (n > 0) {
        RIGC_CUDA(cudaMemcpyAsync(F.type.ptr, c.cons.type.ptr, n * 4, cudaMemcpyDeviceToDevice, st));
        RIGC_CUDA(cudaMemcpyAsync(F.verts.ptr, c.cons.verts.ptr, n * 16, cudaMemcpyDeviceToDevice, st));
        RIGC_CUDA(cudaMemcpyAsync(F.bodies.ptr, c.cons.bodies.ptr, n * 8, cudaMemcpyDeviceToDevice, st));
        RIGC_TRY(F.V0.reserve((size_t)c.s.nv * 3 * 8 + 8));
        RIGC_TRY(compute_world_vertices_rn(c, x0, F.V0.as<double>(), c.scratch[5]));
        FrictionSetupArgs a;
        a.ctype = F.type.as<int>();
        a.cverts = F.verts.as<int>();
        a.cweight = c.cons.weight.as<double>();
        a.V0 = F.V0.as<double>();
        a.n = n;
        a.dhat = dhat;
        a.dmin = dmin;
        a.kappa = kappa;
        a.coef = F.coef.as<double>();
        a.v0c = F.v0c.as<double>();
        RIGC_COUNT_LAUNCH();
        k_friction_setup<<<grid_for(n, 128), 128, 0, st>>>(a);
        RIGC_CUDA(cudaGetLastError());
    }
    F.num = n;
    return RIGC_OK;
}

int launch_friction_local(Ctx& c, const double* x, double epsvh, int flags, double* energy,
                          double* grad, double* blocks, double* hess)
{
    Friction& F = c.fric;
    RIGC_TRY(launch_body_frames(c, x));
    if (F.num == 0) return RIGC_OK;
    static bool attr = false;
    if (!attr) {
        RIGC_CUDA(cudaFuncSetAttribute(k_friction_local, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)local_terms_smem_bytes()));
        attr = true;
    }
    FrictionArgs a;
    a.rest = c.s.rest;
    a.frames = c.frames.as<double>();
    a.ctype = F.type.as<int>();
    a.cverts = F.verts.as<int>();
    a.cbodies = F.bodies.as<int>();
    a.coef = F.coef.as<double>();
    a.v0c = F.v0c.as<double>();
    a.n = F.num;
    a.mu = F.mu;
    a.epsvh = epsvh;
    a.flags = flags;
    a.energy = energy;
    a.grad = grad;
    a.blocks = blocks;
    a.hess = hess;
    const int pw = local_terms_per_warp(F.num);
    RIGC_COUNT_LAUNCH();
    k_friction_local<<<grid_for(F.num, pw), kBarrierTPB, local_terms_smem_bytes(), c.stream>>>(a, pw);
    RIGC_CUDA(cudaGetLastError());
    return RIGC_OK;
}

// energy (to the host), assembled gradient and block-sparse Hessian
int friction_term(Ctx& c, const double* x, double epsvh, int flags, rigc_barrier_out* out)
{
    Friction& F = c.fric;
    const int64_t n = F.num;
    const bool g = (flags & (RIGC_GRAD | RIGC_HESS)) != 0, h = (flags & RIGC_HESS) != 0;
    RIGC_TRY(F.c_energy.reserve((size_t)n * 8 + 8));
    if (g) RIGC_TRY(F.c_grad.reserve((size_t)n * 96 + 8));
    if (h) RIGC_TRY(F.c_blocks.reserve((size_t)n * 144 * 8 + 8));
    RIGC_TRY(launch_friction_local(c, x, epsvh, flags, F.c_energy.as<double>(),
                                   g ? F.c_grad.as<double>() : nullptr,
                                   h ? F.c_blocks.as<double>() : nullptr, nullptr));
    double* e_dev = reinterpret_cast<double*>(c.d_scalars.as<char>() + 2056);
    if (n > 0) {
        RIGC_TRY(sum_f64(F.c_energy.as<double>(), n, e_dev, c.scratch[6], c.stream));
    } else {
        RIGC_CUDA(cudaMemsetAsync(e_dev, 0, sizeof(double), c.stream));
    }
    int32_t* nseg = c.d_scalars.as<int32_t>() + 2;
    if (g)
        RIGC_TRY(assemble_terms(c, F.bodies.as<int>(), n, F.c_grad.as<double>(),
                                F.c_blocks.as<double>(), F.grad, F.row_ptr, F.col, F.val, nseg, h));
    RIGC_CUDA(cudaMemcpyAsync(c.h_scalars + 2, e_dev, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    if (h && n > 0)
        RIGC_CUDA(cudaMemcpyAsync(c.h_scalars + 3, nseg + 1, sizeof(int32_t), cudaMemcpyDeviceToHost,
                                  c.stream));
    RIGC_CUDA(cudaStreamSynchronize(c.stream));
    F.nnzb = 0;
    if (h && n > 0) {
        int32_t nn;
        std::memcpy(&nn, c.h_scalars + 3, sizeof(int32_t));
        F.nnzb = nn;
    }
    if (out) {
        out->energy = c.h_scalars[2];
        out->nnzb = h ? F.nnzb : 0;
        out->grad = g ? F.grad.as<double>() : nullptr;
        out->row_ptr = h ? F.row_ptr.as<int32_t>() : nullptr;
        out->col = h ? F.col.as<int32_t>() : nullptr;
        out->val = h ? F.val.as<double>() : nullptr;
    }
    return RIGC_OK;
}

} // namespace rigc
