// Device helpers shared by the per-constraint local terms (barrier and
// friction): vertex positions with their rotation derivatives, body-space
// images of vertex-space vectors, shared-memory 12x12 accumulators, the rigid
// curvature term of apply_chain_rule
// (src/problems/distance_barrier_rb_problem.cpp:1182-1248) and the
// warp-parallel PSD projection.
#pragma once

#include "common.cuh"
#include "rotation.cuh"

namespace rigc {

// ---------------------------------------------------------------------------

constexpr int kBarrierTPB = 32;

struct Vtx {
    double X[3];     // world position
    double D[3][3];  // dX/dtheta  [coord][k]
};

__device__ __forceinline__ void cross(const double* a, const double* b, double* r)
{
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ __forceinline__ double dot(const double* a, const double* b)
{
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// shared-memory symmetric 12x12 accumulator: the upper triangle (r <= c)
// packed row by row (78 entries), entry-major / thread-minor
constexpr int kSymEntries = 78;
struct SMat {
    double* base;
    __device__ __forceinline__ double& at(int r, int c) const
    {
        return base[(r * (23 - r) / 2 + c) * kBarrierTPB];
    }
};

// H += coef * (a b^T + b a^T) on the upper triangle (a, b in body space)
__device__ __forceinline__ void add_sym_outer(SMat H, double coef, const double* a, const double* b)
{
    for (int r = 0; r < 12; r++) {
        double ar = coef * a[r], br = coef * b[r];
        for (int c = r; c < 12; c++) H.at(r, c) += ar * b[c] + br * a[c];
    }
}
__device__ __forceinline__ void add_outer(SMat H, double coef, const double* a)
{
    for (int r = 0; r < 12; r++) {
        double ar = coef * a[r];
        for (int c = r; c < 12; c++) H.at(r, c) += ar * a[c];
    }
}

// body-space image of a per-vertex vector field: out[6 lb + 0..2] += g_i,
// out[6 lb + 3 + k] += D_i[:, k] . g_i
__device__ __forceinline__ void to_body(const Vtx* V, const int* lbody, int nvc,
                                        const double (*g)[3], double* out)
{
    for (int k = 0; k < 12; k++) out[k] = 0;
    for (int i = 0; i < nvc; i++) {
        int o = 6 * lbody[i];
        for (int j = 0; j < 3; j++) out[o + j] += g[i][j];
        for (int k = 0; k < 3; k++)
            out[o + 3 + k] += V[i].D[0][k] * g[i][0] + V[i].D[1][k] * g[i][1] + V[i].D[2][k] * g[i][2];
    }
}

// Gram term H += coef * JM^T JM where JM (3 x 12) = sum_i M_i J_i and
// M_i = m_i * I + (skew parts): here M_i given as full 3x3 per vertex.
__device__ __forceinline__ void add_gram(SMat H, double coef, const Vtx* V, const int* lbody,
                                         int nvc, const double (*M)[9])
{
    double JM[3][12];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 12; c++) JM[r][c] = 0;
    for (int i = 0; i < nvc; i++) {
        int o = 6 * lbody[i];
        for (int r = 0; r < 3; r++) {
            for (int j = 0; j < 3; j++) JM[r][o + j] += M[i][3 * r + j];
            for (int k = 0; k < 3; k++)
                JM[r][o + 3 + k] += M[i][3 * r] * V[i].D[0][k] + M[i][3 * r + 1] * V[i].D[1][k]
                    + M[i][3 * r + 2] * V[i].D[2][k];
        }
    }
    for (int r = 0; r < 12; r++) {
        double a0 = coef * JM[0][r], a1 = coef * JM[1][r], a2 = coef * JM[2][r];
        for (int c = r; c < 12; c++) H.at(r, c) += a0 * JM[0][c] + a1 * JM[1][c] + a2 * JM[2][c];
    }
}

// skew pair block: H(i-part, j-part) += J_i^T [s]x J_j, and its transpose
__device__ __forceinline__ void add_skew_pair(SMat H, const Vtx& Vi, int oi, const Vtx& Vj,
                                              int oj, const double* s)
{
    // K = [s]x
    const double K[3][3] = { { 0, -s[2], s[1] }, { s[2], 0, -s[0] }, { -s[1], s[0], 0 } };
    // blocks: [K, K Dj ; Di^T K, Di^T K Dj]
    double KD[3][3], DK[3][3], DKD[3][3];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            KD[r][c] = K[r][0] * Vj.D[0][c] + K[r][1] * Vj.D[1][c] + K[r][2] * Vj.D[2][c];
            DK[r][c] = Vi.D[0][r] * K[0][c] + Vi.D[1][r] * K[1][c] + Vi.D[2][r] * K[2][c];
        }
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
            DKD[r][c] = Vi.D[0][r] * KD[0][c] + Vi.D[1][r] * KD[1][c] + Vi.D[2][r] * KD[2][c];
    // B (6x6) = [[K, KD], [DK, DKD]] goes to rows oi.., cols oj..; its
    // transpose to rows oj.., cols oi..; accumulate into the upper triangle.
    for (int r = 0; r < 6; r++)
        for (int c = 0; c < 6; c++) {
            double v = r < 3 ? (c < 3 ? K[r][c] : KD[r][c - 3])
                             : (c < 3 ? DK[r - 3][c] : DKD[r - 3][c - 3]);
            int R = oi + r, C = oj + c;
            // entry (R, C) of B and entry (C, R) of B^T are both v
            if (R <= C) H.at(R, C) += v;
            if (C <= R) H.at(C, R) += v;
        }
}

// curvature term: H(rot lb, rot lb) += sum_j g_j (d2R_kl v)_j
__device__ __forceinline__ void add_curvature(SMat H, const double* frame, int lb,
                                              const double* v, const double* g)
{
    const double* d2 = frame + 36;
    int o = 6 * lb + 3;
    for (int k = 0; k < 3; k++)
        for (int l = k; l < 3; l++) {
            const double* M = d2 + 9 * sym_index(k, l);
            double acc = 0;
            for (int j = 0; j < 3; j++)
                acc += g[j] * (M[3 * j] * v[0] + M[3 * j + 1] * v[1] + M[3 * j + 2] * v[2]);
            H.at(o + k, o + l) += acc;
        }
}

// ---------------------------------------------------------------------------
// PSD projection of one 12x12 (upper triangle filled, in the packed layout
// of its owner thread) by the whole warp: V max(L, 0) V^T from the
// eigen-decomposition A = V L V^T.  As project_to_psd does, a matrix whose
// eigenvalues are all >= 0 is left as it is.
//
// The decomposition is a parallel cyclic Jacobi in round-robin order (each
// round rotates six disjoint (p, q) planes at once, eleven rounds visit all
// 66 pairs), run twice:
//  1. in single precision on A rounded to float, to convergence: it gives
//     eigenvectors V32 accurate to single precision;
//  2. in double precision on B = Q^T A Q, Q being V32 orthonormalised in
//     double; B is diagonal up to the single-precision error, so the Jacobi
//     sweeps converge quadratically from there (two or three sweeps where
//     seven or eight were needed from A itself), the rotations accumulated
//     into Q.
// An FP64 warp instruction costs this GPU's FP64 unit 64 cycles whatever its
// active lanes, a single-precision one one cycle of issue, so the sweeps of
// step 1 are nearly free and the FP64 work drops to a few 12 x 12 products
// and the refining sweeps.  The double-precision stopping rule is the one-step
// method's (off-diagonal sum of squares <= 1e-30 of the diagonal's), so the
// result is the same decomposition to rounding.  (A double-precision
// refinement of V32 by matrix products alone, with no rotations, does not
// reach double precision when the eigenvalues span more decades than single
// precision resolves, as these Hessians' do.)
// Rotation (c, s) per plane follows the textbook symmetric Schur step:
// theta = (a_qq - a_pp) / (2 a_pq), t = sign(theta) / (|theta| +
// sqrt(theta^2 + 1)), c = 1 / sqrt(t^2 + 1), s = t c; the single-precision
// sweeps take it with the fast reciprocal and reciprocal square root (they
// only seed step 2).

constexpr int kLd = 13;  // padded row stride of the warp's work matrices
// doubles: A, Q, T, U (12 x kLd each), 6 (c, s) + 4; then floats A32, V32
// (12 x kLd each), 6 (c, s) + 4
constexpr int kWorkDoubles = 4 * 12 * kLd + 16 + (2 * 12 * kLd + 16) / 2;

// round-robin schedule over 12 indices: round r pairs (r, 11) and
// (pos_k, pos_{11-k}) for k = 1 .. 5, pos_k = (k + r) mod 11; (p, q) with p < q
__device__ __forceinline__ void round_pair(int round, int k, int& p, int& q)
{
    if (k == 0) {
        p = round;
        q = 11;
        return;
    }
    int a = k + round, b = 11 - k + round;
    a = a >= 11 ? a - 11 : a;
    b = b >= 11 ? b - 11 : b;
    p = min(a, b);
    q = max(a, b);
}

// row and column of upper-triangle entry u (row-major, 0 <= u < 78)
__device__ __forceinline__ void upper_rc(int u, int& r, int& c)
{
    r = 0;
    int start = 0;
    while (u >= start + 12 - r) {
        start += 12 - r;
        r++;
    }
    c = r + (u - start);
}

template <class T> __device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ void jacobi_angle(float app, float aqq, float apq, float& c, float& s)
{
    const float theta = __fdividef(aqq - app, 2.0f * apq);
    const float at = fabsf(theta);
    // |theta| > 2^40: t = 1 / (2 theta) to single precision (and theta^2 is
    // not formed)
    float t;
    if (at > 1.0995116e12f) {
        t = __fdividef(0.5f, at);
    } else {
        const float h = fmaf(theta, theta, 1.0f);
        t = __frcp_rn(at + h * rsqrtf(h));
    }
    t = theta >= 0.0f ? t : -t;
    c = rsqrtf(fmaf(t, t, 1.0f));
    s = t * c;
}
__device__ __forceinline__ void jacobi_angle(double app, double aqq, double apq, double& c, double& s)
{
    const double theta = (aqq - app) / (2 * apq);
    const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1));
    c = 1.0 / sqrt(t * t + 1);
    s = t * c;
}

// Cyclic Jacobi on the warp's A (12 x kLd, symmetric) accumulating the
// rotations into V, until the off-diagonal sum of squares is <= tol of the
// diagonal's (or max_sweeps); cs holds 12 scalars of scratch.
template <class T>
__device__ void warp_jacobi(T* A, T* V, T* cs, int lane, T tol, int max_sweeps)
{
    for (int sweep = 0; sweep < max_sweeps; sweep++) {
        T off = 0, diag = 0;
        for (int e = lane; e < 144; e += 32) {
            int r = e / 12, c = e % 12;
            T v = A[r * kLd + c];
            if (r == c) diag += v * v;
            else if (r < c) off += v * v;
        }
        off = warp_sum(off);
        diag = warp_sum(diag);
        if (off <= tol * diag || off == T(0)) break;
        for (int round = 0; round < 11; round++) {
            if (lane < 6) {
                int p, q;
                round_pair(round, lane, p, q);
                T apq = A[p * kLd + q];
                T c = 1, sn = 0;
                if (apq != T(0)) jacobi_angle(A[p * kLd + p], A[q * kLd + q], apq, c, sn);
                cs[2 * lane] = c;
                cs[2 * lane + 1] = sn;
            }
            __syncwarp();
            // columns of A and V: 2 x 6 planes x 12 rows
            for (int it = lane; it < 144; it += 32) {
                T* M = it < 72 ? A : V;
                int j = it < 72 ? it : it - 72;
                int pr = j % 6, k = j / 6;
                int p, q;
                round_pair(round, pr, p, q);
                T c = cs[2 * pr], sn = cs[2 * pr + 1];
                T mkp = M[k * kLd + p], mkq = M[k * kLd + q];
                M[k * kLd + p] = c * mkp - sn * mkq;
                M[k * kLd + q] = sn * mkp + c * mkq;
            }
            __syncwarp();
            // rows of A: 6 planes x 12 columns
            for (int it = lane; it < 72; it += 32) {
                int pr = it % 6, k = it / 6;
                int p, q;
                round_pair(round, pr, p, q);
                T c = cs[2 * pr], sn = cs[2 * pr + 1];
                T apk = A[p * kLd + k], aqk = A[q * kLd + k];
                A[p * kLd + k] = c * apk - sn * aqk;
                A[q * kLd + k] = sn * apk + c * aqk;
            }
            __syncwarp();
        }
    }
}

// C = op(X) Y for 12 x 12 matrices with row stride kLd (op(X) = X or X^T),
// by the warp, entry-strided over the lanes
__device__ __forceinline__ void warp_mm(const double* X, bool xt, const double* Y, double* C, int lane)
{
    for (int e = lane; e < 144; e += 32) {
        const int r = e / 12, c = e % 12;
        double acc = 0;
        for (int k = 0; k < 12; k++) acc += (xt ? X[k * kLd + r] : X[r * kLd + k]) * Y[k * kLd + c];
        C[r * kLd + c] = acc;
    }
    __syncwarp();
}

static __device__ void warp_psd_project(SMat H, double* work, int lane)
{
    double* A = work;               // the matrix
    double* Q = work + 12 * kLd;    // eigenvectors
    double* T = work + 24 * kLd;    // scratch, then B = Q^T A Q
    double* U = work + 36 * kLd;    // scratch
    double* cs = work + 48 * kLd;   // 6 x (c, s)
    float* A32 = reinterpret_cast<float*>(work + 48 * kLd + 16);
    float* V32 = A32 + 12 * kLd;
    float* cs32 = V32 + 12 * kLd;
    // 1. single-precision eigenvectors
    for (int e = lane; e < 144; e += 32) {
        int r = e / 12, c = e % 12;
        const double a = r <= c ? H.at(r, c) : H.at(c, r);
        A[r * kLd + c] = a;
        A32[r * kLd + c] = (float)a;
        V32[r * kLd + c] = r == c ? 1.0f : 0.0f;
    }
    __syncwarp();
    warp_jacobi<float>(A32, V32, cs32, lane, 1e-14f, 12);
    // 2. orthonormalise them in double (two Newton-Schulz steps
    // Q <- Q (3 I - Q^T Q) / 2: the single-precision rotations leave them
    // orthogonal to ~1e-6, each step squares that)
    for (int e = lane; e < 144; e += 32) Q[(e / 12) * kLd + e % 12] = (double)V32[(e / 12) * kLd + e % 12];
    __syncwarp();
    for (int step = 0; step < 2; step++) {
        warp_mm(Q, true, Q, T, lane);
        for (int e = lane; e < 144; e += 32) {
            const int r = e / 12, c = e % 12;
            T[r * kLd + c] = (r == c ? 1.5 : 0.0) - 0.5 * T[r * kLd + c];
        }
        __syncwarp();
        warp_mm(Q, false, T, U, lane);
        for (int e = lane; e < 144; e += 32) Q[(e / 12) * kLd + e % 12] = U[(e / 12) * kLd + e % 12];
        __syncwarp();
    }
    // 3. B = Q^T A Q (symmetric: the upper triangle, mirrored), then the
    // double-precision Jacobi from there, the rotations accumulated into Q
    warp_mm(A, false, Q, U, lane);
    warp_mm(Q, true, U, T, lane);
    for (int e = lane; e < 144; e += 32) {
        const int r = e / 12, c = e % 12;
        if (r > c) T[r * kLd + c] = T[c * kLd + r];
    }
    __syncwarp();
    warp_jacobi<double>(T, Q, cs, lane, 1e-30, 30);
    double wmin = INFINITY;
#pragma unroll
    for (int i = 0; i < 12; i++) wmin = fmin(wmin, T[i * kLd + i]);
    if (wmin >= 0.0) return;  // already PSD: keep the matrix as it is
    // rebuild the upper triangle: sum over positive eigenvalues
    for (int u = lane; u < kSymEntries; u += 32) {
        int r, c;
        upper_rc(u, r, c);
        double acc = 0;
        for (int k = 0; k < 12; k++) {
            const double w = T[k * kLd + k];
            if (w > 0) acc += Q[r * kLd + k] * w * Q[c * kLd + k];
        }
        H.at(r, c) = acc;
    }
    __syncwarp();
}

// local Hessian (symmetric from the upper triangle) to the outputs
__device__ __forceinline__ void write_local_hessian(SMat H, int64_t ci, double* hess, double* blocks)
{
    for (int r = 0; r < 12; r++)
        for (int c = 0; c < 12; c++) {
            double v = r <= c ? H.at(r, c) : H.at(c, r);
            if (hess) hess[ci * 144 + 12 * r + c] = v;
            if (blocks) {
                int blk = (r / 6) * 2 + (c / 6);
                blocks[ci * 144 + blk * 36 + (r % 6) * 6 + (c % 6)] = v;
            }
        }
}

// Generic deterministic assembly of per-constraint body-space terms: cgrad
// (n x 12, two 6-blocks per constraint) into grad (nb x 6) and cblocks
// (n x 4 x 36) into a block-sparse matrix (row_ptr, col, val).  nseg_dev
// points at two device ints: the gradient segment count and the number of
// Hessian blocks (read back by the caller after a sync).
int assemble_terms(Ctx& c, const int* bodies, int64_t n, const double* cgrad,
                   const double* cblocks, DevBuf& grad, DevBuf& row_ptr, DevBuf& col,
                   DevBuf& val, int32_t* nseg_dev, bool with_hess);

size_t local_terms_smem_bytes();
int local_terms_per_warp(int64_t n);
int launch_body_frames(Ctx& c, const double* x);

} // namespace rigc
