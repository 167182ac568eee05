// Rotation-vector kinematics on the device.
//
// R(theta) = I + sinc(|theta|)[theta]x + 1/2 sinc(|theta|/2)^2 [theta]x^2
// (src/physics/pose.tpp:203-218) with sinc as src/utils/sinc.cpp:5-34 defines
// it.  Two flavours:
//  * rot_rn: every operation an explicit round-to-nearest intrinsic in a fixed
//    order, so the result is the same bits on any device and on the host
//    restatement (used wherever an exact decision depends on the vertex
//    positions: constraint sets, broad-phase boxes);
//  * body_frame: R with its first and second derivatives in theta, from the
//    closed-form gradient/Hessian of sinc(|x|) (sinc.cpp:103-141) and the
//    product rule on I + a K + b K^2 (contraction allowed; used by the
//    barrier derivatives).
// sin/cos are evaluated by a Cody-Waite reduction by pi/2 (three-part split,
// 33-bit leading parts) and the Taylor series of sin and cos to degree 19/20
// (coefficients 1/n!) by Horner's rule; the error is below 2^-50|y| + 2^-60
// for |x| < 2^20.
#pragma once

#include <cuda_runtime.h>

namespace rigc {

#define RADD(a, b) __dadd_rn((a), (b))
#define RSUB(a, b) __dsub_rn((a), (b))
#define RMUL(a, b) __dmul_rn((a), (b))
#define RDIV(a, b) __ddiv_rn((a), (b))

__device__ __forceinline__ double det_reduce(double x, long long& k)
{
    const double kTwoOverPi = 0.6366197723675814;
    const double kP1 = 1.5707963267341256;
    const double kP2 = 6.077100506303966e-11;
    const double kP3 = 2.0222662487959506e-21;
    double kd = rint(RMUL(x, kTwoOverPi));
    k = (long long)kd;
    double r = RSUB(x, RMUL(kd, kP1));
    r = RSUB(r, RMUL(kd, kP2));
    r = RSUB(r, RMUL(kd, kP3));
    return r;
}

__device__ __forceinline__ double det_sin_poly(double r)
{
    double z = RMUL(r, r);
    double s = -1.0 / 121645100408832000.0;
    s = RMUL(s, z);
    s = RADD(1.0 / 355687428096000.0, s);
    s = RMUL(s, z);
    s = RADD(-1.0 / 1307674368000.0, s);
    s = RMUL(s, z);
    s = RADD(1.0 / 6227020800.0, s);
    s = RMUL(s, z);
    s = RADD(-1.0 / 39916800.0, s);
    s = RMUL(s, z);
    s = RADD(1.0 / 362880.0, s);
    s = RMUL(s, z);
    s = RADD(-1.0 / 5040.0, s);
    s = RMUL(s, z);
    s = RADD(1.0 / 120.0, s);
    s = RMUL(s, z);
    s = RADD(-1.0 / 6.0, s);
    double r3 = RMUL(r, z);
    return RADD(r, RMUL(r3, s));
}

__device__ __forceinline__ double det_cos_poly(double r)
{
    double z = RMUL(r, r);
    double p = 1.0 / 2432902008176640000.0;
    p = RMUL(p, z);
    p = RADD(-1.0 / 6402373705728000.0, p);
    p = RMUL(p, z);
    p = RADD(1.0 / 20922789888000.0, p);
    p = RMUL(p, z);
    p = RADD(-1.0 / 87178291200.0, p);
    p = RMUL(p, z);
    p = RADD(1.0 / 479001600.0, p);
    p = RMUL(p, z);
    p = RADD(-1.0 / 3628800.0, p);
    p = RMUL(p, z);
    p = RADD(1.0 / 40320.0, p);
    p = RMUL(p, z);
    p = RADD(-1.0 / 720.0, p);
    p = RMUL(p, z);
    p = RADD(1.0 / 24.0, p);
    p = RMUL(p, z);
    p = RADD(-0.5, p);
    p = RMUL(p, z);
    return RADD(1.0, p);
}

__device__ __forceinline__ double det_sin(double x)
{
    long long k;
    double r = det_reduce(x, k);
    switch (k & 3) {
    case 0: return det_sin_poly(r);
    case 1: return det_cos_poly(r);
    case 2: return -det_sin_poly(r);
    default: return -det_cos_poly(r);
    }
}

__device__ __forceinline__ double det_cos(double x)
{
    long long k;
    double r = det_reduce(x, k);
    switch (k & 3) {
    case 0: return det_cos_poly(r);
    case 1: return -det_sin_poly(r);
    case 2: return -det_cos_poly(r);
    default: return det_sin_poly(r);
    }
}

// both at once (shared reduction)
__device__ __forceinline__ void det_sincos(double x, double& s, double& c)
{
    long long k;
    double r = det_reduce(x, k);
    double sp = det_sin_poly(r), cp = det_cos_poly(r);
    switch (k & 3) {
    case 0: s = sp; c = cp; break;
    case 1: s = cp; c = -sp; break;
    case 2: s = -sp; c = -cp; break;
    default: s = -cp; c = sp; break;
    }
}

__device__ __forceinline__ double det_trig_err(double y)
{
    return RADD(RMUL(fabs(y), 8.881784197001252e-16), 8.673617379884035e-19);
}

// sinc (sinc.cpp:10-34) with round-to-nearest intrinsics
__device__ __forceinline__ double sinc_rn(double x)
{
    const double kT0 = 2.220446049250313e-16, kT2 = 1.4901161193847656e-08,
                 kTN = 1.220703125e-04;
    double ax = fabs(x);
    if (ax >= kTN) return RDIV(det_sin(x), x);
    double r = 1.0;
    if (ax >= kT0) {
        double x2 = RMUL(x, x);
        r = RSUB(r, RDIV(x2, 6.0));
        if (ax >= kT2) r = RADD(r, RDIV(RMUL(x2, x2), 120.0));
    }
    return r;
}

__device__ __forceinline__ double norm3_rn(double a, double b, double c)
{
    a = fabs(a);
    b = fabs(b);
    c = fabs(c);
    return __dsqrt_rn(RADD(RADD(RMUL(a, a), RMUL(b, b)), RMUL(c, c)));
}

// R row-major, exact operation order shared with the host restatement
__device__ __forceinline__ void rot_rn(const double t[3], double R[9])
{
    double a = sinc_rn(norm3_rn(t[0], t[1], t[2]));
    double s = sinc_rn(norm3_rn(RDIV(t[0], 2.0), RDIV(t[1], 2.0), RDIV(t[2], 2.0)));
    double b = RMUL(RMUL(0.5, s), s);
    double K[9] = { 0.0, -t[2], t[1], t[2], 0.0, -t[0], -t[1], t[0], 0.0 };
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            double k2 = RADD(RADD(RMUL(K[3 * i], K[j]), RMUL(K[3 * i + 1], K[3 + j])),
                             RMUL(K[3 * i + 2], K[6 + j]));
            double r = RADD(RMUL(a, K[3 * i + j]), RMUL(b, k2));
            R[3 * i + j] = i == j ? RADD(r, 1.0) : r;
        }
}

// V_j = ((v0 R_j0 + v1 R_j1) + v2 R_j2) + p_j
__device__ __forceinline__ void world_vertex_rn(const double R[9], const double p[3],
                                                const double v[3], double out[3])
{
#pragma unroll
    for (int j = 0; j < 3; j++)
        out[j] = RADD(RADD(RADD(RMUL(v[0], R[3 * j]), RMUL(v[1], R[3 * j + 1])),
                           RMUL(v[2], R[3 * j + 2])),
                      p[j]);
}

// ---------------------------------------------------------------------------
// body frame with derivatives (contraction allowed)

// d sinc(x)/dx / x and (d2 sinc/dx2 / x^2 - d sinc/dx / x^3) (sinc.cpp:103-141)
__device__ __forceinline__ double dsinc_over_x(double x, double s, double c)
{
    double x2 = x * x;
    if (fabs(x) > 1e-4) return (x * c - s) / (x2 * x);
    return x2 * (-x2 / 840.0 + 1.0 / 30.0) - 1.0 / 3.0;
}
__device__ __forceinline__ double ddsinc_term(double x, double s, double c)
{
    double x2 = x * x, x4 = x2 * x2;
    if (fabs(x) > 0.1) return ((3 - x2) * s - 3 * x * c) / (x4 * x);
    return x4 / 7560.0 - x2 / 210.0 + 1.0 / 15.0;
}

// Frame layout: R[9] | dR[3][9] | d2R[6][9] (pairs 00 01 02 11 12 22), all
// row-major 3x3.  dR[k] = dR/dtheta_k.
constexpr int kFrameDoubles = 90;

__device__ __forceinline__ int sym_index(int k, int l)
{
    // (0,0)=0 (0,1)=1 (0,2)=2 (1,1)=3 (1,2)=4 (2,2)=5
    if (k > l) { int t = k; k = l; l = t; }
    return k == 0 ? l : (k == 1 ? 2 + l : 5);
}

__device__ inline void body_frame(const double t[3], double* F)
{
    // a(t) = sinc(|t|), g_a = dsinc_over_x(|t|) t, H_a = dd(|t|) t t^T + g1 I
    double n = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    double sn, cn;
    det_sincos(n, sn, cn);
    double a = n >= 1.220703125e-04 ? sn / n : sinc_rn(n);
    double g1 = dsinc_over_x(n, sn, cn), g2 = ddsinc_term(n, sn, cn);
    // half angle: s(t) = sinc(|t/2|), ds = 1/2 g(t/2), d2s = 1/4 H(t/2)
    double h[3] = { 0.5 * t[0], 0.5 * t[1], 0.5 * t[2] };
    double nh = 0.5 * n;
    double shn, chn;
    det_sincos(nh, shn, chn);
    double sh = nh >= 1.220703125e-04 ? shn / nh : sinc_rn(nh);
    double h1 = dsinc_over_x(nh, shn, chn), h2 = ddsinc_term(nh, shn, chn);
    double ga[3], gs[3], Ha[3][3], Hs[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        ga[i] = g1 * t[i];
        gs[i] = 0.5 * h1 * h[i];
#pragma unroll
        for (int j = 0; j < 3; j++) {
            Ha[i][j] = g2 * t[i] * t[j] + (i == j ? g1 : 0.0);
            Hs[i][j] = 0.25 * (h2 * h[i] * h[j] + (i == j ? h1 : 0.0));
        }
    }
    // b = 1/2 s^2: gb = s gs, Hb = gs gs^T + s Hs
    double b = 0.5 * sh * sh, gb[3], Hb[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        gb[i] = sh * gs[i];
#pragma unroll
        for (int j = 0; j < 3; j++) Hb[i][j] = gs[i] * gs[j] + sh * Hs[i][j];
    }
    // K = [t]x, E_k = [e_k]x, K2 = K K
    double K[9] = { 0, -t[2], t[1], t[2], 0, -t[0], -t[1], t[0], 0 };
    double K2[9];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            K2[3 * i + j] = K[3 * i] * K[j] + K[3 * i + 1] * K[3 + j] + K[3 * i + 2] * K[6 + j];
    auto E = [](int k, int i, int j) -> double {
        // [e_k]x entries
        if (k == 0) return (i == 1 && j == 2) ? -1.0 : ((i == 2 && j == 1) ? 1.0 : 0.0);
        if (k == 1) return (i == 0 && j == 2) ? 1.0 : ((i == 2 && j == 0) ? -1.0 : 0.0);
        return (i == 0 && j == 1) ? -1.0 : ((i == 1 && j == 0) ? 1.0 : 0.0);
    };
    // (E_k K + K E_k) and (E_k E_l + E_l E_k)
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            F[3 * i + j] = a * K[3 * i + j] + b * K2[3 * i + j] + (i == j ? 1.0 : 0.0);
#pragma unroll
    for (int k = 0; k < 3; k++) {
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                double EK = 0, KE = 0;
#pragma unroll
                for (int m = 0; m < 3; m++) {
                    EK += E(k, i, m) * K[3 * m + j];
                    KE += K[3 * i + m] * E(k, m, j);
                }
                F[9 + 9 * k + 3 * i + j] = ga[k] * K[3 * i + j] + a * E(k, i, j)
                    + gb[k] * K2[3 * i + j] + b * (EK + KE);
            }
    }
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
        for (int l = k; l < 3; l++) {
            int idx = sym_index(k, l);
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int j = 0; j < 3; j++) {
                    double EkK = 0, KEk = 0, ElK = 0, KEl = 0, EkEl = 0, ElEk = 0;
#pragma unroll
                    for (int m = 0; m < 3; m++) {
                        EkK += E(k, i, m) * K[3 * m + j];
                        KEk += K[3 * i + m] * E(k, m, j);
                        ElK += E(l, i, m) * K[3 * m + j];
                        KEl += K[3 * i + m] * E(l, m, j);
                        EkEl += E(k, i, m) * E(l, m, j);
                        ElEk += E(l, i, m) * E(k, m, j);
                    }
                    F[36 + 9 * idx + 3 * i + j] = Ha[k][l] * K[3 * i + j] + ga[k] * E(l, i, j)
                        + ga[l] * E(k, i, j) + Hb[k][l] * K2[3 * i + j]
                        + gb[k] * (ElK + KEl) + gb[l] * (EkK + KEk) + b * (EkEl + ElEk);
                }
        }
}

} // namespace rigc
