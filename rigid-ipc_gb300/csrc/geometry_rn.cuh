// Distances and closest-feature classification with explicit round-to-nearest
// operations in a fixed order, so every exact decision (distance type, active
// test, mollification) is the same bit pattern on any device and in the host
// restatement.  Formulas: squared point-point, point-line, point-plane and
// line-line distances of the IPC formulation (Li et al. 2020); triangle
// classification by 2x2 solves in each edge's (edge, in-plane normal) frame;
// segment classification by Sunday's segment-segment closest-point algorithm.
#pragma once

#include "rotation.cuh"

namespace rigc {

enum { PT_P_T0 = 0, PT_P_T1, PT_P_T2, PT_P_E0, PT_P_E1, PT_P_E2, PT_P_T };
enum {
    EE_EA0_EB0 = 0, EE_EA0_EB1, EE_EA1_EB0, EE_EA1_EB1,
    EE_EA_EB0, EE_EA_EB1, EE_EA0_EB, EE_EA1_EB, EE_EA_EB
};

__device__ __forceinline__ void sub3_rn(const double* a, const double* b, double* r)
{
    r[0] = RSUB(a[0], b[0]);
    r[1] = RSUB(a[1], b[1]);
    r[2] = RSUB(a[2], b[2]);
}
__device__ __forceinline__ double dot3_rn(const double* a, const double* b)
{
    return RADD(RADD(RMUL(a[0], b[0]), RMUL(a[1], b[1])), RMUL(a[2], b[2]));
}
__device__ __forceinline__ void cross3_rn(const double* a, const double* b, double* r)
{
    r[0] = RSUB(RMUL(a[1], b[2]), RMUL(a[2], b[1]));
    r[1] = RSUB(RMUL(a[2], b[0]), RMUL(a[0], b[2]));
    r[2] = RSUB(RMUL(a[0], b[1]), RMUL(a[1], b[0]));
}

__device__ __forceinline__ double pp_sqdist_rn(const double* p, const double* q)
{
    double d[3];
    sub3_rn(p, q, d);
    return dot3_rn(d, d);
}

__device__ __forceinline__ double pl_sqdist_rn(const double* p, const double* e0, const double* e1)
{
    double a[3], b[3], c[3], e[3];
    sub3_rn(e0, p, a);
    sub3_rn(e1, p, b);
    cross3_rn(a, b, c);
    sub3_rn(e1, e0, e);
    return RDIV(dot3_rn(c, c), dot3_rn(e, e));
}

__device__ __forceinline__ double ptplane_sqdist_rn(const double* p, const double* t0,
                                                    const double* t1, const double* t2)
{
    double a[3], b[3], n[3], w[3];
    sub3_rn(t1, t0, a);
    sub3_rn(t2, t0, b);
    cross3_rn(a, b, n);
    sub3_rn(p, t0, w);
    double u = dot3_rn(n, w);
    return RDIV(RMUL(u, u), dot3_rn(n, n));
}

__device__ __forceinline__ double ll_sqdist_rn(const double* a0, const double* a1,
                                               const double* b0, const double* b1)
{
    double a[3], b[3], n[3], w[3];
    sub3_rn(a1, a0, a);
    sub3_rn(b1, b0, b);
    cross3_rn(a, b, n);
    sub3_rn(b0, a0, w);
    double u = dot3_rn(n, w);
    return RDIV(RMUL(u, u), dot3_rn(n, n));
}

__device__ __forceinline__ double ee_cross_sqnorm_rn(const double* a0, const double* a1,
                                                     const double* b0, const double* b1)
{
    double a[3], b[3], n[3];
    sub3_rn(a1, a0, a);
    sub3_rn(b1, b0, b);
    cross3_rn(a, b, n);
    return dot3_rn(n, n);
}

__device__ __forceinline__ void edge_frame_params_rn(const double* p, const double* a,
                                                     const double* b, const double* n,
                                                     double& s, double& t)
{
    double e[3], m[3], w[3];
    sub3_rn(b, a, e);
    cross3_rn(e, n, m);
    sub3_rn(p, a, w);
    double A00 = dot3_rn(e, e), A01 = dot3_rn(e, m), A11 = dot3_rn(m, m);
    double r0 = dot3_rn(e, w), r1 = dot3_rn(m, w);
    double det = RSUB(RMUL(A00, A11), RMUL(A01, A01));
    s = RDIV(RSUB(RMUL(A11, r0), RMUL(A01, r1)), det);
    t = RDIV(RSUB(RMUL(A00, r1), RMUL(A01, r0)), det);
}

__device__ __forceinline__ int pt_type_rn(const double* p, const double* t0, const double* t1,
                                          const double* t2)
{
    double a[3], b[3], n[3];
    sub3_rn(t1, t0, a);
    sub3_rn(t2, t0, b);
    cross3_rn(a, b, n);
    double s0, q0, s1, q1, s2, q2;
    edge_frame_params_rn(p, t0, t1, n, s0, q0);
    if (s0 > 0.0 && s0 < 1.0 && q0 >= 0.0) return PT_P_E0;
    edge_frame_params_rn(p, t1, t2, n, s1, q1);
    if (s1 > 0.0 && s1 < 1.0 && q1 >= 0.0) return PT_P_E1;
    edge_frame_params_rn(p, t2, t0, n, s2, q2);
    if (s2 > 0.0 && s2 < 1.0 && q2 >= 0.0) return PT_P_E2;
    if (s0 <= 0.0 && s2 >= 1.0) return PT_P_T0;
    if (s1 <= 0.0 && s0 >= 1.0) return PT_P_T1;
    if (s2 <= 0.0 && s1 >= 1.0) return PT_P_T2;
    return PT_P_T;
}

__device__ __forceinline__ int ee_type_rn(const double* ea0, const double* ea1,
                                          const double* eb0, const double* eb1)
{
    double u[3], v[3], w[3];
    sub3_rn(ea1, ea0, u);
    sub3_rn(eb1, eb0, v);
    sub3_rn(ea0, eb0, w);
    double a = dot3_rn(u, u), b = dot3_rn(u, v), c = dot3_rn(v, v);
    double d = dot3_rn(u, w), e = dot3_rn(v, w);
    double D = RSUB(RMUL(a, c), RMUL(b, b));
    if (a == 0.0 && c == 0.0) return EE_EA0_EB0;
    if (a == 0.0) return EE_EA0_EB;
    if (c == 0.0) return EE_EA_EB0;
    double n[3];
    cross3_rn(u, v, n);
    double ac = RMUL(a, c);
    double par_tol = RMUL(1e-20, ac > 1.0 ? ac : 1.0);
    int def = EE_EA_EB;
    double tN, tD;
    if (dot3_rn(n, n) < par_tol) {
        tN = e;
        tD = c;
        def = EE_EA0_EB;
    } else {
        double sN = RSUB(RMUL(b, e), RMUL(c, d));
        if (sN <= 0.0) {
            tN = e;
            tD = c;
            def = EE_EA0_EB;
        } else if (sN >= D) {
            tN = RADD(e, b);
            tD = c;
            def = EE_EA1_EB;
        } else {
            tN = RSUB(RMUL(a, e), RMUL(b, d));
            tD = D;
        }
    }
    if (tN <= 0.0) {
        if (-d <= 0.0) return EE_EA0_EB0;
        if (-d >= a) return EE_EA1_EB0;
        return EE_EA_EB0;
    }
    if (tN >= tD) {
        double q = RADD(-d, b);
        if (q <= 0.0) return EE_EA0_EB1;
        if (q >= a) return EE_EA1_EB1;
        return EE_EA_EB1;
    }
    return def;
}

// squared distance of two segments by their closest features: the distance
// of an EE constraint (ipc-toolkit EdgeEdgeConstraint computes the type at
// the current positions, since near-parallel pairs whose closest points are
// endpoints are kept as mollified EE constraints)
__device__ __forceinline__ double ee_sqdist_rn(const double* a0, const double* a1,
                                               const double* b0, const double* b1)
{
    switch (ee_type_rn(a0, a1, b0, b1)) {
    case EE_EA0_EB0: return pp_sqdist_rn(a0, b0);
    case EE_EA0_EB1: return pp_sqdist_rn(a0, b1);
    case EE_EA1_EB0: return pp_sqdist_rn(a1, b0);
    case EE_EA1_EB1: return pp_sqdist_rn(a1, b1);
    case EE_EA_EB0: return pl_sqdist_rn(b0, a0, a1);
    case EE_EA_EB1: return pl_sqdist_rn(b1, a0, a1);
    case EE_EA0_EB: return pl_sqdist_rn(a0, b0, b1);
    case EE_EA1_EB: return pl_sqdist_rn(a1, b0, b1);
    default: return ll_sqdist_rn(a0, a1, b0, b1);
    }
}

} // namespace rigc
