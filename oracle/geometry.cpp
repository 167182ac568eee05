// Oracle: rotations, world vertices and their derivatives, distances, barrier,
// constraint set, chain rule, PSD projection, assembly and body energy.
// Test infrastructure only (see oracle.hpp).
#include "oracle.hpp"
#include "trig.hpp"

#include <map>
#include <stdexcept>
#include <unordered_map>

namespace orc {

void Scene::finalize()
{
    vbody.assign(nv, 0);
    ebody.assign(ne, 0);
    fbody.assign(nf, 0);
    for (int b = 0; b < nb; b++) {
        for (int i = bvs[b]; i < bvs[b + 1]; i++) vbody[i] = b;
        for (int i = bes[b]; i < bes[b + 1]; i++) ebody[i] = b;
        for (int i = bfs[b]; i < bfs[b + 1]; i++) fbody[i] = b;
    }
    edge_len.assign(ne, 0);
    for (int e = 0; e < ne; e++) {
        const double* a = rest + 3 * edges[2 * e];
        const double* b = rest + 3 * edges[2 * e + 1];
        double d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2];
        edge_len[e] = std::sqrt((d0 * d0 + d1 * d1) + d2 * d2);
    }
}

// ---------------------------------------------------------------------------
// sinc and its derivatives along |x| (src/utils/sinc.cpp:5-141)

static const double kTaylor0 = 2.220446049250313e-16;   // epsilon
static const double kTaylor2 = 1.4901161193847656e-08;  // sqrt(eps)
static const double kTaylorN = 1.220703125e-04;         // eps^(1/4)

static double sinc_d(double x)
{
    if (std::fabs(x) >= kTaylorN) return det_sin(x) / x;
    double r = 1;
    if (std::fabs(x) >= kTaylor0) {
        double x2 = x * x;
        r = r - x2 / 6.0;
        if (std::fabs(x) >= kTaylor2) r = r + (x2 * x2) / 120.0;
    }
    return r;
}

static double dsinc_over_x(double x)
{
    double x2 = x * x;
    if (std::fabs(x) > 1e-4)
        return (x * det_cos(x) - det_sin(x)) / (x2 * x);
    return x2 * (-x2 / 840.0 + 1.0 / 30.0) - 1.0 / 3.0;
}

static double ddsinc_over_x2_minus_dsinc_over_x3(double x)
{
    double x2 = x * x, x4 = x2 * x2;
    if (std::fabs(x) > 0.1)
        return ((3 - x2) * det_sin(x) - 3 * x * det_cos(x)) / (x4 * x);
    return x4 / 7560.0 - x2 / 210.0 + 1.0 / 15.0;
}

static double norm3(const double* x)
{
    double a = std::fabs(x[0]), b = std::fabs(x[1]), c = std::fabs(x[2]);
    return std::sqrt((a * a + b * b) + c * c);
}

// sinc(|x|) on autodiff values (sinc.hpp:67-98): value and closed-form
// gradient/Hessian at the values, then the chain rule into the variables.
template <int N> static D2<N> sinc_normx(const D2<N> x[3])
{
    double xv[3] = { x[0].v, x[1].v, x[2].v };
    double n = norm3(xv);
    double value = sinc_d(n);
    double g1 = dsinc_over_x(n);
    double g2 = ddsinc_over_x2_minus_dsinc_over_x3(n);
    double grad[3], hess[3][3];
    for (int i = 0; i < 3; i++) grad[i] = g1 * xv[i];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            hess[i][j] = g2 * xv[i] * xv[j] + (i == j ? g1 : 0.0);
    D2<N> r(value);
    for (int k = 0; k < 3; k++)
        for (int a = 0; a < N; a++) r.g[a] += grad[k] * x[k].g[a];
    for (int k = 0; k < 3; k++) {
        for (int l = 0; l < 3; l++)
            for (int a = 0; a < N; a++)
                for (int b = 0; b < N; b++)
                    r.h[a][b] += hess[k][l] * x[l].g[a] * x[k].g[b];
        for (int a = 0; a < N; a++)
            for (int b = 0; b < N; b++) r.h[a][b] += grad[k] * x[k].h[a][b];
    }
    return r;
}

// R(theta) = I + sinc(|t|)[t] + 1/2 sinc(|t/2|)^2 [t]^2  (pose.tpp:203-218)
// The double version fixes the summation order every implementation uses:
// (K^2)_ij = (K_i0 K_0j + K_i1 K_1j) + K_i2 K_2j.
void rotation_matrix(const double* t, double R[9])
{
    double a = sinc_d(norm3(t));
    double th[3] = { t[0] / 2.0, t[1] / 2.0, t[2] / 2.0 };
    double s = sinc_d(norm3(th));
    double b = 0.5 * s * s;
    double K[9] = { 0, -t[2], t[1], t[2], 0, -t[0], -t[1], t[0], 0 };
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double k2 = (K[3 * i] * K[j] + K[3 * i + 1] * K[3 + j])
                + K[3 * i + 2] * K[6 + j];
            double r = a * K[3 * i + j] + b * k2;
            R[3 * i + j] = i == j ? r + 1.0 : r;
        }
}

template <int N> static void rotation_matrix_ad(const D2<N> t[3], D2<N> R[9])
{
    D2<N> a = sinc_normx<N>(t);
    D2<N> th[3] = { t[0] / 2.0, t[1] / 2.0, t[2] / 2.0 };
    D2<N> s = sinc_normx<N>(th);
    D2<N> b = 0.5 * s * s;
    D2<N> zero(0.0);
    D2<N> K[9] = { zero, -t[2], t[1], t[2], zero, -t[0], -t[1], t[0], zero };
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            D2<N> k2 = (K[3 * i] * K[j] + K[3 * i + 1] * K[3 + j])
                + K[3 * i + 2] * K[6 + j];
            D2<N> r = a * K[3 * i + j] + b * k2;
            R[3 * i + j] = i == j ? r + 1.0 : r;
        }
}

// world vertex V_j = ((v0 R_j0 + v1 R_j1) + v2 R_j2) + p_j
static void world_vertex(const double* R, const double* p, const double* v, double* out)
{
    for (int j = 0; j < 3; j++)
        out[j] = ((v[0] * R[3 * j] + v[1] * R[3 * j + 1]) + v[2] * R[3 * j + 2]) + p[j];
}

void world_vertices(const Scene& s, const double* x, std::vector<double>& V)
{
    V.assign(3 * s.nv, 0.0);
    for (int b = 0; b < s.nb; b++) {
        double R[9];
        rotation_matrix(x + 6 * b + 3, R);
        for (int i = s.bvs[b]; i < s.bvs[b + 1]; i++)
            world_vertex(R, x + 6 * b, s.rest + 3 * i, &V[3 * i]);
    }
}

// RigidBody::world_vertices_diff (rigid_body.tpp:27-78) with autodiff over the
// rotation vector only; position derivatives are the identity.
void world_vertices_diff(
    const Scene& s, const double* x, std::vector<double>& V,
    std::vector<double>& dV, std::vector<double>& d2V)
{
    world_vertices(s, x, V);
    dV.assign(9 * s.nv, 0.0);
    d2V.assign(27 * s.nv, 0.0);
    // each body writes its own vertices (threads for large scenes only: the
    // time step calls this for every objective evaluation)
    parallel_for(s.nb, s.nv >= 200000 ? 4 : s.nb, [&](long long bl) {
        const int b = (int)bl;
        D2<3> t[3];
        for (int k = 0; k < 3; k++) t[k] = D2<3>::var(x[6 * b + 3 + k], k);
        D2<3> R[9];
        rotation_matrix_ad<3>(t, R);
        for (int i = s.bvs[b]; i < s.bvs[b + 1]; i++) {
            const double* v = s.rest + 3 * i;
            for (int j = 0; j < 3; j++) {
                D2<3> vj = (v[0] * R[3 * j] + v[1] * R[3 * j + 1]) + v[2] * R[3 * j + 2];
                for (int k = 0; k < 3; k++) dV[9 * i + 3 * j + k] = vj.g[k];
                for (int k = 0; k < 3; k++)
                    for (int l = 0; l < 3; l++)
                        d2V[27 * i + 9 * j + 3 * k + l] = vj.h[k][l];
            }
        }
    });
}

// ---------------------------------------------------------------------------
// distances (squared) and distance types (ipc-toolkit; IPC paper, Li et al.
// 2020).  The double versions fix the evaluation order the CUDA path uses.

static inline void sub3(const double* a, const double* b, double* r)
{
    r[0] = a[0] - b[0];
    r[1] = a[1] - b[1];
    r[2] = a[2] - b[2];
}
static inline double dot3(const double* a, const double* b)
{
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}
static inline void cross3(const double* a, const double* b, double* r)
{
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}

double point_point_sqdist(const double* p, const double* q)
{
    double d[3];
    sub3(p, q, d);
    return dot3(d, d);
}

double point_line_sqdist(const double* p, const double* e0, const double* e1)
{
    double a[3], b[3], c[3], e[3];
    sub3(e0, p, a);
    sub3(e1, p, b);
    cross3(a, b, c);
    sub3(e1, e0, e);
    return dot3(c, c) / dot3(e, e);
}

double point_plane_sqdist(const double* p, const double* t0, const double* t1, const double* t2)
{
    double a[3], b[3], n[3], w[3];
    sub3(t1, t0, a);
    sub3(t2, t0, b);
    cross3(a, b, n);
    sub3(p, t0, w);
    double u = dot3(n, w);
    return (u * u) / dot3(n, n);
}

double line_line_sqdist(const double* ea0, const double* ea1, const double* eb0, const double* eb1)
{
    double a[3], b[3], n[3], w[3];
    sub3(ea1, ea0, a);
    sub3(eb1, eb0, b);
    cross3(a, b, n);
    sub3(eb0, ea0, w);
    double u = dot3(n, w);
    return (u * u) / dot3(n, n);
}

double ee_cross_sqnorm(const double* ea0, const double* ea1, const double* eb0, const double* eb1)
{
    double a[3], b[3], n[3];
    sub3(ea1, ea0, a);
    sub3(eb1, eb0, b);
    cross3(a, b, n);
    return dot3(n, n);
}

// Closest-feature classification of a point against a triangle: project onto
// each edge's (edge, in-plane normal) frame by a 2x2 solve; see the IPC
// paper's distance-type selection.
static void edge_frame_params(const double* p, const double* a, const double* b,
                              const double* n, double& s, double& t)
{
    double e[3], m[3], w[3];
    sub3(b, a, e);
    cross3(e, n, m);
    sub3(p, a, w);
    double A00 = dot3(e, e), A01 = dot3(e, m), A11 = dot3(m, m);
    double r0 = dot3(e, w), r1 = dot3(m, w);
    double det = A00 * A11 - A01 * A01;
    s = (A11 * r0 - A01 * r1) / det;
    t = (A00 * r1 - A01 * r0) / det;
}

int point_triangle_distance_type(const double* p, const double* t0, const double* t1, const double* t2)
{
    double a[3], b[3], n[3];
    sub3(t1, t0, a);
    sub3(t2, t0, b);
    cross3(a, b, n);
    double s0, q0, s1, q1, s2, q2;
    edge_frame_params(p, t0, t1, n, s0, q0);
    if (s0 > 0.0 && s0 < 1.0 && q0 >= 0.0) return PT_P_E0;
    edge_frame_params(p, t1, t2, n, s1, q1);
    if (s1 > 0.0 && s1 < 1.0 && q1 >= 0.0) return PT_P_E1;
    edge_frame_params(p, t2, t0, n, s2, q2);
    if (s2 > 0.0 && s2 < 1.0 && q2 >= 0.0) return PT_P_E2;
    if (s0 <= 0.0 && s2 >= 1.0) return PT_P_T0;
    if (s1 <= 0.0 && s0 >= 1.0) return PT_P_T1;
    if (s2 <= 0.0 && s1 >= 1.0) return PT_P_T2;
    return PT_P_T;
}

// Segment-segment closest-feature classification (Sunday's published
// segment-segment closest-point algorithm, as the IPC distance-type selection
// uses it), with the parallel case falling back to the s = 0 end.
int edge_edge_distance_type(const double* ea0, const double* ea1, const double* eb0, const double* eb1)
{
    double u[3], v[3], w[3];
    sub3(ea1, ea0, u);
    sub3(eb1, eb0, v);
    sub3(ea0, eb0, w);
    double a = dot3(u, u), b = dot3(u, v), c = dot3(v, v);
    double d = dot3(u, w), e = dot3(v, w);
    double D = a * c - b * b;
    if (a == 0.0 && c == 0.0) return EE_EA0_EB0;
    if (a == 0.0) return EE_EA0_EB;
    if (c == 0.0) return EE_EA_EB0;

    double n[3];
    cross3(u, v, n);
    double par_tol = 1e-20 * std::max(1.0, a * c);
    int def = EE_EA_EB;
    double sN, tN, tD;
    if (dot3(n, n) < par_tol) {
        // parallel: use the s = 0 end of edge a
        sN = 0.0;
        tN = e;
        tD = c;
        def = EE_EA0_EB;
    } else {
        sN = b * e - c * d;
        if (sN <= 0.0) {
            tN = e;
            tD = c;
            def = EE_EA0_EB;
        } else if (sN >= D) {
            tN = e + b;
            tD = c;
            def = EE_EA1_EB;
        } else {
            tN = a * e - b * d;
            tD = D;
        }
    }
    if (tN <= 0.0) {
        if (-d <= 0.0) return EE_EA0_EB0;
        if (-d >= a) return EE_EA1_EB0;
        return EE_EA_EB0;
    }
    if (tN >= tD) {
        if ((-d + b) <= 0.0) return EE_EA0_EB1;
        if ((-d + b) >= a) return EE_EA1_EB1;
        return EE_EA_EB1;
    }
    return def;
}

// IPC log barrier of the squared distance: b(d) = -(d - s)^2 ln(d / s), d < s
template <class T> static T barrier_t(const T& d, double s)
{
    if (val(d) <= 0.0) return T(INFINITY);
    if (val(d) >= s) return T(0.0);
    T dm = d - s;
    using std::log;
    return -(dm * dm) * log(d / s);
}
double barrier(double d, double s) { return barrier_t<double>(d, s); }

// ---------------------------------------------------------------------------
// squared distance of two segments by their closest features
// (ipc-toolkit edge_edge_distance with the type computed)
double edge_edge_sqdist(const double* a0, const double* a1, const double* b0, const double* b1)
{
    switch (edge_edge_distance_type(a0, a1, b0, b1)) {
    case EE_EA0_EB0: return point_point_sqdist(a0, b0);
    case EE_EA0_EB1: return point_point_sqdist(a0, b1);
    case EE_EA1_EB0: return point_point_sqdist(a1, b0);
    case EE_EA1_EB1: return point_point_sqdist(a1, b1);
    case EE_EA_EB0: return point_line_sqdist(b0, a0, a1);
    case EE_EA_EB1: return point_line_sqdist(b1, a0, a1);
    case EE_EA0_EB: return point_line_sqdist(a0, b0, b1);
    case EE_EA1_EB: return point_line_sqdist(a1, b0, b1);
    default: return line_line_sqdist(a0, a1, b0, b1);
    }
}

// constraint set from candidates (ipc::construct_constraint_set as called at
// src/opt/distance_barrier_constraint.cpp:297, V_rest = V)

namespace {
struct PairKey {
    long long a, b;
    bool operator==(const PairKey& o) const { return a == o.a && b == o.b; }
};
struct PairHash {
    size_t operator()(const PairKey& k) const
    {
        return std::hash<long long>()(k.a * 1000003LL ^ k.b);
    }
};
} // namespace

void construct_constraint_set(
    const Scene& s, const Candidates& cand, const std::vector<double>& V,
    double dhat, double dmin, std::vector<Constraint>& out)
{
    const double off = (dhat + dmin) * (dhat + dmin);
    std::vector<Constraint> vv, ev, ee, fv;
    std::unordered_map<PairKey, int, PairHash> vv_idx, ev_idx;
    auto P = [&](int i) { return &V[3 * i]; };

    auto add_vv = [&](int a, int b) {
        PairKey k { std::min(a, b), std::max(a, b) };
        auto it = vv_idx.find(k);
        if (it != vv_idx.end()) {
            vv[it->second].weight += 1;
            return;
        }
        Constraint c {};
        c.type = C_VV;
        c.v[0] = a;
        c.v[1] = b;
        c.v[2] = c.v[3] = -1;
        c.prim[0] = a;
        c.prim[1] = b;
        c.body[0] = s.vbody[a];
        c.body[1] = s.vbody[b];
        c.weight = 1;
        c.eps_x = 0;
        vv_idx[k] = int(vv.size());
        vv.push_back(c);
    };
    auto add_ev = [&](int e, int v) {
        PairKey k { e, v };
        auto it = ev_idx.find(k);
        if (it != ev_idx.end()) {
            ev[it->second].weight += 1;
            return;
        }
        Constraint c {};
        c.type = C_EV;
        c.v[0] = v;
        c.v[1] = s.edges[2 * e];
        c.v[2] = s.edges[2 * e + 1];
        c.v[3] = -1;
        c.prim[0] = e;
        c.prim[1] = v;
        c.body[0] = s.vbody[v];
        c.body[1] = s.ebody[e];
        c.weight = 1;
        c.eps_x = 0;
        ev_idx[k] = int(ev.size());
        ev.push_back(c);
    };

    for (const auto& c : cand.ee) {
        int ea = c[0], eb = c[1];
        int a0 = s.edges[2 * ea], a1 = s.edges[2 * ea + 1];
        int b0 = s.edges[2 * eb], b1 = s.edges[2 * eb + 1];
        int t = edge_edge_distance_type(P(a0), P(a1), P(b0), P(b1));
        double d;
        switch (t) {
        case EE_EA0_EB0: d = point_point_sqdist(P(a0), P(b0)); break;
        case EE_EA0_EB1: d = point_point_sqdist(P(a0), P(b1)); break;
        case EE_EA1_EB0: d = point_point_sqdist(P(a1), P(b0)); break;
        case EE_EA1_EB1: d = point_point_sqdist(P(a1), P(b1)); break;
        case EE_EA_EB0: d = point_line_sqdist(P(b0), P(a0), P(a1)); break;
        case EE_EA_EB1: d = point_line_sqdist(P(b1), P(a0), P(a1)); break;
        case EE_EA0_EB: d = point_line_sqdist(P(a0), P(b0), P(b1)); break;
        case EE_EA1_EB: d = point_line_sqdist(P(a1), P(b0), P(b1)); break;
        default: d = line_line_sqdist(P(a0), P(a1), P(b0), P(b1)); break;
        }
        if (!(d < off)) continue;
        // mollifier threshold eps_x = 1e-3 |ea|^2 |eb|^2 with V_rest = V
        double ua[3], ub[3];
        sub3(P(a0), P(a1), ua);
        sub3(P(b0), P(b1), ub);
        double eps_x = 1e-3 * dot3(ua, ua) * dot3(ub, ub);
        if (ee_cross_sqnorm(P(a0), P(a1), P(b0), P(b1)) < eps_x) t = EE_EA_EB;
        switch (t) {
        case EE_EA0_EB0: add_vv(a0, b0); break;
        case EE_EA0_EB1: add_vv(a0, b1); break;
        case EE_EA1_EB0: add_vv(a1, b0); break;
        case EE_EA1_EB1: add_vv(a1, b1); break;
        case EE_EA_EB0: add_ev(ea, b0); break;
        case EE_EA_EB1: add_ev(ea, b1); break;
        case EE_EA0_EB: add_ev(eb, a0); break;
        case EE_EA1_EB: add_ev(eb, a1); break;
        default: {
            Constraint k {};
            k.type = C_EE;
            k.v[0] = a0;
            k.v[1] = a1;
            k.v[2] = b0;
            k.v[3] = b1;
            k.prim[0] = ea;
            k.prim[1] = eb;
            k.body[0] = s.ebody[ea];
            k.body[1] = s.ebody[eb];
            k.weight = 1;
            k.eps_x = eps_x;
            ee.push_back(k);
        }
        }
    }
    for (const auto& c : cand.fv) {
        int f = c[0], v = c[1];
        int f0 = s.faces[3 * f], f1 = s.faces[3 * f + 1], f2 = s.faces[3 * f + 2];
        int t = point_triangle_distance_type(P(v), P(f0), P(f1), P(f2));
        double d;
        switch (t) {
        case PT_P_T0: d = point_point_sqdist(P(v), P(f0)); break;
        case PT_P_T1: d = point_point_sqdist(P(v), P(f1)); break;
        case PT_P_T2: d = point_point_sqdist(P(v), P(f2)); break;
        case PT_P_E0: d = point_line_sqdist(P(v), P(f0), P(f1)); break;
        case PT_P_E1: d = point_line_sqdist(P(v), P(f1), P(f2)); break;
        case PT_P_E2: d = point_line_sqdist(P(v), P(f2), P(f0)); break;
        default: d = point_plane_sqdist(P(v), P(f0), P(f1), P(f2)); break;
        }
        if (!(d < off)) continue;
        switch (t) {
        case PT_P_T0: add_vv(v, f0); break;
        case PT_P_T1: add_vv(v, f1); break;
        case PT_P_T2: add_vv(v, f2); break;
        case PT_P_E0: add_ev(s.f2e[3 * f + 0], v); break;
        case PT_P_E1: add_ev(s.f2e[3 * f + 1], v); break;
        case PT_P_E2: add_ev(s.f2e[3 * f + 2], v); break;
        default: {
            Constraint k {};
            k.type = C_FV;
            k.v[0] = v;
            k.v[1] = f0;
            k.v[2] = f1;
            k.v[3] = f2;
            k.prim[0] = f;
            k.prim[1] = v;
            k.body[0] = s.vbody[v];
            k.body[1] = s.fbody[f];
            k.weight = 1;
            k.eps_x = 0;
            fv.push_back(k);
        }
        }
    }
    out.clear();
    out.insert(out.end(), vv.begin(), vv.end());
    out.insert(out.end(), ev.begin(), ev.end());
    out.insert(out.end(), ee.begin(), ee.end());
    out.insert(out.end(), fv.begin(), fv.end());
}

// ---------------------------------------------------------------------------
// symmetric eigen-decomposition by cyclic Jacobi rotations (a published
// method), used for the PSD projection: if the smallest eigenvalue is >= 0
// the matrix is returned unchanged, otherwise V max(D, 0) V^T.

static void jacobi_eigen(int n, double* A, double* Vm, double* w)
{
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) Vm[i * n + j] = i == j ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0, diag = 0;
        for (int i = 0; i < n; i++) {
            diag += A[i * n + i] * A[i * n + i];
            for (int j = i + 1; j < n; j++) off += A[i * n + j] * A[i * n + j];
        }
        if (off <= 1e-32 * diag || off == 0.0) break;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) {
                double apq = A[p * n + q];
                if (apq == 0.0) continue;
                double app = A[p * n + p], aqq = A[q * n + q];
                double theta = (aqq - app) / (2 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0)
                    / (std::fabs(theta) + std::sqrt(theta * theta + 1));
                double c = 1 / std::sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < n; k++) {
                    double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; k++) {
                    double vkp = Vm[k * n + p], vkq = Vm[k * n + q];
                    Vm[k * n + p] = c * vkp - s * vkq;
                    Vm[k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < n; i++) w[i] = A[i * n + i];
}

void project_to_psd(int n, const double* A, double* out)
{
    std::vector<double> B(A, A + n * n), Vm(n * n), w(n);
    // symmetrise exactly (the input is symmetric up to rounding)
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++) {
            double m = 0.5 * (B[i * n + j] + B[j * n + i]);
            B[i * n + j] = B[j * n + i] = m;
        }
    jacobi_eigen(n, B.data(), Vm.data(), w.data());
    double wmin = *std::min_element(w.begin(), w.end());
    if (wmin >= 0.0) {
        std::copy(A, A + n * n, out);
        return;
    }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            double acc = 0;
            for (int k = 0; k < n; k++)
                if (w[k] > 0) acc += Vm[i * n + k] * w[k] * Vm[j * n + k];
            out[i * n + j] = acc;
        }
}

// ---------------------------------------------------------------------------
// per-constraint potential with autodiff over the 12 vertex coordinates
// (constraint.compute_potential/_gradient/_hessian as called at
// distance_barrier_rb_problem.cpp:1350-1369), then apply_chain_rule
// (:1182-1248) with the PSD projection of the 12x12 body-space Hessian.

using AD = D2<12>;

static void ad_sub(const AD* a, const AD* b, AD* r)
{
    for (int i = 0; i < 3; i++) r[i] = a[i] - b[i];
}
static AD ad_dot(const AD* a, const AD* b)
{
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}
static void ad_cross(const AD* a, const AD* b, AD* r)
{
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}

static AD constraint_potential_ad(const Constraint& c, const AD X[4][3], double dhat, double dmin)
{
    AD d;
    switch (c.type) {
    case C_VV: {
        AD w[3];
        ad_sub(X[0], X[1], w);
        d = ad_dot(w, w);
        break;
    }
    case C_EV: {
        AD a[3], b[3], n[3], e[3];
        ad_sub(X[1], X[0], a);
        ad_sub(X[2], X[0], b);
        ad_cross(a, b, n);
        ad_sub(X[2], X[1], e);
        d = ad_dot(n, n) / ad_dot(e, e);
        break;
    }
    case C_EE: {
        // the closest-feature distance of the two segments: near-parallel
        // pairs whose closest points are endpoints are kept as (mollified)
        // EE constraints, so the type is taken at the current positions
        // (ipc-toolkit EdgeEdgeConstraint: "the distance type is unknown")
        double P[4][3];
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 3; j++) P[i][j] = X[i][j].v;
        const int t = edge_edge_distance_type(P[0], P[1], P[2], P[3]);
        auto pp = [&](int i, int j) {
            AD w[3];
            ad_sub(X[i], X[j], w);
            return ad_dot(w, w);
        };
        auto pl = [&](int p, int e0, int e1) {
            AD a[3], b[3], n[3], e[3];
            ad_sub(X[e0], X[p], a);
            ad_sub(X[e1], X[p], b);
            ad_cross(a, b, n);
            ad_sub(X[e1], X[e0], e);
            return ad_dot(n, n) / ad_dot(e, e);
        };
        switch (t) {
        case EE_EA0_EB0: d = pp(0, 2); break;
        case EE_EA0_EB1: d = pp(0, 3); break;
        case EE_EA1_EB0: d = pp(1, 2); break;
        case EE_EA1_EB1: d = pp(1, 3); break;
        case EE_EA_EB0: d = pl(2, 0, 1); break;
        case EE_EA_EB1: d = pl(3, 0, 1); break;
        case EE_EA0_EB: d = pl(0, 2, 3); break;
        case EE_EA1_EB: d = pl(1, 2, 3); break;
        default: {
            AD a[3], b[3], n[3], w[3];
            ad_sub(X[1], X[0], a);
            ad_sub(X[3], X[2], b);
            ad_cross(a, b, n);
            ad_sub(X[2], X[0], w);
            AD u = ad_dot(n, w);
            d = (u * u) / ad_dot(n, n);
        }
        }
        break;
    }
    default: {
        AD a[3], b[3], n[3], w[3];
        ad_sub(X[2], X[1], a);
        ad_sub(X[3], X[1], b);
        ad_cross(a, b, n);
        ad_sub(X[0], X[1], w);
        AD u = ad_dot(n, w);
        d = (u * u) / ad_dot(n, n);
        break;
    }
    }
    // distance_barrier: shift by dmin^2, s = 2 dmin dhat + dhat^2
    // (src/opt/distance_barrier_constraint.tpp:11-17)
    AD f = barrier_t<AD>(d - dmin * dmin, 2 * dmin * dhat + dhat * dhat);
    if (c.type == C_EE) {
        // EE mollifier m(x) = (-x/eps + 2) x/eps for x < eps
        AD a[3], b[3], n[3];
        ad_sub(X[1], X[0], a);
        ad_sub(X[3], X[2], b);
        ad_cross(a, b, n);
        AD x = ad_dot(n, n);
        if (x.v < c.eps_x) {
            AD xe = x / c.eps_x;
            AD m = (2.0 - xe) * xe;
            f = m * f;
        }
    }
    return c.weight * f;
}

void constraint_local_term(
    const Scene& s, const Constraint& c, const std::vector<double>& V,
    const std::vector<double>& dV, const std::vector<double>& d2V,
    double dhat, double dmin, bool project, LocalTerm& out)
{
    const int nvc = c.nverts();
    AD X[4][3];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 3; j++) {
            if (i < nvc) X[i][j] = AD::var(V[3 * c.v[i] + j], 3 * i + j);
            else X[i][j] = AD(0.0);
        }
    AD f = constraint_potential_ad(c, X, dhat, dmin);
    out.energy = f.v;
    // body-space Jacobian of each vertex: dV_i/dx_body = [I | dV/dtheta]
    double J[12][12] = {};
    for (int i = 0; i < nvc; i++) {
        int lb = local_body(c.type, i);
        int vi = c.v[i];
        for (int j = 0; j < 3; j++) {
            J[3 * i + j][6 * lb + j] = 1.0;
            for (int k = 0; k < 3; k++)
                J[3 * i + j][6 * lb + 3 + k] = dV[9 * vi + 3 * j + k];
        }
    }
    for (int a = 0; a < 12; a++) {
        double acc = 0;
        for (int r = 0; r < 12; r++) acc += J[r][a] * f.g[r];
        out.grad[a] = acc;
    }
    double H[144];
    for (int a = 0; a < 12; a++)
        for (int b = 0; b < 12; b++) {
            double acc = 0;
            for (int r = 0; r < 12; r++) {
                if (J[r][a] == 0.0) continue;
                for (int q = 0; q < 12; q++) acc += J[r][a] * f.h[r][q] * J[q][b];
            }
            H[12 * a + b] = acc;
        }
    // + sum_ij grad_f[ij] * d2V_ij/dtheta2 on the body's rotation block
    for (int i = 0; i < nvc; i++) {
        int lb = local_body(c.type, i);
        int vi = c.v[i];
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++)
                for (int l = 0; l < 3; l++)
                    H[12 * (6 * lb + 3 + k) + 6 * lb + 3 + l] +=
                        f.g[3 * i + j] * d2V[27 * vi + 9 * j + 3 * k + l];
    }
    if (project) project_to_psd(12, H, out.hess);
    else std::copy(H, H + 144, out.hess);
}

double barrier_term(
    const Scene& s, const double* x, const std::vector<Constraint>& cs,
    double dhat, double dmin, std::vector<double>& grad, BSR& hess, bool project)
{
    std::vector<double> V, dV, d2V;
    world_vertices_diff(s, x, V, dV, d2V);
    grad.assign(6 * s.nb, 0.0);
    std::map<std::pair<int, int>, std::array<double, 36>> blocks;
    double energy = 0;
    // the constraints' local terms over the host's threads, then summed in
    // constraint order
    std::vector<LocalTerm> terms(cs.size());
    parallel_for((long long)cs.size(), cs.size() >= 512 ? 16 : (long long)cs.size(), [&](long long i) {
        constraint_local_term(s, cs[i], V, dV, d2V, dhat, dmin, project, terms[i]);
    });
    for (size_t ci = 0; ci < cs.size(); ci++) {
        const Constraint& c = cs[ci];
        const LocalTerm& t = terms[ci];
        energy += t.energy;
        for (int lb = 0; lb < 2; lb++)
            for (int k = 0; k < 6; k++) grad[6 * c.body[lb] + k] += t.grad[6 * lb + k];
        for (int bi = 0; bi < 2; bi++)
            for (int bj = 0; bj < 2; bj++) {
                auto key = std::make_pair(c.body[bi], c.body[bj]);
                auto it = blocks.find(key);
                if (it == blocks.end()) {
                    std::array<double, 36> z {};
                    it = blocks.emplace(key, z).first;
                }
                for (int r = 0; r < 6; r++)
                    for (int q = 0; q < 6; q++)
                        it->second[6 * r + q] += t.hess[12 * (6 * bi + r) + 6 * bj + q];
            }
    }
    hess.row_ptr.assign(s.nb + 1, 0);
    hess.col.clear();
    hess.val.clear();
    for (const auto& kv : blocks) hess.row_ptr[kv.first.first + 1]++;
    for (int i = 0; i < s.nb; i++) hess.row_ptr[i + 1] += hess.row_ptr[i];
    for (const auto& kv : blocks) {
        hess.col.push_back(kv.first.second);
        hess.val.insert(hess.val.end(), kv.second.begin(), kv.second.end());
    }
    return energy;
}

// ---------------------------------------------------------------------------
// body energy with implicit Euler (the default integration,
// distance_barrier_rb_problem.hpp:26), autodiff over the 6 body dofs.
double body_energy(
    const BodyState& b, const double* x6, const double gravity[3], double h,
    double grad[6], double hess[36])
{
    using A6 = D2<6>;
    A6 q[6];
    for (int i = 0; i < 6; i++) q[i] = A6::var(x6[i], i);
    A6 e(0.0);
    bool pos_fixed = b.fixed[0] && b.fixed[1] && b.fixed[2];
    bool rot_fixed = b.fixed[3] && b.fixed[4] && b.fixed[5];
    if (b.type == 2) {
        if (!pos_fixed) {
            // 1/2 m q.q - m q.(q_t0 + h (qdot_t0 + h g))
            A6 qq = (q[0] * q[0] + q[1] * q[1]) + q[2] * q[2];
            double hat[3];
            for (int i = 0; i < 3; i++)
                hat[i] = b.pose_t0[i] + h * (b.vel_t0[i] + h * gravity[i]);
            A6 qh = (q[0] * hat[0] + q[1] * hat[1]) + q[2] * hat[2];
            e = e + 0.5 * b.mass * qq - b.mass * qh;
        }
        if (!rot_fixed) {
            A6 Q[9];
            rotation_matrix_ad<6>(q + 3, Q);
            double Q0[9];
            rotation_matrix(b.pose_t0 + 3, Q0);
            double J[3] = { 0.5 * (-b.moment[0] + b.moment[1] + b.moment[2]),
                            0.5 * (b.moment[0] - b.moment[1] + b.moment[2]),
                            0.5 * (b.moment[0] + b.moment[1] - b.moment[2]) };
            // 1/2 tr(Q J Q^T) - tr(Q J (Q0 + h Qdot0)^T)
            A6 t1(0.0), t2(0.0);
            for (int i = 0; i < 3; i++)
                for (int k = 0; k < 3; k++) {
                    t1 = t1 + J[k] * (Q[3 * i + k] * Q[3 * i + k]);
                    double tk = Q0[3 * i + k] + h * b.Qdot[3 * i + k];
                    t2 = t2 + (J[k] * tk) * Q[3 * i + k];
                }
            e = e + 0.5 * t1 - t2;
        }
    }
    for (int i = 0; i < 6; i++) grad[i] = e.g[i];
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < 6; j++) hess[6 * i + j] = e.h[i][j];
    // project the position block (distance_barrier_rb_problem.cpp:767-768);
    // it is m I here, already PSD
    return e.v;
}

// The same energy over 24 variables: the pose x6 (0-5), the start-of-step
// pose (6-11), linear velocity (12-14) and Qdot (15-23), for the adjoint of
// a time step (its mixed block d2E / dx ds and the Hessian at x = pose_t0).
void body_energy_state_derivs(
    const BodyState& b, const double* x6, const double gravity[3], double h,
    double grad[24], double hess[576])
{
    using A = D2<24>;
    A q[6], q0[6], v0[3], Qd[9];
    for (int i = 0; i < 6; i++) q[i] = A::var(x6[i], i);
    for (int i = 0; i < 6; i++) q0[i] = A::var(b.pose_t0[i], 6 + i);
    for (int i = 0; i < 3; i++) v0[i] = A::var(b.vel_t0[i], 12 + i);
    for (int i = 0; i < 9; i++) Qd[i] = A::var(b.Qdot[i], 15 + i);
    A e(0.0);
    bool pos_fixed = b.fixed[0] && b.fixed[1] && b.fixed[2];
    bool rot_fixed = b.fixed[3] && b.fixed[4] && b.fixed[5];
    if (b.type == 2) {
        if (!pos_fixed)
            for (int i = 0; i < 3; i++) {
                A hat = q0[i] + h * (v0[i] + h * gravity[i]);
                e = e + 0.5 * b.mass * (q[i] * q[i]) - b.mass * (q[i] * hat);
            }
        if (!rot_fixed) {
            A Q[9], Q0[9];
            rotation_matrix_ad<24>(q + 3, Q);
            rotation_matrix_ad<24>(q0 + 3, Q0);
            double J[3] = { 0.5 * (-b.moment[0] + b.moment[1] + b.moment[2]),
                            0.5 * (b.moment[0] - b.moment[1] + b.moment[2]),
                            0.5 * (b.moment[0] + b.moment[1] - b.moment[2]) };
            for (int i = 0; i < 3; i++)
                for (int k = 0; k < 3; k++) {
                    A t = Q0[3 * i + k] + h * Qd[3 * i + k];
                    e = e + J[k] * (0.5 * (Q[3 * i + k] * Q[3 * i + k]) - Q[3 * i + k] * t);
                }
        }
    }
    for (int i = 0; i < 24; i++) grad[i] = e.g[i];
    for (int i = 0; i < 24; i++)
        for (int j = 0; j < 24; j++) hess[24 * i + j] = e.h[i][j];
}

void rotation_matrix_hessian(const double* theta, double d2R[81])
{
    D2<3> t[3], R[9];
    for (int i = 0; i < 3; i++) t[i] = D2<3>::var(theta[i], i);
    rotation_matrix_ad<3>(t, R);
    for (int a = 0; a < 3; a++)
        for (int c = 0; c < 3; c++)
            for (int k = 0; k < 9; k++) d2R[27 * a + 9 * c + k] = R[k].h[a][c];
}

void rotation_matrix_jacobian(const double* theta, double dR[27])
{
    D2<3> t[3], R[9];
    for (int i = 0; i < 3; i++) t[i] = D2<3>::var(theta[i], i);
    rotation_matrix_ad<3>(t, R);
    for (int a = 0; a < 3; a++)
        for (int k = 0; k < 9; k++) dR[9 * a + k] = R[k].g[a];
}


// ---------------------------------------------------------------------------
// lagged friction (IPC paper, Li et al. 2020 sec. 5, as ipc-toolkit provides
// it to compute_friction_term, distance_barrier_rb_problem.cpp:1410-1572):
// per collision constraint at the start of the step, a normal force
// magnitude lambda = -kappa w b'(d - dmin^2) 2 sqrt(d), closest-point weights
// Gamma (3 x 3n blocks) and an orthonormal tangent basis T (3 x 2) of the
// contact plane; D = mu lambda f0(|T^T Gamma (X - X0)|) with the mollified
// f0 of eps_v h.

namespace {
void normalize3(double* v)
{
    double n = std::sqrt(dot3(v, v));
    for (int i = 0; i < 3; i++) v[i] /= n;
}
// two orthonormal vectors spanning the plane orthogonal to n
void basis_from_normal(const double* n_in, double* t1, double* t2)
{
    double n[3] = { n_in[0], n_in[1], n_in[2] };
    normalize3(n);
    double ax[3] = { 1, 0, 0 };
    if (std::fabs(n[0]) > 0.9) { ax[0] = 0; ax[1] = 1; }
    cross3(n, ax, t1);
    normalize3(t1);
    cross3(n, t1, t2);
}
// barrier derivative of the shifted squared distance
double barrier_gradient_d(double d, double s)
{
    if (d <= 0.0 || d >= s) return 0.0;
    return (s - d) * (2 * std::log(d / s) - s / d + 1);
}
} // namespace

void construct_friction_constraints(
    const Scene& s, const std::vector<Constraint>& cs, const std::vector<double>& V0,
    double dhat, double dmin, double kappa, std::vector<FrictionConstraint>& out)
{
    out.clear();
    auto P = [&](int i) { return &V0[3 * i]; };
    const double sb = 2 * dmin * dhat + dhat * dhat;
    for (const auto& c : cs) {
        FrictionConstraint f;
        f.c = c;
        f.p0 = f.p1 = 0;
        double d = 0, n[3], t1[3], t2[3];
        switch (c.type) {
        case C_VV: {
            sub3(P(c.v[0]), P(c.v[1]), n);
            d = dot3(n, n);
            basis_from_normal(n, t1, t2);
            break;
        }
        case C_EV: {
            const double *p = P(c.v[0]), *e0 = P(c.v[1]), *e1 = P(c.v[2]);
            double e[3], w[3];
            sub3(e1, e0, e);
            sub3(p, e0, w);
            f.p0 = dot3(e, w) / dot3(e, e);
            d = point_line_sqdist(p, e0, e1);
            double c3[3];
            for (int i = 0; i < 3; i++) n[i] = w[i] - f.p0 * e[i];
            for (int i = 0; i < 3; i++) t1[i] = e[i];
            normalize3(t1);
            cross3(e, n, c3);
            for (int i = 0; i < 3; i++) t2[i] = c3[i];
            normalize3(t2);
            break;
        }
        case C_EE: {
            const double *a0 = P(c.v[0]), *a1 = P(c.v[1]), *b0 = P(c.v[2]), *b1 = P(c.v[3]);
            double a[3], b[3], w[3];
            sub3(a1, a0, a);
            sub3(b1, b0, b);
            sub3(b0, a0, w);
            // minimise |a0 + alpha a - b0 - beta b|^2
            double aa = dot3(a, a), ab = dot3(a, b), bb = dot3(b, b), aw = dot3(a, w), bw = dot3(b, w);
            double det = aa * bb - ab * ab;
            f.p0 = (aw * bb - ab * bw) / det;
            f.p1 = (aw * ab - aa * bw) / det;
            d = edge_edge_sqdist(a0, a1, b0, b1);
            cross3(a, b, n);
            for (int i = 0; i < 3; i++) t1[i] = a[i];
            normalize3(t1);
            double nn[3] = { n[0], n[1], n[2] };
            normalize3(nn);
            cross3(nn, t1, t2);
            break;
        }
        default: {
            const double *p = P(c.v[0]), *q0 = P(c.v[1]), *q1 = P(c.v[2]), *q2 = P(c.v[3]);
            double e1[3], e2[3], w[3];
            sub3(q1, q0, e1);
            sub3(q2, q0, e2);
            sub3(p, q0, w);
            double a11 = dot3(e1, e1), a12 = dot3(e1, e2), a22 = dot3(e2, e2);
            double r1 = dot3(e1, w), r2 = dot3(e2, w);
            double det = a11 * a22 - a12 * a12;
            f.p0 = (a22 * r1 - a12 * r2) / det;
            f.p1 = (a11 * r2 - a12 * r1) / det;
            d = point_plane_sqdist(p, q0, q1, q2);
            cross3(e1, e2, n);
            for (int i = 0; i < 3; i++) t1[i] = e1[i];
            normalize3(t1);
            double nn[3] = { n[0], n[1], n[2] };
            normalize3(nn);
            cross3(nn, t1, t2);
            break;
        }
        }
        f.lambda = -kappa * c.weight * barrier_gradient_d(d - dmin * dmin, sb) * 2 * std::sqrt(d);
        for (int i = 0; i < 3; i++) {
            f.T[i] = t1[i];
            f.T[3 + i] = t2[i];
        }
        out.push_back(f);
    }
}

// closest-point weights of the relative displacement: Delta = sum_i g_i U_i
static void friction_weights(const FrictionConstraint& f, double g[4])
{
    switch (f.c.type) {
    case C_VV: g[0] = 1; g[1] = -1; g[2] = g[3] = 0; break;
    case C_EV: g[0] = 1; g[1] = -(1 - f.p0); g[2] = -f.p0; g[3] = 0; break;
    case C_EE: g[0] = 1 - f.p0; g[1] = f.p0; g[2] = -(1 - f.p1); g[3] = -f.p1; break;
    default: g[0] = 1; g[1] = -(1 - f.p0 - f.p1); g[2] = -f.p0; g[3] = -f.p1; break;
    }
}

void friction_local_term(
    const Scene& s, const FrictionConstraint& f, const std::vector<double>& V,
    const std::vector<double>& V0, const std::vector<double>& dV,
    const std::vector<double>& d2V, double mu, double epsvh, bool project, LocalTerm& out)
{
    const Constraint& c = f.c;
    const int nvc = c.nverts();
    double g[4];
    friction_weights(f, g);
    // A (2 x 12) = T^T Gamma
    double A[2][12] = {};
    for (int i = 0; i < nvc; i++)
        for (int r = 0; r < 2; r++)
            for (int j = 0; j < 3; j++) A[r][3 * i + j] = g[i] * f.T[3 * r + j];
    double u[2] = { 0, 0 };
    for (int i = 0; i < nvc; i++)
        for (int j = 0; j < 3; j++) {
            double Uij = V[3 * c.v[i] + j] - V0[3 * c.v[i] + j];
            u[0] += A[0][3 * i + j] * Uij;
            u[1] += A[1][3 * i + j] * Uij;
        }
    double x = std::sqrt(u[0] * u[0] + u[1] * u[1]);
    const double ml = mu * f.lambda;
    double f0, f1_over_x, hu[2][2];
    if (x >= epsvh) {
        f0 = x;
        f1_over_x = 1 / x;
        for (int a = 0; a < 2; a++)
            for (int b = 0; b < 2; b++)
                hu[a][b] = -u[a] * u[b] / (x * x * x) + (a == b ? 1 / x : 0.0);
    } else {
        f0 = -x * x * x / (3 * epsvh * epsvh) + x * x / epsvh + epsvh / 3;
        f1_over_x = 2 / epsvh - x / (epsvh * epsvh);
        for (int a = 0; a < 2; a++)
            for (int b = 0; b < 2; b++)
                hu[a][b] = (x > 0 ? -u[a] * u[b] / (epsvh * epsvh * x) : 0.0)
                    + (a == b ? f1_over_x : 0.0);
    }
    out.energy = ml * f0;
    double gx[12] = {};
    for (int k = 0; k < 12; k++) gx[k] = ml * f1_over_x * (A[0][k] * u[0] + A[1][k] * u[1]);
    double Hx[12][12];
    for (int k = 0; k < 12; k++)
        for (int l = 0; l < 12; l++) {
            double acc = 0;
            for (int a = 0; a < 2; a++)
                for (int b = 0; b < 2; b++) acc += A[a][k] * hu[a][b] * A[b][l];
            Hx[k][l] = ml * acc;
        }
    // rigid chain rule (apply_chain_rule)
    double J[12][12] = {};
    for (int i = 0; i < nvc; i++) {
        int lb = local_body(c.type, i);
        int vi = c.v[i];
        for (int j = 0; j < 3; j++) {
            J[3 * i + j][6 * lb + j] = 1.0;
            for (int k = 0; k < 3; k++) J[3 * i + j][6 * lb + 3 + k] = dV[9 * vi + 3 * j + k];
        }
    }
    for (int a = 0; a < 12; a++) {
        double acc = 0;
        for (int r = 0; r < 12; r++) acc += J[r][a] * gx[r];
        out.grad[a] = acc;
    }
    double H[144];
    for (int a = 0; a < 12; a++)
        for (int b = 0; b < 12; b++) {
            double acc = 0;
            for (int r = 0; r < 12; r++) {
                if (J[r][a] == 0.0) continue;
                for (int q = 0; q < 12; q++) acc += J[r][a] * Hx[r][q] * J[q][b];
            }
            H[12 * a + b] = acc;
        }
    for (int i = 0; i < nvc; i++) {
        int lb = local_body(c.type, i);
        int vi = c.v[i];
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++)
                for (int l = 0; l < 3; l++)
                    H[12 * (6 * lb + 3 + k) + 6 * lb + 3 + l] += gx[3 * i + j] * d2V[27 * vi + 9 * j + 3 * k + l];
    }
    if (project) project_to_psd(12, H, out.hess);
    else std::copy(H, H + 144, out.hess);
}

// assembled friction term (compute_friction_term,
// distance_barrier_rb_problem.cpp:1469-1572): U = V(x) - V(x_t0)
double friction_term(
    const Scene& s, const double* x, const double* x0, const std::vector<FrictionConstraint>& fcs,
    double mu, double epsvh, std::vector<double>& grad, BSR& hess, bool project)
{
    std::vector<double> V, dV, d2V, V0;
    world_vertices_diff(s, x, V, dV, d2V);
    world_vertices(s, x0, V0);
    grad.assign(6 * s.nb, 0.0);
    std::map<std::pair<int, int>, std::array<double, 36>> blocks;
    double energy = 0;
    for (const auto& f : fcs) {
        LocalTerm t;
        friction_local_term(s, f, V, V0, dV, d2V, mu, epsvh, project, t);
        energy += t.energy;
        for (int lb = 0; lb < 2; lb++)
            for (int k = 0; k < 6; k++) grad[6 * f.c.body[lb] + k] += t.grad[6 * lb + k];
        for (int bi = 0; bi < 2; bi++)
            for (int bj = 0; bj < 2; bj++) {
                auto key = std::make_pair(f.c.body[bi], f.c.body[bj]);
                auto it = blocks.find(key);
                if (it == blocks.end()) {
                    std::array<double, 36> z {};
                    it = blocks.emplace(key, z).first;
                }
                for (int r = 0; r < 6; r++)
                    for (int q = 0; q < 6; q++)
                        it->second[6 * r + q] += t.hess[12 * (6 * bi + r) + 6 * bj + q];
            }
    }
    hess.row_ptr.assign(s.nb + 1, 0);
    hess.col.clear();
    hess.val.clear();
    for (const auto& kv : blocks) hess.row_ptr[kv.first.first + 1]++;
    for (int i = 0; i < s.nb; i++) hess.row_ptr[i + 1] += hess.row_ptr[i];
    for (const auto& kv : blocks) {
        hess.col.push_back(kv.first.second);
        hess.val.insert(hess.val.end(), kv.second.begin(), kv.second.end());
    }
    return energy;
}

// barrier energy only (the value of compute_barrier_term), in doubles
double barrier_energy(const Scene& s, const double* x, const std::vector<Constraint>& cs,
                      double dhat, double dmin)
{
    std::vector<double> V;
    world_vertices(s, x, V);
    auto P = [&](int i) { return &V[3 * i]; };
    double e = 0;
    for (const auto& c : cs) {
        double d;
        switch (c.type) {
        case C_VV: d = point_point_sqdist(P(c.v[0]), P(c.v[1])); break;
        case C_EV: d = point_line_sqdist(P(c.v[0]), P(c.v[1]), P(c.v[2])); break;
        case C_EE: d = edge_edge_sqdist(P(c.v[0]), P(c.v[1]), P(c.v[2]), P(c.v[3])); break;
        default: d = point_plane_sqdist(P(c.v[0]), P(c.v[1]), P(c.v[2]), P(c.v[3])); break;
        }
        double f = barrier_t<double>(d - dmin * dmin, 2 * dmin * dhat + dhat * dhat);
        if (c.type == C_EE) {
            double x2 = ee_cross_sqnorm(P(c.v[0]), P(c.v[1]), P(c.v[2]), P(c.v[3]));
            if (x2 < c.eps_x) {
                double xe = x2 / c.eps_x;
                f = ((2.0 - xe) * xe) * f;
            }
        }
        e += c.weight * f;
    }
    return e;
}

} // namespace orc
