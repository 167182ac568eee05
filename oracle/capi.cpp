// C entry points of the oracle for the Python test harness (test
// infrastructure only; never linked into the product library).
#include "interval.hpp"
#include "oracle.hpp"

#include <cmath>
#include <cstring>
#include <memory>

using namespace orc;

namespace orc {
I isinc(const I& x);
void irotation(const I r[3], I R[9]);
}

namespace {
struct OwnedScene {
    Scene s;
    std::vector<double> rest, rmax;
    std::vector<int> edges, faces, f2e, bvs, bes, bfs, group, type;
};

std::vector<Constraint> unpack_constraints(
    long long n, const int* types, const int* verts, const int* prims,
    const int* bodies, const double* weight, const double* eps)
{
    std::vector<Constraint> cs(n);
    for (long long i = 0; i < n; i++) {
        Constraint& c = cs[i];
        c.type = types[i];
        for (int k = 0; k < 4; k++) c.v[k] = verts[4 * i + k];
        c.prim[0] = prims[2 * i];
        c.prim[1] = prims[2 * i + 1];
        c.body[0] = bodies[2 * i];
        c.body[1] = bodies[2 * i + 1];
        c.weight = weight[i];
        c.eps_x = eps[i];
    }
    return cs;
}

Candidates pack_candidates(const int* ee, long long nee, const int* fv, long long nfv)
{
    Candidates c;
    c.ee.resize(nee);
    c.fv.resize(nfv);
    for (long long i = 0; i < nee; i++) c.ee[i] = { ee[2 * i], ee[2 * i + 1] };
    for (long long i = 0; i < nfv; i++) c.fv[i] = { fv[2 * i], fv[2 * i + 1] };
    return c;
}
} // namespace

extern "C" {

void* orc_scene_new(
    int nb, int nv, int ne, int nf, const double* rest, const int* edges,
    const int* faces, const int* f2e, const int* bvs, const int* bes,
    const int* bfs, const int* group, const int* type, const double* rmax,
    double avg_edge_len)
{
    auto* o = new OwnedScene;
    o->rest.assign(rest, rest + 3 * nv);
    o->edges.assign(edges, edges + 2 * ne);
    o->faces.assign(faces, faces + 3 * nf);
    o->f2e.assign(f2e, f2e + 3 * nf);
    o->bvs.assign(bvs, bvs + nb + 1);
    o->bes.assign(bes, bes + nb + 1);
    o->bfs.assign(bfs, bfs + nb + 1);
    o->group.assign(group, group + nb);
    o->type.assign(type, type + nb);
    o->rmax.assign(rmax, rmax + nb);
    Scene& s = o->s;
    s.nb = nb;
    s.nv = nv;
    s.ne = ne;
    s.nf = nf;
    s.rest = o->rest.data();
    s.edges = o->edges.data();
    s.faces = o->faces.data();
    s.f2e = o->f2e.data();
    s.bvs = o->bvs.data();
    s.bes = o->bes.data();
    s.bfs = o->bfs.data();
    s.group = o->group.data();
    s.type = o->type.data();
    s.rmax = o->rmax.data();
    s.avg_edge_len = avg_edge_len;
    s.finalize();
    return o;
}

void orc_scene_free(void* p) { delete static_cast<OwnedScene*>(p); }

void orc_rotation_matrix(const double* theta, double* R) { rotation_matrix(theta, R); }

void orc_world_vertices(void* p, const double* x, double* V)
{
    std::vector<double> v;
    world_vertices(static_cast<OwnedScene*>(p)->s, x, v);
    std::memcpy(V, v.data(), v.size() * sizeof(double));
}

void orc_world_vertices_diff(void* p, const double* x, double* V, double* dV, double* d2V)
{
    std::vector<double> v, d, dd;
    world_vertices_diff(static_cast<OwnedScene*>(p)->s, x, v, d, dd);
    std::memcpy(V, v.data(), v.size() * sizeof(double));
    std::memcpy(dV, d.data(), d.size() * sizeof(double));
    std::memcpy(d2V, dd.data(), dd.size() * sizeof(double));
}

int orc_point_triangle_distance_type(const double* p, const double* t0, const double* t1, const double* t2)
{
    return point_triangle_distance_type(p, t0, t1, t2);
}

int orc_edge_edge_distance_type(const double* a0, const double* a1, const double* b0, const double* b1)
{
    return edge_edge_distance_type(a0, a1, b0, b1);
}

double orc_barrier(double d, double s) { return barrier(d, s); }

void orc_project_to_psd(int n, const double* A, double* out) { project_to_psd(n, A, out); }

// candidates: returns 0 and fills when capacities suffice, else 1 (counts set)
int orc_detect_candidates(
    void* p, const double* x0, const double* x1, int continuous,
    double inflation, int brute, int* ee, long long ee_cap, int* fv,
    long long fv_cap, long long* n_ee, long long* n_fv)
{
    Candidates c;
    detect_candidates(static_cast<OwnedScene*>(p)->s, x0, x1, continuous != 0,
                      inflation, brute != 0, c);
    *n_ee = (long long)c.ee.size();
    *n_fv = (long long)c.fv.size();
    if (*n_ee > ee_cap || *n_fv > fv_cap) return 1;
    for (size_t i = 0; i < c.ee.size(); i++) {
        ee[2 * i] = c.ee[i][0];
        ee[2 * i + 1] = c.ee[i][1];
    }
    for (size_t i = 0; i < c.fv.size(); i++) {
        fv[2 * i] = c.fv[i][0];
        fv[2 * i + 1] = c.fv[i][1];
    }
    return 0;
}

long long orc_close_bodies(void* p, const double* x0, const double* x1,
                           double inflation, int* out, long long cap)
{
    auto pairs = close_bodies(static_cast<OwnedScene*>(p)->s, x0, x1, inflation);
    for (size_t i = 0; i < pairs.size() && (long long)i < cap; i++) {
        out[2 * i] = pairs[i][0];
        out[2 * i + 1] = pairs[i][1];
    }
    return (long long)pairs.size();
}

// element boxes (lo, hi per element; included flags)
void orc_element_aabbs(
    void* p, const double* x0, const double* x1, int continuous,
    double inflation, double* vbox, double* ebox, double* fbox, char* vin,
    char* ein, char* fin)
{
    const Scene& s = static_cast<OwnedScene*>(p)->s;
    auto pairs = close_bodies(s, x0, continuous ? x1 : x0, inflation);
    std::vector<AABB> vb, eb, fb;
    std::vector<char> vi, ei, fi;
    element_aabbs(s, x0, x1, continuous != 0, inflation, pairs, vb, eb, fb, vi, ei, fi);
    for (int i = 0; i < s.nv; i++) {
        std::memcpy(vbox + 6 * i, vb[i].lo, 3 * sizeof(double));
        std::memcpy(vbox + 6 * i + 3, vb[i].hi, 3 * sizeof(double));
        vin[i] = vi[i];
    }
    for (int i = 0; i < s.ne; i++) {
        std::memcpy(ebox + 6 * i, eb[i].lo, 3 * sizeof(double));
        std::memcpy(ebox + 6 * i + 3, eb[i].hi, 3 * sizeof(double));
        ein[i] = ei[i];
    }
    for (int i = 0; i < s.nf; i++) {
        std::memcpy(fbox + 6 * i, fb[i].lo, 3 * sizeof(double));
        std::memcpy(fbox + 6 * i + 3, fb[i].hi, 3 * sizeof(double));
        fin[i] = fi[i];
    }
}

int orc_constraint_set(
    void* p, const double* x, const int* ee, long long nee, const int* fv,
    long long nfv, double dhat, double dmin, int* types, int* verts,
    int* prims, int* bodies, double* weight, double* eps, long long cap,
    long long* n_out)
{
    const Scene& s = static_cast<OwnedScene*>(p)->s;
    std::vector<double> V;
    world_vertices(s, x, V);
    std::vector<Constraint> cs;
    construct_constraint_set(s, pack_candidates(ee, nee, fv, nfv), V, dhat, dmin, cs);
    *n_out = (long long)cs.size();
    if (*n_out > cap) return 1;
    for (size_t i = 0; i < cs.size(); i++) {
        types[i] = cs[i].type;
        for (int k = 0; k < 4; k++) verts[4 * i + k] = cs[i].v[k];
        prims[2 * i] = cs[i].prim[0];
        prims[2 * i + 1] = cs[i].prim[1];
        bodies[2 * i] = cs[i].body[0];
        bodies[2 * i + 1] = cs[i].body[1];
        weight[i] = cs[i].weight;
        eps[i] = cs[i].eps_x;
    }
    return 0;
}

// orientation of d against the plane a b c: the sign of det[b - a, c - a,
// d - a] in round-to-nearest double, fixed order
static int orient_sign(const double* a, const double* b, const double* c, const double* d)
{
    const double u0 = b[0] - a[0], u1 = b[1] - a[1], u2 = b[2] - a[2];
    const double v0 = c[0] - a[0], v1 = c[1] - a[1], v2 = c[2] - a[2];
    const double w0 = d[0] - a[0], w1 = d[1] - a[1], w2 = d[2] - a[2];
    const double c0 = v1 * w2 - v2 * w1;
    const double c1 = v2 * w0 - v0 * w2;
    const double c2 = v0 * w1 - v1 * w0;
    const double det = (u0 * c0 + u1 * c1) + u2 * c2;
    return det > 0 ? 1 : (det < 0 ? -1 : 0);
}

// the segment e0 e1 crosses the triangle t0 t1 t2 (orientation test: the
// endpoints on different sides of the plane, not both on it, and the line
// inside the triangle)
static bool edge_crosses_triangle(const double* e0, const double* e1, const double* t0,
                                  const double* t1, const double* t2)
{
    const int s0 = orient_sign(t0, t1, t2, e0), s1 = orient_sign(t0, t1, t2, e1);
    if (s0 == s1) return false;
    const int a = orient_sign(e0, e1, t0, t1), b = orient_sign(e0, e1, t1, t2),
              c = orient_sign(e0, e1, t2, t0);
    return (a >= 0 && b >= 0 && c >= 0) || (a <= 0 && b <= 0 && c <= 0);
}

// RigidBodyProblem::detect_intersections (src/physics/rigid_body_problem.cpp:
// 289-360), 3D: the number of crossing (edge, face) pairs at poses x
long long orc_detect_intersections(void* p, const double* x)
{
    const Scene& s = static_cast<OwnedScene*>(p)->s;
    std::vector<std::array<int, 2>> fe;
    edge_face_candidates(s, x, fe);
    if (fe.empty()) return 0;
    std::vector<double> V;
    world_vertices(s, x, V);
    long long n = 0;
    for (const auto& c : fe) {
        const int f = c[0], e = c[1];
        if (edge_crosses_triangle(&V[3 * s.edges[2 * e]], &V[3 * s.edges[2 * e + 1]],
                                  &V[3 * s.faces[3 * f]], &V[3 * s.faces[3 * f + 1]],
                                  &V[3 * s.faces[3 * f + 2]]))
            n++;
    }
    return n;
}

// DistanceBarrierRBProblem::compute_min_distance(x)
// (src/problems/distance_barrier_rb_problem.cpp:1583-1589) over
// DistanceBarrierConstraint::compute_minimum_distance
// (src/opt/distance_barrier_constraint.cpp:308-323): the constraint set at x
// (discrete candidates inflated by (dhat + dmin) / 2), the smallest squared
// distance over it, its square root; -1 when the set is empty.
double orc_min_distance(void* p, const double* x, double dhat, double dmin)
{
    const Scene& s = static_cast<OwnedScene*>(p)->s;
    Candidates cand;
    detect_candidates(s, x, x, false, (dhat + dmin) / 2, false, cand);
    std::vector<double> V;
    world_vertices(s, x, V);
    std::vector<Constraint> cs;
    construct_constraint_set(s, cand, V, dhat, dmin, cs);
    double m = INFINITY;
    for (const auto& c : cs) m = std::min(m, constraint_sqdist(c, V));
    return std::isfinite(m) ? std::sqrt(m) : -1.0;
}

void orc_local_terms(
    void* p, const double* x, long long n, const int* types, const int* verts,
    const int* prims, const int* bodies, const double* weight,
    const double* eps, double dhat, double dmin, int project, double* energy,
    double* grad, double* hess)
{
    const Scene& s = static_cast<OwnedScene*>(p)->s;
    auto cs = unpack_constraints(n, types, verts, prims, bodies, weight, eps);
    std::vector<double> V, dV, d2V;
    world_vertices_diff(s, x, V, dV, d2V);
    for (long long i = 0; i < n; i++) {
        LocalTerm t;
        constraint_local_term(s, cs[i], V, dV, d2V, dhat, dmin, project != 0, t);
        energy[i] = t.energy;
        std::memcpy(grad + 12 * i, t.grad, 12 * sizeof(double));
        std::memcpy(hess + 144 * i, t.hess, 144 * sizeof(double));
    }
}

// assembled barrier term; returns 1 when the block capacity is too small
int orc_barrier_term(
    void* p, const double* x, long long n, const int* types, const int* verts,
    const int* prims, const int* bodies, const double* weight,
    const double* eps, double dhat, double dmin, int project, double* energy,
    double* grad, int* row_ptr, int* col, double* val, long long cap,
    long long* nnzb)
{
    const Scene& s = static_cast<OwnedScene*>(p)->s;
    auto cs = unpack_constraints(n, types, verts, prims, bodies, weight, eps);
    std::vector<double> g;
    BSR h;
    *energy = barrier_term(s, x, cs, dhat, dmin, g, h, project != 0);
    std::memcpy(grad, g.data(), g.size() * sizeof(double));
    *nnzb = (long long)h.col.size();
    if (*nnzb > cap) return 1;
    std::memcpy(row_ptr, h.row_ptr.data(), h.row_ptr.size() * sizeof(int));
    std::memcpy(col, h.col.data(), h.col.size() * sizeof(int));
    std::memcpy(val, h.val.data(), h.val.size() * sizeof(double));
    return 0;
}

double orc_body_energy(
    double mass, const double* moment, const double* pose_t0,
    const double* vel_t0, const double* Qdot, const int* fixed, int type,
    const double* x6, const double* gravity, double h, double* grad,
    double* hess)
{
    BodyState b;
    b.mass = mass;
    for (int i = 0; i < 3; i++) b.moment[i] = moment[i];
    for (int i = 0; i < 6; i++) {
        b.pose_t0[i] = pose_t0[i];
        b.vel_t0[i] = vel_t0[i];
        b.fixed[i] = fixed[i] != 0;
    }
    for (int i = 0; i < 9; i++) b.Qdot[i] = Qdot[i];
    b.type = type;
    return body_energy(b, x6, gravity, h, grad, hess);
}

int orc_edge_edge_toi(void* p, const double* x0, const double* x1, int ea,
                      int eb, double bound, double tol, double* toi,
                      long long* boxes)
{
    CCDStats st;
    bool hit = edge_edge_toi(static_cast<OwnedScene*>(p)->s, x0, x1, ea, eb, bound, tol, *toi, &st);
    *boxes = st.boxes;
    return hit ? 1 : 0;
}

int orc_face_vertex_toi(void* p, const double* x0, const double* x1, int f,
                        int v, double bound, double tol, double* toi,
                        long long* boxes)
{
    CCDStats st;
    bool hit = face_vertex_toi(static_cast<OwnedScene*>(p)->s, x0, x1, f, v, bound, tol, *toi, &st);
    *boxes = st.boxes;
    return hit ? 1 : 0;
}

double orc_earliest_toi(
    void* p, const double* x0, const double* x1, const int* ee, long long nee,
    const int* fv, long long nfv, double tol, int nthreads, double* per,
    long long* boxes, long long max_boxes, int* status)
{
    std::vector<double> tois;
    CCDStats st;
    st.max_boxes = max_boxes;
    double t = earliest_toi(static_cast<OwnedScene*>(p)->s, x0, x1,
                            pack_candidates(ee, nee, fv, nfv), tol, nthreads,
                            per ? &tois : nullptr, &st);
    if (per) std::memcpy(per, tois.data(), tois.size() * sizeof(double));
    if (boxes) *boxes = st.boxes;
    if (status) *status = st.status;
    return t;
}

// piecewise-linear CCD: one candidate (kind 0 EE (a, b) = edges, 1 FV
// (a, b) = (face, vertex)), stats = { boxes, pieces, status }
int orc_pl_toi(void* p, const double* x0, const double* x1, int kind, int a, int b, double bound,
               double dmin, double* toi, long long* stats)
{
    PLStats st;
    const Scene& s = static_cast<OwnedScene*>(p)->s;
    const bool hit = kind == 0 ? pl_edge_edge_toi(s, x0, x1, a, b, bound, dmin, *toi, &st)
                               : pl_face_vertex_toi(s, x0, x1, a, b, bound, dmin, *toi, &st);
    if (stats) {
        stats[0] = st.boxes;
        stats[1] = st.pieces;
        stats[2] = st.status;
    }
    return hit ? 1 : 0;
}

int orc_linear_ccd(int fv, const double* p0, const double* p1, double ms, double* toi,
                   long long* stats)
{
    long long boxes = 0;
    int status = 0;
    const bool hit = linear_ccd(fv != 0, p0, p1, ms, *toi, boxes, status);
    if (stats) {
        stats[0] = boxes;
        stats[1] = 0;
        stats[2] = status;
    }
    return hit ? 1 : 0;
}

double orc_pl_earliest_toi(void* p, const double* x0, const double* x1, const int* ee, long long nee,
                           const int* fv, long long nfv, double dmin, int nthreads, double* per,
                           long long* stats)
{
    std::vector<double> tois;
    PLStats st;
    const double t = pl_earliest_toi(static_cast<OwnedScene*>(p)->s, x0, x1,
                                     pack_candidates(ee, nee, fv, nfv), dmin, nthreads,
                                     per ? &tois : nullptr, &st);
    if (per) std::memcpy(per, tois.data(), tois.size() * sizeof(double));
    if (stats) {
        stats[0] = st.boxes;
        stats[1] = st.pieces;
        stats[2] = st.status;
    }
    return t;
}

// interval primitives: op 0 add, 1 sub, 2 mul, 3 div, 4 sqrt, 5 cos, 6 sin,
// 7 sinc, 8 abs
void orc_interval_op(int op, double al, double ah, double bl, double bh, double* out)
{
    I a(al, ah), b(bl, bh), r;
    switch (op) {
    case 0: r = a + b; break;
    case 1: r = a - b; break;
    case 2: r = a * b; break;
    case 3: r = a / b; break;
    case 4: r = isqrt(a); break;
    case 5: r = icos(a); break;
    case 6: r = isin(a); break;
    case 7: r = isinc(a); break;
    default: r = iabs(a); break;
    }
    out[0] = r.lo;
    out[1] = r.hi;
}

void orc_interval_rotation(const double* rlo, const double* rhi, double* Rlo, double* Rhi)
{
    I r[3] = { I(rlo[0], rhi[0]), I(rlo[1], rhi[1]), I(rlo[2], rhi[2]) };
    I R[9];
    irotation(r, R);
    for (int i = 0; i < 9; i++) {
        Rlo[i] = R[i].lo;
        Rhi[i] = R[i].hi;
    }
}

double orc_det_sin(double x) { return det_sin(x); }
double orc_det_cos(double x) { return det_cos(x); }


// ---------------------------------------------------------------------------
// lagged friction

static std::vector<FrictionConstraint> unpack_friction(
    const std::vector<Constraint>& cs, const double* lambda, const double* params,
    const double* T)
{
    std::vector<FrictionConstraint> fcs(cs.size());
    for (size_t i = 0; i < cs.size(); i++) {
        fcs[i].c = cs[i];
        fcs[i].lambda = lambda[i];
        fcs[i].p0 = params[2 * i];
        fcs[i].p1 = params[2 * i + 1];
        for (int k = 0; k < 6; k++) fcs[i].T[k] = T[6 * i + k];
    }
    return fcs;
}

void orc_friction_constraints(
    void* p, const double* x0, long long n, const int* types, const int* verts,
    const int* prims, const int* bodies, const double* weight, const double* eps,
    double dhat, double dmin, double kappa, double* lambda, double* params, double* T)
{
    const Scene& s = static_cast<OwnedScene*>(p)->s;
    auto cs = unpack_constraints(n, types, verts, prims, bodies, weight, eps);
    std::vector<double> V0;
    world_vertices(s, x0, V0);
    std::vector<FrictionConstraint> fcs;
    construct_friction_constraints(s, cs, V0, dhat, dmin, kappa, fcs);
    for (long long i = 0; i < n; i++) {
        lambda[i] = fcs[i].lambda;
        params[2 * i] = fcs[i].p0;
        params[2 * i + 1] = fcs[i].p1;
        for (int k = 0; k < 6; k++) T[6 * i + k] = fcs[i].T[k];
    }
}

void orc_friction_local_terms(
    void* p, const double* x, const double* x0, long long n, const int* types,
    const int* verts, const int* prims, const int* bodies, const double* weight,
    const double* eps, const double* lambda, const double* params, const double* T,
    double mu, double epsvh, int project, double* energy, double* grad, double* hess)
{
    const Scene& s = static_cast<OwnedScene*>(p)->s;
    auto cs = unpack_constraints(n, types, verts, prims, bodies, weight, eps);
    auto fcs = unpack_friction(cs, lambda, params, T);
    std::vector<double> V, dV, d2V, V0;
    world_vertices_diff(s, x, V, dV, d2V);
    world_vertices(s, x0, V0);
    for (long long i = 0; i < n; i++) {
        LocalTerm t;
        friction_local_term(s, fcs[i], V, V0, dV, d2V, mu, epsvh, project != 0, t);
        energy[i] = t.energy;
        std::memcpy(grad + 12 * i, t.grad, 12 * sizeof(double));
        std::memcpy(hess + 144 * i, t.hess, 144 * sizeof(double));
    }
}

int orc_friction_term(
    void* p, const double* x, const double* x0, long long n, const int* types,
    const int* verts, const int* prims, const int* bodies, const double* weight,
    const double* eps, const double* lambda, const double* params, const double* T,
    double mu, double epsvh, int project, double* energy, double* grad, int* row_ptr,
    int* col, double* val, long long cap, long long* nnzb)
{
    const Scene& s = static_cast<OwnedScene*>(p)->s;
    auto cs = unpack_constraints(n, types, verts, prims, bodies, weight, eps);
    auto fcs = unpack_friction(cs, lambda, params, T);
    std::vector<double> g;
    BSR h;
    *energy = friction_term(s, x, x0, fcs, mu, epsvh, g, h, project != 0);
    std::memcpy(grad, g.data(), g.size() * sizeof(double));
    *nnzb = (long long)h.col.size();
    if (*nnzb > cap) return 1;
    std::memcpy(row_ptr, h.row_ptr.data(), h.row_ptr.size() * sizeof(int));
    std::memcpy(col, h.col.data(), h.col.size() * sizeof(int));
    std::memcpy(val, h.val.data(), h.val.size() * sizeof(double));
    return 0;
}


// one simulation step; per-body arrays are updated in place.  params:
// h, gravity (3), dhat, dmin, mu, epsv, max_newton_iterations,
// velocity_conv_tol, velocity_conv_tol_abs, line_search_lower_bound,
// dhat_epsilon, min_barrier_stiffness_scale, bbox_diagonal, average_mass,
// newton_polish, ccd_rescale, trajectory (19 doubles).  stats: newton iterations, newton steps, objective
// evaluations, CCD calls.
static std::vector<BodyState> unpack_bodies(int nb, const double* mass, const double* moment,
                                            const double* pose, const double* vel,
                                            const double* Qdot, const int* fixed, const int* type)
{
    std::vector<BodyState> bodies(nb);
    for (int b = 0; b < nb; b++) {
        BodyState& B = bodies[b];
        B.mass = mass[b];
        for (int i = 0; i < 3; i++) B.moment[i] = moment[3 * b + i];
        for (int i = 0; i < 6; i++) {
            B.pose_t0[i] = pose[6 * b + i];
            B.vel_t0[i] = vel[6 * b + i];
            B.fixed[i] = fixed[6 * b + i] != 0;
        }
        for (int i = 0; i < 9; i++) B.Qdot[i] = Qdot[9 * b + i];
        B.type = type[b];
    }
    return bodies;
}

static SimParams unpack_params(const double* params)
{
    SimParams sp;
    sp.h = params[0];
    for (int i = 0; i < 3; i++) sp.gravity[i] = params[1 + i];
    sp.dhat = params[4];
    sp.dmin = params[5];
    sp.mu = params[6];
    sp.epsv = params[7];
    sp.max_newton_iterations = (int)params[8];
    sp.velocity_conv_tol = params[9];
    sp.velocity_conv_tol_abs = (int)params[10];
    sp.line_search_lower_bound = params[11];
    sp.dhat_epsilon = params[12];
    sp.min_barrier_stiffness_scale = params[13];
    sp.bbox_diagonal = params[14];
    sp.average_mass = params[15];
    sp.newton_polish = (int)params[16];
    sp.ccd_rescale = params[17];
    sp.trajectory = (int)params[18];
    return sp;
}

// x_out (6 nb) and rec_out (kappa, d kappa / d kappa0) are optional
void orc_simulation_step_rec(
    void* p, const double* mass, const double* moment, double* pose, double* vel,
    double* Qdot, const int* fixed, const int* type, const double* params, double* kappa,
    long long* stats, double* x_out, double* rec_out, const double* kin_target)
{
    const Scene& s = static_cast<OwnedScene*>(p)->s;
    std::vector<BodyState> bodies = unpack_bodies(s.nb, mass, moment, pose, vel, Qdot, fixed, type);
    // kin_target (optional, 6 per body): a kinematic body's target pose, NaN
    // in its first component for none
    if (kin_target)
        for (int b = 0; b < s.nb; b++)
            if (!std::isnan(kin_target[6 * b])) {
                bodies[b].has_target = true;
                for (int i = 0; i < 6; i++) bodies[b].kin_target[i] = kin_target[6 * b + i];
            }
    SimParams sp = unpack_params(params);
    SimStats st;
    StepRecord rec;
    simulation_step(s, bodies, sp, *kappa, &st, &rec);
    for (int b = 0; b < s.nb; b++) {
        for (int i = 0; i < 6; i++) {
            pose[6 * b + i] = bodies[b].pose_t0[i];
            vel[6 * b + i] = bodies[b].vel_t0[i];
        }
        for (int i = 0; i < 9; i++) Qdot[9 * b + i] = bodies[b].Qdot[i];
    }
    if (stats) {
        stats[0] = st.newton_iterations;
        stats[1] = st.newton_steps;
        stats[2] = st.objective_evals;
        stats[3] = st.ccd_calls;
    }
    if (x_out) std::memcpy(x_out, rec.x.data(), rec.x.size() * sizeof(double));
    if (rec_out) {
        rec_out[0] = rec.kappa;
        rec_out[1] = rec.dkappa_dk0;
    }
}

void orc_simulation_step(
    void* p, const double* mass, const double* moment, double* pose, double* vel,
    double* Qdot, const int* fixed, const int* type, const double* params, double* kappa,
    long long* stats)
{
    orc_simulation_step_rec(p, mass, moment, pose, vel, Qdot, fixed, type, params, kappa, stats,
                            nullptr, nullptr, nullptr);
}

// adjoint of one step: the start-of-step state (pose, vel, Qdot), the step's
// solution x (6 nb) and rec (kappa, d kappa / d kappa0); d_* in are the
// gradients with respect to the state after the step, d_* out (overwritten)
// those with respect to the state before.  Returns 0, or 1 when the Hessian
// cannot be factorised.
int orc_adjoint_step(
    void* p, const double* mass, const double* moment, const double* pose, const double* vel,
    const double* Qdot, const int* fixed, const int* type, const double* params,
    const double* x, const double* rec, const double* d_pose_in, const double* d_vel_in,
    const double* d_Qdot_in, double* d_pose_out, double* d_vel_out, double* d_Qdot_out)
{
    const Scene& s = static_cast<OwnedScene*>(p)->s;
    const int nb = s.nb;
    std::vector<BodyState> pre = unpack_bodies(nb, mass, moment, pose, vel, Qdot, fixed, type);
    SimParams sp = unpack_params(params);
    StepRecord r;
    r.x.assign(x, x + 6 * (size_t)nb);
    r.kappa = rec[0];
    r.dkappa_dk0 = rec[1];
    AdjointState in, out;
    in.pose.assign(d_pose_in, d_pose_in + 6 * (size_t)nb);
    in.vel.assign(d_vel_in, d_vel_in + 6 * (size_t)nb);
    in.Qdot.assign(d_Qdot_in, d_Qdot_in + 9 * (size_t)nb);
    if (!adjoint_step(s, pre, sp, r, in, out)) return 1;
    std::memcpy(d_pose_out, out.pose.data(), out.pose.size() * sizeof(double));
    std::memcpy(d_vel_out, out.vel.data(), out.vel.size() * sizeof(double));
    std::memcpy(d_Qdot_out, out.Qdot.data(), out.Qdot.size() * sizeof(double));
    return 0;
}

} // extern "C"
