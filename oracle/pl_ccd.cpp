// Piecewise-linear trajectory CCD of the oracle (test infrastructure only).
//
// Restates compute_piecewise_linear_edge_edge_time_of_impact and
// compute_piecewise_linear_face_vertex_time_of_impact
// (src/ccd/piecewise_linear/time_of_impact.cpp:326-651): the time interval is
// cut into pieces over which each body's pose moves linearly
// (Pose::interpolate, src/physics/pose.tpp:142-148), the vertices of a piece
// move on straight lines between their positions at its ends, and a linear
// CCD with a minimum separation finds the first time the straight-line
// motions come within that separation.  Per piece [ti0, ti1]:
//  * distance_ti0 = |closest features at ti0|; if it dropped below 0.2 of
//    distance_t0 and ti0 >= 1e-6, the time of impact is ti0 (:372-379);
//  * the deviation of the rigid trajectory from the straight line, an
//    interval bound over the piece per vertex
//    |R(t) v + p(t) - ((v(ti1) - v(ti0)) t + v(ti0))|, summed over the two
//    sides (largest vertex of each) (:381-430);
//  * a piece whose deviation is >= 0.5 distance_ti0 is halved (while fewer
//    than 1000 halvings were made, or always at ti0 = 0) (:432-437);
//  * the linear CCD of the piece with minimum separation deviation + dmin;
//    an impact at the piece's start is not taken: the piece is halved
//    (:440-470).
// The reference's linear CCD is Tight-Inclusion's inclusion-based root
// finder (Wang et al. 2021, "A Large-Scale Benchmark and an Inclusion-Based
// Algorithm for Continuous Collision Detection"; library pinned at
// b913416aecf1bbb8a51726039dcb94f395849cab, not vendored, so its last bits
// are not pinned here).  The restatement keeps the published method:
//  * the distance function F(t, u, v) between the straight-line points (EE:
//    a point of each edge; FV: the vertex minus a point of the triangle) is
//    multilinear in (t, u, v), so its range over a box is the hull of its
//    values at the eight corners; the corners are evaluated in interval
//    arithmetic, which takes the place of Tight-Inclusion's a-priori
//    floating-point error filter;
//  * a box whose range misses [-ms, ms]^3 holds no impact; a box whose range
//    is inside [-ms, ms]^3, or no wider than the co-domain tolerance 1e-6
//    plus ms in every coordinate, is a root, and the time of impact is the
//    t.lo of the earliest root.  (With the tolerance alone, the boxes near
//    the first contact of a large separation would have to be resolved to
//    1e-6 over the whole ms-wide patch of the (u, v) plane that comes within
//    ms: ~(ms / 1e-6)^2 boxes; the looser rule keeps every root conservative
//    and resolves the time to ~ms of F's travel);
//  * other boxes are halved along the dimension whose halving shrinks the
//    range most (the largest change of F between opposite corners), the
//    earlier half searched first; boxes starting at or after the earliest
//    root are skipped; after 10^6 boxes the smallest unexplored t.lo is
//    reported (a conservative time), and so is the start of a box that
//    cannot be halved exactly (120 halvings, or 52 in one dimension).
// For face-vertex boxes, u + v must meet [0, 1] (the triangle).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "interval.hpp"
#include "oracle.hpp"

namespace orc {

void irotation(const I r[3], I R[9]);
void iworld_vertex(const I R[9], const I p[3], const double* v, I out[3]);

namespace {

constexpr double kLinearTol = 1e-6;          // co-domain tolerance
constexpr long long kLinearMaxBoxes = 1000000;
constexpr int kMaxSubdivisions = 1000;
constexpr int kMaxPieceDepth = 60;           // halvings of one piece
constexpr double kTrajectoryFactor = 0.5;
constexpr double kDecreasingFactor = 0.2;
constexpr double kDecreasingMinTime = 1e-6;

// Pose::interpolate on doubles: (x1 - x0) t + x0
void pose_at(const double* x0, const double* x1, double t, double* x)
{
    for (int k = 0; k < 6; k++) x[k] = (x1[k] - x0[k]) * t + x0[k];
}

// world vertex ((v0 R0 + v1 R1) + v2 R2) + p at a double pose
void vertex_at_pose(const double* x, const double* v, double* out)
{
    double R[9];
    rotation_matrix(x + 3, R);
    for (int j = 0; j < 3; j++)
        out[j] = ((v[0] * R[3 * j] + v[1] * R[3 * j + 1]) + v[2] * R[3 * j + 2]) + x[j];
}

double point_triangle_sqdist(const double* p, const double* t0, const double* t1, const double* t2)
{
    switch (point_triangle_distance_type(p, t0, t1, t2)) {
    case PT_P_T0: return point_point_sqdist(p, t0);
    case PT_P_T1: return point_point_sqdist(p, t1);
    case PT_P_T2: return point_point_sqdist(p, t2);
    case PT_P_E0: return point_line_sqdist(p, t0, t1);
    case PT_P_E1: return point_line_sqdist(p, t1, t2);
    case PT_P_E2: return point_line_sqdist(p, t2, t0);
    default: return point_plane_sqdist(p, t0, t1, t2);
    }
}

// distance of the candidate's features (EE: a0 a1 b0 b1; FV: v f0 f1 f2)
double feature_distance(bool fv, const double P[4][3])
{
    return std::sqrt(fv ? point_triangle_sqdist(P[0], P[1], P[2], P[3])
                        : edge_edge_sqdist(P[0], P[1], P[2], P[3]));
}

// a box of the linear CCD: dyadic in each dimension (level = number of
// halvings), depth = halvings from [0, 1]^3
struct LBox {
    double lo[3], hi[3];  // t, u, v
    int lv[3];
    int depth;
};
constexpr int kLinearMaxDepth = 120;
constexpr int kLinearMaxLevel = 52;

// F at one corner (t, u, v) of the straight-line motion P0 -> P1, as
// intervals (the corner coordinates are exact)
void corner_value(bool fv, const double P0[4][3], const double P1[4][3], double t, double u,
                  double v, I y[3])
{
    for (int j = 0; j < 3; j++) {
        I q[4];
        for (int k = 0; k < 4; k++) q[k] = (I(P1[k][j]) - I(P0[k][j])) * I(t) + I(P0[k][j]);
        if (fv) {
            const I fp = ((q[2] - q[1]) * I(u) + (q[3] - q[1]) * I(v)) + q[1];
            y[j] = q[0] - fp;
        } else {
            const I a = (q[1] - q[0]) * I(u) + q[0];
            const I b = (q[3] - q[2]) * I(v) + q[2];
            y[j] = a - b;
        }
    }
}

// range of F over the box (hull of the corner enclosures) and the change of
// F along each dimension (largest over coordinates and corner pairs of the
// difference of the corner midpoints)
void box_range(bool fv, const double P0[4][3], const double P1[4][3], const LBox& x, I range[3],
               double change[3])
{
    I c[8][3];
    for (int k = 0; k < 8; k++)
        corner_value(fv, P0, P1, (k & 1) ? x.hi[0] : x.lo[0], (k & 2) ? x.hi[1] : x.lo[1],
                     (k & 4) ? x.hi[2] : x.lo[2], c[k]);
    for (int j = 0; j < 3; j++) {
        range[j] = c[0][j];
        for (int k = 1; k < 8; k++) range[j] = hull(range[j], c[k][j]);
    }
    for (int d = 0; d < 3; d++) {
        double m = 0;
        for (int k = 0; k < 8; k++) {
            if (k & (1 << d)) continue;
            for (int j = 0; j < 3; j++) {
                const double a = 0.5 * (c[k][j].lo + c[k][j].hi);
                const double b = 0.5 * (c[k | (1 << d)][j].lo + c[k | (1 << d)][j].hi);
                m = std::max(m, std::fabs(b - a));
            }
        }
        change[d] = m;
    }
}

// the linear CCD of one piece: first t in [0, 1] at which the straight-line
// motions P0 -> P1 come within ms; status 5 when the box budget ran out
bool linear_toi(bool fv, const double P0[4][3], const double P1[4][3], double ms, double& toi,
                long long& boxes, int& status)
{
    std::vector<LBox> stack;
    stack.push_back(LBox { { 0, 0, 0 }, { 1, 1, 1 }, { 0, 0, 0 }, 0 });
    double earliest = INFINITY;
    long long n = 0;
    while (!stack.empty()) {
        const LBox x = stack.back();
        stack.pop_back();
        if (x.lo[0] >= earliest) continue;
        if (fv && !(add_down(x.lo[1], x.lo[2]) <= 1.0)) continue;
        if (n >= kLinearMaxBoxes) {
            double m = x.lo[0];
            for (const LBox& b : stack) m = std::min(m, b.lo[0]);
            earliest = std::min(earliest, m);
            status = std::max(status, 5);
            break;
        }
        n++;
        I r[3];
        double ch[3];
        box_range(fv, P0, P1, x, r, ch);
        bool meets = true, inside = true, small = true;
        for (int j = 0; j < 3; j++) {
            meets = meets && r[j].lo <= ms && r[j].hi >= -ms;
            inside = inside && r[j].lo >= -ms && r[j].hi <= ms;
            small = small && width(r[j]) <= kLinearTol + ms;
        }
        if (!meets) continue;
        if (inside || small) {
            earliest = x.lo[0];
            continue;
        }
        int split = 0;
        for (int d = 1; d < 3; d++)
            if (ch[d] > ch[split]) split = d;
        if (x.depth >= kLinearMaxDepth || x.lv[split] >= kLinearMaxLevel) {
            // the box cannot be halved exactly: its start is a conservative root
            earliest = x.lo[0];
            status = std::max(status, 4);
            continue;
        }
        const double mid = 0.5 * (x.lo[split] + x.hi[split]);
        LBox a = x, b = x;
        a.hi[split] = mid;
        b.lo[split] = mid;
        a.lv[split] = b.lv[split] = x.lv[split] + 1;
        a.depth = b.depth = x.depth + 1;
        stack.push_back(b);
        stack.push_back(a);
    }
    boxes += n;
    toi = earliest;
    return earliest < INFINITY;
}

// the largest deviation of a body's vertices from their straight lines over
// the piece between poses xa (at ti0) and xb (at ti1) (:381-430)
double piece_deviation(const Scene& s, const double* xa, const double* xb, const int* vids, int nv)
{
    I p[3], r[3], R[9];
    const I t(0.0, 1.0);
    for (int k = 0; k < 3; k++) {
        p[k] = (I(xb[k]) - I(xa[k])) * t + I(xa[k]);
        r[k] = (I(xb[3 + k]) - I(xa[3 + k])) * t + I(xa[3 + k]);
    }
    irotation(r, R);
    double dev = 0;
    for (int i = 0; i < nv; i++) {
        const double* v = s.rest + 3 * vids[i];
        double va[3], vb[3];
        vertex_at_pose(xa, v, va);
        vertex_at_pose(xb, v, vb);
        I w[3];
        iworld_vertex(R, p, v, w);
        I sq(0.0);
        for (int j = 0; j < 3; j++) {
            const I e = w[j] - ((I(vb[j]) - I(va[j])) * t + I(va[j]));
            sq = j == 0 ? e * e : sq + e * e;
        }
        dev = std::max(dev, isqrt(sq).hi);
    }
    return dev;
}

// the piecewise-linear time of impact of one candidate: vertices (EE: a0 a1
// b0 b1; FV: v f0 f1 f2), na of them on body A
bool pl_toi(const Scene& s, const double* x0, const double* x1, bool fv, const int vid[4], int A,
            int B, double earliest_bound, double dmin, double& toi, PLStats* st)
{
    const int na = fv ? 1 : 2;
    const double* xa0 = x0 + 6 * A;
    const double* xa1 = x1 + 6 * A;
    const double* xb0 = x0 + 6 * B;
    const double* xb1 = x1 + 6 * B;
    auto points = [&](const double* pa, const double* pb, double P[4][3]) {
        for (int k = 0; k < 4; k++) vertex_at_pose(k < na ? pa : pb, s.rest + 3 * vid[k], P[k]);
    };
    double P0[4][3], P1[4][3];
    points(xa0, xb0, P0);
    const double distance_t0 = feature_distance(fv, P0);
    if (distance_t0 <= dmin) {
        toi = 0;
        return true;
    }
    // the stack of piece ends; the current piece is [ti0, ts[top]]
    double ts[kMaxPieceDepth + 1];
    int top = 0;
    ts[0] = earliest_bound;
    int subdivisions = 1;
    double ti0 = 0;
    double pa0[6], pb0[6];
    std::memcpy(pa0, xa0, sizeof(pa0));
    std::memcpy(pb0, xb0, sizeof(pb0));
    long long boxes = 0;
    int status = 0;
    bool hit = false;
    double result = INFINITY;
    while (top >= 0) {
        const double ti1 = ts[top];
        double pa1[6], pb1[6];
        pose_at(xa0, xa1, ti1, pa1);
        pose_at(xb0, xb1, ti1, pb1);
        points(pa0, pb0, P0);
        const double distance_ti0 = feature_distance(fv, P0);
        if (distance_ti0 < kDecreasingFactor * distance_t0 && ti0 >= kDecreasingMinTime) {
            result = ti0;
            hit = true;
            break;
        }
        const double dev = piece_deviation(s, pa0, pa1, vid, na)
            + piece_deviation(s, pb0, pb1, vid + na, 4 - na);
        const bool may_split = top < kMaxPieceDepth;
        if (dev >= kTrajectoryFactor * distance_ti0 && (subdivisions < kMaxSubdivisions || ti0 == 0)) {
            if (!may_split) {
                // the piece cannot be halved further: its start is a
                // conservative time of impact
                result = ti0;
                hit = true;
                status = std::max(status, 4);
                break;
            }
            ts[++top] = 0.5 * (ti1 + ti0);
            subdivisions++;
            continue;
        }
        points(pa1, pb1, P1);
        double t;
        if (linear_toi(fv, P0, P1, dev + dmin, t, boxes, status)) {
            const double tt = (ti1 - ti0) * t + ti0;
            if (tt == 0) {
                if (!may_split) {
                    result = 0;
                    hit = true;
                    status = std::max(status, 4);
                    break;
                }
                ts[++top] = 0.5 * (ti1 + ti0);
                subdivisions++;
                continue;
            }
            result = tt;
            hit = true;
            break;
        }
        top--;
        ti0 = ti1;
        std::memcpy(pa0, pa1, sizeof(pa0));
        std::memcpy(pb0, pb1, sizeof(pb0));
    }
    if (st) {
        st->boxes += boxes;
        st->pieces += subdivisions;
        st->status = std::max(st->status, status);
    }
    toi = result;
    return hit;
}

} // namespace

bool linear_ccd(bool fv, const double* p0, const double* p1, double ms, double& toi,
                long long& boxes, int& status)
{
    double P0[4][3], P1[4][3];
    for (int k = 0; k < 4; k++)
        for (int j = 0; j < 3; j++) {
            P0[k][j] = p0[3 * k + j];
            P1[k][j] = p1[3 * k + j];
        }
    return linear_toi(fv, P0, P1, ms, toi, boxes, status);
}

bool pl_edge_edge_toi(const Scene& s, const double* x0, const double* x1, int ea, int eb,
                      double earliest_bound, double dmin, double& toi, PLStats* st)
{
    const int vid[4] = { s.edges[2 * ea], s.edges[2 * ea + 1], s.edges[2 * eb], s.edges[2 * eb + 1] };
    return pl_toi(s, x0, x1, false, vid, s.ebody[ea], s.ebody[eb], earliest_bound, dmin, toi, st);
}

bool pl_face_vertex_toi(const Scene& s, const double* x0, const double* x1, int f, int v,
                        double earliest_bound, double dmin, double& toi, PLStats* st)
{
    const int vid[4] = { v, s.faces[3 * f], s.faces[3 * f + 1], s.faces[3 * f + 2] };
    return pl_toi(s, x0, x1, true, vid, s.vbody[v], s.fbody[f], earliest_bound, dmin, toi, st);
}

// compute_earliest_toi_narrow_phase with trajectory PIECEWISE_LINEAR: every
// candidate searches [0, 1] (the reference's first candidate's domain)
double pl_earliest_toi(const Scene& s, const double* x0, const double* x1, const Candidates& c,
                       double dmin, int nthreads, std::vector<double>* per, PLStats* st)
{
    const size_t nee = c.ee.size(), nfv = c.fv.size(), n = nee + nfv;
    std::vector<double> tois(n, INFINITY);
    std::atomic<size_t> next(0);
    const int nt = std::max(1, nthreads);
    std::vector<PLStats> local(nt);
    auto work = [&](int tid) {
        for (;;) {
            const size_t i = next.fetch_add(16);
            if (i >= n) break;
            for (size_t k = i; k < std::min(n, i + 16); k++) {
                double toi;
                if (k < nee) pl_edge_edge_toi(s, x0, x1, c.ee[k][0], c.ee[k][1], 1.0, dmin, toi, &local[tid]);
                else pl_face_vertex_toi(s, x0, x1, c.fv[k - nee][0], c.fv[k - nee][1], 1.0, dmin, toi,
                                        &local[tid]);
                tois[k] = toi;
            }
        }
    };
    if (nt == 1) {
        work(0);
    } else {
        std::vector<std::thread> th;
        for (int t = 0; t < nt; t++) th.emplace_back(work, t);
        for (auto& t : th) t.join();
    }
    double m = INFINITY;
    for (double t : tois) m = std::min(m, t);
    if (st)
        for (const PLStats& l : local) {
            st->boxes += l.boxes;
            st->pieces += l.pieces;
            st->status = std::max(st->status, l.status);
        }
    if (per) *per = tois;
    return m;
}

} // namespace orc
