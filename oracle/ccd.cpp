// Oracle: rigid-trajectory interval CCD (test infrastructure only).
//
// Restates src/ccd/rigid/time_of_impact.cpp:158-310 (EE and FV time of
// impact), src/ccd/rigid/rigid_trajectory_aabb.cpp:7-103 (interval point
// positions), src/interval/interval_root_finder.cpp:97-203 (the branch and
// bound), src/utils/sinc.cpp:36-101 (interval sinc) and the interval form of
// Pose::interpolate / construct_rotation_matrix (src/physics/pose.tpp:142-148,
// 203-218).  Evaluation order follows Eigen 3.3's coefficient-based products:
// 3x3 fixed-size products sum as x0 + (x1 + x2); row-vector times dynamic
// 3x3 products and dot products of dynamic 3-vectors sum as (x0 + x1) + x2.
//
// Each candidate searches t in [0, 1] (the reference's first-candidate
// domain), so its time of impact is a function of the candidate alone; the
// earliest time of impact is the minimum over candidates.
#include "interval.hpp"
#include <cstring>

#include "oracle.hpp"

#include <atomic>
#include <thread>
#include <vector>

namespace orc {

static const double kTaylorN = 1.220703125e-04;
static const double kSincMonotone = 4.4934094579;

static I sinc_interval_taylor(double xd)
{
    I x(xd);
    if (std::fabs(x.lo) >= kTaylorN) return isin(x) / x;
    I x2 = x * x;
    return 1.0 + (x2 / 6.0) * (x2 / 20.0 - 1.0);
}

// sinc over an interval (sinc.cpp:49-101)
I isinc(const I& x)
{
    I y = I::empty(), x_pos = x;
    if (x.lo < 0) {
        if (x.hi <= 0) return isinc(-x);
        y = isinc(I(0.0, -x.lo));
        x_pos = I(0.0, x.hi);
    }
    I x_gt = x_pos;
    if (x_pos.lo <= kSincMonotone) {
        I x_mono = x_pos;
        if (x_mono.hi > kSincMonotone) {
            x_mono = I(x_mono.lo, kSincMonotone);
            x_gt = I(kSincMonotone, x_pos.hi);
        } else {
            x_gt = I::empty();
        }
        y = hull(y, I(std::max(sinc_interval_taylor(x_mono.hi).lo, -0.271724),
                      std::min(sinc_interval_taylor(x_mono.lo).hi, 1.0)));
    }
    if (!x_gt.is_empty()) y = hull(y, isin(x_gt) / x_gt);
    return y;
}

// sinc(|r|) with |r| = sqrt(|r0|^2 + |r1|^2 + |r2|^2) (sinc.hpp:16-33)
static I isinc_norm(const I r[3])
{
    I a0 = iabs(r[0]), a1 = iabs(r[1]), a2 = iabs(r[2]);
    I d = (a0 * a0 + a1 * a1) + a2 * a2;
    return isinc(isqrt(d));
}

// interval rotation matrix (pose.tpp:203-218)
void irotation(const I r[3], I R[9])
{
    I sa = isinc_norm(r);
    I two(2.0);
    I rh[3] = { r[0] / two, r[1] / two, r[2] / two };
    I sh = isinc_norm(rh);
    I z(0.0);
    I K[9] = { z, -r[2], r[1], r[2], z, -r[0], -r[1], r[0], z };
    I c = (0.5 * sh) * sh;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            I k2 = K[3 * i] * K[j] + (K[3 * i + 1] * K[3 + j] + K[3 * i + 2] * K[6 + j]);
            I v = sa * K[3 * i + j] + c * k2;
            R[3 * i + j] = i == j ? v + I(1.0) : v;
        }
}

// pose at interval time t (Pose::interpolate on intervals)
static void ipose(const double* x0, const double* x1, const I& t, I p[3], I r[3])
{
    for (int k = 0; k < 3; k++) {
        p[k] = (I(x1[k]) - I(x0[k])) * t + I(x0[k]);
        r[k] = (I(x1[3 + k]) - I(x0[3 + k])) * t + I(x0[3 + k]);
    }
}

// world vertex R v + p over intervals (rigid_body.tpp:19-24)
void iworld_vertex(const I R[9], const I p[3], const double* v, I out[3])
{
    for (int j = 0; j < 3; j++)
        out[j] = ((v[0] * R[3 * j] + v[1] * R[3 * j + 1]) + v[2] * R[3 * j + 2]) + p[j];
}

struct BodyTraj {
    const double* x0;
    const double* x1;
};

static void vertex_at(const Scene& s, const BodyTraj& b, int vid, const I& t, I out[3])
{
    I p[3], r[3], R[9];
    ipose(b.x0, b.x1, t, p, r);
    irotation(r, R);
    iworld_vertex(R, p, s.rest + 3 * vid, out);
}

// ---------------------------------------------------------------------------
// branch and bound over boxes (interval_root_finder.cpp:97-203)

struct Box {
    I x[3];
};

template <class F, class Valid>
static bool root_finder(F f, Valid valid, const Box& x0, double tol[3],
                        Box& root, CCDStats* st)
{
    Box earliest;
    for (int i = 0; i < 3; i++) earliest.x[i] = I(INFINITY);
    bool found = false;
    std::vector<Box> stack;
    stack.push_back(x0);
    Box xt;
    for (int i = 0; i < 3; i++) xt.x[i] = I(0.0, tol[i]);
    {
        I y[3];
        f(xt, y);
        if (zero_in(y[0]) && zero_in(y[1]) && zero_in(y[2])) tol[0] /= 1e2;
    }
    long long nbox = 0;
    const long long budget = st ? st->max_boxes : 0;
    while (!stack.empty()) {
        Box x = stack.back();
        stack.pop_back();
        if (x.x[0].lo >= earliest.x[0].lo) continue;
        if (st && st->gmin) {
            unsigned long long gb = st->gmin->load(std::memory_order_relaxed);
            double g;
            std::memcpy(&g, &gb, sizeof(g));
            if (x.x[0].lo >= g) continue;
        }
        if (!valid(x)) continue;
        if (budget > 0 && nbox >= budget) {
            // budget exhausted: the earliest unexplored t.lo is conservative
            double m = x.x[0].lo;
            for (const Box& b : stack) m = std::min(m, b.x[0].lo);
            earliest.x[0] = I(std::min(earliest.x[0].lo, m));
            found = true;
            st->status = std::max(st->status, 5);
            break;
        }
        nbox++;
        I y[3];
        f(x, y);
        if (st) st->boxes++;
        if (!(zero_in(y[0]) && zero_in(y[1]) && zero_in(y[2]))) continue;
        double w[3] = { width(x.x[0]), width(x.x[1]), width(x.x[2]) };
        bool all_tol = w[0] <= tol[0] && w[1] <= tol[1] && w[2] <= tol[2];
        bool all_zero = w[0] <= 1e-10 && w[1] <= 1e-10 && w[2] <= 1e-10;
        if ((x.x[0].lo > 0 || all_zero) && all_tol) {
            earliest = x;
            found = true;
            if (st && st->gmin) {
                unsigned long long nb, ob = st->gmin->load();
                std::memcpy(&nb, &x.x[0].lo, sizeof(nb));
                while (nb < ob && !st->gmin->compare_exchange_weak(ob, nb)) {
                }
            }
            continue;
        }
        int split = -1;
        for (int i = 0; i < 3; i++)
            if ((all_tol || w[i] > tol[i])
                && (split == -1 || w[i] * tol[split] > w[split] * tol[i]))
                split = i;
        double m = median(x.x[split]);
        Box a = x, b = x;
        a.x[split] = I(x.x[split].lo, m);
        b.x[split] = I(m, x.x[split].hi);
        stack.push_back(b);
        stack.push_back(a);
    }
    root = earliest;
    return found;
}

// edge-edge (time_of_impact.cpp:158-217; rigid_trajectory_aabb.cpp:22-34,76-89)
bool edge_edge_toi(
    const Scene& s, const double* x0, const double* x1, int ea, int eb,
    double earliest_bound, double toi_tol, double& toi, CCDStats* st)
{
    int A = s.ebody[ea], B = s.ebody[eb];
    BodyTraj ta { x0 + 6 * A, x1 + 6 * A }, tb { x0 + 6 * B, x1 + 6 * B };
    int a0 = s.edges[2 * ea], a1 = s.edges[2 * ea + 1];
    int b0 = s.edges[2 * eb], b1 = s.edges[2 * eb + 1];
    auto f = [&](const Box& x, I y[3]) {
        I pa0[3], pa1[3], pb0[3], pb1[3];
        vertex_at(s, ta, a0, x.x[0], pa0);
        vertex_at(s, ta, a1, x.x[0], pa1);
        vertex_at(s, tb, b0, x.x[0], pb0);
        vertex_at(s, tb, b1, x.x[0], pb1);
        for (int j = 0; j < 3; j++) {
            I ea_pt = (pa1[j] - pa0[j]) * x.x[1] + pa0[j];
            I eb_pt = (pb1[j] - pb0[j]) * x.x[2] + pb0[j];
            y[j] = ea_pt - eb_pt;
        }
    };
    auto valid = [](const Box&) { return true; };
    double tol[3] = { toi_tol, 1e-4 / s.edge_len[ea], 1e-4 / s.edge_len[eb] };
    Box bx;
    bx.x[0] = I(0.0, earliest_bound);
    bx.x[1] = I(0.0, 1.0);
    bx.x[2] = I(0.0, 1.0);
    Box root;
    bool hit = root_finder(f, valid, bx, tol, root, st);
    toi = hit ? root.x[0].lo : INFINITY;
    return hit;
}

// face-vertex (time_of_impact.cpp:248-310; rigid_trajectory_aabb.cpp:36-49,91-103)
bool face_vertex_toi(
    const Scene& s, const double* x0, const double* x1, int fi, int vi,
    double earliest_bound, double toi_tol, double& toi, CCDStats* st)
{
    int A = s.vbody[vi], B = s.fbody[fi];
    BodyTraj ta { x0 + 6 * A, x1 + 6 * A }, tb { x0 + 6 * B, x1 + 6 * B };
    int f0 = s.faces[3 * fi], f1 = s.faces[3 * fi + 1], f2 = s.faces[3 * fi + 2];
    auto f = [&](const Box& x, I y[3]) {
        I pv[3], q0[3], q1[3], q2[3];
        vertex_at(s, ta, vi, x.x[0], pv);
        vertex_at(s, tb, f0, x.x[0], q0);
        vertex_at(s, tb, f1, x.x[0], q1);
        vertex_at(s, tb, f2, x.x[0], q2);
        for (int j = 0; j < 3; j++) {
            I fp = ((q1[j] - q0[j]) * x.x[1] + (q2[j] - q0[j]) * x.x[2]) + q0[j];
            y[j] = pv[j] - fp;
        }
    };
    auto valid = [](const Box& x) { return overlap(x.x[1] + x.x[2], I(0.0, 1.0)); };
    double tol[3] = { toi_tol, 1e-4 / s.edge_len[s.f2e[3 * fi]],
                      1e-4 / s.edge_len[s.f2e[3 * fi + 1]] };
    Box bx;
    bx.x[0] = I(0.0, earliest_bound);
    bx.x[1] = I(0.0, 1.0);
    bx.x[2] = I(0.0, 1.0);
    Box root;
    bool hit = root_finder(f, valid, bx, tol, root, st);
    toi = hit ? root.x[0].lo : INFINITY;
    return hit;
}

// compute_earliest_toi_narrow_phase (distance_barrier_constraint.cpp:151-265),
// candidates ordered ev | ee | fv, per-candidate domain [0, 1].
double earliest_toi(
    const Scene& s, const double* x0, const double* x1, const Candidates& c,
    double toi_tol, int nthreads, std::vector<double>* per, CCDStats* st)
{
    const size_t nee = c.ee.size(), nfv = c.fv.size(), n = nee + nfv;
    std::vector<double> tois(n, INFINITY);
    std::atomic<size_t> next(0);
    std::vector<long long> boxes(std::max(1, nthreads), 0);
    std::vector<int> status(std::max(1, nthreads), 0);
    // without per-candidate results the search skips boxes at or after the
    // running minimum over all candidates
    std::atomic<unsigned long long> gmin(0x7ff0000000000000ull);
    auto work = [&](int tid) {
        CCDStats local;
        local.max_boxes = st ? st->max_boxes : 0;
        if (!per) local.gmin = &gmin;
        for (;;) {
            size_t i = next.fetch_add(64);
            if (i >= n) break;
            size_t e = std::min(n, i + 64);
            for (size_t k = i; k < e; k++) {
                double toi;
                if (k < nee) edge_edge_toi(s, x0, x1, c.ee[k][0], c.ee[k][1], 1.0, toi_tol, toi, &local);
                else face_vertex_toi(s, x0, x1, c.fv[k - nee][0], c.fv[k - nee][1], 1.0, toi_tol, toi, &local);
                tois[k] = toi;
            }
        }
        boxes[tid] = local.boxes;
        status[tid] = local.status;
    };
    if (nthreads <= 1) {
        work(0);
    } else {
        std::vector<std::thread> th;
        for (int t = 0; t < nthreads; t++) th.emplace_back(work, t);
        for (auto& t : th) t.join();
    }
    double m = INFINITY;
    for (double t : tois) m = std::min(m, t);
    if (per) *per = tois;
    if (st) {
        for (long long b : boxes) st->boxes += b;
        for (int v : status) st->status = std::max(st->status, v);
    }
    return m;
}

} // namespace orc
