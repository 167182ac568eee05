// Piecewise-linear trajectory CCD over EE and FV candidates.
//
// Replaces compute_earliest_toi_narrow_phase
// (src/opt/distance_barrier_constraint.cpp:151-265) with trajectory
// PIECEWISE_LINEAR: compute_piecewise_linear_edge_edge_time_of_impact and
// compute_piecewise_linear_face_vertex_time_of_impact
// (src/ccd/piecewise_linear/time_of_impact.cpp:326-651).  The time interval
// is cut into pieces over which each body's pose moves linearly
// (Pose::interpolate), the vertices move on straight lines between their
// positions at a piece's ends, and a linear CCD with a minimum separation
// (the interval bound of the rigid trajectory's deviation from the straight
// line, plus dmin) finds the first time the straight-line motions come that
// close.  Piece rules: an impact at the start of a piece whose features came
// below 0.2 of their initial distance (after t = 1e-6); a piece whose
// deviation is >= 0.5 of the features' distance at its start is halved
// (while fewer than 1000 halvings were made, or always at t = 0); an impact
// of the linear CCD at the piece's start halves the piece.
//
// The reference's linear CCD is Tight-Inclusion's inclusion-based root
// finder (Wang et al. 2021); the one here keeps its published method: the
// distance function F(t, u, v) of the straight-line motions is multilinear,
// so its range over a box is the hull of its values at the eight corners
// (evaluated in interval arithmetic); a box whose range misses [-ms, ms]^3
// holds no impact; one inside [-ms, ms]^3 or no wider than 1e-6 + ms in
// every coordinate is a root; others are halved along the dimension with the
// largest change of F between opposite corners, earlier half first; at most
// 10^6 boxes per piece (then the smallest unexplored t.lo, a conservative
// time).
//
// One candidate per warp.  The search state is the same in every lane; a
// box's 8 corners x 3 coordinates are evaluated on 24 lanes (lane 8 j + k:
// coordinate j at corner k), the hull and the changes by shuffles.  The
// piece's straight-line end points come from 4 lanes per end (one vertex
// each) and its deviation bound from 4 (one vertex each: its body's interval
// pose and rotation over the piece).  Every candidate searches t in [0, 1],
// the reference's first candidate's domain; the operations and their order
// are the oracle's, so the per-candidate times of impact are the same bits.
#include <algorithm>

#include "common.cuh"
#include "geometry_rn.cuh"
#include "interval.cuh"
#include "search_tree.cuh"

namespace rigc {

namespace {

constexpr int kPLThreads = 128;
constexpr double kLinearTol = 1e-6;
constexpr long long kLinearMaxBoxes = 1000000;
constexpr int kMaxSubdivisions = 1000;
constexpr int kMaxPieceDepth = 60;
constexpr double kTrajectoryFactor = 0.5;
constexpr double kDecreasingFactor = 0.2;
constexpr double kDecreasingMinTime = 1e-6;

// Every piece is a node of the dyadic bisection tree of [0, 1]
// ([k 2^-d, (k + 1) 2^-d]: the pieces are halvings of [0, 1] visited in order),
// and a body's interval frame over a piece and its rotation at a piece end
// depend on the body and the time only, not on the candidate.  So both are
// computed once per call for the pieces of depth < kPLTableDepth and their
// end points (k_pl_table) and shared by all the body's candidates; deeper
// pieces compute theirs on the spot.  The same operations either way.
constexpr int kPLTableDepth = 7;
constexpr int kPLNodes = (1 << kPLTableDepth) - 1;  // 127 pieces per body
constexpr int kPLPoints = (1 << (kPLTableDepth - 1)) + 1;  // 65 piece ends: k / 64
constexpr int kPLFrame = 24;                         // R (9 intervals) + p (3 intervals)

struct PLArgs {
    const double* rest;
    const int* edges;
    const int* faces;
    const int* vbody;
    const int* ebody;
    const int* fbody;
    const double* x0;
    const double* x1;
    const int2* ee;
    const int2* fv;
    int64_t nee, nfv;
    double dmin;
    double* per;                 // per-candidate time of impact (INFINITY: none)
    unsigned long long* gmin;    // earliest over all candidates (double bits)
    unsigned long long* next;    // next candidate
    unsigned long long* boxes;   // linear-CCD boxes over all candidates
    unsigned long long* pieces;  // pieces over all candidates
    int* status;                 // worst status
    const double* frames;        // per body: kPLNodes piece frames (kPLFrame doubles)
    const double* rots;          // per body: kPLPoints rotations at k / 64 (9 doubles)
};

// the interval pose of a body over a piece between the poses xa, xb (the
// piece's ends) and its interval rotation (time_of_impact.cpp:381-403)
__device__ void piece_frame(const double* xa, const double* xb, Itv R[9], Itv p[3])
{
    const Itv t { 0.0, 1.0 };
    Itv r[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        p[k] = iadd(imul_nonneg(isub(pt(xb[k]), pt(xa[k])), t), pt(xa[k]));
        r[k] = iadd(imul_nonneg(isub(pt(xb[3 + k]), pt(xa[3 + k])), t), pt(xa[3 + k]));
    }
    irotation(r, R);
}

// (x1 - x0) t + x0 per pose coordinate, round to nearest (Pose::interpolate)
__device__ __forceinline__ void pose_lerp(const double* x0, const double* x1, double t, double* x)
{
#pragma unroll
    for (int k = 0; k < 6; k++) x[k] = __dadd_rn(__dmul_rn(__dsub_rn(x1[k], x0[k]), t), x0[k]);
}

// thread per (body, slot): slots 0 .. kPLNodes-1 the piece frames of depth
// < kPLTableDepth, then the kPLPoints rotations at the piece ends
__global__ void k_pl_table(const double* __restrict__ x0, const double* __restrict__ x1, int nb,
                           double* __restrict__ frames, double* __restrict__ rots)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int per = kPLNodes + kPLPoints;
    if (i >= (int64_t)nb * per) return;
    const int b = (int)(i / per), slot = (int)(i % per);
    const double* xb0 = x0 + 6 * b;
    const double* xb1 = x1 + 6 * b;
    if (slot < kPLNodes) {
        const int d = 31 - __clz(slot + 1), k = slot + 1 - (1 << d);
        const double ta = ldexp((double)k, -d), tb = ldexp((double)(k + 1), -d);
        double xa[6], xc[6];
        pose_lerp(xb0, xb1, ta, xa);
        pose_lerp(xb0, xb1, tb, xc);
        Itv R[9], p[3];
        piece_frame(xa, xc, R, p);
        double* o = frames + ((size_t)b * kPLNodes + slot) * kPLFrame;
#pragma unroll
        for (int j = 0; j < 9; j++) {
            o[2 * j] = R[j].lo;
            o[2 * j + 1] = R[j].hi;
        }
#pragma unroll
        for (int j = 0; j < 3; j++) {
            o[18 + 2 * j] = p[j].lo;
            o[19 + 2 * j] = p[j].hi;
        }
    } else {
        const int k = slot - kPLNodes;
        double x[6], R[9];
        pose_lerp(xb0, xb1, ldexp((double)k, -(kPLTableDepth - 1)), x);
        rot_rn(x + 3, R);
        double* o = rots + ((size_t)b * kPLPoints + k) * 9;
#pragma unroll
        for (int j = 0; j < 9; j++) o[j] = R[j];
    }
}

// the node of the piece [ti0, ti1]: pieces are aligned dyadic intervals
// (halvings of [0, 1] visited in order), so ti1 - ti0 = 2^-depth exactly and
// ti0 = k 2^-depth
__device__ __forceinline__ void piece_node(double ti0, double ti1, int& depth, long long& k)
{
    const double len = __dsub_rn(ti1, ti0);
    depth = 1023 - (int)((__double_as_longlong(len) >> 52) & 0x7ff);
    k = (long long)ldexp(ti0, depth);
}

// the frame of a body over the piece (node (1 << depth) + k) between the
// poses xa, xb: from the table for depth < kPLTableDepth
__device__ void body_piece_frame(const PLArgs& a, int body, int depth, long long k, const double* xa,
                                 const double* xb, Itv R[9], Itv p[3])
{
    if (depth < kPLTableDepth) {
        const double* e = a.frames + ((size_t)body * kPLNodes + (1 << depth) - 1 + k) * kPLFrame;
#pragma unroll
        for (int j = 0; j < 9; j++) R[j] = Itv { e[2 * j], e[2 * j + 1] };
#pragma unroll
        for (int j = 0; j < 3; j++) p[j] = Itv { e[18 + 2 * j], e[19 + 2 * j] };
        return;
    }
    piece_frame(xa, xb, R, p);
}

// the rotation of a body at the piece end t = e 2^-depth (pose x there): from
// the table when t is a multiple of 1/64
__device__ void body_point_rot(const PLArgs& a, int body, int depth, long long e, const double* x,
                               double R[9])
{
    if (depth < kPLTableDepth) {
        const double* o = a.rots + ((size_t)body * kPLPoints + (e << (kPLTableDepth - 1 - depth))) * 9;
#pragma unroll
        for (int j = 0; j < 9; j++) R[j] = o[j];
        return;
    }
    rot_rn(x + 3, R);
}

__device__ __forceinline__ double shfl(double v, int src)
{
    return __shfl_sync(0xffffffffu, v, src);
}

// (x1 - x0) t + x0, round to nearest
__device__ __forceinline__ double lerp_rn(double a, double b, double t)
{
    return RADD(RMUL(RSUB(b, a), t), a);
}

__device__ __forceinline__ double pt_sqdist_rn(const double* p, const double* t0, const double* t1,
                                               const double* t2)
{
    switch (pt_type_rn(p, t0, t1, t2)) {
    case PT_P_T0: return pp_sqdist_rn(p, t0);
    case PT_P_T1: return pp_sqdist_rn(p, t1);
    case PT_P_T2: return pp_sqdist_rn(p, t2);
    case PT_P_E0: return pl_sqdist_rn(p, t0, t1);
    case PT_P_E1: return pl_sqdist_rn(p, t1, t2);
    case PT_P_E2: return pl_sqdist_rn(p, t2, t0);
    default: return ptplane_sqdist_rn(p, t0, t1, t2);
    }
}

__device__ __forceinline__ double feature_distance(bool fv, const double P[4][3])
{
    return __dsqrt_rn(fv ? pt_sqdist_rn(P[0], P[1], P[2], P[3]) : ee_sqdist_rn(P[0], P[1], P[2], P[3]));
}

// Every lane gets the four points at the poses pa (body A) and pb (body B):
// lane m < 4 computes point m, the others take it by shuffles.
__device__ void gather_points(const PLArgs& a, const int vid[4], int na, int A, int B,
                              const double* pa, const double* pb, int depth, long long e, int lane,
                              double P[4][3])
{
    double w[3] = { 0, 0, 0 };
    if (lane < 4) {
        const double* x = lane < na ? pa : pb;
        double R[9], v[3];
        body_point_rot(a, lane < na ? A : B, depth, e, x, R);
#pragma unroll
        for (int c = 0; c < 3; c++) v[c] = a.rest[3 * (size_t)vid[lane] + c];
        world_vertex_rn(R, x, v, w);
    }
#pragma unroll
    for (int m = 0; m < 4; m++)
#pragma unroll
        for (int c = 0; c < 3; c++) P[m][c] = shfl(w[c], m);
}

// The largest deviation of each side's vertices from their straight lines
// over the piece between the poses at its ends (pa0 -> pa1, pb0 -> pb1):
// lane m < 4 bounds vertex m; returns the sum of the two sides' largest.
__device__ double piece_deviation(const PLArgs& a, const int vid[4], int na, int A, int B,
                                  const double* pa0, const double* pa1, const double* pb0,
                                  const double* pb1, int depth, long long k, const double P0[4][3],
                                  const double P1[4][3], int lane)
{
    double dev = 0;
    if (lane < 4) {
        const double* xa = lane < na ? pa0 : pb0;
        const double* xb = lane < na ? pa1 : pb1;
        const Itv t { 0.0, 1.0 };
        Itv p[3], R[9];
        body_piece_frame(a, lane < na ? A : B, depth, k, xa, xb, R, p);
        double v[3];
#pragma unroll
        for (int c = 0; c < 3; c++) v[c] = a.rest[3 * (size_t)vid[lane] + c];
        Itv w[3];
        iworld_vertex(R, p, v, w);
        Itv sq { 0.0, 0.0 };
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const Itv line = iadd(imul_nonneg(isub(pt(P1[lane][j]), pt(P0[lane][j])), t), pt(P0[lane][j]));
            const Itv e = isub(w[j], line);
            sq = j == 0 ? imul(e, e) : iadd(sq, imul(e, e));
        }
        dev = isqrt(sq).hi;
    }
    // largest of each side (lanes 0 .. na-1: A; na .. 3: B), then their sum
    double da = 0, db = 0;
#pragma unroll
    for (int m = 0; m < 4; m++) {
        const double d = shfl(dev, m);
        if (m < na) da = da < d ? d : da;
        else db = db < d ? d : db;
    }
    return RADD(da, db);
}

// The linear CCD of one piece by the warp: the first t in [0, 1] at which
// the straight-line motions P0 -> P1 come within ms (INFINITY: none).
__device__ double linear_toi(bool fv, const double P0[4][3], const double P1[4][3], double ms,
                             int lane, long long& boxes, int& status)
{
    // lanes < 24 in three roles per box, lane = 8 j + r for coordinate j:
    //  1. r = 4 it + m: point m's position at t = t_it (it 0: t0, 1: t1);
    //  2. r = 4 it + 2 iw + ab: the edge terms a(t_it, u_iw) (ab = 0) and
    //     b(t_it, v_iw) (ab = 1) of the distance function;
    //  3. r = k: F at corner k = it + 2 iu + 4 iv, b - a combined.
    // The same operations on the same operands as corner by corner.
    const int j = lane >> 3, k = lane & 7;
    const bool clane = lane < 24;
    const int it1 = (k >> 2) & 1, m1 = k & 3;         // role 1
    const int iw2 = (k >> 1) & 1, ab2 = k & 1;        // role 2 (it = it1)
    const int iu3 = (k >> 1) & 1, iv3 = (k >> 2) & 1, it3 = k & 1;  // role 3
    const double p0m = clane ? P0[m1][j] : 0.0, p1m = clane ? P1[m1][j] : 0.0;
    Node cn { { 0, 0, 0 }, { 0ull, 0ull, 0ull }, 0 };
    bool has_cn = true;
    u128 pend = 0, mt = 0, ma = 0;
    double earliest = INFINITY;
    long long n = 0;
    while (has_cn || pend != 0) {
        if (has_cn) {
            has_cn = false;
        } else {
            const int b = msb128(pend);
            pend &= ~bit128(b);
            cn = pending_node(cn, mt, ma, b);
        }
        const double t0 = dyadic(cn.ix[0], cn.lv[0]), t1 = dyadic(cn.ix[0] + 1, cn.lv[0]);
        const double u0 = dyadic(cn.ix[1], cn.lv[1]), u1 = dyadic(cn.ix[1] + 1, cn.lv[1]);
        const double v0 = dyadic(cn.ix[2], cn.lv[2]), v1 = dyadic(cn.ix[2] + 1, cn.lv[2]);
        if (t0 >= earliest) continue;
        if (fv && !(add_dn(u0, v0) <= 1.0)) continue;
        if (n >= kLinearMaxBoxes) {
            double m = t0;
            for (u128 r = pend; r != 0; r &= r - 1) {
                const Node g = pending_node(cn, mt, ma, lsb128(r));
                const double g0 = dyadic(g.ix[0], g.lv[0]);
                m = g0 < m ? g0 : m;
            }
            earliest = m < earliest ? m : earliest;
            status = status > 5 ? status : 5;
            break;
        }
        n++;
        // 1. the points at t0 and t1
        const Itv q = iadd(imul_nonneg(isub(pt(p1m), pt(p0m)), pt(it1 ? t1 : t0)), pt(p0m));
        // 2. the edge terms: EE a = (q1 - q0) u + q0, b = (q3 - q2) v + q2;
        //    FV a = (q2 - q1) u, b = (q3 - q1) v
        const int qb = 8 * j + 4 * it1;  // role-1 lanes of (j, t_it)
        const int sa = fv ? (ab2 ? 3 : 2) : (ab2 ? 3 : 1);
        const int sb = fv ? 1 : (ab2 ? 2 : 0);
        const Itv qa { __shfl_sync(0xffffffffu, q.lo, qb + sa), __shfl_sync(0xffffffffu, q.hi, qb + sa) };
        const Itv qs { __shfl_sync(0xffffffffu, q.lo, qb + sb), __shfl_sync(0xffffffffu, q.hi, qb + sb) };
        const Itv w = pt(ab2 ? (iw2 ? v1 : v0) : (iw2 ? u1 : u0));
        const Itv d = imul_nonneg(isub(qa, qs), w);
        const Itv term = fv ? d : iadd(d, qs);
        // 3. F at corner k
        const int tb0 = 8 * j + 4 * it3;  // role-2 and role-1 lanes of (j, t_it)
        const Itv ta { __shfl_sync(0xffffffffu, term.lo, tb0 + 2 * iu3), __shfl_sync(0xffffffffu, term.hi, tb0 + 2 * iu3) };
        const Itv tb { __shfl_sync(0xffffffffu, term.lo, tb0 + 2 * iv3 + 1),
                       __shfl_sync(0xffffffffu, term.hi, tb0 + 2 * iv3 + 1) };
        Itv y { 0.0, 0.0 };
        if (fv) {
            const Itv q0 { __shfl_sync(0xffffffffu, q.lo, tb0), __shfl_sync(0xffffffffu, q.hi, tb0) };
            const Itv q1 { __shfl_sync(0xffffffffu, q.lo, tb0 + 1), __shfl_sync(0xffffffffu, q.hi, tb0 + 1) };
            if (clane) y = isub(q0, iadd(iadd(ta, tb), q1));
        } else if (clane) {
            y = isub(ta, tb);
        }
        // the changes of F along t, u, v: |mid(corner with the bit) -
        // mid(corner without)|, largest over the lanes
        const double mid = RMUL(0.5, RADD(y.lo, y.hi));
        double ch[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const double other = __shfl_xor_sync(0xffffffffu, mid, 1 << d);
            double c = (clane && !(k & (1 << d))) ? fabs(RSUB(other, mid)) : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double w = __shfl_xor_sync(0xffffffffu, c, o);
                c = c < w ? w : c;
            }
            ch[d] = c;
        }
        // hull over the corners of each coordinate (the 8 lanes of j)
        double lo = y.lo, hi = y.hi;
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) {
            const double l = __shfl_xor_sync(0xffffffffu, lo, o);
            const double h = __shfl_xor_sync(0xffffffffu, hi, o);
            lo = l < lo ? l : lo;
            hi = hi < h ? h : hi;
        }
        const bool meets_j = !clane || (lo <= ms && hi >= -ms);
        const bool inside_j = !clane || (lo >= -ms && hi <= ms);
        const bool small_j = !clane || sub_up(hi, lo) <= RADD(kLinearTol, ms);
        if (!__all_sync(0xffffffffu, meets_j)) continue;
        if (__all_sync(0xffffffffu, inside_j) || __all_sync(0xffffffffu, small_j)) {
            earliest = t0;
            continue;
        }
        int split = 0;
        if (ch[1] > ch[split]) split = 1;
        if (ch[2] > ch[split]) split = 2;
        if (cn.depth >= kMaxDepth || cn.lv[split] >= kMaxLevel) {
            earliest = t0;
            status = status > 4 ? status : 4;
            continue;
        }
        descend(cn, pend, mt, ma, split);
        has_cn = true;
    }
    boxes += n;
    return earliest;
}

// the piecewise-linear time of impact of one candidate (INFINITY: none)
__device__ double pl_toi(const PLArgs& a, bool fv, const int vid[4], int A, int B, int lane,
                         long long& boxes, long long& npieces, int& status)
{
    const int na = fv ? 1 : 2;
    const double* xa0 = a.x0 + 6 * A;
    const double* xa1 = a.x1 + 6 * A;
    const double* xb0 = a.x0 + 6 * B;
    const double* xb1 = a.x1 + 6 * B;
    double P0[4][3], P1[4][3];
    gather_points(a, vid, na, A, B, xa0, xb0, 0, 0, lane, P0);
    const double distance_t0 = feature_distance(fv, P0);
    if (distance_t0 <= a.dmin) return 0.0;
    double ts[kMaxPieceDepth + 1];
    int top = 0;
    ts[0] = 1.0;
    int subdivisions = 1;
    double ti0 = 0;
    double pa0[6], pb0[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
        pa0[k] = xa0[k];
        pb0[k] = xb0[k];
    }
    double result = INFINITY;
    // the points and the distance at ti0 change only when a piece is passed
    // (a halving keeps ti0): P0 holds them for the current ti0
    double distance_ti0 = distance_t0;
    while (top >= 0) {
        const double ti1 = ts[top];
        double pa1[6], pb1[6];
#pragma unroll
        for (int k = 0; k < 6; k++) {
            pa1[k] = lerp_rn(xa0[k], xa1[k], ti1);
            pb1[k] = lerp_rn(xb0[k], xb1[k], ti1);
        }
        if (distance_ti0 < RMUL(kDecreasingFactor, distance_t0) && ti0 >= kDecreasingMinTime) {
            result = ti0;
            break;
        }
        int depth;
        long long k;
        piece_node(ti0, ti1, depth, k);
        gather_points(a, vid, na, A, B, pa1, pb1, depth, k + 1, lane, P1);
        const double dev = piece_deviation(a, vid, na, A, B, pa0, pa1, pb0, pb1, depth, k, P0, P1, lane);
        const bool may_split = top < kMaxPieceDepth;
        if (dev >= RMUL(kTrajectoryFactor, distance_ti0) && (subdivisions < kMaxSubdivisions || ti0 == 0)) {
            if (!may_split) {
                result = ti0;
                status = status > 4 ? status : 4;
                break;
            }
            ts[++top] = RMUL(0.5, RADD(ti1, ti0));
            subdivisions++;
            continue;
        }
        const double t = linear_toi(fv, P0, P1, RADD(dev, a.dmin), lane, boxes, status);
        if (t < INFINITY) {
            const double tt = RADD(RMUL(RSUB(ti1, ti0), t), ti0);
            if (tt == 0) {
                if (!may_split) {
                    result = 0;
                    status = status > 4 ? status : 4;
                    break;
                }
                ts[++top] = RMUL(0.5, RADD(ti1, ti0));
                subdivisions++;
                continue;
            }
            result = tt;
            break;
        }
        top--;
        ti0 = ti1;
#pragma unroll
        for (int k = 0; k < 6; k++) {
            pa0[k] = pa1[k];
            pb0[k] = pb1[k];
        }
#pragma unroll
        for (int m = 0; m < 4; m++)
#pragma unroll
            for (int c = 0; c < 3; c++) P0[m][c] = P1[m][c];
        distance_ti0 = feature_distance(fv, P0);
    }
    npieces += subdivisions;
    return result;
}

// ---------------------------------------------------------------------------
// One candidate per lane: the same operations in the same order, each lane
// on its own candidate (its corners, points and deviations one after the
// other).  An FP64 warp instruction costs the same 64 cycles with one lane
// active as with 32, which favours this form on paper; in practice the
// lanes' searches diverge (3 of 32 lanes active per instruction on the
// 100-icosphere pile) and the warp form is faster, so this one is an option
// (rigc_set_pl_search).

__device__ __forceinline__ void lane_points(const PLArgs& a, const int vid[4], int na, int A, int B,
                                            const double* pa, const double* pb, int depth, long long e,
                                            double P[4][3])
{
    double RA[9], RB[9];
    body_point_rot(a, A, depth, e, pa, RA);
    body_point_rot(a, B, depth, e, pb, RB);
#pragma unroll
    for (int m = 0; m < 4; m++) {
        double v[3];
#pragma unroll
        for (int c = 0; c < 3; c++) v[c] = a.rest[3 * (size_t)vid[m] + c];
        world_vertex_rn(m < na ? RA : RB, m < na ? pa : pb, v, P[m]);
    }
}

// the largest deviation of one side's vertices m0 .. m1-1 over the piece
__device__ double lane_side_deviation(const PLArgs& a, const int vid[4], int m0, int m1, int body,
                                      const double* xa, const double* xb, int depth, long long k,
                                      const double P0[4][3], const double P1[4][3])
{
    const Itv t { 0.0, 1.0 };
    Itv p[3], R[9];
    body_piece_frame(a, body, depth, k, xa, xb, R, p);
    double dev = 0;
    for (int m = m0; m < m1; m++) {
        double v[3];
#pragma unroll
        for (int c = 0; c < 3; c++) v[c] = a.rest[3 * (size_t)vid[m] + c];
        Itv w[3];
        iworld_vertex(R, p, v, w);
        Itv sq { 0.0, 0.0 };
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const Itv line = iadd(imul_nonneg(isub(pt(P1[m][j]), pt(P0[m][j])), t), pt(P0[m][j]));
            const Itv e = isub(w[j], line);
            sq = j == 0 ? imul(e, e) : iadd(sq, imul(e, e));
        }
        const double d = isqrt(sq).hi;
        dev = dev < d ? d : dev;
    }
    return dev;
}

__device__ double lane_linear_toi(bool fv, const double P0[4][3], const double P1[4][3], double ms,
                                  long long& boxes, int& status)
{
    Node cn { { 0, 0, 0 }, { 0ull, 0ull, 0ull }, 0 };
    bool has_cn = true;
    u128 pend = 0, mt = 0, ma = 0;
    double earliest = INFINITY;
    long long n = 0;
    while (has_cn || pend != 0) {
        if (has_cn) {
            has_cn = false;
        } else {
            const int b = msb128(pend);
            pend &= ~bit128(b);
            cn = pending_node(cn, mt, ma, b);
        }
        const double t0 = dyadic(cn.ix[0], cn.lv[0]), t1 = dyadic(cn.ix[0] + 1, cn.lv[0]);
        const double u0 = dyadic(cn.ix[1], cn.lv[1]), u1 = dyadic(cn.ix[1] + 1, cn.lv[1]);
        const double v0 = dyadic(cn.ix[2], cn.lv[2]), v1 = dyadic(cn.ix[2] + 1, cn.lv[2]);
        if (t0 >= earliest) continue;
        if (fv && !(add_dn(u0, v0) <= 1.0)) continue;
        if (n >= kLinearMaxBoxes) {
            double m = t0;
            for (u128 r = pend; r != 0; r &= r - 1) {
                const Node g = pending_node(cn, mt, ma, lsb128(r));
                const double g0 = dyadic(g.ix[0], g.lv[0]);
                m = g0 < m ? g0 : m;
            }
            earliest = m < earliest ? m : earliest;
            status = status > 5 ? status : 5;
            break;
        }
        n++;
        // F at the 8 corners: the hull per coordinate and the corner
        // midpoints.  The points' positions depend on t only and the edge
        // (or face-edge) terms on (t, u) or (t, v), so they are formed once
        // per value and combined per corner: the same operations on the same
        // operands as corner by corner.
        double mid[8][3], lo[3], hi[3];
#pragma unroll
        for (int j = 0; j < 3; j++) {
            Itv q[2][4];
#pragma unroll
            for (int it = 0; it < 2; it++) {
                const Itv t = pt(it ? t1 : t0);
#pragma unroll
                for (int m = 0; m < 4; m++)
                    q[it][m] = iadd(imul_nonneg(isub(pt(P1[m][j]), pt(P0[m][j])), t), pt(P0[m][j]));
            }
            // EE: a(t, u) = (q1 - q0) u + q0, b(t, v) = (q3 - q2) v + q2;
            // FV: a(t, u) = (q2 - q1) u, b(t, v) = (q3 - q1) v
            Itv ta[2][2], tb[2][2];
#pragma unroll
            for (int it = 0; it < 2; it++)
#pragma unroll
                for (int iw = 0; iw < 2; iw++) {
                    const Itv u = pt(iw ? u1 : u0), v = pt(iw ? v1 : v0);
                    const Itv* qt = q[it];
                    if (fv) {
                        ta[it][iw] = imul_nonneg(isub(qt[2], qt[1]), u);
                        tb[it][iw] = imul_nonneg(isub(qt[3], qt[1]), v);
                    } else {
                        ta[it][iw] = iadd(imul_nonneg(isub(qt[1], qt[0]), u), qt[0]);
                        tb[it][iw] = iadd(imul_nonneg(isub(qt[3], qt[2]), v), qt[2]);
                    }
                }
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const int it = k & 1, iu = (k >> 1) & 1, iv = (k >> 2) & 1;
                const Itv y = fv ? isub(q[it][0], iadd(iadd(ta[it][iu], tb[it][iv]), q[it][1]))
                                 : isub(ta[it][iu], tb[it][iv]);
                mid[k][j] = RMUL(0.5, RADD(y.lo, y.hi));
                if (k == 0) {
                    lo[j] = y.lo;
                    hi[j] = y.hi;
                } else {
                    lo[j] = y.lo < lo[j] ? y.lo : lo[j];
                    hi[j] = hi[j] < y.hi ? y.hi : hi[j];
                }
            }
        }
        double ch[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            double c = 0;
#pragma unroll
            for (int k = 0; k < 8; k++) {
                if (k & (1 << d)) continue;
#pragma unroll
                for (int j = 0; j < 3; j++) {
                    const double x = fabs(RSUB(mid[k | (1 << d)][j], mid[k][j]));
                    c = c < x ? x : c;
                }
            }
            ch[d] = c;
        }
        bool meets = true, inside = true, small = true;
#pragma unroll
        for (int j = 0; j < 3; j++) {
            meets = meets && lo[j] <= ms && hi[j] >= -ms;
            inside = inside && lo[j] >= -ms && hi[j] <= ms;
            small = small && sub_up(hi[j], lo[j]) <= RADD(kLinearTol, ms);
        }
        if (!meets) continue;
        if (inside || small) {
            earliest = t0;
            continue;
        }
        int split = 0;
        if (ch[1] > ch[split]) split = 1;
        if (ch[2] > ch[split]) split = 2;
        if (cn.depth >= kMaxDepth || cn.lv[split] >= kMaxLevel) {
            earliest = t0;
            status = status > 4 ? status : 4;
            continue;
        }
        descend(cn, pend, mt, ma, split);
        has_cn = true;
    }
    boxes += n;
    return earliest;
}

__device__ double lane_pl_toi(const PLArgs& a, bool fv, const int vid[4], int A, int B,
                              long long& boxes, long long& npieces, int& status)
{
    const int na = fv ? 1 : 2;
    const double* xa0 = a.x0 + 6 * A;
    const double* xa1 = a.x1 + 6 * A;
    const double* xb0 = a.x0 + 6 * B;
    const double* xb1 = a.x1 + 6 * B;
    double P0[4][3], P1[4][3];
    lane_points(a, vid, na, A, B, xa0, xb0, 0, 0, P0);
    const double distance_t0 = feature_distance(fv, P0);
    if (distance_t0 <= a.dmin) return 0.0;
    double ts[kMaxPieceDepth + 1];
    int top = 0;
    ts[0] = 1.0;
    int subdivisions = 1;
    double ti0 = 0;
    double pa0[6], pb0[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
        pa0[k] = xa0[k];
        pb0[k] = xb0[k];
    }
    double result = INFINITY;
    double distance_ti0 = distance_t0;
    while (top >= 0) {
        const double ti1 = ts[top];
        double pa1[6], pb1[6];
#pragma unroll
        for (int k = 0; k < 6; k++) {
            pa1[k] = lerp_rn(xa0[k], xa1[k], ti1);
            pb1[k] = lerp_rn(xb0[k], xb1[k], ti1);
        }
        if (distance_ti0 < RMUL(kDecreasingFactor, distance_t0) && ti0 >= kDecreasingMinTime) {
            result = ti0;
            break;
        }
        int depth;
        long long k;
        piece_node(ti0, ti1, depth, k);
        lane_points(a, vid, na, A, B, pa1, pb1, depth, k + 1, P1);
        const double dev = RADD(lane_side_deviation(a, vid, 0, na, A, pa0, pa1, depth, k, P0, P1),
                                lane_side_deviation(a, vid, na, 4, B, pb0, pb1, depth, k, P0, P1));
        const bool may_split = top < kMaxPieceDepth;
        if (dev >= RMUL(kTrajectoryFactor, distance_ti0) && (subdivisions < kMaxSubdivisions || ti0 == 0)) {
            if (!may_split) {
                result = ti0;
                status = status > 4 ? status : 4;
                break;
            }
            ts[++top] = RMUL(0.5, RADD(ti1, ti0));
            subdivisions++;
            continue;
        }
        const double t = lane_linear_toi(fv, P0, P1, RADD(dev, a.dmin), boxes, status);
        if (t < INFINITY) {
            const double tt = RADD(RMUL(RSUB(ti1, ti0), t), ti0);
            if (tt == 0) {
                if (!may_split) {
                    result = 0;
                    status = status > 4 ? status : 4;
                    break;
                }
                ts[++top] = RMUL(0.5, RADD(ti1, ti0));
                subdivisions++;
                continue;
            }
            result = tt;
            break;
        }
        top--;
        ti0 = ti1;
#pragma unroll
        for (int k = 0; k < 6; k++) {
            pa0[k] = pa1[k];
            pb0[k] = pb1[k];
        }
#pragma unroll
        for (int m = 0; m < 4; m++)
#pragma unroll
            for (int c = 0; c < 3; c++) P0[m][c] = P1[m][c];
        distance_ti0 = feature_distance(fv, P0);
    }
    npieces += subdivisions;
    return result;
}

// the candidate's vertices (EE: a0 a1 b0 b1; FV: v f0 f1 f2) and bodies
__device__ __forceinline__ bool pl_candidate(const PLArgs& a, int64_t w, int vid[4], int& A, int& B)
{
    if (w < a.nee) {
        const int ea = a.ee[w].x, eb = a.ee[w].y;
        vid[0] = a.edges[2 * ea];
        vid[1] = a.edges[2 * ea + 1];
        vid[2] = a.edges[2 * eb];
        vid[3] = a.edges[2 * eb + 1];
        A = a.ebody[ea];
        B = a.ebody[eb];
        return false;
    }
    const int f = a.fv[w - a.nee].x, v = a.fv[w - a.nee].y;
    vid[0] = v;
    vid[1] = a.faces[3 * f];
    vid[2] = a.faces[3 * f + 1];
    vid[3] = a.faces[3 * f + 2];
    A = a.vbody[v];
    B = a.fbody[f];
    return true;
}

__global__ void __launch_bounds__(kPLThreads) k_pl_ccd_lane(PLArgs a)
{
    const int64_t n = a.nee + a.nfv;
    long long boxes = 0, npieces = 0;
    int status = RIGC_OK;
    double local_min = INFINITY;
    while (true) {
        const long long w = (long long)atomicAdd(a.next, 1ull);
        if (w >= n) break;
        int vid[4], A, B;
        const bool fv = pl_candidate(a, w, vid, A, B);
        const double toi = lane_pl_toi(a, fv, vid, A, B, boxes, npieces, status);
        if (a.per) a.per[w] = toi;
        local_min = toi < local_min ? toi : local_min;
    }
    if (local_min < INFINITY) atomicMin(a.gmin, (unsigned long long)__double_as_longlong(local_min));
    atomicAdd(a.boxes, (unsigned long long)boxes);
    atomicAdd(a.pieces, (unsigned long long)npieces);
    if (status != RIGC_OK) atomicMax(a.status, status);
}

__global__ void __launch_bounds__(kPLThreads) k_pl_ccd(PLArgs a)
{
    const int lane = threadIdx.x & 31;
    const int64_t n = a.nee + a.nfv;
    long long boxes = 0, npieces = 0;
    int status = RIGC_OK;
    double local_min = INFINITY;
    while (true) {
        long long w = 0;
        if (lane == 0) w = (long long)atomicAdd(a.next, 1ull);
        w = __shfl_sync(0xffffffffu, w, 0);
        if (w >= n) break;
        int vid[4], A, B;
        const bool fv = pl_candidate(a, w, vid, A, B);
        const double toi = pl_toi(a, fv, vid, A, B, lane, boxes, npieces, status);
        if (lane == 0 && a.per) a.per[w] = toi;
        local_min = toi < local_min ? toi : local_min;
    }
    if (lane == 0) {
        if (local_min < INFINITY) atomicMin(a.gmin, (unsigned long long)__double_as_longlong(local_min));
        atomicAdd(a.boxes, (unsigned long long)boxes);
        atomicAdd(a.pieces, (unsigned long long)npieces);
        if (status != RIGC_OK) atomicMax(a.status, status);
    }
}

} // namespace

// counters in the context's device scalars (byte offset 512): [0] earliest
// time of impact (bits), [1] boxes, [2] pieces, [3] status, [4] next
int run_pl_ccd(Ctx& c, const double* x0, const double* x1, double dmin, double* toi_host, double* per)
{
    cudaStream_t st = c.stream;
    const int64_t n = c.cand.num_ee + c.cand.num_fv;
    unsigned long long* cnt = reinterpret_cast<unsigned long long*>(c.d_scalars.as<char>() + 512);
    const unsigned long long init[5] = { 0x7ff0000000000000ull, 0, 0, 0, 0 };
    RIGC_CUDA(cudaMemcpyAsync(cnt, init, sizeof(init), cudaMemcpyHostToDevice, st));
    if (n > 0) {
        PLArgs a;
        a.rest = c.s.rest;
        a.edges = c.s.edges;
        a.faces = c.s.faces;
        a.vbody = c.s.vbody;
        a.ebody = c.s.ebody;
        a.fbody = c.s.fbody;
        a.x0 = x0;
        a.x1 = x1;
        a.ee = c.cand.ee.as<int2>();
        a.fv = c.cand.fv.as<int2>();
        a.nee = c.cand.num_ee;
        a.nfv = c.cand.num_fv;
        a.dmin = dmin;
        a.per = per;
        a.gmin = cnt;
        a.boxes = cnt + 1;
        a.pieces = cnt + 2;
        a.status = reinterpret_cast<int*>(cnt + 3);
        a.next = cnt + 4;
        const size_t frame_doubles = (size_t)c.s.nb * kPLNodes * kPLFrame;
        RIGC_TRY(c.pl_table.reserve((frame_doubles + (size_t)c.s.nb * kPLPoints * 9) * sizeof(double)));
        a.frames = c.pl_table.as<double>();
        a.rots = c.pl_table.as<double>() + frame_doubles;
        RIGC_COUNT_LAUNCH();
        k_pl_table<<<grid_for((int64_t)c.s.nb * (kPLNodes + kPLPoints), 128), 128, 0, st>>>(
            x0, x1, c.s.nb, const_cast<double*>(a.frames), const_cast<double*>(a.rots));
        int dev = 0, sms = kNumSMs;
        RIGC_CUDA(cudaGetDevice(&dev));
        RIGC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        // one candidate per warp unless tuned to one per lane (per warp
        // measured faster on every workload here once the piece frames come
        // from the table: 0.61 against 2.10 s on the 1000-icosphere pile)
        const bool per_lane = c.tune.pl_per_lane == 1;
        int blocks = 0;
        if (per_lane)
            RIGC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_pl_ccd_lane, kPLThreads, 0));
        else
            RIGC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_pl_ccd, kPLThreads, 0));
        const int per_block = per_lane ? kPLThreads : kPLThreads / 32;
        const int64_t want = (n + per_block - 1) / per_block;
        const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * std::max(1, blocks)));
        RIGC_COUNT_LAUNCH();
        if (per_lane) k_pl_ccd_lane<<<grid, kPLThreads, 0, st>>>(a);
        else k_pl_ccd<<<grid, kPLThreads, 0, st>>>(a);
        RIGC_CUDA(cudaGetLastError());
    }
    unsigned long long out[4];
    RIGC_CUDA(cudaMemcpyAsync(out, cnt, sizeof(out), cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaStreamSynchronize(st));
    double g;
    std::memcpy(&g, &out[0], sizeof(g));
    *toi_host = g;
    c.stats.ccd_boxes = (int64_t)out[1];
    c.stats.ccd_candidates = n;
    c.stats.last_status = (int)(out[3] & 0xffffffffu);
    return c.stats.last_status;
}

} // namespace rigc
