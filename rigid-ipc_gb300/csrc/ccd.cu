// Conservative rigid-trajectory interval CCD over EE and FV candidates.
//
// Replaces compute_earliest_toi_narrow_phase
// (src/opt/distance_barrier_constraint.cpp:151-265) with trajectory RIGID:
// compute_edge_edge_time_of_impact / compute_face_vertex_time_of_impact
// (src/ccd/rigid/time_of_impact.cpp:158-310) over the interval point
// functions of src/ccd/rigid/rigid_trajectory_aabb.cpp:7-103, searched by the
// branch and bound of src/interval/interval_root_finder.cpp:97-203:
//  * boxes (t, alpha, beta) / (t, u, v) start at [0, 1]^3;
//  * if f([0, tol]) contains zero the time tolerance shrinks 100x;
//  * a box is skipped when its t.lo is not before the earliest root found,
//    when (FV) u + v misses [0, 1], or when f(box) excludes zero;
//  * a box within tolerance (and with t.lo > 0 or all widths <= 1e-10)
//    becomes the new earliest root; otherwise it is split at the midpoint of
//    the dimension with the largest width / tolerance, second half pushed
//    first.
// The time of impact of a candidate (the t.lo of its earliest root box) does
// not depend on the order boxes are visited, so boxes whose t.lo is not below
// the running minimum over all candidates can be skipped too: that never
// changes the minimum.  One thread per candidate at a time, a depth-first
// search whose pending boxes are encoded as bits of the current tree path (in
// registers, no stack in memory), the interval vertex positions cached per
// time interval; the warp advances in lock step, one box per lane per iteration
// (a lane whose search ends takes the next candidate in the same iteration),
// and the per-candidate set-up that needs no search (tolerances, the
// tolerance test) runs beforehand in a kernel of its own.  The
// interval frames R(t), p(t) of a body depend only on the body and the time
// interval, which is always a node of the dyadic bisection tree of [0, 1]:
// the top levels come from a table built per call, deeper nodes from a hash
// table shared by all candidates of the body.  A lane whose box needs a frame
// that is not there yet pushes the box back; at the top of the next
// iteration the whole warp computes that frame together with its sibling and
// their descendants three levels down (one converged pass instead of many
// single-lane ones) and publishes them.  Every search is bounded in depth
// (kMaxDepth splits, kMaxLevel per dimension) and in boxes: on overflow or
// budget exhaustion the candidate reports the smallest t.lo still unexplored
// (a conservative time of impact) and an error status.
#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "interval.cuh"
#include "search_tree.cuh"

namespace rigc {

constexpr int kCCDThreads = 128;
// search pieces: boxes a piece evaluates before handing off its pending
// boxes (built-in choice), slots per hand-off buffer, launches per call
constexpr int kHandOff = 64;
constexpr unsigned long long kPiecesCap = 1ull << 18;
constexpr int kMaxLaunches = 32;
// time windows (search groups, prune mode): the first window 2^-k (built-in
// k, from kWindowMinCandidates candidates on: below, the launches they add
// cost more than the boxes they skip), each later launch's twice the last
// one's, none from 1 on; slots per piece buffer at most kWindowCap
constexpr int kWindowLog2 = 6;
constexpr int64_t kWindowMinCandidates = 1 << 16;
constexpr unsigned long long kWindowCap = 1ull << 22;

struct CCDArgs {
    const double* rest;
    const int* edges;
    const int* faces;
    const int* f2e;
    const int* vbody;
    const int* ebody;
    const int* fbody;
    const double* edge_len;
    const double* x0;
    const double* x1;
    const int2* ee;
    const int2* fv;
    int64_t nee, nfv;
    double toi_tol;
    int prune;
    int seeds_log2;             // prune mode: each candidate's search starts from the
                                // 2^seeds_log2 boxes of its subdivision tree at that depth
    long long max_boxes;
    unsigned long long* gmin;   // running minimum time of impact (double bits)
    unsigned long long* scene_gmin;  // batched contexts: the same per scene, else null
    const int* bscene;          // scene of each body
    double* per;                // optional per-candidate result
    int* status;                // worst status
    unsigned long long* boxes;  // total boxes evaluated
    unsigned long long* hits;   // candidates with an impact
    unsigned long long* next;   // next unprocessed candidate
    const double* table;        // per-body frames over the top dyadic time intervals
    unsigned long long* fkeys;  // frame cache: keys (0 = empty)
    double* fvals;              // frame cache: kTableEntry doubles per slot
    unsigned long long fmask;   // slots - 1 (a power of two)
    const double* traj;         // per body: x0 (6), I(x1) - I(x0) (6 intervals)
    const int* bfixed;          // per body: 1 when the body does not move
    double* ctol;               // per candidate: the three tolerances
    // Search pieces (prune mode).  Once the work list is exhausted (a lane of
    // the warp is idle), a lane whose current piece has evaluated hand_off
    // boxes writes its pending boxes to pieces_out and ends the piece; the
    // next launch of the call searches pieces_in instead of the candidates'
    // seeds, so the deep searches of the tail spread over the whole GPU.
    const struct Piece* pieces_in;
    long long n_pieces;         // pieces in pieces_in (launch 0: none, seeds)
    struct Piece* pieces_out;
    unsigned long long* n_out;
    unsigned long long out_cap;
    unsigned long long hand_off;  // boxes per piece before a hand-off (0: never)
    // Time window (prune mode, search groups): a box starting at or after
    // it is written to pieces_out instead of being searched, and the next
    // launch searches it under a later window (+inf: no window).  The boxes
    // of all candidates are so searched roughly in time order, and the
    // running minimum, once some candidate's root is found, skips the boxes
    // after it in every candidate.
    double window;
};

struct Box {
    double t0, t1, a0, a1, b0, b1;
};

// One piece of a candidate's search: the subtree below a node, the earliest
// root time found so far (boxes at or after it are skipped) and the boxes
// the search path leading to it has evaluated (the budget counts along
// every path).  cand < 0 marks an unused slot.
struct Piece {
    long long cand;
    double earliest;
    unsigned long long ix[3];
    int lv[3];
    int depth;
    unsigned long long boxes;
};

struct BodyTraj {
    double x0[6];
    Itv dx[6];  // I(x1) - I(x0)
};

constexpr int kTrajDoubles = 18;

__device__ __forceinline__ void load_traj(const double* x0, const double* x1, int b, BodyTraj& T)
{
#pragma unroll
    for (int k = 0; k < 6; k++) {
        double a = x0[6 * b + k], c = x1[6 * b + k];
        T.x0[k] = a;
        T.dx[k] = Itv { sub_dn(c, a), sub_up(c, a) };
    }
}

__device__ __forceinline__ void traj_from_table(const double* traj, int b, BodyTraj& T)
{
    const double* e = traj + (size_t)b * kTrajDoubles;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        T.x0[k] = e[k];
        T.dx[k] = Itv { e[6 + 2 * k], e[7 + 2 * k] };
    }
}

// R(t), p(t) of a body over the time interval t
__device__ __forceinline__ void body_at(const BodyTraj& T, const Itv& t, Itv R[9], Itv p[3])
{
    Itv r[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        p[k] = iadd(imul_nonneg(T.dx[k], t), pt(T.x0[k]));
        r[k] = iadd(imul_nonneg(T.dx[3 + k], t), pt(T.x0[3 + k]));
    }
    irotation(r, R);
}

// Bisection-tree node of a time interval: (1 << d) + k for [k 2^-d, (k + 1) 2^-d]
// with d < kNodeDepth, else 0.  Every time interval of the search is such a
// node (midpoints of dyadic intervals are exact), up to depth 1074.
constexpr int kNodeDepth = 40;

// t * 2^52 for t in [0, 1] when that is an integer, else ~0 (bit operations)
__device__ __forceinline__ unsigned long long fixed52(double t)
{
    const unsigned long long b = (unsigned long long)dbits(t);
    if (b == 0) return 0;
    const int e = (int)(b >> 52);                      // biased exponent, t > 0
    const unsigned long long m = (b & 0xfffffffffffffull) | (1ull << 52);
    const int sh = 1023 - e;                           // t * 2^52 = m >> sh
    if (e == 0 || sh < 0 || sh > 52) return ~0ull;     // subnormal, > 1 or < 2^-52
    if (m & ((1ull << sh) - 1)) return ~0ull;          // not a multiple of 2^-52
    return m >> sh;
}

__device__ __forceinline__ unsigned long long time_node(double t0, double t1)
{
    const unsigned long long k0 = fixed52(t0), k1 = fixed52(t1);
    if (k0 == ~0ull || k1 == ~0ull || k1 <= k0) return 0;
    const unsigned long long w = k1 - k0;              // 2^(52 - d) for a node
    if (w & (w - 1)) return 0;
    const int lw = 63 - __clzll((long long)w);
    if (k0 & (w - 1)) return 0;                        // aligned to its width
    const int d = 52 - lw;
    if (d >= kNodeDepth) return 0;
    return (1ull << d) + (k0 >> lw);
}

// Frame cache: an open-addressing hash table of (body, time node) -> R(t),
// p(t) intervals shared by every thread of the launch.  A slot is claimed by
// a compare-and-swap of its key with the pending bit set, filled, and
// published by clearing the bit after a fence; readers acquire the key and
// read the frame through L2.  A thread that meets a pending slot, or that
// finds no slot within kProbes, computes the frame itself: the cache only
// skips recomputation, the bits are the same either way.
constexpr unsigned long long kPending = 1ull << 63;
constexpr int kProbes = 16;

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p)
{
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long x)
{
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

__device__ __forceinline__ void frame_store(double* o, const Itv R[9], const Itv p[3])
{
#pragma unroll
    for (int j = 0; j < 9; j++) {
        o[2 * j] = R[j].lo;
        o[2 * j + 1] = R[j].hi;
    }
#pragma unroll
    for (int j = 0; j < 3; j++) {
        o[18 + 2 * j] = p[j].lo;
        o[18 + 2 * j + 1] = p[j].hi;
    }
}

// Interval rotation and position of every body over the dyadic time
// intervals [k 2^-d, (k + 1) 2^-d] of the first kTableDepth levels of the
// bisection tree (slot (1 << d) - 1 + k), and over [0, toi_tol] (the
// interval of the tolerance test every candidate starts with, slot
// kTableNodes), computed once per call and shared by all candidates of the
// body.  The same operations produce the same bits as evaluating them inside
// a box.
constexpr int kTableDepth = 7;                          // levels 0..6
constexpr int kTableNodes = (1 << kTableDepth) - 1;     // 127
constexpr int kTableSlots = kTableNodes + 1;            // + [0, toi_tol]
constexpr int kTableEntry = 24;                         // R (9 intervals) + p (3)
static_assert(kTableSlots == kRotTableSlots && kTableEntry == kRotTableEntry, "table layout");

// a body's trajectory (x0, I(x1) - I(x0)) and fixed flag
__device__ __forceinline__ void store_traj(const BodyTraj& T, int b, double* __restrict__ traj,
                                           int* __restrict__ bfixed)
{
    double* e = traj + (size_t)b * kTrajDoubles;
    bool fixed = true;
    for (int k = 0; k < 6; k++) {
        e[k] = T.x0[k];
        e[6 + 2 * k] = T.dx[k].lo;
        e[7 + 2 * k] = T.dx[k].hi;
        fixed = fixed && is_zero(T.dx[k].lo) && is_zero(T.dx[k].hi);
    }
    bfixed[b] = fixed ? 1 : 0;
}

// tree_ready: the slots of the tree nodes already hold these poses' frames
// for every body a candidate can have (the continuous broad phase computed
// them); only [0, toi_tol], the trajectories and the fixed flags are left
__global__ void k_rot_table(const double* __restrict__ x0, const double* __restrict__ x1, int nb,
                            double toi_tol, double* __restrict__ table, double* __restrict__ traj,
                            int* __restrict__ bfixed, int tree_ready)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)nb * kTableSlots) return;
    int b = (int)(i / kTableSlots), node = (int)(i % kTableSlots);
    int d = 31 - __clz(node + 1);
    int k = node + 1 - (1 << d);
    Itv t { ldexp((double)k, -d), ldexp((double)(k + 1), -d) };
    if (node == kTableNodes) t = Itv { 0.0, toi_tol };
    BodyTraj T;
    load_traj(x0, x1, b, T);
    Itv R[9], p[3];
    if (!tree_ready || node == kTableNodes) {
        body_at(T, t, R, p);
        frame_store(table + (size_t)i * kTableEntry, R, p);
    }
    if (node == 0) store_traj(T, b, traj, bfixed);
}

// every slot, [0, toi_tol] included, already holds these poses' frames:
// the trajectories and fixed flags alone, one thread per body
__global__ void k_traj_table(const double* __restrict__ x0, const double* __restrict__ x1, int nb,
                             double* __restrict__ traj, int* __restrict__ bfixed)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    BodyTraj T;
    load_traj(x0, x1, b, T);
    store_traj(T, b, traj, bfixed);
}


struct Query {
    bool fv;            // face-vertex (else edge-edge)
    bool a_fixed;       // body A does not move: its vertex intervals never change
    bool b_fixed;
    bool fresh;         // no vertex interval computed yet for this candidate
    int body_a, body_b;
    double v[4][3];     // rest vertices: EE (a0, a1, b0, b1); FV (v, f0, f1, f2)
    // cached vertex intervals for one time interval
    double ct0, ct1;
    Itv P[4][3];
};

__device__ __forceinline__ void frame_load(const double* e, Itv R[9], Itv p[3])
{
#pragma unroll
    for (int j = 0; j < 9; j++) R[j] = Itv { e[2 * j], e[2 * j + 1] };
#pragma unroll
    for (int j = 0; j < 3; j++) p[j] = Itv { e[18 + 2 * j], e[18 + 2 * j + 1] };
}

__device__ __forceinline__ void frame_load_cg(const double* e, Itv R[9], Itv p[3])
{
#pragma unroll
    for (int j = 0; j < 9; j++) R[j] = Itv { __ldcg(e + 2 * j), __ldcg(e + 2 * j + 1) };
#pragma unroll
    for (int j = 0; j < 3; j++) p[j] = Itv { __ldcg(e + 18 + 2 * j), __ldcg(e + 19 + 2 * j) };
}

// frame of a body over a time interval computed from its trajectory
static __device__ __noinline__ void frame_compute(const CCDArgs& a, int body, const Itv& t,
                                                  Itv R[9], Itv p[3])
{
    BodyTraj T;
    traj_from_table(a.traj, body, T);
    body_at(T, t, R, p);
}

// Frame cache lookup: true (and the frame) when the key is published.
__device__ __forceinline__ bool cache_find(const CCDArgs& a, unsigned long long key, Itv R[9],
                                          Itv p[3])
{
    unsigned long long h = mix64(key);
    for (int probe = 0; probe < kProbes; probe++, h++) {
        const unsigned long long k = ld_acquire(a.fkeys + (h & a.fmask));
        if (k == key) {
            frame_load_cg(a.fvals + (h & a.fmask) * kTableEntry, R, p);
            return true;
        }
        if (k == 0 || k == (key | kPending)) return false;
    }
    return false;
}

// Publish a frame unless the key is present or claimed, or no slot is free
// within kProbes.
__device__ __forceinline__ void cache_insert(const CCDArgs& a, unsigned long long key,
                                             const Itv R[9], const Itv p[3])
{
    unsigned long long h = mix64(key);
    for (int probe = 0; probe < kProbes; probe++, h++) {
        unsigned long long* slot = a.fkeys + (h & a.fmask);
        unsigned long long k = ld_acquire(slot);
        if (k == 0) k = atomicCAS(slot, 0ull, key | kPending);
        if (k == 0) {
            frame_store(a.fvals + (h & a.fmask) * kTableEntry, R, p);
            __threadfence();
            atomicExch(slot, key);
            return;
        }
        if (k == key || k == (key | kPending)) return;
    }
}

__device__ __forceinline__ unsigned long long frame_key(int body, unsigned long long node)
{
    return ((unsigned long long)(body + 1) << kNodeDepth) | node;
}

// Frames of the two sides (body A, body B) a lane received in the last
// batched computation, so that the box that asked for them can always go on.
struct OwnFrames {
    unsigned long long key[2];
    double f[2][kTableEntry];
};

// Frame of a body over t: the table, the lane's own frames, the cache; a
// time interval that is not a tree node is computed on the spot.  False
// when the frame still has to be computed.
__device__ __forceinline__ bool frame_find(const CCDArgs& a, const OwnFrames& own, int side,
                                          int body, unsigned long long node, const Itv& t,
                                          Itv R[9], Itv p[3])
{
    if (node != 0 && node < (1ull << kTableDepth)) {
        frame_load(a.table + ((size_t)body * kTableSlots + (node - 1)) * kTableEntry, R, p);
        return true;
    }
    if (node == 0) {
        frame_compute(a, body, t, R, p);
        return true;
    }
    const unsigned long long key = frame_key(body, node);
    if (own.key[side] == key) {
        frame_load(own.f[side], R, p);
        return true;
    }
    return cache_find(a, key, R, p);
}

// Vertex intervals of the bodies over t (a body that does not move has
// t-independent intervals: computed at the candidate's first evaluation
// only).  Returns 0, or a mask of the sides whose frame is missing (the
// cached intervals are then left invalid).
static __device__ __noinline__ int eval_vertices(const CCDArgs& a, const OwnFrames& own, Query& q,
                                                 const Itv& t)
{
    Itv R[9], p[3];
    const int na = q.fv ? 1 : 2;
    const unsigned long long node = time_node(t.lo, t.hi);
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    q.ct0 = q.ct1 = nan;
    int miss = 0;
    if (q.fresh || !q.a_fixed) {
        if (frame_find(a, own, 0, q.body_a, node, t, R, p)) {
            for (int i = 0; i < na; i++) iworld_vertex(R, p, q.v[i], q.P[i]);
        } else {
            miss |= 1;
        }
    }
    if (q.fresh || !q.b_fixed) {
        if (frame_find(a, own, 1, q.body_b, node, t, R, p)) {
            for (int i = na; i < 4; i++) iworld_vertex(R, p, q.v[i], q.P[i]);
        } else {
            miss |= 2;
        }
    }
    if (miss) return miss;
    q.fresh = false;
    q.ct0 = t.lo;
    q.ct1 = t.hi;
    return 0;
}

// Batched frame computation, executed by a group of W lanes (the whole
// warp, or one half of it).  For each lane of the group with a missing frame
// (body, node n at depth d), the W - 1 other lanes compute the frames of the
// subtree below n's parent (n, its sibling and their descendants down to
// depth d + 3 for a warp, d + 2 for a half-warp), publish them in the cache,
// and the requesting lane (every lane of the group with to_all) receives n's
// frame.  The depth-first search keeps asking for those nodes, so one
// converged pass replaces up to W - 1 single-lane rotation enclosures.
template <int W>
static __device__ __noinline__ void group_compute_frames(const CCDArgs& a, OwnFrames& own,
                                                         unsigned req, int req_side,
                                                         int req_body,
                                                         unsigned long long req_node,
                                                         bool to_all = false)
{
    const int lane = threadIdx.x & 31;
    const int gl = lane & (W - 1);
    const unsigned gmask = W == 32 ? 0xffffffffu : (0xffffu << (lane & 16));
    while (req) {
        const int src = __ffs(req) - 1;
        req &= req - 1;
        const int side = __shfl_sync(gmask, req_side, src, W);
        const int body = __shfl_sync(gmask, req_body, src, W);
        const unsigned long long node = __shfl_sync(gmask, req_node, src, W);
        const int d = 63 - __clzll((long long)node);           // node depth (>= kTableDepth)
        const unsigned long long root = node >> 1;             // depth d - 1
        // lane L < W - 1: subtree node L + 1 below root, level l = log2(L + 1)
        const int l = 31 - __clz(gl + 1);
        const unsigned long long mine = (root << l) + (unsigned long long)(gl + 1 - (1 << l));
        const int dm = d - 1 + l;
        Itv R[9], p[3];
        const bool work = gl < W - 1 && l >= 1 && dm < kNodeDepth;
        if (work) {
            const unsigned long long k = mine - (1ull << dm);
            const Itv t { ldexp((double)k, -dm), ldexp((double)(k + 1), -dm) };
            frame_compute(a, body, t, R, p);
            cache_insert(a, frame_key(body, mine), R, p);
        }
        // hand n's frame to the lane that asked for it
        const int owner = (int)(node - (root << 1)) + 1;       // lane of n (level 1)
        double f[kTableEntry];
#pragma unroll
        for (int j = 0; j < 9; j++) {
            f[2 * j] = __shfl_sync(gmask, R[j].lo, owner, W);
            f[2 * j + 1] = __shfl_sync(gmask, R[j].hi, owner, W);
        }
#pragma unroll
        for (int j = 0; j < 3; j++) {
            f[18 + 2 * j] = __shfl_sync(gmask, p[j].lo, owner, W);
            f[19 + 2 * j] = __shfl_sync(gmask, p[j].hi, owner, W);
        }
        if (to_all || gl == src) {
            own.key[side] = frame_key(body, node);
#pragma unroll
            for (int j = 0; j < kTableEntry; j++) own.f[side][j] = f[j];
        }
    }
}

// zero in f(box), with the vertex intervals already at the box's t
__device__ __forceinline__ bool f_zero(const Query& q, const Box& x)
{
    Itv a { x.a0, x.a1 }, b { x.b0, x.b1 };
#pragma unroll
    for (int j = 0; j < 3; j++) {
        Itv y;
        if (q.fv) {
            Itv fp = iadd(iadd(imul_nonneg(isub(q.P[2][j], q.P[1][j]), a),
                               imul_nonneg(isub(q.P[3][j], q.P[1][j]), b)),
                          q.P[1][j]);
            y = isub(q.P[0][j], fp);
        } else {
            Itv ea = iadd(imul_nonneg(isub(q.P[1][j], q.P[0][j]), a), q.P[0][j]);
            Itv eb = iadd(imul_nonneg(isub(q.P[3][j], q.P[2][j]), b), q.P[2][j]);
            y = isub(ea, eb);
        }
        if (!zero_in(y)) return false;
    }
    return true;
}

// rest vertices and bodies of candidate i
__device__ __forceinline__ void load_candidate(const CCDArgs& a, int64_t i, Query& q)
{
    int vid[4];
    if (i < a.nee) {
        q.fv = false;
        int ea = a.ee[i].x, eb = a.ee[i].y;
        vid[0] = a.edges[2 * ea];
        vid[1] = a.edges[2 * ea + 1];
        vid[2] = a.edges[2 * eb];
        vid[3] = a.edges[2 * eb + 1];
        q.body_a = a.ebody[ea];
        q.body_b = a.ebody[eb];
    } else {
        q.fv = true;
        int64_t k = i - a.nee;
        int f = a.fv[k].x, v = a.fv[k].y;
        vid[0] = v;
        vid[1] = a.faces[3 * f];
        vid[2] = a.faces[3 * f + 1];
        vid[3] = a.faces[3 * f + 2];
        q.body_a = a.vbody[v];
        q.body_b = a.fbody[f];
    }
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
        for (int j = 0; j < 3; j++) q.v[k][j] = a.rest[3 * (size_t)vid[k] + j];
    q.a_fixed = a.bfixed[q.body_a] != 0;
    q.b_fixed = a.bfixed[q.body_b] != 0;
    q.fresh = true;
    q.ct0 = q.ct1 = __longlong_as_double(0x7ff8000000000000ll);
}

// Per-candidate set-up, one thread per candidate: the tolerances (length
// tolerances 1e-4 / edge length; the time tolerance divided by 100 when f
// over [0, toi_tol] x [0, tol_a] x [0, tol_b] contains zero).
__global__ void __launch_bounds__(128) k_ccd_prepare(CCDArgs a)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nee + a.nfv) return;
    Query q;
    load_candidate(a, i, q);
    double tol[3];
    if (i < a.nee) {
        tol[1] = RDIV(1e-4, a.edge_len[a.ee[i].x]);
        tol[2] = RDIV(1e-4, a.edge_len[a.ee[i].y]);
    } else {
        int f = a.fv[i - a.nee].x;
        tol[1] = RDIV(1e-4, a.edge_len[a.f2e[3 * f]]);
        tol[2] = RDIV(1e-4, a.edge_len[a.f2e[3 * f + 1]]);
    }
    tol[0] = a.toi_tol;
    Box xt { 0.0, tol[0], 0.0, tol[1], 0.0, tol[2] };
    Itv R[9], p[3];
    const int na = q.fv ? 1 : 2;
    frame_load(a.table + ((size_t)q.body_a * kTableSlots + kTableNodes) * kTableEntry, R, p);
    for (int k = 0; k < na; k++) iworld_vertex(R, p, q.v[k], q.P[k]);
    frame_load(a.table + ((size_t)q.body_b * kTableSlots + kTableNodes) * kTableEntry, R, p);
    for (int k = na; k < 4; k++) iworld_vertex(R, p, q.v[k], q.P[k]);
    if (f_zero(q, xt)) tol[0] = RDIV(tol[0], 1e2);
    a.ctol[3 * i] = tol[0];
    a.ctol[3 * i + 1] = tol[1];
    a.ctol[3 * i + 2] = tol[2];
}

// a <= b for non-negative doubles (+0 and +inf included), on the bit pattern
__device__ __forceinline__ bool le_nn(double a, double b)
{
    return dbits(a) <= dbits(b);
}

// running minimum of the candidate's scene (the whole context unless batched)
__device__ __forceinline__ unsigned long long* gmin_of(const CCDArgs& a, const Query& q)
{
    return a.scene_gmin ? a.scene_gmin + a.bscene[q.body_a] : a.gmin;
}

__device__ __forceinline__ double load_gmin(const CCDArgs& a, const Query& q)
{
    return __longlong_as_double((long long)*(volatile unsigned long long*)gmin_of(a, q));
}

__device__ __forceinline__ void record_min(const CCDArgs& a, const Query& q, double t)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(t);
    if (a.scene_gmin) atomicMin(gmin_of(a, q), b);
    atomicMin(a.gmin, b);
}

// Search tree nodes and the path-encoded depth-first search: see
// search_tree.cuh.  The boxes of nodes, and the root finder's split rule.
__device__ __forceinline__ Box node_box(const Node& c)
{
    return Box { dyadic(c.ix[0], c.lv[0]), dyadic(c.ix[0] + 1, c.lv[0]),
                 dyadic(c.ix[1], c.lv[1]), dyadic(c.ix[1] + 1, c.lv[1]),
                 dyadic(c.ix[2], c.lv[2]), dyadic(c.ix[2] + 1, c.lv[2]) };
}

// The split rule of interval_root_finder.cpp:151-178: the dimension with the
// largest width / tolerance among those above tolerance (among all when
// every width is within tolerance).
__device__ __forceinline__ int split_dim(const double w[3], const double tol[3], bool all_tol)
{
    int split = -1;
#pragma unroll
    for (int d = 0; d < 3; d++)
        if ((all_tol || !le_nn(w[d], tol[d]))
            && (split == -1 || !le_nn(RMUL(w[d], tol[split]), RMUL(w[split], tol[d]))))
            split = d;
    return split;
}

// split_dim without multiplications.  A node's width is w[k] =
// (1 + 2^-52) 2^-lv[k] (node_widths), so RMUL(w[d], tol[s]) =
// 2^-lv[d] RN((1 + 2^-52) tol[s]) exactly while the results stay normal,
// and the comparison of split_dim orders the keys
// K[k] = bits(RN((1 + 2^-52) tol[k])) + lv[k] 2^52 (a power-of-two scaling
// adds to the exponent field): the split moves to d when K[d] < K[split].
// tk[k] = bits(RN((1 + 2^-52) tol[k])); ok = every tk is at least 2^-960, so
// that the scaled products are normal (else split_dim decides).
struct TolKeys {
    long long tk[3];
    bool ok;
};

__device__ __forceinline__ TolKeys tol_keys(const double tol[3])
{
    TolKeys r;
    const double wunit = __longlong_as_double(0x3ff0000000000001ll);  // 1 + 2^-52
    r.ok = true;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const double t = RMUL(wunit, tol[k]);
        r.tk[k] = __double_as_longlong(t);
        r.ok = r.ok && is_pos(t) && r.tk[k] >= (63ll << 52) && r.tk[k] < (2046ll << 52);
    }
    return r;
}

__device__ __forceinline__ int split_dim_keys(const Node& c, const TolKeys& K, const double w[3],
                                              const double tol[3], bool all_tol)
{
    if (!K.ok) return split_dim(w, tol, all_tol);
    int split = -1;
    long long ks = 0;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const long long kd = K.tk[d] + ((long long)c.lv[d] << 52);
        if ((all_tol || !le_nn(w[d], tol[d])) && (split == -1 || kd < ks)) {
            split = d;
            ks = kd;
        }
    }
    return split;
}

// The node of the candidate's subdivision tree at depth d reached by the
// branches in the bits of j (most significant first, 0 = lower half).  The
// split rule depends only on the widths and tolerances, so every box of a
// level splits along the same dimension and these boxes are exactly the
// tree's nodes at depth d: searching them one by one visits the tree's
// leaves below them, hence finds the same earliest root box.
__device__ __forceinline__ Node seed_node(int d, int64_t j, const double* tol, u128& mt, u128& ma)
{
    Node c { { 0, 0, 0 }, { 0ull, 0ull, 0ull }, 0 };
    for (int l = d - 1; l >= 0; l--) {
        double w[3];
        node_widths(c, w);
        const bool all_tol = le_nn(w[0], tol[0]) && le_nn(w[1], tol[1]) && le_nn(w[2], tol[2]);
        const int s = split_dim(w, tol, all_tol);
        record_split(mt, ma, c.depth, s);
        c.lv[s]++;
        c.ix[s] = 2 * c.ix[s] + (unsigned long long)((j >> l) & 1);
        c.depth++;
    }
    return c;
}

// The rare paths of the search loops (k_ccd, k_ccd_group), kept out of
// their bodies so that the loop run box after box stays short.
// Hand-off: the pending boxes of the group's search (and its current box)
// become pieces of the next launch; without room for all of them the slots
// taken are voided and the search goes on (no further hand-offs).
template <int W>
static __device__ __noinline__ void hand_off_pending(const CCDArgs& a, const Node& cn, u128 mt, u128 ma,
                                                     u128& pend_hi, bool& has_cn, bool& hand_ok,
                                                     long long cur, double earliest,
                                                     unsigned long long boxes, int gl, unsigned gmask)
{
    const int k = popc128(pend_hi) + (has_cn ? 1 : 0);
    unsigned long long s = 0;
    if (gl == 0) s = atomicAdd(a.n_out, (unsigned long long)k);
    s = __shfl_sync(gmask, s, 0, W);
    if (s + k <= a.out_cap) {
        if (gl == 0) {
            Piece pc;
            pc.cand = cur;
            pc.earliest = earliest;
            pc.boxes = boxes;
            unsigned long long o = s;
            for (u128 r = pend_hi; r != 0; r &= r - 1) {
                const Node g = pending_node(cn, mt, ma, lsb128(r));
                for (int d = 0; d < 3; d++) {
                    pc.ix[d] = g.ix[d];
                    pc.lv[d] = g.lv[d];
                }
                pc.depth = g.depth;
                a.pieces_out[o++] = pc;
            }
            if (has_cn) {
                for (int d = 0; d < 3; d++) {
                    pc.ix[d] = cn.ix[d];
                    pc.lv[d] = cn.lv[d];
                }
                pc.depth = cn.depth;
                a.pieces_out[o++] = pc;
            }
        }
        pend_hi = 0;
        has_cn = false;
    } else {
        if (gl == 0)
            for (unsigned long long t = s; t < s + k && t < a.out_cap; t++) a.pieces_out[t].cand = -1;
        hand_ok = false;
    }
}

// A box after the launch's time window becomes a piece of the next launch;
// false when there is no room for it (it is searched now).
template <int W>
static __device__ __noinline__ bool defer_node(const CCDArgs& a, const Node& cn, long long cur,
                                               double earliest, unsigned long long boxes, int gl,
                                               unsigned gmask)
{
    unsigned long long s = 0;
    if (gl == 0) s = atomicAdd(a.n_out, 1ull);
    s = __shfl_sync(gmask, s, 0, W);
    if (s >= a.out_cap) return false;
    if (gl == 0) {
        Piece pc;
        pc.cand = cur;
        pc.earliest = earliest;
        pc.boxes = boxes;
        for (int d = 0; d < 3; d++) {
            pc.ix[d] = cn.ix[d];
            pc.lv[d] = cn.lv[d];
        }
        pc.depth = cn.depth;
        a.pieces_out[s] = pc;
    }
    return true;
}

// the smallest t.lo of the current box and the pending boxes
static __device__ __noinline__ double earliest_unexplored(const Node& cn, u128 mt, u128 ma, u128 pend_hi,
                                                          double t0)
{
    double m = t0;
    for (u128 r = pend_hi; r != 0; r &= r - 1) {
        const Node g = pending_node(cn, mt, ma, lsb128(r));
        m = smin(m, dyadic(g.ix[0], g.lv[0]));
    }
    return m;
}

// Persistent kernel: each lane takes the next unprocessed candidate from a
// global counter whenever its search runs out of boxes.  Every iteration each
// lane pops boxes until one survives the cheap tests (or takes a new
// candidate's root box), then all lanes evaluate their boxes together.  The
// search state is the current node, the pending mask and the split masks
// (all in registers): no box stack in local memory.
__global__ void __launch_bounds__(kCCDThreads)
k_ccd(CCDArgs a)
{
    const int64_t n = a.nee + a.nfv;
    unsigned long long tot_boxes = 0, tot_hits = 0, pops = 0;
    Query q;
    double tol[3] = { 0, 0, 0 };
    Node cn { { 0, 0, 0 }, { 0ull, 0ull, 0ull }, 0 };  // current node
    bool has_cn = false;      // cn is still to be processed (lower child, retry, taken box)
    u128 pend_hi = 0;         // depths whose upper child is pending
    u128 mt = 0, ma = 0;      // depths that split t / alpha
    int64_t cur = -1;
    double earliest = INFINITY;
    bool found = false;
    int status = RIGC_OK;
    unsigned long long cboxes = 0;  // boxes of the current piece
    unsigned long long cbase = 0;   // boxes of the path before the piece
    bool hand_ok = a.hand_off != 0;
    double gbound = INFINITY;
    bool done = false;
    OwnFrames own;
    own.key[0] = own.key[1] = 0;
    bool pend = false;
    int req_side = 0, req_body = 0;
    unsigned long long req_node = 0;
    const int lane = threadIdx.x & 31;
    while (true) {
        // frames asked for in the last iteration, computed by the whole warp
        const unsigned req = __ballot_sync(0xffffffffu, pend);
        if (req) {
            group_compute_frames<32>(a, own, req, req_side, req_body, req_node);
            pend = false;
        }
        // Once the candidate list is exhausted, a lane with nothing left takes
        // the bottom (largest) box of the fullest stack in its warp together
        // with its candidate.  Prune mode only: split searches find the same
        // earliest time of impact, but a search stopped by the box budget
        // would not report what one search reports.
        bool tail = false;  // a lane of this warp found no work left
        if (a.prune) {
            const unsigned idle = __ballot_sync(0xffffffffu, done);
            tail = idle != 0;
            if (idle) {
                // boxes left in a lane's search: pending upper children + cn
                int best = done ? 0 : popc128(pend_hi) + (has_cn ? 1 : 0) - 1, bl = lane;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const int ob = __shfl_xor_sync(0xffffffffu, best, o);
                    const int ol = __shfl_xor_sync(0xffffffffu, bl, o);
                    if (ob > best || (ob == best && ol < bl)) {
                        best = ob;
                        bl = ol;
                    }
                }
                if (best >= 1) {
                    const int thief = __ffs(idle) - 1;
                    // the victim's shallowest pending upper child (best >= 1
                    // leaves at least one pending depth)
                    Node g = cn;
                    if (lane == bl) {
                        const int j = lsb128(pend_hi);
                        g = pending_node(cn, mt, ma, j);
                        pend_hi &= ~bit128(j);
                    }
                    const double e = __shfl_sync(0xffffffffu, earliest, bl);
                    const long long c = __shfl_sync(0xffffffffu, (long long)cur, bl);
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        g.lv[k] = __shfl_sync(0xffffffffu, g.lv[k], bl);
                        g.ix[k] = __shfl_sync(0xffffffffu, g.ix[k], bl);
                    }
                    g.depth = __shfl_sync(0xffffffffu, g.depth, bl);
                    if (lane == thief) {
                        cur = c;
                        load_candidate(a, cur, q);
                        tol[0] = a.ctol[3 * cur];
                        tol[1] = a.ctol[3 * cur + 1];
                        tol[2] = a.ctol[3 * cur + 2];
                        gbound = load_gmin(a, q);
                        earliest = e;
                        found = false;
                        status = RIGC_OK;
                        cboxes = 0;
                        cbase = 0;
                        cn = g;
                        has_cn = true;
                        pend_hi = 0;
                        done = false;
                    }
                }
            }
        }
        bool have = false;
        Box x;
        if (!done && tail && hand_ok && cboxes >= a.hand_off && (pend_hi != 0 || has_cn)) {
            // Once the work list runs dry (idle lanes in the warp), a long
            // piece hands its pending boxes to the next launch, which spreads
            // them over the whole GPU, and ends
            const int k = popc128(pend_hi) + (has_cn ? 1 : 0);
            const unsigned long long s = atomicAdd(a.n_out, (unsigned long long)k);
            if (s + k <= a.out_cap) {
                Piece pc;
                pc.cand = cur;
                pc.earliest = earliest;
                pc.boxes = cbase + cboxes;
                unsigned long long o = s;
                for (u128 r = pend_hi; r != 0; r &= r - 1) {
                    const Node g = pending_node(cn, mt, ma, lsb128(r));
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        pc.ix[d] = g.ix[d];
                        pc.lv[d] = g.lv[d];
                    }
                    pc.depth = g.depth;
                    a.pieces_out[o++] = pc;
                }
                if (has_cn) {
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        pc.ix[d] = cn.ix[d];
                        pc.lv[d] = cn.lv[d];
                    }
                    pc.depth = cn.depth;
                    a.pieces_out[o++] = pc;
                }
                pend_hi = 0;
                has_cn = false;
            } else {
                // no room: the reserved slots stay unused, the lane keeps searching
                for (unsigned long long t = s; t < s + k && t < a.out_cap; t++) a.pieces_out[t].cand = -1;
                hand_ok = false;
            }
        }
        if (!done) {
            while (has_cn || pend_hi != 0) {
                if (has_cn) {
                    has_cn = false;
                } else {
                    const int j = msb128(pend_hi);
                    pend_hi &= ~bit128(j);
                    cn = pending_node(cn, mt, ma, j);
                }
                x = node_box(cn);
                if (le_nn(earliest, x.t0)) continue;
                if (a.prune) {
                    if ((++pops & 7) == 0) gbound = load_gmin(a, q);
                    if (le_nn(gbound, x.t0)) continue;
                }
                if (q.fv) {
                    double sl = add_dn(x.a0, x.b0), sh = add_up(x.a1, x.b1);
                    if (!(le_nn(sl, 1.0) && !is_neg(sh))) continue;
                }
                have = true;
                break;
            }
            if (!have) {
                if (cur >= 0) {
                    double toi = found ? earliest : INFINITY;
                    if (found) {
                        record_min(a, q, toi);
                        tot_hits++;
                    }
                    if (a.per && found)
                        atomicMin(reinterpret_cast<unsigned long long*>(a.per) + cur,
                                  (unsigned long long)__double_as_longlong(toi));
                    if (status != RIGC_OK) atomicMax(a.status, status);
                }
                // work item w: seed w / n of candidate w % n (seed-major, so
                // early times of every candidate come first), or piece w
                const int64_t w = (int64_t)atomicAdd(a.next, 1ull);
                if (w >= (a.pieces_in ? a.n_pieces : (n << a.seeds_log2))) {
                    done = true;
                } else if (a.pieces_in) {
                    // the piece's node is popped (and tested) in the next iteration
                    const Piece pc = a.pieces_in[w];
                    cur = pc.cand;
                    if (cur >= 0) {
                        load_candidate(a, cur, q);
                        tol[0] = a.ctol[3 * cur];
                        tol[1] = a.ctol[3 * cur + 1];
                        tol[2] = a.ctol[3 * cur + 2];
                        gbound = load_gmin(a, q);
                        earliest = pc.earliest;
                        found = false;
                        status = RIGC_OK;
                        cboxes = 0;
                        cbase = pc.boxes;
                        pend_hi = 0;
#pragma unroll
                        for (int d = 0; d < 3; d++) {
                            cn.ix[d] = pc.ix[d];
                            cn.lv[d] = pc.lv[d];
                        }
                        cn.depth = pc.depth;
                        has_cn = true;
                    }
                } else {
                    cur = w % n;
                    load_candidate(a, cur, q);
                    tol[0] = a.ctol[3 * cur];
                    tol[1] = a.ctol[3 * cur + 1];
                    tol[2] = a.ctol[3 * cur + 2];
                    if (a.prune) gbound = load_gmin(a, q);
                    earliest = INFINITY;
                    found = false;
                    status = RIGC_OK;
                    cboxes = 0;
                    cbase = 0;
                    pend_hi = 0;
                    has_cn = false;
                    cn = seed_node(a.seeds_log2, w / n, tol, mt, ma);
                    x = node_box(cn);
                    have = !(a.prune && le_nn(gbound, x.t0));
                    if (have && q.fv) {
                        double sl = add_dn(x.a0, x.b0), sh = add_up(x.a1, x.b1);
                        have = le_nn(sl, 1.0) && !is_neg(sh);
                    }
                }
            }
        }
        // every lane reaches this point once per iteration
        if (__all_sync(0xffffffffu, done)) break;
        if (!have) continue;
        if (cbase + cboxes >= (unsigned long long)a.max_boxes) {
            // budget exhausted: the earliest unexplored t.lo is conservative
            earliest = smin(earliest, earliest_unexplored(cn, mt, ma, pend_hi, x.t0));
            found = true;
            status = RIGC_ERR_ITER_LIMIT;
            pend_hi = 0;
            has_cn = false;
            continue;
        }
        if (!(dbits(x.t0) == dbits(q.ct0) && dbits(x.t1) == dbits(q.ct1))) {
            const int miss = eval_vertices(a, own, q, Itv { x.t0, x.t1 });
            if (miss) {
                // retry the box once the warp has computed the frame
                has_cn = true;
                pend = true;
                req_side = (miss & 1) ? 0 : 1;
                req_body = req_side ? q.body_b : q.body_a;
                req_node = time_node(x.t0, x.t1);
                continue;
            }
        }
        cboxes++;
        tot_boxes++;
        if (!f_zero(q, x)) continue;
        double w[3];
        node_widths(cn, w);
        bool all_tol = le_nn(w[0], tol[0]) && le_nn(w[1], tol[1]) && le_nn(w[2], tol[2]);
        bool all_zero = le_nn(w[0], 1e-10) && le_nn(w[1], 1e-10) && le_nn(w[2], 1e-10);
        if ((is_pos(x.t0) || all_zero) && all_tol) {
            earliest = x.t0;
            found = true;
            if (a.prune) {
                record_min(a, q, earliest);
                gbound = smin(gbound, earliest);
            }
            continue;
        }
        const int split = split_dim(w, tol, all_tol);
        if (cn.depth >= kMaxDepth || cn.lv[split] >= kMaxLevel) {
            // cannot descend: keep the box's start as a conservative root
            earliest = smin(earliest, x.t0);
            found = true;
            status = RIGC_ERR_QUEUE_OVERFLOW;
            continue;
        }
        // go to the lower half; the upper half is pending at this depth
        descend(cn, pend_hi, mt, ma, split);
        has_cn = true;
    }
    // warp-aggregated counters
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        tot_boxes += __shfl_down_sync(0xffffffffu, tot_boxes, o);
        tot_hits += __shfl_down_sync(0xffffffffu, tot_hits, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (tot_boxes) atomicAdd(a.boxes, tot_boxes);
        if (tot_hits) atomicAdd(a.hits, tot_hits);
    }
}

// ---------------------------------------------------------------------------
// One search per group of W lanes: the whole warp (W = 32) or each half of
// it (W = 16, two searches per warp).  The same branch and bound, pruning,
// seeds, budget and search pieces as k_ccd, but a box is evaluated by the
// group's lanes together, each FP64 expression of the box on its own lane:
//  * W = 32: lane 12 b + 3 v + c computes bound b (0 lower, 1 upper) of
//    coordinate c of vertex v's interval position (iworld_vertex's
//    expression for that bound: a lower bound takes only lower-bound
//    operations);
//  * W = 16: lane 3 v + c computes that coordinate's interval (both bounds);
//  * both: lane 6 b + 3 h + c computes bound b of half h of the interval
//    distance function's coordinate c (f_zero's expressions), the lanes with
//    h = 0 combine the halves, and a vote of the group decides.
// The chain of FP64 instructions per box is a tenth of one lane's.  With
// W = 16 the two searches of a warp share every instruction they execute
// together (the search control, which all lanes of a group execute on the
// same state, and the FP64 of the box), at the price of running apart where
// their paths differ.  The search state is identical in every lane of a
// group; the group's first lane does the atomics.  Same bits as k_ccd for
// every box.

// rest vertex v of a candidate (EE: a0 a1 b0 b1; FV: v f0 f1 f2), its bodies
// and kind
__device__ __forceinline__ void warp_candidate(const CCDArgs& a, int64_t i, int vtx, bool& fv,
                                               int& body_a, int& body_b, double rv[3])
{
    int vid;
    if (i < a.nee) {
        fv = false;
        const int ea = a.ee[i].x, eb = a.ee[i].y;
        const int e = vtx < 2 ? ea : eb;
        vid = a.edges[2 * e + (vtx & 1)];
        body_a = a.ebody[ea];
        body_b = a.ebody[eb];
    } else {
        fv = true;
        const int64_t k = i - a.nee;
        const int f = a.fv[k].x, v = a.fv[k].y;
        vid = vtx == 0 ? v : a.faces[3 * f + (vtx - 1)];
        body_a = a.vbody[v];
        body_b = a.fbody[f];
    }
#pragma unroll
    for (int j = 0; j < 3; j++) rv[j] = a.rest[3 * (size_t)vid + j];
}

// row c of R and p[c] of a frame entry (kTableEntry doubles)
__device__ __forceinline__ void frame_row(const double* e, int c, Itv r[3], Itv& pc, bool cg)
{
#pragma unroll
    for (int k = 0; k < 3; k++)
        r[k] = cg ? Itv { __ldcg(e + 6 * c + 2 * k), __ldcg(e + 6 * c + 2 * k + 1) }
                  : Itv { e[6 * c + 2 * k], e[6 * c + 2 * k + 1] };
    pc = cg ? Itv { __ldcg(e + 18 + 2 * c), __ldcg(e + 19 + 2 * c) } : Itv { e[18 + 2 * c], e[19 + 2 * c] };
}

// Row c of the frame of a body over t: the table, the warp's own frames, the
// cache; a time interval that is not a tree node is computed on the spot.
// False when the frame still has to be computed.
__device__ __forceinline__ bool frame_find_row(const CCDArgs& a, const OwnFrames& own, int side,
                                              int body, unsigned long long node, const Itv& t, int c,
                                              Itv r[3], Itv& pc)
{
    if (node != 0 && node < (1ull << kTableDepth)) {
        frame_row(a.table + ((size_t)body * kTableSlots + (node - 1)) * kTableEntry, c, r, pc, false);
        return true;
    }
    if (node == 0) {
        Itv R[9], p[3];
        frame_compute(a, body, t, R, p);
#pragma unroll
        for (int k = 0; k < 3; k++) r[k] = R[3 * c + k];
        pc = p[c];
        return true;
    }
    const unsigned long long key = frame_key(body, node);
    if (own.key[side] == key) {
        frame_row(own.f[side], c, r, pc, false);
        return true;
    }
    unsigned long long h = mix64(key);
    for (int probe = 0; probe < kProbes; probe++, h++) {
        const unsigned long long k = ld_acquire(a.fkeys + (h & a.fmask));
        if (k == key) {
            frame_row(a.fvals + (h & a.fmask) * kTableEntry, c, r, pc, true);
            return true;
        }
        if (k == 0 || k == (key | kPending)) return false;
    }
    return false;
}

__device__ __forceinline__ unsigned long long* gmin_body(const CCDArgs& a, int body_a)
{
    return a.scene_gmin ? a.scene_gmin + a.bscene[body_a] : a.gmin;
}

// MinBlocks > 1 asks the compiler to fit that many blocks per SM (fewer
// registers, some spilled to local memory, more warps to hide latency)
template <int W, int MinBlocks>
__global__ void __launch_bounds__(kCCDThreads, MinBlocks)
k_ccd_group(CCDArgs a)
{
    static_assert(W == 32 || W == 16, "a warp or a half-warp per search");
    const int64_t n = a.nee + a.nfv;
    const int64_t nwork = a.pieces_in ? a.n_pieces : (n << a.seeds_log2);
    const int lane = threadIdx.x & 31;
    const int gl = lane & (W - 1);  // lane within the group
    const unsigned gmask = W == 32 ? 0xffffffffu : (0xffffu << (lane & 16));
    const int gshift = W == 32 ? 0 : (lane & 16);
    // vertex lanes: W = 32, lanes 0..23: bound vb of coordinate crd of
    // vertex vtx; W = 16, lanes 0..11: the interval of coordinate crd of
    // vertex vtx.  Distance lanes 0..11: bound db of the half dh of the
    // distance function's coordinate dc
    const int vb = W == 32 && gl >= 12 ? 1 : 0;
    const int vtx = (gl % 12) / 3, crd = gl % 3;
    const bool vlane = gl < (W == 32 ? 24 : 12);
    const int db = gl >= 6 ? 1 : 0, dh = (gl % 6) / 3, dc = gl % 3;
    unsigned long long tot_boxes = 0, tot_hits = 0, pops = 0;
    // search state (the same in every lane of the group)
    Node cn { { 0, 0, 0 }, { 0ull, 0ull, 0ull }, 0 };
    bool has_cn = false;
    u128 pend_hi = 0, mt = 0, ma = 0;
    long long cur = -1;
    double earliest = INFINITY;
    bool found = false;
    int status = RIGC_OK;
    unsigned long long cboxes = 0, cbase = 0;
    bool hand_ok = a.hand_off != 0, tail = false;
    double gbound = INFINITY;
    double tol[3] = { 0, 0, 0 };
    TolKeys tkeys { { 0, 0, 0 }, false };
    bool fv = false, a_fixed = false, b_fixed = false;
    int body_a = 0, body_b = 0;
    // this lane's vertex and its bound (W = 32) or interval (W = 16) of the
    // coordinate over [ct0, ct1]
    double rv[3] = { 0, 0, 0 };
    Itv pcrd { 0, 0 };
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    double ct0 = nan, ct1 = nan;
    bool fresh = true;
    OwnFrames own;
    own.key[0] = own.key[1] = 0;
    while (true) {
        // hand the pending boxes of a long piece to the next launch once
        // the work list has run dry
        if (tail && hand_ok && cboxes >= a.hand_off && (pend_hi != 0 || has_cn))
            hand_off_pending<W>(a, cn, mt, ma, pend_hi, has_cn, hand_ok, cur, earliest, cbase + cboxes, gl,
                                gmask);
        bool have = false;
        Box x;
        while (has_cn || pend_hi != 0) {
            if (has_cn) {
                has_cn = false;
            } else {
                const int j = msb128(pend_hi);
                pend_hi &= ~bit128(j);
                cn = pending_node(cn, mt, ma, j);
            }
            x = node_box(cn);
            if (le_nn(earliest, x.t0)) continue;
            if (a.prune) {
                if ((++pops & 7) == 0) {
                    // values read while other warps write them: the group's
                    // first lane's copy for all, so that its state stays uniform
                    gbound = __shfl_sync(gmask, __longlong_as_double(
                        (long long)*(volatile unsigned long long*)gmin_body(a, body_a)), 0, W);
                    tail = __shfl_sync(gmask,
                        (int)(*(volatile unsigned long long*)a.next >= (unsigned long long)nwork), 0, W) != 0;
                }
                if (le_nn(gbound, x.t0)) continue;
            }
            if (fv) {
                double sl = add_dn(x.a0, x.b0), sh = add_up(x.a1, x.b1);
                if (!(le_nn(sl, 1.0) && !is_neg(sh))) continue;
            }
            // after the window: a piece of the next launch (searched now
            // when there is no room for it)
            if (x.t0 >= a.window && defer_node<W>(a, cn, cur, earliest, cbase + cboxes, gl, gmask)) continue;
            have = true;
            break;
        }
        if (!have) {
            if (cur >= 0 && gl == 0) {
                if (found) {
                    unsigned long long* g = gmin_body(a, body_a);
                    const unsigned long long b = (unsigned long long)__double_as_longlong(earliest);
                    if (a.scene_gmin) atomicMin(g, b);
                    atomicMin(a.gmin, b);
                    tot_hits++;
                    if (a.per) atomicMin(reinterpret_cast<unsigned long long*>(a.per) + cur, b);
                }
                if (status != RIGC_OK) atomicMax(a.status, status);
            }
            // next work item: seed w / n of candidate w % n, or piece w
            long long w = 0;
            if (gl == 0) w = (long long)atomicAdd(a.next, 1ull);
            w = __shfl_sync(gmask, w, 0, W);
            if (w >= nwork) break;  // the group is done
            tail = tail || w + 1 >= nwork;
            found = false;
            status = RIGC_OK;
            cboxes = 0;
            pend_hi = 0;
            has_cn = false;
            if (a.pieces_in) {
                const Piece pc = a.pieces_in[w];
                cur = pc.cand;
                if (cur < 0) continue;
                if (a.prune && !a.scene_gmin) {
                    // the group's first lane's copy of the running minimum
                    const double g = __shfl_sync(gmask, __longlong_as_double(
                        (long long)*(volatile unsigned long long*)a.gmin), 0, W);
                    if (le_nn(g, dyadic(pc.ix[0], pc.lv[0]))) {
                        cur = -1;  // the piece starts at or after it
                        continue;
                    }
                }
                earliest = pc.earliest;
                cbase = pc.boxes;
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    cn.ix[d] = pc.ix[d];
                    cn.lv[d] = pc.lv[d];
                }
                cn.depth = pc.depth;
                has_cn = true;
            } else {
                cur = w % n;
                earliest = INFINITY;
                cbase = 0;
            }
            warp_candidate(a, cur, vlane ? vtx : 0, fv, body_a, body_b, rv);
            a_fixed = a.bfixed[body_a] != 0;
            b_fixed = a.bfixed[body_b] != 0;
            fresh = true;
            ct0 = ct1 = nan;
            tol[0] = a.ctol[3 * cur];
            tol[1] = a.ctol[3 * cur + 1];
            tol[2] = a.ctol[3 * cur + 2];
            tkeys = tol_keys(tol);
            if (a.prune)
                gbound = __shfl_sync(gmask, __longlong_as_double(
                    (long long)*(volatile unsigned long long*)gmin_body(a, body_a)), 0, W);
            if (a.pieces_in) continue;  // the piece's node is popped next
            cn = seed_node(a.seeds_log2, w / n, tol, mt, ma);
            x = node_box(cn);
            have = !(a.prune && le_nn(gbound, x.t0));
            if (have && fv) {
                double sl = add_dn(x.a0, x.b0), sh = add_up(x.a1, x.b1);
                have = le_nn(sl, 1.0) && !is_neg(sh);
            }
            if (!have) continue;
        }
        if (cbase + cboxes >= (unsigned long long)a.max_boxes) {
            // budget exhausted: the earliest unexplored t.lo is conservative
            earliest = smin(earliest, earliest_unexplored(cn, mt, ma, pend_hi, x.t0));
            found = true;
            status = RIGC_ERR_ITER_LIMIT;
            pend_hi = 0;
            has_cn = false;
            continue;
        }
        // vertex coordinates over the box's time interval
        if (!(dbits(x.t0) == dbits(ct0) && dbits(x.t1) == dbits(ct1))) {
            const int na = fv ? 1 : 2;
            const int side = vtx < na ? 0 : 1;
            const bool need = vlane && (fresh || !(side ? b_fixed : a_fixed));
            const Itv t { x.t0, x.t1 };
            // the time interval's tree node straight from the box's node
            // (time_node(x.t0, x.t1) gives the same: t0 = ix 2^-lv, t1 = (ix + 1) 2^-lv)
            const unsigned long long node = cn.lv[0] < kNodeDepth ? (1ull << cn.lv[0]) + cn.ix[0] : 0ull;
            bool miss = false;
            if (need) {
                Itv r[3], pc;
                if (frame_find_row(a, own, side, side ? body_b : body_a, node, t, crd, r, pc)) {
                    // W = 32 keeps its one bound in pcrd.lo
                    if (W == 16) {
                        pcrd = iadd(iadd(iadd(imul(rv[0], r[0]), imul(rv[1], r[1])), imul(rv[2], r[2])), pc);
                    } else if (vb == 0) {
                        // one bound of iworld_vertex's coordinate expression
                        // iadd(iadd(iadd(imul(v0, r0), imul(v1, r1)), imul(v2, r2)), p):
                        // the lower bound takes only lower-bound operations, the
                        // upper only upper
                        double q = mul_dn(rv[0], is_neg(rv[0]) ? r[0].hi : r[0].lo);
                        q = add_dn(q, mul_dn(rv[1], is_neg(rv[1]) ? r[1].hi : r[1].lo));
                        q = add_dn(q, mul_dn(rv[2], is_neg(rv[2]) ? r[2].hi : r[2].lo));
                        pcrd.lo = add_dn(q, pc.lo);
                    } else {
                        double q = mul_up(rv[0], is_neg(rv[0]) ? r[0].lo : r[0].hi);
                        q = add_up(q, mul_up(rv[1], is_neg(rv[1]) ? r[1].lo : r[1].hi));
                        q = add_up(q, mul_up(rv[2], is_neg(rv[2]) ? r[2].lo : r[2].hi));
                        pcrd.lo = add_up(q, pc.hi);
                    }
                } else {
                    miss = true;
                }
            }
            const unsigned mm = __ballot_sync(gmask, miss) >> gshift;
            if (mm) {
                // the group computes the missing frames (its lane 0 asks for
                // body A's, lane 1 for body B's), every lane keeps them; retry
                bool miss_a = false, miss_b = false;
#pragma unroll
                for (int l = 0; l < (W == 32 ? 24 : 12); l++)
                    if ((mm >> l) & 1) {
                        if ((l % 12) / 3 < na) miss_a = true;
                        else miss_b = true;
                    }
                const unsigned req = (miss_a ? 1u : 0u) | (miss_b ? 2u : 0u);
                group_compute_frames<W>(a, own, req, gl == 1 ? 1 : 0, gl == 1 ? body_b : body_a,
                                        node, true);
                ct0 = ct1 = nan;
                has_cn = true;
                continue;
            }
            fresh = false;
            ct0 = x.t0;
            ct1 = x.t1;
        }
        cboxes++;
        if (gl == 0) tot_boxes++;
        // f(box) contains zero: the expressions and operand order of f_zero,
        // each interval bound on its own lane.  Distance lane (db, dh, dc)
        // evaluates bound db of half dh of coordinate dc (EE: the point of
        // edge dh; FV: the face-edge term dh): d = A - B, m = d * w
        // (w = alpha or beta, non-negative), EE adds q0 = B.  Lanes with
        // dh = 0 then combine the halves: EE y = part0 - part1; FV
        // y = P0 - ((part0 + part1) + P1).  A lower bound takes only lower
        // bounds of its operands (and upper bounds of subtrahends), so the
        // bits are those of the interval expressions.
        const int va = fv ? (dh ? 3 : 2) : (dh ? 3 : 1);
        const int vq = fv ? 1 : (dh ? 2 : 0);
        double A, Bx, Bs, P0 = 0, P1 = 0;
        if (W == 32) {
            // vertex v's bound b of coordinate c lives on lane 12 b + 3 v + c
            A = __shfl_sync(gmask, pcrd.lo, 12 * db + 3 * va + dc);
            Bx = __shfl_sync(gmask, pcrd.lo, 12 * (1 - db) + 3 * vq + dc);
            Bs = __shfl_sync(gmask, pcrd.lo, 12 * db + 3 * vq + dc);
            if (fv) {
                P1 = __shfl_sync(gmask, pcrd.lo, 12 * db + 3 + dc);
                P0 = __shfl_sync(gmask, pcrd.lo, 12 * db + dc);
            }
        } else {
            // vertex v's interval of coordinate c lives on lane 3 v + c
            const double alo = __shfl_sync(gmask, pcrd.lo, 3 * va + dc, W);
            const double ahi = __shfl_sync(gmask, pcrd.hi, 3 * va + dc, W);
            const double qlo = __shfl_sync(gmask, pcrd.lo, 3 * vq + dc, W);
            const double qhi = __shfl_sync(gmask, pcrd.hi, 3 * vq + dc, W);
            A = db ? ahi : alo;
            Bx = db ? qlo : qhi;
            Bs = db ? qhi : qlo;
            if (fv) {
                const double p1lo = __shfl_sync(gmask, pcrd.lo, 3 + dc, W);
                const double p1hi = __shfl_sync(gmask, pcrd.hi, 3 + dc, W);
                const double p0lo = __shfl_sync(gmask, pcrd.lo, dc, W);
                const double p0hi = __shfl_sync(gmask, pcrd.hi, dc, W);
                P1 = db ? p1hi : p1lo;
                P0 = db ? p0hi : p0lo;
            }
        }
        const Itv pw = dh ? Itv { x.b0, x.b1 } : Itv { x.a0, x.a1 };
        double part;
        if (db == 0) {
            const double d = sub_dn(A, Bx);
            part = mul_dn(d, is_neg(d) ? pw.hi : pw.lo);
            if (!fv) part = add_dn(part, Bs);
        } else {
            const double d = sub_up(A, Bx);
            part = mul_up(d, is_neg(d) ? pw.lo : pw.hi);
            if (!fv) part = add_up(part, Bs);
        }
        // the other half's bound: EE the opposite bound, FV the same
        const int osrc = 6 * (fv ? db : 1 - db) + 3 + dc;
        const double other = __shfl_sync(gmask, part, osrc, W);
        bool zin = true;
        if (fv) {
            const double tb = db == 0 ? add_dn(add_dn(part, other), P1) : add_up(add_up(part, other), P1);
            const double tx = __shfl_sync(gmask, tb, 6 * (1 - db) + dc, W);
            if (gl < 12 && dh == 0) zin = db == 0 ? !is_pos(sub_dn(P0, tx)) : !is_neg(sub_up(P0, tx));
        } else if (gl < 12 && dh == 0) {
            zin = db == 0 ? !is_pos(sub_dn(part, other)) : !is_neg(sub_up(part, other));
        }
        if (!__all_sync(gmask, zin)) continue;
        double w[3];
        node_widths(cn, w);
        bool all_tol = le_nn(w[0], tol[0]) && le_nn(w[1], tol[1]) && le_nn(w[2], tol[2]);
        bool all_zero = le_nn(w[0], 1e-10) && le_nn(w[1], 1e-10) && le_nn(w[2], 1e-10);
        if ((is_pos(x.t0) || all_zero) && all_tol) {
            earliest = x.t0;
            found = true;
            if (a.prune) {
                if (gl == 0) {
                    const unsigned long long b = (unsigned long long)__double_as_longlong(earliest);
                    if (a.scene_gmin) atomicMin(gmin_body(a, body_a), b);
                    atomicMin(a.gmin, b);
                }
                gbound = smin(gbound, earliest);
            }
            continue;
        }
        const int split = split_dim_keys(cn, tkeys, w, tol, all_tol);
        if (cn.depth >= kMaxDepth || cn.lv[split] >= kMaxLevel) {
            earliest = smin(earliest, x.t0);
            found = true;
            status = RIGC_ERR_QUEUE_OVERFLOW;
            continue;
        }
        descend(cn, pend_hi, mt, ma, split);
        has_cn = true;
    }
    if (gl == 0) {
        if (tot_boxes) atomicAdd(a.boxes, tot_boxes);
        if (tot_hits) atomicAdd(a.hits, tot_hits);
    }
}

// The pieces of the last launch (out, *n_out of them, at most cap) and those
// kept for later windows (kept, n_kept): the ones that start before `window`
// go to `now`, the others to `later`, the ones that start at or after the
// running minimum `gmin` (single scene; null: none) nowhere.  A list that is
// full takes the piece into the other (their capacities sum to at least
// the pieces given); counts[0] / counts[1] end as the appends to now / later
// (above cap: only the first cap slots were written).
__global__ void __launch_bounds__(256) k_split_pieces(
    const Piece* __restrict__ out, const unsigned long long* __restrict__ n_out, unsigned long long cap,
    const Piece* __restrict__ kept, unsigned long long n_kept, double window,
    const unsigned long long* __restrict__ gmin, Piece* __restrict__ now, Piece* __restrict__ later,
    unsigned long long* __restrict__ counts)
{
    const unsigned long long n0 = n_out ? (*n_out < cap ? *n_out : cap) : 0ull;
    const unsigned long long total = n0 + n_kept;
    const double g = gmin ? __longlong_as_double((long long)*gmin) : INFINITY;
    const int lane = threadIdx.x & 31;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    // whole warps iterate together (the ballots below)
    const unsigned long long span = (total + 31) & ~31ull;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < span;
         i += stride) {
        Piece pc;
        bool keep = false, soon = false;
        if (i < total) {
            pc = i < n0 ? out[i] : kept[i - n0];
            const double t0 = dyadic(pc.ix[0], pc.lv[0]);
            keep = pc.cand >= 0 && t0 < g;
            soon = t0 < window;
        }
        // one append per warp and list
        const unsigned m_now = __ballot_sync(0xffffffffu, keep && soon);
        const unsigned m_later = __ballot_sync(0xffffffffu, keep && !soon);
        unsigned long long b_now = 0, b_later = 0;
        if (lane == 0) {
            if (m_now) b_now = atomicAdd(counts, (unsigned long long)__popc(m_now));
            if (m_later) b_later = atomicAdd(counts + 1, (unsigned long long)__popc(m_later));
        }
        b_now = __shfl_sync(0xffffffffu, b_now, 0);
        b_later = __shfl_sync(0xffffffffu, b_later, 0);
        if (!keep) continue;
        const unsigned below = (1u << lane) - 1u;
        unsigned long long slot = soon ? b_now + __popc(m_now & below) : b_later + __popc(m_later & below);
        bool to_now = soon;
        if (slot >= cap) {
            // that list is full: the other one
            to_now = !soon;
            slot = atomicAdd(counts + (to_now ? 0 : 1), 1ull);
        }
        if (slot < cap) (to_now ? now : later)[slot] = pc;
    }
}

__global__ void k_fill_inf(double* __restrict__ v, int64_t n)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = INFINITY;
}

// resident blocks per SM of the CCD kernel of a search mode (0: k_ccd;
// 1, 2, 3: one search per warp, as compiled and fitted to 4 and 5 blocks per
// SM; 4, 5: one search per half-warp, as compiled and fitted to 4 blocks)
constexpr int kSearchModes = 6;

int ccd_max_blocks_per_sm(int* out, int mode)
{
    static int blocks_per_sm[kSearchModes] = { 0, 0, 0, 0, 0, 0 };
    if (mode < 0 || mode >= kSearchModes) return RIGC_ERR_ARG;
    int& b = blocks_per_sm[mode];
    if (!b) {
        switch (mode) {
        case 5: RIGC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_ccd_group<16, 4>, kCCDThreads, 0)); break;
        case 4: RIGC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_ccd_group<16, 1>, kCCDThreads, 0)); break;
        case 3: RIGC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_ccd_group<32, 5>, kCCDThreads, 0)); break;
        case 2: RIGC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_ccd_group<32, 4>, kCCDThreads, 0)); break;
        case 1: RIGC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_ccd_group<32, 1>, kCCDThreads, 0)); break;
        default: RIGC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_ccd, kCCDThreads, 0));
        }
        if (b < 1) b = 1;
    }
    *out = b;
    return RIGC_OK;
}

// the search mode: one search per warp (k_ccd_group<32, 1>) unless the context's
// tuning asks for another; per warp measured faster than per lane on every
// workload here (the 1000-icosphere pile, the 256-scene batch, the cube
// lattices, the chain)
int ccd_search_mode(const Ctx& c)
{
    return c.tune.ccd_warp >= 0 ? c.tune.ccd_warp : 1;
}

// the frame table, the trajectories and the fixed flags (rot_table)
int reserve_rot_table(Ctx& c)
{
    const size_t table_bytes = (size_t)c.s.nb * kTableSlots * kTableEntry * sizeof(double);
    const size_t traj_bytes = (size_t)c.s.nb * kTrajDoubles * sizeof(double);
    return c.rot_table.reserve(table_bytes + traj_bytes + (size_t)c.s.nb * sizeof(int) + 64);
}

// counters layout in the context's device scalars (byte offset 256):
// [0] gmin bits, [1] boxes, [2] hits, [3] status, [4] next work item,
// [5] search pieces handed off
int run_ccd(Ctx& c, const double* x0, const double* x1, double toi_tol, int flags,
            double* toi_host, double* per)
{
    cudaStream_t st = c.stream;
    const int64_t n = c.cand.num_ee + c.cand.num_fv;
    unsigned long long* cnt = reinterpret_cast<unsigned long long*>(c.d_scalars.as<char>() + 256);
    unsigned long long init[6] = { (unsigned long long)0x7ff0000000000000ull, 0, 0, 0, 0, 0 };
    RIGC_CUDA(cudaMemcpyAsync(cnt, init, sizeof(init), cudaMemcpyHostToDevice, st));
    if (n > 0) {
        CCDArgs a;
        a.rest = c.s.rest;
        a.edges = c.s.edges;
        a.faces = c.s.faces;
        a.f2e = c.s.f2e;
        a.vbody = c.s.vbody;
        a.ebody = c.s.ebody;
        a.fbody = c.s.fbody;
        a.edge_len = c.s.edge_len;
        a.x0 = x0;
        a.x1 = x1;
        a.ee = c.cand.ee.as<int2>();
        a.fv = c.cand.fv.as<int2>();
        a.nee = c.cand.num_ee;
        a.nfv = c.cand.num_fv;
        a.toi_tol = toi_tol;
        a.prune = (flags & RIGC_TOI_NO_PRUNE) ? 0 : 1;
        a.max_boxes = c.ccd_max_boxes;
        a.gmin = cnt;
        a.bscene = c.s.bscene;
        a.scene_gmin = nullptr;
        if (c.s.nscenes > 1) {
            RIGC_TRY(c.scene_toi.reserve((size_t)c.s.nscenes * 8 + 8));
            std::vector<unsigned long long> inf(c.s.nscenes, 0x7ff0000000000000ull);
            RIGC_CUDA(cudaMemcpyAsync(c.scene_toi.ptr, inf.data(), inf.size() * 8,
                                      cudaMemcpyHostToDevice, st));
            RIGC_CUDA(cudaStreamSynchronize(st));
            a.scene_gmin = c.scene_toi.as<unsigned long long>();
        }
        a.per = per;
        a.status = reinterpret_cast<int*>(cnt + 3);
        a.boxes = cnt + 1;
        a.hits = cnt + 2;
        a.next = cnt + 4;
        // per-body frames over the table's time intervals, then the
        // per-body trajectories and fixed flags, then per-candidate tolerances
        const size_t table_bytes = (size_t)c.s.nb * kTableSlots * kTableEntry * sizeof(double);
        const size_t traj_bytes = (size_t)c.s.nb * kTrajDoubles * sizeof(double);
        RIGC_TRY(reserve_rot_table(c));
        RIGC_TRY(c.cand_tol.reserve((size_t)n * 3 * sizeof(double)));
        a.table = c.rot_table.as<double>();
        a.traj = reinterpret_cast<double*>(c.rot_table.as<char>() + table_bytes);
        a.bfixed = reinterpret_cast<int*>(c.rot_table.as<char>() + table_bytes + traj_bytes);
        a.ctol = c.cand_tol.as<double>();
        // the continuous broad phase just computed the tree nodes' frames of
        // every body a candidate can have, for these poses
        const int tree_ready = c.bp_table.valid && c.bp_table.x0 == x0 && c.bp_table.x1 == x1;
        RIGC_COUNT_LAUNCH();
        if (tree_ready && c.bp_table.toi_tol == toi_tol)
            k_traj_table<<<grid_for(c.s.nb, 128), 128, 0, st>>>(
                x0, x1, c.s.nb, const_cast<double*>(a.traj), const_cast<int*>(a.bfixed));
        else
            k_rot_table<<<grid_for((int64_t)c.s.nb * kTableSlots, 128), 128, 0, st>>>(
                x0, x1, c.s.nb, toi_tol, const_cast<double*>(a.table), const_cast<double*>(a.traj),
                const_cast<int*>(a.bfixed), tree_ready);
        // frame cache: 1024 slots per body (or the tuned count), at least
        // 2^16, at most 2^22
        const size_t per_body = c.tune.cache_slots_per_body > 0 ? c.tune.cache_slots_per_body : 1024;
        size_t slots = 1u << 16;
        while (slots < (size_t)c.s.nb * per_body && slots < (1u << 22)) slots <<= 1;
        RIGC_TRY(c.frame_keys.reserve(slots * sizeof(unsigned long long)));
        RIGC_TRY(c.frame_vals.reserve(slots * kTableEntry * sizeof(double)));
        RIGC_CUDA(cudaMemsetAsync(c.frame_keys.ptr, 0, slots * sizeof(unsigned long long), st));
        a.fkeys = c.frame_keys.as<unsigned long long>();
        a.fvals = c.frame_vals.as<double>();
        a.fmask = slots - 1;
        RIGC_COUNT_LAUNCH();
        k_ccd_prepare<<<grid_for(n, 128), 128, 0, st>>>(a);
        if (per) {
            // per-candidate results are minima over the lanes that share a search
            RIGC_COUNT_LAUNCH();
            k_fill_inf<<<grid_for(n, 256), 256, 0, st>>>(per, n);
        }
        const int mode = ccd_search_mode(c);
        // searches per block
        const int per_block = mode >= 4 ? kCCDThreads / 16 : mode ? kCCDThreads / 32 : kCCDThreads;
        int blocks_per_sm;
        RIGC_TRY(ccd_max_blocks_per_sm(&blocks_per_sm, mode));
        int dev = 0, sms = kNumSMs;
        RIGC_CUDA(cudaGetDevice(&dev));
        RIGC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const int bps = c.tune.ccd_blocks_per_sm > 0 ? std::min(c.tune.ccd_blocks_per_sm, blocks_per_sm)
                                                     : blocks_per_sm;
        int64_t full = (int64_t)sms * bps;
        // few candidates: start each search from 2^d boxes of its tree so
        // that the searches fill the GPU (prune mode; at most 32 per candidate)
        a.seeds_log2 = 0;
        if (a.prune) {
            if (c.tune.ccd_seeds_log2 >= 0) a.seeds_log2 = std::min(c.tune.ccd_seeds_log2, 5);
            else
                while (a.seeds_log2 < 5 && (n << a.seeds_log2) * 4 < full * per_block) a.seeds_log2++;
        }
        // search pieces (prune mode): launch 0 searches the seeds; a search
        // that reaches hand_off boxes once the work list has run dry hands its
        // pending boxes on, and boxes after the launch's time window are
        // deferred; k_split_pieces then gives the next launch those that
        // start before its window and keeps the others for later ones; the
        // last launch hands nothing on
        a.pieces_in = nullptr;
        a.n_pieces = 0;
        a.hand_off = 0;
        a.n_out = cnt + 5;
        a.out_cap = 0;
        a.pieces_out = nullptr;
        a.window = INFINITY;
        if (a.prune) {
            const int ho = c.tune.ccd_hand_off >= 0 ? c.tune.ccd_hand_off : kHandOff;
            const int wl = mode == 0                     ? 0
                           : c.tune.ccd_window_log2 >= 0 ? c.tune.ccd_window_log2
                           : n >= kWindowMinCandidates   ? kWindowLog2
                                                         : 0;
            unsigned long long cap = ho > 0 ? kPiecesCap : 0;
            if (wl > 0) {
                // deferred boxes: a few per candidate whose search goes deeper
                // than its root box
                if (!cap) cap = kPiecesCap;
                while (cap < kWindowCap && cap < (unsigned long long)(n << a.seeds_log2) * 2) cap *= 2;
                a.window = std::ldexp(1.0, -wl);
            }
            if (cap > 0) {
                for (int b = 0; b < 4; b++) RIGC_TRY(c.ccd_pieces[b].reserve(cap * sizeof(Piece)));
                a.hand_off = (unsigned long long)std::max(ho, 0);
                a.out_cap = cap;
                a.pieces_out = c.ccd_pieces[0].as<Piece>();
            }
        }
        // pieces: [0] a launch's output, [1] the next launch's input, [2] / [3]
        // those after its window (ping-pong)
        unsigned long long* split_n = cnt + 6;
        unsigned long long n_later = 0;
        int later = 2;
        int dev_sms = kNumSMs;
        {
            int dv = 0;
            RIGC_CUDA(cudaGetDevice(&dv));
            RIGC_CUDA(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, dv));
        }
        int64_t want = ((n << a.seeds_log2) + per_block - 1) / per_block;
        c.stats.ccd_launches = 0;
        c.stats.ccd_pieces = 0;
        for (int launch = 0;; launch++) {
            RIGC_COUNT_LAUNCH();
            const unsigned grid = (unsigned)std::min(want, full);
            switch (mode) {
            case 5: k_ccd_group<16, 4><<<grid, kCCDThreads, 0, st>>>(a); break;
            case 4: k_ccd_group<16, 1><<<grid, kCCDThreads, 0, st>>>(a); break;
            case 3: k_ccd_group<32, 5><<<grid, kCCDThreads, 0, st>>>(a); break;
            case 2: k_ccd_group<32, 4><<<grid, kCCDThreads, 0, st>>>(a); break;
            case 1: k_ccd_group<32, 1><<<grid, kCCDThreads, 0, st>>>(a); break;
            default: k_ccd<<<grid, kCCDThreads, 0, st>>>(a);
            }
            RIGC_CUDA(cudaGetLastError());
            c.stats.ccd_launches++;
            if (!a.out_cap) break;
            // the next launch's pieces: those that start before its window,
            // among this launch's and the later windows' (none after the
            // running minimum of a single scene); empty windows are skipped
            const bool last_launch = launch + 1 >= kMaxLaunches - 1;
            unsigned long long n_now = 0;
            bool from_out = true;
            for (;;) {
                const double next_window = last_launch || !(a.window < 0.5) ? INFINITY : 2 * a.window;
                RIGC_CUDA(cudaMemsetAsync(split_n, 0, 2 * sizeof(unsigned long long), st));
                RIGC_COUNT_LAUNCH();
                k_split_pieces<<<4 * dev_sms, 256, 0, st>>>(
                    c.ccd_pieces[0].as<Piece>(), from_out ? a.n_out : nullptr, a.out_cap,
                    c.ccd_pieces[later].as<Piece>(), n_later, next_window,
                    c.s.nscenes > 1 ? nullptr : a.gmin, c.ccd_pieces[1].as<Piece>(),
                    c.ccd_pieces[5 - later].as<Piece>(), split_n);
                RIGC_CUDA(cudaGetLastError());
                unsigned long long h[2];
                RIGC_CUDA(cudaMemcpyAsync(h, split_n, sizeof(h), cudaMemcpyDeviceToHost, st));
                RIGC_CUDA(cudaStreamSynchronize(st));
                n_now = std::min(h[0], a.out_cap);
                n_later = std::min(h[1], a.out_cap);
                later = 5 - later;
                a.window = next_window;
                from_out = false;
                if (n_now > 0 || n_later == 0) break;
            }
            if (n_now == 0) break;
            const unsigned long long zero[2] = { 0, 0 };
            RIGC_CUDA(cudaMemcpyAsync(a.next, zero, sizeof(zero), cudaMemcpyHostToDevice, st));
            a.pieces_in = c.ccd_pieces[1].as<Piece>();
            a.n_pieces = (long long)n_now;
            c.stats.ccd_pieces += (int64_t)n_now;
            if (last_launch) a.hand_off = 0;
            want = ((int64_t)n_now + per_block - 1) / per_block;
        }
    }
    c.bp_table.valid = false;
    unsigned long long out[4];
    RIGC_CUDA(cudaMemcpyAsync(out, cnt, sizeof(out), cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaStreamSynchronize(st));
    double g;
    std::memcpy(&g, &out[0], sizeof(g));
    *toi_host = g;  // +inf bits when no candidate found an impact
    c.h_scene_toi.assign(c.s.nscenes, INFINITY);
    if (n > 0 && c.s.nscenes > 1) {
        RIGC_CUDA(cudaMemcpyAsync(c.h_scene_toi.data(), c.scene_toi.ptr, (size_t)c.s.nscenes * 8,
                                  cudaMemcpyDeviceToHost, st));
        RIGC_CUDA(cudaStreamSynchronize(st));
    } else {
        c.h_scene_toi.assign(c.s.nscenes, g);
    }
    c.stats.ccd_boxes = (int64_t)out[1];
    c.stats.ccd_candidates = n;
    c.stats.ccd_collisions = (int64_t)out[2];
    int status = (int)(out[3] & 0xffffffffu);
    c.stats.last_status = status;
    return status;
}

} // namespace rigc
