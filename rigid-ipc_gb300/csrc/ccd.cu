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
// changes the minimum.  One thread per candidate, a depth-first stack in
// local memory, the interval vertex positions cached per time interval.  The
// interval frames R(t), p(t) of a body depend only on the body and the time
// interval, which is always a node of the dyadic bisection tree of [0, 1]:
// the top levels come from a table built per call, deeper nodes from a hash
// table filled on first use and shared by all candidates of the body.  Every
// stack and every search is bounded: on overflow or budget exhaustion the
// candidate reports the smallest t.lo still unexplored (a conservative time
// of impact) and an error status.
#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "interval.cuh"

namespace rigc {

constexpr int kCCDStack = 128;
constexpr int kCCDThreads = 128;

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
    long long max_boxes;
    unsigned long long* gmin;   // running minimum time of impact (double bits)
    double* per;                // optional per-candidate result
    int* status;                // worst status
    unsigned long long* boxes;  // total boxes evaluated
    unsigned long long* hits;   // candidates with an impact
    unsigned long long* next;   // next unprocessed candidate
    const double* table;        // per-body frames over the top dyadic time intervals
    unsigned long long* fkeys;  // frame cache: keys (0 = empty)
    double* fvals;              // frame cache: kTableEntry doubles per slot
    unsigned long long fmask;   // slots - 1 (a power of two)
};

struct Box {
    double t0, t1, a0, a1, b0, b1;
};

struct BodyTraj {
    double x0[6];
    Itv dx[6];  // I(x1) - I(x0)
};

__device__ __forceinline__ void load_traj(const double* x0, const double* x1, int b, BodyTraj& T)
{
#pragma unroll
    for (int k = 0; k < 6; k++) {
        double a = x0[6 * b + k], c = x1[6 * b + k];
        T.x0[k] = a;
        T.dx[k] = Itv { sub_dn(c, a), sub_up(c, a) };
    }
}

// R(t), p(t) of a body over the time interval t
__device__ __forceinline__ void body_at(const BodyTraj& T, const Itv& t, Itv R[9], Itv p[3])
{
    Itv r[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        p[k] = iadd(imul(T.dx[k], t), pt(T.x0[k]));
        r[k] = iadd(imul(T.dx[3 + k], t), pt(T.x0[3 + k]));
    }
    irotation(r, R);
}

// Bisection-tree node of a time interval: (1 << d) + k for [k 2^-d, (k + 1) 2^-d]
// with d < kNodeDepth, else 0.  Every time interval of the search is such a
// node (midpoints of dyadic intervals are exact), up to depth 1074.
constexpr int kNodeDepth = 40;

__device__ __forceinline__ unsigned long long time_node(double t0, double t1)
{
    int e;
    double m = frexp(t1 - t0, &e);   // exact for dyadic widths
    if (m != 0.5) return 0;
    int d = 1 - e;
    if (d < 0 || d >= kNodeDepth) return 0;
    double kd = ldexp(t0, d);
    if (kd != floor(kd) || ldexp(kd + 1.0, -d) != t1) return 0;
    return (1ull << d) + (unsigned long long)kd;
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
// bisection tree (node (1 << d) - 1 + k), computed once per call and shared by
// all candidates of the body.  The same operations produce the same bits as
// evaluating them inside a box.
constexpr int kTableDepth = 7;                          // levels 0..6
constexpr int kTableNodes = (1 << kTableDepth) - 1;     // 127
constexpr int kTableEntry = 24;                         // R (9 intervals) + p (3)

__global__ void k_rot_table(const double* __restrict__ x0, const double* __restrict__ x1, int nb,
                            double* __restrict__ table)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)nb * kTableNodes) return;
    int b = (int)(i / kTableNodes), node = (int)(i % kTableNodes);
    int d = 31 - __clz(node + 1);
    int k = node + 1 - (1 << d);
    Itv t { ldexp((double)k, -d), ldexp((double)(k + 1), -d) };
    BodyTraj T;
    load_traj(x0, x1, b, T);
    Itv R[9], p[3];
    body_at(T, t, R, p);
    frame_store(table + (size_t)i * kTableEntry, R, p);
}


struct Query {
    bool fv;            // face-vertex (else edge-edge)
    bool a_fixed;       // body A does not move: its vertex intervals never change
    bool b_fixed;
    int body_a, body_b;
    const double* table;
    unsigned long long* fkeys;
    double* fvals;
    unsigned long long fmask;
    double v[4][3];     // rest vertices: EE (a0, a1, b0, b1); FV (v, f0, f1, f2)
    BodyTraj A, B;      // EE: edge a / edge b bodies; FV: vertex / face bodies
    // cached vertex intervals for one time interval
    double ct0, ct1;
    Itv P[4][3];
};

__device__ __forceinline__ bool traj_fixed(const BodyTraj& T)
{
    bool z = true;
#pragma unroll
    for (int k = 0; k < 6; k++) z = z && T.dx[k].lo == 0.0 && T.dx[k].hi == 0.0;
    return z;
}

// vertex intervals of the bodies over t (a body that does not move has
// t-independent intervals, computed once per query)
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

static __device__ __noinline__ void frame_cached(const Query& q, const BodyTraj& T, int body,
                                                 unsigned long long node, const Itv& t,
                                                 Itv R[9], Itv p[3])
{
    const unsigned long long key = ((unsigned long long)(body + 1) << kNodeDepth) | node;
    unsigned long long h = mix64(key);
    for (int probe = 0; probe < kProbes; probe++, h++) {
        unsigned long long* slot = q.fkeys + (h & q.fmask);
        unsigned long long k = ld_acquire(slot);
        if (k == 0) {
            k = atomicCAS(slot, 0ull, key | kPending);
            if (k == 0) {
                body_at(T, t, R, p);
                frame_store(q.fvals + (h & q.fmask) * kTableEntry, R, p);
                __threadfence();
                atomicExch(slot, key);
                return;
            }
        }
        if (k == key) {
            frame_load_cg(q.fvals + (h & q.fmask) * kTableEntry, R, p);
            return;
        }
        if (k == (key | kPending)) break;
    }
    body_at(T, t, R, p);
}

__device__ __forceinline__ void frame_at(const Query& q, const BodyTraj& T, int body,
                                         unsigned long long node, const Itv& t, Itv R[9], Itv p[3])
{
    if (node != 0 && node < (1ull << kTableDepth) && q.table) {
        frame_load(q.table + ((size_t)body * kTableNodes + (node - 1)) * kTableEntry, R, p);
    } else if (node != 0 && q.fkeys) {
        frame_cached(q, T, body, node, t, R, p);
    } else {
        body_at(T, t, R, p);
    }
}

static __device__ __noinline__ void eval_vertices(Query& q, const Itv& t, bool all)
{
    Itv R[9], p[3];
    const int na = q.fv ? 1 : 2;
    const unsigned long long node = time_node(t.lo, t.hi);
    if (all || !q.a_fixed) {
        frame_at(q, q.A, q.body_a, node, t, R, p);
        for (int i = 0; i < na; i++) iworld_vertex(R, p, q.v[i], q.P[i]);
    }
    if (all || !q.b_fixed) {
        frame_at(q, q.B, q.body_b, node, t, R, p);
        for (int i = na; i < 4; i++) iworld_vertex(R, p, q.v[i], q.P[i]);
    }
    q.ct0 = t.lo;
    q.ct1 = t.hi;
}

// zero in f(box)?
__device__ __forceinline__ bool f_contains_zero(Query& q, const Box& x)
{
    Itv t { x.t0, x.t1 };
    if (!(x.t0 == q.ct0 && x.t1 == q.ct1)) eval_vertices(q, t, false);
    Itv a { x.a0, x.a1 }, b { x.b0, x.b1 };
#pragma unroll
    for (int j = 0; j < 3; j++) {
        Itv y;
        if (q.fv) {
            Itv fp = iadd(iadd(imul(isub(q.P[2][j], q.P[1][j]), a), imul(isub(q.P[3][j], q.P[1][j]), b)),
                          q.P[1][j]);
            y = isub(q.P[0][j], fp);
        } else {
            Itv ea = iadd(imul(isub(q.P[1][j], q.P[0][j]), a), q.P[0][j]);
            Itv eb = iadd(imul(isub(q.P[3][j], q.P[2][j]), b), q.P[2][j]);
            y = isub(ea, eb);
        }
        if (!zero_in(y)) return false;
    }
    return true;
}

// load candidate i and its tolerances; returns the time tolerance
__device__ __forceinline__ void load_query(const CCDArgs& a, int64_t i, Query& q, double tol[3])
{
    q.ct0 = q.ct1 = __longlong_as_double(0x7ff8000000000000ll);
    if (i < a.nee) {
        q.fv = false;
        int ea = a.ee[i].x, eb = a.ee[i].y;
        int va[2] = { a.edges[2 * ea], a.edges[2 * ea + 1] };
        int vb[2] = { a.edges[2 * eb], a.edges[2 * eb + 1] };
        for (int j = 0; j < 3; j++) {
            q.v[0][j] = a.rest[3 * (size_t)va[0] + j];
            q.v[1][j] = a.rest[3 * (size_t)va[1] + j];
            q.v[2][j] = a.rest[3 * (size_t)vb[0] + j];
            q.v[3][j] = a.rest[3 * (size_t)vb[1] + j];
        }
        q.body_a = a.ebody[ea];
        q.body_b = a.ebody[eb];
        load_traj(a.x0, a.x1, q.body_a, q.A);
        load_traj(a.x0, a.x1, q.body_b, q.B);
        tol[1] = RDIV(1e-4, a.edge_len[ea]);
        tol[2] = RDIV(1e-4, a.edge_len[eb]);
    } else {
        q.fv = true;
        int64_t k = i - a.nee;
        int f = a.fv[k].x, v = a.fv[k].y;
        int fvx[3] = { a.faces[3 * f], a.faces[3 * f + 1], a.faces[3 * f + 2] };
        for (int j = 0; j < 3; j++) {
            q.v[0][j] = a.rest[3 * (size_t)v + j];
            q.v[1][j] = a.rest[3 * (size_t)fvx[0] + j];
            q.v[2][j] = a.rest[3 * (size_t)fvx[1] + j];
            q.v[3][j] = a.rest[3 * (size_t)fvx[2] + j];
        }
        q.body_a = a.vbody[v];
        q.body_b = a.fbody[f];
        load_traj(a.x0, a.x1, q.body_a, q.A);
        load_traj(a.x0, a.x1, q.body_b, q.B);
        tol[1] = RDIV(1e-4, a.edge_len[a.f2e[3 * f]]);
        tol[2] = RDIV(1e-4, a.edge_len[a.f2e[3 * f + 1]]);
    }
    q.table = a.table;
    q.fkeys = a.fkeys;
    q.fvals = a.fvals;
    q.fmask = a.fmask;
    q.a_fixed = traj_fixed(q.A);
    q.b_fixed = traj_fixed(q.B);
    tol[0] = a.toi_tol;
    // every interval of a fixed body is the same for any t: fill all once
    Box xt { 0.0, tol[0], 0.0, tol[1], 0.0, tol[2] };
    eval_vertices(q, Itv { xt.t0, xt.t1 }, true);
    if (f_contains_zero(q, xt)) tol[0] = RDIV(tol[0], 1e2);
}

// Persistent kernel: each thread takes the next unprocessed candidate from a
// global counter whenever its box stack runs empty, so lanes of a warp keep
// evaluating boxes instead of waiting for the warp's longest search.
__global__ void __launch_bounds__(kCCDThreads)
k_ccd(CCDArgs a)
{
    const int64_t n = a.nee + a.nfv;
    unsigned long long tot_boxes = 0, tot_hits = 0;
    Query q;
    double tol[3];
    Box stack[kCCDStack];
    int sp = 0;
    int64_t cur = -1;
    double earliest = INFINITY;
    bool found = false;
    int status = RIGC_OK;
    unsigned long long cboxes = 0;
    double gbound = INFINITY;
    while (true) {
        if (sp == 0) {
            if (cur >= 0) {
                double toi = found ? earliest : INFINITY;
                if (found) {
                    atomicMin(a.gmin, (unsigned long long)__double_as_longlong(toi));
                    tot_hits++;
                }
                if (a.per) a.per[cur] = toi;
                if (status != RIGC_OK) atomicMax(a.status, status);
            }
            cur = (int64_t)atomicAdd(a.next, 1ull);
            if (cur >= n) break;
            load_query(a, cur, q, tol);
            if (a.prune)
                gbound = __longlong_as_double((long long)*(volatile unsigned long long*)a.gmin);
            stack[sp++] = Box { 0.0, 1.0, 0.0, 1.0, 0.0, 1.0 };
            earliest = INFINITY;
            found = false;
            status = RIGC_OK;
            cboxes = 0;
            continue;
        }
        Box x = stack[--sp];
        if (x.t0 >= earliest) continue;
        if (a.prune) {
            if ((tot_boxes & 7) == 0)
                gbound = __longlong_as_double((long long)*(volatile unsigned long long*)a.gmin);
            if (x.t0 >= gbound) continue;
        }
        if (q.fv) {
            double sl = add_dn(x.a0, x.b0), sh = add_up(x.a1, x.b1);
            if (!(sl <= 1.0 && 0.0 <= sh)) continue;
        }
        if (cboxes >= (unsigned long long)a.max_boxes) {
            // budget exhausted: the earliest unexplored t.lo is conservative
            double m = x.t0;
            for (int s = 0; s < sp; s++) m = smin(m, stack[s].t0);
            earliest = smin(earliest, m);
            found = true;
            status = RIGC_ERR_ITER_LIMIT;
            sp = 0;
            continue;
        }
        cboxes++;
        tot_boxes++;
        if (!f_contains_zero(q, x)) continue;
        double w[3] = { sub_up(x.t1, x.t0), sub_up(x.a1, x.a0), sub_up(x.b1, x.b0) };
        bool all_tol = w[0] <= tol[0] && w[1] <= tol[1] && w[2] <= tol[2];
        bool all_zero = w[0] <= 1e-10 && w[1] <= 1e-10 && w[2] <= 1e-10;
        if ((x.t0 > 0 || all_zero) && all_tol) {
            earliest = x.t0;
            found = true;
            if (a.prune) {
                atomicMin(a.gmin, (unsigned long long)__double_as_longlong(earliest));
                gbound = smin(gbound, earliest);
            }
            continue;
        }
        int split = -1;
#pragma unroll
        for (int d = 0; d < 3; d++)
            if ((all_tol || w[d] > tol[d])
                && (split == -1 || RMUL(w[d], tol[split]) > RMUL(w[split], tol[d])))
                split = d;
        Box lo = x, hi = x;
        if (split == 0) {
            double m = RMUL(0.5, RADD(x.t0, x.t1));
            lo.t1 = m;
            hi.t0 = m;
        } else if (split == 1) {
            double m = RMUL(0.5, RADD(x.a0, x.a1));
            lo.a1 = m;
            hi.a0 = m;
        } else {
            double m = RMUL(0.5, RADD(x.b0, x.b1));
            lo.b1 = m;
            hi.b0 = m;
        }
        if (sp + 2 > kCCDStack) {
            // cannot descend: keep the box's start as a conservative root
            earliest = smin(earliest, x.t0);
            found = true;
            status = RIGC_ERR_QUEUE_OVERFLOW;
            continue;
        }
        stack[sp++] = hi;
        stack[sp++] = lo;
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

// counters layout in the context's device scalars (byte offset 256):
// [0] gmin bits, [1] boxes, [2] hits, [3] status, [4] next candidate
int run_ccd(Ctx& c, const double* x0, const double* x1, double toi_tol, int flags,
            double* toi_host, double* per)
{
    cudaStream_t st = c.stream;
    const int64_t n = c.cand.num_ee + c.cand.num_fv;
    unsigned long long* cnt = reinterpret_cast<unsigned long long*>(c.d_scalars.as<char>() + 256);
    unsigned long long init[5] = { (unsigned long long)0x7ff0000000000000ull, 0, 0, 0, 0 };
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
        a.max_boxes = 1ll << 22;
        a.gmin = cnt;
        a.per = per;
        a.status = reinterpret_cast<int*>(cnt + 3);
        a.boxes = cnt + 1;
        a.hits = cnt + 2;
        a.next = cnt + 4;
        RIGC_TRY(c.rot_table.reserve((size_t)c.s.nb * kTableNodes * kTableEntry * sizeof(double)));
        RIGC_COUNT_LAUNCH();
        k_rot_table<<<grid_for((int64_t)c.s.nb * kTableNodes, 128), 128, 0, st>>>(
            x0, x1, c.s.nb, c.rot_table.as<double>());
        a.table = c.rot_table.as<double>();
        // frame cache: 1024 slots per body, at least 2^16, at most 2^22
        size_t slots = 1u << 16;
        while (slots < (size_t)c.s.nb * 1024 && slots < (1u << 22)) slots <<= 1;
        RIGC_TRY(c.frame_keys.reserve(slots * sizeof(unsigned long long)));
        RIGC_TRY(c.frame_vals.reserve(slots * kTableEntry * sizeof(double)));
        RIGC_CUDA(cudaMemsetAsync(c.frame_keys.ptr, 0, slots * sizeof(unsigned long long), st));
        a.fkeys = c.frame_keys.as<unsigned long long>();
        a.fvals = c.frame_vals.as<double>();
        a.fmask = slots - 1;
        static int blocks_per_sm = 0;
        if (!blocks_per_sm) {
            RIGC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_ccd,
                                                                    kCCDThreads, 0));
            if (blocks_per_sm < 1) blocks_per_sm = 1;
        }
        int dev = 0, sms = kNumSMs;
        RIGC_CUDA(cudaGetDevice(&dev));
        RIGC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        int64_t want = (n + kCCDThreads - 1) / kCCDThreads;
        int64_t full = (int64_t)sms * blocks_per_sm;
        RIGC_COUNT_LAUNCH();
        k_ccd<<<(unsigned)std::min(want, full), kCCDThreads, 0, st>>>(a);
        RIGC_CUDA(cudaGetLastError());
    }
    unsigned long long out[4];
    RIGC_CUDA(cudaMemcpyAsync(out, cnt, sizeof(out), cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaStreamSynchronize(st));
    double g;
    std::memcpy(&g, &out[0], sizeof(g));
    *toi_host = out[2] ? g : INFINITY;
    c.stats.ccd_boxes = (int64_t)out[1];
    c.stats.ccd_candidates = n;
    c.stats.ccd_collisions = (int64_t)out[2];
    int status = (int)(out[3] & 0xffffffffu);
    c.stats.last_status = status;
    return status;
}

} // namespace rigc
