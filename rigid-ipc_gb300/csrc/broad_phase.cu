// Rigid hash-grid broad phase on the device.
//
// Replaces detect_collision_candidates_rigid with DetectionMethod::HASH_GRID
// (src/ccd/rigid/broad_phase.cpp:19-91 discrete, 127-204 continuous):
//  1. body boxes (RigidBody::compute_bounding_box, src/physics/rigid_body.cpp:
//     246-272) grown by the inflation radius; bodies in some overlapping pair
//     of different groups are included (close_bodies_bvh,
//     src/physics/rigid_body_assembler.cpp:307-356);
//  2. vertex boxes: continuous -- interval positions over t in [0, 1] with one
//     forced bisection, bisected further while a body's vertices leave the
//     padded scene box (RigidBodyHashGrid::compute_vertices_intervals,
//     src/ccd/rigid/rigid_body_hash_grid.cpp:164-246): a thread per vertex
//     over the two forced halves, and one CUDA block per body for the bodies
//     that need deeper bisection; discrete -- the world vertex +- inflation.
//     Edge and face boxes are unions of their vertex boxes (:265-344);
//  3. pairs: ipc-toolkit's HashGrid reports element pairs that share a cell,
//     belong to different groups and whose boxes overlap (center /
//     half-extent test).  Because the boxes overlap, that set does not depend
//     on the cell layout, which leaves the grid free:
//     * the grid (origin, cell size) is computed on the device from the
//       element boxes;
//     * a cell filter marks every cell that elements of two or more groups
//       cover (one int per cell, or per hashed slot of cells: a collision
//       only marks more cells); only marked cells are binned, so cells
//       inside one body's surface -- most of a contact scene -- cost nothing;
//     * items are sorted by (scene, cell, group, first-cell bits); an item
//       pairs only with items of later groups of its cell, and a pair is
//       reported in the first cell both elements cover (the cell where each
//       axis starts one of the two ranges: three bits per item);
//     * a conservative single-precision box test (outward-rounded floats)
//       rejects most pairs before the double-precision overlap test;
//     * elements spanning more than kLargeCells cells are tested against all
//       elements of their scene instead of being binned.
//     The output is the same set, sorted: ee as (edge0 < edge1), fv as
//     (face, vertex).
#include "common.cuh"
#include "interval.cuh"
#include "sort.cuh"

namespace rigc {

constexpr int kLargeCells = 64;

// ---------------------------------------------------------------------------
// 1. body boxes and inclusion

__global__ void k_body_boxes(const double* __restrict__ x0, const double* __restrict__ x1,
                             const double* __restrict__ rest, const int* __restrict__ bvs,
                             const int* __restrict__ type, const double* __restrict__ rmax, int nb,
                             double* __restrict__ box)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nb) return;
    const int b = warp;
    const double* p0 = x0 + 6 * b;
    const double* p1 = x1 + 6 * b;
    double lo[3], hi[3];
    bool same_rot = p0[3] == p1[3] && p0[4] == p1[4] && p0[5] == p1[5];
    if (type[b] == RIGC_BODY_STATIC || same_rot) {
        for (int j = 0; j < 3; j++) {
            lo[j] = INFINITY;
            hi[j] = -INFINITY;
        }
        for (int s = 0; s < 2; s++) {
            const double* pp = s ? p1 : p0;
            double t[3] = { pp[3], pp[4], pp[5] };
            double R[9];
            rot_rn(t, R);
            double p[3] = { pp[0], pp[1], pp[2] };
            for (int v = bvs[b] + lane; v < bvs[b + 1]; v += 32) {
                double r[3] = { rest[3 * (size_t)v], rest[3 * (size_t)v + 1], rest[3 * (size_t)v + 2] };
                double w[3];
                world_vertex_rn(R, p, r, w);
                for (int j = 0; j < 3; j++) {
                    lo[j] = smin(lo[j], w[j]);
                    hi[j] = smax(hi[j], w[j]);
                }
            }
        }
        for (int o = 16; o > 0; o >>= 1)
            for (int j = 0; j < 3; j++) {
                lo[j] = smin(lo[j], __shfl_xor_sync(0xffffffffu, lo[j], o));
                hi[j] = smax(hi[j], __shfl_xor_sync(0xffffffffu, hi[j], o));
            }
    } else {
        for (int j = 0; j < 3; j++) {
            lo[j] = RSUB(smin(p0[j], p1[j]), rmax[b]);
            hi[j] = RADD(smax(p0[j], p1[j]), rmax[b]);
        }
    }
    if (lane == 0)
        for (int j = 0; j < 3; j++) {
            box[6 * b + j] = lo[j];
            box[6 * b + 3 + j] = hi[j];
        }
}

// body pairs of one scene whose inflated boxes overlap (different groups):
// one thread per (body, later body of the same scene)
__global__ void k_close_bodies(const double* __restrict__ box, const int* __restrict__ group,
                               const int* __restrict__ bscene, const int* __restrict__ scene_bstart,
                               const int* __restrict__ scene_on, int nb, int chunk, double infl,
                               int* __restrict__ body_in)
{
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int i = (int)(t / chunk);
    if (i >= nb) return;
    if (scene_on && !scene_on[bscene[i]]) return;
    const int end = scene_bstart[bscene[i] + 1];
    for (int j = i + 1 + (int)(t % chunk); j < end; j += chunk) {
        if (group[i] == group[j]) continue;
        bool overlap = true;
        for (int k = 0; k < 3; k++) {
            double li = RSUB(box[6 * i + k], infl), hi_i = RADD(box[6 * i + 3 + k], infl);
            double lj = RSUB(box[6 * j + k], infl), hj = RADD(box[6 * j + 3 + k], infl);
            if (li > hj || lj > hi_i) overlap = false;
        }
        if (overlap) {
            body_in[i] = 1;
            body_in[j] = 1;
        }
    }
}

// scene box over included bodies (unpadded box of compute_bounding_box)
__global__ void k_scene_box(const double* __restrict__ box, const int* __restrict__ body_in, int nb,
                            double* __restrict__ out)
{
    // per thread over a stride of bodies, then a tree over the block (the
    // minimum and maximum are exact, so the order does not matter)
    __shared__ double sh[6][256];
    double lo[3] = { INFINITY, INFINITY, INFINITY }, hi[3] = { -INFINITY, -INFINITY, -INFINITY };
    for (int b = threadIdx.x; b < nb; b += blockDim.x)
        if (body_in[b])
            for (int j = 0; j < 3; j++) {
                lo[j] = smin(lo[j], box[6 * b + j]);
                hi[j] = smax(hi[j], box[6 * b + 3 + j]);
            }
    for (int j = 0; j < 3; j++) {
        sh[j][threadIdx.x] = lo[j];
        sh[3 + j][threadIdx.x] = hi[j];
    }
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int j = 0; j < 3; j++) {
                sh[j][threadIdx.x] = smin(sh[j][threadIdx.x], sh[j][threadIdx.x + w]);
                sh[3 + j][threadIdx.x] = smax(sh[3 + j][threadIdx.x], sh[3 + j][threadIdx.x + w]);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int j = 0; j < 3; j++) {
            lo[j] = sh[j][0];
            hi[j] = sh[3 + j][0];
        }
        double d0 = RSUB(hi[0], lo[0]), d1 = RSUB(hi[1], lo[1]), d2 = RSUB(hi[2], lo[2]);
        double diag = __dsqrt_rn(RADD(RADD(RMUL(d0, d0), RMUL(d1, d1)), RMUL(d2, d2)));
        for (int j = 0; j < 3; j++) {
            out[j] = RSUB(lo[j], RMUL(1e-8, diag));
            out[3 + j] = RADD(hi[j], RMUL(1e-8, diag));
        }
    }
}

// ---------------------------------------------------------------------------
// 2. vertex boxes

constexpr int kVBThreads = 256;
constexpr int kHalfFrame = 24;                   // doubles per interval frame: R (9 intervals), p (3)
constexpr int kVBBatch = 32;                     // time nodes evaluated together
constexpr int kMaxTNodes = 17 * 2 * kVBBatch;    // pending nodes (see below)
constexpr int kMaxTDepth = 16;                   // bisection stops at this depth

// interval frame (R as 9 intervals, p as 3) of body b over the time
// interval [tl, th]: the interpolated pose of PoseI::interpolate
// (src/physics/pose.tpp:142-148) through the rotation-vector map
__device__ void body_time_frame(const double* __restrict__ x0, const double* __restrict__ x1, int b,
                                double tl, double th, double* __restrict__ out)
{
    const Itv t { tl, th };
    Itv r[3], p[3];
    for (int k = 0; k < 3; k++) {
        double a = x0[6 * b + k], c = x1[6 * b + k];
        p[k] = iadd(imul(Itv { sub_dn(c, a), sub_up(c, a) }, t), pt(a));
        double ar = x0[6 * b + 3 + k], cr = x1[6 * b + 3 + k];
        r[k] = iadd(imul(Itv { sub_dn(cr, ar), sub_up(cr, ar) }, t), pt(ar));
    }
    Itv R[9];
    irotation(r, R);
    for (int k = 0; k < 9; k++) {
        out[2 * k] = R[k].lo;
        out[2 * k + 1] = R[k].hi;
    }
    for (int k = 0; k < 3; k++) {
        out[18 + 2 * k] = p[k].lo;
        out[19 + 2 * k] = p[k].hi;
    }
}

__device__ __forceinline__ void vertex_at_frame(const double* f, const double rv[3], Itv w[3])
{
    Itv R[9], p[3];
    for (int k = 0; k < 9; k++) R[k] = Itv { f[2 * k], f[2 * k + 1] };
    for (int k = 0; k < 3; k++) p[k] = Itv { f[18 + 2 * k], f[19 + 2 * k] };
    iworld_vertex(R, p, rv, w);
}

// The whole bisection of RigidBodyHashGrid::compute_vertices_intervals for
// one body per block: block b handles body b when it is included and
// k_vertex_boxes_half flagged it (a vertex of one of the forced halves left
// the padded scene box).  A time node is accepted when every vertex fits
// the padded scene box (or at depth 16), else both halves are visited; the
// result per vertex is the hull over the accepted nodes, which does not
// depend on the order nodes are visited.  So nodes are taken from the stack
// kVBBatch at a time: warp 0 computes their frames in parallel (one interval
// rotation is a long chain of dependent FP64 operations), then the block
// checks and hulls every (node, vertex) pair.  Each round pops up to
// kVBBatch nodes and pushes at most twice as many one level deeper, so the
// stack never holds more than 2 kVBBatch nodes per depth.
// vbox holds lo[3], hi[3] per vertex.
__global__ void __launch_bounds__(kVBThreads)
k_vertex_boxes_cont(const double* __restrict__ x0, const double* __restrict__ x1,
                    const double* __restrict__ rest, const int* __restrict__ bvs,
                    const int* __restrict__ body_in, const int* __restrict__ deeper,
                    const double* __restrict__ table, const double* __restrict__ domain,
                    double infl, double* __restrict__ vbox, char* __restrict__ vin)
{
    __shared__ double st_lo[kMaxTNodes], st_hi[kMaxTNodes];
    __shared__ int st_depth[kMaxTNodes];
    __shared__ int sp, nbat;
    __shared__ double b_lo[kVBBatch], b_hi[kVBBatch];
    __shared__ int b_depth[kVBBatch], b_fail[kVBBatch];
    __shared__ double sF[kVBBatch][kHalfFrame];
    const int b = blockIdx.x;
    if (!body_in[b] || !deeper[b]) return;  // uniform over the block
    const int v0 = bvs[b], v1 = bvs[b + 1], nvb = v1 - v0;
    double dlo[3] = { domain[0], domain[1], domain[2] }, dhi[3] = { domain[3], domain[4], domain[5] };
    // hull accumulators in the output array
    for (int v = v0 + threadIdx.x; v < v1; v += blockDim.x)
        for (int j = 0; j < 3; j++) {
            vbox[6 * (size_t)v + j] = INFINITY;
            vbox[6 * (size_t)v + 3 + j] = -INFINITY;
        }
    if (threadIdx.x == 0) {
        // forced first bisection: [0, 0.5] and [0.5, 1], depth 1
        sp = 0;
        double m = RMUL(0.5, RADD(0.0, 1.0));
        st_lo[sp] = m; st_hi[sp] = 1.0; st_depth[sp] = 1; sp++;
        st_lo[sp] = 0.0; st_hi[sp] = m; st_depth[sp] = 1; sp++;
    }
    while (true) {
        __syncthreads();
        if (sp == 0) break;
        // pop up to kVBBatch nodes
        if (threadIdx.x < kVBBatch) {
            const int nb_ = min(sp, kVBBatch);
            if ((int)threadIdx.x < nb_) {
                const int q = sp - nb_ + threadIdx.x;
                b_lo[threadIdx.x] = st_lo[q];
                b_hi[threadIdx.x] = st_hi[q];
                b_depth[threadIdx.x] = st_depth[q];
                b_fail[threadIdx.x] = 0;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            nbat = min(sp, kVBBatch);
            sp -= nbat;
        }
        __syncthreads();
        const int nq = nbat;
        if ((int)threadIdx.x < nq) {
            // nodes of depth <= 6 from the table (their intervals are the
            // dyadic [k 2^-d, (k + 1) 2^-d], midpoints being exact), deeper
            // ones computed here
            const int d = b_depth[threadIdx.x];
            if (d < 7) {
                const int k = (int)ldexp(b_lo[threadIdx.x], d);
                const double* f = table + ((size_t)b * kRotTableSlots + (1 << d) - 1 + k) * kRotTableEntry;
                for (int j = 0; j < kHalfFrame; j++) sF[threadIdx.x][j] = f[j];
            } else {
                body_time_frame(x0, x1, b, b_lo[threadIdx.x], b_hi[threadIdx.x], sF[threadIdx.x]);
            }
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < nq * nvb; idx += blockDim.x) {
            const int k = idx / nvb, v = v0 + idx % nvb;
            const double rv[3] = { rest[3 * (size_t)v], rest[3 * (size_t)v + 1], rest[3 * (size_t)v + 2] };
            Itv w[3];
            vertex_at_frame(sF[k], rv, w);
            for (int j = 0; j < 3; j++)
                if (RSUB(w[j].lo, infl) < dlo[j] || RADD(w[j].hi, infl) > dhi[j]) b_fail[k] = 1;
        }
        __syncthreads();
        // accepted nodes: hull into the vertex boxes (each thread owns its vertices)
        for (int v = v0 + threadIdx.x; v < v1; v += blockDim.x) {
            const double rv[3] = { rest[3 * (size_t)v], rest[3 * (size_t)v + 1], rest[3 * (size_t)v + 2] };
            for (int k = 0; k < nq; k++) {
                if (b_fail[k] && b_depth[k] < kMaxTDepth) continue;
                Itv w[3];
                vertex_at_frame(sF[k], rv, w);
                for (int j = 0; j < 3; j++) {
                    vbox[6 * (size_t)v + j] = smin(vbox[6 * (size_t)v + j], w[j].lo);
                    vbox[6 * (size_t)v + 3 + j] = smax(vbox[6 * (size_t)v + 3 + j], w[j].hi);
                }
            }
        }
        // rejected nodes: both halves, one level deeper
        if (threadIdx.x == 0)
            for (int k = 0; k < nq; k++) {
                if (!b_fail[k] || b_depth[k] >= kMaxTDepth) continue;
                const double tl = b_lo[k], th = b_hi[k];
                const double m = RMUL(0.5, RADD(tl, th));
                if (sp + 2 <= kMaxTNodes) {
                    st_lo[sp] = m; st_hi[sp] = th; st_depth[sp] = b_depth[k] + 1; sp++;
                    st_lo[sp] = tl; st_hi[sp] = m; st_depth[sp] = b_depth[k] + 1; sp++;
                }
            }
    }
    // inflate; a vertex with an empty coordinate stays excluded
    for (int v = v0 + threadIdx.x; v < v1; v += blockDim.x) {
        bool ok = true;
        for (int j = 0; j < 3; j++) {
            double lo = vbox[6 * (size_t)v + j], hi = vbox[6 * (size_t)v + 3 + j];
            if (!(lo <= hi)) ok = false;
            vbox[6 * (size_t)v + j] = RSUB(lo, infl);
            vbox[6 * (size_t)v + 3 + j] = RADD(hi, infl);
        }
        vin[v] = ok ? 1 : 0;
    }
}

// Interval frames of every included body over the dyadic time nodes of
// depth 0 .. 6 (table slot 2^d - 1 + k for [k 2^-d, (k + 1) 2^-d]): the
// forced halves and the nodes the deeper bisection visits first.  They are
// the CCD's frames for the same poses (PoseI::interpolate through the same
// interval operations; a product with a non-negative time interval gives
// the same bits in either form), so the CCD that follows on these poses
// takes them over, with slot 127: [0, toi_tol], the interval of the
// tolerance test every candidate's search starts with.  One thread per
// (included body, slot).
constexpr int kBPTableNodes = 127;  // slots 0 .. 126: depths 0 .. 6

__global__ void k_bp_frames(const double* __restrict__ x0, const double* __restrict__ x1,
                            const int* __restrict__ body_in, int nb, double toi_tol,
                            double* __restrict__ table)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)nb * kRotTableSlots) return;
    const int b = (int)(i / kRotTableSlots), slot = (int)(i % kRotTableSlots);
    if (!body_in[b]) return;
    const int d = 31 - __clz(slot + 1);
    const int k = slot + 1 - (1 << d);
    double* out = table + ((size_t)b * kRotTableSlots + slot) * kRotTableEntry;
    if (slot == kBPTableNodes) body_time_frame(x0, x1, b, 0.0, toi_tol, out);
    else body_time_frame(x0, x1, b, ldexp((double)k, -d), ldexp((double)(k + 1), -d), out);
}

// One thread per vertex: its interval positions over the two forced halves,
// their hull, inflated.  When every vertex of a body stays inside the padded
// scene box on both halves, this is the body's whole bisection (both halves
// accepted at depth 1, hulled in the order the stack visits them: [0, 1/2]
// first); otherwise the body is flagged in `deeper` and k_vertex_boxes_cont
// redoes it.
__global__ void k_vertex_boxes_half(const double* __restrict__ rest, const int* __restrict__ vbody,
                                    const int* __restrict__ body_in, int nv,
                                    const double* __restrict__ fr, const double* __restrict__ domain,
                                    double infl, double* __restrict__ vbox, char* __restrict__ vin,
                                    int* __restrict__ deeper)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    const int b = vbody[v];
    if (!body_in[b]) {
        vin[v] = 0;
        return;
    }
    const double rv[3] = { rest[3 * (size_t)v], rest[3 * (size_t)v + 1], rest[3 * (size_t)v + 2] };
    double lo[3] = { INFINITY, INFINITY, INFINITY }, hi[3] = { -INFINITY, -INFINITY, -INFINITY };
    bool fits = true;
    for (int half = 0; half < 2; half++) {
        Itv w[3];
        vertex_at_frame(fr + ((size_t)b * kRotTableSlots + 1 + half) * kRotTableEntry, rv, w);
        for (int j = 0; j < 3; j++) {
            if (RSUB(w[j].lo, infl) < domain[j] || RADD(w[j].hi, infl) > domain[3 + j]) fits = false;
            lo[j] = smin(lo[j], w[j].lo);
            hi[j] = smax(hi[j], w[j].hi);
        }
    }
    if (!fits) atomicOr(&deeper[b], 1);
    bool ok = true;
    for (int j = 0; j < 3; j++) {
        if (!(lo[j] <= hi[j])) ok = false;
        vbox[6 * (size_t)v + j] = RSUB(lo[j], infl);
        vbox[6 * (size_t)v + 3 + j] = RADD(hi[j], infl);
    }
    vin[v] = ok ? 1 : 0;
}

__global__ void k_vertex_boxes_disc(const double* __restrict__ rot, const double* __restrict__ rest,
                                    const int* __restrict__ vbody, const int* __restrict__ body_in,
                                    int nv, double infl, double* __restrict__ vbox,
                                    char* __restrict__ vin)
{
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    int b = vbody[v];
    if (!body_in[b]) {
        vin[v] = 0;
        return;
    }
    const double* f = rot + 12 * b;
    double R[9], p[3], r[3], w[3];
    for (int k = 0; k < 9; k++) R[k] = f[k];
    for (int k = 0; k < 3; k++) {
        p[k] = f[9 + k];
        r[k] = rest[3 * (size_t)v + k];
    }
    world_vertex_rn(R, p, r, w);
    for (int j = 0; j < 3; j++) {
        vbox[6 * (size_t)v + j] = RSUB(w[j], infl);
        vbox[6 * (size_t)v + 3 + j] = RADD(w[j], infl);
    }
    vin[v] = 1;
}

__global__ void k_edge_face_boxes(const int* __restrict__ E, int ne, const int* __restrict__ F, int nf,
                                  const double* __restrict__ vbox, const char* __restrict__ vin,
                                  double* __restrict__ ebox, char* __restrict__ ein,
                                  double* __restrict__ fbox, char* __restrict__ fin)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ne) {
        int a = E[2 * i], b = E[2 * i + 1];
        bool ok = vin[a] && vin[b];
        ein[i] = ok;
        if (ok)
            for (int j = 0; j < 3; j++) {
                ebox[6 * (size_t)i + j] = smin(vbox[6 * (size_t)a + j], vbox[6 * (size_t)b + j]);
                ebox[6 * (size_t)i + 3 + j] = smax(vbox[6 * (size_t)a + 3 + j], vbox[6 * (size_t)b + 3 + j]);
            }
    } else if (i < ne + nf) {
        int k = i - ne;
        int a = F[3 * k], b = F[3 * k + 1], c = F[3 * k + 2];
        bool ok = vin[a] && vin[b] && vin[c];
        fin[k] = ok;
        if (ok)
            for (int j = 0; j < 3; j++) {
                double lo = smin(smin(vbox[6 * (size_t)a + j], vbox[6 * (size_t)b + j]), vbox[6 * (size_t)c + j]);
                double hi = smax(smax(vbox[6 * (size_t)a + 3 + j], vbox[6 * (size_t)b + 3 + j]),
                                 vbox[6 * (size_t)c + 3 + j]);
                fbox[6 * (size_t)k + j] = lo;
                fbox[6 * (size_t)k + 3 + j] = hi;
            }
    }
}

// ---------------------------------------------------------------------------
// 3. hash grid

// The grid of one call, computed on the device from the element boxes.
struct Grid {
    double lo[3];
    double cell, grow;
    double inv_cell;            // RN(1 / cell): cell indices by multiplication
    long long dims[3];
    unsigned long long ncells;  // dims[0] * dims[1] * dims[2]
    int dense;                  // cell-filter slot = (scene, cell) key; else a hash of it
    int key_bits;               // bits of the largest (scene, cell) key
};

constexpr int kStatBlocks = 1024;
constexpr int kStatThreads = 256;
constexpr long long kMaxAxisCells = 1ll << 21;
// cell-filter slot states; a group rank (>= 0) otherwise
constexpr int kSlotEmpty = -1;
constexpr int kSlotMulti = -2;

// element tags: type in the top 2 bits (0 vertex, 1 edge, 2 face)
__device__ __forceinline__ uint32_t tag(int type, int id) { return ((uint32_t)type << 30) | (uint32_t)id; }

// every element in one index space: vertices, then edges, then faces
struct Elems {
    const double* vb;
    const double* eb;
    const double* fb;
    const char* vin;
    const char* ein;
    const char* fin;
    const int* vbody;
    const int* ebody;
    const int* fbody;
    int nv, ne, nf;
    __device__ __forceinline__ int type(int64_t e) const { return e < nv ? 0 : (e < nv + ne ? 1 : 2); }
    __device__ __forceinline__ int id(int64_t e, int t) const
    {
        return (int)(t == 0 ? e : (t == 1 ? e - nv : e - nv - ne));
    }
    __device__ __forceinline__ int64_t index(int t, int i) const
    {
        return t == 0 ? i : (t == 1 ? (int64_t)nv + i : (int64_t)nv + ne + i);
    }
    __device__ __forceinline__ const double* box(int t, int i) const
    {
        return (t == 0 ? vb : (t == 1 ? eb : fb)) + 6 * (size_t)i;
    }
    __device__ __forceinline__ bool in(int t, int i) const
    {
        return (t == 0 ? vin : (t == 1 ? ein : fin))[i] != 0;
    }
    __device__ __forceinline__ int body(int t, int i) const
    {
        return (t == 0 ? vbody : (t == 1 ? ebody : fbody))[i];
    }
};

// Cell index along axis j: floor((x - lo) / cell) computed as a product with
// the reciprocal.  Any index function works as long as it is monotone in x
// and the same for every element (two boxes sharing a point share that
// point's cell); round-to-nearest subtraction and multiplication are.
__device__ __forceinline__ long long cell_of(double x, const Grid& g, int j)
{
    long long c = (long long)floor(RMUL(RSUB(x, g.lo[j]), g.inv_cell));
    return c < 0 ? 0 : (c >= g.dims[j] ? g.dims[j] - 1 : c);
}

__device__ __forceinline__ void cell_range(const double* b, const Grid& g, long long c0[3], long long c1[3])
{
    for (int j = 0; j < 3; j++) {
        c0[j] = cell_of(RSUB(b[j], g.grow), g, j);
        c1[j] = cell_of(RADD(b[3 + j], g.grow), g, j);
    }
}

// ipc-toolkit's AABB overlap test (center / half-extent), in round-to-nearest
__device__ __forceinline__ bool boxes_overlap(const double* a, const double* b)
{
#pragma unroll
    for (int i = 0; i < 3; i++) {
        double ha = RSUB(a[3 + i], a[i]) / 2, hb = RSUB(b[3 + i], b[i]) / 2;
        double ca = RADD(a[i], ha), cb = RADD(b[i], hb);
        if (!(fabs(RSUB(ca, cb)) <= RADD(ha, hb))) return false;
    }
    return true;
}

// Single-precision boxes rounded outward.  If they are disjoint on an axis,
// a float lies strictly between the two double intervals, so their gap is
// at least one float ulp of the coordinates -- far beyond the few double
// ulps by which the round-to-nearest test above can misjudge a gap -- and
// that test rejects the pair too.  So this test only drops pairs the exact
// test drops.
__device__ __forceinline__ bool fboxes_disjoint(const float* a, const float* b)
{
#pragma unroll
    for (int i = 0; i < 3; i++)
        if (a[i] > b[3 + i] || b[i] > a[3 + i]) return true;
    return false;
}

__device__ __forceinline__ uint64_t mix64(uint64_t x)
{
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

__device__ __forceinline__ uint64_t slot_of(uint64_t key, const Grid& g, uint64_t mask)
{
    return g.dense ? key : (mix64(key) & mask);
}

// bounds of the included element boxes and the sum of the included edges'
// largest box extents (fixed grid, fixed reduction order: deterministic)
__global__ void __launch_bounds__(kStatThreads) k_elem_stats(Elems E, double* __restrict__ part,
                                                             int* __restrict__ part_n)
{
    __shared__ double sh[7][kStatThreads];
    __shared__ int shn[kStatThreads];
    double lo[3] = { INFINITY, INFINITY, INFINITY }, hi[3] = { -INFINITY, -INFINITY, -INFINITY };
    double ext = 0;
    int ned = 0;
    const int64_t n = (int64_t)E.nv + E.ne + E.nf;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int t = E.type(e), i = E.id(e, t);
        if (!E.in(t, i)) continue;
        const double* b = E.box(t, i);
        double x = 0;
        for (int j = 0; j < 3; j++) {
            lo[j] = smin(lo[j], b[j]);
            hi[j] = smax(hi[j], b[3 + j]);
            x = smax(x, RSUB(b[3 + j], b[j]));
        }
        if (t == 1) {
            ext = RADD(ext, x);
            ned++;
        }
    }
    for (int j = 0; j < 3; j++) {
        sh[j][threadIdx.x] = lo[j];
        sh[3 + j][threadIdx.x] = hi[j];
    }
    sh[6][threadIdx.x] = ext;
    shn[threadIdx.x] = ned;
    __syncthreads();
    for (int o = kStatThreads / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            for (int j = 0; j < 3; j++) {
                sh[j][threadIdx.x] = smin(sh[j][threadIdx.x], sh[j][threadIdx.x + o]);
                sh[3 + j][threadIdx.x] = smax(sh[3 + j][threadIdx.x], sh[3 + j][threadIdx.x + o]);
            }
            sh[6][threadIdx.x] = RADD(sh[6][threadIdx.x], sh[6][threadIdx.x + o]);
            shn[threadIdx.x] += shn[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int j = 0; j < 7; j++) part[7 * blockIdx.x + j] = sh[j][0];
        part_n[blockIdx.x] = shn[0];
    }
}

__device__ __forceinline__ int dbits_for(unsigned long long v)
{
    return v == 0 ? 1 : 64 - __clzll((long long)v);
}

// Grid from the partial statistics: cell = the mean extent of the included
// edge boxes (at least half the mean rest edge length), doubled while the
// grid is too large for the keys (a cell size changes only the work, never
// the pairs); one thread
__global__ void k_grid_setup(const double* __restrict__ part, const int* __restrict__ part_n, int nblk,
                             double avg_edge_len, int nscenes, int group_bits, uint64_t nslots,
                             Grid* __restrict__ out)
{
    // one warp reduces the partials in a fixed order (lane-strided, then a
    // butterfly), lane 0 sets the grid up
    const int lane = threadIdx.x & 31;
    double lo[3] = { INFINITY, INFINITY, INFINITY }, hi[3] = { -INFINITY, -INFINITY, -INFINITY };
    double ext = 0;
    long long ned = 0;
    for (int b = lane; b < nblk; b += 32) {
        for (int j = 0; j < 3; j++) {
            lo[j] = smin(lo[j], part[7 * b + j]);
            hi[j] = smax(hi[j], part[7 * b + 3 + j]);
        }
        ext = RADD(ext, part[7 * b + 6]);
        ned += part_n[b];
    }
    for (int o = 16; o > 0; o >>= 1) {
        for (int j = 0; j < 3; j++) {
            lo[j] = smin(lo[j], __shfl_xor_sync(0xffffffffu, lo[j], o));
            hi[j] = smax(hi[j], __shfl_xor_sync(0xffffffffu, hi[j], o));
        }
        // the same sum in both lanes of a pair: lower lane's value first
        const double e2 = __shfl_xor_sync(0xffffffffu, ext, o);
        ext = (lane & o) ? RADD(e2, ext) : RADD(ext, e2);
        ned += __shfl_xor_sync(0xffffffffu, ned, o);
    }
    if (lane != 0) return;
    Grid g;
    bool empty = false;
    for (int j = 0; j < 3; j++)
        if (!(lo[j] <= hi[j]) || !isfinite(lo[j]) || !isfinite(hi[j])) empty = true;
    double cell = ned > 0 ? ext / (double)ned : 0.0;
    cell = fmax(cell, avg_edge_len * 0.5);
    cell = fmax(cell, 1e-9);
    if (!isfinite(cell)) empty = true;
    unsigned long long tot = 1;
    // each doubling shrinks the grid; 2100 doublings exceed any double range
    for (int it = 0;; it++) {
        if (it == 2100) empty = true;
        bool ok = true;
        tot = 1;
        for (int j = 0; j < 3; j++) {
            double d = empty ? 1.0 : ceil((hi[j] - lo[j]) / cell) + 1.0;
            if (!(d <= (double)kMaxAxisCells)) {
                ok = false;
                d = 1;
            }
            g.dims[j] = (long long)d;
            tot *= (unsigned long long)g.dims[j];
        }
        if (ok) {
            const unsigned long long keys = (unsigned long long)nscenes * tot;
            ok = dbits_for(keys - 1) + group_bits + 3 <= 64 && keys / (unsigned long long)nscenes == tot;
        }
        if (ok) break;
        cell *= 2;
    }
    for (int j = 0; j < 3; j++) g.lo[j] = empty ? 0.0 : lo[j];
    g.cell = cell;
    g.inv_cell = 1.0 / cell;
    // The margin makes boxes that the round-to-nearest overlap test accepts
    // (disjoint by at most a few ulps) share a cell even after the rounding
    // of the index computation (at most a few ulps of dims, 2^21 at most).
    g.grow = 1e-7 * cell;
    g.ncells = tot;
    const unsigned long long keys = (unsigned long long)nscenes * tot;
    g.dense = keys <= nslots ? 1 : 0;
    g.key_bits = dbits_for(keys - 1);
    *out = g;
}

// The cell filter.  A thread per element: its float box, its cell range
// (first cell packed 21 bits per axis; extents 6 bits per axis, flags in the
// top bits), and for every cell it covers the slot's group: empty -> this
// element's group rank -> kSlotMulti once a second group arrives.  Elements
// spanning more than kLargeCells cells go to the large list instead.
constexpr uint32_t kExtActive = 1u << 31;  // included and binned
constexpr uint32_t kExtLarge = 1u << 30;   // included, tested against all elements

__global__ void k_mark_cells(Elems E, const int* __restrict__ bscene, const int* __restrict__ grank,
                             const Grid* __restrict__ gp, int* __restrict__ sig, uint64_t mask,
                             uint64_t* __restrict__ ec0, uint32_t* __restrict__ eext,
                             float* __restrict__ f32, uint32_t* __restrict__ large_list,
                             int* __restrict__ nlarge)
{
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = (int64_t)E.nv + E.ne + E.nf;
    if (e >= n) return;
    const int t = E.type(e), i = E.id(e, t);
    if (!E.in(t, i)) {
        eext[e] = 0;
        return;
    }
    const Grid g = *gp;
    const double* b = E.box(t, i);
    for (int j = 0; j < 3; j++) {
        f32[6 * e + j] = __double2float_rd(b[j]);
        f32[6 * e + 3 + j] = __double2float_ru(b[3 + j]);
    }
    long long c0[3], c1[3];
    cell_range(b, g, c0, c1);
    const long long k = (c1[0] - c0[0] + 1) * (c1[1] - c0[1] + 1) * (c1[2] - c0[2] + 1);
    if (k > kLargeCells) {
        eext[e] = kExtLarge;
        large_list[atomicAdd(nlarge, 1)] = tag(t, i);
        return;
    }
    ec0[e] = (uint64_t)c0[0] | ((uint64_t)c0[1] << 21) | ((uint64_t)c0[2] << 42);
    eext[e] = kExtActive | (uint32_t)(c1[0] - c0[0]) | ((uint32_t)(c1[1] - c0[1]) << 6)
              | ((uint32_t)(c1[2] - c0[2]) << 12);
    const int body = E.body(t, i);
    const int gr = grank[body];
    const uint64_t base = (uint64_t)bscene[body] * g.ncells;
    for (long long z = c0[2]; z <= c1[2]; z++)
        for (long long y = c0[1]; y <= c1[1]; y++)
            for (long long x = c0[0]; x <= c1[0]; x++) {
                const uint64_t key = base + (uint64_t)((z * g.dims[1] + y) * g.dims[0] + x);
                int* sl = sig + slot_of(key, g, mask);
                const int s = *sl;
                if (s == gr || s == kSlotMulti) continue;
                const int old = atomicCAS(sl, kSlotEmpty, gr);
                if (old != kSlotEmpty && old != gr && old != kSlotMulti) atomicExch(sl, kSlotMulti);
            }
}

__device__ __forceinline__ void unpack_range(uint64_t c0p, uint32_t ext, long long c0[3], long long c1[3])
{
    for (int j = 0; j < 3; j++) {
        c0[j] = (long long)((c0p >> (21 * j)) & ((1ull << 21) - 1));
        c1[j] = c0[j] + (long long)((ext >> (6 * j)) & 63u);
    }
}

// items per element: the marked cells it covers
__global__ void k_count_items(Elems E, const int* __restrict__ bscene, const Grid* __restrict__ gp,
                              const int* __restrict__ sig, uint64_t mask,
                              const uint64_t* __restrict__ ec0, const uint32_t* __restrict__ eext,
                              int32_t* __restrict__ cnt)
{
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = (int64_t)E.nv + E.ne + E.nf;
    if (e >= n) return;
    const uint32_t ext = eext[e];
    if (!(ext & kExtActive)) {
        cnt[e] = 0;
        return;
    }
    const Grid g = *gp;
    const int t = E.type(e), i = E.id(e, t);
    const uint64_t base = (uint64_t)bscene[E.body(t, i)] * g.ncells;
    long long c0[3], c1[3];
    unpack_range(ec0[e], ext, c0, c1);
    int k = 0;
    for (long long z = c0[2]; z <= c1[2]; z++)
        for (long long y = c0[1]; y <= c1[1]; y++)
            for (long long x = c0[0]; x <= c1[0]; x++) {
                const uint64_t key = base + (uint64_t)((z * g.dims[1] + y) * g.dims[0] + x);
                k += sig[slot_of(key, g, mask)] == kSlotMulti;
            }
    cnt[e] = k;
}

// items of the marked cells: key ((scene, cell) << group_bits | group rank)
// << 3 | first-cell bits (bit j: the cell is the first of the element's range
// along axis j); value the element tag
__global__ void k_emit_items(Elems E, const int* __restrict__ bscene, const int* __restrict__ grank,
                             const Grid* __restrict__ gp, const int* __restrict__ sig, uint64_t mask,
                             const uint64_t* __restrict__ ec0, const uint32_t* __restrict__ eext,
                             const int32_t* __restrict__ cnt, const int32_t* __restrict__ off,
                             int group_bits, uint64_t* __restrict__ keys, uint32_t* __restrict__ vals)
{
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = (int64_t)E.nv + E.ne + E.nf;
    if (e >= n || cnt[e] == 0) return;
    const Grid g = *gp;
    const int t = E.type(e), i = E.id(e, t);
    const int body = E.body(t, i);
    const uint64_t gr = (uint64_t)grank[body];
    const uint64_t base = (uint64_t)bscene[body] * g.ncells;
    long long c0[3], c1[3];
    unpack_range(ec0[e], eext[e], c0, c1);
    const uint32_t tg = tag(t, i);
    int64_t o = off[e];
    for (long long z = c0[2]; z <= c1[2]; z++)
        for (long long y = c0[1]; y <= c1[1]; y++)
            for (long long x = c0[0]; x <= c1[0]; x++) {
                const uint64_t key = base + (uint64_t)((z * g.dims[1] + y) * g.dims[0] + x);
                if (sig[slot_of(key, g, mask)] != kSlotMulti) continue;
                const uint64_t first = (uint64_t)(x == c0[0]) | ((uint64_t)(y == c0[1]) << 1)
                                       | ((uint64_t)(z == c0[2]) << 2);
                keys[o] = (((key << group_bits) | gr) << 3) | first;
                vals[o] = tg;
                o++;
            }
}

struct PairOut {
    unsigned long long* ee;  // keys ea * ne + eb
    unsigned long long* fv;  // keys f * nv + v
    unsigned long long cap_ee, cap_fv;
    unsigned long long* n_ee;
    unsigned long long* n_fv;
};

// one slot per pair; the lanes that push together take their slots of a
// stream with one atomic
__device__ __forceinline__ void push_pair(const PairOut& o, bool is_ee, unsigned long long key)
{
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, is_ee ? 1u : 0u);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(is_ee ? o.n_ee : o.n_fv, (unsigned long long)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    const unsigned long long k = base + (unsigned long long)__popc(peers & ((1u << lane) - 1u));
    if (is_ee) {
        if (k < o.cap_ee) o.ee[k] = key;
    } else {
        if (k < o.cap_fv) o.fv[k] = key;
    }
}

// The pair kinds of a call: EE and FV (collision candidates), or EF (edge,
// face: intersection candidates).
constexpr int kPairsEEFV = 0;
constexpr int kPairsEF = 1;

__device__ __forceinline__ bool pair_types(int kind, int ta, int tb)
{
    return kind == kPairsEF ? ta + tb == 3 : ((ta == 1 && tb == 1) || (ta + tb == 2 && ta != tb));
}

// an EE (edges) or FV (face, vertex in either order) pair of elements whose
// groups differ, or an EF pair (edge, face in either order; output in the FV
// stream, key face * ne + edge): the overlap tests and the output key
// (after the float boxes overlap) the double boxes and the output key
__device__ __forceinline__ void exact_pair(const Elems& E, int ta, int ia, int tb, int ib,
                                           const PairOut& o)
{
    if (!boxes_overlap(E.box(ta, ia), E.box(tb, ib))) return;
    if (ta + tb == 3) {
        const int f = ta == 2 ? ia : ib, e = ta == 2 ? ib : ia;
        push_pair(o, false, (unsigned long long)f * (unsigned long long)E.ne + (unsigned long long)e);
    } else if (ta == 1) {
        const int lo = min(ia, ib), hi = max(ia, ib);
        push_pair(o, true, (unsigned long long)lo * (unsigned long long)E.ne + (unsigned long long)hi);
    } else {
        const int f = ta == 2 ? ia : ib, v = ta == 2 ? ib : ia;
        push_pair(o, false, (unsigned long long)f * (unsigned long long)E.nv + (unsigned long long)v);
    }
}

__device__ __forceinline__ void test_pair(const Elems& E, const float* __restrict__ f32, int ta, int ia,
                                          int tb, int ib, const PairOut& o)
{
    if (fboxes_disjoint(f32 + 6 * E.index(ta, ia), f32 + 6 * E.index(tb, ib))) return;
    exact_pair(E, ta, ia, tb, ib, o);
}

// One thread per sorted item: pairs with the items of later groups in its
// cell (the earlier groups' items pair with it), reported in the first cell
// both elements cover.
__global__ void k_cell_pairs(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                             int64_t m, int group_bits, int kind, Elems E,
                             const float* __restrict__ f32, PairOut o)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    // the ends of each item's run (same scene, cell and group) and cell
    // (same scene and cell): the warp's 32 consecutive items mark where runs
    // and cells end, and an item takes the first mark at or after it; a run
    // or cell that goes on past the warp's items is followed in memory
    const int lane = threadIdx.x & 31;
    const bool valid = i < m;
    const int cs = 3 + group_bits;
    const uint64_t ki = valid ? keys[i] : 0;
    const uint64_t kn = valid && i + 1 < m ? keys[i + 1] : 0;
    const bool next = valid && i + 1 < m;
    const bool run_last = !next || (kn >> 3) != (ki >> 3);
    const bool cell_last = !next || (kn >> cs) != (ki >> cs);
    const unsigned above = 0xffffffffu << lane;
    const unsigned run_ends = __ballot_sync(0xffffffffu, run_last) & above;
    const unsigned cell_ends = __ballot_sync(0xffffffffu, cell_last) & above;
    if (!valid) return;
    const uint64_t run = ki >> 3;     // (scene, cell, group)
    const uint64_t cellk = ki >> cs;  // (scene, cell)
    const unsigned fa = (unsigned)(ki & 7);
    int64_t j0, j1;
    if (run_ends) {
        j0 = i - lane + __ffs(run_ends);
    } else {
        j0 = i - lane + 32;
        while (j0 < m && (keys[j0] >> 3) == run) j0++;
    }
    if (cell_ends) {
        j1 = i - lane + __ffs(cell_ends);
    } else {
        j1 = j0 > i - lane + 32 ? j0 : i - lane + 32;
        while (j1 < m && (keys[j1] >> cs) == cellk) j1++;
    }
    if (j0 >= j1) return;
    const uint32_t a = vals[i];
    const int ta = a >> 30, ia = a & 0x3fffffff;
    float fa_box[6];
    {
        const float* p = f32 + 6 * E.index(ta, ia);
#pragma unroll
        for (int k = 0; k < 6; k++) fa_box[k] = p[k];
    }
    // the later groups' items of the cell, four at a time: their keys and
    // values, then the float boxes of those that pair, then the tests
    constexpr int kU = 4;
    for (int64_t j = j0; j < j1; j += kU) {
        uint64_t kk[kU];
        uint32_t bb[kU];
        bool want[kU];
#pragma unroll
        for (int u = 0; u < kU; u++) {
            const bool in = j + u < j1;
            kk[u] = in ? keys[j + u] : 0;
            bb[u] = in ? vals[j + u] : 0;
            want[u] = in && (fa | (unsigned)(kk[u] & 7)) == 7 && pair_types(kind, ta, (int)(bb[u] >> 30));
        }
        float fb[kU][6];
#pragma unroll
        for (int u = 0; u < kU; u++) {
            if (!want[u]) continue;
            const float* p = f32 + 6 * E.index((int)(bb[u] >> 30), (int)(bb[u] & 0x3fffffff));
#pragma unroll
            for (int k = 0; k < 6; k++) fb[u][k] = p[k];
        }
#pragma unroll
        for (int u = 0; u < kU; u++)
            if (want[u] && !fboxes_disjoint(fa_box, fb[u]))
                exact_pair(E, ta, ia, (int)(bb[u] >> 30), (int)(bb[u] & 0x3fffffff), o);
    }
}

// large elements against every included element of the matching type in
// their scene: grid row y = large element, its blocks stride over the
// scene's element range (from the per-body prefix arrays)
__global__ void k_large_pairs(const uint32_t* __restrict__ large, int nl, int row0, int kind, Elems E,
                              const int* __restrict__ bscene, const int* __restrict__ scene_bstart,
                              const int* __restrict__ bvs, const int* __restrict__ bes,
                              const int* __restrict__ bfs, const int* __restrict__ grank,
                              const uint32_t* __restrict__ eext, const float* __restrict__ f32,
                              PairOut o)
{
    const int li = row0 + blockIdx.y;
    if (li >= nl) return;
    const uint32_t a = large[li];
    const int ta = a >> 30, ia = a & 0x3fffffff;
    const int body_a = E.body(ta, ia);
    const int s = bscene[body_a];
    const int ga = grank[body_a];
    // EE / FV: edges meet edges, faces meet vertices (and vertices faces);
    // EF: edges meet faces (and faces edges), vertices nothing
    const int tb = kind == kPairsEF ? 3 - ta : (ta == 1 ? 1 : (ta == 2 ? 0 : 2));
    if (tb > 2) return;
    const int* start = tb == 0 ? bvs : (tb == 1 ? bes : bfs);
    const int lo = start[scene_bstart[s]], hi = start[scene_bstart[s + 1]];
    for (int ib = lo + blockIdx.x * blockDim.x + threadIdx.x; ib < hi; ib += gridDim.x * blockDim.x) {
        const uint32_t ext = eext[E.index(tb, ib)];
        if (!(ext & (kExtActive | kExtLarge))) continue;  // not included
        // a pair of two large elements is reported by the one with the smaller tag
        if ((ext & kExtLarge) && tag(tb, ib) < a) continue;
        if (grank[E.body(tb, ib)] == ga) continue;
        test_pair(E, f32, ta, ia, tb, ib, o);
    }
}

// the two pair streams as one array of sort keys: EE keys as they are, FV
// keys with bit tbit set (above every key of either stream), values 0 .. n-1
__global__ void k_pack_pairs(const unsigned long long* __restrict__ kee, int64_t nee,
                             const unsigned long long* __restrict__ kfv, int64_t nfv, int tbit,
                             unsigned long long* __restrict__ keys, uint32_t* __restrict__ vals)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nee + nfv) return;
    keys[i] = i < nee ? kee[i] : (kfv[i - nee] | (1ull << tbit));
    vals[i] = (uint32_t)i;
}

// sorted keys back to (first, second) pairs: EE first (stride ne), then FV
__global__ void k_decode_pairs(const unsigned long long* __restrict__ keys, int64_t nee, int64_t nfv,
                               int tbit, unsigned long long ee_stride, unsigned long long fv_stride,
                               int2* __restrict__ out_ee, int2* __restrict__ out_fv)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nee + nfv) return;
    const unsigned long long k = keys[i] & ((1ull << tbit) - 1);
    if (i < nee) out_ee[i] = make_int2((int)(k / ee_stride), (int)(k % ee_stride));
    else out_fv[i - nee] = make_int2((int)(k / fv_stride), (int)(k % fv_stride));
}

// Canonical order of the two pair streams by buckets: a pair's bucket is its
// first element (EE: the lower edge, bucket e; FV / EF: the face, bucket
// ne + f), the buckets in order hold the pairs in the order of their keys
// once each bucket is sorted by the second element.  k_bucket_count counts,
// k_bucket_fill places the second elements at the scanned bucket offsets
// (in any order within a bucket), k_bucket_pairs sorts each bucket (a few
// pairs: insertion) and writes the (first, second) pairs, EE then FV.
__device__ __forceinline__ void pair_bucket(unsigned long long key, bool ee, unsigned long long ee_stride,
                                            unsigned long long fv_stride, int ne, int& bucket, int& second)
{
    const unsigned long long stride = ee ? ee_stride : fv_stride;
    const unsigned long long first = key / stride;
    second = (int)(key - first * stride);
    bucket = ee ? (int)first : ne + (int)first;
}

__global__ void k_bucket_count(const unsigned long long* __restrict__ kee, int64_t nee,
                               const unsigned long long* __restrict__ kfv, int64_t nfv,
                               unsigned long long ee_stride, unsigned long long fv_stride, int ne,
                               int32_t* __restrict__ count)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nee + nfv) return;
    const bool ee = i < nee;
    int b, sec;
    pair_bucket(ee ? kee[i] : kfv[i - nee], ee, ee_stride, fv_stride, ne, b, sec);
    atomicAdd(count + b, 1);
}

__global__ void k_bucket_fill(const unsigned long long* __restrict__ kee, int64_t nee,
                              const unsigned long long* __restrict__ kfv, int64_t nfv,
                              unsigned long long ee_stride, unsigned long long fv_stride, int ne,
                              const int32_t* __restrict__ offset, int32_t* __restrict__ fill,
                              int32_t* __restrict__ second)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nee + nfv) return;
    const bool ee = i < nee;
    int b, sec;
    pair_bucket(ee ? kee[i] : kfv[i - nee], ee, ee_stride, fv_stride, ne, b, sec);
    second[offset[b] + atomicAdd(fill + b, 1)] = sec;
}

// buckets of up to kSmallBucket pairs: sorted here; larger ones (a large
// element's bucket: the floor's faces) are listed for k_bucket_large
constexpr int kSmallBucket = 32;

__device__ __forceinline__ void write_pair(int b, int ne, int64_t nee, int64_t pos, int sec,
                                           int2* __restrict__ out_ee, int2* __restrict__ out_fv)
{
    if (b < ne) out_ee[pos] = make_int2(b, sec);
    else out_fv[pos - nee] = make_int2(b - ne, sec);
}

__global__ void k_bucket_pairs(const int32_t* __restrict__ count, const int32_t* __restrict__ offset,
                               int nbuckets, int ne, int64_t nee, int32_t* __restrict__ second,
                               int2* __restrict__ out_ee, int2* __restrict__ out_fv,
                               int32_t* __restrict__ large, int32_t* __restrict__ nlarge)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbuckets) return;
    const int n = count[b];
    if (n == 0) return;
    if (n > kSmallBucket) {
        large[atomicAdd(nlarge, 1)] = b;
        return;
    }
    // sorted in a thread-local copy (L1-resident), then written
    const int64_t o = offset[b];
    int v[kSmallBucket];
    for (int k = 0; k < n; k++) {
        const int x = second[o + k];
        int j = k - 1;
        while (j >= 0 && v[j] > x) {
            v[j + 1] = v[j];
            j--;
        }
        v[j + 1] = x;
    }
    for (int k = 0; k < n; k++) write_pair(b, ne, nee, o + k, v[k], out_ee, out_fv);
}

// One block per listed bucket (grid-stride over the list): its second
// elements (distinct: each pair is found once) as bits of a bitmap over
// their range (EE: edges; FV: vertices; EF: edges), then written in the
// order of the bits.  bitmap: words_per_block words per block.
__global__ void __launch_bounds__(1024) k_bucket_large(
    const int32_t* __restrict__ large, const int32_t* __restrict__ nlarge,
    const int32_t* __restrict__ count, const int32_t* __restrict__ offset,
    const int32_t* __restrict__ second, int ne, int64_t nee, int fv_range,
    unsigned* __restrict__ bitmap_all, int64_t words_per_block,
    int2* __restrict__ out_ee, int2* __restrict__ out_fv)
{
    __shared__ int32_t warp_sum[32];
    __shared__ int32_t carry;
    unsigned* bitmap = bitmap_all + (int64_t)blockIdx.x * words_per_block;
    const int nl = *nlarge;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int li = blockIdx.x; li < nl; li += gridDim.x) {
        const int b = large[li];
        const int n = count[b];
        const int64_t o = offset[b];
        const int range = b < ne ? ne : fv_range;
        const int64_t words = ((int64_t)range + 31) / 32;
        for (int64_t w = threadIdx.x; w < words; w += blockDim.x) bitmap[w] = 0u;
        __syncthreads();
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            const int x = second[o + k];
            atomicOr(bitmap + (x >> 5), 1u << (x & 31));
        }
        if (threadIdx.x == 0) carry = 0;
        __syncthreads();
        // the set bits in order: a block scan of the words' bit counts per
        // chunk of blockDim words
        for (int64_t w0 = 0; w0 < words; w0 += blockDim.x) {
            const int64_t w = w0 + threadIdx.x;
            const unsigned bits = w < words ? bitmap[w] : 0u;
            const int c = __popc(bits);
            int incl = c;
            for (int d = 1; d < 32; d <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d) incl += y;
            }
            if (lane == 31) warp_sum[warp] = incl;
            __syncthreads();
            if (warp == 0) {
                int t = lane < nwarps ? warp_sum[lane] : 0;
                for (int d = 1; d < 32; d <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, t, d);
                    if (lane >= d) t += y;
                }
                if (lane < nwarps) warp_sum[lane] = t;
            }
            __syncthreads();
            int pos = carry + (warp ? warp_sum[warp - 1] : 0) + incl - c;
            for (unsigned r = bits; r; r &= r - 1) {
                const int x = (int)(w * 32) + __ffs(r) - 1;
                write_pair(b, ne, nee, o + pos, x, out_ee, out_fv);
                pos++;
            }
            __syncthreads();
            if (threadIdx.x == 0) carry += warp_sum[nwarps - 1];
            __syncthreads();
        }
    }
}

__global__ void k_iota(uint32_t* __restrict__ v, int64_t n)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = (uint32_t)i;
}

// ---------------------------------------------------------------------------

int body_rot_rn(Ctx& c, const double* x, double* out);
int reserve_rot_table(Ctx& c);

// slots of the cell filter for ntot elements: a power of two, about four per
// element (elements cover a few cells each), 2^16 .. 2^27
static uint64_t filter_slots(int64_t ntot)
{
    uint64_t t = 1u << 16;
    while (t < (uint64_t)ntot * 4 && t < (1ull << 27)) t <<= 1;
    return t;
}

// Candidate pairs of the kind (kPairsEEFV: out.ee, out.fv; kPairsEF: (face,
// edge) pairs in out.fv) between x0 and x1 (continuous) or at x0.
int detect_pairs(Ctx& c, const double* x0, const double* x1, bool continuous, double infl, int kind,
                 Candidates& out)
{
    Scene& s = c.s;
    cudaStream_t st = c.stream;
    out.num_ee = out.num_fv = 0;
    c.bp_table.valid = false;
    c.stats.grid_items = 0;
    c.stats.large_elements = 0;
    if (s.nb <= 1) return RIGC_OK;
    if (!continuous) x1 = x0;
    DevBuf* S = c.scratch;
    const int64_t ntot = (int64_t)s.nv + s.ne + s.nf;
    // small device state of the call: domain (6 doubles), grid, statistics,
    // counters
    constexpr size_t kOffGrid = 64, kOffPart = 256, kOffPartN = kOffPart + 7 * 8 * kStatBlocks,
                     kOffCount = kOffPartN + 4 * kStatBlocks, kMiscBytes = kOffCount + 64;
    RIGC_TRY(c.bp_misc.reserve(kMiscBytes));
    char* misc = c.bp_misc.as<char>();
    double* d_domain = reinterpret_cast<double*>(misc);
    Grid* d_grid = reinterpret_cast<Grid*>(misc + kOffGrid);
    double* d_part = reinterpret_cast<double*>(misc + kOffPart);
    int* d_part_n = reinterpret_cast<int*>(misc + kOffPartN);
    int32_t* d_count = reinterpret_cast<int32_t*>(misc + kOffCount);  // [0] items, [1] large
    // ---- 1. bodies
    RIGC_TRY(c.body_box.reserve((size_t)6 * s.nb * sizeof(double)));
    RIGC_TRY(c.body_in.reserve((size_t)(s.nb + 1) * sizeof(int)));
    RIGC_COUNT_LAUNCH();
    k_body_boxes<<<grid_for((int64_t)s.nb * 32, 128), 128, 0, st>>>(
        x0, x1, s.rest, s.bvs, s.type, s.rmax, s.nb, c.body_box.as<double>());
    RIGC_CUDA(cudaMemsetAsync(c.body_in.ptr, 0, (size_t)s.nb * sizeof(int), st));
    {
        // threads per body: enough to cover the largest scene's pairs
        int maxs = 1;
        for (int k = 0; k < s.nscenes; k++)
            maxs = std::max(maxs, s.h_scene_bstart[k + 1] - s.h_scene_bstart[k]);
        const int chunk = std::min(256, maxs);
        RIGC_COUNT_LAUNCH();
        k_close_bodies<<<grid_for((int64_t)s.nb * chunk, 256), 256, 0, st>>>(
            c.body_box.as<double>(), s.group, s.bscene, s.scene_bstart, c.scene_on, s.nb, chunk,
            infl, c.body_in.as<int>());
    }
    // ---- 2. element boxes
    RIGC_TRY(c.vbox.reserve((size_t)6 * s.nv * sizeof(double) + 8));
    RIGC_TRY(c.ebox.reserve((size_t)6 * s.ne * sizeof(double) + 8));
    RIGC_TRY(c.fbox.reserve((size_t)6 * s.nf * sizeof(double) + 8));
    RIGC_TRY(c.vin.reserve((size_t)s.nv + 8));
    RIGC_TRY(c.ein.reserve((size_t)s.ne + 8));
    RIGC_TRY(c.fin.reserve((size_t)s.nf + 8));
    if (continuous) {
        RIGC_TRY(reserve_rot_table(c));
        RIGC_TRY(c.bp_deeper.reserve((size_t)s.nb * sizeof(int)));
        double* table = c.rot_table.as<double>();
        RIGC_COUNT_LAUNCH();
        k_scene_box<<<1, 256, 0, st>>>(c.body_box.as<double>(), c.body_in.as<int>(), s.nb, d_domain);
        RIGC_COUNT_LAUNCH();
        k_bp_frames<<<grid_for((int64_t)s.nb * kRotTableSlots, 128), 128, 0, st>>>(
            x0, x1, c.body_in.as<int>(), s.nb, kDefaultToiTol, table);
        RIGC_CUDA(cudaMemsetAsync(c.bp_deeper.ptr, 0, (size_t)s.nb * sizeof(int), st));
        RIGC_COUNT_LAUNCH();
        k_vertex_boxes_half<<<grid_for(s.nv, 128), 128, 0, st>>>(
            s.rest, s.vbody, c.body_in.as<int>(), s.nv, table, d_domain, infl,
            c.vbox.as<double>(), c.vin.as<char>(), c.bp_deeper.as<int>());
        RIGC_COUNT_LAUNCH();
        k_vertex_boxes_cont<<<(unsigned)s.nb, kVBThreads, 0, st>>>(
            x0, x1, s.rest, s.bvs, c.body_in.as<int>(), c.bp_deeper.as<int>(), table, d_domain,
            infl, c.vbox.as<double>(), c.vin.as<char>());
    } else {
        RIGC_TRY(S[0].reserve((size_t)12 * s.nb * sizeof(double)));
        RIGC_TRY(body_rot_rn(c, x0, S[0].as<double>()));
        RIGC_COUNT_LAUNCH();
        k_vertex_boxes_disc<<<grid_for(s.nv, 256), 256, 0, st>>>(
            S[0].as<double>(), s.rest, s.vbody, c.body_in.as<int>(), s.nv, infl, c.vbox.as<double>(),
            c.vin.as<char>());
    }
    RIGC_COUNT_LAUNCH();
    k_edge_face_boxes<<<grid_for((int64_t)s.ne + s.nf, 256), 256, 0, st>>>(
        s.edges, s.ne, s.faces, s.nf, c.vbox.as<double>(), c.vin.as<char>(), c.ebox.as<double>(),
        c.ein.as<char>(), c.fbox.as<double>(), c.fin.as<char>());
    RIGC_CUDA(cudaGetLastError());
    const Elems E { c.vbox.as<double>(), c.ebox.as<double>(), c.fbox.as<double>(),
                    c.vin.as<char>(), c.ein.as<char>(), c.fin.as<char>(),
                    s.vbody, s.ebody, s.fbody, s.nv, s.ne, s.nf };
    // ---- 3. grid and cell filter
    RIGC_COUNT_LAUNCH();
    k_elem_stats<<<kStatBlocks, kStatThreads, 0, st>>>(E, d_part, d_part_n);
    const uint64_t nslots = filter_slots(ntot);
    RIGC_COUNT_LAUNCH();
    k_grid_setup<<<1, 32, 0, st>>>(d_part, d_part_n, kStatBlocks, s.avg_edge_len, s.nscenes,
                                   s.group_bits, nslots, d_grid);
    RIGC_TRY(c.bp_sig.reserve(nslots * sizeof(int)));
    RIGC_TRY(c.bp_ec0.reserve((size_t)ntot * sizeof(uint64_t) + 8));
    RIGC_TRY(c.bp_eext.reserve((size_t)ntot * sizeof(uint32_t) + 8));
    RIGC_TRY(c.bp_f32.reserve((size_t)ntot * 6 * sizeof(float) + 8));
    RIGC_TRY(c.bp_cnt.reserve((size_t)(2 * ntot + 2) * sizeof(int32_t)));
    RIGC_TRY(c.large_list.reserve((size_t)(ntot + 1) * sizeof(uint32_t)));
    RIGC_CUDA(cudaMemsetAsync(c.bp_sig.ptr, 0xff, nslots * sizeof(int), st));
    RIGC_CUDA(cudaMemsetAsync(d_count, 0, 2 * sizeof(int32_t), st));
    int32_t* icnt = c.bp_cnt.as<int32_t>();
    int32_t* ioff = icnt + ntot + 1;
    RIGC_COUNT_LAUNCH();
    k_mark_cells<<<grid_for(ntot, 256), 256, 0, st>>>(
        E, s.bscene, s.grank, d_grid, c.bp_sig.as<int>(), nslots - 1, c.bp_ec0.as<uint64_t>(),
        c.bp_eext.as<uint32_t>(), c.bp_f32.as<float>(), c.large_list.as<uint32_t>(), d_count + 1);
    RIGC_COUNT_LAUNCH();
    k_count_items<<<grid_for(ntot, 256), 256, 0, st>>>(
        E, s.bscene, d_grid, c.bp_sig.as<int>(), nslots - 1, c.bp_ec0.as<uint64_t>(),
        c.bp_eext.as<uint32_t>(), icnt);
    RIGC_TRY(exclusive_scan_i32(icnt, ioff, ntot, d_count, S[7], st));
    // the host sizes the item buffers and the sort: one read-back
    Grid hg;
    int32_t counts[2];
    RIGC_CUDA(cudaMemcpyAsync(counts, d_count, sizeof(counts), cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaMemcpyAsync(&hg, d_grid, sizeof(Grid), cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaStreamSynchronize(st));
    const int64_t nitems = counts[0];
    const int nlarge = counts[1];
    c.stats.grid_items = nitems;
    c.stats.large_elements = nlarge;
    // ---- 4. items of the marked cells, sorted
    RIGC_TRY(c.items_key.reserve((size_t)nitems * 8 + 8));
    RIGC_TRY(c.items_val.reserve((size_t)nitems * 4 + 8));
    RIGC_TRY(c.items_key2.reserve((size_t)nitems * 8 + 8));
    RIGC_TRY(c.items_val2.reserve((size_t)nitems * 4 + 8));
    if (nitems > 0) {
        RIGC_COUNT_LAUNCH();
        k_emit_items<<<grid_for(ntot, 256), 256, 0, st>>>(
            E, s.bscene, s.grank, d_grid, c.bp_sig.as<int>(), nslots - 1, c.bp_ec0.as<uint64_t>(),
            c.bp_eext.as<uint32_t>(), icnt, ioff, s.group_bits, c.items_key.as<uint64_t>(),
            c.items_val.as<uint32_t>());
        RIGC_TRY(radix_sort_pairs<uint64_t>(c.items_key.as<uint64_t>(), c.items_val.as<uint32_t>(),
                                            c.items_key2.as<uint64_t>(), c.items_val2.as<uint32_t>(),
                                            nitems, hg.key_bits + s.group_bits + 3, S[4], S[5], S[7],
                                            st));
    }
    // ---- 5. pairs (retry once with exact capacity on overflow)
    unsigned long long* pn = reinterpret_cast<unsigned long long*>(c.d_scalars.as<char>() + 1024);
    unsigned long long cap_ee = std::max<unsigned long long>(1 << 16, (unsigned long long)nitems);
    unsigned long long cap_fv = cap_ee;
    cap_ee = std::max<unsigned long long>(cap_ee, (unsigned long long)c.bp_pair_hint[0]);
    cap_fv = std::max<unsigned long long>(cap_fv, (unsigned long long)c.bp_pair_hint[1]);
    const float* f32 = c.bp_f32.as<float>();
    for (int attempt = 0; attempt < 3; attempt++) {
        RIGC_TRY(c.pair_out.reserve((size_t)(cap_ee + cap_fv) * 8));
        PairOut o { c.pair_out.as<unsigned long long>(), c.pair_out.as<unsigned long long>() + cap_ee,
                    cap_ee, cap_fv, pn, pn + 1 };
        RIGC_CUDA(cudaMemsetAsync(pn, 0, 2 * sizeof(unsigned long long), st));
        if (nitems > 0) {
            RIGC_COUNT_LAUNCH();
            k_cell_pairs<<<grid_for(nitems, 128), 128, 0, st>>>(
                c.items_key2.as<uint64_t>(), c.items_val2.as<uint32_t>(), nitems, s.group_bits, kind,
                E, f32, o);
        }
        if (nlarge > 0) {
            // enough blocks per large element to cover a whole scene's elements
            const unsigned bx = (unsigned)std::min<int64_t>(
                1024, std::max<int64_t>(1, (ntot / s.nscenes + 255) / 256));
            for (int row0 = 0; row0 < nlarge; row0 += 65535) {
                const unsigned rows = (unsigned)std::min(65535, nlarge - row0);
                RIGC_COUNT_LAUNCH();
                k_large_pairs<<<dim3(bx, rows), 256, 0, st>>>(
                    c.large_list.as<uint32_t>(), nlarge, row0, kind, E, s.bscene, s.scene_bstart, s.bvs,
                    s.bes, s.bfs, s.grank, c.bp_eext.as<uint32_t>(), f32, o);
            }
        }
        RIGC_CUDA(cudaGetLastError());
        unsigned long long hn[2];
        RIGC_CUDA(cudaMemcpyAsync(hn, pn, sizeof(hn), cudaMemcpyDeviceToHost, st));
        RIGC_CUDA(cudaStreamSynchronize(st));
        if (hn[0] <= cap_ee && hn[1] <= cap_fv) {
            out.num_ee = (int64_t)hn[0];
            out.num_fv = (int64_t)hn[1];
            break;
        }
        cap_ee = std::max(cap_ee, hn[0]);
        cap_fv = std::max(cap_fv, hn[1]);
        c.bp_pair_hint[0] = std::max<int64_t>(c.bp_pair_hint[0], (int64_t)hn[0]);
        c.bp_pair_hint[1] = std::max<int64_t>(c.bp_pair_hint[1], (int64_t)hn[1]);
        if (attempt == 2) return RIGC_ERR_OOM;
    }
    // ---- 6. canonical order
    const int64_t nee = out.num_ee, nfv = out.num_fv;
    unsigned long long* kee = c.pair_out.as<unsigned long long>();
    unsigned long long* kfv = kee + cap_ee;
    RIGC_TRY(out.ee.reserve((size_t)nee * sizeof(int2) + 8));
    RIGC_TRY(out.fv.reserve((size_t)nfv * sizeof(int2) + 8));
    // the second stream: (face, vertex) keys f * nv + v, or (face, edge)
    // keys f * ne + e
    const unsigned long long fv_stride = kind == kPairsEF ? (unsigned long long)s.ne
                                                          : (unsigned long long)s.nv;
    // one sort of both streams (FV keys above EE keys by a type bit)
    const int tbit = std::max(bits_for((uint64_t)s.ne * (uint64_t)s.ne),
                              bits_for((uint64_t)s.nf * fv_stride));
    const int64_t np = nee + nfv;
    const int64_t nbuckets = (int64_t)s.ne + s.nf;
    if (np > 0 && np < (int64_t)INT32_MAX && nbuckets < (int64_t)INT32_MAX) {
        // by buckets of the first element
        RIGC_TRY(S[0].reserve((size_t)2 * nbuckets * sizeof(int32_t)));
        RIGC_TRY(S[1].reserve((size_t)(nbuckets + np) * sizeof(int32_t)));
        int32_t* count = S[0].as<int32_t>();
        int32_t* fill = count + nbuckets;
        int32_t* offset = S[1].as<int32_t>();
        int32_t* second = offset + nbuckets;
        RIGC_CUDA(cudaMemsetAsync(count, 0, (size_t)2 * nbuckets * sizeof(int32_t), st));
        RIGC_COUNT_LAUNCH();
        k_bucket_count<<<grid_for(np, 256), 256, 0, st>>>(kee, nee, kfv, nfv, (unsigned long long)s.ne,
                                                           fv_stride, s.ne, count);
        RIGC_TRY(exclusive_scan_i32(count, offset, nbuckets, d_count + 2, S[7], st));
        RIGC_COUNT_LAUNCH();
        k_bucket_fill<<<grid_for(np, 256), 256, 0, st>>>(kee, nee, kfv, nfv, (unsigned long long)s.ne,
                                                          fv_stride, s.ne, offset, fill, second);
        RIGC_TRY(S[2].reserve((size_t)nbuckets * sizeof(int32_t)));
        int32_t* nlarge = d_count + 3;
        RIGC_CUDA(cudaMemsetAsync(nlarge, 0, sizeof(int32_t), st));
        RIGC_COUNT_LAUNCH();
        k_bucket_pairs<<<grid_for(nbuckets, 256), 256, 0, st>>>(count, offset, (int)nbuckets, s.ne, nee,
                                                                 second, out.ee.as<int2>(),
                                                                 out.fv.as<int2>(), S[2].as<int32_t>(),
                                                                 nlarge);
        // the large buckets, a block each (at most kLargeBlocks at a time)
        constexpr int kLargeBlocks = 32;
        const int fv_range = kind == kPairsEF ? s.ne : s.nv;
        const int64_t words = ((int64_t)std::max(s.ne, fv_range) + 31) / 32;
        RIGC_TRY(S[3].reserve((size_t)kLargeBlocks * words * sizeof(unsigned)));
        RIGC_COUNT_LAUNCH();
        k_bucket_large<<<kLargeBlocks, 1024, 0, st>>>(S[2].as<int32_t>(), nlarge, count, offset, second, s.ne,
                                                     nee, fv_range, S[3].as<unsigned>(), words,
                                                     out.ee.as<int2>(), out.fv.as<int2>());
    } else if (np > 0) {
        RIGC_TRY(c.pair_key.reserve((size_t)np * 8 + 8));
        RIGC_TRY(S[0].reserve((size_t)np * 4 + 8));
        RIGC_TRY(S[1].reserve((size_t)np * 4 + 8));
        RIGC_COUNT_LAUNCH();
        k_pack_pairs<<<grid_for(np, 256), 256, 0, st>>>(kee, nee, kfv, nfv, tbit, c.pair_key.as<unsigned long long>(),
                                                        S[0].as<uint32_t>());
        // the packed keys sort into the pair buffer (its streams are consumed)
        RIGC_TRY(radix_sort_pairs<uint64_t>(c.pair_key.as<uint64_t>(), S[0].as<uint32_t>(),
                                            reinterpret_cast<uint64_t*>(kee), S[1].as<uint32_t>(), np,
                                            tbit + 1, S[4], S[5], S[7], st));
        RIGC_COUNT_LAUNCH();
        k_decode_pairs<<<grid_for(np, 256), 256, 0, st>>>(kee, nee, nfv, tbit, (unsigned long long)s.ne,
                                                          fv_stride, out.ee.as<int2>(), out.fv.as<int2>());
    }
    RIGC_CUDA(cudaGetLastError());
    if (continuous && kind == kPairsEEFV) {
        c.bp_table.x0 = x0;
        c.bp_table.x1 = x1;
        c.bp_table.toi_tol = kDefaultToiTol;
        c.bp_table.valid = true;
    }
    return RIGC_OK;
}

int detect_candidates(Ctx& c, const double* x0, const double* x1, bool continuous, double infl)
{
    return detect_pairs(c, x0, x1, continuous, infl, kPairsEEFV, c.cand);
}

} // namespace rigc
