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
//     src/ccd/rigid/rigid_body_hash_grid.cpp:164-246), one CUDA block per
//     body; discrete -- the world vertex +- inflation.  Edge and face boxes are
//     unions of their vertex boxes (:265-344);
//  3. pairs: ipc-toolkit's HashGrid reports element pairs that share a cell,
//     belong to different groups and whose boxes overlap (center /
//     half-extent test).  Here elements are binned into cells (radix sort of
//     (cell, element) items), each pair is reported once, in the first cell
//     both elements cover, and elements spanning more than kLargeCells cells
//     are tested against all elements instead of being binned.  The output is
//     the same set, sorted: ee as (edge0 < edge1), fv as (face, vertex).
#include "common.cuh"
#include "interval.cuh"
#include "sort.cuh"

namespace rigc {

constexpr int kLargeCells = 64;
// item counts up to which cell pairs are enumerated by a warp per item
constexpr int64_t kWarpPairItems = 1 << 16;

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
    if (threadIdx.x == 0) {
        for (int t = 1; t < blockDim.x; t++)
            for (int j = 0; j < 3; j++) {
                lo[j] = smin(lo[j], sh[j][t]);
                hi[j] = smax(hi[j], sh[3 + j][t]);
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
constexpr int kMaxTNodes = 40;

// one block per included body; vbox holds lo[3], hi[3] per vertex
__global__ void __launch_bounds__(kVBThreads)
k_vertex_boxes_cont(const double* __restrict__ x0, const double* __restrict__ x1,
                    const double* __restrict__ rest, const int* __restrict__ bvs,
                    const int* __restrict__ body_list, const double* __restrict__ domain,
                    double infl, double* __restrict__ vbox, char* __restrict__ vin)
{
    __shared__ double st_lo[kMaxTNodes], st_hi[kMaxTNodes];
    __shared__ int st_depth[kMaxTNodes];
    __shared__ int sp;
    __shared__ Itv sR[9], sp3[3];
    const int b = body_list[blockIdx.x];
    const int v0 = bvs[b], v1 = bvs[b + 1];
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
    __syncthreads();
    while (true) {
        __syncthreads();
        if (sp == 0) break;
        double tl = st_lo[sp - 1], th = st_hi[sp - 1];
        int depth = st_depth[sp - 1];
        __syncthreads();
        if (threadIdx.x == 0) {
            sp--;
            Itv t { tl, th };
            Itv r[3];
            for (int k = 0; k < 3; k++) {
                double a = x0[6 * b + k], c = x1[6 * b + k];
                sp3[k] = iadd(imul(Itv { sub_dn(c, a), sub_up(c, a) }, t), pt(a));
                double ar = x0[6 * b + 3 + k], cr = x1[6 * b + 3 + k];
                r[k] = iadd(imul(Itv { sub_dn(cr, ar), sub_up(cr, ar) }, t), pt(ar));
            }
            Itv R[9];
            irotation(r, R);
            for (int k = 0; k < 9; k++) sR[k] = R[k];
        }
        __syncthreads();
        Itv R[9], p[3];
        for (int k = 0; k < 9; k++) R[k] = sR[k];
        for (int k = 0; k < 3; k++) p[k] = sp3[k];
        bool fits = true;
        for (int v = v0 + threadIdx.x; v < v1; v += blockDim.x) {
            double rv[3] = { rest[3 * (size_t)v], rest[3 * (size_t)v + 1], rest[3 * (size_t)v + 2] };
            Itv w[3];
            iworld_vertex(R, p, rv, w);
            for (int j = 0; j < 3; j++)
                if (RSUB(w[j].lo, infl) < dlo[j] || RADD(w[j].hi, infl) > dhi[j]) fits = false;
        }
        bool all_fit = __syncthreads_and(fits) != 0;
        if (all_fit || depth >= 16) {
            for (int v = v0 + threadIdx.x; v < v1; v += blockDim.x) {
                double rv[3] = { rest[3 * (size_t)v], rest[3 * (size_t)v + 1], rest[3 * (size_t)v + 2] };
                Itv w[3];
                iworld_vertex(R, p, rv, w);
                for (int j = 0; j < 3; j++) {
                    vbox[6 * (size_t)v + j] = smin(vbox[6 * (size_t)v + j], w[j].lo);
                    vbox[6 * (size_t)v + 3 + j] = smax(vbox[6 * (size_t)v + 3 + j], w[j].hi);
                }
            }
        } else if (threadIdx.x == 0) {
            double m = RMUL(0.5, RADD(tl, th));
            if (sp + 2 <= kMaxTNodes) {
                st_lo[sp] = m; st_hi[sp] = th; st_depth[sp] = depth + 1; sp++;
                st_lo[sp] = tl; st_hi[sp] = m; st_depth[sp] = depth + 1; sp++;
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

__global__ void k_clear_flags(char* __restrict__ f, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) f[i] = 0;
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

struct Grid {
    double lo[3];
    double cell, grow;
    long long dims[3];
};

// element tags: type in the top 2 bits (0 vertex, 1 edge, 2 face)
__device__ __forceinline__ uint32_t tag(int type, int id) { return ((uint32_t)type << 30) | (uint32_t)id; }

__device__ __forceinline__ const double* elem_box(uint32_t t, const double* vb, const double* eb,
                                                  const double* fb)
{
    int type = t >> 30, id = t & 0x3fffffff;
    return (type == 0 ? vb : (type == 1 ? eb : fb)) + 6 * (size_t)id;
}

__device__ __forceinline__ long long cell_of(double x, const Grid& g, int j)
{
    long long c = (long long)floor(RDIV(RSUB(x, g.lo[j]), g.cell));
    return c < 0 ? 0 : (c >= g.dims[j] ? g.dims[j] - 1 : c);
}

__device__ __forceinline__ void cell_range(const double* b, const Grid& g, long long c0[3], long long c1[3])
{
    for (int j = 0; j < 3; j++) {
        c0[j] = cell_of(RSUB(b[j], g.grow), g, j);
        c1[j] = cell_of(RADD(b[3 + j], g.grow), g, j);
    }
}

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

// element list: all included vertices, edges, faces (tags)
__global__ void k_elem_flags(const char* __restrict__ vin, const char* __restrict__ ein,
                             const char* __restrict__ fin, int nv, int ne, int nf,
                             int32_t* __restrict__ flag)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int n = nv + ne + nf;
    if (i >= n) return;
    flag[i] = i < nv ? vin[i] : (i < nv + ne ? ein[i - nv] : fin[i - nv - ne]);
}

__global__ void k_elem_list(const int32_t* __restrict__ flag, const int32_t* __restrict__ pos, int nv,
                            int ne, int nf, uint32_t* __restrict__ elems)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int n = nv + ne + nf;
    if (i >= n || !flag[i]) return;
    uint32_t t = i < nv ? tag(0, i) : (i < nv + ne ? tag(1, i - nv) : tag(2, i - nv - ne));
    elems[pos[i]] = t;
}

// extent statistics: bounds of all element boxes, sum of edge box extents
__global__ void k_elem_bounds(const uint32_t* __restrict__ elems, int m, const double* __restrict__ vb,
                              const double* __restrict__ eb, const double* __restrict__ fb,
                              double* __restrict__ part, double* __restrict__ ext)
{
    // part: per block lo[3], hi[3]; ext: per element extent (edges only, else 0)
    __shared__ double sh[6][256];
    double lo[3] = { INFINITY, INFINITY, INFINITY }, hi[3] = { -INFINITY, -INFINITY, -INFINITY };
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const double* b = elem_box(elems[i], vb, eb, fb);
        double e = 0;
        for (int j = 0; j < 3; j++) {
            lo[j] = smin(lo[j], b[j]);
            hi[j] = smax(hi[j], b[3 + j]);
            e = smax(e, RSUB(b[3 + j], b[j]));
        }
        ext[i] = (elems[i] >> 30) == 1 ? e : 0.0;
    }
    for (int j = 0; j < 3; j++) {
        sh[j][threadIdx.x] = lo[j];
        sh[3 + j][threadIdx.x] = hi[j];
    }
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int j = 0; j < 3; j++) {
                sh[j][threadIdx.x] = smin(sh[j][threadIdx.x], sh[j][threadIdx.x + o]);
                sh[3 + j][threadIdx.x] = smax(sh[3 + j][threadIdx.x], sh[3 + j][threadIdx.x + o]);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int j = 0; j < 6; j++) part[6 * blockIdx.x + j] = sh[j][0];
}

__global__ void k_count_cells(const uint32_t* __restrict__ elems, int m, const double* __restrict__ vb,
                              const double* __restrict__ eb, const double* __restrict__ fb, Grid g,
                              int32_t* __restrict__ cnt, int32_t* __restrict__ large_flag)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    long long c0[3], c1[3];
    cell_range(elem_box(elems[i], vb, eb, fb), g, c0, c1);
    long long k = (c1[0] - c0[0] + 1) * (c1[1] - c0[1] + 1) * (c1[2] - c0[2] + 1);
    bool large = k > kLargeCells;
    cnt[i] = large ? 0 : (int32_t)k;
    large_flag[i] = large ? 1 : 0;
}

// scene of an element (tag: type << 30 | index)
struct ElemScene {
    const int* vbody;
    const int* ebody;
    const int* fbody;
    const int* bscene;
    __device__ __forceinline__ uint64_t of(uint32_t tag) const
    {
        const int t = tag >> 30, i = tag & 0x3fffffff;
        const int b = t == 0 ? vbody[i] : (t == 1 ? ebody[i] : fbody[i]);
        return (uint64_t)bscene[b];
    }
};

// (scene, cell) keys: elements of different scenes never share a key
__global__ void k_emit_items(const uint32_t* __restrict__ elems, int m, const double* __restrict__ vb,
                             const double* __restrict__ eb, const double* __restrict__ fb, Grid g,
                             ElemScene es, uint64_t ncells, const int32_t* __restrict__ cnt,
                             const int32_t* __restrict__ off, uint64_t* __restrict__ keys,
                             uint32_t* __restrict__ vals)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m || cnt[i] == 0) return;
    long long c0[3], c1[3];
    cell_range(elem_box(elems[i], vb, eb, fb), g, c0, c1);
    const uint64_t base = es.of(elems[i]) * ncells;
    int o = off[i];
    for (long long z = c0[2]; z <= c1[2]; z++)
        for (long long y = c0[1]; y <= c1[1]; y++)
            for (long long x = c0[0]; x <= c1[0]; x++) {
                keys[o] = base + (uint64_t)((z * g.dims[1] + y) * g.dims[0] + x);
                vals[o] = elems[i];
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

__device__ __forceinline__ void push_pair(const PairOut& o, bool is_ee, unsigned long long key)
{
    if (is_ee) {
        unsigned long long k = atomicAdd(o.n_ee, 1ull);
        if (k < o.cap_ee) o.ee[k] = key;
    } else {
        unsigned long long k = atomicAdd(o.n_fv, 1ull);
        if (k < o.cap_fv) o.fv[k] = key;
    }
}

struct PairCtx {
    const double* vb;
    const double* eb;
    const double* fb;
    const int* vbody;
    const int* ebody;
    const int* fbody;
    const int* group;
    int nv, ne;
};

// test one element pair (any order); returns true and the output if it is an
// EE or FV candidate passing the group and overlap filters
__device__ __forceinline__ bool pair_filter(const PairCtx& P, uint32_t a, uint32_t b, bool& is_ee,
                                            unsigned long long& key)
{
    int ta = a >> 30, tb = b >> 30;
    int ia = a & 0x3fffffff, ib = b & 0x3fffffff;
    int ga, gb;
    if (ta == 1 && tb == 1) {
        if (ia == ib) return false;
        ga = P.group[P.ebody[ia]];
        gb = P.group[P.ebody[ib]];
        if (ga == gb) return false;
        if (!boxes_overlap(P.eb + 6 * (size_t)ia, P.eb + 6 * (size_t)ib)) return false;
        is_ee = true;
        int lo = min(ia, ib), hi = max(ia, ib);
        key = (unsigned long long)lo * (unsigned long long)P.ne + (unsigned long long)hi;
        return true;
    }
    if ((ta == 2 && tb == 0) || (ta == 0 && tb == 2)) {
        int f = ta == 2 ? ia : ib, v = ta == 2 ? ib : ia;
        if (P.group[P.fbody[f]] == P.group[P.vbody[v]]) return false;
        if (!boxes_overlap(P.fb + 6 * (size_t)f, P.vb + 6 * (size_t)v)) return false;
        is_ee = false;
        key = (unsigned long long)f * (unsigned long long)P.nv + (unsigned long long)v;
        return true;
    }
    return false;
}

// one thread per sorted item: pairs with later items of the same cell,
// reported only in the first cell both elements cover
__global__ void k_cell_pairs(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                             int64_t m, PairCtx P, Grid g, ElemScene es, uint64_t ncells, PairOut o)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    uint64_t key = keys[i];
    uint32_t a = vals[i];
    long long a0[3], a1[3];
    bool have_a = false;
    // Within a cell the items keep the element order of the emission (the
    // radix sort is stable, elements are ordered vertices, edges, faces):
    // a face's later items are faces (no pair), an edge's are edges, then
    // faces (no more pairs), a vertex's reach the faces after the edges.
    if ((a >> 30) == 2) return;
    for (int64_t j = i + 1; j < m && keys[j] == key; j++) {
        uint32_t b = vals[j];
        bool is_ee;
        unsigned long long pk;
        int ta = a >> 30, tb = b >> 30;
        if (ta == 1 && tb == 2) break;
        if (!((ta == 1 && tb == 1) || (ta + tb == 2 && ta != tb))) continue;
        if (!pair_filter(P, a, b, is_ee, pk)) continue;
        if (!have_a) {
            cell_range(elem_box(a, P.vb, P.eb, P.fb), g, a0, a1);
            have_a = true;
        }
        long long b0[3], b1[3];
        cell_range(elem_box(b, P.vb, P.eb, P.fb), g, b0, b1);
        long long fx = max(a0[0], b0[0]), fy = max(a0[1], b0[1]), fz = max(a0[2], b0[2]);
        uint64_t first = es.of(a) * ncells + (uint64_t)((fz * g.dims[1] + fy) * g.dims[0] + fx);
        if (first != key) continue;
        push_pair(o, is_ee, pk);
    }
}

// The same with one warp per sorted item, its lanes striding over the later
// items of the cell: for small item counts, where the cells are few and
// full and one thread per item would walk a whole cell alone.
__global__ void k_cell_pairs_warp(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                                  int64_t m, PairCtx P, Grid g, ElemScene es, uint64_t ncells,
                                  PairOut o)
{
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= m) return;
    const uint64_t key = keys[i];
    const uint32_t a = vals[i];
    long long a0[3], a1[3];
    bool have_a = false;
    if ((a >> 30) == 2) return;  // faces: only faces follow in the cell
    for (int64_t j = i + 1 + lane; j < m && keys[j] == key; j += 32) {
        uint32_t b = vals[j];
        bool is_ee;
        unsigned long long pk;
        int ta = a >> 30, tb = b >> 30;
        if (ta == 1 && tb == 2) break;  // an edge's later items: edges, then faces
        if (!((ta == 1 && tb == 1) || (ta + tb == 2 && ta != tb))) continue;
        if (!pair_filter(P, a, b, is_ee, pk)) continue;
        if (!have_a) {
            cell_range(elem_box(a, P.vb, P.eb, P.fb), g, a0, a1);
            have_a = true;
        }
        long long b0[3], b1[3];
        cell_range(elem_box(b, P.vb, P.eb, P.fb), g, b0, b1);
        long long fx = max(a0[0], b0[0]), fy = max(a0[1], b0[1]), fz = max(a0[2], b0[2]);
        uint64_t first = es.of(a) * ncells + (uint64_t)((fz * g.dims[1] + fy) * g.dims[0] + fx);
        if (first != key) continue;
        push_pair(o, is_ee, pk);
    }
}

// large elements against every included element of the matching type in
// their scene: grid row y = large element, its blocks stride over the range;
// range[s * 3 + t] is the first
// position in elems of scene s's type-t elements (vertices, edges, faces;
// elems is ordered by type, then by element index, hence by scene)
__global__ void k_large_pairs(const uint32_t* __restrict__ large, int nl, int row0,
                              const uint32_t* __restrict__ elems, const int32_t* __restrict__ is_large,
                              const int32_t* __restrict__ range, int nscenes, ElemScene es, PairCtx P,
                              PairOut o)
{
    const int li = row0 + blockIdx.y;
    if (li >= nl) return;
    const uint32_t a = large[li];
    const int ta = a >> 30;
    const int s = (int)es.of(a);
    // edges meet edges, faces meet vertices (and vertices faces)
    const int tb = ta == 1 ? 1 : (ta == 2 ? 0 : 2);
    const int lo = range[3 * s + tb];
    const int hi = range[3 * (s + 1) + tb];
    for (int ei = lo + blockIdx.x * blockDim.x + threadIdx.x; ei < hi; ei += gridDim.x * blockDim.x) {
        const uint32_t b = elems[ei];
        // a pair of two large elements is reported by the one with the smaller tag
        if (is_large[ei] && b < a) continue;
        bool is_ee;
        unsigned long long pk;
        if (pair_filter(P, a, b, is_ee, pk)) push_pair(o, is_ee, pk);
    }
}

// positions in elems of each scene's first vertex, edge and face (from the
// exclusive scan of the inclusion flags over all elements); row nscenes
// holds the end of each type
__global__ void k_scene_ranges(const int32_t* __restrict__ pos, const int* __restrict__ scene_bstart,
                               const int* __restrict__ bvs, const int* __restrict__ bes,
                               const int* __restrict__ bfs, int nscenes, int nv, int ne, int nf,
                               int m, int32_t* __restrict__ range)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s > nscenes) return;
    const int ntot = nv + ne + nf;
    auto at = [&](int idx) { return idx < ntot ? pos[idx] : m; };
    if (s == nscenes) {
        range[3 * s] = at(nv);
        range[3 * s + 1] = at(nv + ne);
        range[3 * s + 2] = m;
        return;
    }
    const int b = scene_bstart[s];
    range[3 * s] = at(bvs[b]);
    range[3 * s + 1] = at(nv + bes[b]);
    range[3 * s + 2] = at(nv + ne + bfs[b]);
}

__global__ void k_large_list(const uint32_t* __restrict__ elems, const int32_t* __restrict__ flag,
                             const int32_t* __restrict__ pos, int m, uint32_t* __restrict__ out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m && flag[i]) out[pos[i]] = elems[i];
}

__global__ void k_decode_pairs(const unsigned long long* __restrict__ keys, int64_t n,
                               unsigned long long stride, int2* __restrict__ out)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned long long k = keys[i];
    out[i] = make_int2((int)(k / stride), (int)(k % stride));
}

__global__ void k_iota(uint32_t* __restrict__ v, int64_t n)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = (uint32_t)i;
}

// ---------------------------------------------------------------------------

int compute_world_vertices_rn(Ctx& c, const double* x, double* V, DevBuf& rotbuf);
int body_rot_rn(Ctx& c, const double* x, double* out);

int detect_candidates(Ctx& c, const double* x0, const double* x1, bool continuous, double infl)
{
    Scene& s = c.s;
    cudaStream_t st = c.stream;
    c.cand.num_ee = c.cand.num_fv = 0;
    c.stats.grid_items = 0;
    c.stats.large_elements = 0;
    if (s.nb <= 1) return RIGC_OK;
    if (!continuous) x1 = x0;
    DevBuf* S = c.scratch;
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
    std::vector<int> h_in(s.nb);
    RIGC_CUDA(cudaMemcpyAsync(h_in.data(), c.body_in.ptr, (size_t)s.nb * sizeof(int),
                              cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaStreamSynchronize(st));
    std::vector<int> blist;
    for (int b = 0; b < s.nb; b++)
        if (h_in[b]) blist.push_back(b);
    if (blist.empty()) return RIGC_OK;
    // ---- 2. element boxes
    RIGC_TRY(c.vbox.reserve((size_t)6 * s.nv * sizeof(double)));
    RIGC_TRY(c.ebox.reserve((size_t)6 * s.ne * sizeof(double) + 8));
    RIGC_TRY(c.fbox.reserve((size_t)6 * s.nf * sizeof(double) + 8));
    RIGC_TRY(c.vin.reserve((size_t)s.nv + 8));
    RIGC_TRY(c.ein.reserve((size_t)s.ne + 8));
    RIGC_TRY(c.fin.reserve((size_t)s.nf + 8));
    if (continuous) {
        RIGC_TRY(S[0].reserve((size_t)blist.size() * sizeof(int) + 64 * sizeof(double)));
        int* d_list = S[0].as<int>();
        double* d_domain = reinterpret_cast<double*>(S[0].as<char>() + ((blist.size() * sizeof(int) + 63) / 64) * 64);
        RIGC_CUDA(cudaMemcpyAsync(d_list, blist.data(), blist.size() * sizeof(int),
                                  cudaMemcpyHostToDevice, st));
        RIGC_COUNT_LAUNCH();
        k_scene_box<<<1, 256, 0, st>>>(c.body_box.as<double>(), c.body_in.as<int>(), s.nb, d_domain);
        RIGC_COUNT_LAUNCH();
        k_clear_flags<<<grid_for(s.nv, 256), 256, 0, st>>>(c.vin.as<char>(), s.nv);
        RIGC_COUNT_LAUNCH();
        k_vertex_boxes_cont<<<(unsigned)blist.size(), kVBThreads, 0, st>>>(
            x0, x1, s.rest, s.bvs, d_list, d_domain, infl, c.vbox.as<double>(), c.vin.as<char>());
        // the host copy of blist must outlive the async copy
        RIGC_CUDA(cudaStreamSynchronize(st));
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
    // ---- 3. element list
    const int ntot = s.nv + s.ne + s.nf;
    RIGC_TRY(S[1].reserve((size_t)(2 * ntot + 16) * sizeof(int32_t)));
    int32_t* flag = S[1].as<int32_t>();
    int32_t* pos = flag + ntot;
    int32_t* cnt_dev = c.d_scalars.as<int32_t>();
    RIGC_COUNT_LAUNCH();
    k_elem_flags<<<grid_for(ntot, 256), 256, 0, st>>>(c.vin.as<char>(), c.ein.as<char>(),
                                                     c.fin.as<char>(), s.nv, s.ne, s.nf, flag);
    RIGC_TRY(exclusive_scan_i32(flag, pos, ntot, cnt_dev, S[7], st));
    int32_t m, epos[2];
    RIGC_CUDA(cudaMemcpyAsync(&m, cnt_dev, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaMemcpyAsync(epos, pos + s.nv, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    if (s.nf > 0)
        RIGC_CUDA(cudaMemcpyAsync(epos + 1, pos + s.nv + s.ne, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaStreamSynchronize(st));
    if (s.nf == 0) epos[1] = m;
    const int n_edges_in = epos[1] - epos[0];
    if (m == 0) return RIGC_OK;
    RIGC_TRY(S[2].reserve((size_t)m * sizeof(uint32_t) + (size_t)m * sizeof(double) + 4096 * 6 * 8));
    uint32_t* elems = S[2].as<uint32_t>();
    double* ext = reinterpret_cast<double*>(S[2].as<char>() + (((size_t)m * 4 + 255) / 256) * 256);
    double* part = ext + m;
    RIGC_COUNT_LAUNCH();
    k_elem_list<<<grid_for(ntot, 256), 256, 0, st>>>(flag, pos, s.nv, s.ne, s.nf, elems);
    const int nbk = 256;
    RIGC_COUNT_LAUNCH();
    k_elem_bounds<<<nbk, 256, 0, st>>>(elems, m, c.vbox.as<double>(), c.ebox.as<double>(),
                                       c.fbox.as<double>(), part, ext);
    double* d_sum = reinterpret_cast<double*>(c.d_scalars.as<char>() + 512);
    RIGC_TRY(sum_f64(ext, m, d_sum, S[7], st));
    std::vector<double> hpart(6 * nbk);
    double hsum;
    RIGC_CUDA(cudaMemcpyAsync(hpart.data(), part, hpart.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaMemcpyAsync(&hsum, d_sum, sizeof(double), cudaMemcpyDeviceToHost, st));
    // count included edges for the mean extent
    RIGC_CUDA(cudaStreamSynchronize(st));
    Grid g;
    double glo[3] = { INFINITY, INFINITY, INFINITY }, ghi[3] = { -INFINITY, -INFINITY, -INFINITY };
    for (int b = 0; b < nbk; b++)
        for (int j = 0; j < 3; j++) {
            glo[j] = std::min(glo[j], hpart[6 * b + j]);
            ghi[j] = std::max(ghi[j], hpart[6 * b + 3 + j]);
        }
    // cell size: mean extent of the included edge boxes
    double cell = hsum / std::max(1, n_edges_in);
    cell = std::max(cell, s.avg_edge_len * 0.5);
    cell = std::max(cell, 1e-9);
    for (int j = 0; j < 3; j++) g.lo[j] = glo[j];
    for (;;) {
        double tot = 1;
        for (int j = 0; j < 3; j++) {
            g.dims[j] = (long long)std::ceil((ghi[j] - glo[j]) / cell) + 1;
            tot *= (double)g.dims[j];
        }
        if (tot < 4e12) break;
        cell *= 2;
    }
    g.cell = cell;
    g.grow = 1e-9 * cell;
    uint64_t ncells = (uint64_t)g.dims[0] * g.dims[1] * g.dims[2];
    const ElemScene es { s.vbody, s.ebody, s.fbody, s.bscene };
    // positions of each scene's elements in elems, per type
    RIGC_TRY(c.seg.reserve((size_t)(3 * (s.nscenes + 1) + 8) * sizeof(int32_t)));
    int32_t* srange = c.seg.as<int32_t>();
    RIGC_COUNT_LAUNCH();
    k_scene_ranges<<<grid_for(s.nscenes + 1, 128), 128, 0, st>>>(
        pos, s.scene_bstart, s.bvs, s.bes, s.bfs, s.nscenes, s.nv, s.ne, s.nf, m, srange);
    // ---- 4. items
    RIGC_TRY(S[3].reserve((size_t)(3 * m + 16) * sizeof(int32_t)));
    int32_t* icnt = S[3].as<int32_t>();
    int32_t* ioff = icnt + m;
    int32_t* lflag = ioff + m;
    RIGC_COUNT_LAUNCH();
    k_count_cells<<<grid_for(m, 256), 256, 0, st>>>(elems, m, c.vbox.as<double>(), c.ebox.as<double>(),
                                                   c.fbox.as<double>(), g, icnt, lflag);
    RIGC_TRY(exclusive_scan_i32(icnt, ioff, m, cnt_dev, S[7], st));
    RIGC_TRY(S[6].reserve((size_t)(m + 16) * sizeof(int32_t)));
    int32_t* lpos = S[6].as<int32_t>();
    RIGC_TRY(exclusive_scan_i32(lflag, lpos, m, cnt_dev + 1, S[7], st));
    int32_t counts[2];
    RIGC_CUDA(cudaMemcpyAsync(counts, cnt_dev, sizeof(counts), cudaMemcpyDeviceToHost, st));
    RIGC_CUDA(cudaStreamSynchronize(st));
    const int64_t nitems = counts[0];
    const int nlarge = counts[1];
    c.stats.grid_items = nitems;
    c.stats.large_elements = nlarge;
    RIGC_TRY(c.items_key.reserve((size_t)nitems * 8 + 8));
    RIGC_TRY(c.items_val.reserve((size_t)nitems * 4 + 8));
    RIGC_TRY(c.items_key2.reserve((size_t)nitems * 8 + 8));
    RIGC_TRY(c.items_val2.reserve((size_t)nitems * 4 + 8));
    RIGC_COUNT_LAUNCH();
    k_emit_items<<<grid_for(m, 256), 256, 0, st>>>(elems, m, c.vbox.as<double>(), c.ebox.as<double>(),
                                                  c.fbox.as<double>(), g, es, ncells, icnt, ioff,
                                                  c.items_key.as<uint64_t>(), c.items_val.as<uint32_t>());
    RIGC_TRY(radix_sort_pairs<uint64_t>(c.items_key.as<uint64_t>(), c.items_val.as<uint32_t>(),
                                        c.items_key2.as<uint64_t>(), c.items_val2.as<uint32_t>(),
                                        nitems, bits_for(ncells * (uint64_t)s.nscenes - 1), S[4],
                                        S[5], S[7], st));
    RIGC_TRY(c.large_list.reserve((size_t)(nlarge + 1) * sizeof(uint32_t)));
    RIGC_COUNT_LAUNCH();
    k_large_list<<<grid_for(m, 256), 256, 0, st>>>(elems, lflag, lpos, m, c.large_list.as<uint32_t>());
    // ---- 5. pairs (retry once with exact capacity on overflow)
    PairCtx P { c.vbox.as<double>(), c.ebox.as<double>(), c.fbox.as<double>(), s.vbody, s.ebody,
                s.fbody, s.group, s.nv, s.ne };
    unsigned long long* pn = reinterpret_cast<unsigned long long*>(c.d_scalars.as<char>() + 1024);
    unsigned long long cap_ee = std::max<unsigned long long>(1 << 16, (unsigned long long)nitems);
    unsigned long long cap_fv = cap_ee;
    for (int attempt = 0; attempt < 3; attempt++) {
        RIGC_TRY(c.pair_out.reserve((size_t)(cap_ee + cap_fv) * 8));
        PairOut o { c.pair_out.as<unsigned long long>(), c.pair_out.as<unsigned long long>() + cap_ee,
                    cap_ee, cap_fv, pn, pn + 1 };
        RIGC_CUDA(cudaMemsetAsync(pn, 0, 2 * sizeof(unsigned long long), st));
        if (nitems > 0 && nitems <= kWarpPairItems) {
            RIGC_COUNT_LAUNCH();
            k_cell_pairs_warp<<<grid_for(nitems * 32, 128), 128, 0, st>>>(
                c.items_key2.as<uint64_t>(), c.items_val2.as<uint32_t>(), nitems, P, g, es, ncells, o);
        } else if (nitems > 0) {
            RIGC_COUNT_LAUNCH();
            k_cell_pairs<<<grid_for(nitems, 128), 128, 0, st>>>(c.items_key2.as<uint64_t>(),
                                                              c.items_val2.as<uint32_t>(), nitems, P, g,
                                                              es, ncells, o);
        }
        if (nlarge > 0) {
            // enough blocks per large element to cover a whole scene's elements
            const unsigned bx = (unsigned)std::min<int64_t>(
                1024, std::max<int64_t>(1, ((int64_t)m / s.nscenes + 255) / 256));
            for (int row0 = 0; row0 < nlarge; row0 += 65535) {
                const unsigned rows = (unsigned)std::min(65535, nlarge - row0);
                RIGC_COUNT_LAUNCH();
                k_large_pairs<<<dim3(bx, rows), 256, 0, st>>>(c.large_list.as<uint32_t>(), nlarge, row0,
                                                            elems, lflag, srange, s.nscenes, es, P, o);
            }
        }
        RIGC_CUDA(cudaGetLastError());
        unsigned long long hn[2];
        RIGC_CUDA(cudaMemcpyAsync(hn, pn, sizeof(hn), cudaMemcpyDeviceToHost, st));
        RIGC_CUDA(cudaStreamSynchronize(st));
        if (hn[0] <= cap_ee && hn[1] <= cap_fv) {
            c.cand.num_ee = (int64_t)hn[0];
            c.cand.num_fv = (int64_t)hn[1];
            break;
        }
        cap_ee = std::max(cap_ee, hn[0]);
        cap_fv = std::max(cap_fv, hn[1]);
        if (attempt == 2) return RIGC_ERR_OOM;
    }
    // ---- 6. canonical order
    const int64_t nee = c.cand.num_ee, nfv = c.cand.num_fv;
    unsigned long long* kee = c.pair_out.as<unsigned long long>();
    unsigned long long* kfv = kee + cap_ee;
    RIGC_TRY(c.cand.ee.reserve((size_t)nee * sizeof(int2) + 8));
    RIGC_TRY(c.cand.fv.reserve((size_t)nfv * sizeof(int2) + 8));
    int64_t nmax = std::max(nee, nfv);
    RIGC_TRY(c.pair_key.reserve((size_t)nmax * 8 + 8));
    RIGC_TRY(S[0].reserve((size_t)nmax * 4 + 8));
    RIGC_TRY(S[1].reserve((size_t)nmax * 4 + 8));
    if (nee > 0) {
        RIGC_COUNT_LAUNCH();
        k_iota<<<grid_for(nee, 256), 256, 0, st>>>(S[0].as<uint32_t>(), nee);
        RIGC_TRY(radix_sort_pairs<uint64_t>(reinterpret_cast<uint64_t*>(kee), S[0].as<uint32_t>(), c.pair_key.as<uint64_t>(),
                                            S[1].as<uint32_t>(), nee,
                                            bits_for((uint64_t)s.ne * (uint64_t)s.ne), S[4], S[5], S[7], st));
        RIGC_COUNT_LAUNCH();
        k_decode_pairs<<<grid_for(nee, 256), 256, 0, st>>>(c.pair_key.as<unsigned long long>(), nee,
                                                          (unsigned long long)s.ne, c.cand.ee.as<int2>());
    }
    if (nfv > 0) {
        RIGC_COUNT_LAUNCH();
        k_iota<<<grid_for(nfv, 256), 256, 0, st>>>(S[0].as<uint32_t>(), nfv);
        RIGC_TRY(radix_sort_pairs<uint64_t>(reinterpret_cast<uint64_t*>(kfv), S[0].as<uint32_t>(), c.pair_key.as<uint64_t>(),
                                            S[1].as<uint32_t>(), nfv,
                                            bits_for((uint64_t)s.nf * (uint64_t)s.nv), S[4], S[5], S[7], st));
        RIGC_COUNT_LAUNCH();
        k_decode_pairs<<<grid_for(nfv, 256), 256, 0, st>>>(c.pair_key.as<unsigned long long>(), nfv,
                                                          (unsigned long long)s.nv, c.cand.fv.as<int2>());
    }
    RIGC_CUDA(cudaGetLastError());
    return RIGC_OK;
}

} // namespace rigc
