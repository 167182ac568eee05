// Oracle: rigid broad phase (test infrastructure only).
//
// Restates detect_collision_candidates_rigid with the hash grid
// (src/ccd/rigid/broad_phase.cpp:19-91, 127-204), the body-pair culling
// (RigidBodyAssembler::close_bodies_bvh, src/physics/rigid_body_assembler.cpp:
// 307-356; RigidBody::compute_bounding_box, src/physics/rigid_body.cpp:
// 246-272) and the element boxes of RigidBodyHashGrid (src/ccd/rigid/
// rigid_body_hash_grid.cpp:36-344: interval vertex trajectories with one
// forced bisection of [0, 1], hulls, edge/face boxes as unions of vertex
// boxes).  ipc-toolkit's HashGrid reports the element pairs that share a cell
// and whose boxes overlap (center / half-extent test) and belong to different
// groups; that set does not depend on the cell layout, so it is produced here
// both by a sequential hash grid and by brute force.
#include "interval.hpp"
#include "oracle.hpp"

#include <algorithm>
#include <atomic>
#include <thread>

#include <algorithm>
#include <unordered_map>

namespace orc {

void irotation(const I r[3], I R[9]);
void iworld_vertex(const I R[9], const I p[3], const double* v, I out[3]);

static AABB make_box(const double lo[3], const double hi[3])
{
    AABB b;
    for (int i = 0; i < 3; i++) {
        b.lo[i] = lo[i];
        b.hi[i] = hi[i];
    }
    return b;
}

static AABB box_union(const AABB& a, const AABB& b)
{
    AABB r;
    for (int i = 0; i < 3; i++) {
        r.lo[i] = std::min(a.lo[i], b.lo[i]);
        r.hi[i] = std::max(a.hi[i], b.hi[i]);
    }
    return r;
}

bool aabb_overlap(const AABB& a, const AABB& b)
{
    for (int i = 0; i < 3; i++) {
        double ha = (a.hi[i] - a.lo[i]) / 2, hb = (b.hi[i] - b.lo[i]) / 2;
        double ca = a.lo[i] + ha, cb = b.lo[i] + hb;
        if (!(std::fabs(ca - cb) <= ha + hb)) return false;
    }
    return true;
}

void body_bounding_box(
    const Scene& s, int b, const double* x0, const double* x1, double lo[3],
    double hi[3])
{
    const double* p0 = x0 + 6 * b;
    const double* p1 = x1 + 6 * b;
    bool same_rot = p0[3] == p1[3] && p0[4] == p1[4] && p0[5] == p1[5];
    if (s.type[b] == 0 || same_rot) {
        for (int i = 0; i < 3; i++) {
            lo[i] = INFINITY;
            hi[i] = -INFINITY;
        }
        for (const double* pp : { p0, p1 }) {
            double R[9];
            rotation_matrix(pp + 3, R);
            for (int v = s.bvs[b]; v < s.bvs[b + 1]; v++) {
                const double* r = s.rest + 3 * v;
                for (int j = 0; j < 3; j++) {
                    double w = ((r[0] * R[3 * j] + r[1] * R[3 * j + 1]) + r[2] * R[3 * j + 2]) + pp[j];
                    lo[j] = std::min(lo[j], w);
                    hi[j] = std::max(hi[j], w);
                }
            }
        }
    } else {
        for (int j = 0; j < 3; j++) {
            lo[j] = std::min(p0[j], p1[j]) - s.rmax[b];
            hi[j] = std::max(p0[j], p1[j]) + s.rmax[b];
        }
    }
}

std::vector<std::array<int, 2>> close_bodies(
    const Scene& s, const double* x0, const double* x1, double inflation)
{
    std::vector<AABB> boxes(s.nb);
    for (int b = 0; b < s.nb; b++) {
        double lo[3], hi[3];
        body_bounding_box(s, b, x0, x1, lo, hi);
        for (int j = 0; j < 3; j++) {
            lo[j] -= inflation;
            hi[j] += inflation;
        }
        boxes[b] = make_box(lo, hi);
    }
    std::vector<std::array<int, 2>> out;
    for (int i = 0; i < s.nb; i++)
        for (int j = i + 1; j < s.nb; j++) {
            if (s.group[i] == s.group[j]) continue;
            bool ov = true;
            for (int k = 0; k < 3; k++)
                if (boxes[i].lo[k] > boxes[j].hi[k] || boxes[j].lo[k] > boxes[i].hi[k]) ov = false;
            if (ov) out.push_back({ i, j });
        }
    return out;
}

// scene box of the included bodies, padded by 1e-8 of its diagonal
// (compute_scene_conservative_bbox, rigid_body_hash_grid.cpp:64-88)
static void scene_box(const Scene& s, const double* x0, const double* x1,
                      const std::vector<char>& body_in, double lo[3], double hi[3])
{
    for (int j = 0; j < 3; j++) {
        lo[j] = INFINITY;
        hi[j] = -INFINITY;
    }
    for (int b = 0; b < s.nb; b++) {
        if (!body_in[b]) continue;
        double blo[3], bhi[3];
        body_bounding_box(s, b, x0, x1, blo, bhi);
        for (int j = 0; j < 3; j++) {
            lo[j] = std::min(lo[j], blo[j]);
            hi[j] = std::max(hi[j], bhi[j]);
        }
    }
    double d0 = hi[0] - lo[0], d1 = hi[1] - lo[1], d2 = hi[2] - lo[2];
    double diag = std::sqrt((d0 * d0 + d1 * d1) + d2 * d2);
    for (int j = 0; j < 3; j++) {
        lo[j] -= 1e-8 * diag;
        hi[j] += 1e-8 * diag;
    }
}

// interval vertex positions over t, bisected until they fit the domain
// (compute_vertices_intervals, rigid_body_hash_grid.cpp:188-246); the first
// call forces one bisection; recursion stops after 16 levels.
static void body_vertex_intervals(
    const Scene& s, int b, const double* x0, const double* x1, const I& t,
    int force, int depth, const double dlo[3], const double dhi[3],
    double inflation, std::vector<I>& out)
{
    const int n = s.bvs[b + 1] - s.bvs[b];
    if (force <= 0) {
        I p[3], r[3], R[9];
        const double* a = x0 + 6 * b;
        const double* c = x1 + 6 * b;
        for (int k = 0; k < 3; k++) {
            p[k] = (I(c[k]) - I(a[k])) * t + I(a[k]);
            r[k] = (I(c[3 + k]) - I(a[3 + k])) * t + I(a[3 + k]);
        }
        irotation(r, R);
        out.resize(3 * n);
        bool fits = true;
        for (int v = 0; v < n; v++) {
            iworld_vertex(R, p, s.rest + 3 * (s.bvs[b] + v), &out[3 * v]);
            for (int j = 0; j < 3; j++)
                if (out[3 * v + j].lo - inflation < dlo[j] || out[3 * v + j].hi + inflation > dhi[j])
                    fits = false;
        }
        if (fits || depth >= 16) return;
    }
    double m = median(t);
    std::vector<I> A, B;
    body_vertex_intervals(s, b, x0, x1, I(t.lo, m), force - 1, depth + 1, dlo, dhi, inflation, A);
    body_vertex_intervals(s, b, x0, x1, I(m, t.hi), force - 1, depth + 1, dlo, dhi, inflation, B);
    out.resize(3 * n);
    for (int i = 0; i < 3 * n; i++) out[i] = hull(A[i], B[i]);
}

void element_aabbs(
    const Scene& s, const double* x0, const double* x1, bool continuous,
    double inflation, const std::vector<std::array<int, 2>>& body_pairs,
    std::vector<AABB>& vbox, std::vector<AABB>& ebox, std::vector<AABB>& fbox,
    std::vector<char>& vin, std::vector<char>& ein, std::vector<char>& fin)
{
    std::vector<char> body_in(s.nb, 0);
    for (const auto& p : body_pairs) body_in[p[0]] = body_in[p[1]] = 1;
    vbox.assign(s.nv, AABB {});
    ebox.assign(s.ne, AABB {});
    fbox.assign(s.nf, AABB {});
    vin.assign(s.nv, 0);
    ein.assign(s.ne, 0);
    fin.assign(s.nf, 0);
    if (continuous) {
        double dlo[3], dhi[3];
        scene_box(s, x0, x1, body_in, dlo, dhi);
        // the bodies over the host's threads (each writes its own vertices;
        // threads for large scenes only, the time step calls this often)
        const bool big = (long long)s.nv + s.ne + s.nf >= 100000;
        parallel_for(s.nb, big ? 1 : s.nb, [&](long long bl) {
            const int b = (int)bl;
            if (!body_in[b]) return;
            std::vector<I> iv;
            body_vertex_intervals(s, b, x0, x1, I(0.0, 1.0), 1, 0, dlo, dhi, inflation, iv);
            for (int v = 0; v < s.bvs[b + 1] - s.bvs[b]; v++) {
                double lo[3], hi[3];
                bool ok = true;
                for (int j = 0; j < 3; j++) {
                    const I& q = iv[3 * v + j];
                    if (q.is_empty()) ok = false;
                    lo[j] = q.lo - inflation;
                    hi[j] = q.hi + inflation;
                }
                int gv = s.bvs[b] + v;
                if (ok) {
                    vbox[gv] = make_box(lo, hi);
                    vin[gv] = 1;
                }
            }
        });
    } else {
        std::vector<double> V;
        world_vertices(s, x0, V);
        for (int v = 0; v < s.nv; v++) {
            if (!body_in[s.vbody[v]]) continue;
            double lo[3], hi[3];
            for (int j = 0; j < 3; j++) {
                lo[j] = V[3 * v + j] - inflation;
                hi[j] = V[3 * v + j] + inflation;
            }
            vbox[v] = make_box(lo, hi);
            vin[v] = 1;
        }
    }
    for (int e = 0; e < s.ne; e++) {
        int a = s.edges[2 * e], b = s.edges[2 * e + 1];
        if (vin[a] && vin[b]) {
            ebox[e] = box_union(vbox[a], vbox[b]);
            ein[e] = 1;
        }
    }
    for (int f = 0; f < s.nf; f++) {
        int a = s.faces[3 * f], b = s.faces[3 * f + 1], c = s.faces[3 * f + 2];
        if (vin[a] && vin[b] && vin[c]) {
            fbox[f] = box_union(box_union(vbox[a], vbox[b]), vbox[c]);
            fin[f] = 1;
        }
    }
}

namespace {
struct Item {
    long long key;
    int id;
    bool operator<(const Item& o) const { return key < o.key || (key == o.key && id < o.id); }
};
} // namespace

void detect_candidates(
    const Scene& s, const double* x0, const double* x1, bool continuous,
    double inflation, bool brute_force, Candidates& out)
{
    out.ev.clear();
    out.ee.clear();
    out.fv.clear();
    if (s.nb <= 1) return;
    auto pairs = close_bodies(s, x0, continuous ? x1 : x0, inflation);
    if (pairs.empty()) return;
    std::vector<AABB> vb, eb, fb;
    std::vector<char> vi, ei, fi;
    element_aabbs(s, x0, x1, continuous, inflation, pairs, vb, eb, fb, vi, ei, fi);
    auto egrp = [&](int e) { return s.group[s.ebody[e]]; };
    auto vgrp = [&](int v) { return s.group[s.vbody[v]]; };
    auto fgrp = [&](int f) { return s.group[s.fbody[f]]; };

    if (brute_force) {
        for (int a = 0; a < s.ne; a++) {
            if (!ei[a]) continue;
            for (int b = a + 1; b < s.ne; b++)
                if (ei[b] && egrp(a) != egrp(b) && aabb_overlap(eb[a], eb[b]))
                    out.ee.push_back({ a, b });
        }
        for (int f = 0; f < s.nf; f++) {
            if (!fi[f]) continue;
            for (int v = 0; v < s.nv; v++)
                if (vi[v] && fgrp(f) != vgrp(v) && aabb_overlap(fb[f], vb[v]))
                    out.fv.push_back({ f, v });
        }
        return;
    }

    // hash grid over the boxes of the included elements
    double lo[3] = { INFINITY, INFINITY, INFINITY }, hi[3] = { -INFINITY, -INFINITY, -INFINITY };
    double len = 0;
    long nl = 0;
    for (int v = 0; v < s.nv; v++)
        if (vi[v])
            for (int j = 0; j < 3; j++) {
                lo[j] = std::min(lo[j], vb[v].lo[j]);
                hi[j] = std::max(hi[j], vb[v].hi[j]);
            }
    for (int e = 0; e < s.ne; e++)
        if (ei[e]) {
            double m = 0;
            for (int j = 0; j < 3; j++) m = std::max(m, eb[e].hi[j] - eb[e].lo[j]);
            len += m;
            nl++;
        }
    double cell = std::max(nl ? len / nl : 1.0, 1e-6);
    long long dims[3];
    for (int j = 0; j < 3; j++) dims[j] = std::max(1LL, (long long)std::ceil((hi[j] - lo[j]) / cell) + 1);
    auto cidx = [&](double x, int j) {
        long long c = (long long)std::floor((x - lo[j]) / cell);
        return std::min(std::max(c, 0LL), dims[j] - 1);
    };
    // cell ranges of slightly grown boxes: pairs that overlap by the
    // center / half-extent test always share a cell
    const double grow = 1e-9 * cell;
    auto add = [&](const AABB& b, int id, std::vector<Item>& items) {
        long long c0[3], c1[3];
        for (int j = 0; j < 3; j++) {
            c0[j] = cidx(b.lo[j] - grow, j);
            c1[j] = cidx(b.hi[j] + grow, j);
        }
        for (long long x = c0[0]; x <= c1[0]; x++)
            for (long long y = c0[1]; y <= c1[1]; y++)
                for (long long z = c0[2]; z <= c1[2]; z++)
                    items.push_back({ (z * dims[1] + y) * dims[0] + x, id });
    };
    // the items of each kind (chunks of elements over the host's threads,
    // concatenated in chunk order), sorted by (cell, element): the same
    // sorted lists as one sequential pass
    const int nt = (long long)s.nv + s.ne + s.nf >= 100000
                       ? std::max(1, (int)std::thread::hardware_concurrency())
                       : 1;
    auto items_of = [&](int n, const std::vector<AABB>& box, const std::vector<char>& in) {
        std::vector<std::vector<Item>> part(nt);
        const long long per = (n + nt - 1) / nt;
        parallel_for(nt, 1, [&](long long t) {
            for (long long k = t * per; k < std::min<long long>(n, (t + 1) * per); k++)
                if (in[k]) add(box[k], (int)k, part[t]);
        });
        std::vector<Item> all;
        for (auto& q : part) all.insert(all.end(), q.begin(), q.end());
        // sorted chunks, then merged pairwise
        std::vector<size_t> cut(nt + 1);
        for (int t = 0; t <= nt; t++) cut[t] = all.size() * t / nt;
        parallel_for(nt, 1, [&](long long t) { std::sort(all.begin() + cut[t], all.begin() + cut[t + 1]); });
        for (int w = 1; w < nt; w *= 2) {
            std::vector<long long> lefts;
            for (int t = 0; t + w < nt; t += 2 * w) lefts.push_back(t);
            parallel_for((long long)lefts.size(), 1, [&](long long k) {
                const int t = (int)lefts[k];
                std::inplace_merge(all.begin() + cut[t], all.begin() + cut[t + w],
                                   all.begin() + cut[std::min(nt, t + 2 * w)]);
            });
        }
        return all;
    };
    std::vector<Item> vitems = items_of(s.nv, vb, vi), eitems = items_of(s.ne, eb, ei),
                      fitems = items_of(s.nf, fb, fi);
    // cell runs of a sorted list split over the threads at cell boundaries
    auto runs = [&](const std::vector<Item>& it) {
        std::vector<size_t> cut(nt + 1, it.size());
        cut[0] = 0;
        for (int t = 1; t < nt; t++) {
            size_t c = std::max(cut[t - 1], it.size() * t / nt);
            while (c > 0 && c < it.size() && it[c].key == it[c - 1].key) c++;
            cut[t] = std::min(c, it.size());
        }
        return cut;
    };
    std::vector<std::vector<std::array<int, 2>>> pee(nt), pfv(nt);
    // edge-edge within cells
    {
        const std::vector<size_t> cut = runs(eitems);
        parallel_for(nt, 1, [&](long long t) {
            for (size_t i = cut[t]; i < cut[t + 1];) {
                size_t j = i;
                while (j < eitems.size() && eitems[j].key == eitems[i].key) j++;
                for (size_t a = i; a < j; a++)
                    for (size_t b = a + 1; b < j; b++) {
                        int ea = eitems[a].id, ebb = eitems[b].id;
                        if (egrp(ea) != egrp(ebb) && aabb_overlap(eb[ea], eb[ebb]))
                            pee[t].push_back({ std::min(ea, ebb), std::max(ea, ebb) });
                    }
                i = j;
            }
        });
    }
    // face-vertex within cells (merge of the two sorted lists)
    {
        const std::vector<size_t> cut = runs(fitems);
        parallel_for(nt, 1, [&](long long t) {
            if (cut[t] >= cut[t + 1]) return;
            size_t vpos = std::lower_bound(vitems.begin(), vitems.end(), Item { fitems[cut[t]].key, -1 })
                          - vitems.begin();
            for (size_t i = cut[t]; i < cut[t + 1];) {
                size_t j = i;
                while (j < fitems.size() && fitems[j].key == fitems[i].key) j++;
                long long key = fitems[i].key;
                while (vpos < vitems.size() && vitems[vpos].key < key) vpos++;
                size_t vend = vpos;
                while (vend < vitems.size() && vitems[vend].key == key) vend++;
                for (size_t a = i; a < j; a++)
                    for (size_t b = vpos; b < vend; b++) {
                        int f = fitems[a].id, v = vitems[b].id;
                        if (fgrp(f) != vgrp(v) && aabb_overlap(fb[f], vb[v]))
                            pfv[t].push_back({ f, v });
                    }
                i = j;
            }
        });
    }
    for (int t = 0; t < nt; t++) {
        out.ee.insert(out.ee.end(), pee[t].begin(), pee[t].end());
        out.fv.insert(out.fv.end(), pfv[t].begin(), pfv[t].end());
    }
    std::sort(out.ee.begin(), out.ee.end());
    out.ee.erase(std::unique(out.ee.begin(), out.ee.end()), out.ee.end());
    std::sort(out.fv.begin(), out.fv.end());
    out.fv.erase(std::unique(out.fv.begin(), out.fv.end()), out.fv.end());
}

// Edge-face intersection candidates at poses x: close bodies and element
// boxes with no inflation (detect_intersection_candidates_rigid_bvh,
// src/ccd/rigid/broad_phase.cpp:265-302), every (face, edge) pair of
// different groups whose boxes overlap, tested pairwise over the close body
// pairs (test-sized scenes: no grid); sorted, unique.
void edge_face_candidates(const Scene& s, const double* x, std::vector<std::array<int, 2>>& out)
{
    out.clear();
    if (s.nb <= 1) return;
    auto pairs = close_bodies(s, x, x, 0.0);
    if (pairs.empty()) return;
    std::vector<AABB> vb, eb, fb;
    std::vector<char> vi, ei, fi;
    element_aabbs(s, x, x, false, 0.0, pairs, vb, eb, fb, vi, ei, fi);
    for (const auto& bp : pairs)
        for (int side = 0; side < 2; side++) {
            const int be = bp[side], bf = bp[1 - side];
            if (s.group[be] == s.group[bf]) continue;
            for (int e = s.bes[be]; e < s.bes[be + 1]; e++) {
                if (!ei[e]) continue;
                for (int f = s.bfs[bf]; f < s.bfs[bf + 1]; f++)
                    if (fi[f] && aabb_overlap(eb[e], fb[f])) out.push_back({ f, e });
            }
        }
    std::sort(out.begin(), out.end());
    out.erase(std::unique(out.begin(), out.end()), out.end());
}

} // namespace orc
