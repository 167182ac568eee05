// CPU check of the CCD search's path encoding (rigid-ipc_gb300/csrc/
// search_tree.cuh, compiled here as plain C++): a depth-first search over
// random subdivision trees driven by the encoding visits the same boxes in
// the same order as an explicit box stack that pushes the upper half first,
// hands out the same bottom box to work sharing, and reports the same
// smallest pending t.lo (the box budget's conservative bound).  Also checks
// dyadic() and node_widths() against ldexp and nextafter.  Prints "ok" and
// the number of checks, or the first mismatch (exit 1).
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "search_tree.cuh"

using namespace rigc;

struct Box {
    double t0, t1, a0, a1, b0, b1;
};

static Box node_box(const Node& c)
{
    return Box { dyadic(c.ix[0], c.lv[0]), dyadic(c.ix[0] + 1, c.lv[0]),
                 dyadic(c.ix[1], c.lv[1]), dyadic(c.ix[1] + 1, c.lv[1]),
                 dyadic(c.ix[2], c.lv[2]), dyadic(c.ix[2] + 1, c.lv[2]) };
}

static bool same(const Box& a, const Box& b)
{
    return a.t0 == b.t0 && a.t1 == b.t1 && a.a0 == b.a0 && a.a1 == b.a1 && a.b0 == b.b0
        && a.b1 == b.b1;
}

// the root finder's split rule on exact widths
static int split_of(const Box& x, const double* tol)
{
    double w[3] = { x.t1 - x.t0, x.a1 - x.a0, x.b1 - x.b0 };
    bool all = w[0] <= tol[0] && w[1] <= tol[1] && w[2] <= tol[2];
    int s = -1;
    for (int d = 0; d < 3; d++)
        if ((all || !(w[d] <= tol[d])) && (s == -1 || !(w[d] * tol[s] <= w[s] * tol[d]))) s = d;
    return s;
}

int main()
{
    long long checks = 0;
    std::mt19937_64 rng(7);
    // dyadic / widths
    for (int k = 0; k < 2000000; k++) {
        const int l = (int)(rng() % (kMaxLevel + 1));
        const unsigned long long i = rng() & ((1ull << l) - 1);
        if (dyadic(i, l) != std::ldexp((double)i, -l) || dyadic(i + 1, l) != std::ldexp((double)(i + 1), -l)) {
            std::printf("dyadic mismatch %llu %d\n", i, l);
            return 1;
        }
        Node c { { l, 0, 0 }, { 0, 0, 0 }, 0 };
        double w[3];
        node_widths(c, w);
        if (w[0] != std::nextafter(std::ldexp(1.0, -l), INFINITY)) {
            std::printf("width mismatch %d\n", l);
            return 1;
        }
        checks += 2;
    }
    // searches
    for (int trial = 0; trial < 20000; trial++) {
        double tol[3] = { std::ldexp(1.0, -(int)(rng() % 12)) * (1 + (rng() % 7) / 8.0),
                          std::ldexp(1.0, -(int)(rng() % 10)) * (1 + (rng() % 5) / 4.0),
                          std::ldexp(1.0, -(int)(rng() % 10)) };
        const double pleaf = 0.2 + 0.6 * ((rng() % 100) / 100.0);
        std::vector<Box> st { Box { 0, 1, 0, 1, 0, 1 } };
        size_t sb = 0;  // shared from the bottom
        Node cn { { 0, 0, 0 }, { 0, 0, 0 }, 0 };
        bool has = true;
        u128 pend = 0, mt = 0, ma = 0;
        std::mt19937_64 r2(trial);
        for (int steps = 0; steps < 3000; steps++) {
            if (st.size() - sb >= 2 && r2() % 13 == 0) {
                // work sharing takes the bottom box
                const int j = lsb128(pend);
                const Node g = pending_node(cn, mt, ma, j);
                pend &= ~bit128(j);
                if (!same(st[sb++], node_box(g)) || (int)(st.size() - sb) != popc128(pend) + (has ? 1 : 0)) {
                    std::printf("shared box mismatch, trial %d\n", trial);
                    return 1;
                }
                checks++;
            }
            if (r2() % 17 == 0) {
                // smallest pending t.lo
                double m1 = INFINITY, m2 = has ? node_box(cn).t0 : INFINITY;
                for (size_t s = sb; s < st.size(); s++) m1 = std::fmin(m1, st[s].t0);
                for (u128 r = pend; r != 0; r &= r - 1) {
                    const Node g = pending_node(cn, mt, ma, lsb128(r));
                    m2 = std::fmin(m2, dyadic(g.ix[0], g.lv[0]));
                }
                if (m1 != m2) {
                    std::printf("pending minimum mismatch, trial %d\n", trial);
                    return 1;
                }
                checks++;
            }
            const bool e1 = st.size() > sb, e2 = has || pend != 0;
            if (e1 != e2) {
                std::printf("emptiness mismatch, trial %d\n", trial);
                return 1;
            }
            if (!e1) break;
            const Box x = st.back();
            st.pop_back();
            if (has) {
                has = false;
            } else {
                const int j = msb128(pend);
                pend &= ~bit128(j);
                cn = pending_node(cn, mt, ma, j);
            }
            if (!same(x, node_box(cn))) {
                std::printf("pop mismatch, trial %d step %d\n", trial, steps);
                return 1;
            }
            checks++;
            if ((r2() % 1000) < pleaf * 1000 || cn.depth >= 100) continue;
            const int s = split_of(x, tol);
            if (cn.lv[s] >= kMaxLevel) continue;
            Box lo = x, hi = x;
            if (s == 0) {
                const double m = 0.5 * (x.t0 + x.t1);
                lo.t1 = m;
                hi.t0 = m;
            } else if (s == 1) {
                const double m = 0.5 * (x.a0 + x.a1);
                lo.a1 = m;
                hi.a0 = m;
            } else {
                const double m = 0.5 * (x.b0 + x.b1);
                lo.b1 = m;
                hi.b0 = m;
            }
            st.push_back(hi);
            st.push_back(lo);
            descend(cn, pend, mt, ma, s);
            has = true;
        }
    }
    std::printf("ok %lld\n", checks);
    return 0;
}
