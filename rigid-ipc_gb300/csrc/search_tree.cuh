// Nodes of a CCD candidate's subdivision tree and the path encoding of a
// depth-first search over them (integer operations only; host and device).
//
// Every box of a candidate's search is dyadic: per dimension (t, alpha,
// beta) it is [i 2^-l, (i + 1) 2^-l] for a level l and an index i, because
// the root is [0, 1]^3 and a split halves one dimension at its midpoint,
// which is exact while l <= kMaxLevel.  So a box is a node (levels,
// indices, depth = number of splits from the root), and the depth-first
// search needs no box stack: the boxes a stack would hold are the upper
// children of the depths at which the current path went to the lower child.
// A search keeps the current node, a 128-bit mask of the depths whose upper
// child is still pending, and two masks recording which depths split t and
// which split alpha (the others split beta); a pending box is rebuilt from
// the current node by undoing the splits below its depth.  Popping the
// deepest pending depth visits boxes in the order of a stack that pushes the
// upper half first; the shallowest pending depth is the stack's bottom, the
// box a work-sharing search takes.
//
// The header compiles as CUDA (nvcc) and as plain C++, so that the encoding
// is checked on the CPU against an explicit box stack.
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define RIGC_HD __host__ __device__ __forceinline__
#else
#define RIGC_HD inline
#endif

namespace rigc {

typedef unsigned __int128 u128;
constexpr int kMaxDepth = 120;  // splits along one path (mask bits)
constexpr int kMaxLevel = 52;   // splits along one dimension (exact bounds)

struct Node {
    int lv[3];
    unsigned long long ix[3];
    int depth;
};

RIGC_HD int st_popc64(unsigned long long x)
{
#ifdef __CUDA_ARCH__
    return __popcll(x);
#else
    return __builtin_popcountll(x);
#endif
}

// leading zeros of a non-zero value
RIGC_HD int st_clz64(unsigned long long x)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}

// 1 + index of the lowest set bit of a non-zero value
RIGC_HD int st_ffs64(unsigned long long x)
{
#ifdef __CUDA_ARCH__
    return __ffsll((long long)x);
#else
    return __builtin_ffsll((long long)x);
#endif
}

RIGC_HD double st_bits_to_double(unsigned long long b)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double d;
    std::memcpy(&d, &b, sizeof d);
    return d;
#endif
}

RIGC_HD u128 bit128(int k) { return (u128)1 << k; }

RIGC_HD int popc128(u128 m)
{
    return st_popc64((unsigned long long)m) + st_popc64((unsigned long long)(m >> 64));
}

// highest / lowest set bit of a non-zero mask
RIGC_HD int msb128(u128 m)
{
    const unsigned long long h = (unsigned long long)(m >> 64);
    return h ? 127 - st_clz64(h) : 63 - st_clz64((unsigned long long)m);
}

RIGC_HD int lsb128(u128 m)
{
    const unsigned long long l = (unsigned long long)m;
    return l ? st_ffs64(l) - 1 : 63 + st_ffs64((unsigned long long)(m >> 64));
}

// mask of the depths [lo, hi), hi <= kMaxDepth + 1
RIGC_HD u128 range128(int lo, int hi) { return (bit128(hi) - 1) & ~(bit128(lo) - 1); }

// i 2^-l for i <= 2^52, l <= kMaxLevel, assembled from its bits: exponent
// from the leading one, mantissa from the bits below it
RIGC_HD double dyadic(unsigned long long i, int l)
{
    const int e = 63 - st_clz64(i | 1ull);  // i in [2^e, 2^(e + 1))
    const unsigned long long m = (i << (52 - e)) & 0xfffffffffffffull;
    const double v = st_bits_to_double(((unsigned long long)(1023 + e - l) << 52) | m);
    return i ? v : 0.0;
}

// The box widths of the root finder, sub_up(hi, lo): the exact difference
// 2^-l stepped one ulp up (the bit pattern of 2^-l plus one)
RIGC_HD void node_widths(const Node& c, double w[3])
{
    for (int k = 0; k < 3; k++)
        w[k] = st_bits_to_double(((unsigned long long)(1023 - c.lv[k]) << 52) + 1ull);
}

// record that depth k splits dimension s
RIGC_HD void record_split(u128& mt, u128& ma, int k, int s)
{
    const u128 b = bit128(k);
    mt = s == 0 ? (mt | b) : (mt & ~b);
    ma = s == 1 ? (ma | b) : (ma & ~b);
}

// The upper child of c's ancestor at depth j, where c's path went to the
// lower child: c's node at depth j + 1 with the splits of depths
// j + 1 .. c.depth - 1 undone and its last index bit set.
RIGC_HD Node pending_node(const Node& c, u128 mt, u128 ma, int j)
{
    const u128 r = range128(j + 1, c.depth);
    const int ct = popc128(mt & r), ca = popc128(ma & r);
    const int cb = c.depth - j - 1 - ct - ca;
    Node g;
    g.lv[0] = c.lv[0] - ct;
    g.lv[1] = c.lv[1] - ca;
    g.lv[2] = c.lv[2] - cb;
    g.ix[0] = c.ix[0] >> ct;
    g.ix[1] = c.ix[1] >> ca;
    g.ix[2] = c.ix[2] >> cb;
    const int s = (mt & bit128(j)) ? 0 : ((ma & bit128(j)) ? 1 : 2);
    g.ix[s] |= 1ull;
    g.depth = j + 1;
    return g;
}

// descend from c to its lower child along dimension s; the upper child
// becomes pending at c's depth
RIGC_HD void descend(Node& c, u128& pend_hi, u128& mt, u128& ma, int s)
{
    record_split(mt, ma, c.depth, s);
    pend_hi |= bit128(c.depth);
    c.lv[s]++;
    c.ix[s] <<= 1;
    c.depth++;
}

} // namespace rigc
