// Interval arithmetic on the device for the rigid CCD.
//
// Semantics of the reference's Interval (src/interval/interval.hpp:25-30):
// Boost.Interval operations over the FILibRounding policy
// (src/interval/filib_rounding.cpp:12-60), i.e. each bound is the
// round-to-nearest result stepped one ulp outward, with exact-zero results
// kept exact (x == -y for sums, x == y for differences, a zero factor for
// products, a zero dividend for quotients).  Products and quotients use the
// sign-case tables; widths round up; cos/sin reduce by an enclosure of 2*pi and
// evaluate the monotone pieces with the deterministic cosine of rotation.cuh
// widened by its error bound.  The ulp steps are integer operations on the
// bit pattern.
#pragma once

#include "rotation.cuh"

namespace rigc {

struct Itv {
    double lo, hi;
};

__device__ __forceinline__ Itv mk(double l, double h) { return Itv { l, h }; }
__device__ __forceinline__ Itv pt(double x) { return Itv { x, x }; }
__device__ __forceinline__ Itv iempty()
{
    return Itv { __longlong_as_double(0x7ff8000000000000ll), __longlong_as_double(0x7ff8000000000000ll) };
}
__device__ __forceinline__ bool is_empty(const Itv& x) { return !(x.lo <= x.hi); }

// Bit pattern of a double through an opaque move: the optimizer cannot turn
// the integer tests below back into double-precision compares.
__device__ __forceinline__ long long dbits(double x)
{
    long long r;
    asm("mov.b64 %0, %1;" : "=l"(r) : "d"(x));
    return r;
}

// next double towards -inf / +inf (nextafter semantics, finite and zero inputs)
__device__ __forceinline__ double dpred(double x)
{
    long long b = dbits(x);
    if ((b & 0x7fffffffffffffffll) == 0) return __longlong_as_double(0x8000000000000001ll);
    if (b == (long long)0xfff0000000000000ull) return x;
    return __longlong_as_double(b > 0 ? b - 1 : b + 1);
}
__device__ __forceinline__ double dsucc(double x)
{
    long long b = dbits(x);
    if ((b & 0x7fffffffffffffffll) == 0) return __longlong_as_double(1ll);
    if (b == 0x7ff0000000000000ll) return x;
    return __longlong_as_double(b > 0 ? b + 1 : b - 1);
}

// Sign and order tests on the bit pattern (integer instructions; the
// double-precision pipe is the scarce one on this GPU).  Exact for every
// non-NaN double, +-0 and +-inf included; no NaN reaches them.
__device__ __forceinline__ bool is_zero(double x) { return (dbits(x) << 1) == 0; }
// x < 0: sign bit set and not -0
__device__ __forceinline__ bool is_neg(double x)
{
    return (unsigned long long)dbits(x) > 0x8000000000000000ull;
}
// x > 0
__device__ __forceinline__ bool is_pos(double x) { return dbits(x) > 0; }
// monotone integer key: key(x) < key(y) iff x < y, except -0 < +0
__device__ __forceinline__ long long order_key(double x)
{
    long long b = dbits(x);
    return b ^ ((b >> 63) & 0x7fffffffffffffffll);
}
// x < y
__device__ __forceinline__ bool lt(double x, double y)
{
    return order_key(x) < order_key(y) && !(is_zero(x) && is_zero(y));
}

// A sum or difference of finite doubles is zero only when exact (no
// underflow to zero), so the exact-zero rule tests the rounded result.
__device__ __forceinline__ double add_dn(double x, double y)
{
    double r = RADD(x, y);
    return is_zero(r) ? 0.0 : dpred(r);
}
__device__ __forceinline__ double add_up(double x, double y)
{
    double r = RADD(x, y);
    return is_zero(r) ? 0.0 : dsucc(r);
}
__device__ __forceinline__ double sub_dn(double x, double y)
{
    double r = RSUB(x, y);
    return is_zero(r) ? 0.0 : dpred(r);
}
__device__ __forceinline__ double sub_up(double x, double y)
{
    double r = RSUB(x, y);
    return is_zero(r) ? 0.0 : dsucc(r);
}
__device__ __forceinline__ double mul_dn(double x, double y)
{
    return (is_zero(x) || is_zero(y)) ? 0.0 : dpred(RMUL(x, y));
}
__device__ __forceinline__ double mul_up(double x, double y)
{
    return (is_zero(x) || is_zero(y)) ? 0.0 : dsucc(RMUL(x, y));
}
__device__ __forceinline__ double div_dn(double x, double y) { return is_zero(x) ? 0.0 : dpred(RDIV(x, y)); }
__device__ __forceinline__ double div_up(double x, double y) { return is_zero(x) ? 0.0 : dsucc(RDIV(x, y)); }

__device__ __forceinline__ double smin(double a, double b) { return lt(b, a) ? b : a; }
__device__ __forceinline__ double smax(double a, double b) { return lt(a, b) ? b : a; }

__device__ __forceinline__ Itv ineg(const Itv& x) { return Itv { -x.hi, -x.lo }; }
__device__ __forceinline__ Itv iadd(const Itv& x, const Itv& y)
{
    return Itv { add_dn(x.lo, y.lo), add_up(x.hi, y.hi) };
}
__device__ __forceinline__ Itv iadd(double x, const Itv& y) { return Itv { add_dn(x, y.lo), add_up(x, y.hi) }; }
__device__ __forceinline__ Itv isub(const Itv& x, const Itv& y)
{
    return Itv { sub_dn(x.lo, y.hi), sub_up(x.hi, y.lo) };
}
__device__ __forceinline__ Itv isub(const Itv& x, double y) { return Itv { sub_dn(x.lo, y), sub_up(x.hi, y) }; }

__device__ __forceinline__ Itv imul(const Itv& x, const Itv& y)
{
    const double xl = x.lo, xu = x.hi, yl = y.lo, yu = y.hi;
    if (is_neg(xl)) {
        if (is_pos(xu)) {
            if (is_neg(yl)) {
                if (is_pos(yu))
                    return Itv { smin(mul_dn(xl, yu), mul_dn(xu, yl)), smax(mul_up(xl, yl), mul_up(xu, yu)) };
                return Itv { mul_dn(xu, yl), mul_up(xl, yl) };
            }
            if (is_pos(yu)) return Itv { mul_dn(xl, yu), mul_up(xu, yu) };
            return Itv { 0.0, 0.0 };
        }
        if (is_neg(yl)) {
            if (is_pos(yu)) return Itv { mul_dn(xl, yu), mul_up(xl, yl) };
            return Itv { mul_dn(xu, yu), mul_up(xl, yl) };
        }
        if (is_pos(yu)) return Itv { mul_dn(xl, yu), mul_up(xu, yl) };
        return Itv { 0.0, 0.0 };
    }
    if (is_pos(xu)) {
        if (is_neg(yl)) {
            if (is_pos(yu)) return Itv { mul_dn(xu, yl), mul_up(xu, yu) };
            return Itv { mul_dn(xu, yl), mul_up(xl, yu) };
        }
        if (is_pos(yu)) return Itv { mul_dn(xl, yl), mul_up(xu, yu) };
        return Itv { 0.0, 0.0 };
    }
    return Itv { 0.0, 0.0 };
}

// Product with an interval y whose lower bound is not negative (time and
// barycentric intervals): the sign-case table reduces to one choice of
// factor per bound, made without branches.
__device__ __forceinline__ Itv imul_nonneg(const Itv& x, const Itv& y)
{
    const double yl = is_neg(x.lo) ? y.hi : y.lo;
    const double yu = is_neg(x.hi) ? y.lo : y.hi;
    return Itv { mul_dn(x.lo, yl), mul_up(x.hi, yu) };
}

// scalar times interval (a zero scalar gives [0, 0] through the zero rule)
__device__ __forceinline__ Itv imul(double x, const Itv& y)
{
    const bool neg = is_neg(x);
    return Itv { mul_dn(x, neg ? y.hi : y.lo), mul_up(x, neg ? y.lo : y.hi) };
}

// quotient by an interval that excludes zero (the only case on this path)
__device__ __forceinline__ Itv idiv(const Itv& x, const Itv& y)
{
    const double xl = x.lo, xu = x.hi, yl = y.lo, yu = y.hi;
    if (yl <= 0 && yu >= 0) {
        if (xl == 0 && xu == 0) return Itv { 0.0, 0.0 };
        return Itv { -INFINITY, INFINITY };
    }
    if (is_neg(xu)) {
        if (is_neg(yu)) return Itv { div_dn(xu, yl), div_up(xl, yu) };
        return Itv { div_dn(xl, yl), div_up(xu, yu) };
    }
    if (is_neg(xl)) {
        if (is_neg(yu)) return Itv { div_dn(xu, yu), div_up(xl, yu) };
        return Itv { div_dn(xl, yl), div_up(xu, yl) };
    }
    if (is_neg(yu)) return Itv { div_dn(xu, yu), div_up(xl, yl) };
    return Itv { div_dn(xl, yu), div_up(xu, yl) };
}
__device__ __forceinline__ Itv idiv(const Itv& x, double y)
{
    if (is_neg(y)) return Itv { div_dn(x.hi, y), div_up(x.lo, y) };
    return Itv { div_dn(x.lo, y), div_up(x.hi, y) };
}

__device__ __forceinline__ Itv isqrt(const Itv& x)
{
    if (is_empty(x) || is_neg(x.hi)) return iempty();
    double l = !is_pos(x.lo) ? 0.0 : (x.lo == 0 ? 0.0 : dpred(__dsqrt_rn(x.lo)));
    double h = x.hi == 0 ? 0.0 : dsucc(__dsqrt_rn(x.hi));
    return Itv { l, h };
}

__device__ __forceinline__ Itv iabs(const Itv& x)
{
    if (!is_neg(x.lo)) return x;
    if (!is_pos(x.hi)) return ineg(x);
    return Itv { 0.0, smax(-x.lo, x.hi) };
}

__device__ __forceinline__ Itv ihull(const Itv& x, const Itv& y)
{
    if (is_empty(x)) return y;
    if (is_empty(y)) return x;
    return Itv { smin(x.lo, y.lo), smax(x.hi, y.hi) };
}

__device__ __forceinline__ bool zero_in(const Itv& x) { return !is_pos(x.lo) && !is_neg(x.hi); }
__device__ __forceinline__ double iwidth(const Itv& x) { return sub_up(x.hi, x.lo); }

// ---------------------------------------------------------------------------
// cos / sin

constexpr double kPiLo = 3.141592653589793116;
constexpr double kPiHi = 3.141592653589793560;

__device__ __forceinline__ double clamp_pm1(double r) { return r < -1.0 ? -1.0 : (r > 1.0 ? 1.0 : r); }

__device__ __forceinline__ double cos_dn(double x)
{
    if (fabs(x) > 1048576.0) return -1.0;
    double c = det_cos(x);
    return clamp_pm1(dpred(RSUB(c, det_trig_err(c))));
}
__device__ __forceinline__ double cos_up(double x)
{
    if (fabs(x) > 1048576.0) return 1.0;
    double c = det_cos(x);
    return clamp_pm1(dsucc(RADD(c, det_trig_err(c))));
}

__device__ __forceinline__ Itv ifmod(const Itv& x, const Itv& y)
{
    double yb = is_neg(x.lo) ? y.lo : y.hi;
    double n = floor(div_dn(x.lo, yb));
    return isub(x, imul(n, y));
}

static __device__ __noinline__ Itv icos(Itv x)
{
    const Itv pi2 { kPiLo * 2, kPiHi * 2 };
    bool negate = false;
    Itv r;
    for (int pass = 0; pass < 2; pass++) {
        Itv tmp = ifmod(x, pi2);
        if (iwidth(tmp) >= pi2.lo) {
            r = Itv { -1.0, 1.0 };
            break;
        }
        if (tmp.lo >= kPiHi && pass == 0) {
            x = isub(tmp, Itv { kPiLo, kPiHi });
            negate = true;
            continue;
        }
        double l = tmp.lo, u = tmp.hi;
        if (u <= kPiLo) r = Itv { cos_dn(u), cos_up(l) };
        else if (u <= pi2.lo) r = Itv { -1.0, cos_up(smin(sub_dn(pi2.lo, u), l)) };
        else r = Itv { -1.0, 1.0 };
        break;
    }
    return negate ? ineg(r) : r;
}

__device__ __forceinline__ Itv isin(const Itv& x)
{
    return icos(isub(x, Itv { kPiLo / 2, kPiHi / 2 }));
}

// sinc of a point (sinc.cpp:36-47)
static __device__ __noinline__ Itv sinc_taylor(double xd)
{
    Itv x = pt(xd);
    if (fabs(xd) >= 1.220703125e-04) return idiv(isin(x), x);
    Itv x2 = imul(x, x);
    return iadd(1.0, imul(idiv(x2, 6.0), isub(idiv(x2, 20.0), 1.0)));
}

// sinc over a non-negative interval (sinc.cpp:49-101; the input is a norm)
static __device__ __noinline__ Itv isinc_nonneg(const Itv& x)
{
    const double kMono = 4.4934094579;
    Itv y = iempty();
    Itv x_gt = x;
    if (x.lo <= kMono) {
        Itv x_mono = x;
        if (x_mono.hi > kMono) {
            x_mono = Itv { x_mono.lo, kMono };
            x_gt = Itv { kMono, x.hi };
        } else {
            x_gt = iempty();
        }
        y = Itv { smax(sinc_taylor(x_mono.hi).lo, -0.271724), smin(sinc_taylor(x_mono.lo).hi, 1.0) };
    }
    if (!is_empty(x_gt)) y = ihull(y, idiv(isin(x_gt), x_gt));
    return y;
}

__device__ __forceinline__ Itv isinc_norm(const Itv r[3])
{
    Itv a0 = iabs(r[0]), a1 = iabs(r[1]), a2 = iabs(r[2]);
    Itv d = iadd(iadd(imul(a0, a0), imul(a1, a1)), imul(a2, a2));
    return isinc_nonneg(isqrt(d));
}

// interval rotation matrix (pose.tpp:203-218), row-major
static __device__ __noinline__ void irotation(const Itv r[3], Itv R[9])
{
    Itv sa = isinc_norm(r);
    Itv rh[3];
#pragma unroll
    for (int k = 0; k < 3; k++) rh[k] = Itv { div_dn(r[k].lo, 2.0), div_up(r[k].hi, 2.0) };
    Itv sh = isinc_norm(rh);
    const Itv z { 0.0, 0.0 };
    const Itv K[9] = { z, ineg(r[2]), r[1], r[2], z, ineg(r[0]), ineg(r[1]), r[0], z };
    Itv c = imul(imul(0.5, sh), sh);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            Itv k2 = iadd(imul(K[3 * i], K[j]),
                          iadd(imul(K[3 * i + 1], K[3 + j]), imul(K[3 * i + 2], K[6 + j])));
            Itv v = iadd(imul(sa, K[3 * i + j]), imul(c, k2));
            R[3 * i + j] = i == j ? iadd(v, pt(1.0)) : v;
        }
}

// world vertex over intervals: ((v0 R_j0 + v1 R_j1) + v2 R_j2) + p_j
__device__ __forceinline__ void iworld_vertex(const Itv R[9], const Itv p[3], const double v[3],
                                              Itv out[3])
{
#pragma unroll
    for (int j = 0; j < 3; j++)
        out[j] = iadd(iadd(iadd(imul(v[0], R[3 * j]), imul(v[1], R[3 * j + 1])),
                           imul(v[2], R[3 * j + 2])),
                      p[j]);
}

} // namespace rigc
