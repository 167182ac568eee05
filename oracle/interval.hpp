// Interval arithmetic of the oracle (test infrastructure only).
//
// Restates the reference's interval type (src/interval/interval.hpp:25-30):
// Boost.Interval 1.86 operations (sign-case multiplication and division,
// checking_catch_nan empties, width/median/bisect/hull/overlap) over the
// FILibRounding wrapper (src/interval/filib_rounding.cpp:12-60), whose
// directed operations round to nearest and then step one ulp outward
// (filib q_pred/q_succ), with exact zeros kept exact:
//   add_down(x, y) = x == -y ? 0 : pred(x + y)
//   mul_down(x, y) = x == 0 || y == 0 ? 0 : pred(x * y), ...
// cos/sin follow Boost's range reduction (fmod by an enclosure of 2*pi, then
// monotone pieces); the point evaluation is the deterministic det_cos of
// trig.hpp widened by its error bound, not filib's q_cos (parity with filib's
// last bits is not pinned).
#pragma once

#include <cmath>
#include <limits>

#include "trig.hpp"

namespace orc {

inline double pred(double x) { return std::nextafter(x, -INFINITY); }
inline double succ(double x) { return std::nextafter(x, INFINITY); }

inline double add_down(double x, double y) { return x == -y ? 0.0 : pred(x + y); }
inline double add_up(double x, double y) { return x == -y ? 0.0 : succ(x + y); }
inline double sub_down(double x, double y) { return x == y ? 0.0 : pred(x - y); }
inline double sub_up(double x, double y) { return x == y ? 0.0 : succ(x - y); }
inline double mul_down(double x, double y) { return (x == 0 || y == 0) ? 0.0 : pred(x * y); }
inline double mul_up(double x, double y) { return (x == 0 || y == 0) ? 0.0 : succ(x * y); }
inline double div_down(double x, double y) { return x == 0 ? 0.0 : pred(x / y); }
inline double div_up(double x, double y) { return x == 0 ? 0.0 : succ(x / y); }
inline double sqrt_down(double x) { return x == 0 ? 0.0 : pred(std::sqrt(x)); }
inline double sqrt_up(double x) { return x == 0 ? 0.0 : succ(std::sqrt(x)); }

struct I {
    double lo, hi;
    I() : lo(0), hi(0) {}
    explicit I(double x) : lo(x), hi(x) {}
    I(double l, double u) : lo(l), hi(u) {}
    static I empty()
    {
        return I(std::numeric_limits<double>::quiet_NaN(),
                 std::numeric_limits<double>::quiet_NaN());
    }
    bool is_empty() const { return !(lo <= hi); }
};

inline bool is_neg(double x) { return x < 0; }
inline bool is_pos(double x) { return x > 0; }

inline I operator-(const I& x)
{
    if (x.is_empty()) return I::empty();
    return I(-x.hi, -x.lo);
}
inline I operator+(const I& x, const I& y)
{
    if (x.is_empty() || y.is_empty()) return I::empty();
    return I(add_down(x.lo, y.lo), add_up(x.hi, y.hi));
}
inline I operator+(double x, const I& y)
{
    if (y.is_empty()) return I::empty();
    return I(add_down(x, y.lo), add_up(x, y.hi));
}
inline I operator+(const I& x, double y) { return y + x; }
inline I operator-(const I& x, const I& y)
{
    if (x.is_empty() || y.is_empty()) return I::empty();
    return I(sub_down(x.lo, y.hi), sub_up(x.hi, y.lo));
}
inline I operator-(const I& x, double y)
{
    if (x.is_empty()) return I::empty();
    return I(sub_down(x.lo, y), sub_up(x.hi, y));
}
inline I operator-(double x, const I& y)
{
    if (y.is_empty()) return I::empty();
    return I(sub_down(x, y.hi), sub_up(x, y.lo));
}

// sign-case interval product
inline I operator*(const I& x, const I& y)
{
    if (x.is_empty() || y.is_empty()) return I::empty();
    const double xl = x.lo, xu = x.hi, yl = y.lo, yu = y.hi;
    if (is_neg(xl)) {
        if (is_pos(xu)) {
            if (is_neg(yl)) {
                if (is_pos(yu))  // M * M
                    return I(std::min(mul_down(xl, yu), mul_down(xu, yl)),
                             std::max(mul_up(xl, yl), mul_up(xu, yu)));
                return I(mul_down(xu, yl), mul_up(xl, yl));  // M * N
            }
            if (is_pos(yu)) return I(mul_down(xl, yu), mul_up(xu, yu));  // M * P
            return I(0.0, 0.0);  // M * Z
        }
        if (is_neg(yl)) {
            if (is_pos(yu)) return I(mul_down(xl, yu), mul_up(xl, yl));  // N * M
            return I(mul_down(xu, yu), mul_up(xl, yl));  // N * N
        }
        if (is_pos(yu)) return I(mul_down(xl, yu), mul_up(xu, yl));  // N * P
        return I(0.0, 0.0);  // N * Z
    }
    if (is_pos(xu)) {
        if (is_neg(yl)) {
            if (is_pos(yu)) return I(mul_down(xu, yl), mul_up(xu, yu));  // P * M
            return I(mul_down(xu, yl), mul_up(xl, yu));  // P * N
        }
        if (is_pos(yu)) return I(mul_down(xl, yl), mul_up(xu, yu));  // P * P
        return I(0.0, 0.0);  // P * Z
    }
    return I(0.0, 0.0);  // Z * ?
}

inline I operator*(double x, const I& y)
{
    if (y.is_empty()) return I::empty();
    if (is_neg(x)) return I(mul_down(x, y.hi), mul_up(x, y.lo));
    if (x == 0) return I(0.0, 0.0);
    return I(mul_down(x, y.lo), mul_up(x, y.hi));
}
inline I operator*(const I& x, double y) { return y * x; }

inline I div_non_zero(const I& x, const I& y)
{
    const double xl = x.lo, xu = x.hi, yl = y.lo, yu = y.hi;
    if (is_neg(xu)) {
        if (is_neg(yu)) return I(div_down(xu, yl), div_up(xl, yu));
        return I(div_down(xl, yl), div_up(xu, yu));
    }
    if (is_neg(xl)) {
        if (is_neg(yu)) return I(div_down(xu, yu), div_up(xl, yu));
        return I(div_down(xl, yl), div_up(xu, yl));
    }
    if (is_neg(yu)) return I(div_down(xu, yu), div_up(xl, yl));
    return I(div_down(xl, yu), div_up(xu, yl));
}

inline I operator/(const I& x, const I& y)
{
    if (x.is_empty() || y.is_empty()) return I::empty();
    if (y.lo <= 0 && y.hi >= 0) {
        // divisor contains zero: only whole-line or half-line results; the
        // rigid CCD path never divides by such an interval
        if (x.lo == 0 && x.hi == 0) return I(0.0, 0.0);
        return I(-INFINITY, INFINITY);
    }
    return div_non_zero(x, y);
}
inline I operator/(const I& x, double y)
{
    if (x.is_empty() || y == 0) return I::empty();
    if (is_neg(y)) return I(div_down(x.hi, y), div_up(x.lo, y));
    return I(div_down(x.lo, y), div_up(x.hi, y));
}

inline I isqrt(const I& x)
{
    if (x.is_empty() || is_neg(x.hi)) return I::empty();
    double l = !is_pos(x.lo) ? 0.0 : sqrt_down(x.lo);
    return I(l, sqrt_up(x.hi));
}

inline I iabs(const I& x)
{
    if (x.is_empty()) return I::empty();
    if (!is_neg(x.lo)) return x;
    if (!is_pos(x.hi)) return -x;
    return I(0.0, std::max(-x.lo, x.hi));
}

inline I hull(const I& x, const I& y)
{
    if (x.is_empty()) return y;
    if (y.is_empty()) return x;
    return I(std::min(x.lo, y.lo), std::max(x.hi, y.hi));
}

inline bool zero_in(const I& x) { return !x.is_empty() && x.lo <= 0 && x.hi >= 0; }
inline bool overlap(const I& x, const I& y)
{
    return !x.is_empty() && !y.is_empty() && x.lo <= y.hi && y.lo <= x.hi;
}
inline double width(const I& x) { return x.is_empty() ? 0.0 : sub_up(x.hi, x.lo); }
inline double median(const I& x) { return 0.5 * (x.lo + x.hi); }

// ---------------------------------------------------------------------------
// cos / sin (Boost.Interval's structure over the cos_down/cos_up of the
// rounding policy, filib_rounding.cpp:94-134)

constexpr double kPiLo = 3.141592653589793116;   // 0x1.921fb54442d18p+1
constexpr double kPiHi = 3.141592653589793560;   // 0x1.921fb54442d19p+1

inline double cos_down(double x)
{
    if (std::fabs(x) > kTrigMaxArg) return -1.0;
    double c = det_cos(x);
    double r = pred(c - trig_err(c));
    return r < -1.0 ? -1.0 : (r > 1.0 ? 1.0 : r);
}
inline double cos_up(double x)
{
    if (std::fabs(x) > kTrigMaxArg) return 1.0;
    double c = det_cos(x);
    double r = succ(c + trig_err(c));
    return r < -1.0 ? -1.0 : (r > 1.0 ? 1.0 : r);
}

inline I pi_interval() { return I(kPiLo, kPiHi); }
inline I pi_half_interval() { return I(kPiLo / 2, kPiHi / 2); }
inline I pi_twice_interval() { return I(kPiLo * 2, kPiHi * 2); }

inline I ifmod(const I& x, const I& y)
{
    if (x.is_empty() || y.is_empty()) return I::empty();
    double yb = is_neg(x.lo) ? y.lo : y.hi;
    double n = std::floor(div_down(x.lo, yb));
    return x - n * y;
}

inline I icos(const I& x)
{
    if (x.is_empty()) return I::empty();
    const I pi2 = pi_twice_interval();
    I tmp = ifmod(x, pi2);
    if (width(tmp) >= pi2.lo) return I(-1.0, 1.0);
    if (tmp.lo >= kPiHi) return -icos(tmp - pi_interval());
    double l = tmp.lo, u = tmp.hi;
    if (u <= kPiLo) return I(cos_down(u), cos_up(l));
    if (u <= pi2.lo) return I(-1.0, cos_up(std::min(sub_down(pi2.lo, u), l)));
    return I(-1.0, 1.0);
}

inline I isin(const I& x)
{
    if (x.is_empty()) return I::empty();
    return icos(x - pi_half_interval());
}

} // namespace orc
