// Deterministic sin/cos for the oracle (test infrastructure only).
//
// Both the oracle and the CUDA path evaluate sin/cos with the same published
// method so rotation matrices agree to the bit: Cody-Waite reduction by pi/2
// with a three-part split of pi/2 (P1, P2 carry 33 significant bits, so k*P1
// and k*P2 are exact for |k| < 2^20), then the Taylor series of sin and cos
// (coefficients 1/n!) to degree 19/20 on |r| <= pi/4, evaluated by Horner's
// rule with separate multiply and add (no fused multiply-add).  The error of
// the result is below 2^-50 |y| + 2^-60 for |x| < 2^20; interval enclosures
// widen by that bound.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace orc {

constexpr double kTwoOverPi = 0.6366197723675814;
constexpr double kP1 = 1.5707963267341256;        // 0x1.921fb544p+0
constexpr double kP2 = 6.077100506303966e-11;     // 0x1.0b4611a6p-34
constexpr double kP3 = 2.0222662487959506e-21;    // 0x1.3198a2e037073p-69
constexpr double kTrigMaxArg = 1048576.0;         // 2^20

inline double trig_reduce(double x, long long& k)
{
    double kd = std::nearbyint(x * kTwoOverPi);
    k = (long long)kd;
    double r = x - kd * kP1;
    r = r - kd * kP2;
    r = r - kd * kP3;
    return r;
}

// Taylor polynomials on the reduced argument
inline double sin_poly(double r)
{
    // sin r = r + r^3 S(r^2), S(z) = -1/3! + z/5! - z^2/7! + ... - z^8/19!
    double z = r * r;
    double s = -1.0 / 121645100408832000.0;         // -1/19!
    s = s * z;
    s = 1.0 / 355687428096000.0 + s;                // 1/17!
    s = s * z;
    s = -1.0 / 1307674368000.0 + s;                 // -1/15!
    s = s * z;
    s = 1.0 / 6227020800.0 + s;                     // 1/13!
    s = s * z;
    s = -1.0 / 39916800.0 + s;                      // -1/11!
    s = s * z;
    s = 1.0 / 362880.0 + s;                         // 1/9!
    s = s * z;
    s = -1.0 / 5040.0 + s;                          // -1/7!
    s = s * z;
    s = 1.0 / 120.0 + s;                            // 1/5!
    s = s * z;
    s = -1.0 / 6.0 + s;                             // -1/3!
    double r3 = r * z;
    return r + r3 * s;
}

inline double cos_poly(double r)
{
    double r2 = r * r;
    double p = 1.0 / 2432902008176640000.0;         // 1/20!
    p = p * r2;
    p = -1.0 / 6402373705728000.0 + p;              // -1/18!
    p = p * r2;
    p = 1.0 / 20922789888000.0 + p;                 // 1/16!
    p = p * r2;
    p = -1.0 / 87178291200.0 + p;                   // -1/14!
    p = p * r2;
    p = 1.0 / 479001600.0 + p;                      // 1/12!
    p = p * r2;
    p = -1.0 / 3628800.0 + p;                       // -1/10!
    p = p * r2;
    p = 1.0 / 40320.0 + p;                          // 1/8!
    p = p * r2;
    p = -1.0 / 720.0 + p;                           // -1/6!
    p = p * r2;
    p = 1.0 / 24.0 + p;                             // 1/4!
    p = p * r2;
    p = -0.5 + p;                                   // -1/2!
    p = p * r2;
    return 1.0 + p;
}

inline double det_sin(double x)
{
    long long k;
    double r = trig_reduce(x, k);
    switch (k & 3) {
    case 0: return sin_poly(r);
    case 1: return cos_poly(r);
    case 2: return -sin_poly(r);
    default: return -cos_poly(r);
    }
}

inline double det_cos(double x)
{
    long long k;
    double r = trig_reduce(x, k);
    switch (k & 3) {
    case 0: return cos_poly(r);
    case 1: return -sin_poly(r);
    case 2: return -cos_poly(r);
    default: return sin_poly(r);
    }
}

// error bound used to widen enclosures: 2^-50 |y| + 2^-60
inline double trig_err(double y)
{
    return std::fabs(y) * 8.881784197001252e-16 + 8.673617379884035e-19;
}

} // namespace orc
