// sincos.hpp -- TEST INFRASTRUCTURE (oracle).  Deterministic sine/cosine used
// for the rotation update of RigidBody.expRodrigues (RigidBody.java:382-401).
//
// Java's Math.sin/cos are only specified to 1 ulp, so no libm reproduces them
// bit for bit.  The oracle and the CUDA integrator therefore both evaluate
// the same published method, written out here with a fixed operation order:
//   * Cody-Waite argument reduction by pi/2 with a two-term constant
//     (W. J. Cody and W. Waite, "Software Manual for the Elementary
//     Functions", 1980): k = nearest integer to x*2/pi,
//     r = (x - k*C1) - k*C2 with C1 = pi/2 rounded to 33 significant bits
//     (so k*C1 is exact for k < 2^20) and C2 = pi/2 - C1;
//   * Taylor series of sin and cos on |r| <= pi/4 (coefficients (-1)^n/n!,
//     sin to r^17, cos to r^18), Horner in r^2.
// Valid for 0 <= x < 2^20; the integrator only feeds |omega| dt >= 0.
#pragma once
#include <cmath>

namespace orc {

inline void det_sincos(double x, double* s_out, double* c_out) {
    const double TWO_OVER_PI = 0.6366197723675814;   // 2/pi
    const double C1 = 1.5707963267341256;             // pi/2, 33 significant bits
    const double C2 = 6.077100506506192e-11;          // pi/2 - C1
    double k = std::floor(x * TWO_OVER_PI + 0.5);
    double r = (x - k * C1) - k * C2;
    double z = r * r;
    // sin(r) = r + r*z*(S1 + z*(S2 + ...))
    double ps = 2.8114572543455206e-15;                //  1/17!
    ps = -7.647163731819816e-13 + z * ps;              // -1/15!
    ps = 1.6059043836821613e-10 + z * ps;              //  1/13!
    ps = -2.505210838544172e-08 + z * ps;              // -1/11!
    ps = 2.7557319223985893e-06 + z * ps;              //  1/9!
    ps = -1.984126984126984e-04 + z * ps;              // -1/7!
    ps = 8.333333333333333e-03 + z * ps;               //  1/5!
    ps = -1.6666666666666666e-01 + z * ps;             // -1/3!
    double sr = r + (r * z) * ps;
    // cos(r) = 1 - z/2 + z*z*(C4 + z*(C6 + ...))
    double pc = -1.5619206968586225e-16;               // -1/18!
    pc = 4.779477332387385e-14 + z * pc;               //  1/16!
    pc = -1.1470745597729725e-11 + z * pc;             // -1/14!
    pc = 2.08767569878681e-09 + z * pc;                //  1/12!
    pc = -2.755731922398589e-07 + z * pc;              // -1/10!
    pc = 2.48015873015873e-05 + z * pc;                //  1/8!
    pc = -1.388888888888889e-03 + z * pc;              // -1/6!
    pc = 4.1666666666666664e-02 + z * pc;              //  1/4!
    double cr = (1.0 - 0.5 * z) + (z * z) * pc;
    long q = (long)k & 3;
    if (q == 0) { *s_out = sr; *c_out = cr; }
    else if (q == 1) { *s_out = cr; *c_out = -sr; }
    else if (q == 2) { *s_out = -sr; *c_out = -cr; }
    else { *s_out = -cr; *c_out = sr; }
}

}  // namespace orc
