// Oracle (test infrastructure only): portable transcendental functions.
//
// The reference calls std::sin / std::cos (common/basic_utils.cpp:36-44,
// quaternion exponential), std::acos / std::sin inside Eigen's slerp
// (model/state.cpp:55-70) and std::pow(S, 3/2) in the edge-edge Newton step
// (collision_detection/continuous_comparison.h:631).  libm and CUDA disagree
// in the last bit for some arguments, which would make a bit-exact comparison
// between this oracle and the GPU kernels impossible.  Both sides therefore
// evaluate these functions with the SAME published methods, in the same
// operation order, with no fused multiply-add but the ones written out:
//   * sin / cos : Cody & Waite (1980) additive range reduction by pi/2 with a
//                 three-part split of pi/2, then the Maclaurin series of sin
//                 and cos on [-pi/4, pi/4] (terms through r^19 / r^18),
//                 evaluated by Horner's rule, each step (and the final
//                 r + (r z) p, 1 + z p) one fused multiply-add (std::fma,
//                 correctly rounded on every IEEE machine).
//   * asin / acos: Maclaurin series of asin on [0, 1/2] (30 terms); acos(x)
//                 = pi/2 - asin(x) for x <= 1/2 and 2 asin(sqrt((1-x)/2))
//                 otherwise.
//   * log      : frexp reduction to [sqrt(1/2), sqrt(2)) and the series
//                 log(m) = 2 atanh((m-1)/(m+1)) (used only by scene set-up).
// The constants are the Taylor coefficients (-1)^n/(2n+1)!, (-1)^n/(2n)!,
// (2n)!/(4^n (n!)^2 (2n+1)) and the digits of pi, rounded to double.
// Accuracy against libm is a few ulp; tests/test_oracle_math.py checks it.
#pragma once
#include <cmath>
#include <cstdint>

namespace d2o {

static const double kPio2Hi = 1.5707963267341256;     // pi/2, 33 significant bits
static const double kPio2Mid = 6.077100506506192e-11; // next bits of pi/2
static const double kPio2Lo = 3.5215598651832e-27;    // remaining bits
static const double kTwoOverPi = 0.6366197723675814;
static const double kPi = 3.141592653589793;
static const double kPio2 = 1.5707963267948966;
static const double kLn2 = 0.6931471805599453;

// sin(r) on |r| <= pi/4: r + r*z*(S1 + z*(S2 + ... + z*S9)), z = r*r.
inline double kernel_sin(double r) {
    const double z = r * r;
    double p = -8.22063524662433e-18;
    p = std::fma(z, p, 2.8114572543455206e-15);
    p = std::fma(z, p, -7.647163731819816e-13);
    p = std::fma(z, p, 1.6059043836821613e-10);
    p = std::fma(z, p, -2.505210838544172e-08);
    p = std::fma(z, p, 2.7557319223985893e-06);
    p = std::fma(z, p, -0.0001984126984126984);
    p = std::fma(z, p, 0.008333333333333333);
    p = std::fma(z, p, -0.16666666666666666);
    return std::fma(r * z, p, r);
}

// cos(r) on |r| <= pi/4: 1 + z*(C1 + z*(C2 + ... + z*C9)).
inline double kernel_cos(double r) {
    const double z = r * r;
    double p = -1.5619206968586225e-16;
    p = std::fma(z, p, 4.779477332387385e-14);
    p = std::fma(z, p, -1.1470745597729725e-11);
    p = std::fma(z, p, 2.08767569878681e-09);
    p = std::fma(z, p, -2.755731922398589e-07);
    p = std::fma(z, p, 2.48015873015873e-05);
    p = std::fma(z, p, -0.001388888888888889);
    p = std::fma(z, p, 0.041666666666666664);
    p = std::fma(z, p, -0.5);
    return std::fma(z, p, 1.0);
}

// Reduce x to r in [-pi/4, pi/4] and quadrant q = k mod 4 (x = k*pi/2 + r).
inline void reduce_pio2(double x, double& r, int& q) {
    if (std::fabs(x) <= 0.7853981633974483) {
        r = x;
        q = 0;
        return;
    }
    const double k = std::nearbyint(x * kTwoOverPi);
    r = ((x - k * kPio2Hi) - k * kPio2Mid) - k * kPio2Lo;
    const long long ki = (long long)k;
    q = (int)(ki & 3LL);
}

inline double psin(double x) {
    if (!(std::fabs(x) < 1e9)) return x - x;  // inf/nan -> nan; huge args out of range
    double r;
    int q;
    reduce_pio2(x, r, q);
    switch (q) {
        case 0: return kernel_sin(r);
        case 1: return kernel_cos(r);
        case 2: return -kernel_sin(r);
        default: return -kernel_cos(r);
    }
}

inline double pcos(double x) {
    if (!(std::fabs(x) < 1e9)) return x - x;
    double r;
    int q;
    reduce_pio2(x, r, q);
    switch (q) {
        case 0: return kernel_cos(r);
        case 1: return -kernel_sin(r);
        case 2: return -kernel_cos(r);
        default: return kernel_sin(r);
    }
}

// asin(y) for 0 <= y <= 1/2.
inline double series_asin(double y) {
    static const double c[30] = {
        1.0, 0.16666666666666666, 0.075, 0.044642857142857144, 0.030381944444444444,
        0.022372159090909092, 0.017352764423076924, 0.01396484375, 0.011551800896139705,
        0.009761609529194078, 0.008390335809616815, 0.0073125258735988454,
        0.006447210311889649, 0.005740037670841924, 0.005153309682319905,
        0.004660143486915096, 0.004240907093679363, 0.003880964558837669,
        0.0035692053938259347, 0.003297059503473485, 0.0030578216492580306,
        0.002846178401108942, 0.00265787063820729, 0.0024894486782468836,
        0.002338091892111975, 0.0022014739737101384, 0.0020776610325181676,
        0.0019650336162772837, 0.0018622264064031275, 0.0017680811205154183};
    const double z = y * y;
    double p = c[29];
    for (int n = 28; n >= 0; n--) p = c[n] + z * p;
    return y * p;
}

// acos(x) for 0 <= x <= 1 (the only range Eigen's slerp uses).
inline double pacos(double x) {
    if (x <= 0.5) return kPio2 - series_asin(x);
    return 2.0 * series_asin(std::sqrt((1.0 - x) / 2.0));
}

// log(x) for finite x > 0 (scene generation only).
inline double plog(double x) {
    int e;
    double m = std::frexp(x, &e);  // x = m * 2^e, m in [0.5, 1)
    if (m < 0.7071067811865476) {
        m = m * 2.0;
        e = e - 1;
    }
    const double s = (m - 1.0) / (m + 1.0);
    const double z = s * s;
    // 2*atanh(s) = 2*(s + s^3/3 + s^5/5 + ...), |s| <= 0.1716
    double p = 1.0 / 41.0;
    for (int n = 19; n >= 1; n--) p = 1.0 / (2.0 * n + 1.0) + z * p;
    const double ls = 2.0 * (s + (s * z) * p);
    return ls + (double)e * kLn2;
}

// x^(3/2) written as x*sqrt(x) (replaces std::pow(S, 3.0/2.0)).
inline double pow15(double x) { return x * std::sqrt(x); }

}  // namespace d2o
