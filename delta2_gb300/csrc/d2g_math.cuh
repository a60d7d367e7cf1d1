// Portable transcendental functions shared by host set-up code and the
// sm_103a kernels.  The reference's quaternion exponential
// (common/basic_utils.cpp:36-44) calls std::sin/std::cos, its slerp
// (model/state.cpp:55-70, through Eigen) calls acos/sin, and the edge-edge
// Newton step (collision_detection/continuous_comparison.h:631) calls
// pow(S, 3/2).  CUDA's and glibc's versions of these differ in the last bit
// for some arguments, so this library evaluates them with its own code:
//
//   sin, cos : Cody & Waite (1980) reduction x = k*pi/2 + r with pi/2 split
//              into three parts (33-bit head), then the Maclaurin series of
//              sin(r) through r^19 and cos(r) through r^18 by Horner's rule,
//              each step one fused multiply-add.
//   acos     : pi/2 - asin(x) for x <= 1/2, else 2*asin(sqrt((1-x)/2)); asin
//              by its Maclaurin series (30 terms) on [0, 1/2].
//   log      : frexp reduction and log(m) = 2*atanh((m-1)/(m+1)) (set-up only).
//   x^(3/2)  : x*sqrt(x).
//   x / y    : with y's reciprocal known (m_div_recip), Markstein's
//              correction of x * (1 / y); the correctly rounded quotient,
//              the same bits as the division.
//
// Every kernel translation unit is compiled with -fmad=false and every host
// unit with -ffp-contract=off, so each operation is rounded on its own (the
// fused multiply-adds written out as such are single IEEE operations) and the
// results are the same bits on the GPU, on x86-64 and on Arm.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define D2G_HD __host__ __device__ __forceinline__
#else
#define D2G_HD inline
#endif

namespace d2g {

// x y + z rounded once (the IEEE fused multiply-add, the same on every
// machine).
D2G_HD double m_fma(double x, double y, double z) {
#ifdef __CUDA_ARCH__
    return fma(x, y, z);
#else
    return std::fma(x, y, z);
#endif
}

// Horner coefficients, highest order first, of sin(r) = r + r z S(z) and
// cos(r) = 1 + z C(z), z = r^2.
D2G_HD double m_sincos_coef(int i, bool cosine) {
    switch (i) {
        case 0: return cosine ? -1.5619206968586225e-16 : -8.22063524662433e-18;
        case 1: return cosine ? 4.779477332387385e-14 : 2.8114572543455206e-15;
        case 2: return cosine ? -1.1470745597729725e-11 : -7.647163731819816e-13;
        case 3: return cosine ? 2.08767569878681e-09 : 1.6059043836821613e-10;
        case 4: return cosine ? -2.755731922398589e-07 : -2.505210838544172e-08;
        case 5: return cosine ? 2.48015873015873e-05 : 2.7557319223985893e-06;
        case 6: return cosine ? -0.001388888888888889 : -0.0001984126984126984;
        case 7: return cosine ? 0.041666666666666664 : 0.008333333333333333;
        default: return cosine ? -0.5 : -0.16666666666666666;
    }
}

// The sine (cosine = false) or cosine series on the reduced argument r.  One
// instruction stream for both: lanes of a warp may evaluate different ones.
D2G_HD double m_kernel_sincos(double r, bool cosine) {
    const double z = r * r;
    double p = m_sincos_coef(0, cosine);
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
    for (int i = 1; i < 9; i++) p = m_fma(z, p, m_sincos_coef(i, cosine));  // Horner steps as fused multiply-adds
    const double a = cosine ? z : r * z;
    const double b = cosine ? 1.0 : r;
    return m_fma(a, p, b);  // sin: r + (r z) S, cos: 1 + z C
}

D2G_HD double m_kernel_sin(double r) { return m_kernel_sincos(r, false); }

D2G_HD double m_kernel_cos(double r) { return m_kernel_sincos(r, true); }

// x = k*pi/2 + r, |r| <= pi/4 (for |x| <= pi/4 no reduction).
D2G_HD void m_reduce(double x, double& r, int& q) {
    const double ax = x < 0.0 ? -x : x;
    if (ax <= 0.7853981633974483) {
        r = x;
        q = 0;
        return;
    }
#ifdef __CUDA_ARCH__
    const double k = rint(x * 0.6366197723675814);
#else
    const double k = std::nearbyint(x * 0.6366197723675814);
#endif
    r = ((x - k * 1.5707963267341256) - k * 6.077100506506192e-11) - k * 3.5215598651832e-27;
    const long long ki = (long long)k;
    q = (int)(ki & 3LL);
}

D2G_HD double m_sin(double x) {
    const double ax = x < 0.0 ? -x : x;
    if (!(ax < 1e9)) return x - x;
    double r;
    int q;
    m_reduce(x, r, q);
    if (q == 0) return m_kernel_sin(r);
    if (q == 1) return m_kernel_cos(r);
    if (q == 2) return -m_kernel_sin(r);
    return -m_kernel_cos(r);
}

D2G_HD double m_cos(double x) {
    const double ax = x < 0.0 ? -x : x;
    if (!(ax < 1e9)) return x - x;
    double r;
    int q;
    m_reduce(x, r, q);
    if (q == 0) return m_kernel_cos(r);
    if (q == 1) return -m_kernel_sin(r);
    if (q == 2) return -m_kernel_cos(r);
    return m_kernel_sin(r);
}

D2G_HD double m_series_asin(double y) {
    const double z = y * y;
    double p = 0.0017680811205154183;
    p = 0.0018622264064031275 + z * p;
    p = 0.0019650336162772837 + z * p;
    p = 0.0020776610325181676 + z * p;
    p = 0.0022014739737101384 + z * p;
    p = 0.002338091892111975 + z * p;
    p = 0.0024894486782468836 + z * p;
    p = 0.00265787063820729 + z * p;
    p = 0.002846178401108942 + z * p;
    p = 0.0030578216492580306 + z * p;
    p = 0.003297059503473485 + z * p;
    p = 0.0035692053938259347 + z * p;
    p = 0.003880964558837669 + z * p;
    p = 0.004240907093679363 + z * p;
    p = 0.004660143486915096 + z * p;
    p = 0.005153309682319905 + z * p;
    p = 0.005740037670841924 + z * p;
    p = 0.006447210311889649 + z * p;
    p = 0.0073125258735988454 + z * p;
    p = 0.008390335809616815 + z * p;
    p = 0.009761609529194078 + z * p;
    p = 0.011551800896139705 + z * p;
    p = 0.01396484375 + z * p;
    p = 0.017352764423076924 + z * p;
    p = 0.022372159090909092 + z * p;
    p = 0.030381944444444444 + z * p;
    p = 0.044642857142857144 + z * p;
    p = 0.075 + z * p;
    p = 0.16666666666666666 + z * p;
    p = 1.0 + z * p;
    return y * p;
}

// acos on [0, 1].
D2G_HD double m_acos(double x) {
    if (x <= 0.5) return 1.5707963267948966 - m_series_asin(x);
    return 2.0 * m_series_asin(sqrt((1.0 - x) / 2.0));
}

D2G_HD double m_pow15(double x) { return x * sqrt(x); }

// Host-only natural logarithm for scene generation.
inline double m_log(double x) {
    int e;
    double m = std::frexp(x, &e);
    if (m < 0.7071067811865476) {
        m = m * 2.0;
        e = e - 1;
    }
    const double s = (m - 1.0) / (m + 1.0);
    const double z = s * s;
    double p = 1.0 / 41.0;
    for (int n = 19; n >= 1; n--) p = 1.0 / (2.0 * n + 1.0) + z * p;
    const double ls = 2.0 * (s + (s * z) * p);
    return ls + (double)e * 0.6931471805599453;
}

// The biased exponent field of v (0 for zeros and subnormals, 2047 for
// infinities and NaNs).
D2G_HD uint64_t m_bits(double v) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(v);
#else
    uint64_t b;
    std::memcpy(&b, &v, sizeof b);
    return b;
#endif
}

D2G_HD int m_exp_field(double v) { return (int)((m_bits(v) >> 52) & 0x7ff); }

D2G_HD bool m_is_zero(double v) { return (m_bits(v) << 1) == 0; }

// x / y rounded to nearest, given ry = 1 / y rounded to nearest (P. W.
// Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Dev. 34(1), 1990): q = RN(x ry) lies
// within one ulp of x / y, the residual r = x - q y is exact when formed by
// one fused multiply-add, and RN(q + r ry) is the correctly rounded
// quotient.  The argument needs q and y well inside the exponent range (so
// r neither underflows nor overflows): for others it divides.  A zero x
// gives q, which carries the quotient's sign.  Three FP64 operations in
// place of a division when a divisor repeats (masses, time steps, counts).
D2G_HD double m_div_recip(double x, double y, double ry) {
    const double q = x * ry;
    const int ey = m_exp_field(y);
    if (ey < 573 || ey > 1473) return x / y;  // |y| outside [2^-450, 2^451)
    if (m_is_zero(x)) return q;
    const int eq = m_exp_field(q);
    if (eq < 573 || eq > 1473) return x / y;
#ifdef __CUDA_ARCH__
    const double r = fma(-q, y, x);
    return fma(r, ry, q);
#else
    const double r = std::fma(-q, y, x);
    return std::fma(r, ry, q);
#endif
}

}  // namespace d2g
