// Bit-reproducible FP64 elementary functions, the Philox-4x32-10 counter-based
// generator and the Box-Muller normal transform, compiled identically for the
// host and for sm_103a.
//
// Why this file exists: the replay mode must reproduce, bit for bit on the
// GPU, the arithmetic of the CPU restatement of the reference's
// Feynman-Kac path loop (Integrators/FKACIntegrator.hpp:46-57, 168-222) and
// of its RBF exit weights (Meshes/stencil.cpp:244-307, BVPs/BVP.hpp:84-87).
// libm and the CUDA math library differ in the last ulp of exp/log/sin/cos,
// and the RBF interpolation matrices have condition numbers near 1e10, so a
// one-ulp difference would already show at 1e-7 relative in G.  Every
// function below uses only IEEE-754 operations that are correctly rounded on
// both sides (+, -, *, /, sqrt, floor) and must be compiled without FMA
// contraction (-ffp-contract=off on the host, -fmad=false on the device).
//
// Methods (all standard, restated from the mathematics):
//   exp : Cody-Waite reduction x = k ln2 + r with a two-part ln2, then the
//         Taylor series of e^r to degree 13 (|r| <= ln2/2, truncation < 1e-17),
//         scaled by 2^k built from its exponent bits.
//   log : x = m 2^e with m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(f),
//         f = (m-1)/(m+1), atanh by its odd power series to f^25.
//   sin/cos : Cody-Waite reduction by pi/2 with a three-part pi/2 (exact
//         products for |k| < 2^20), Taylor series on [-pi/4, pi/4] to degree
//         17/16, quadrant selection.
// The split constants were derived with 60-digit decimal arithmetic: the high
// parts are ln2 (pi/2) truncated to 32 (33) significant bits, so k*HI is exact.
//
// Philox-4x32-10: J. K. Salmon, M. A. Moraes, R. O. Dror, D. E. Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11.  Multipliers and
// Weyl key increments are the published ones.
#pragma once
#include <stdint.h>
#include <string.h>
#include <math.h>

#if defined(__CUDACC__)
#define PDDS_HD __host__ __device__ __forceinline__
#else
#define PDDS_HD inline
#endif

namespace pdds {

namespace pm {  // portable math

static constexpr double LN2_HI = 0.6931471803691238;        // 0x1.62e42fee00000p-1
static constexpr double LN2_LO = 1.9082149292705877e-10;    // ln2 - LN2_HI
static constexpr double INV_LN2 = 1.4426950408889634;
static constexpr double PIO2_1 = 1.5707963267341256;        // 0x1.921fb54400000p+0
static constexpr double PIO2_2 = 6.077100506303966e-11;     // 0x1.0b4611a600000p-34
static constexpr double PIO2_3 = 2.0222662487959506e-21;
static constexpr double TWO_OVER_PI = 0.6366197723675814;
static constexpr double PI = 3.141592653589793;
static constexpr double TWO_PI = 6.283185307179586;
// 1.5 * 2^52: adding and subtracting it rounds a double of magnitude < 2^51
// to the nearest integer (ties to even) with two correctly rounded operations.
static constexpr double ROUND_MAGIC = 6755399441055744.0;

PDDS_HD double bits_to_double(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, sizeof d);
  return d;
#endif
}
PDDS_HD uint64_t double_to_bits(double d) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t b;
  memcpy(&b, &d, sizeof b);
  return b;
#endif
}
// 2^k for -1022 <= k <= 1023, exact.
PDDS_HD double pow2i(int k) { return bits_to_double((uint64_t)(k + 1023) << 52); }

PDDS_HD double round_nearest(double x) { return (x + ROUND_MAGIC) - ROUND_MAGIC; }

PDDS_HD double exp(double x) {
  if (x != x) return x;
  if (x > 709.782712893384) return bits_to_double(0x7ff0000000000000ULL);
  if (x < -745.1332191019412) return 0.0;
  const double kd = round_nearest(x * INV_LN2);
  const int k = (int)kd;
  const double r = (x - kd * LN2_HI) - kd * LN2_LO;
  // Taylor coefficients 1/n!, n = 13 .. 2, Horner form.
  double p = 1.6059043836821613e-10;            // 1/13!
  p = p * r + 2.08767569878681e-09;             // 1/12!
  p = p * r + 2.505210838544172e-08;            // 1/11!
  p = p * r + 2.755731922398589e-07;            // 1/10!
  p = p * r + 2.7557319223985893e-06;           // 1/9!
  p = p * r + 2.48015873015873e-05;             // 1/8!
  p = p * r + 0.0001984126984126984;            // 1/7!
  p = p * r + 0.001388888888888889;             // 1/6!
  p = p * r + 0.008333333333333333;             // 1/5!
  p = p * r + 0.041666666666666664;             // 1/4!
  p = p * r + 0.16666666666666666;              // 1/3!
  p = p * r + 0.5;                              // 1/2!
  p = p * r;
  p = p * r + r;                                // r + r^2/2 + ...
  const double e = 1.0 + p;
  if (k >= -1021 && k <= 1023) return e * pow2i(k);
  // Very small results: scale in two exact-exponent steps.
  return (e * pow2i(k + 200)) * pow2i(-200);
}

PDDS_HD double log(double x) {
  if (x != x) return x;
  if (x <= 0.0) return (x == 0.0) ? -bits_to_double(0x7ff0000000000000ULL)
                                  : bits_to_double(0x7ff8000000000000ULL);
  if (x == bits_to_double(0x7ff0000000000000ULL)) return x;
  int bias = 0;
  if (x < 2.2250738585072014e-308) {  // subnormal: scale by 2^54 first
    x = x * 18014398509481984.0;
    bias = -54;
  }
  uint64_t b = double_to_bits(x);
  int e = (int)((b >> 52) & 0x7ff) - 1023 + bias;
  double m = bits_to_double((b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);
  if (m > 1.4142135623730951) {
    m = m * 0.5;
    e += 1;
  }
  const double f = (m - 1.0) / (m + 1.0);
  const double s = f * f;
  // atanh(f)/f = sum s^k / (2k+1), k = 0 .. 12
  double p = 0.04;                 // 1/25
  p = p * s + 0.043478260869565216;  // 1/23
  p = p * s + 0.047619047619047616;  // 1/21
  p = p * s + 0.05263157894736842;   // 1/19
  p = p * s + 0.058823529411764705;  // 1/17
  p = p * s + 0.06666666666666667;   // 1/15
  p = p * s + 0.07692307692307693;   // 1/13
  p = p * s + 0.09090909090909091;   // 1/11
  p = p * s + 0.1111111111111111;    // 1/9
  p = p * s + 0.14285714285714285;   // 1/7
  p = p * s + 0.2;                   // 1/5
  p = p * s + 0.3333333333333333;    // 1/3
  const double lm = 2.0 * f + (2.0 * f) * (s * p);
  const double ed = (double)e;
  return (ed * LN2_HI) + (lm + ed * LN2_LO);
}

// sin and cos of r for |r| <= pi/4 (Taylor, Horner in r^2).
PDDS_HD double sin_kernel(double r) {
  const double s = r * r;
  double p = 2.8114572543455206e-15;    // 1/17!
  p = p * s - 7.647163731819816e-13;    // -1/15!
  p = p * s + 1.6059043836821613e-10;   // 1/13!
  p = p * s - 2.505210838544172e-08;    // -1/11!
  p = p * s + 2.7557319223985893e-06;   // 1/9!
  p = p * s - 0.0001984126984126984;    // -1/7!
  p = p * s + 0.008333333333333333;     // 1/5!
  p = p * s - 0.16666666666666666;      // -1/3!
  return r + r * (s * p);
}
PDDS_HD double cos_kernel(double r) {
  const double s = r * r;
  double p = 4.779477332387385e-14;     // 1/16!
  p = p * s - 1.1470745597729725e-11;   // -1/14!
  p = p * s + 2.08767569878681e-09;     // 1/12!
  p = p * s - 2.755731922398589e-07;    // -1/10!
  p = p * s + 2.48015873015873e-05;     // 1/8!
  p = p * s - 0.001388888888888889;     // -1/6!
  p = p * s + 0.041666666666666664;     // 1/4!
  p = p * s - 0.5;                      // -1/2!
  return 1.0 + s * p;
}
// Simultaneous sin and cos; valid for |x| < 2^20 * pi/2.
PDDS_HD void sincos(double x, double* sn, double* cs) {
  const double kd = round_nearest(x * TWO_OVER_PI);
  const double r = ((x - kd * PIO2_1) - kd * PIO2_2) - kd * PIO2_3;
  const double s = sin_kernel(r), c = cos_kernel(r);
  const int q = ((int)kd) & 3;
  if (q == 0) { *sn = s;  *cs = c; }
  else if (q == 1) { *sn = c;  *cs = -s; }
  else if (q == 2) { *sn = -s; *cs = -c; }
  else { *sn = -c; *cs = s; }
}
PDDS_HD double sin(double x) { double s, c; sincos(x, &s, &c); return s; }
PDDS_HD double cos(double x) { double s, c; sincos(x, &s, &c); return c; }

}  // namespace pm

// ---------------------------------------------------------------- Philox
struct u32x4 { uint32_t v[4]; };

PDDS_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
#endif
}

PDDS_HD u32x4 philox4x32_10(u32x4 ctr, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#if defined(__CUDACC__)
#pragma unroll
#endif
  for (int round = 0; round < 10; ++round) {
    const uint32_t hi0 = mulhi32(M0, ctr.v[0]), lo0 = M0 * ctr.v[0];
    const uint32_t hi1 = mulhi32(M1, ctr.v[2]), lo1 = M1 * ctr.v[2];
    u32x4 n;
    n.v[0] = hi1 ^ ctr.v[1] ^ k0;
    n.v[1] = lo1;
    n.v[2] = hi0 ^ ctr.v[3] ^ k1;
    n.v[3] = lo0;
    ctr = n;
    k0 += W0;
    k1 += W1;
  }
  return ctr;
}

// Counter layout shared by every mode: one Philox call yields the four
// uniforms of two consecutive Euler-Maruyama steps of one path.
//   key     = (seed low word, seed high word)
//   counter = (step pair, path, knot, instance)
PDDS_HD u32x4 path_block(uint64_t seed, uint32_t instance, uint32_t knot,
                         uint32_t path, uint32_t step_pair) {
  u32x4 c;
  c.v[0] = step_pair;
  c.v[1] = path;
  c.v[2] = knot;
  c.v[3] = instance;
  return philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

// uint32 -> uniform in (0, 1), exact in double: (a + 1/2) 2^-32.
PDDS_HD double u01_fp64(uint32_t a) { return ((double)a + 0.5) * 2.3283064365386963e-10; }

// Box-Muller with the portable functions: the pair of standard normals of
// one step.  z0 = rho cos(2 pi u1), z1 = rho sin(2 pi u1), rho = sqrt(-2 ln u0).
PDDS_HD void box_muller_portable(uint32_t a, uint32_t b, double* z0, double* z1) {
  const double u0 = u01_fp64(a), u1 = u01_fp64(b);
  const double rho = sqrt(-2.0 * pm::log(u0));
  double s, c;
  pm::sincos(pm::TWO_PI * u1, &s, &c);
  *z0 = rho * c;
  *z1 = rho * s;
}

}  // namespace pdds
