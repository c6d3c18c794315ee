// Device-side view of the layout, problem functors and the rectangle exit
// geometry shared by the path kernels.
//
// Problems replace the reference's host function pointers (struct bvp,
// BVPs/BVP.hpp:89-137) and its __device__ function-pointer table (bvpdev,
// BVPs/BVP.cuh:44-77) by compiled functors selected with a template argument.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pdds_portable.h"

namespace pdds {

struct DevLayout {
  int K, S, D, P;
  double dom[4];  // domain rectangle {SW.x, SW.y, NE.x, NE.y}
  // 0: rectangular stencils {x0, y0, x1, y1}; 1: polar stencils
  // {rho0, phi0, rho1, phi1} on a disk of radius `radius` (arcs and rays)
  int geom;
  double radius;
  const double* sh_R;  // per shape: arc radius (RBF distance = chord), 0 for straight sides
  // knots
  const double* kx;
  const double* ky;
  const int* knot_stencil;
  const int64_t* row_ptr;
  // stencils
  const double* st_rect;     // [S][4]
  const int* st_side;        // [S][4] side id per N,S,E,W or -1
  const int* st_glob;        // [S][4]
  const int64_t* st_map_off; // [S]
  const int* map_pos;
  const unsigned char* map_owner;
  // sides
  const int* sd_n;
  const int* sd_orient;
  const int* sd_shape;
  const double* sd_c;
  const double* sd_origin;
  const int64_t* sd_knot_off;
  const int* side_knot;
  const double* side_px;
  const double* side_py;
  // shapes
  const int* sh_n;
  const double* sh_c;
  const double* sh_lo;
  const double* sh_delta;
  const int* sh_nbins;
  const int64_t* sh_tab_off;
  const int64_t* sh_ipsi_off;
  const int64_t* sh_t_off;
  const double* sh_t;
  const float* tab;
  const double* ipsi;
  // batch of independent instances (null for one layout): instance of each
  // knot, first knot of each instance, 8 problem parameters per instance
  const int* knot_inst;
  const int* inst_knot0;
  const double* inst_p;
  const double* inst_h;  // step per instance (0: the run's), batches only
  // Philox knot word of each knot (null: the knot's own index); set for
  // layouts built from caller stencils, whose knots carry the caller's ids
  const int* knot_rng;
};

// Philox knot word of knot k outside batches.
__device__ __forceinline__ uint32_t knot_word(const DevLayout& L, int k) {
  return L.knot_rng ? (uint32_t)L.knot_rng[k] : (uint32_t)k;
}

// Coefficient tables of the PK_LUT problem: node (i, j) of an nx x ny grid
// over [x0, x0 + (nx-1) dx] x [y0, y0 + (ny-1) dy] holds two float4,
// (sigma11, sigma22, b1, b2) and (c, f, du/dx, du/dy); g holds the
// boundary/solution values on the same grid.
struct LutDev {
  const float4* coef;
  const float* g;
  int nx, ny;
  double x0, y0, inv_dx, inv_dy;
  // the FP32 sampler's textures (fields 0-3 and 4-7, linear filtering,
  // clamped): tex_mode 1 cubic B-spline coefficients, 2 the node values
  // (bilinear); 0 no textures, it samples the nodes (Catmull-Rom)
  unsigned long long tex[2];
  int tex_mode;
};

struct ProblemDev {
  int kind;
  int use_cv;
  double p[8];
  LutDev lut;
};

enum { PK_POISSON_SINCOS = 0, PK_MONEGROS = 1, PK_HELMHOLTZ = 2, PK_VARCOEF = 3, PK_LUT = 4, PK_CIRCLE = 5, PK_ROBIN = 6 };
// The PK_LUT problem sampled from its textures: an instantiation of the FP32
// path kernel only (the problem's kind stays PK_LUT), so that neither form
// carries the other's sampler in its registers.
constexpr int PK_LUT_TEX = 7;
__host__ __device__ constexpr bool is_lut_kind(int k) { return k == PK_LUT || k == PK_LUT_TEX; }

// Problem parameters of the instance that owns knot k (batches), else P's own.
__device__ __forceinline__ void instance_params(const DevLayout& L, int k, ProblemDev& P, uint32_t& rng_inst,
                                                uint32_t& rng_knot) {
  if (L.knot_inst) {
    const int i = L.knot_inst[k];
#pragma unroll
    for (int q = 0; q < 8; q++) P.p[q] = L.inst_p[8 * i + q];
    rng_inst += (uint32_t)i;
    rng_knot = (uint32_t)(k - L.inst_knot0[i]);
  } else {
    rng_knot = knot_word(L, k);
  }
}

// ------------------------------------------------------------------ tables
// Bicubic Catmull-Rom (Keys cubic convolution, a = -1/2) interpolation,
// clamped to the table edges like the reference's clamp-addressed LUT
// texture (BVPs/LUT2.cuh:11-45).  The same arithmetic is used in FP32
// (MIXED), FP64 (FP64 mode) and, compiled without FMA contraction, in the
// replay kernels and the host restatement.
template <typename T>
__host__ __device__ __forceinline__ void cr_weights(T t, T* w) {
  const T t2 = t * t, t3 = t2 * t;
  w[0] = T(0.5) * ((T(2) * t2 - t3) - t);
  w[1] = T(0.5) * ((T(3) * t3 - T(5) * t2) + T(2));
  w[2] = T(0.5) * ((T(4) * t2 - T(3) * t3) + t);
  w[3] = T(0.5) * (t3 - t2);
}
template <typename T>
__host__ __device__ __forceinline__ void lut_coord(T x, T x0, T inv_dx, int n, int& i, T& t) {
  T g = (x - x0) * inv_dx;
  g = g < T(0) ? T(0) : g;
  g = g > T(n - 1) ? T(n - 1) : g;
  i = (int)floor(g);
  if (i > n - 2) i = n - 2;
  t = g - T(i);
}
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// One table node, its 8 fields as two float4 (32 bytes, 32-byte aligned: the
// table comes from cudaMalloc and nodes are 32 bytes apart), in one 256-bit
// read-only load: half the L1 requests of two 128-bit loads.
__device__ __forceinline__ void ldg_node(const float4* p, float4& a, float4& b) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(p));
}

// all eight fields (nf = 8) or the first four (nf = 4: sigma11, sigma22, b1, b2)
template <typename T, int NF>
__device__ __forceinline__ void lut_sample(const LutDev& L, T x, T y, T* out) {
  int ix, iy;
  T tx, ty, wx[4], wy[4];
  lut_coord<T>(x, (T)L.x0, (T)L.inv_dx, L.nx, ix, tx);
  lut_coord<T>(y, (T)L.y0, (T)L.inv_dy, L.ny, iy, ty);
  cr_weights<T>(tx, wx);
  cr_weights<T>(ty, wy);
#pragma unroll
  for (int f = 0; f < NF; f++) out[f] = T(0);
#pragma unroll
  for (int r = 0; r < 4; r++) {
    const float4* row = L.coef + (int64_t)2 * clampi(iy - 1 + r, 0, L.ny - 1) * L.nx;
    T acc[NF];
#pragma unroll
    for (int f = 0; f < NF; f++) acc[f] = T(0);
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const int xx = clampi(ix - 1 + c, 0, L.nx - 1);
      float4 a, b;
      if (NF == 8) ldg_node(row + 2 * xx, a, b);
      else a = __ldg(row + 2 * xx);
      acc[0] += wx[c] * (T)a.x; acc[1] += wx[c] * (T)a.y; acc[2] += wx[c] * (T)a.z; acc[3] += wx[c] * (T)a.w;
      if (NF == 8) {
        acc[NF > 4 ? 4 : 0] += wx[c] * (T)b.x; acc[NF > 5 ? 5 : 0] += wx[c] * (T)b.y;
        acc[NF > 6 ? 6 : 0] += wx[c] * (T)b.z; acc[NF > 7 ? 7 : 0] += wx[c] * (T)b.w;
      }
    }
#pragma unroll
    for (int f = 0; f < NF; f++) out[f] += wy[r] * acc[f];
  }
}
template <typename T>
__device__ __forceinline__ T lut_sample_g(const LutDev& L, T x, T y) {
  int ix, iy;
  T tx, ty, wx[4], wy[4];
  lut_coord<T>(x, (T)L.x0, (T)L.inv_dx, L.nx, ix, tx);
  lut_coord<T>(y, (T)L.y0, (T)L.inv_dy, L.ny, iy, ty);
  cr_weights<T>(tx, wx);
  cr_weights<T>(ty, wy);
  T out = T(0);
  for (int r = 0; r < 4; r++) {
    const float* row = L.g + (int64_t)clampi(iy - 1 + r, 0, L.ny - 1) * L.nx;
    T acc = T(0);
    for (int c = 0; c < 4; c++) acc += wx[c] * (T)__ldg(row + clampi(ix - 1 + c, 0, L.nx - 1));
    out += wy[r] * acc;
  }
  return out;
}

// Cubic B-spline interpolation of the tables from textures of their B-spline
// coefficients (prefiltered on the host so that the spline takes the table's
// values at the nodes), each axis' four weights folded into two linearly
// filtered fetches (Sigg and Hadwiger, "Fast third-order texture filtering",
// GPU Gems 2, ch. 20): four fetches per texture in place of sixteen node
// loads.  The filtering hardware blends with 8-bit fractions, an error of at
// most |c_{i+1} - c_i| / 512 per blend: O(node spacing x gradient) / 512 for
// smooth tables.
__device__ __forceinline__ void bspline_axis(float p, int n, float& c0, float& c1, float& g0, float& g1) {
  p = fminf(fmaxf(p, 0.f), (float)(n - 1));  // clamped to the table, as the node sampler clamps
  const float i = floorf(p);
  const float t = p - i, t2 = t * t, t3 = t2 * t;
  const float s = 1.f - t;
  const float w0 = (1.f / 6.f) * (s * s * s);
  const float w1 = (1.f / 6.f) * ((3.f * t3 - 6.f * t2) + 4.f);
  const float w3 = (1.f / 6.f) * t3;
  const float w2 = (1.f - w0) - (w1 + w3);
  g0 = w0 + w1;  // >= 1/6 for t in [0, 1]
  g1 = w2 + w3;  // >= 1/6
  // node k's texel centre is k + 0.5: blend nodes i-1, i and nodes i+1, i+2
  c0 = (i - 0.5f) + w1 / g0;
  c1 = (i + 1.5f) + w3 / g1;
}
template <int NF>
__device__ __forceinline__ void lut_sample_tex(const LutDev& L, float x, float y, float* out) {
  float cx0, cx1, gx0, gx1, cy0, cy1, gy0, gy1;
  bspline_axis((x - (float)L.x0) * (float)L.inv_dx, L.nx, cx0, cx1, gx0, gx1);
  bspline_axis((y - (float)L.y0) * (float)L.inv_dy, L.ny, cy0, cy1, gy0, gy1);
#pragma unroll
  for (int t = 0; t < (NF > 4 ? 2 : 1); t++) {
    const cudaTextureObject_t tx = (cudaTextureObject_t)L.tex[t];
    const float4 a = tex2D<float4>(tx, cx0, cy0), b = tex2D<float4>(tx, cx1, cy0);
    const float4 c = tex2D<float4>(tx, cx0, cy1), d = tex2D<float4>(tx, cx1, cy1);
    out[4 * t + 0] = gy0 * (gx0 * a.x + gx1 * b.x) + gy1 * (gx0 * c.x + gx1 * d.x);
    out[4 * t + 1] = gy0 * (gx0 * a.y + gx1 * b.y) + gy1 * (gx0 * c.y + gx1 * d.y);
    out[4 * t + 2] = gy0 * (gx0 * a.z + gx1 * b.z) + gy1 * (gx0 * c.z + gx1 * d.z);
    out[4 * t + 3] = gy0 * (gx0 * a.w + gx1 * b.w) + gy1 * (gx0 * c.w + gx1 * d.w);
  }
}
// Bilinear interpolation of the node values, one linearly filtered fetch per
// texture (8-bit blend fractions: an error of at most |f_{i+1} - f_i| / 512
// per axis on top of the O(node spacing^2) interpolation error).
template <int NF>
__device__ __forceinline__ void lut_sample_lin(const LutDev& L, float x, float y, float* out) {
  const float px = fminf(fmaxf((x - (float)L.x0) * (float)L.inv_dx, 0.f), (float)(L.nx - 1)) + 0.5f;
  const float py = fminf(fmaxf((y - (float)L.y0) * (float)L.inv_dy, 0.f), (float)(L.ny - 1)) + 0.5f;
#pragma unroll
  for (int t = 0; t < (NF > 4 ? 2 : 1); t++) {
    const float4 a = tex2D<float4>((cudaTextureObject_t)L.tex[t], px, py);
    out[4 * t + 0] = a.x;
    out[4 * t + 1] = a.y;
    out[4 * t + 2] = a.z;
    out[4 * t + 3] = a.w;
  }
}
// The FP32 (MIXED) sampler of a path-kernel instantiation: PK_LUT_TEX the
// problem's textures (cubic B-spline, or bilinear with tex_mode 2), PK_LUT
// the Catmull-Rom node sampler of the FP64 and replay forms.
template <int KIND, int NF>
__device__ __forceinline__ void lut_sample_f32(const LutDev& L, float x, float y, float* out) {
  if constexpr (KIND == PK_LUT_TEX) {
    if (L.tex_mode == 2) lut_sample_lin<NF>(L, x, y, out);
    else lut_sample_tex<NF>(L, x, y, out);
  } else {
    lut_sample<float, NF>(L, x, y, out);
  }
}

// Single-precision approximations (the PTX .approx forms, flush-to-zero) for
// the FP32 path, whose Euler step error is far above their rounding.
__device__ __forceinline__ float sqrt_approx(float x) {
  float y;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float lg2_approx(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

template <typename T>
struct Coef {
  T s00, s01, s10, s11;  // sigma, row-major
  T b0, b1;              // drift
  T c;                   // reaction
  T f;                   // source
  T g0, g1;              // gradient of u (control variate)
};

// ------------------------------------------------------------------ FP32
// Fast-intrinsic single precision (MIXED mode paths).
template <int KIND>
__device__ __forceinline__ void coef_f32(const ProblemDev& P, float x, float y, Coef<float>& k) {
  const float PI = 3.14159265358979f;
  if (is_lut_kind(KIND)) {
    float v[8];
    lut_sample_f32<KIND, 8>(P.lut, x, y, v);
    k.s00 = v[0]; k.s01 = 0.f; k.s10 = 0.f; k.s11 = v[1];
    k.b0 = v[2]; k.b1 = v[3]; k.c = v[4]; k.f = v[5]; k.g0 = v[6]; k.g1 = v[7];
  } else if (KIND == PK_POISSON_SINCOS) {
    // the x and y halves in paired FP32 instructions (same roundings)
    const float2 arg = __fmul2_rn(make_float2(PI, PI), make_float2(x, y));
    float sx, cx, sy, cy;
    __sincosf(arg.x, &sx, &cx);
    __sincosf(arg.y, &sy, &cy);
    k.s00 = 1.41421356f; k.s01 = 0.f; k.s10 = 0.f; k.s11 = 1.41421356f;
    k.b0 = 0.f; k.b1 = 0.f; k.c = 0.f;
    k.f = 19.7392088f * (sx * cy);
    // g = (pi cx cy + y, x - pi sx sy)
    const float2 g = __ffma2_rn(make_float2(PI, -PI), __fmul2_rn(make_float2(cx, sx), make_float2(cy, sy)),
                                make_float2(y, x));
    k.g0 = g.x;
    k.g1 = g.y;
  } else if (KIND == PK_HELMHOLTZ) {
    const float a = (float)P.p[0], b = (float)P.p[1], c = (float)P.p[2];
    // the x and y halves in paired FP32 instructions (same roundings)
    const float2 arg = __fmul2_rn(make_float2(a, b), make_float2(x, y));
    float sa, ca, sb, cb;
    __sincosf(arg.x, &sa, &ca);
    __sincosf(arg.y, &sb, &cb);
    k.s00 = 1.41421356f; k.s01 = 0.f; k.s10 = 0.f; k.s11 = 1.41421356f;
    k.b0 = 0.f; k.b1 = 0.f; k.c = c;
    k.f = ((a * a + b * b) - c) * (sa * cb);
    // g = (a ca cb, -b sa sb)
    const float2 g = __fmul2_rn(make_float2(a, -b), __fmul2_rn(make_float2(ca, sa), make_float2(cb, sb)));
    k.g0 = g.x;
    k.g1 = g.y;
  } else if (KIND == PK_VARCOEF) {
    const float s1 = 1.f + 0.5f * (x * x), s2 = 1.f + 0.5f * (y * y);
    float sn, cs;
    __sincosf(2.f * y, &sn, &cs);
    const float ex = __expf(x);
    const float ux = ex * cs, uy = -2.f * (ex * sn), uxx = ux, uyy = -4.f * ux;
    const float c = -(1.f + x * x + y * y);
    k.s00 = s1; k.s01 = 0.f; k.s10 = 0.f; k.s11 = s2;
    k.b0 = y; k.b1 = -x; k.c = c;
    k.f = -(0.5f * (s1 * s1 * uxx + s2 * s2 * uyy) + (y * ux - x * uy) + c * (ux + 1.f));
    k.g0 = ux;
    k.g1 = uy;
  } else if (KIND == PK_CIRCLE) {
    // u = r^2 sin 3t + cos x: with c = x / r, s = y / r, sin 3t = 3s - 4s^3,
    // cos 3t = 4c^3 - 3c; f = -Lap u = 5 sin 3t + cos x (bounded, continuous
    // away from r = 0); grad u = (2r sin3t c - 3r cos3t s - sin x,
    // 2r sin3t s + 3r cos3t c)
    const float r2 = x * x + y * y;
    const float ir = r2 > 1e-30f ? rsqrt_approx(r2) : 0.f;
    const float r = r2 * ir;
    const float c1 = r2 > 1e-30f ? x * ir : 1.f, s1 = y * ir;
    const float s3 = s1 * (3.f - 4.f * s1 * s1), c3 = c1 * (4.f * c1 * c1 - 3.f);
    float sx, cx;
    __sincosf(x, &sx, &cx);
    k.s00 = 1.41421356f; k.s01 = 0.f; k.s10 = 0.f; k.s11 = 1.41421356f;
    k.b0 = 0.f; k.b1 = 0.f; k.c = 0.f;
    k.f = 5.f * s3 + cx;
    k.g0 = r * (2.f * s3 * c1 - 3.f * c3 * s1) - sx;
    k.g1 = r * (2.f * s3 * s1 + 3.f * c3 * c1);
  } else if (KIND == PK_ROBIN) {
    // BVPs/EDPs/poisson_3.hpp: u = sin(A) + cos(B), A = pi (0.23 x + 0.49 y),
    // B = pi (0.331 x + 0.667 y), f = -Lap u
    float sa, ca, sb, cb;
    __sincosf(PI * (0.23f * x + 0.49f * y), &sa, &ca);
    __sincosf(PI * (0.331f * x + 0.667f * y), &sb, &cb);
    k.s00 = 1.41421356f; k.s01 = 0.f; k.s10 = 0.f; k.s11 = 1.41421356f;
    k.b0 = 0.f; k.b1 = 0.f; k.c = 0.f;
    k.f = 9.8696044f * (0.2930f * sa + 0.554450f * cb);
    k.g0 = PI * (0.23f * ca - 0.331f * sb);
    k.g1 = PI * (0.49f * ca - 0.667f * sb);
  } else {  // PK_MONEGROS (BVPs/EDPs/Monegros_Poisson_CPP.hpp)
    const float k2 = 0.01f, k3 = 0.02f, k4 = 0.12f, k5 = 0.05f, k6 = 0.05f, k7 = -0.12f, sf = 0.333f;
    const float q = 1.f + k2 * x * x + k3 * y * y;
    const float ia1 = rsqrt_approx(q);  // q >= 1
    const float a1 = q * ia1;
    float s1, c1, sA, cA, sB, cB;
    __sincosf(a1, &s1, &c1);
    __sincosf(k4 * x + k5 * y, &sA, &cA);
    __sincosf(k6 * x + k7 * y, &sB, &cB);
    const float a2 = tanhf(sA + sB);
    const float m = a2 * a2 - 1.f;
    const float p4 = k4 * cA + k6 * cB, p5 = k5 * cA + k7 * cB;
    const float ia2 = ia1 * ia1, ia3 = ia2 * ia1;
    const float dxx = ((k2 * ia1) - (k2 * k2 * x * x * ia3)) * c1 - (x * x * k2 * k2 * ia2) * s1 +
                      2.f * p4 * p4 * m * a2 + (k4 * k4 * sA + k6 * k6 * sB) * m;
    const float dyy = ((k3 * ia1) - (k3 * k3 * y * y * ia3)) * c1 - (y * y * k3 * k3 * ia2) * s1 +
                      2.f * p5 * p5 * m * a2 + (k5 * k5 * sA + k7 * k7 * sB) * m;
    k.s00 = 1.41421356237f; k.s01 = 0.f; k.s10 = 0.f; k.s11 = 1.41421356237f;
    k.b0 = 0.f; k.b1 = 0.f; k.c = 0.f;
    k.f = -sf * dxx - sf * dyy;
    k.g0 = sf * (c1 * k2 * x * ia1 - p4 * m);
    k.g1 = sf * (c1 * k3 * y * ia1 - p5 * m);
  }
  // the control variate is switched off by the caller (P.use_cv), which
  // drops the accumulated xi at the exit instead of zeroing g every step
}

// Terms of the FP32 step that a problem kind has, known at compile time:
// sigma is diagonal for every kind; iso kinds have sigma = sqrt2 I and no
// drift; react kinds have a reaction term c.
template <int KIND>
struct KindTraits {
  static constexpr bool iso = KIND == PK_POISSON_SINCOS || KIND == PK_MONEGROS || KIND == PK_HELMHOLTZ ||
                              KIND == PK_CIRCLE || KIND == PK_ROBIN;
  static constexpr bool react = KIND == PK_HELMHOLTZ || KIND == PK_VARCOEF || is_lut_kind(KIND);
};

// sigma alone (for the exit threshold)
template <int KIND>
__device__ __forceinline__ void sigma_f32(const ProblemDev& P, float x, float y, float& s00, float& s01,
                                          float& s10, float& s11) {
  if (is_lut_kind(KIND)) {
    float v[4];
    lut_sample_f32<KIND, 4>(P.lut, x, y, v);
    s00 = v[0]; s01 = 0.f; s10 = 0.f; s11 = v[1];
  } else if (KIND == PK_VARCOEF) {
    s00 = 1.f + 0.5f * (x * x); s01 = 0.f; s10 = 0.f; s11 = 1.f + 0.5f * (y * y);
  } else if (KIND == PK_MONEGROS) {
    s00 = 1.41421356237f; s01 = 0.f; s10 = 0.f; s11 = 1.41421356237f;
  } else {
    s00 = 1.41421356f; s01 = 0.f; s10 = 0.f; s11 = 1.41421356f;
  }
}

// |N^T sigma| for the x normal (1,0) and the y normal (0,1) (diagonal sigma)
template <int KIND>
__device__ __forceinline__ void sigma_normals_f32(const ProblemDev& P, float x, float y, float& nx, float& ny) {
  if (is_lut_kind(KIND)) {
    float v[4];
    lut_sample_f32<KIND, 4>(P.lut, x, y, v);
    nx = fabsf(v[0]);
    ny = fabsf(v[1]);
  } else if (KIND == PK_VARCOEF) {
    nx = 1.f + 0.5f * (x * x);
    ny = 1.f + 0.5f * (y * y);
  } else if (KIND == PK_MONEGROS) {
    nx = ny = 1.41421356237f;
  } else {
    nx = ny = 1.41421356f;
  }
}

template <int KIND>
__device__ __forceinline__ float u_f32(const ProblemDev& P, float x, float y) {
  if (is_lut_kind(KIND)) {
    return lut_sample_g<float>(P.lut, x, y);
  } else if (KIND == PK_POISSON_SINCOS) {
    float sx, cx, sy, cy;
    __sincosf(3.14159265358979f * x, &sx, &cx);
    __sincosf(3.14159265358979f * y, &sy, &cy);
    return sx * cy + x * y;
  } else if (KIND == PK_HELMHOLTZ) {
    return __sinf((float)P.p[0] * x) * __cosf((float)P.p[1] * y);
  } else if (KIND == PK_VARCOEF) {
    return __expf(x) * __cosf(2.f * y) + 1.f;
  } else if (KIND == PK_CIRCLE) {
    const float r = sqrtf(x * x + y * y);
    const float s1 = r > 1e-30f ? y / r : 0.f;
    return r * r * (s1 * (3.f - 4.f * s1 * s1)) + __cosf(x);
  } else if (KIND == PK_ROBIN) {
    return __sinf(3.14159265f * (0.23f * x + 0.49f * y)) + __cosf(3.14159265f * (0.331f * x + 0.667f * y));
  } else {
    const float q = 1.f + 0.01f * x * x + 0.02f * y * y;
    return 3.f + 0.333f * (__sinf(sqrtf(q)) + tanhf(__sinf(0.12f * x + 0.05f * y) + __sinf(0.05f * x - 0.12f * y)));
  }
}

// ------------------------------------------------------------------ FP64
// Plain double precision with the CUDA math library (FP64 mode).
template <int KIND>
__device__ __forceinline__ void coef_f64(const ProblemDev& P, double x, double y, Coef<double>& k) {
  const double PI = 3.141592653589793;
  if (is_lut_kind(KIND)) {
    double v[8];
    lut_sample<double, 8>(P.lut, x, y, v);
    k.s00 = v[0]; k.s01 = 0.0; k.s10 = 0.0; k.s11 = v[1];
    k.b0 = v[2]; k.b1 = v[3]; k.c = v[4]; k.f = v[5]; k.g0 = v[6]; k.g1 = v[7];
  } else if (KIND == PK_POISSON_SINCOS) {
    double sx, cx, sy, cy;
    sincospi(x, &sx, &cx);
    sincospi(y, &sy, &cy);
    k.s00 = 1.4142135623730951; k.s01 = 0.0; k.s10 = 0.0; k.s11 = 1.4142135623730951;
    k.b0 = 0.0; k.b1 = 0.0; k.c = 0.0;
    k.f = 19.739208802178716 * (sx * cy);
    k.g0 = PI * (cx * cy) + y;
    k.g1 = x - PI * (sx * sy);
  } else if (KIND == PK_HELMHOLTZ) {
    const double a = P.p[0], b = P.p[1], c = P.p[2];
    double sa, ca, sb, cb;
    sincos(a * x, &sa, &ca);
    sincos(b * y, &sb, &cb);
    k.s00 = 1.4142135623730951; k.s01 = 0.0; k.s10 = 0.0; k.s11 = 1.4142135623730951;
    k.b0 = 0.0; k.b1 = 0.0; k.c = c;
    k.f = ((a * a + b * b) - c) * (sa * cb);
    k.g0 = a * (ca * cb);
    k.g1 = -(b * (sa * sb));
  } else if (KIND == PK_VARCOEF) {
    const double s1 = 1.0 + 0.5 * (x * x), s2 = 1.0 + 0.5 * (y * y);
    double sn, cs;
    sincos(2.0 * y, &sn, &cs);
    const double ex = ::exp(x);
    const double ux = ex * cs, uy = -2.0 * (ex * sn), uxx = ux, uyy = -4.0 * ux;
    const double c = -(1.0 + x * x + y * y);
    k.s00 = s1; k.s01 = 0.0; k.s10 = 0.0; k.s11 = s2;
    k.b0 = y; k.b1 = -x; k.c = c;
    k.f = -(0.5 * (s1 * s1 * uxx + s2 * s2 * uyy) + (y * ux - x * uy) + c * (ux + 1.0));
    k.g0 = ux;
    k.g1 = uy;
  } else if (KIND == PK_CIRCLE) {
    const double r = ::sqrt(x * x + y * y);
    const double c1 = r > 1e-300 ? x / r : 1.0, s1 = r > 1e-300 ? y / r : 0.0;
    const double s3 = s1 * (3.0 - 4.0 * s1 * s1), c3 = c1 * (4.0 * c1 * c1 - 3.0);
    double sx, cx;
    sincos(x, &sx, &cx);
    k.s00 = 1.4142135623730951; k.s01 = 0.0; k.s10 = 0.0; k.s11 = 1.4142135623730951;
    k.b0 = 0.0; k.b1 = 0.0; k.c = 0.0;
    k.f = 5.0 * s3 + cx;
    k.g0 = r * (2.0 * s3 * c1 - 3.0 * c3 * s1) - sx;
    k.g1 = r * (2.0 * s3 * s1 + 3.0 * c3 * c1);
  } else if (KIND == PK_ROBIN) {
    double sa, ca, sb, cb;
    sincospi(0.23 * x + 0.49 * y, &sa, &ca);
    sincospi(0.331 * x + 0.667 * y, &sb, &cb);
    k.s00 = 1.4142135623730951; k.s01 = 0.0; k.s10 = 0.0; k.s11 = 1.4142135623730951;
    k.b0 = 0.0; k.b1 = 0.0; k.c = 0.0;
    k.f = 9.869604401089358 * (0.2930 * sa + 0.554450 * cb);
    k.g0 = PI * (0.23 * ca - 0.331 * sb);
    k.g1 = PI * (0.49 * ca - 0.667 * sb);
  } else {
    const double k2 = 0.01, k3 = 0.02, k4 = 0.12, k5 = 0.05, k6 = 0.05, k7 = -0.12, sf = 0.333;
    const double q = 1.0 + k2 * x * x + k3 * y * y;
    const double a1 = ::sqrt(q);
    double s1, c1, sA, cA, sB, cB;
    sincos(a1, &s1, &c1);
    sincos(k4 * x + k5 * y, &sA, &cA);
    sincos(k6 * x + k7 * y, &sB, &cB);
    const double a2 = ::tanh(sA + sB);
    const double m = a2 * a2 - 1.0;
    const double p4 = k4 * cA + k6 * cB, p5 = k5 * cA + k7 * cB;
    const double dxx = ((k2 / a1) - (k2 * k2 * x * x / (a1 * a1 * a1))) * c1 - (x * x * k2 * k2 / (a1 * a1)) * s1 +
                       2.0 * p4 * p4 * m * a2 + (k4 * k4 * sA + k6 * k6 * sB) * m;
    const double dyy = ((k3 / a1) - (k3 * k3 * y * y / (a1 * a1 * a1))) * c1 - (y * y * k3 * k3 / (a1 * a1)) * s1 +
                       2.0 * p5 * p5 * m * a2 + (k5 * k5 * sA + k7 * k7 * sB) * m;
    k.s00 = 1.41421356237; k.s01 = 0.0; k.s10 = 0.0; k.s11 = 1.41421356237;
    k.b0 = 0.0; k.b1 = 0.0; k.c = 0.0;
    k.f = -sf * dxx - sf * dyy;
    k.g0 = sf * (c1 * k2 * x / a1 - p4 * m);
    k.g1 = sf * (c1 * k3 * y / a1 - p5 * m);
  }
  if (!P.use_cv) { k.g0 = 0.0; k.g1 = 0.0; }
}

template <int KIND>
__device__ __forceinline__ double u_f64(const ProblemDev& P, double x, double y) {
  if (is_lut_kind(KIND)) {
    return lut_sample_g<double>(P.lut, x, y);
  } else if (KIND == PK_POISSON_SINCOS) {
    double sx, cx, sy, cy;
    sincospi(x, &sx, &cx);
    sincospi(y, &sy, &cy);
    return sx * cy + x * y;
  } else if (KIND == PK_HELMHOLTZ) {
    return ::sin(P.p[0] * x) * ::cos(P.p[1] * y);
  } else if (KIND == PK_VARCOEF) {
    return ::exp(x) * ::cos(2.0 * y) + 1.0;
  } else if (KIND == PK_CIRCLE) {
    const double r = ::sqrt(x * x + y * y);
    const double s1 = r > 1e-300 ? y / r : 0.0;
    return r * r * (s1 * (3.0 - 4.0 * s1 * s1)) + ::cos(x);
  } else if (KIND == PK_ROBIN) {
    return sinpi(0.23 * x + 0.49 * y) + cospi(0.331 * x + 0.667 * y);
  } else {
    const double q = 1.0 + 0.01 * x * x + 0.02 * y * y;
    return 3.0 + 0.333 * (::sin(::sqrt(q)) + ::tanh(::sin(0.12 * x + 0.05 * y) + ::sin(0.05 * x - 0.12 * y)));
  }
}

// Robin data of PK_ROBIN (poisson_3.hpp): varphi = -2 + sin(pi y) and
// psi = n.grad u - varphi u at a boundary point with outward normal n, so
// that n.grad u - varphi u = psi there; along a reflected path
// Y += varphi Y dL and Z += psi Y dL with dL the local time.
template <typename T>
__device__ __forceinline__ void robin_data(T x, T y, T n0, T n1, T& varphi, T& psi) {
  const T PI = T(3.141592653589793);
  T sa, ca, sb, cb, sy;
  if constexpr (sizeof(T) == 4) {
    __sincosf(PI * (T(0.23) * x + T(0.49) * y), &sa, &ca);
    __sincosf(PI * (T(0.331) * x + T(0.667) * y), &sb, &cb);
    sy = __sinf(PI * y);
  } else {
    sincospi(T(0.23) * x + T(0.49) * y, &sa, &ca);
    sincospi(T(0.331) * x + T(0.667) * y, &sb, &cb);
    sy = sinpi(y);
  }
  const T gx = PI * (T(0.23) * ca - T(0.331) * sb), gy = PI * (T(0.49) * ca - T(0.667) * sb);
  varphi = T(-2) + sy;
  psi = n0 * gx + n1 * gy - (sa + cb) * varphi;
}

// ------------------------------------------------------------------ rectangle
// Rectangle2D (BVPs/Domains/rectangle.hpp:7-229) with the same branch table:
// signed distance (negative inside), projection E onto the nearest side and
// the outward normal N.  `onmask` reports the sides E lies on (bit d for
// Dir d) so the exit side can be taken without comparing coordinates.
template <typename T>
__device__ __forceinline__ T rect2d(const T* p, T x, T y, T& Ex, T& Ey, T& Nx, T& Ny, int& onmask) {
  const T c0 = T(0.5) * (p[0] + p[2]), c1 = T(0.5) * (p[1] + p[3]);
  const T h0 = p[2] - c0, h1 = p[3] - c1;
  const T d0 = fabs(x - c0), d1 = fabs(y - c1);
  const bool right = x > c0, top = y > c1;
  const T ex = right ? (h0 + c0) : (-h0 + c0);
  const T ey = top ? (h1 + c1) : (-h1 + c1);
  const T nx = right ? T(1) : T(-1), ny = top ? T(1) : T(-1);
  const int xside = right ? (1 << 2) : (1 << 3);   // E : W
  const int yside = top ? (1 << 0) : (1 << 1);     // N : S
  Ex = x; Ey = y;
  if (d0 <= h0 && d1 <= h1) {
    if (d0 - h0 > d1 - h1) { Ex = ex; Nx = nx; Ny = T(0); onmask = xside; return d0 - h0; }
    Ey = ey; Nx = T(0); Ny = ny; onmask = yside; return d1 - h1;
  }
  if (d0 > h0) {
    if (d1 > h1) {
      const T diag = T(0.70710678118f);
      Ex = ex; Ey = ey; Nx = right ? diag : -diag; Ny = top ? diag : -diag;
      onmask = xside | yside;
      return sqrt((d0 - h0) * (d0 - h0) + (d1 - h1) * (d1 - h1));
    }
    Ex = ex; Nx = nx; Ny = T(0); onmask = xside;
    return d0 - h0;
  }
  Ey = ey; Nx = T(0); Ny = ny; onmask = yside;
  return d1 - h1;
}

// Adaptive step of a knot (PDDSparseGM.cpp:4026-4028):
// h_k = min(h0, (d / (|N^T sigma(x0)| * 2 * 0.5826))^2) when d <= -1e-4.
template <typename T>
__device__ __forceinline__ double adaptive_step(const double* rect, double x0, double y0, double h0,
                                                const Coef<T>& k) {
  double Ex, Ey, Nx, Ny;
  int om;
  const double d = rect2d<double>(rect, x0, y0, Ex, Ey, Nx, Ny, om);
  if (!(d <= -1e-04)) return h0;
  const double w0 = Nx * (double)k.s00 + Ny * (double)k.s10;
  const double w1 = Nx * (double)k.s01 + Ny * (double)k.s11;
  const double q = d / (sqrt(w0 * w0 + w1 * w1) * 2 * 0.5826);
  const double ha = q * q;
  return h0 < ha ? h0 : ha;
}

// The same step on a polar stencil {rho0, phi0, rho1, phi1} (isotropic
// sigma): d = the largest outside distance to the inner arc (none at the
// centre), the outer arc and the two rays, as in the polar exit test.
template <typename T>
__device__ __forceinline__ double adaptive_step_polar(const double* rect, double x0, double y0, double h0,
                                                      const Coef<T>& k) {
  const double rho = sqrt(x0 * x0 + y0 * y0);
  double d = rho - rect[2];
  if (rect[0] > 0.0) d = fmax(d, rect[0] - rho);
  if (rect[3] - rect[1] < 6.2) {  // a full disk has no rays
    d = fmax(d, sin(rect[1]) * x0 - cos(rect[1]) * y0);
    d = fmax(d, cos(rect[3]) * y0 - sin(rect[3]) * x0);
  }
  if (!(d <= -1e-04)) return h0;
  const double q = d / (fabs((double)k.s00) * 2 * 0.5826);
  const double ha = q * q;
  return h0 < ha ? h0 : ha;
}

// Exit side by the reference's priority S, N, W, E (G_update, stencil.cpp:246-301).
__device__ __forceinline__ int exit_side(int onmask) {
  if (onmask & (1 << 1)) return 1;  // S
  if (onmask & (1 << 0)) return 0;  // N
  if (onmask & (1 << 3)) return 3;  // W
  if (onmask & (1 << 2)) return 2;  // E
  return -1;
}

// Cubic Lagrange weights for nodes -1, 0, 1, 2 at offset u in [0, 1).
__device__ __forceinline__ void cubic_weights(float u, float& w0, float& w1, float& w2, float& w3) {
  const float um1 = u - 1.f, um2 = u - 2.f, up1 = u + 1.f;
  w0 = -u * um1 * um2 * (1.f / 6.f);
  w1 = up1 * um1 * um2 * 0.5f;
  w2 = -up1 * u * um2 * 0.5f;
  w3 = up1 * u * um1 * (1.f / 6.f);
}

}  // namespace pdds
