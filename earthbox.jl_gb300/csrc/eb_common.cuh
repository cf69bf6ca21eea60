// eb_common.cuh -- shared device helpers for the sm_103a marker-in-cell kernels.
//
// Precision policy (GB300 runs FP64 at 1/72 of the FP32 rate: 1.0 vs 73 TFLOP/s
// measured with dependent-chain FMA kernels on this part):
//   * marker state and grid fields are stored in FP64, as in the reference;
//   * cell indices are computed exactly with integer comparisons of the IEEE
//     bit patterns (no FP64 arithmetic), so they equal searchsortedlast;
//   * the exclusive-quadrant tests (dx <= 0.5 etc.) are decided exactly: an FP32
//     estimate settles all markers farther than 4e-7 from the half line, the
//     rest use the exact FP64 test derived from round-to-nearest-even;
//   * weights, products and per-cell sums run in FP32 with compensated
//     (Neumaier) summation; the error budget is < 5e-7 relative per field.
#pragma once
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

#define EB_DEV __device__ __forceinline__

// ---- order-preserving integer key of an IEEE double --------------------------
// For finite doubles a <= b  <=>  key(a) <= key(b) as unsigned 64-bit integers.
// Both zeros map to the same key, as IEEE compares -0.0 == +0.0.
__host__ __device__ __forceinline__ uint64_t dkey(double v) {
#ifdef __CUDA_ARCH__
  uint64_t u = (uint64_t)__double_as_longlong(v);
#else
  uint64_t u; memcpy(&u, &v, 8);
#endif
  if ((u << 1) == 0) u = 0;  // -0.0 -> +0.0
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

// ---- FP64 <-> FP32 conversion with integer operations ---------------------------
// On GB300 the F2F conversion instructions issue on the FP64 pipe (0.5 T op/s,
// measured: a gather kernel doing ~33 conversions per marker ran with that pipe
// 95% busy), so the hot kernels convert with 32-bit integer operations instead.
// d2f rounds to nearest (a tie rounds away from zero, IEEE rounds it to even:
// the two differ by one FP32 ulp on exact ties only); magnitudes below FLT_MIN
// become a signed zero, above FLT_MAX infinity.  Every value on this path lies
// well inside the FP32 range.
EB_DEV float d2f(double d) {
  const uint32_t hi = (uint32_t)__double2hiint(d), lo = (uint32_t)__double2loint(d);
  const int32_t e = (int32_t)((hi >> 20) & 0x7FFu) - 896;  // FP32 exponent field
  uint32_t bits = ((uint32_t)e << 23) + (((hi & 0xFFFFFu) << 3) | (lo >> 29)) + ((lo >> 28) & 1u);
  bits = (e <= 0) ? 0u : ((e >= 255) ? 0x7F800000u : bits);
  return __uint_as_float((hi & 0x80000000u) | bits);
}
// Exact FP32 -> FP64 widening (FP32 subnormals, never produced here, become zero).
EB_DEV double f2d(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t ex = (b >> 23) & 0xFFu, man = b & 0x7FFFFFu;
  uint32_t hi = b & 0x80000000u, lo = 0u;
  if (ex != 0u) {
    hi |= ((ex == 255u ? 2047u : ex + 896u) << 20) | (man >> 3);
    lo = man << 29;
  }
  return __hiloint2double((int)hi, (int)lo);
}

// ---- exact searchsortedlast with a bucket accelerator ------------------------
// A 1-D grid coordinate array v[1..n] (stored 0-based) is described by its keys
// and by a table that maps a uniform bucket over [v1, vn] to the
// searchsortedlast index of the bucket's lower edge.  The FP32 bucket estimate
// only chooses where the exact integer walk starts; the walk makes the result
// exact for any estimate.
struct Axis {
  const uint64_t* key;   // [n] order keys of the coordinates
  const int32_t* bucket; // [nb+1] searchsortedlast(v, lower edge of bucket b)
  int32_t n, nb;
  float v0, inv_h;       // bucket b = floor((x - v0) * inv_h)
};

// Returns searchsortedlast(v, x) in [0, n] (1-based index of the last v <= x).
EB_DEV int32_t axis_search(const Axis& a, double x) {
  const uint64_t kx = dkey(x);
  // clamp before the conversion (fmaxf maps NaN to 0), so b is always in [0, nb]
  const float t = fminf(fmaxf((d2f(x) - a.v0) * a.inv_h, 0.f), (float)a.nb);
  const int32_t b = (int32_t)t;
  int32_t i = __ldg(&a.bucket[b]);
  // walk up while v[i+1] <= x, then down while v[i] > x (1-based indices)
  while (i < a.n && __ldg(&a.key[i]) <= kx) ++i;
  while (i > 0 && __ldg(&a.key[i - 1]) > kx) --i;
  return i;
}

EB_DEV int32_t clamp_i(int32_t v, int32_t lo, int32_t hi) { return v < lo ? lo : (v > hi ? hi : v); }

// ---- compensated FP32 accumulation ------------------------------------------------
// Each add records its exact rounding error (Knuth's TwoSum: six additions, no
// comparison) in a running correction c; the result is s + c.
struct KSum {
  float s, c;
  EB_DEV void init() { s = 0.f; c = 0.f; }
  EB_DEV void add(float v) {
    const float t = s + v;
    const float z = t - s;
    c += (s - (t - z)) + (v - z);
    s = t;
  }
  EB_DEV float get() const { return s + c; }
};
// Two compensated accumulators in packed FP32x2 arithmetic (TwoSum per lane of the
// pair; a - b is computed as fma(b, -1, a), which rounds once like a subtraction).
EB_DEV void two_sum2(float2& s, float2& c, float2 v) {
  const float2 m1 = make_float2(-1.f, -1.f);
  const float2 t = __fadd2_rn(s, v);
  const float2 z = __ffma2_rn(s, m1, t);                                    // t - s
  const float2 e = __fadd2_rn(__ffma2_rn(__ffma2_rn(z, m1, t), m1, s),      // s - (t - z)
                              __ffma2_rn(z, m1, v));                        // v - z
  c = __fadd2_rn(c, e);
  s = t;
}
struct KSum2 {
  float2 s, c;
  EB_DEV void init() { s = make_float2(0.f, 0.f); c = s; }
  EB_DEV void add(float2 v) { two_sum2(s, c, v); }
  EB_DEV float x() const { return s.x + c.x; }
  EB_DEV float y() const { return s.y + c.y; }
};

// ---- marker flag byte written by the locate kernel ----------------------------
enum : uint8_t {
  MF_INSIDE = 1,   // inside_flags == 1
  MF_VYRIGHT = 2,  // marker_xn_vy == marker_xn + 1
  MF_XLE = 4,      // fl((x - gx[xn]) / xstp[xn]) <= 0.5   (exact)
  MF_XGE = 8,      // ... >= 0.5
  MF_YLE = 16,
  MF_YGE = 32,
};

// Bilinear weights from fractional offsets (reference calc_marker_weights:
// UL=(1-dx)(1-dy), LL=(1-dx)dy, UR=dx(1-dy), LR=dx*dy).
struct W4 { float ul, ll, ur, lr; };
EB_DEV W4 wts(float dx, float dy) {
  float ox = 1.f - dx, oy = 1.f - dy;
  return W4{ox * oy, ox * dy, dx * oy, dx * dy};
}

// 4-point bilinear gather on a column-major grid (rows = leading dimension),
// 1-based upper-left node (iy, ix), FP32 weights, FP64 grid values.
EB_DEV float gather4(const double* __restrict__ g, int32_t rows, int32_t iy, int32_t ix, float dx,
                     float dy) {
  const W4 w = wts(dx, dy);
  const size_t o = (size_t)(ix - 1) * rows + (iy - 1);
  float v = w.ul * d2f(__ldg(&g[o]));
  v = fmaf(w.ll, d2f(__ldg(&g[o + 1])), v);
  v = fmaf(w.ur, d2f(__ldg(&g[o + rows])), v);
  v = fmaf(w.lr, d2f(__ldg(&g[o + rows + 1])), v);
  return v;
}
// The 4-point gather from the four node values (UL, LL, UR, LR) already in registers
// (the arithmetic of gather4f below).
EB_DEV float gather4v(float n0, float n1, float n2, float n3, float dx, float dy) {
  const W4 w = wts(dx, dy);
  float v = w.ul * n0;
  v = fmaf(w.ll, n1, v);
  v = fmaf(w.ur, n2, v);
  v = fmaf(w.lr, n3, v);
  return v;
}

// (a grid holds fewer than 2^31 nodes: the offset is formed in 32 bits)
EB_DEV float gather4f(const float* __restrict__ g, int32_t rows, int32_t iy, int32_t ix, float dx,
                      float dy) {
  const W4 w = wts(dx, dy);
  const float* p = g + ((ix - 1) * rows + (iy - 1));
  float v = w.ul * __ldg(p);
  v = fmaf(w.ll, __ldg(p + 1), v);
  v = fmaf(w.ur, __ldg(p + rows), v);
  v = fmaf(w.lr, __ldg(p + rows + 1), v);
  return v;
}
