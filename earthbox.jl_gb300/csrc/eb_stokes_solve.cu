// eb_stokes_solve.cu -- iterative solve of the Stokes-continuity system on the GPU.
//
// Replaces the reference's direct sparse solve (SystemSolver.solve_system_optimized,
// src/stokes_continuity_solver/solver/system_solver/SystemSolver.jl:67-91, which
// calls MUMPS through ParallelSolver.jl:52-126 or UMFPACK through `sparse(...) \ R`).
//
// Method.  FGMRES in FP64 on the symmetrically scaled system (W L W) y = W R,
// S = W y, with W = 1/sqrt(|diag L|) on the momentum rows and sqrt(2 eta_n)/pscale
// on the continuity rows (the inverse square root of the Schur-complement
// diagonal), so that the residual FGMRES minimises weighs weak (sticky-air) and
// stiff regions alike.  Right preconditioner: block upper-triangular,
//   z_p = (2 eta_n / pscale^2) r_p   (1/L_pp on pressure-condition rows),
//   z_u = MG(r_u - L_up z_p),
// where MG is one V-cycle of FP32 geometric multigrid on the coupled velocity
// block: red-black Gauss-Seidel on vx then vy, coarse levels rediscretised from
// arithmetic averages of the viscosity on grids with every other node (the last
// coarse cell takes three fine cells when the count is odd), linear transfer
// operators in physical coordinates with the boundary-condition coefficients
// folded in, and an exact dense solve on the coarsest level.  The V-cycle is
// captured once per solve into a CUDA graph and replayed every iteration.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>
#include "eb_internal.h"

namespace {

constexpr int kB = 256;
constexpr int kRmax = 8;  // restriction entries per coarse index and axis
constexpr int kMaxRestart = 500;
// Classical Gram-Schmidt re-orthogonalises a new direction only when the projection
// removed all but 5% of its norm (squared ratio below).
constexpr double kReorth2 = 0.05 * 0.05;
// Default residual level (relative to the target) below which the mixed method's
// Gram-Schmidt runs in FP32 on the basis copies.
constexpr double kGsRelax = 1e3;
// The mixed method's FP64 residual "fails to fall" when an FGMRES cycle leaves the true
// residual above this fraction of its value at the start of the cycle.
constexpr double kStallFactor = 0.5;
// Velocity stage of the block preconditioner: GCR steps (each one V-cycle) at most, and the
// velocity residual reduction at which they stop.
constexpr int kGcrDefaultSteps = 1;
constexpr double kGcrDefaultTol = 0.1;
constexpr int kMaxDots = kMaxRestart + 8;  // dot products per reduction

unsigned nblk(int64_t n) { return (unsigned)((n + kB - 1) / kB); }

// ---- double-float helpers (the mixed method's Krylov vectors, below) ----
// x = hi + lo: hi = x rounded to FP32 (d2f), lo = x - hi rounded to FP32, by integer
// operations; |x - hi - lo| <= 2^-48 |x|.  Magnitudes below 2^-74 keep hi alone (the
// dropped lo is below 2^-98), below FLT_MIN both are zero; above FLT_MAX, and NaN, hi is
// infinite.
EB_DEV void split_df(double x, float& hi, float& lo) {
  const uint32_t H = (uint32_t)__double2hiint(x), L = (uint32_t)__double2loint(x);
  const uint32_t e = (H >> 20) & 0x7FFu;
  hi = d2f(x);
  // the 29 significand bits below hi's last place, as a signed count of units 2^(e - 1075):
  // r, or r - 2^29 when d2f rounded the magnitude up (bit 28 set)
  const int32_t r = (int32_t)(L & 0x1FFFFFFFu);
  const int32_t t = ((L >> 28) & 1u) ? r - (1 << 29) : r;
  const float mag = __fmul_rn(__int2float_rn(t), __uint_as_float((e - 948u) << 23));  // exact: power of 2
  lo = (e >= 949u && e <= 1150u) ? __uint_as_float(__float_as_uint(mag) ^ (H & 0x80000000u)) : 0.f;
}
// (s, c) += p + e (TwoSum of s and p; e and the rounding error go to c)
EB_DEV void two_sum_acc(float p, float e, float& s, float& c) {
  const float t = __fadd_rn(s, p);
  const float z = __fsub_rn(t, s);
  c = __fadd_rn(c, __fadd_rn(__fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z)), e));
  s = t;
}
// (s, c) += (ah + al) x for an FP32 x
EB_DEV void df_axpy_acc(float ah, float al, float x, float& s, float& c) {
  const float p = __fmul_rn(ah, x);
  const float e = fmaf(al, x, fmaf(ah, x, -p));
  two_sum_acc(p, e, s, c);
}
// (s, c) += (ah + al)(bh + bl), the al bl term dropped
EB_DEV void df_fma_acc(float ah, float al, float bh, float bl, float& s, float& c) {
  const float p = __fmul_rn(ah, bh);
  const float e = fmaf(al, bh, fmaf(ah, bl, fmaf(ah, bh, -p)));
  two_sum_acc(p, e, s, c);
}
// normalised pair h + l = s + c with |l| <= ulp(h) / 2 (TwoSum)
EB_DEV void df_norm(float s, float c, float& h, float& l) {
  h = __fadd_rn(s, c);
  const float z = __fsub_rn(h, s);
  l = __fadd_rn(__fsub_rn(s, __fsub_rn(h, z)), __fsub_rn(c, z));
}


// ------------------------------------------------------- FP64 operator ---
// y = L x on SoA vectors [vx | vy | p] (cell c = j ny + i), optionally y -= sub and an FP32
// copy y32.  The FGMRES iteration passes the pre-scaled stencil W L W (k_prescale), the
// residual checks the assembled one.  Cell indices fit 32 bits (27 nc doubles of stencil
// would exceed the device's memory first).
__global__ void __launch_bounds__(kB) k_apply64(const double* __restrict__ coef, const double* __restrict__ x,
                                                double* __restrict__ y, int32_t nx, int32_t ny, int32_t nc,
                                                const double* __restrict__ sub = nullptr,
                                                float* __restrict__ y32 = nullptr) {
  const int32_t c = (int32_t)(blockIdx.x * blockDim.x + threadIdx.x);
  if (c >= nc) return;
  const int32_t j = c / ny, i = c - j * ny;
  const double *vx = x, *vy = x + nc, *p = x + 2 * (int64_t)nc;
  const bool hu = i > 0, hd = i < ny - 1, hl = j > 0, hr = j < nx - 1;
  auto cf = [&](int s) { return __ldg(&coef[(int64_t)s * nc + c]); };
  double ax = cf(0) * vx[c];
  if (hl) ax += cf(1) * vx[c - ny];
  if (hr) ax += cf(2) * vx[c + ny];
  if (hu) ax += cf(3) * vx[c - 1];
  if (hd) ax += cf(4) * vx[c + 1];
  if (hu) ax += cf(5) * vy[c - 1];
  if (hu && hr) ax += cf(6) * vy[c + ny - 1];
  ax += cf(7) * vy[c];
  if (hr) ax += cf(8) * vy[c + ny];
  ax += cf(9) * p[c];
  if (hr) ax += cf(10) * p[c + ny];
  double ay = cf(11) * vy[c];
  if (hu) ay += cf(12) * vy[c - 1];
  if (hd) ay += cf(13) * vy[c + 1];
  if (hl) ay += cf(14) * vy[c - ny];
  if (hr) ay += cf(15) * vy[c + ny];
  if (hl) ay += cf(16) * vx[c - ny];
  ay += cf(17) * vx[c];
  if (hl && hd) ay += cf(18) * vx[c + 1 - ny];
  if (hd) ay += cf(19) * vx[c + 1];
  ay += cf(20) * p[c];
  if (hd) ay += cf(21) * p[c + 1];
  double ap = cf(22) * p[c];
  if (hl) ap += cf(23) * vx[c - ny];
  ap += cf(24) * vx[c];
  if (hu) ap += cf(25) * vy[c - 1];
  ap += cf(26) * vy[c];
  if (sub) {
    ax -= sub[c];
    ay -= sub[nc + c];
    ap -= sub[2 * (int64_t)nc + c];
  }
  y[c] = ax;
  y[nc + c] = ay;
  y[2 * (int64_t)nc + c] = ap;
  if (y32) {  // FP32 copy for the FP32 Gram-Schmidt products
    y32[c] = (float)ax;
    y32[nc + c] = (float)ay;
    y32[2 * (int64_t)nc + c] = (float)ap;
  }
}
// Stencil slots of k_apply64: row block (0 vx, 1 vy, 2 p), column block, and the neighbour
// cell (i + di, j + dj) whose unknown the slot multiplies.
struct StencilSlot {
  int8_t row, col, di, dj;
};
__constant__ StencilSlot kSlots[27] = {
    {0, 0, 0, 0},  {0, 0, 0, -1}, {0, 0, 0, 1},  {0, 0, -1, 0}, {0, 0, 1, 0},  {0, 1, -1, 0}, {0, 1, -1, 1},
    {0, 1, 0, 0},  {0, 1, 0, 1},  {0, 2, 0, 0},  {0, 2, 0, 1},  {1, 1, 0, 0},  {1, 1, -1, 0}, {1, 1, 1, 0},
    {1, 1, 0, -1}, {1, 1, 0, 1},  {1, 0, 0, -1}, {1, 0, 0, 0},  {1, 0, 1, -1}, {1, 0, 1, 0},  {1, 2, 0, 0},
    {1, 2, 1, 0},  {2, 2, 0, 0},  {2, 0, 0, -1}, {2, 0, 0, 0},  {2, 1, -1, 0}, {2, 1, 0, 0}};
// coefS[s][c] = w_row(c) coef[s][c] w_col(neighbour): the stencil of W L W, so that the
// scaled product costs one FMA per slot (0 where the neighbour lies outside the grid).
__global__ void k_prescale(const double* __restrict__ coef, const double* __restrict__ w,
                           double* __restrict__ coefS, int32_t nx, int32_t ny, int32_t nc) {
  const int32_t c = (int32_t)(blockIdx.x * blockDim.x + threadIdx.x);
  if (c >= nc) return;
  const int32_t j = c / ny, i = c - j * ny;
#pragma unroll
  for (int s = 0; s < 27; ++s) {
    const StencilSlot q = kSlots[s];
    const int32_t ii = i + q.di, jj = j + q.dj;
    double v = 0.0;
    if (ii >= 0 && ii < ny && jj >= 0 && jj < nx)
      v = w[(int64_t)q.row * nc + c] * coef[(int64_t)s * nc + c] * w[(int64_t)q.col * nc + jj * ny + ii];
    coefS[(int64_t)s * nc + c] = v;
  }
}

// W and the pressure preconditioner factor.
// (winv = 1 / w: the preconditioner multiplies by it instead of dividing by w, the FP64
// divisions having bound its two kernels)
__global__ void k_scaling(const double* __restrict__ coef, const double* __restrict__ etan0, double pscale,
                          double* __restrict__ w, double* __restrict__ prep, double* __restrict__ winv, int64_t nc) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  w[c] = 1.0 / sqrt(fabs(coef[c]));
  w[nc + c] = 1.0 / sqrt(fabs(coef[11 * nc + c]));
  const double pc = coef[22 * nc + c];
  if (pc != 0.0) {  // pressure-condition row
    w[2 * nc + c] = 1.0 / sqrt(fabs(pc));
    prep[c] = 1.0 / pc;
  } else {
    const double s = 2.0 * etan0[c] / (pscale * pscale);  // etan0 is (ynum-1, xnum-1): same cell order
    w[2 * nc + c] = sqrt(s);
    prep[c] = s;
  }
  for (int k = 0; k < 3; ++k) winv[k * nc + c] = 1.0 / w[k * nc + c];
}

// ------------------------------------------------------ FGMRES helpers ---
// Dot products with the Krylov basis V (nv vectors of n, `stride` apart):
// block (b, v) reduces a grid-stride slice of V_v . u, so the blocks of one
// vector run together and stream it (u stays in L2 across vectors).
constexpr int kDotBlocks = 2 * 152;
__global__ void __launch_bounds__(kB) k_mdot(const double* __restrict__ V, int64_t stride, const double* __restrict__ u,
                                             int64_t n, double* __restrict__ partial) {
  const double* a = V + (int64_t)blockIdx.y * stride;
  // four independent partial sums: eight loads in flight per thread
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; k + 3 * step < n; k += 4 * step) {
    const double a0 = __ldcs(a + k), a1 = __ldcs(a + k + step), a2 = __ldcs(a + k + 2 * step),
                 a3 = __ldcs(a + k + 3 * step);
    const double u0 = __ldg(u + k), u1 = __ldg(u + k + step), u2 = __ldg(u + k + 2 * step), u3 = __ldg(u + k + 3 * step);
    s0 += a0 * u0;
    s1 += a1 * u1;
    s2 += a2 * u2;
    s3 += a3 * u3;
  }
  for (; k < n; k += step) s0 += a[k] * u[k];
  double s = (s0 + s1) + (s2 + s3);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ double sh[kB / 32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kB / 32; ++w) t += sh[w];
    partial[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = t;
  }
}
__global__ void k_mdot_final(const double* __restrict__ partial, int nb, double* __restrict__ out) {
  const int v = blockIdx.x;
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) s += partial[(int64_t)v * nb + b];
  __shared__ double sh[kB];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = kB / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[v] = sh[0];
}
// u -= sum_v h[v] V_v.  Each thread owns kAxPer elements and streams four
// basis vectors at a time (16 independent loads in flight).
constexpr int kAxThreads = 256, kAxPer = 4, kAxTile = kAxThreads * kAxPer;
__global__ void __launch_bounds__(kAxThreads) k_maxpy(double* __restrict__ u, const double* __restrict__ V,
                                                      int64_t stride, const double* __restrict__ h, int nv,
                                                      int64_t n) {
  extern __shared__ double hs[];
  for (int v = threadIdx.x; v < nv; v += blockDim.x) hs[v] = h[v];
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kAxTile;
  const bool full = base + kAxTile <= n;
  double ur[kAxPer];
#pragma unroll
  for (int q = 0; q < kAxPer; ++q) {
    const int64_t e = base + q * kAxThreads + threadIdx.x;
    ur[q] = (full || e < n) ? u[e] : 0.0;
  }
  if (full) {
    int v = 0;
    for (; v + 4 <= nv; v += 4) {
      double x[4][kAxPer];
#pragma unroll
      for (int g = 0; g < 4; ++g)
#pragma unroll
        for (int q = 0; q < kAxPer; ++q) x[g][q] = __ldcs(V + (int64_t)(v + g) * stride + base + q * kAxThreads + threadIdx.x);
#pragma unroll
      for (int g = 0; g < 4; ++g)
#pragma unroll
        for (int q = 0; q < kAxPer; ++q) ur[q] -= hs[v + g] * x[g][q];
    }
    for (; v < nv; ++v)
#pragma unroll
      for (int q = 0; q < kAxPer; ++q) ur[q] -= hs[v] * V[(int64_t)v * stride + base + q * kAxThreads + threadIdx.x];
  } else {
    for (int v = 0; v < nv; ++v)
#pragma unroll
      for (int q = 0; q < kAxPer; ++q) {
        const int64_t e = base + q * kAxThreads + threadIdx.x;
        if (e < n) ur[q] -= hs[v] * V[(int64_t)v * stride + e];
      }
  }
#pragma unroll
  for (int q = 0; q < kAxPer; ++q) {
    const int64_t e = base + q * kAxThreads + threadIdx.x;
    if (full || e < n) u[e] = ur[q];
  }
}
// dst may alias src (in-place scaling)
__global__ void k_scale_copy(double* dst, const double* src, double a, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) dst[k] = a * src[k];
}
// ---- Gram-Schmidt on FP32 copies of the basis (mixed method, late iterations) ----
// Inexact Krylov theory (Simoncini & Szyld 2003; Bouras & Fraysse 2005) lets the error an
// iteration adds to the Arnoldi relation grow like 1/|r| once the residual is small.  The
// mixed method therefore keeps an FP32 copy of every basis vector (slots ld32 floats apart,
// ld32 a multiple of 4, padding zero) and, below a residual threshold, projects with FP32
// products on those copies: half the bytes, and the FP32 pipe instead of the FP64 one that
// bounds k_mdot / k_maxpy.  The new direction itself stays FP64, and its norm is measured.
//
// dots: block (b, g) reduces a grid-stride slice of V32_v . u32 for the four vectors
// v = 4g .. 4g+3 (< nv) over float4 chunks (n4 = ld32 / 4), so each chunk of u32 is read once
// per four vectors; FP32 partial sums per thread (about 50 chunks each at 14M unknowns) go to
// FP64 for the block reduction.  partial[v * gridDim.x + b].
constexpr int kDot32Vecs = 4;
__global__ void __launch_bounds__(kB) k_mdot32(const float* __restrict__ V, int64_t ld, const float* __restrict__ u,
                                               int64_t n4, int nv, double* __restrict__ partial) {
  const int v0 = blockIdx.y * kDot32Vecs;
  const int nvb = min(kDot32Vecs, nv - v0);
  const float4* b = reinterpret_cast<const float4*>(u);
  const float4* a[kDot32Vecs];
#pragma unroll
  for (int g = 0; g < kDot32Vecs; ++g)
    a[g] = reinterpret_cast<const float4*>(V + (int64_t)(v0 + min(g, nvb - 1)) * ld);
  float4 s[kDot32Vecs];
#pragma unroll
  for (int g = 0; g < kDot32Vecs; ++g) s[g] = make_float4(0.f, 0.f, 0.f, 0.f);
  auto acc4 = [](const float4 x, const float4 y, float4& t) {
    t.x = fmaf(x.x, y.x, t.x);
    t.y = fmaf(x.y, y.y, t.y);
    t.z = fmaf(x.z, y.z, t.z);
    t.w = fmaf(x.w, y.w, t.w);
  };
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; k + step < n4; k += 2 * step) {  // up to ten 16-byte loads in flight
    const float4 u0 = __ldg(b + k), u1 = __ldg(b + k + step);
    float4 x0[kDot32Vecs], x1[kDot32Vecs];
#pragma unroll
    for (int g = 0; g < kDot32Vecs; ++g)
      if (g < nvb) {
        x0[g] = __ldcs(a[g] + k);
        x1[g] = __ldcs(a[g] + k + step);
      }
#pragma unroll
    for (int g = 0; g < kDot32Vecs; ++g)
      if (g < nvb) {
        acc4(x0[g], u0, s[g]);
        acc4(x1[g], u1, s[g]);
      }
  }
  if (k < n4) {
    const float4 u0 = __ldg(b + k);
#pragma unroll
    for (int g = 0; g < kDot32Vecs; ++g)
      if (g < nvb) acc4(__ldcs(a[g] + k), u0, s[g]);
  }
  // lanes and warp reduced as double-float pairs on the FP32 pipe (an FP64 reduction would
  // convert on the FP64 pipe); the block's eight warp sums are added in FP64
  __shared__ double sh[kDot32Vecs][kB / 32];
#pragma unroll
  for (int g = 0; g < kDot32Vecs; ++g) {
    float S = s[g].x, C = 0.f;
    two_sum_acc(s[g].y, 0.f, S, C);
    two_sum_acc(s[g].z, 0.f, S, C);
    two_sum_acc(s[g].w, 0.f, S, C);
    for (int o = 16; o > 0; o >>= 1) {
      const float s2 = __shfl_xor_sync(0xffffffffu, S, o), c2 = __shfl_xor_sync(0xffffffffu, C, o);
      two_sum_acc(s2, c2, S, C);
    }
    if ((threadIdx.x & 31) == 0) sh[g][threadIdx.x >> 5] = f2d(S) + f2d(C);
  }
  __syncthreads();
  if ((int)threadIdx.x < nvb) {
    double t = 0.0;
    for (int w = 0; w < kB / 32; ++w) t += sh[threadIdx.x][w];
    partial[(int64_t)(v0 + threadIdx.x) * gridDim.x + blockIdx.x] = t;
  }
}
// float4 chunks per thread of the split-basis updates (template parameter P): 2 on long vectors,
// 1 where two would leave the GPU's 152 SMs with few blocks
constexpr int64_t kAxP2Chunks = (int64_t)152 * 8 * kAxThreads * 2;  // n/4 from which P = 2

// ---- The mixed method's Arnoldi step in double-float ----
// On this part the FP64 pipe (about 1.6 FMA per SM per clock, measured) also executes the
// FP64 <-> FP32 conversion instructions (about 2 per SM per clock), so FP64 arithmetic and
// conversions, not HBM, bound elementwise kernels on FP64 vectors.  The mixed method therefore
// keeps each Krylov vector as the unevaluated sum hi + lo of two FP32 vectors (about 2^-47
// relative), forms the operator product and the Gram-Schmidt products from FMA-based exact
// products (TwoProduct: p + e = a b exactly with e = fma(a, b, -p)) summed with Knuth's TwoSum
// (the Dot2 scheme of Ogita, Rump & Oishi, SIAM J. Sci. Comput. 26, 2005), and converts with
// integer operations; once its residual is small (gs_relax) the Gram-Schmidt products drop to
// FP32 on the hi parts.
// Every kernel of the step then runs on the FP32 pipe and streams HBM; the Hessenberg matrix
// and the Givens rotations stay FP64 on the host.  The _rn intrinsics keep the compiler from
// contracting a product into a following sum, which would break the error-free transforms.

// d = (W L W) x - v_k for the mixed method: x = Z_k (FP32, exact), the stencil as the pair
// ch + cl, v_k = vh + vl; d is written as the normalised pair (dh, dl).  Same cells, slots
// and neighbour order as k_apply64.
__global__ void __launch_bounds__(kB) k_apply_df(const float* __restrict__ ch, const float* __restrict__ cl,
                                                 const float* __restrict__ x, const float* __restrict__ vh,
                                                 const float* __restrict__ vl, float* __restrict__ dh,
                                                 float* __restrict__ dl, int32_t nx, int32_t ny, int32_t nc) {
  const int32_t c = (int32_t)(blockIdx.x * blockDim.x + threadIdx.x);
  if (c >= nc) return;
  const int32_t j = c / ny, i = c - j * ny;
  const float *vx = x, *vy = x + nc, *p = x + 2 * (int64_t)nc;
  const bool hu = i > 0, hd = i < ny - 1, hl = j > 0, hr = j < nx - 1;
  float s, e;
  auto t = [&](int slot, float xv) {
    df_axpy_acc(__ldg(&ch[(int64_t)slot * nc + c]), __ldg(&cl[(int64_t)slot * nc + c]), xv, s, e);
  };
  auto out = [&](int64_t o) {
    two_sum_acc(-vh[o], -vl[o], s, e);
    float h, l;
    df_norm(s, e, h, l);
    dh[o] = h;
    dl[o] = l;
  };
  s = e = 0.f;
  t(0, vx[c]);
  if (hl) t(1, vx[c - ny]);
  if (hr) t(2, vx[c + ny]);
  if (hu) t(3, vx[c - 1]);
  if (hd) t(4, vx[c + 1]);
  if (hu) t(5, vy[c - 1]);
  if (hu && hr) t(6, vy[c + ny - 1]);
  t(7, vy[c]);
  if (hr) t(8, vy[c + ny]);
  t(9, p[c]);
  if (hr) t(10, p[c + ny]);
  out(c);
  s = e = 0.f;
  t(11, vy[c]);
  if (hu) t(12, vy[c - 1]);
  if (hd) t(13, vy[c + 1]);
  if (hl) t(14, vy[c - ny]);
  if (hr) t(15, vy[c + ny]);
  if (hl) t(16, vx[c - ny]);
  t(17, vx[c]);
  if (hl && hd) t(18, vx[c + 1 - ny]);
  if (hd) t(19, vx[c + 1]);
  t(20, p[c]);
  if (hd) t(21, p[c + 1]);
  out(nc + (int64_t)c);
  s = e = 0.f;
  t(22, p[c]);
  if (hl) t(23, vx[c - ny]);
  t(24, vx[c]);
  if (hu) t(25, vy[c - 1]);
  t(26, vy[c]);
  out(2 * (int64_t)nc + c);
}
// dots: block (b, g) reduces a grid-stride slice of (Vh_v + Vl_v) . (Vh_{nv-1} + Vl_{nv-1}) for
// v = G g .. G g + G - 1 (< nv) over float4 chunks, U chunks per thread and step; the last slot
// holds the new direction, so its own product is |d|^2.  partial[v * gridDim.x + b].
constexpr int kDfVecs = 2, kDfUnroll = 2;
__global__ void __launch_bounds__(kB) k_mdot_df(const float* __restrict__ Vh, const float* __restrict__ Vl, int64_t ld,
                                                int64_t n4, int nv, double* __restrict__ partial) {
  constexpr int G = kDfVecs, U = kDfUnroll;
  const int v0 = blockIdx.y * G;
  const int nvb = min(G, nv - v0);
  const float4* bh = reinterpret_cast<const float4*>(Vh + (int64_t)(nv - 1) * ld);
  const float4* bl = reinterpret_cast<const float4*>(Vl + (int64_t)(nv - 1) * ld);
  const float4 *ah[G], *al[G];
#pragma unroll
  for (int g = 0; g < G; ++g) {
    ah[g] = reinterpret_cast<const float4*>(Vh + (int64_t)(v0 + min(g, nvb - 1)) * ld);
    al[g] = reinterpret_cast<const float4*>(Vl + (int64_t)(v0 + min(g, nvb - 1)) * ld);
  }
  float4 s[G], cs[G];
#pragma unroll
  for (int g = 0; g < G; ++g) s[g] = cs[g] = make_float4(0.f, 0.f, 0.f, 0.f);
  auto acc4 = [](const float4 xh, const float4 xl, const float4 yh, const float4 yl, float4& s, float4& c) {
    df_fma_acc(xh.x, xl.x, yh.x, yl.x, s.x, c.x);
    df_fma_acc(xh.y, xl.y, yh.y, yl.y, s.y, c.y);
    df_fma_acc(xh.z, xl.z, yh.z, yl.z, s.z, c.z);
    df_fma_acc(xh.w, xl.w, yh.w, yl.w, s.w, c.w);
  };
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; k + (U - 1) * step < n4; k += U * step) {
    float4 yh[U], yl[U], xh[U][G], xl[U][G];
#pragma unroll
    for (int q = 0; q < U; ++q) {
      yh[q] = __ldg(bh + k + q * step);
      yl[q] = __ldg(bl + k + q * step);
#pragma unroll
      for (int g = 0; g < G; ++g)
        if (g < nvb) {
          xh[q][g] = __ldcs(ah[g] + k + q * step);
          xl[q][g] = __ldcs(al[g] + k + q * step);
        }
    }
#pragma unroll
    for (int q = 0; q < U; ++q)
#pragma unroll
      for (int g = 0; g < G; ++g)
        if (g < nvb) acc4(xh[q][g], xl[q][g], yh[q], yl[q], s[g], cs[g]);
  }
  for (; k < n4; k += step) {
    const float4 yh = __ldg(bh + k), yl = __ldg(bl + k);
#pragma unroll
    for (int g = 0; g < G; ++g)
      if (g < nvb) acc4(__ldcs(ah[g] + k), __ldcs(al[g] + k), yh, yl, s[g], cs[g]);
  }
  // the thread's four lanes and then the warp reduced as double-float pairs (FP32 pipe); only
  // the eight warp sums of the block are added in FP64
  __shared__ double sh[G][kB / 32];
#pragma unroll
  for (int g = 0; g < G; ++g) {
    float S = s[g].x, C = cs[g].x;
    two_sum_acc(s[g].y, cs[g].y, S, C);
    two_sum_acc(s[g].z, cs[g].z, S, C);
    two_sum_acc(s[g].w, cs[g].w, S, C);
    for (int o = 16; o > 0; o >>= 1) {
      const float s2 = __shfl_xor_sync(0xffffffffu, S, o), c2 = __shfl_xor_sync(0xffffffffu, C, o);
      two_sum_acc(s2, c2, S, C);
    }
    if ((threadIdx.x & 31) == 0) sh[g][threadIdx.x >> 5] = f2d(S) + f2d(C);
  }
  __syncthreads();
  if ((int)threadIdx.x < nvb) {
    double t = 0.0;
    for (int w = 0; w < kB / 32; ++w) t += sh[threadIdx.x][w];
    partial[(int64_t)(v0 + threadIdx.x) * gridDim.x + blockIdx.x] = t;
  }
}
// u = (uh + ul) - sum_v h[v] (Vh_v + Vl_v) in place (u the slot after the nv basis vectors),
// normalised; partial[block] = the block's sum of u^2.  A thread owns P float4 chunks of
// consecutive elements and streams four basis vectors at a time.
template <int P>
__global__ void __launch_bounds__(kAxThreads) k_maxpy_df(const float* __restrict__ Vh, const float* __restrict__ Vl,
                                                         int64_t ld, const double* __restrict__ h, int nv,
                                                         float* __restrict__ uhp, float* __restrict__ ulp,
                                                         double* __restrict__ partial) {
  extern __shared__ float hsd[];  // hi parts at [0, nv), lo parts at [nv, 2 nv)
  for (int v = threadIdx.x; v < nv; v += blockDim.x) split_df(h[v], hsd[v], hsd[nv + v]);
  __syncthreads();
  const int64_t n4 = ld >> 2;
  float4* uh = reinterpret_cast<float4*>(uhp);
  float4* ul = reinterpret_cast<float4*>(ulp);
  int64_t ch[P];
  bool ok[P];
  float4 as[P], ac[P];
#pragma unroll
  for (int q = 0; q < P; ++q) {
    ch[q] = (int64_t)blockIdx.x * (kAxThreads * P) + q * kAxThreads + threadIdx.x;
    ok[q] = ch[q] < n4;
    as[q] = ac[q] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  auto acc4 = [](float bh, float bl, const float4 xh, const float4 xl, float4& s, float4& c) {
    df_fma_acc(xh.x, xl.x, bh, bl, s.x, c.x);
    df_fma_acc(xh.y, xl.y, bh, bl, s.y, c.y);
    df_fma_acc(xh.z, xl.z, bh, bl, s.z, c.z);
    df_fma_acc(xh.w, xl.w, bh, bl, s.w, c.w);
  };
  int v = 0;
  for (; v + 4 <= nv; v += 4) {
    float4 xh[4][P], xl[4][P];
#pragma unroll
    for (int g = 0; g < 4; ++g)
#pragma unroll
      for (int q = 0; q < P; ++q) {
        xh[g][q] = ok[q] ? __ldcs(reinterpret_cast<const float4*>(Vh + (int64_t)(v + g) * ld) + ch[q]) : zero;
        xl[g][q] = ok[q] ? __ldcs(reinterpret_cast<const float4*>(Vl + (int64_t)(v + g) * ld) + ch[q]) : zero;
      }
#pragma unroll
    for (int g = 0; g < 4; ++g)
#pragma unroll
      for (int q = 0; q < P; ++q) acc4(hsd[v + g], hsd[nv + v + g], xh[g][q], xl[g][q], as[q], ac[q]);
  }
  for (; v < nv; ++v)
#pragma unroll
    for (int q = 0; q < P; ++q)
      if (ok[q])
        acc4(hsd[v], hsd[nv + v], __ldcs(reinterpret_cast<const float4*>(Vh + (int64_t)v * ld) + ch[q]),
             __ldcs(reinterpret_cast<const float4*>(Vl + (int64_t)v * ld) + ch[q]), as[q], ac[q]);
  float sh2 = 0.f, sl2 = 0.f;  // sum of u^2 as a pair
  auto fin = [&](float& xh, float& xl, float s, float c) {
    float t = 0.f, e = 0.f;
    two_sum_acc(xh, xl, t, e);
    two_sum_acc(-s, -c, t, e);
    df_norm(t, e, xh, xl);
    df_fma_acc(xh, xl, xh, xl, sh2, sl2);
  };
#pragma unroll
  for (int q = 0; q < P; ++q) {
    if (!ok[q]) continue;
    float4 xh = uh[ch[q]], xl = ul[ch[q]];
    fin(xh.x, xl.x, as[q].x, ac[q].x);
    fin(xh.y, xl.y, as[q].y, ac[q].y);
    fin(xh.z, xl.z, as[q].z, ac[q].z);
    fin(xh.w, xl.w, as[q].w, ac[q].w);
    uh[ch[q]] = xh;
    ul[ch[q]] = xl;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const float s2 = __shfl_xor_sync(0xffffffffu, sh2, o), c2 = __shfl_xor_sync(0xffffffffu, sl2, o);
    two_sum_acc(s2, c2, sh2, sl2);
  }
  __shared__ double sh[kAxThreads / 32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = f2d(sh2) + f2d(sl2);
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kAxThreads / 32; ++w) t += sh[w];
    partial[blockIdx.x] = t;
  }
}
// FP32 projection once the residual is small: u = (uh + ul) - sum_v h[v] Vh_v in place (u the
// slot after the nv basis vectors), the sum over the FP32 hi parts in FP32 and the update in
// double-float, so that u keeps the accuracy of the operator product (d = A z - v cancels most
// of A z: rounding d's own terms to FP32 first cost FGMRES iterations);
// partial[block] = the block's sum of u^2.
template <int P>
__global__ void __launch_bounds__(kAxThreads) k_maxpy32(float* __restrict__ V, float* __restrict__ ulp, int64_t ld,
                                                        const double* __restrict__ h, int nv,
                                                        double* __restrict__ partial) {
  extern __shared__ float hs32[];
  for (int v = threadIdx.x; v < nv; v += blockDim.x) hs32[v] = d2f(h[v]);
  __syncthreads();
  const int64_t n4 = ld >> 2;
  float4* u = reinterpret_cast<float4*>(V + (int64_t)nv * ld);
  int64_t ch[P];
  bool ok[P];
  float4 acc[P];
#pragma unroll
  for (int q = 0; q < P; ++q) {
    ch[q] = (int64_t)blockIdx.x * (kAxThreads * P) + q * kAxThreads + threadIdx.x;
    ok[q] = ch[q] < n4;
    acc[q] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  auto fma4 = [](float a, const float4 x, float4& s) {
    s.x = fmaf(a, x.x, s.x);
    s.y = fmaf(a, x.y, s.y);
    s.z = fmaf(a, x.z, s.z);
    s.w = fmaf(a, x.w, s.w);
  };
  int v = 0;
  for (; v + 4 <= nv; v += 4) {
    float4 x[4][P];
#pragma unroll
    for (int g = 0; g < 4; ++g)
#pragma unroll
      for (int q = 0; q < P; ++q)
        x[g][q] = ok[q] ? __ldcs(reinterpret_cast<const float4*>(V + (int64_t)(v + g) * ld) + ch[q]) : zero;
#pragma unroll
    for (int g = 0; g < 4; ++g)
#pragma unroll
      for (int q = 0; q < P; ++q) fma4(hs32[v + g], x[g][q], acc[q]);
  }
  for (; v < nv; ++v)
#pragma unroll
    for (int q = 0; q < P; ++q)
      if (ok[q]) fma4(hs32[v], __ldcs(reinterpret_cast<const float4*>(V + (int64_t)v * ld) + ch[q]), acc[q]);
  float4* ul = reinterpret_cast<float4*>(ulp);
  float sh2 = 0.f, sl2 = 0.f;  // sum of u^2 as a pair
  auto fin = [&](float& xh, float& xl, float a) {
    float t = 0.f, e = 0.f;
    two_sum_acc(xh, xl, t, e);
    two_sum_acc(-a, 0.f, t, e);
    df_norm(t, e, xh, xl);
    df_fma_acc(xh, xl, xh, xl, sh2, sl2);
  };
#pragma unroll
  for (int q = 0; q < P; ++q) {
    if (!ok[q]) continue;
    float4 xh = u[ch[q]], xl = ul[ch[q]];
    fin(xh.x, xl.x, acc[q].x);
    fin(xh.y, xl.y, acc[q].y);
    fin(xh.z, xl.z, acc[q].z);
    fin(xh.w, xl.w, acc[q].w);
    u[ch[q]] = xh;
    ul[ch[q]] = xl;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const float s2 = __shfl_xor_sync(0xffffffffu, sh2, o), c2 = __shfl_xor_sync(0xffffffffu, sl2, o);
    two_sum_acc(s2, c2, sh2, sl2);
  }
  __shared__ double sh[kAxThreads / 32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = f2d(sh2) + f2d(sl2);
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kAxThreads / 32; ++w) t += sh[w];
    partial[blockIdx.x] = t;
  }
}
// (vh + vl) *= ah + al in place, normalised
__global__ void k_scale_df(float* __restrict__ vh, float* __restrict__ vl, float ah, float al, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float xh = vh[k], xl = vl[k];
  const float p = __fmul_rn(xh, ah);
  const float e = fmaf(xl, ah, fmaf(xh, al, fmaf(xh, ah, -p)));
  float h, l;
  df_norm(p, e, h, l);
  vh[k] = h;
  vl[k] = l;
}
// (vh, vl) = split(a src) (the first basis vector of a cycle, from the FP64 residual)
__global__ void k_split_scale(float* __restrict__ vh, float* __restrict__ vl, const double* __restrict__ src, double a,
                              int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) split_df(a * src[k], vh[k], vl[k]);
}
// u -= sum_v h[v] Z_v (FP32 directions): the sum in double-float, subtracted from the FP64 u
constexpr int kUpdVecs = 8;
__global__ void k_update_df(double* __restrict__ u, const float* __restrict__ Z, int64_t stride,
                            const double* __restrict__ h, int nv, int64_t n) {
  extern __shared__ float ysd[];  // hi parts at [0, nv), lo parts at [nv, 2 nv)
  for (int v = threadIdx.x; v < nv; v += blockDim.x) split_df(h[v], ysd[v], ysd[nv + v]);
  __syncthreads();
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  float s = 0.f, c = 0.f;
  int v = 0;
  for (; v + kUpdVecs <= nv; v += kUpdVecs) {
    float z[kUpdVecs];
#pragma unroll
    for (int g = 0; g < kUpdVecs; ++g) z[g] = __ldcs(Z + (int64_t)(v + g) * stride + k);
#pragma unroll
    for (int g = 0; g < kUpdVecs; ++g) df_axpy_acc(ysd[v + g], ysd[nv + v + g], z[g], s, c);
  }
  for (; v < nv; ++v) df_axpy_acc(ysd[v], ysd[nv + v], Z[(int64_t)v * stride + k], s, c);
  u[k] -= f2d(s) + f2d(c);
}
// The mixed method's FP32 copies of the scaled system: the W L W stencil as pairs (ch, cl),
// the four pressure-coupling slots 9, 10, 20, 21 of the assembled stencil (cq), 1/w (winv32)
// and prep * winv_p (pw32), the pressure factor of the preconditioner's input.
__global__ void k_split_setup(const double* __restrict__ coefS, const double* __restrict__ coef,
                              const double* __restrict__ winv, const double* __restrict__ prep,
                              float* __restrict__ ch, float* __restrict__ cl, float* __restrict__ cq,
                              float* __restrict__ winv32, float* __restrict__ pw32, int64_t nc) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  for (int s = 0; s < 27; ++s) split_df(coefS[s * nc + c], ch[s * nc + c], cl[s * nc + c]);
  const int slots[4] = {9, 10, 20, 21};
  for (int q = 0; q < 4; ++q) cq[q * nc + c] = d2f(coef[slots[q] * nc + c]);
  for (int k = 0; k < 3; ++k) winv32[k * nc + c] = d2f(winv[k * nc + c]);
  pw32[c] = d2f(prep[c] * winv[2 * nc + c]);
}
// FP32 preconditioner input of the mixed method from the basis vector's hi part rh:
// zhat_p = (prep winv_p rh_p) winv_p into Z_k, and the velocity right-hand sides
// f = winv_u rh_u - L_up z_p for the V-cycle (as k_prec_in, in FP32).
__global__ void k_prec_in32(const float* __restrict__ cq, const float* __restrict__ rh, const float* __restrict__ winv32,
                            const float* __restrict__ pw32, float* __restrict__ Zk, float* __restrict__ fx,
                            float* __restrict__ fy, int32_t nx, int32_t ny) {
  const int64_t nc = (int64_t)nx * ny;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const int32_t j = (int32_t)c / ny, i = (int32_t)c - j * ny;
  auto z = [&](int64_t k) { return pw32[k] * rh[2 * nc + k]; };
  const float zc = z(c);
  Zk[2 * nc + c] = zc * winv32[2 * nc + c];
  float gx = cq[c] * zc;
  if (j < nx - 1) gx = fmaf(cq[nc + c], z(c + ny), gx);
  float gy = cq[2 * nc + c] * zc;
  if (i < ny - 1) gy = fmaf(cq[3 * nc + c], z(c + 1), gy);
  fx[c] = rh[c] * winv32[c] - gx;
  fy[c] = rh[nc + c] * winv32[nc + c] - gy;
}
__global__ void k_prec_out32(const float* __restrict__ ux, const float* __restrict__ uy,
                             const float* __restrict__ winv32, float* __restrict__ Zk, int64_t nc) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  Zk[c] = ux[c] * winv32[c];
  Zk[nc + c] = uy[c] * winv32[nc + c];
}
// dst = a src (dst may alias src)
__global__ void k_scale_copy2(double* dst, const double* src, double a, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) dst[k] = a * src[k];
}
// BiCGStab vector updates
__global__ void k_bicg_p(double* __restrict__ p, const double* __restrict__ r, const double* __restrict__ v, double beta,
                         double omega, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) p[k] = r[k] + beta * (p[k] - omega * v[k]);
}
__global__ void k_bicg_s(double* __restrict__ s, const double* __restrict__ r, const double* __restrict__ v, double alpha,
                         int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) s[k] = r[k] - alpha * v[k];
}
__global__ void k_bicg_xr(double* __restrict__ x, double* __restrict__ r, const double* __restrict__ ph,
                          const double* __restrict__ sh, const double* __restrict__ s, const double* __restrict__ t,
                          double alpha, double omega, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  x[k] += alpha * ph[k] + omega * sh[k];
  r[k] = s[k] - omega * t[k];
}
// dst = a - b (elementwise)
__global__ void k_sub(double* __restrict__ dst, const double* __restrict__ a, const double* __restrict__ b, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) dst[k] = a[k] - b[k];
}
// dst = a .* b or a ./ b (dst may alias a)
__global__ void k_mul(double* dst, const double* a, const double* __restrict__ b, int64_t n, int div) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) dst[k] = div ? a[k] / b[k] : a[k] * b[k];
}
__global__ void k_abs_sub(double* __restrict__ dst, const double* __restrict__ a, const double* __restrict__ b, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) dst[k] = fabs(a[k] - b[k]);
}

// interleaved host layout <-> SoA device layout
__global__ void k_interleave(const double* __restrict__ soa, double* __restrict__ il, int64_t nc) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  il[3 * c] = soa[c];
  il[3 * c + 1] = soa[nc + c];
  il[3 * c + 2] = soa[2 * nc + c];
}
__global__ void k_deinterleave(const double* __restrict__ il, double* __restrict__ soa, int64_t nc) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  soa[c] = il[3 * c];
  soa[nc + c] = il[3 * c + 1];
  soa[2 * nc + c] = il[3 * c + 2];
}

// ----------------------------------------------------------- multigrid ---
// The V-cycle runs in FP32 (the mixed-precision method) or in FP64 (the plain method): every
// multigrid kernel is a template on the level arithmetic T.  The transfer weights and the
// boundary-condition coefficients of the coarse operators stay FP32 tables in both.
struct Axis2 { int32_t* idx; float* w; };   // prolongation: 2 (coarse index, weight) per fine index
struct AxisR { int32_t* idx; float* w; };   // restriction: kRmax (fine index, weight) per coarse index

// Host view of one level; the arrays hold T = float or double (StokesState::mg64).
struct Level {
  int32_t nx = 0, ny = 0;
  int64_t nc = 0;
  void *X = nullptr, *Y = nullptr;                        // [9][nc]
  void *ux = nullptr, *uy = nullptr, *fx = nullptr, *fy = nullptr, *rx = nullptr, *ry = nullptr;
  void *etas = nullptr, *etan = nullptr;                  // [(ny+1)(nx+1)], [ny nx]
  void *xstp = nullptr, *ystp = nullptr, *xstpc = nullptr, *ystpc = nullptr;
  int32_t *kx = nullptr, *ky = nullptr;                   // nodes of this level in the finer level
  // transfers to the next coarser level
  Axis2 pvx_x{}, pvx_y{}, pvy_x{}, pvy_y{};
  AxisR rvx_x{}, rvx_y{}, rvy_x{}, rvy_y{};
  // host geometry
  std::vector<double> x, y;                               // basic node coordinates
};

struct B2 { float topx, botx, topy, boty, leftx, rightx, lefty, righty; };

// Coarse-level velocity stencil from averaged viscosity (same formulas as the
// fine assembly, uniform boundary-condition coefficients, no stabilisation).
template <class T>
__global__ void k_redisc(int32_t nx, int32_t ny, const T* __restrict__ etas, const T* __restrict__ etan,
                         const T* __restrict__ xstp, const T* __restrict__ ystp, const T* __restrict__ xstpc,
                         const T* __restrict__ ystpc, B2 b, T* __restrict__ X, T* __restrict__ Y) {
  const int64_t nc = (int64_t)nx * ny;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const int32_t i = (int32_t)(c % ny) + 1, j = (int32_t)(c / ny) + 1;  // 1-based cell
  const int32_t xnum = nx + 1, ynum = ny + 1;
  auto eS = [&](int ii, int jj) { return etas[(int64_t)(jj - 1) * ynum + (ii - 1)]; };
  auto eN = [&](int ii, int jj) { return etan[(int64_t)(jj - 1) * ny + (ii - 1)]; };
  const T two = T(2);
  T x[9] = {0}, y[9] = {0};
  if (j < xnum - 1) {
    const bool left = j == 1, right2 = j >= xnum - 2, top = i == 1, bot = i >= ynum - 1;
    const T cL = two * eN(i, j) / xstp[j - 1] / xstpc[j];
    const T cR = two * eN(i, j + 1) / xstp[j] / xstpc[j];
    const T cU = eS(i, j + 1) / ystpc[i - 1] / ystp[i - 1];
    const T cD = eS(i + 1, j + 1) / ystpc[i] / ystp[i - 1];
    T C = -(cL + cR) - (cU + cD);
    const T gUL = eS(i, j + 1) / xstpc[j] / ystp[i - 1], gUR = -gUL;
    const T gLL = -eS(i + 1, j + 1) / xstpc[j] / ystp[i - 1], gLR = -gLL;
    if (left) C += (T)b.leftx * cL; else x[1] = cL;
    if (right2) C += (T)b.rightx * cR; else x[2] = cR;
    if (top) C += (T)b.topx * cU; else x[3] = cU;
    if (bot) C += (T)b.botx * cD; else x[4] = cD;
    x[0] = C;
    T vUL = 0, vUR = 0, vLL = 0, vLR = 0;
    if (!top) { vUL = gUL; vUR = gUR; } else { vLL = (T)b.topy * gUL; vLR = (T)b.topy * gUR; }
    if (!bot) { vLL += gLL; vLR += gLR; } else { vUL += (T)b.boty * gLL; vUR += (T)b.boty * gLR; }
    x[5] = vUL; x[6] = vUR; x[7] = vLL; x[8] = vLR;
  } else {
    x[0] = T(1);
  }
  if (i < ynum - 1) {
    const bool top = i == 1, bot2 = i >= ynum - 2, left = j == 1, right = j >= xnum - 1;
    const T cU = two * eN(i, j) / ystp[i - 1] / ystpc[i];
    const T cD = two * eN(i + 1, j) / ystp[i] / ystpc[i];
    const T cL = eS(i + 1, j) / xstpc[j - 1] / xstp[j - 1];
    const T cR = eS(i + 1, j + 1) / xstpc[j] / xstp[j - 1];
    T C = -(cU + cD) - (cL + cR);
    const T hUL = eS(i + 1, j) / ystpc[i] / xstp[j - 1], hLL = -hUL;
    const T hUR = -eS(i + 1, j + 1) / ystpc[i] / xstp[j - 1], hLR = -hUR;
    if (top) C += (T)b.topy * cU; else y[1] = cU;
    if (bot2) C += (T)b.boty * cD; else y[2] = cD;
    if (left) C += (T)b.lefty * cL; else y[3] = cL;
    if (right) C += (T)b.righty * cR; else y[4] = cR;
    y[0] = C;
    T xUL = 0, xUR = 0, xLL = 0, xLR = 0;
    if (!left) { xUL = hUL; xLL = hLL; } else { xUR = (T)b.leftx * hUL; xLR = (T)b.leftx * hLL; }
    if (!right) { xUR += hUR; xLR += hLR; } else { xUL += (T)b.rightx * hUR; xLL += (T)b.rightx * hLR; }
    y[5] = xUL; y[6] = xUR; y[7] = xLL; y[8] = xLR;
  } else {
    y[0] = T(1);
  }
  for (int k = 0; k < 9; ++k) { X[(int64_t)k * nc + c] = x[k]; Y[(int64_t)k * nc + c] = y[k]; }
}

// Level 0 takes the assembled FP64 velocity block.
template <class T>
__global__ void k_level0(const double* __restrict__ coef, T* __restrict__ X, T* __restrict__ Y, int64_t nc) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  for (int k = 0; k < 9; ++k) {
    X[(int64_t)k * nc + c] = (T)coef[(int64_t)k * nc + c];
    Y[(int64_t)k * nc + c] = (T)coef[(int64_t)(11 + k) * nc + c];
  }
}
template <class T>
__global__ void k_to_real(const double* __restrict__ a, T* __restrict__ b, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) b[k] = (T)a[k];
}
// Arithmetic averages of the finer level's viscosity onto this level.  (Geometric and harmonic
// averages, for the node or the cell viscosity or both, all needed more FGMRES iterations on the
// rift's systems, or failed to converge.)
template <class T>
__global__ void k_coarsen_eta(const T* __restrict__ es_f, const T* __restrict__ en_f, int32_t nxf, int32_t nyf,
                              T* __restrict__ es_c, T* __restrict__ en_c, int32_t nxc, int32_t nyc,
                              const int32_t* __restrict__ kx, const int32_t* __restrict__ ky) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nnode = (int64_t)(nxc + 1) * (nyc + 1);
  if (t < nnode) {
    const int32_t I = (int32_t)(t % (nyc + 1)), J = (int32_t)(t / (nyc + 1));
    const int32_t fi = ky[I], fj = kx[J];
    T s = 0; int n = 0;
    for (int32_t jj = max(fj - 1, 0); jj <= min(fj + 1, nxf); ++jj)
      for (int32_t ii = max(fi - 1, 0); ii <= min(fi + 1, nyf); ++ii) { s += es_f[(int64_t)jj * (nyf + 1) + ii]; ++n; }
    es_c[t] = s / (T)n;
  }
  if (t < (int64_t)nxc * nyc) {
    const int32_t I = (int32_t)(t % nyc), J = (int32_t)(t / nyc);
    T s = 0; int n = 0;
    for (int32_t jj = kx[J]; jj < kx[J + 1]; ++jj)
      for (int32_t ii = ky[I]; ii < ky[I + 1]; ++ii) { s += en_f[(int64_t)jj * nyf + ii]; ++n; }
    en_c[t] = s / (T)n;
  }
}

// Velocity-block product of one row kind at cell c.
template <class T>
__device__ __forceinline__ T rowx(const T* __restrict__ X, const T* ux, const T* uy, int64_t c, int32_t i, int32_t j,
                                  int32_t nx, int32_t ny, int64_t nc, bool skip_center) {
  const bool hu = i > 0, hd = i < ny - 1, hl = j > 0, hr = j < nx - 1;
  T a = skip_center ? T(0) : X[c] * ux[c];
  if (hl) a += X[nc + c] * ux[c - ny];
  if (hr) a += X[2 * nc + c] * ux[c + ny];
  if (hu) a += X[3 * nc + c] * ux[c - 1];
  if (hd) a += X[4 * nc + c] * ux[c + 1];
  if (hu) a += X[5 * nc + c] * uy[c - 1];
  if (hu && hr) a += X[6 * nc + c] * uy[c + ny - 1];
  a += X[7 * nc + c] * uy[c];
  if (hr) a += X[8 * nc + c] * uy[c + ny];
  return a;
}
template <class T>
__device__ __forceinline__ T rowy(const T* __restrict__ Y, const T* ux, const T* uy, int64_t c, int32_t i, int32_t j,
                                  int32_t nx, int32_t ny, int64_t nc, bool skip_center) {
  const bool hu = i > 0, hd = i < ny - 1, hl = j > 0, hr = j < nx - 1;
  T a = skip_center ? T(0) : Y[c] * uy[c];
  if (hu) a += Y[nc + c] * uy[c - 1];
  if (hd) a += Y[2 * nc + c] * uy[c + 1];
  if (hl) a += Y[3 * nc + c] * uy[c - ny];
  if (hr) a += Y[4 * nc + c] * uy[c + ny];
  if (hl) a += Y[5 * nc + c] * ux[c - ny];
  a += Y[6 * nc + c] * ux[c];
  if (hl && hd) a += Y[7 * nc + c] * ux[c + 1 - ny];
  if (hd) a += Y[8 * nc + c] * ux[c + 1];
  return a;
}

// Device view of one multigrid level (transfer tables point to the next coarser level).
template <class T>
struct LevelDev {
  int32_t nx, ny;
  int64_t nc;
  const T *X, *Y;
  T *ux, *uy, *fx, *fy, *rx, *ry;
  Axis2 pvx_x, pvx_y, pvy_x, pvy_y;
  AxisR rvx_x, rvx_y, rvy_x, rvy_y;
};

// Red-black Gauss-Seidel update of the t-th cell of one color: comp 0 updates vx,
// 1 updates vy, on cells with (i + j) % 2 == color.  Column j holds the rows
// i = 2q + ((j + color) & 1) of that color, q < ceil(ny / 2).
template <class T>
__device__ __forceinline__ void d_rbgs(const LevelDev<T>& v, int64_t t, int comp, int color) {
  const int32_t half = (v.ny + 1) / 2;
  const int32_t j = (int32_t)t / half;  // t < nx * half < 2^31
  if (j >= v.nx) return;
  const int32_t i = 2 * ((int32_t)t - j * half) + ((j + color) & 1);
  if (i >= v.ny) return;
  const int64_t c = (int64_t)j * v.ny + i;
  if (comp == 0) {
    const T s = rowx(v.X, v.ux, v.uy, c, i, j, v.nx, v.ny, v.nc, true);
    v.ux[c] = (v.fx[c] - s) / v.X[c];
  } else {
    const T s = rowy(v.Y, v.ux, v.uy, c, i, j, v.nx, v.ny, v.nc, true);
    v.uy[c] = (v.fy[c] - s) / v.Y[c];
  }
}
template <class T>
__device__ __forceinline__ int64_t rb_count(const LevelDev<T>& v) { return (int64_t)v.nx * ((v.ny + 1) / 2); }

template <class T>
__device__ __forceinline__ void d_resid(const LevelDev<T>& v, int64_t c) {
  const int32_t j = (int32_t)c / v.ny, i = (int32_t)c - j * v.ny;  // cell indices fit 32 bits
  v.rx[c] = v.fx[c] - rowx(v.X, v.ux, v.uy, c, i, j, v.nx, v.ny, v.nc, false);
  v.ry[c] = v.fy[c] - rowy(v.Y, v.ux, v.uy, c, i, j, v.nx, v.ny, v.nc, false);
}
// coarse f = R r at coarse cell c (tensor product of the axis tables of the fine level f)
template <class T>
__device__ __forceinline__ void d_restrict(const LevelDev<T>& f, const LevelDev<T>& cl, int64_t c) {
  const int32_t J = (int32_t)c / cl.ny, I = (int32_t)c - J * cl.ny;
  T sx = 0, sy = 0;
  for (int a = 0; a < kRmax; ++a) {
    const T wa = (T)f.rvx_x.w[J * kRmax + a];
    if (wa != T(0)) {
      const int64_t col = (int64_t)f.rvx_x.idx[J * kRmax + a] * f.ny;
      for (int b = 0; b < kRmax; ++b) {
        const T wb = (T)f.rvx_y.w[I * kRmax + b];
        if (wb != T(0)) sx += wa * wb * f.rx[col + f.rvx_y.idx[I * kRmax + b]];
      }
    }
    const T va = (T)f.rvy_x.w[J * kRmax + a];
    if (va != T(0)) {
      const int64_t col = (int64_t)f.rvy_x.idx[J * kRmax + a] * f.ny;
      for (int b = 0; b < kRmax; ++b) {
        const T vb = (T)f.rvy_y.w[I * kRmax + b];
        if (vb != T(0)) sy += va * vb * f.ry[col + f.rvy_y.idx[I * kRmax + b]];
      }
    }
  }
  cl.fx[c] = sx;
  cl.fy[c] = sy;
}
// fine u += P e at fine cell c
template <class T>
__device__ __forceinline__ void d_prolong(const LevelDev<T>& f, const LevelDev<T>& cl, int64_t c) {
  const int32_t j = (int32_t)c / f.ny, i = (int32_t)c - j * f.ny;
  T sx = 0, sy = 0;
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) {
      const T w1 = (T)f.pvx_x.w[2 * j + a] * (T)f.pvx_y.w[2 * i + b];
      if (w1 != T(0)) sx += w1 * cl.ux[(int64_t)f.pvx_x.idx[2 * j + a] * cl.ny + f.pvx_y.idx[2 * i + b]];
      const T w2 = (T)f.pvy_x.w[2 * j + a] * (T)f.pvy_y.w[2 * i + b];
      if (w2 != T(0)) sy += w2 * cl.uy[(int64_t)f.pvy_x.idx[2 * j + a] * cl.ny + f.pvy_y.idx[2 * i + b]];
    }
  f.ux[c] += sx;
  f.uy[c] += sy;
}

// With programmatic dependent launch the next V-cycle kernel may start while the previous one
// drains: each waits here (griddepcontrol.wait: until the previous grid has completed and its
// memory is visible) before touching the level arrays.  Without it, a no-op.  (Letting the
// successor launch as soon as every block of this grid runs, griddepcontrol.launch_dependents
// at the start, measured slower: 0.695 against 0.674 ms per FP32 V-cycle on the 40M-marker
// rift, the waiting blocks taking slots from the running grid.)
__device__ __forceinline__ void wait_prior_grid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <class T>
__global__ void k_rbgs(LevelDev<T> v, int comp, int color) {
  wait_prior_grid();
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < rb_count(v)) d_rbgs(v, t, comp, color);
}
// The first half-sweep of a level (vx, red) from a zero start: u_x = f_x / diag on the red
// cells (every neighbour is zero), and the zero start written to the rest of u_x and u_y, so
// that no memset precedes the sweep.  Thread t owns the t-th red and the t-th black cell.
template <class T>
__global__ void k_rbgs_first(LevelDev<T> v) {
  wait_prior_grid();
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= rb_count(v)) return;
  const int32_t half = (v.ny + 1) / 2;
  const int32_t j = (int32_t)t / half;
  const int32_t q = (int32_t)t - j * half;
  const int32_t ir = 2 * q + (j & 1), ib = 2 * q + ((j + 1) & 1);
  if (ir < v.ny) {
    const int64_t c = (int64_t)j * v.ny + ir;
    v.ux[c] = v.fx[c] / v.X[c];
    v.uy[c] = T(0);
  }
  if (ib < v.ny) {
    const int64_t c = (int64_t)j * v.ny + ib;
    v.ux[c] = T(0);
    v.uy[c] = T(0);
  }
}
template <class T>
__global__ void k_resid(LevelDev<T> v) {
  wait_prior_grid();
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < v.nc) d_resid(v, c);
}
template <class T>
__global__ void k_restrict(LevelDev<T> f, LevelDev<T> cl) {
  wait_prior_grid();
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < cl.nc) d_restrict(f, cl, c);
}
template <class T>
__global__ void k_prolong(LevelDev<T> f, LevelDev<T> cl) {
  wait_prior_grid();
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < f.nc) d_prolong(f, cl, c);
}

// The V-cycle below level l0 (all levels small) in one thread block:
// every step is a block-stride loop followed by __syncthreads().
constexpr int kCoarseThreads = 1024;
template <class T>
__global__ void __launch_bounds__(kCoarseThreads) k_coarse_cycle(const LevelDev<T>* __restrict__ lv, int l0, int nl,
                                                                  int sweeps, const T* __restrict__ Ainv, int n) {
  wait_prior_grid();
  auto smooth = [&](const LevelDev<T>& v, bool pre) {
    const int64_t cnt = rb_count(v);
    for (int s = 0; s < sweeps; ++s)
      for (int k = 0; k < 4; ++k) {
        // pre: vx red, vx black, vy red, vy black; post: the reverse order
        const int kk = pre ? k : 3 - k;
        const int comp = kk >> 1, color = kk & 1;
        for (int64_t t = threadIdx.x; t < cnt; t += blockDim.x) d_rbgs(v, t, comp, color);
        __syncthreads();
      }
  };
  for (int l = l0; l < nl - 1; ++l) {
    const LevelDev<T> v = lv[l];
    for (int64_t c = threadIdx.x; c < v.nc; c += blockDim.x) { v.ux[c] = T(0); v.uy[c] = T(0); }
    __syncthreads();
    smooth(v, true);
    for (int64_t c = threadIdx.x; c < v.nc; c += blockDim.x) d_resid(v, c);
    __syncthreads();
    const LevelDev<T> w = lv[l + 1];
    for (int64_t c = threadIdx.x; c < w.nc; c += blockDim.x) d_restrict(v, w, c);
    __syncthreads();
  }
  {  // coarsest: u = Ainv f, the inverse stored by columns (AinvT[k n + r]) so that the warp's
     // rows r read one contiguous line per k
    const LevelDev<T> cl = lv[nl - 1];
    const int half = n / 2;
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
      T s0 = 0, s1 = 0;
      for (int k = 0; k < half; ++k) {
        s0 += Ainv[(int64_t)k * n + r] * cl.fx[k];
        s1 += Ainv[(int64_t)(half + k) * n + r] * cl.fy[k];
      }
      const T s = s0 + s1;
      if (r < half) cl.ux[r] = s; else cl.uy[r - half] = s;
    }
    __syncthreads();
  }
  for (int l = nl - 2; l >= l0; --l) {
    const LevelDev<T> v = lv[l];
    const LevelDev<T> w = lv[l + 1];
    for (int64_t c = threadIdx.x; c < v.nc; c += blockDim.x) d_prolong(v, w, c);
    __syncthreads();
    smooth(v, false);
  }
}

// Preconditioner input, on the scaled residual rhat (r = rhat ./ w):
// z_p = prep r_p, stored scaled (zhat_p = z_p / w_p); level-0 right-hand side f = r_u - L_up z_p.
// FP32 method: zhat_p is rounded to FP32 (Zk, float) and zt holds the same value in FP64.
// FP64 method: zt = zhat_p and Zk (double) repeats it.
template <class T>
__global__ void k_prec_in(const double* __restrict__ coef, const double* __restrict__ rhat,
                          const double* __restrict__ winv, const double* __restrict__ prep, double* __restrict__ zt,
                          void* __restrict__ Zk, T* __restrict__ fx, T* __restrict__ fy, int32_t nx, int32_t ny) {
  const int64_t nc = (int64_t)nx * ny;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const int32_t j = (int32_t)c / ny, i = (int32_t)c - j * ny;
  auto z = [&](int64_t k) { return prep[k] * (rhat[2 * nc + k] * winv[2 * nc + k]); };
  const double zc = z(c);
  if (sizeof(T) == 4) {
    const float zs = (float)(zc * winv[2 * nc + c]);
    static_cast<float*>(Zk)[2 * nc + c] = zs;
    zt[2 * nc + c] = (double)zs;
  } else {
    const double zs = zc * winv[2 * nc + c];
    static_cast<double*>(Zk)[2 * nc + c] = zs;
    zt[2 * nc + c] = zs;
  }
  double gx = coef[9 * nc + c] * zc;
  if (j < nx - 1) gx += coef[10 * nc + c] * z(c + ny);
  double gy = coef[20 * nc + c] * zc;
  if (i < ny - 1) gy += coef[21 * nc + c] * z(c + 1);
  fx[c] = (T)(rhat[c] * winv[c] - gx);
  fy[c] = (T)(rhat[nc + c] * winv[nc + c] - gy);
}
// Preconditioner output: zhat_u = u / w_u (rounded to FP32 in the FP32 method) into Zk and zt.
template <class T>
__global__ void k_prec_out(const T* __restrict__ ux, const T* __restrict__ uy, const double* __restrict__ winv,
                           double* __restrict__ zt, void* __restrict__ Zk, int64_t nc) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  if (sizeof(T) == 4) {
    const float zx = (float)((double)ux[c] * winv[c]);
    const float zy = (float)((double)uy[c] * winv[nc + c]);
    static_cast<float*>(Zk)[c] = zx;
    static_cast<float*>(Zk)[nc + c] = zy;
    zt[c] = (double)zx;
    zt[nc + c] = (double)zy;
  } else {
    const double zx = (double)ux[c] * winv[c], zy = (double)uy[c] * winv[nc + c];
    static_cast<double*>(Zk)[c] = zx;
    static_cast<double*>(Zk)[nc + c] = zy;
    zt[c] = zx;
    zt[nc + c] = zy;
  }
}

// Learned stage: zt += a z2, rounded once to FP32 (Zk) so that zt and Zk stay equal.
__global__ void k_add_round(double* __restrict__ zt, float* __restrict__ Zk, const double* __restrict__ z2, double a,
                            int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float v = (float)(zt[k] + a * z2[k]);
  Zk[k] = v;
  zt[k] = (double)v;
}

// ------------------------------------- velocity-block GCR (inner solve) ---
// The velocity stage of the block preconditioner can run a few steps of GCR on the velocity
// block A_uu (the unscaled level-0 stencil), each step preconditioned by one V-cycle: the
// residual-minimising combination of the V-cycle corrections removes the few error modes that
// the multigrid alone handles poorly (thin low-viscosity layers at sharp viscosity jumps that
// coarse levels cannot represent).  Vectors are [ux | uy] (2 nc values, level arithmetic T).
constexpr int kGcrMax = 8;

struct GcrPtrs { const void* v[kGcrMax + 2]; };
struct GcrCoef { double beta[kGcrMax]; double inv, alpha; int nprev; };

// q = A_uu z on level 0
template <class T>
__global__ void k_vel_apply(LevelDev<T> v, const T* __restrict__ z, T* __restrict__ q) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= v.nc) return;
  const int32_t j = (int32_t)c / v.ny, i = (int32_t)c - j * v.ny;
  q[c] = rowx(v.X, z, z + v.nc, c, i, j, v.nx, v.ny, v.nc, false);
  q[v.nc + c] = rowy(v.Y, z, z + v.nc, c, i, j, v.nx, v.ny, v.nc, false);
}
// partial[w][block] = sum over the block's elements of a . b_w / |diag A_uu| (FP64 accumulation).
// The inner product weights each row by the inverse of its diagonal, as the outer iteration's
// symmetric scaling does: unweighted, the stiff rows (1e23 Pa s rock) would hide the residual of
// the soft ones (1e18 Pa s sticky air) by five orders of magnitude.
template <class T>
__global__ void __launch_bounds__(kB) k_gcr_dots(LevelDev<T> v, const T* __restrict__ a, GcrPtrs b, int64_t n,
                                                 double* __restrict__ partial) {
  const T* bw = static_cast<const T*>(b.v[blockIdx.y]);
  double s = 0.0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const double d = k < v.nc ? (double)v.X[k] : (double)v.Y[k - v.nc];
    s += (double)a[k] * (double)bw[k] / fabs(d);
  }
  __shared__ double sh[kB];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = kB / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = sh[0];
}
// zk = (zk - sum_j beta_j z_j) inv, qk likewise (orthonormal against the earlier q_j);
// u += alpha zk, r -= alpha qk
template <class T>
__global__ void k_gcr_update(T* __restrict__ zk, T* __restrict__ qk, GcrPtrs zp, GcrPtrs qp, GcrCoef cf,
                             T* __restrict__ u, T* __restrict__ r, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double z = zk[k], q = qk[k];
  for (int j = 0; j < cf.nprev; ++j) {
    z -= cf.beta[j] * (double)static_cast<const T*>(zp.v[j])[k];
    q -= cf.beta[j] * (double)static_cast<const T*>(qp.v[j])[k];
  }
  z *= cf.inv;
  q *= cf.inv;
  zk[k] = (T)z;
  qk[k] = (T)q;
  u[k] = (T)((double)u[k] + cf.alpha * z);
  r[k] = (T)((double)r[k] - cf.alpha * q);
}

// ------------------------------------------------------ host geometry ---
std::vector<int32_t> coarse_nodes(int32_t n_cells) {
  const int32_t M = n_cells / 2;
  std::vector<int32_t> k(M + 1);
  for (int32_t m = 0; m < M; ++m) k[m] = 2 * m;
  k[M] = n_cells;
  return k;
}
void stag(const std::vector<double>& b, std::vector<double>& g, std::vector<double>& s) {
  const size_t n = b.size();
  g.assign(n + 1, 0.0);
  s.assign(n, 0.0);
  g[0] = b[0] - (b[1] - b[0]) / 2.0;
  g[n] = b[n - 1] + (b[n - 1] - b[n - 2]) / 2.0;
  for (size_t k = 1; k < n; ++k) g[k] = (b[k] + b[k - 1]) / 2.0;
  s[0] = b[1] - b[0];
  s[n - 1] = b[n - 1] - b[n - 2];
  for (size_t k = 1; k + 1 < n; ++k) s[k] = (b[k + 1] - b[k - 1]) / 2.0;
}
// 1-D linear interpolation fine <- coarse.  cpos[0..m]: coarse positions where 1..m-1 are
// unknowns (index k-1) and 0, m are boundary/ghost values equal to b2lo/b2hi times the
// adjacent unknown.  fpos: fine positions; the last one is a dummy (zero row) if last_dummy.
void interp1d(const std::vector<double>& fpos, bool last_dummy, const std::vector<double>& cpos, double b2lo, double b2hi,
              std::vector<int32_t>& idx, std::vector<float>& w, std::vector<std::vector<std::pair<int32_t, double>>>* cols) {
  const int32_t nf = (int32_t)fpos.size(), m = (int32_t)cpos.size() - 1;
  idx.assign(2 * nf, 0);
  w.assign(2 * nf, 0.f);
  for (int32_t n = 0; n < nf; ++n) {
    if (last_dummy && n == nf - 1) continue;
    const double xv = fpos[n];
    int32_t k = (int32_t)(std::upper_bound(cpos.begin(), cpos.end(), xv) - cpos.begin()) - 1;  // cpos[k] <= xv
    k = std::min(std::max(k, 0), m - 1);
    const double t = (xv - cpos[k]) / (cpos[k + 1] - cpos[k]);
    double wt[2] = {1.0 - t, t};
    int32_t node[2] = {k, k + 1};
    int32_t out_i[2];
    double out_w[2];
    for (int a = 0; a < 2; ++a) {
      int32_t nd = node[a];
      double ww = wt[a];
      if (nd == 0) { nd = 1; ww *= b2lo; }
      else if (nd == m) { nd = m - 1; ww *= b2hi; }
      out_i[a] = nd - 1;
      out_w[a] = ww;
    }
    if (out_i[0] == out_i[1]) { out_w[0] += out_w[1]; out_w[1] = 0.0; }
    for (int a = 0; a < 2; ++a) {
      idx[2 * n + a] = out_i[a];
      w[2 * n + a] = (float)out_w[a];
    }
  }
  (void)cols;
}
// Restriction from the prolongation: R[K][n] = P[n][K] vol[n] / sum_n P[n][K] vol[n].
bool restrict1d(const std::vector<int32_t>& pidx, const std::vector<float>& pw, const std::vector<double>& vol,
                int32_t ncoarse, std::vector<int32_t>& ridx, std::vector<float>& rw) {
  std::vector<std::vector<std::pair<int32_t, double>>> rows(ncoarse);
  const int32_t nf = (int32_t)vol.size();
  for (int32_t n = 0; n < nf; ++n)
    for (int a = 0; a < 2; ++a) {
      const double v = (double)pw[2 * n + a] * vol[n];
      if (v != 0.0) rows[pidx[2 * n + a]].push_back({n, v});
    }
  ridx.assign((size_t)ncoarse * kRmax, 0);
  rw.assign((size_t)ncoarse * kRmax, 0.f);
  for (int32_t K = 0; K < ncoarse; ++K) {
    double s = 0.0;
    for (auto& e : rows[K]) s += e.second;
    if ((int)rows[K].size() > kRmax) return false;
    for (size_t a = 0; a < rows[K].size(); ++a) {
      ridx[(size_t)K * kRmax + a] = rows[K][a].first;
      rw[(size_t)K * kRmax + a] = (float)(rows[K][a].second / s);
    }
  }
  return true;
}

// dense inverse (Gauss-Jordan with partial pivoting), row-major n x n
bool invert_dense(std::vector<double>& A, int n, std::vector<double>& inv) {
  inv.assign((size_t)n * n, 0.0);
  for (int k = 0; k < n; ++k) inv[(size_t)k * n + k] = 1.0;
  for (int col = 0; col < n; ++col) {
    int piv = col;
    for (int r = col + 1; r < n; ++r)
      if (std::fabs(A[(size_t)r * n + col]) > std::fabs(A[(size_t)piv * n + col])) piv = r;
    if (A[(size_t)piv * n + col] == 0.0) return false;
    if (piv != col)
      for (int k = 0; k < n; ++k) {
        std::swap(A[(size_t)piv * n + k], A[(size_t)col * n + k]);
        std::swap(inv[(size_t)piv * n + k], inv[(size_t)col * n + k]);
      }
    const double d = 1.0 / A[(size_t)col * n + col];
    for (int k = 0; k < n; ++k) { A[(size_t)col * n + k] *= d; inv[(size_t)col * n + k] *= d; }
    for (int r = 0; r < n; ++r) {
      if (r == col) continue;
      const double f = A[(size_t)r * n + col];
      if (f == 0.0) continue;
      for (int k = 0; k < n; ++k) {
        A[(size_t)r * n + k] -= f * A[(size_t)col * n + k];
        inv[(size_t)r * n + k] -= f * inv[(size_t)col * n + k];
      }
    }
  }
  return true;
}

}  // namespace

// ------------------------------------------------------------ state ---
// The multigrid hierarchy of one arithmetic (both are kept, so the two methods can alternate
// on one system without rebuilding).
struct Hierarchy {
  std::vector<void*> level_allocs;   // multigrid buffers
  std::vector<Level> levels;
  void* Ainv = nullptr;              // coarsest inverse (FP32 or FP64)
  void* lv_dev = nullptr;            // device copies of the level descriptors
  int n_dense = 0;
  B2 b2_levels{};                    // boundary coefficients the transfer tables were built with
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int64_t graph_kernels = 0;
  bool pdl_ok = true;                // false once a V-cycle with programmatic launches failed to capture
  void* gcr = nullptr;               // velocity GCR vectors: r, u, z[kGcrMax], q[kGcrMax]
};

struct StokesState {
  StokesSystem sys;
  std::vector<void*> allocs;         // system + solver buffers
  Hierarchy hier[2];                 // [0] FP32 V-cycle (mixed method), [1] FP64 (plain method)
  bool mg64 = false;                 // the hierarchy in use
  Hierarchy& H() { return hier[mg64 ? 1 : 0]; }
  double *w = nullptr, *prep = nullptr;  // scaling and pressure factor
  double* winv = nullptr;                // 1 / w
  double* coefS = nullptr;               // stencil of W L W [27][nc]
  // mixed method: coefS as FP32 pairs, FP32 pressure-coupling slots, 1/w and prep * winv_p
  float *coefH = nullptr, *coefL = nullptr, *cq32 = nullptr, *winv32 = nullptr, *pw32 = nullptr;
  // FGMRES workspace
  int m = 0;
  double *V = nullptr, *r = nullptr, *t = nullptr, *xs = nullptr, *bs = nullptr, *zp = nullptr, *zt = nullptr;
  float* Z = nullptr;                // preconditioned directions: FP32 (mixed method) ...
  double* Zd = nullptr;              // ... or FP64 (plain method)
  double *partial = nullptr, *dots = nullptr, *hdev = nullptr;
  int nb_dot = 0;
  float* V32 = nullptr;              // the basis as FP32 hi parts (mixed method), slots ld32 apart
  float* V32lo = nullptr;            // their remainders: the basis as double-float pairs
  int64_t ld32 = 0;
  double* part32 = nullptr;          // per-block norms of k_maxpy32 / k_maxpy_df
  int nb_ax32 = 0, ax_p = 2;          // blocks and float4 chunks per thread of the split updates
  int nb_split = 0;                  // blocks per vector group of the split dot products
  double* il = nullptr;              // interleaved staging vector (N)
  double* tmp = nullptr;             // scratch vector (N)
  double *nn_t = nullptr, *nn_q = nullptr, *nn_z = nullptr;  // learned-stage scratch: [t | q], z2
  int gcr_steps = 1;                 // velocity stage: 1 V-cycle, or up to this many GCR steps
  double gcr_tol = 0.1;              // ... until the velocity residual falls below this fraction
  int64_t gcr_total = 0;             // GCR steps run in the current solve
};

namespace {

template <class T>
int dalloc(eb_ctx* c, std::vector<void*>& owner, T** p, size_t n) {
  EB_CK(c, cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T)));
  owner.push_back(*p);
  return EB_OK;
}
template <class T>
int dupload(eb_ctx* c, std::vector<void*>& owner, T** p, const std::vector<T>& h) {
  int rc = dalloc(c, owner, p, h.size());
  if (rc) return rc;
  if (!h.empty()) EB_CK(c, cudaMemcpyAsync(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, c->stream));
  return EB_OK;
}

int dalloc_bytes(eb_ctx* c, std::vector<void*>& owner, void** p, size_t bytes) {
  EB_CK(c, cudaMalloc(p, std::max<size_t>(bytes, 16)));
  owner.push_back(*p);
  return EB_OK;
}
// h converted to the level arithmetic and uploaded
int upload_real(eb_ctx* c, std::vector<void*>& owner, void** p, const std::vector<double>& h, bool fp64) {
  if (fp64) return dupload(c, owner, reinterpret_cast<double**>(p), h);
  std::vector<float> f(h.begin(), h.end());
  return dupload(c, owner, reinterpret_cast<float**>(p), f);
}

void free_levels(StokesState* st) {
  st->H().gcr = nullptr;  // one of level_allocs
  for (void* p : st->H().level_allocs) cudaFree(p);
  st->H().level_allocs.clear();
  st->H().levels.clear();
  st->H().Ainv = nullptr;
  st->H().lv_dev = nullptr;
  if (st->H().gexec) cudaGraphExecDestroy(st->H().gexec);
  if (st->H().graph) cudaGraphDestroy(st->H().graph);
  st->H().gexec = nullptr;
  st->H().graph = nullptr;
}

}  // namespace

StokesSystem* stokes_system(eb_ctx* c) {
  if (c->st) return &c->st->sys;
  StokesState* st = new StokesState();
  StokesSystem& s = st->sys;
  s.nx = c->xnum - 1;
  s.ny = c->ynum - 1;
  s.nc = (int64_t)s.nx * s.ny;
  const size_t nc = (size_t)s.nc;
  if (dalloc(c, st->allocs, &s.coef, kStencilSlots * nc) || dalloc(c, st->allocs, &s.rhs, 3 * nc) ||
      dalloc(c, st->allocs, &s.S, 3 * nc) || dalloc(c, st->allocs, &s.S_old, 3 * nc) ||
      dalloc(c, st->allocs, &s.resnl, 3 * nc) || dalloc(c, st->allocs, &st->il, 3 * nc) ||
      dalloc(c, st->allocs, &st->tmp, 3 * nc)) {
    for (void* p : st->allocs) cudaFree(p);
    delete st;
    return nullptr;
  }
  cudaMemsetAsync(s.S, 0, 3 * nc * sizeof(double), c->stream);
  cudaMemsetAsync(s.S_old, 0, 3 * nc * sizeof(double), c->stream);
  c->st = st;
  return &st->sys;
}

void stokes_free(eb_ctx* c) {
  if (!c->st) return;
  for (bool b : {false, true}) {
    c->st->mg64 = b;
    free_levels(c->st);
  }
  for (void* p : c->st->allocs) cudaFree(p);
  delete c->st;
  c->st = nullptr;
}

namespace {

// Uniform boundary-condition coefficient per side: the mean of b[:, 2].
int read_b2(eb_ctx* c, B2* b) {
  const int ids[8] = {EB_G_BTOPX, EB_G_BBOTTOMX, EB_G_BTOPY, EB_G_BBOTTOMY, EB_G_BLEFTX, EB_G_BRIGHTX, EB_G_BLEFTY, EB_G_BRIGHTY};
  float* out[8] = {&b->topx, &b->botx, &b->topy, &b->boty, &b->leftx, &b->rightx, &b->lefty, &b->righty};
  for (int k = 0; k < 8; ++k) {
    const size_t n = grid_field_count(c, ids[k]) / 2;
    std::vector<double> h(2 * n);
    EB_CK(c, cudaMemcpyAsync(h.data(), c->gf[ids[k]], 2 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    EB_CK(c, cudaStreamSynchronize(c->stream));
    double s = 0.0;
    for (size_t q = 0; q < n; ++q) s += h[n + q];
    *out[k] = (float)(s / (double)n);
  }
  return EB_OK;
}

// Build the level geometry, buffers and transfer tables (host), for the current grid and b2.
template <class T>
LevelDev<T> level_dev(const Level& v);

int setup_levels(eb_ctx* c, StokesState* st, const B2& b2) {
  free_levels(st);
  std::vector<Level>& L = st->H().levels;
  L.emplace_back();
  L[0].x = c->h_gx;
  L[0].y = c->h_gy;
  while (true) {
    Level& f = L.back();
    f.nx = (int32_t)f.x.size() - 1;
    f.ny = (int32_t)f.y.size() - 1;
    f.nc = (int64_t)f.nx * f.ny;
    if (std::min(f.nx, f.ny) < 4) break;
    Level cl;
    const std::vector<int32_t> kx = coarse_nodes(f.nx), ky = coarse_nodes(f.ny);
    for (int32_t k : kx) cl.x.push_back(f.x[k]);
    for (int32_t k : ky) cl.y.push_back(f.y[k]);
    L.push_back(cl);
    Level& cc = L.back();
    int rc;
    if ((rc = dupload(c, st->H().level_allocs, &cc.kx, kx)) || (rc = dupload(c, st->H().level_allocs, &cc.ky, ky))) return rc;
  }
  const int nlev = (int)L.size();
  st->H().n_dense = 2 * (int)L.back().nc;
  if (st->H().n_dense > 2048)
    return eb_fail(c, EB_BAD_INPUT, "grid aspect ratio too large for the multigrid hierarchy (coarsest level has " +
                                        std::to_string(L.back().nc) + " cells)");
  const size_t es = st->mg64 ? sizeof(double) : sizeof(float);
  for (int l = 0; l < nlev; ++l) {
    Level& v = L[l];
    const size_t nc = (size_t)v.nc;
    int rc;
    auto A = [&](void** p, size_t n) { return dalloc_bytes(c, st->H().level_allocs, p, n * es); };
    if ((rc = A(&v.X, 9 * nc)) || (rc = A(&v.Y, 9 * nc)) || (rc = A(&v.ux, nc)) || (rc = A(&v.uy, nc)) ||
        (rc = A(&v.fx, nc)) || (rc = A(&v.fy, nc)) || (rc = A(&v.rx, nc)) || (rc = A(&v.ry, nc)) ||
        (rc = A(&v.etas, (size_t)(v.nx + 1) * (v.ny + 1))) || (rc = A(&v.etan, nc)))
      return rc;
    // spacing tables for the rediscretisation, in the level arithmetic
    std::vector<double> gxc, sxc, gyc, syc;
    stag(v.x, gxc, sxc);
    stag(v.y, gyc, syc);
    std::vector<double> xs(v.nx), ys(v.ny), xsc(v.nx + 1), ysc(v.ny + 1);
    for (int32_t j = 0; j < v.nx; ++j) xs[j] = v.x[j + 1] - v.x[j];
    for (int32_t i = 0; i < v.ny; ++i) ys[i] = v.y[i + 1] - v.y[i];
    for (int32_t j = 0; j <= v.nx; ++j) xsc[j] = sxc[j];
    for (int32_t i = 0; i <= v.ny; ++i) ysc[i] = syc[i];
    if ((rc = upload_real(c, st->H().level_allocs, &v.xstp, xs, st->mg64)) ||
        (rc = upload_real(c, st->H().level_allocs, &v.ystp, ys, st->mg64)) ||
        (rc = upload_real(c, st->H().level_allocs, &v.xstpc, xsc, st->mg64)) ||
        (rc = upload_real(c, st->H().level_allocs, &v.ystpc, ysc, st->mg64)))
      return rc;
  }
  // transfer tables between level l (fine) and l+1 (coarse)
  for (int l = 0; l + 1 < nlev; ++l) {
    Level& f = L[l];
    Level& cl = L[l + 1];
    std::vector<double> gxf, sxf, gyf, syf, gxc, sxc, gyc, syc;
    stag(f.x, gxf, sxf);
    stag(f.y, gyf, syf);
    stag(cl.x, gxc, sxc);
    stag(cl.y, gyc, syc);
    // fine positions and control lengths
    std::vector<double> vx_x(f.x.begin() + 1, f.x.end());           // nodes 1..nx (last: dummy)
    std::vector<double> vx_y(gyf.begin() + 1, gyf.begin() + 1 + f.ny);  // cell centres
    std::vector<double> vy_x(gxf.begin() + 1, gxf.begin() + 1 + f.nx);
    std::vector<double> vy_y(f.y.begin() + 1, f.y.end());           // last: dummy
    std::vector<double> vol_vx_x(f.nx), vol_vx_y(f.ny), vol_vy_x(f.nx), vol_vy_y(f.ny);
    for (int32_t j = 0; j < f.nx; ++j) {
      vol_vx_x[j] = (j == f.nx - 1) ? 0.0 : sxf[j + 1];
      vol_vy_x[j] = f.x[j + 1] - f.x[j];
    }
    for (int32_t i = 0; i < f.ny; ++i) {
      vol_vx_y[i] = f.y[i + 1] - f.y[i];
      vol_vy_y[i] = (i == f.ny - 1) ? 0.0 : syf[i + 1];
    }
    // coarse positions: [boundary/ghost, unknowns..., boundary/ghost]
    std::vector<double> c_vx_x(cl.x.begin(), cl.x.end());                  // 0..nxc
    std::vector<double> c_vx_y(gyc.begin(), gyc.begin() + cl.ny + 2);      // ghost, centres, ghost
    std::vector<double> c_vy_x(gxc.begin(), gxc.begin() + cl.nx + 2);
    std::vector<double> c_vy_y(cl.y.begin(), cl.y.end());
    std::vector<int32_t> pi[4], ri[4];
    std::vector<float> pw[4], rw[4];
    interp1d(vx_x, true, c_vx_x, b2.leftx, b2.rightx, pi[0], pw[0], nullptr);
    interp1d(vx_y, false, c_vx_y, b2.topx, b2.botx, pi[1], pw[1], nullptr);
    interp1d(vy_x, false, c_vy_x, b2.lefty, b2.righty, pi[2], pw[2], nullptr);
    interp1d(vy_y, true, c_vy_y, b2.topy, b2.boty, pi[3], pw[3], nullptr);
    const std::vector<double>* vols[4] = {&vol_vx_x, &vol_vx_y, &vol_vy_x, &vol_vy_y};
    const int32_t ncs[4] = {cl.nx, cl.ny, cl.nx, cl.ny};
    for (int a = 0; a < 4; ++a)
      if (!restrict1d(pi[a], pw[a], *vols[a], ncs[a], ri[a], rw[a]))
        return eb_fail(c, EB_BAD_INPUT, "multigrid restriction stencil too wide (grid spacing varies too fast)");
    Axis2* P[4] = {&f.pvx_x, &f.pvx_y, &f.pvy_x, &f.pvy_y};
    AxisR* R[4] = {&f.rvx_x, &f.rvx_y, &f.rvy_x, &f.rvy_y};
    for (int a = 0; a < 4; ++a) {
      int rc;
      if ((rc = dupload(c, st->H().level_allocs, &P[a]->idx, pi[a])) || (rc = dupload(c, st->H().level_allocs, &P[a]->w, pw[a])) ||
          (rc = dupload(c, st->H().level_allocs, &R[a]->idx, ri[a])) || (rc = dupload(c, st->H().level_allocs, &R[a]->w, rw[a])))
        return rc;
    }
  }
  int rc = dalloc_bytes(c, st->H().level_allocs, &st->H().Ainv, (size_t)st->H().n_dense * st->H().n_dense * es);
  if (rc) return rc;
  if (st->mg64) {
    std::vector<LevelDev<double>> lv;
    for (const Level& v : L) lv.push_back(level_dev<double>(v));
    LevelDev<double>* d = nullptr;
    if ((rc = dupload(c, st->H().level_allocs, &d, lv))) return rc;
    st->H().lv_dev = d;
  } else {
    std::vector<LevelDev<float>> lv;
    for (const Level& v : L) lv.push_back(level_dev<float>(v));
    LevelDev<float>* d = nullptr;
    if ((rc = dupload(c, st->H().level_allocs, &d, lv))) return rc;
    st->H().lv_dev = d;
  }
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}

// Per-solve operators: level 0 from the FP64 stencil, coarse viscosity and stencils, coarsest inverse.
template <class T>
int refresh_levels_t(eb_ctx* c, StokesState* st, const B2& b2) {
  std::vector<Level>& L = st->H().levels;
  const StokesSystem& s = st->sys;
  auto P = [](void* p) { return static_cast<T*>(p); };
  EB_PROF(c, "k_mg_setup");
  k_level0<T><<<nblk(s.nc), kB, 0, c->stream>>>(s.coef, P(L[0].X), P(L[0].Y), s.nc);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_mg_setup");
  k_to_real<T><<<nblk((int64_t)c->xnum * c->ynum), kB, 0, c->stream>>>(c->gf[EB_G_ETAS0], P(L[0].etas),
                                                                     (int64_t)c->xnum * c->ynum);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_mg_setup");
  k_to_real<T><<<nblk(s.nc), kB, 0, c->stream>>>(c->gf[EB_G_ETAN0], P(L[0].etan), s.nc);
  EB_LAUNCHED(c);
  for (size_t l = 1; l < L.size(); ++l) {
    Level& f = L[l - 1];
    Level& v = L[l];
    const int64_t n = std::max<int64_t>((int64_t)(v.nx + 1) * (v.ny + 1), v.nc);
    EB_PROF(c, "k_mg_setup");
    k_coarsen_eta<T><<<nblk(n), kB, 0, c->stream>>>(P(f.etas), P(f.etan), f.nx, f.ny, P(v.etas), P(v.etan), v.nx, v.ny,
                                                    v.kx, v.ky);
    EB_LAUNCHED(c);
    EB_PROF(c, "k_mg_setup");
    k_redisc<T><<<nblk(v.nc), kB, 0, c->stream>>>(v.nx, v.ny, P(v.etas), P(v.etan), P(v.xstp), P(v.ystp), P(v.xstpc),
                                                  P(v.ystpc), b2, P(v.X), P(v.Y));
    EB_LAUNCHED(c);
  }
  // coarsest velocity block as a dense matrix on the host, inverted in FP64
  const Level& cl = L.back();
  const int nc = (int)cl.nc, n = 2 * nc;
  std::vector<T> hX(9 * (size_t)nc), hY(9 * (size_t)nc);
  EB_CK(c, cudaMemcpyAsync(hX.data(), cl.X, hX.size() * sizeof(T), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaMemcpyAsync(hY.data(), cl.Y, hY.size() * sizeof(T), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  std::vector<double> A((size_t)n * n, 0.0), inv;
  const int32_t ny = cl.ny, nx = cl.nx;
  auto put = [&](int r, int col, double v) { if (v != 0.0) A[(size_t)r * n + col] += v; };
  for (int cc = 0; cc < nc; ++cc) {
    const int i = cc % ny, j = cc / ny;
    const bool hu = i > 0, hd = i < ny - 1, hl = j > 0, hr = j < nx - 1;
    auto Xs = [&](int k) { return (double)hX[(size_t)k * nc + cc]; };
    auto Ys = [&](int k) { return (double)hY[(size_t)k * nc + cc]; };
    put(cc, cc, Xs(0));
    if (hl) put(cc, cc - ny, Xs(1));
    if (hr) put(cc, cc + ny, Xs(2));
    if (hu) put(cc, cc - 1, Xs(3));
    if (hd) put(cc, cc + 1, Xs(4));
    if (hu) put(cc, nc + cc - 1, Xs(5));
    if (hu && hr) put(cc, nc + cc + ny - 1, Xs(6));
    put(cc, nc + cc, Xs(7));
    if (hr) put(cc, nc + cc + ny, Xs(8));
    const int r = nc + cc;
    put(r, nc + cc, Ys(0));
    if (hu) put(r, nc + cc - 1, Ys(1));
    if (hd) put(r, nc + cc + 1, Ys(2));
    if (hl) put(r, nc + cc - ny, Ys(3));
    if (hr) put(r, nc + cc + ny, Ys(4));
    if (hl) put(r, cc - ny, Ys(5));
    put(r, cc, Ys(6));
    if (hl && hd) put(r, cc + 1 - ny, Ys(7));
    if (hd) put(r, cc + 1, Ys(8));
  }
  if (!invert_dense(A, n, inv)) return eb_fail(c, EB_NAN, "coarsest multigrid operator is singular");
  std::vector<T> invf(inv.size());  // transposed: column k of the inverse is contiguous
  for (int r = 0; r < n; ++r)
    for (int k = 0; k < n; ++k) invf[(size_t)k * n + r] = (T)inv[(size_t)r * n + k];
  EB_CK(c, cudaMemcpyAsync(st->H().Ainv, invf.data(), invf.size() * sizeof(T), cudaMemcpyHostToDevice, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}
int refresh_levels(eb_ctx* c, StokesState* st, const B2& b2) {
  return st->mg64 ? refresh_levels_t<double>(c, st, b2) : refresh_levels_t<float>(c, st, b2);
}

template <class T>
LevelDev<T> level_dev(const Level& v) {
  LevelDev<T> d;
  auto P = [](void* p) { return static_cast<T*>(p); };
  d.nx = v.nx; d.ny = v.ny; d.nc = v.nc;
  d.X = P(v.X); d.Y = P(v.Y);
  d.ux = P(v.ux); d.uy = P(v.uy); d.fx = P(v.fx); d.fy = P(v.fy); d.rx = P(v.rx); d.ry = P(v.ry);
  d.pvx_x = v.pvx_x; d.pvx_y = v.pvx_y; d.pvy_x = v.pvy_x; d.pvy_y = v.pvy_y;
  d.rvx_x = v.rvx_x; d.rvx_y = v.rvx_y; d.rvy_x = v.rvy_x; d.rvy_y = v.rvy_y;
  return d;
}

// One V-cycle from level 0's f into level 0's u (launches on c->stream).  Levels
// at or below l0 (the first with at most kCoarseCells cells) run in one block.  Measured on
// the 40M-marker rift (V-cycle time per solve): 8192 -> 107 ms, 2048 -> 95 ms, 1024 -> 98 ms,
// 256 -> 102 ms (one 1024-thread block is slower than launches above a few thousand cells).
constexpr int64_t kCoarseCells = 2048;
template <class T>
int vcycle_launch(eb_ctx* c, StokesState* st, int sweeps, int64_t* nk, bool pdl) {
  std::vector<Level>& L = st->H().levels;
  const int nl = (int)L.size();
  int l0 = 0;
  while (l0 < nl - 1 && L[l0].nc > kCoarseCells) ++l0;
  // every kernel of the cycle through one launcher: with `pdl`, a programmatic dependent launch
  // (the kernel waits for its predecessor in wait_prior_grid)
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  auto launch = [&](auto kernel, unsigned grid, unsigned block, auto... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.stream = c->stream;
    cfg.attrs = pdl ? attr : nullptr;
    cfg.numAttrs = pdl ? 1 : 0;
    ++*nk;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
  };
  auto rb = [&](const LevelDev<T>& v, int comp, int color) {
    const int64_t cnt = (int64_t)v.nx * ((v.ny + 1) / 2);
    return launch(k_rbgs<T>, nblk(cnt), kB, v, comp, color);
  };
  for (int l = 0; l < l0; ++l) {
    const LevelDev<T> v = level_dev<T>(L[l]);
    for (int s = 0; s < sweeps; ++s)
      for (int k = 0; k < 4; ++k) {
        if (s == 0 && k == 0) {  // zero start folded into the first half-sweep
          const int64_t cnt = (int64_t)v.nx * ((v.ny + 1) / 2);
          EB_CK(c, launch(k_rbgs_first<T>, nblk(cnt), kB, v));
        } else {
          EB_CK(c, rb(v, k >> 1, k & 1));
        }
      }
    EB_CK(c, launch(k_resid<T>, nblk(v.nc), kB, v));
    const LevelDev<T> w = level_dev<T>(L[l + 1]);
    EB_CK(c, launch(k_restrict<T>, nblk(w.nc), kB, v, w));
  }
  EB_CK(c, launch(k_coarse_cycle<T>, 1, kCoarseThreads, static_cast<const LevelDev<T>*>(st->H().lv_dev), l0, nl, sweeps,
                  static_cast<const T*>(st->H().Ainv), st->H().n_dense));
  for (int l = l0 - 1; l >= 0; --l) {
    const LevelDev<T> v = level_dev<T>(L[l]);
    const LevelDev<T> w = level_dev<T>(L[l + 1]);
    EB_CK(c, launch(k_prolong<T>, nblk(v.nc), kB, v, w));
    for (int s = 0; s < sweeps; ++s)
      for (int k = 3; k >= 0; --k) EB_CK(c, rb(v, k >> 1, k & 1));
  }
  EB_CK(c, cudaGetLastError());
  return EB_OK;
}

int capture_vcycle(eb_ctx* c, StokesState* st, int sweeps) {
  if (st->H().gexec) { cudaGraphExecDestroy(st->H().gexec); st->H().gexec = nullptr; }
  if (st->H().graph) { cudaGraphDestroy(st->H().graph); st->H().graph = nullptr; }
  const bool prof = c->prof.on;
  c->prof.on = false;
  // with programmatic dependent launches first; if that graph cannot be captured or
  // instantiated, plain launches (and never programmatic ones again on this hierarchy)
  for (int attempt = 0; attempt < 2; ++attempt) {
    const bool pdl = attempt == 0;
    if (pdl && !st->H().pdl_ok) continue;
    int64_t nk = 0;
    EB_CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int rc = st->mg64 ? vcycle_launch<double>(c, st, sweeps, &nk, pdl) : vcycle_launch<float>(c, st, sweeps, &nk, pdl);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    cudaGraphExec_t ge = nullptr;
    if (rc == EB_OK && e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
    if (rc == EB_OK && e == cudaSuccess) {
      c->prof.on = prof;
      st->H().graph = g;
      st->H().gexec = ge;
      st->H().graph_kernels = nk;
      return EB_OK;
    }
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    if (!pdl) {
      c->prof.on = prof;
      if (rc) return rc;
      return eb_cuda(c, e, "V-cycle graph capture");
    }
    st->H().pdl_ok = false;
  }
  c->prof.on = prof;
  return eb_fail(c, EB_CUDA_ERROR, "V-cycle graph capture failed");
}

// Velocity stage by GCR: the level-0 right-hand side (fx, fy) in, the solution (ux, uy) out.
// Each step runs the captured V-cycle on the current residual, applies A_uu to the correction,
// orthonormalises it against the earlier steps' products (one fused reduction, Pythagorean
// norm) and moves the solution and the residual along it.  Stops after gcr_steps steps, or when
// |r| <= gcr_tol |f| (|r| follows from the same reduction), or when a correction adds nothing.
template <class T>
int velocity_gcr(eb_ctx* c, StokesState* st) {
  Hierarchy& H = st->H();
  Level& L0 = H.levels[0];
  const LevelDev<T> v = level_dev<T>(L0);
  const int64_t nc = v.nc, n = 2 * nc;
  const int K = std::min(st->gcr_steps, kGcrMax);
  int rc;
  if (!H.gcr && (rc = dalloc_bytes(c, H.level_allocs, &H.gcr, (size_t)(2 + 2 * kGcrMax) * n * sizeof(T)))) return rc;
  T* R = static_cast<T*>(H.gcr);
  T* U = R + n;
  auto Zs = [&](int k) { return U + n + (size_t)k * n; };
  auto Qs = [&](int k) { return U + n + (size_t)(kGcrMax + k) * n; };
  const size_t hb = nc * sizeof(T);
  EB_CK(c, cudaMemcpyAsync(R, L0.fx, hb, cudaMemcpyDeviceToDevice, c->stream));
  EB_CK(c, cudaMemcpyAsync(R + nc, L0.fy, hb, cudaMemcpyDeviceToDevice, c->stream));
  EB_CK(c, cudaMemsetAsync(U, 0, n * sizeof(T), c->stream));
  double rr0 = 0.0, rr = 0.0;
  int done = 0;
  for (int k = 0; k < K; ++k) {
    if (k > 0) {
      EB_CK(c, cudaMemcpyAsync(L0.fx, R, hb, cudaMemcpyDeviceToDevice, c->stream));
      EB_CK(c, cudaMemcpyAsync(L0.fy, R + nc, hb, cudaMemcpyDeviceToDevice, c->stream));
    }
    EB_PROF(c, "vcycle_graph");
    EB_CK(c, cudaGraphLaunch(H.gexec, c->stream));
    c->launches += H.graph_kernels - 1;
    EB_LAUNCHED(c);
    EB_CK(c, cudaMemcpyAsync(Zs(k), L0.ux, hb, cudaMemcpyDeviceToDevice, c->stream));
    EB_CK(c, cudaMemcpyAsync(Zs(k) + nc, L0.uy, hb, cudaMemcpyDeviceToDevice, c->stream));
    EB_PROF(c, "k_vel_apply");
    k_vel_apply<T><<<nblk(nc), kB, 0, c->stream>>>(v, Zs(k), Qs(k));
    EB_LAUNCHED(c);
    // dots: q_k.q_j (j < k), q_k.q_k, q_k.r, and r.r at the first step
    GcrPtrs b{};
    int nv = 0;
    for (int j = 0; j < k; ++j) b.v[nv++] = Qs(j);
    b.v[nv++] = Qs(k);
    b.v[nv++] = R;
    EB_PROF(c, "k_gcr_dots");
    k_gcr_dots<T><<<dim3(st->nb_dot, nv), kB, 0, c->stream>>>(v, Qs(k), b, n, st->partial);
    EB_LAUNCHED(c);
    int nall = nv;
    if (k == 0) {
      GcrPtrs br{};
      br.v[0] = R;
      k_gcr_dots<T><<<dim3(st->nb_dot, 1), kB, 0, c->stream>>>(v, R, br, n, st->partial + (size_t)nv * st->nb_dot);
      EB_LAUNCHED(c);
      ++nall;
    }
    k_mdot_final<<<nall, kB, 0, c->stream>>>(st->partial, st->nb_dot, st->dots);
    EB_LAUNCHED(c);
    double h[kGcrMax + 3];
    EB_CK(c, cudaMemcpyAsync(h, st->dots, nall * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    EB_CK(c, cudaStreamSynchronize(c->stream));
    if (k == 0) rr0 = rr = h[nv];
    double qq = h[k];
    GcrCoef cf{};
    cf.nprev = k;
    for (int j = 0; j < k; ++j) {
      cf.beta[j] = h[j];
      qq -= h[j] * h[j];
    }
    if (!(qq > 1e-12 * h[k]) || !std::isfinite(qq) || !(rr0 > 0.0)) break;
    const double nrm = std::sqrt(qq);
    cf.inv = 1.0 / nrm;
    cf.alpha = h[k + 1] / nrm;
    EB_PROF(c, "k_gcr_update");
    k_gcr_update<T><<<nblk(n), kB, 0, c->stream>>>(Zs(k), Qs(k), GcrPtrs{{Zs(0), Zs(1), Zs(2), Zs(3), Zs(4), Zs(5),
                                                                         Zs(6), Zs(7)}},
                                                   GcrPtrs{{Qs(0), Qs(1), Qs(2), Qs(3), Qs(4), Qs(5), Qs(6), Qs(7)}},
                                                   cf, U, R, n);
    EB_LAUNCHED(c);
    ++done;
    ++st->gcr_total;
    rr -= cf.alpha * cf.alpha;
    if (rr <= st->gcr_tol * st->gcr_tol * rr0) break;
  }
  if (done == 0) {  // no usable step: the V-cycle's correction as it is
    EB_CK(c, cudaMemcpyAsync(U, Zs(0), n * sizeof(T), cudaMemcpyDeviceToDevice, c->stream));
  }
  EB_CK(c, cudaMemcpyAsync(L0.ux, U, hb, cudaMemcpyDeviceToDevice, c->stream));
  EB_CK(c, cudaMemcpyAsync(L0.uy, U + nc, hb, cudaMemcpyDeviceToDevice, c->stream));
  return EB_OK;
}

// zhat = W^-1 M^-1 W^-1 rhat (rhat: SoA FP64 of 3 nc), kept in Zk (the stored direction:
// FP32 in the mixed method, FP64 in the plain one) and zt (its FP64 value, the input of the
// operator product).
int precondition(eb_ctx* c, StokesState* st, const double* rhat, double* zt, void* Zk) {
  const StokesSystem& s = st->sys;
  Level& v = st->H().levels[0];
  EB_PROF(c, "k_precond");
  if (st->mg64)
    k_prec_in<double><<<nblk(s.nc), kB, 0, c->stream>>>(s.coef, rhat, st->winv, st->prep, zt, Zk,
                                                        static_cast<double*>(v.fx), static_cast<double*>(v.fy), s.nx, s.ny);
  else
    k_prec_in<float><<<nblk(s.nc), kB, 0, c->stream>>>(s.coef, rhat, st->winv, st->prep, zt, Zk,
                                                       static_cast<float*>(v.fx), static_cast<float*>(v.fy), s.nx, s.ny);
  EB_LAUNCHED(c);
  if (st->gcr_steps > 1) {
    const int rc = st->mg64 ? velocity_gcr<double>(c, st) : velocity_gcr<float>(c, st);
    if (rc) return rc;
  } else {
    EB_PROF(c, "vcycle_graph");
    EB_CK(c, cudaGraphLaunch(st->H().gexec, c->stream));
    c->launches += st->H().graph_kernels - 1;
    EB_LAUNCHED(c);
  }
  EB_PROF(c, "k_precond");
  if (st->mg64)
    k_prec_out<double><<<nblk(s.nc), kB, 0, c->stream>>>(static_cast<double*>(v.ux), static_cast<double*>(v.uy), st->winv,
                                                         zt, Zk, s.nc);
  else
    k_prec_out<float><<<nblk(s.nc), kB, 0, c->stream>>>(static_cast<float*>(v.ux), static_cast<float*>(v.uy), st->winv, zt,
                                                        Zk, s.nc);
  EB_LAUNCHED(c);
  return EB_OK;
}

// The mixed method's preconditioner on a split basis vector (its FP32 hi part rh): FP32 input
// and output kernels around the captured FP32 V-cycle; the direction goes to Zk only.
int precondition32(eb_ctx* c, StokesState* st, const float* rh, float* Zk) {
  const StokesSystem& s = st->sys;
  Level& v = st->H().levels[0];
  EB_PROF(c, "k_precond");
  k_prec_in32<<<nblk(s.nc), kB, 0, c->stream>>>(st->cq32, rh, st->winv32, st->pw32, Zk, static_cast<float*>(v.fx),
                                                static_cast<float*>(v.fy), s.nx, s.ny);
  EB_LAUNCHED(c);
  EB_PROF(c, "vcycle_graph");
  EB_CK(c, cudaGraphLaunch(st->H().gexec, c->stream));
  c->launches += st->H().graph_kernels - 1;
  EB_LAUNCHED(c);
  EB_PROF(c, "k_precond");
  k_prec_out32<<<nblk(s.nc), kB, 0, c->stream>>>(static_cast<float*>(v.ux), static_cast<float*>(v.uy), st->winv32, Zk,
                                                 s.nc);
  EB_LAUNCHED(c);
  return EB_OK;
}

// dots[v] = V_v . u for v < nv (device), copied to host h
int mdot(eb_ctx* c, StokesState* st, const double* V, int64_t stride, int nv, const double* u, double* h) {
  const int64_t n3 = 3 * st->sys.nc;
  // blocks per vector: at least 8 elements per thread, at most kDotBlocks
  const int nb = (int)std::min<int64_t>(st->nb_dot, std::max<int64_t>(1, (n3 + 8 * kB - 1) / (8 * kB)));
  EB_PROF(c, "k_mdot");
  k_mdot<<<dim3(nb, nv), kB, 0, c->stream>>>(V, stride, u, n3, st->partial);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_mdot");
  k_mdot_final<<<nv, kB, 0, c->stream>>>(st->partial, nb, st->dots);
  EB_LAUNCHED(c);
  EB_CK(c, cudaMemcpyAsync(h, st->dots, nv * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}

// h[v] = V32_v . V32_{nv-1} for v < nv (the last slot holds the FP32 copy of the new direction)
int mdot32(eb_ctx* c, StokesState* st, int nv, double* h) {
  EB_PROF(c, "k_mdot32");
  k_mdot32<<<dim3(st->nb_split, (nv + kDot32Vecs - 1) / kDot32Vecs), kB, 0, c->stream>>>(
      st->V32, st->ld32, st->V32 + (size_t)(nv - 1) * st->ld32, st->ld32 / 4, nv, st->partial);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_mdot_final");
  k_mdot_final<<<nv, kB, 0, c->stream>>>(st->partial, st->nb_split, st->dots);
  EB_LAUNCHED(c);
  EB_CK(c, cudaMemcpyAsync(h, st->dots, nv * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}
// h[v] = V_v . V_{nv-1} for v < nv on the split basis (slot nv-1 holds the new direction)
int mdot_df(eb_ctx* c, StokesState* st, int nv, double* h) {
  EB_PROF(c, "k_mdot_df");
  k_mdot_df<<<dim3(st->nb_split, (nv + kDfVecs - 1) / kDfVecs), kB, 0, c->stream>>>(st->V32, st->V32lo, st->ld32,
                                                                                    st->ld32 / 4, nv, st->partial);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_mdot_final");
  k_mdot_final<<<nv, kB, 0, c->stream>>>(st->partial, st->nb_split, st->dots);
  EB_LAUNCHED(c);
  EB_CK(c, cudaMemcpyAsync(h, st->dots, nv * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}
// slot nv -= sum_{v<nv} hdev[v] V_v on the split basis (double-float); *wn2 = |slot nv|^2
int maxpy_df(eb_ctx* c, StokesState* st, int nv, double* wn2) {
  EB_PROF(c, "k_maxpy_df");
  auto kern = st->ax_p == 2 ? k_maxpy_df<2> : k_maxpy_df<1>;
  kern<<<st->nb_ax32, kAxThreads, (size_t)2 * nv * sizeof(float), c->stream>>>(
      st->V32, st->V32lo, st->ld32, st->hdev, nv, st->V32 + (size_t)nv * st->ld32, st->V32lo + (size_t)nv * st->ld32,
      st->part32);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_mdot_final");
  k_mdot_final<<<1, kB, 0, c->stream>>>(st->part32, st->nb_ax32, st->dots);
  EB_LAUNCHED(c);
  EB_CK(c, cudaMemcpyAsync(wn2, st->dots, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}
// the same with the sum over the FP32 hi parts in FP32
int maxpy32(eb_ctx* c, StokesState* st, int nv, double* wn2) {
  EB_PROF(c, "k_maxpy32");
  auto kern = st->ax_p == 2 ? k_maxpy32<2> : k_maxpy32<1>;
  kern<<<st->nb_ax32, kAxThreads, (size_t)nv * sizeof(float), c->stream>>>(
      st->V32, st->V32lo + (size_t)nv * st->ld32, st->ld32, st->hdev, nv, st->part32);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_mdot_final");
  k_mdot_final<<<1, kB, 0, c->stream>>>(st->part32, st->nb_ax32, st->dots);
  EB_LAUNCHED(c);
  EB_CK(c, cudaMemcpyAsync(wn2, st->dots, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}

int apply_scaled(eb_ctx* c, StokesState* st, const double* x, double* y) {
  const StokesSystem& s = st->sys;
  EB_PROF(c, "k_apply64");
  k_apply64<<<nblk(s.nc), kB, 0, c->stream>>>(st->coefS, x, y, s.nx, s.ny, (int32_t)s.nc);
  EB_LAUNCHED(c);
  return EB_OK;
}

int ensure_solver(eb_ctx* c, StokesState* st, int m) {
  auto drop = [&](void* p) {
    if (!p) return;
    cudaFree(p);
    st->allocs.erase(std::remove(st->allocs.begin(), st->allocs.end(), p), st->allocs.end());
  };
  const size_t n3 = 3 * (size_t)st->sys.nc;
  int rc;
  if (st->m != m || !st->V) {  // (re)allocate the Krylov workspace for m directions
    drop(st->V);
    drop(st->Z);
    drop(st->Zd);
    drop(st->V32);
    drop(st->V32lo);
    st->V32lo = nullptr;
    st->V = nullptr;
    st->Z = nullptr;
    st->Zd = nullptr;
    st->V32 = nullptr;
    st->m = m;
    st->nb_dot = kDotBlocks;
    if ((rc = dalloc(c, st->allocs, &st->V, (size_t)(m + 2) * n3))) return rc;
  }
  // stored directions of the method in use (FP32 mixed, FP64 plain), kept once allocated
  if (st->mg64 && !st->Zd && (rc = dalloc(c, st->allocs, &st->Zd, (size_t)m * n3))) return rc;
  if (!st->mg64 && !st->Z && (rc = dalloc(c, st->allocs, &st->Z, (size_t)m * n3))) return rc;
  if (!st->mg64 && !st->V32) {  // FP32 basis copies, zero padding between the slots
    st->ld32 = (int64_t)((n3 + 3) & ~(size_t)3);
    const int64_t n4 = st->ld32 / 4;
    st->ax_p = n4 >= kAxP2Chunks ? 2 : 1;
    st->nb_ax32 = (int)((n4 + kAxThreads * st->ax_p - 1) / (kAxThreads * st->ax_p));
    // dot-product blocks per group of basis vectors: at least 8 float4 chunks per thread
    st->nb_split = (int)std::min<int64_t>(kDotBlocks, std::max<int64_t>(1, (n4 + 8 * kB - 1) / (8 * kB)));
    if ((rc = dalloc(c, st->allocs, &st->V32, (size_t)(m + 2) * st->ld32))) return rc;
    EB_CK(c, cudaMemsetAsync(st->V32, 0, (size_t)(m + 2) * st->ld32 * sizeof(float), c->stream));
    drop(st->V32lo);
    if ((rc = dalloc(c, st->allocs, &st->V32lo, (size_t)(m + 2) * st->ld32))) return rc;
    EB_CK(c, cudaMemsetAsync(st->V32lo, 0, (size_t)(m + 2) * st->ld32 * sizeof(float), c->stream));
    drop(st->part32);
    if ((rc = dalloc(c, st->allocs, &st->part32, (size_t)st->nb_ax32))) return rc;
  }
  if (!st->r) {
    if ((rc = dalloc(c, st->allocs, &st->r, n3)) || (rc = dalloc(c, st->allocs, &st->t, n3)) ||
        (rc = dalloc(c, st->allocs, &st->xs, n3)) || (rc = dalloc(c, st->allocs, &st->bs, n3)) ||
        (rc = dalloc(c, st->allocs, &st->zt, n3)) ||
        (rc = dalloc(c, st->allocs, &st->w, n3)) || (rc = dalloc(c, st->allocs, &st->winv, n3)) ||
        (rc = dalloc(c, st->allocs, &st->prep, (size_t)st->sys.nc)) ||
        (rc = dalloc(c, st->allocs, &st->partial, (size_t)st->nb_dot * kMaxDots)) ||
        (rc = dalloc(c, st->allocs, &st->dots, kMaxDots)) || (rc = dalloc(c, st->allocs, &st->hdev, kMaxDots)))
      return rc;
  }
  return EB_OK;
}

// The learned stage after the V-cycle (z = zt): t = v - A z, z2 = NN(t), and z += a z2 with
// the step a = <t, A z2> / |A z2|^2 that minimises |t - a A z2|; kept when a > 0, i.e. when
// it lowers the preconditioner residual (the multigrid alone otherwise).
int learned_stage(eb_ctx* c, StokesState* st, const double* v, double* zt, float* Zk) {  // FP32 method only
  const auto t0 = std::chrono::steady_clock::now();
  const StokesSystem& s = st->sys;
  const int64_t n3 = 3 * s.nc;
  int rc;
  if (!st->nn_t) {  // t and q adjacent: one reduction gives t.q and q.q
    if ((rc = dalloc(c, st->allocs, &st->nn_t, 2 * n3)) || (rc = dalloc(c, st->allocs, &st->nn_z, n3))) return rc;
    st->nn_q = st->nn_t + n3;
  }
  if ((rc = apply_scaled(c, st, zt, st->nn_q))) return rc;
  EB_PROF(c, "k_axpy");
  k_sub<<<nblk(n3), kB, 0, c->stream>>>(st->nn_t, v, st->nn_q, n3);
  EB_LAUNCHED(c);
  double tt;
  if ((rc = mdot(c, st, st->nn_t, 0, 1, st->nn_t, &tt))) return rc;
  bool keep = false;
  if (tt > 0.0 && std::isfinite(tt)) {
    if ((rc = nn_correction(c, st->nn_t, std::sqrt(tt / n3), st->nn_z)) || (rc = apply_scaled(c, st, st->nn_z, st->nn_q)))
      return rc;
    double d[2];  // t.q, q.q
    if ((rc = mdot(c, st, st->nn_t, n3, 2, st->nn_q, d))) return rc;
    keep = std::isfinite(d[0]) && std::isfinite(d[1]) && d[1] > 0.0 && d[0] > 0.0;
    if (keep) {
      EB_PROF(c, "k_axpy");
      k_add_round<<<nblk(n3), kB, 0, c->stream>>>(zt, Zk, st->nn_z, d[0] / d[1], n3);
      EB_LAUNCHED(c);
    }
    nn_count(c, keep, std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(),
             keep ? d[0] * d[0] / (d[1] * tt) : 0.0);
  } else {
    nn_count(c, false, std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(), 0.0);
  }
  return EB_OK;
}

// Scaling, multigrid hierarchy and captured V-cycle of the current system, in FP32 or FP64.
int prepare(eb_ctx* c, StokesState* st, int sweeps, int m, bool fp64) {
  int rc;
  st->mg64 = fp64;  // selects the hierarchy and the stored-direction buffer
  B2 b2;
  if ((rc = ensure_solver(c, st, m)) || (rc = read_b2(c, &b2))) return rc;
  if (st->H().levels.empty() || std::memcmp(&b2, &st->H().b2_levels, sizeof(B2)) != 0) {
    if ((rc = setup_levels(c, st, b2))) return rc;
    st->H().b2_levels = b2;
  }
  if ((rc = refresh_levels(c, st, b2)) || (rc = capture_vcycle(c, st, sweeps))) return rc;
  const StokesSystem& s = st->sys;
  EB_PROF(c, "k_scaling");
  k_scaling<<<nblk(s.nc), kB, 0, c->stream>>>(s.coef, c->gf[EB_G_ETAN0], s.pscale, st->w, st->prep, st->winv, s.nc);
  EB_LAUNCHED(c);
  if (s.nc >= (int64_t)1 << 30) return eb_fail(c, EB_BAD_INPUT, "Stokes grid exceeds 2^30 cells");
  if (!st->coefS && (rc = dalloc(c, st->allocs, &st->coefS, (size_t)kStencilSlots * s.nc))) return rc;
  EB_PROF(c, "k_scaling");
  k_prescale<<<nblk(s.nc), kB, 0, c->stream>>>(s.coef, st->w, st->coefS, s.nx, s.ny, (int32_t)s.nc);
  EB_LAUNCHED(c);
  if (!fp64) {
    if (!st->coefH && ((rc = dalloc(c, st->allocs, &st->coefH, (size_t)kStencilSlots * s.nc)) ||
                       (rc = dalloc(c, st->allocs, &st->coefL, (size_t)kStencilSlots * s.nc)) ||
                       (rc = dalloc(c, st->allocs, &st->cq32, (size_t)4 * s.nc)) ||
                       (rc = dalloc(c, st->allocs, &st->winv32, (size_t)3 * s.nc)) ||
                       (rc = dalloc(c, st->allocs, &st->pw32, (size_t)s.nc))))
      return rc;
    EB_PROF(c, "k_scaling");
    k_split_setup<<<nblk(s.nc), kB, 0, c->stream>>>(st->coefS, s.coef, st->winv, st->prep, st->coefH, st->coefL,
                                                    st->cq32, st->winv32, st->pw32, s.nc);
    EB_LAUNCHED(c);
  }
  return EB_OK;
}

}  // namespace

// ------------------------------------------------------------ C-ABI ---
static int need_system(eb_ctx* c, bool built) {
  if (!c) return EB_BAD_INPUT;
  if (!c->have_grid) return eb_fail(c, EB_NOT_READY, "eb_set_grid has not been called");
  cudaSetDevice(c->device);
  if (!stokes_system(c)) return eb_fail(c, EB_CUDA_ERROR, "out of device memory for the Stokes system");
  if (built && !c->st->sys.built) return eb_fail(c, EB_NOT_READY, "eb_build_stokes_system has not been called");
  return EB_OK;
}

// One solve with one method.  With `stall_check` (the mixed method when the fallback is on),
// the solve also stops when the true FP64 residual at the start of an FGMRES cycle is not
// below kStallFactor times its value at the start of the previous cycle, and reports that
// as EB_NOT_CONVERGED: the residual has stopped falling.
static int solve_once(eb_ctx* c, eb_solve_opts opt, bool stall_check, eb_solve_report* rep, bool* input_nan) {
  int rc;
  const auto t0 = std::chrono::steady_clock::now();
  StokesState* st = c->st;
  StokesSystem& s = st->sys;
  if (opt.rtol <= 0) opt.rtol = 1e-8;
  if (opt.max_iters <= 0) opt.max_iters = 3000;
  if (opt.restart <= 0) opt.restart = kMaxRestart;
  if (opt.mg_sweeps <= 0) opt.mg_sweeps = 3;
  st->gcr_steps = opt.mg_inner <= 0 ? kGcrDefaultSteps : std::min(opt.mg_inner, kGcrMax);
  st->gcr_tol = opt.mg_inner_tol > 0.0 ? opt.mg_inner_tol : kGcrDefaultTol;
  st->gcr_total = 0;
  if (opt.method != 1) opt.method = 0;
  const int m = std::max(std::min(opt.restart, kMaxRestart), opt.method == 1 ? 6 : 1);
  const int64_t n3 = 3 * s.nc;
  if (opt.learned && !nn_trained(c))
    return eb_fail(c, EB_NOT_READY, "learned stage requested but eb_learned_train has not run");
  const bool use_nn = opt.learned != 0 && opt.method != 1;
  if (opt.precision != 0 && opt.precision != 1) return eb_fail(c, EB_BAD_INPUT, "precision must be 0 (mixed) or 1 (FP64)");
  if (use_nn && opt.precision == 1) return eb_fail(c, EB_BAD_INPUT, "the learned stage runs with the mixed method");
  if ((rc = prepare(c, st, opt.mg_sweeps, m, opt.precision == 1))) return rc;
  // bhat = W R, xhat = W^-1 S0
  EB_PROF(c, "k_axpy");
  k_mul<<<nblk(n3), kB, 0, c->stream>>>(st->bs, s.rhs, st->w, n3, 0);
  EB_LAUNCHED(c);
  if (opt.use_initial_guess) {
    // S from an earlier system keeps the velocities, and its pressure unknowns p / pscale are
    // brought to this system's pressure scale
    if (s.S_pscale > 0.0 && s.S_pscale != s.pscale) {
      EB_PROF(c, "k_axpy");
      k_scale_copy<<<nblk(s.nc), kB, 0, c->stream>>>(s.S + 2 * s.nc, s.S + 2 * s.nc, s.S_pscale / s.pscale, s.nc);
      EB_LAUNCHED(c);
      s.S_pscale = s.pscale;
    }
    EB_PROF(c, "k_axpy");
    k_mul<<<nblk(n3), kB, 0, c->stream>>>(st->xs, s.S, st->w, n3, 1);
    EB_LAUNCHED(c);
  } else {
    EB_CK(c, cudaMemsetAsync(st->xs, 0, n3 * sizeof(double), c->stream));
  }
  double bn2;
  if ((rc = mdot(c, st, st->bs, 0, 1, st->bs, &bn2))) return rc;
  if (use_nn && opt.use_initial_guess && opt.learned_warm) {
    // the learned stage as a warm start: xhat += a NN(bhat - Khat xhat) when that lowers the
    // residual (the stage's own step and acceptance test); the first stored-direction slot is
    // scratch here
    if ((rc = learned_stage(c, st, st->bs, st->xs, st->Z))) return rc;
  }
  const double bnorm = std::sqrt(bn2);
  if (!std::isfinite(bnorm)) {
    *input_nan = true;
    return eb_fail(c, EB_NAN, "right-hand side has NaN/Inf");
  }
  std::vector<double> H((size_t)(m + 1) * m), g(m + 1), cs(m), sn(m), hcol(m + 2), y(m);
  int it = 0, reorth = 0, relaxed = 0;
  double est = 1.0;
  // The mixed method's FGMRES (without the learned stage or the GCR velocity stage) runs its
  // Arnoldi step on split vectors in double-float; once the residual estimate falls below
  // gs_relax x the target its Gram-Schmidt products are FP32.  gs_relax < 0 keeps the FP64 step.
  const double relax_fac = opt.gs_relax == 0.0 ? kGsRelax : opt.gs_relax;
  const bool split = !st->mg64 && relax_fac > 0.0 && !use_nn && st->gcr_steps <= 1;
  // The Krylov methods run on the scaled system, whose residual norm weights rows by W; the
  // tolerance is on the reference's (unscaled) residual ||R - L S|| / ||R||.  When the scaled
  // target is reached but the unscaled residual is still above rtol, the target is tightened
  // by their ratio and the method restarts from the current iterate.
  double target = opt.rtol, rel = 0.0, rel_s = 0.0;
  double prev_beta = HUGE_VAL;
  bool stalled = false;
  for (int outer = 0;; ++outer) {
  bool converged = (bnorm == 0.0);
  if (opt.method == 1 && !converged) {
    // Right-preconditioned BiCGStab on the scaled system.  Basis slots hold its vectors:
    // 0 r0hat, 1 r (adjacent: one reduction gives r0hat.r and r.r), 2 s, 3 t (s.t, t.t),
    // 4 p, 5 v, 6 shat; phat is zt.  The FP32 copy of each preconditioned vector goes to Z.
    double *rh0 = st->V, *r = st->V + n3, *sv = st->V + 2 * n3, *tv = st->V + 3 * n3, *p = st->V + 4 * n3,
           *v = st->V + 5 * n3, *sh = st->V + 6 * n3, *ph = st->zt;
    if ((rc = apply_scaled(c, st, st->xs, st->t))) return rc;
    EB_PROF(c, "k_axpy");
    k_sub<<<nblk(n3), kB, 0, c->stream>>>(r, st->bs, st->t, n3);
    EB_LAUNCHED(c);
    EB_CK(c, cudaMemcpyAsync(rh0, r, n3 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    EB_CK(c, cudaMemsetAsync(p, 0, n3 * sizeof(double), c->stream));
    EB_CK(c, cudaMemsetAsync(v, 0, n3 * sizeof(double), c->stream));
    double rho = 1.0, alpha = 1.0, omega = 1.0, d2[2];
    if ((rc = mdot(c, st, rh0, n3, 2, r, d2))) return rc;
    double rho_new = d2[0];
    est = std::sqrt(d2[1]) / bnorm;
    converged = est <= target;
    while (!converged && it < opt.max_iters) {
      if (rho_new == 0.0 || omega == 0.0 || !std::isfinite(rho_new))
        return eb_fail(c, std::isfinite(rho_new) ? EB_NOT_CONVERGED : EB_NAN, "BiCGStab breakdown");
      const double beta = (rho_new / rho) * (alpha / omega);
      rho = rho_new;
      EB_PROF(c, "k_axpy");
      k_bicg_p<<<nblk(n3), kB, 0, c->stream>>>(p, r, v, beta, omega, n3);
      EB_LAUNCHED(c);
      void* z0 = st->mg64 ? (void*)st->Zd : (void*)st->Z;
      if ((rc = precondition(c, st, p, ph, z0)) || (rc = apply_scaled(c, st, ph, v))) return rc;
      double rv;
      if ((rc = mdot(c, st, rh0, 0, 1, v, &rv))) return rc;
      alpha = rho / rv;
      EB_PROF(c, "k_axpy");
      k_bicg_s<<<nblk(n3), kB, 0, c->stream>>>(sv, r, v, alpha, n3);
      EB_LAUNCHED(c);
      if ((rc = precondition(c, st, sv, sh, z0)) || (rc = apply_scaled(c, st, sh, tv))) return rc;
      double st2[2];
      if ((rc = mdot(c, st, sv, n3, 2, tv, st2))) return rc;  // s.t, t.t
      omega = st2[1] > 0.0 ? st2[0] / st2[1] : 0.0;
      EB_PROF(c, "k_axpy");
      k_bicg_xr<<<nblk(n3), kB, 0, c->stream>>>(st->xs, r, ph, sh, sv, tv, alpha, omega, n3);
      EB_LAUNCHED(c);
      ++it;
      if ((rc = mdot(c, st, rh0, n3, 2, r, d2))) return rc;
      rho_new = d2[0];
      est = std::sqrt(d2[1]) / bnorm;
      if (!std::isfinite(est)) return eb_fail(c, EB_NAN, "BiCGStab residual became NaN/Inf");
      converged = est <= target;
    }
  }
  while (opt.method != 1 && !converged && it < opt.max_iters) {
    // r = bhat - Khat xhat
    if ((rc = apply_scaled(c, st, st->xs, st->t))) return rc;
    EB_PROF(c, "k_axpy");
    k_sub<<<nblk(n3), kB, 0, c->stream>>>(st->r, st->bs, st->t, n3);
    EB_LAUNCHED(c);
    double beta2;
    if ((rc = mdot(c, st, st->r, 0, 1, st->r, &beta2))) return rc;
    const double beta = std::sqrt(beta2);
    if (!std::isfinite(beta)) return eb_fail(c, EB_NAN, "FGMRES residual became NaN/Inf");
    est = beta / bnorm;
    if (est <= target) { converged = true; break; }
    if (stall_check && beta > kStallFactor * prev_beta) { stalled = true; break; }
    prev_beta = beta;
    EB_PROF(c, "k_axpy");
    if (split)
      k_split_scale<<<nblk(n3), kB, 0, c->stream>>>(st->V32, st->V32lo, st->r, 1.0 / beta, n3);
    else
      k_scale_copy2<<<nblk(n3), kB, 0, c->stream>>>(st->V, st->r, 1.0 / beta, n3);
    EB_LAUNCHED(c);
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int k = 0;
    for (; k < m && it < opt.max_iters; ++k) {
      double* vk = st->V + (size_t)k * n3;
      void* zk = st->mg64 ? (void*)(st->Zd + (size_t)k * n3) : (void*)(st->Z + (size_t)k * n3);
      double* w = st->V + (size_t)(k + 1) * n3;
      float* const vh = st->V32 + (size_t)k * st->ld32;
      float* const vl = st->V32lo + (size_t)k * st->ld32;
      float* const wh = vh + st->ld32;
      float* const wl = vl + st->ld32;
      const bool relax = split && std::fabs(g[k]) <= relax_fac * target * bnorm;
      std::vector<double> h(k + 2);
      if (split) {
        // Shifted Arnoldi (see the FP64 form below) on split vectors; classical Gram-Schmidt
        // with the norm measured in the update's pass, a second pass if the projection removed
        // all but 5% of the norm
        if ((rc = precondition32(c, st, vh, static_cast<float*>(zk)))) return rc;
        if (relax) ++relaxed;
        EB_PROF(c, "k_apply_df");
        k_apply_df<<<nblk(s.nc), kB, 0, c->stream>>>(st->coefH, st->coefL, static_cast<float*>(zk), vh, vl, wh, wl, s.nx,
                                                     s.ny, (int32_t)s.nc);
        EB_LAUNCHED(c);
        auto dots = [&]() { return relax ? mdot32(c, st, k + 2, h.data()) : mdot_df(c, st, k + 2, h.data()); };
        if ((rc = dots())) return rc;
        double wn2_before = h[k + 1];
        for (int pass = 0; pass < 2; ++pass) {
          EB_CK(c, cudaMemcpyAsync(st->hdev, h.data(), (k + 1) * sizeof(double), cudaMemcpyHostToDevice, c->stream));
          double wn2 = 0.0;
          if ((rc = relax ? maxpy32(c, st, k + 1, &wn2) : maxpy_df(c, st, k + 1, &wn2))) return rc;
          for (int q = 0; q <= k; ++q) hcol[q] = (pass == 0 ? 0.0 : hcol[q]) + h[q];
          if (pass == 1 || wn2 > kReorth2 * wn2_before) {
            hcol[k + 1] = std::sqrt(wn2);
            break;
          }
          ++reorth;
          if ((rc = dots())) return rc;
          wn2_before = wn2;
        }
      } else {
        if ((rc = precondition(c, st, vk, st->zt, zk))) return rc;
        if (use_nn && (rc = learned_stage(c, st, vk, st->zt, static_cast<float*>(zk)))) return rc;
        // Shifted Arnoldi: with a good preconditioner A z_k is close to v_k, so the slot holds
        // d = A z_k - v_k and the projection starts from d (h_kk gets the 1 back below); the
        // cancellation that classical Gram-Schmidt suffers is then measured against |d|.
        EB_PROF(c, "k_apply64");
        k_apply64<<<nblk(s.nc), kB, 0, c->stream>>>(st->coefS, st->zt, w, s.nx, s.ny, (int32_t)s.nc, vk);
        EB_LAUNCHED(c);
        // Classical Gram-Schmidt.  One reduction gives V^T d and |d|^2 (d is the slot after V_k);
        // the projected norm follows from Pythagoras unless cancellation is large, in which
        // case a second pass re-orthogonalises and the norm is measured.
        if ((rc = mdot(c, st, st->V, n3, k + 2, w, h.data()))) return rc;
        double wn2_before = h[k + 1];
        for (int pass = 0; pass < 2; ++pass) {
          EB_CK(c, cudaMemcpyAsync(st->hdev, h.data(), (k + 1) * sizeof(double), cudaMemcpyHostToDevice, c->stream));
          EB_PROF(c, "k_maxpy");
          k_maxpy<<<(unsigned)((n3 + kAxTile - 1) / kAxTile), kAxThreads, (size_t)(k + 1) * sizeof(double),
                    c->stream>>>(w, st->V, n3, st->hdev, k + 1, n3);
          EB_LAUNCHED(c);
          double proj = 0.0;
          for (int q = 0; q <= k; ++q) {
            hcol[q] = (pass == 0 ? 0.0 : hcol[q]) + h[q];
            proj += h[q] * h[q];
          }
          const double est = wn2_before - proj;
          if (pass == 0 && est > kReorth2 * wn2_before) {  // no severe cancellation: keep
            hcol[k + 1] = std::sqrt(est);
            break;
          }
          ++reorth;
          if ((rc = mdot(c, st, st->V, n3, k + 2, w, h.data()))) return rc;
          if (pass == 1) {
            hcol[k + 1] = std::sqrt(h[k + 1]);
            break;
          }
          wn2_before = h[k + 1];
        }
      }
      hcol[k] += 1.0;
      if (!std::isfinite(hcol[k + 1])) return eb_fail(c, EB_NAN, "FGMRES basis became NaN/Inf");
      // apply the previous rotations, then a new one
      for (int q = 0; q < k; ++q) {
        const double a = cs[q] * hcol[q] + sn[q] * hcol[q + 1];
        hcol[q + 1] = -sn[q] * hcol[q] + cs[q] * hcol[q + 1];
        hcol[q] = a;
      }
      const double d = std::hypot(hcol[k], hcol[k + 1]);
      cs[k] = (d == 0.0) ? 1.0 : hcol[k] / d;
      sn[k] = (d == 0.0) ? 0.0 : hcol[k + 1] / d;
      const double hk1 = hcol[k + 1];
      hcol[k] = d;
      for (int q = 0; q <= k; ++q) H[(size_t)q * m + k] = hcol[q];
      g[k + 1] = -sn[k] * g[k];
      g[k] = cs[k] * g[k];
      ++it;
      est = std::fabs(g[k + 1]) / bnorm;
      if (hk1 > 0.0) {
        EB_PROF(c, "k_axpy");
        if (split) {
          const double a = 1.0 / hk1;  // as an FP32 pair
          const float ah = (float)a, al = (float)(a - (double)ah);
          k_scale_df<<<nblk(n3), kB, 0, c->stream>>>(wh, wl, ah, al, n3);
        } else {
          k_scale_copy2<<<nblk(n3), kB, 0, c->stream>>>(w, w, 1.0 / hk1, n3);
        }
        EB_LAUNCHED(c);
      }
      if (est <= target || hk1 == 0.0) { ++k; break; }
    }
    // y = H^-1 g (upper triangular k x k), xhat += Z y
    for (int q = k - 1; q >= 0; --q) {
      double sacc = g[q];
      for (int p = q + 1; p < k; ++p) sacc -= H[(size_t)q * m + p] * y[p];
      y[q] = sacc / H[(size_t)q * m + q];
    }
    std::vector<double> negy(k);
    for (int q = 0; q < k; ++q) negy[q] = -y[q];
    EB_CK(c, cudaMemcpyAsync(st->hdev, negy.data(), k * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    EB_PROF(c, "k_maxpy");
    if (st->mg64)
      k_maxpy<<<(unsigned)((n3 + kAxTile - 1) / kAxTile), kAxThreads, (size_t)std::max(k, 1) * sizeof(double),
                c->stream>>>(st->xs, st->Zd, n3, st->hdev, k, n3);
    else
      k_update_df<<<nblk(n3), kB, (size_t)2 * std::max(k, 1) * sizeof(float), c->stream>>>(st->xs, st->Z, n3, st->hdev,
                                                                                          k, n3);
    EB_LAUNCHED(c);
    EB_CK(c, cudaStreamSynchronize(c->stream));
  }
  // S = W xhat; true residual of the unscaled system
  EB_PROF(c, "k_axpy");
  k_mul<<<nblk(n3), kB, 0, c->stream>>>(s.S, st->xs, st->w, n3, 0);
  EB_LAUNCHED(c);
  s.S_pscale = s.pscale;
  EB_PROF(c, "k_apply64");
  k_apply64<<<nblk(s.nc), kB, 0, c->stream>>>(s.coef, s.S, st->t, s.nx, s.ny, (int32_t)s.nc);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_axpy");
  k_sub<<<nblk(n3), kB, 0, c->stream>>>(st->r, s.rhs, st->t, n3);
  EB_LAUNCHED(c);
  double rr, RR, sr2;
  if ((rc = mdot(c, st, st->r, 0, 1, st->r, &rr)) || (rc = mdot(c, st, s.rhs, 0, 1, s.rhs, &RR))) return rc;
  // scaled residual of the final iterate
  if ((rc = apply_scaled(c, st, st->xs, st->t))) return rc;
  EB_PROF(c, "k_axpy");
  k_sub<<<nblk(n3), kB, 0, c->stream>>>(st->r, st->bs, st->t, n3);
  EB_LAUNCHED(c);
  if ((rc = mdot(c, st, st->r, 0, 1, st->r, &sr2))) return rc;
  rel = RR > 0 ? std::sqrt(rr / RR) : std::sqrt(rr);
  rel_s = bnorm > 0 ? std::sqrt(sr2) / bnorm : std::sqrt(sr2);
  if (!std::isfinite(rel)) break;
  if (stalled || rel <= opt.rtol || it >= opt.max_iters || outer >= 8 || bnorm == 0.0) break;
  target = std::min(target, rel_s) * std::max(0.5 * opt.rtol / rel, 1e-4);
  }  // outer
  prof_resolve(c);
  if (rep) {
    rep->iterations = it;
    rep->reorthogonalisations = reorth;
    rep->relaxed_iterations = relaxed;
    rep->levels = (int32_t)st->H().levels.size();
    rep->rel_residual = rel;
    rep->rel_residual_scaled = rel_s;
    rep->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    rep->fallback_used = 0;
    rep->precision_used = opt.precision;
    rep->vcycles = st->gcr_steps > 1 ? st->gcr_total : it;
  }
  if (!std::isfinite(rel)) return eb_fail(c, EB_NAN, "Stokes solution has NaN/Inf");
  if (rel > opt.rtol * 1.0000001)
    return eb_fail(c, EB_NOT_CONVERGED, std::string(stalled ? "Stokes residual stopped falling at " :
                                                              "Stokes solve stopped at relative residual ") +
                                            std::to_string(rel) + " after " + std::to_string(it) + " iterations");
  return EB_OK;
}

// The mixed method falls back to the plain FP64 method whenever its FP64 residual fails to
// fall: when it stops without meeting the tolerance (iteration limit, or a cycle that did not
// lower the true residual), the plain method continues from its iterate with a budget of
// max_iters iterations of its own; when it produced NaN/Inf, the plain method starts from
// zero.  The report then sums both attempts and names the method that finished.
extern "C" int eb_solve_stokes_system(eb_ctx* c, const eb_solve_opts* o, eb_solve_report* rep) {
  int rc = need_system(c, true);
  if (rc) return rc;
  const eb_solve_opts opt = o ? *o : eb_solve_opts{};
  const bool fallback = opt.precision == 0 && opt.fallback >= 0;
  eb_solve_report r1{};
  bool input_nan = false;
  rc = solve_once(c, opt, fallback, &r1, &input_nan);
  if (rep) *rep = r1;
  if (!fallback || input_nan || (rc != EB_NOT_CONVERGED && rc != EB_NAN)) return rc;
  eb_solve_opts o2 = opt;
  o2.precision = 1;
  o2.learned = 0;
  o2.use_initial_guess = rc == EB_NAN ? 0 : 1;
  eb_solve_report r2{};
  const int rc2 = solve_once(c, o2, false, &r2, &input_nan);
  if (rep) {
    *rep = r2;
    rep->iterations = r1.iterations + r2.iterations;
    rep->reorthogonalisations = r1.reorthogonalisations + r2.reorthogonalisations;
    rep->relaxed_iterations = r1.relaxed_iterations;
    rep->seconds = r1.seconds + r2.seconds;
    rep->fallback_used = 1;
    rep->precision_used = 1;
    rep->vcycles = r1.vcycles + r2.vcycles;
  }
  return rc2;
}

extern "C" int eb_set_stokes_params(eb_ctx* c, const eb_stokes_params* p) {
  if (!c || !p) return EB_BAD_INPUT;
  if (p->pressure_bc_mode < 0 || p->pressure_bc_mode > 2) return eb_fail(c, EB_BAD_INPUT, "pressure_bc_mode must be 0, 1 or 2");
  c->SP = *p;
  c->have_stokes_params = true;
  return EB_OK;
}

static int need_fields(eb_ctx* c, std::initializer_list<int> ids) {
  for (int f : ids) {
    int rc = ensure_grid_field(c, f);
    if (rc) return rc;
  }
  return EB_OK;
}

extern "C" int eb_calc_viscoelastic_terms(eb_ctx* c) {
  if (!c) return EB_BAD_INPUT;
  if (!c->have_grid || !c->have_params) return eb_fail(c, EB_NOT_READY, "eb_set_grid and eb_set_params come first");
  cudaSetDevice(c->device);
  int rc = need_fields(c, {EB_G_ETAS1, EB_G_MUS1, EB_G_SXY1, EB_G_ETAS0, EB_G_SXY0, EB_G_ETAN1, EB_G_MUN1, EB_G_SXX1,
                           EB_G_ETAN0, EB_G_SXX0});
  if (rc || (rc = launch_viscoelastic_terms(c))) return rc;
  EB_CK(c, cudaStreamSynchronize(c->stream));
  prof_resolve(c);
  return EB_OK;
}

extern "C" int eb_viscoelastic_rhs(eb_ctx* c) {
  if (!c) return EB_BAD_INPUT;
  if (!c->have_grid || !c->have_stokes_params) return eb_fail(c, EB_NOT_READY, "eb_set_grid and eb_set_stokes_params come first");
  cudaSetDevice(c->device);
  int rc = need_fields(c, {EB_G_RHO1, EB_G_RHO1_VY, EB_G_SXX0, EB_G_SXY0, EB_G_DILAT, EB_G_EII_PLASTIC_PRESSURE, EB_G_RX1,
                           EB_G_RY1, EB_G_RC1});
  if (rc || (rc = launch_viscoelastic_rhs(c))) return rc;
  EB_CK(c, cudaStreamSynchronize(c->stream));
  prof_resolve(c);
  return EB_OK;
}

extern "C" int eb_build_stokes_system(eb_ctx* c) {
  int rc = need_system(c, false);
  if (rc) return rc;
  if (!c->have_params || !c->have_stokes_params) return eb_fail(c, EB_NOT_READY, "eb_set_params and eb_set_stokes_params come first");
  if ((rc = need_fields(c, {EB_G_ETAN0, EB_G_ETAS0, EB_G_RHO1_VY, EB_G_RX1, EB_G_RY1, EB_G_RC1, EB_G_BTOPX, EB_G_BBOTTOMX,
                            EB_G_BTOPY, EB_G_BBOTTOMY, EB_G_BLEFTX, EB_G_BRIGHTX, EB_G_BLEFTY, EB_G_BRIGHTY, EB_G_VX1,
                            EB_G_VY1, EB_G_PR1})))
    return rc;
  StokesSystem* s = &c->st->sys;
  // SystemSolver.initialize_solver!: zero vx1, vy1, pr1; pscale from etan0[1,1]
  const int32_t X = c->xnum, Y = c->ynum;
  EB_CK(c, cudaMemsetAsync(c->gf[EB_G_VX1], 0, sizeof(double) * (size_t)(Y + 1) * X, c->stream));
  EB_CK(c, cudaMemsetAsync(c->gf[EB_G_VY1], 0, sizeof(double) * (size_t)Y * (X + 1), c->stream));
  EB_CK(c, cudaMemsetAsync(c->gf[EB_G_PR1], 0, sizeof(double) * (size_t)(Y - 1) * (X - 1), c->stream));
  double etan11;
  EB_CK(c, cudaMemcpyAsync(&etan11, c->gf[EB_G_ETAN0], sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  s->pscale = 2.0 * etan11 / (c->g.xstpavg + c->g.ystpavg);
  if ((rc = launch_build_stokes_system(c, s))) return rc;
  EB_CK(c, cudaStreamSynchronize(c->stream));
  prof_resolve(c);
  s->built = true;
  return EB_OK;
}

static int grid_step(eb_ctx* c, std::initializer_list<int> fields, int (*launch)(eb_ctx*)) {
  if (!c) return EB_BAD_INPUT;
  if (!c->have_grid || !c->have_params) return eb_fail(c, EB_NOT_READY, "eb_set_grid and eb_set_params come first");
  cudaSetDevice(c->device);
  int rc = need_fields(c, fields);
  if (rc || (rc = launch(c))) return rc;
  EB_CK(c, cudaStreamSynchronize(c->stream));
  prof_resolve(c);
  return EB_OK;
}

extern "C" int eb_update_grid_strain_rate_and_spin(eb_ctx* c) {
  return grid_step(c, {EB_G_VX1, EB_G_VY1, EB_G_EXX, EB_G_EXY, EB_G_ESP, EB_G_EII}, launch_grid_strain_rate);
}
extern "C" int eb_forecast_viscoelastic_grid_stress(eb_ctx* c) {
  return grid_step(c, {EB_G_ETAS1, EB_G_MUS1, EB_G_EXY, EB_G_SXY1, EB_G_SXY2, EB_G_ETAN1, EB_G_MUN1, EB_G_EXX, EB_G_SXX1,
                       EB_G_SXX2}, launch_forecast_stress);
}
extern "C" int eb_calculate_deviatoric_grid_stress_change(eb_ctx* c) {
  return grid_step(c, {EB_G_SXY2, EB_G_SXY1, EB_G_DSXY, EB_G_SXX2, EB_G_SXX1, EB_G_DSXX}, launch_stress_change);
}
extern "C" int eb_interpolate_basic_viscoplastic_viscosity_to_pressure_grid(eb_ctx* c, int iuse_harmonic) {
  if (iuse_harmonic != 1) return c ? EB_OK : EB_BAD_INPUT;
  return grid_step(c, {EB_G_ETAS1, EB_G_PLASTICS, EB_G_PLASTICN, EB_G_PLASTIC_YIELD, EB_G_ETAN1}, launch_harmonic_etan);
}

extern "C" int eb_update_nodes_for_plastic_yielding(eb_ctx* c, const eb_mobile_wall* w, int64_t* nnode_yield,
                                                    double* global_yield_error) {
  if (!c) return EB_BAD_INPUT;
  if (!c->have_grid || !c->have_params) return eb_fail(c, EB_NOT_READY, "eb_set_grid and eb_set_params come first");
  cudaSetDevice(c->device);
  int rc = need_fields(c, {EB_G_PLASTIC_YIELD, EB_G_ETAS1, EB_G_ETA_FLOW, EB_G_MUS1, EB_G_COHESION, EB_G_FRIC_DEG,
                           EB_G_SXY2, EB_G_SXX2, EB_G_PR1, EB_G_YIELD_ERROR, EB_G_ETAVP_BUFFER,
                           EB_G_PLASTIC_STRAIN_RATE_BUFFER, EB_G_PLASTIC_YIELD_BUFFER});
  if (rc) return rc;
  // per-block partial sums go to the context's per-cell scratch (kMaxSlots floats per cell,
  // far more than 2 doubles per 256 basic nodes)
  double* d_part = reinterpret_cast<double*>(c->part);
  int nb = 0;
  if ((rc = launch_nodal_yield(c, w, d_part, &nb))) return rc;
  std::vector<double> h(2 * (size_t)nb);
  EB_CK(c, cudaMemcpyAsync(h.data(), d_part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  prof_resolve(c);
  double cnt = 0.0, esum = 0.0;
  for (int b = 0; b < nb; ++b) { cnt += h[2 * b]; esum += h[2 * b + 1]; }
  const int64_t n = (int64_t)cnt;
  if (nnode_yield) *nnode_yield = n;
  if (global_yield_error) *global_yield_error = n > 0 ? std::sqrt(esum / (double)n) : 0.0;
  return EB_OK;
}

extern "C" int eb_apply_nodal_plastic_yielding(eb_ctx* c) {
  return grid_step(c, {EB_G_ETAS1, EB_G_ETAVP_BUFFER, EB_G_PLASTIC_YIELD, EB_G_PLASTIC_YIELD_BUFFER,
                       EB_G_EII_PLASTIC_BASIC, EB_G_PLASTIC_STRAIN_RATE_BUFFER, EB_G_EII_PLASTIC_PRESSURE},
                   launch_apply_nodal_yield);
}

extern "C" int eb_interpolate_stag_velocity_to_basic_grid(eb_ctx* c) {
  return grid_step(c, {EB_G_VX1, EB_G_VY1, EB_G_VXB, EB_G_VYB}, launch_stag_to_basic);
}

extern "C" int eb_process_stokes_solution(eb_ctx* c) {
  int rc = need_system(c, true);
  if (rc || (rc = need_fields(c, {EB_G_VX1, EB_G_VY1, EB_G_PR1}))) return rc;
  if ((rc = launch_process_stokes_solution(c, &c->st->sys))) return rc;
  EB_CK(c, cudaStreamSynchronize(c->stream));
  prof_resolve(c);
  return EB_OK;
}

extern "C" int eb_stokes_nonlinear_residual(eb_ctx* c) {
  int rc = need_system(c, true);
  if (rc) return rc;
  StokesSystem& s = c->st->sys;
  double* tmp = c->st->il;  // N doubles
  EB_PROF(c, "k_apply64");
  k_apply64<<<nblk(s.nc), kB, 0, c->stream>>>(s.coef, s.S_old, tmp, s.nx, s.ny, (int32_t)s.nc);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_axpy");
  k_abs_sub<<<nblk(3 * s.nc), kB, 0, c->stream>>>(s.resnl, tmp, s.rhs, 3 * s.nc);
  EB_LAUNCHED(c);
  EB_CK(c, cudaStreamSynchronize(c->stream));
  prof_resolve(c);
  return EB_OK;
}

extern "C" int eb_backup_stokes_arrays(eb_ctx* c) {
  int rc = need_system(c, false);
  if (rc || (rc = need_fields(c, {EB_G_VX1, EB_G_VY1, EB_G_PR1, EB_G_VX1_OLD, EB_G_VY1_OLD, EB_G_PR1_OLD}))) return rc;
  StokesSystem& s = c->st->sys;
  EB_CK(c, cudaMemcpyAsync(s.S_old, s.S, 3 * s.nc * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  const int pairs[3][2] = {{EB_G_VX1, EB_G_VX1_OLD}, {EB_G_VY1, EB_G_VY1_OLD}, {EB_G_PR1, EB_G_PR1_OLD}};
  for (const auto& pr : pairs)
    EB_CK(c, cudaMemcpyAsync(c->gf[pr[1]], c->gf[pr[0]], grid_field_count(c, pr[0]) * sizeof(double),
                             cudaMemcpyDeviceToDevice, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}

namespace {
// Per block: sum (a-b)^2, max |a-b|, sum a^2, max |a| (b may be null: b = 0).
__global__ void k_diff_norms(const double* __restrict__ a, const double* __restrict__ b, int64_t n,
                             double* __restrict__ partial) {
  double sd = 0.0, md = 0.0, sa = 0.0, ma = 0.0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const double x = a[k], d = fabs((b ? b[k] : 0.0) - x);
    sd += d * d;
    md = fmax(md, d);
    sa += x * x;
    ma = fmax(ma, fabs(x));
  }
  __shared__ double sh[4][kB];
  sh[0][threadIdx.x] = sd; sh[1][threadIdx.x] = md; sh[2][threadIdx.x] = sa; sh[3][threadIdx.x] = ma;
  __syncthreads();
  for (int o = kB / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + o];
      sh[1][threadIdx.x] = fmax(sh[1][threadIdx.x], sh[1][threadIdx.x + o]);
      sh[2][threadIdx.x] += sh[2][threadIdx.x + o];
      sh[3][threadIdx.x] = fmax(sh[3][threadIdx.x], sh[3][threadIdx.x + o]);
    }
    __syncthreads();
  }
  if (threadIdx.x < 4) partial[(int64_t)blockIdx.x * 4 + threadIdx.x] = sh[threadIdx.x][0];
}
}  // namespace

// {sum d^2, max d, sum a^2, max a} over the whole array, reduced on the host in block order
static int diff_norms(eb_ctx* c, const double* a, const double* b, int64_t n, double out[4]) {
  constexpr int nb = 2 * 152;
  double* part = c->st->tmp;  // 3 nc >= 4 nb doubles for every grid of at least 3x3 nodes
  EB_PROF(c, "k_diff_norms");
  k_diff_norms<<<nb, kB, 0, c->stream>>>(a, b, n, part);
  EB_LAUNCHED(c);
  std::vector<double> h(4 * nb);
  EB_CK(c, cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  out[0] = out[1] = out[2] = out[3] = 0.0;
  for (int k = 0; k < nb; ++k) {
    out[0] += h[4 * k];
    out[1] = std::max(out[1], h[4 * k + 1]);
    out[2] += h[4 * k + 2];
    out[3] = std::max(out[3], h[4 * k + 3]);
  }
  return EB_OK;
}

extern "C" int eb_calculate_stokes_norms(eb_ctx* c, eb_stokes_norms* o) {
  int rc = need_system(c, false);
  if (rc || (rc = need_fields(c, {EB_G_VX1, EB_G_VY1, EB_G_PR1, EB_G_VX1_OLD, EB_G_VY1_OLD, EB_G_PR1_OLD}))) return rc;
  if (!o) return eb_fail(c, EB_BAD_INPUT, "null norms pointer");
  if (3 * c->st->sys.nc < 4 * 2 * 152) return eb_fail(c, EB_BAD_INPUT, "grid too small for the norm reduction");
  StokesSystem& s = c->st->sys;
  double S4[4], X4[4], Y4[4], P4[4], R4[4];
  if ((rc = diff_norms(c, s.S, s.S_old, 3 * s.nc, S4)) ||
      (rc = diff_norms(c, c->gf[EB_G_VX1], c->gf[EB_G_VX1_OLD], (int64_t)grid_field_count(c, EB_G_VX1), X4)) ||
      (rc = diff_norms(c, c->gf[EB_G_VY1], c->gf[EB_G_VY1_OLD], (int64_t)grid_field_count(c, EB_G_VY1), Y4)) ||
      (rc = diff_norms(c, c->gf[EB_G_PR1], c->gf[EB_G_PR1_OLD], (int64_t)grid_field_count(c, EB_G_PR1), P4)) ||
      (rc = diff_norms(c, s.resnl, nullptr, 3 * s.nc, R4)))
    return rc;
  prof_resolve(c);
  // MathTools.get_L2_norms / get_inf_norms: rel = abs / |v|, or 1e38 when |v| = 0
  auto rel = [](double a, double v) { return v != 0.0 ? a / v : 1e38; };
  o->dsoluv1_abs_inf = S4[1]; o->dsoluv1_rel_inf = rel(S4[1], S4[3]);
  o->dsoluv1_abs_L2 = std::sqrt(S4[0]); o->dsoluv1_rel_L2 = rel(std::sqrt(S4[0]), std::sqrt(S4[2]));
  o->dvx1_abs_L2 = std::sqrt(X4[0]); o->dvx1_rel_L2 = rel(std::sqrt(X4[0]), std::sqrt(X4[2]));
  o->dvy1_abs_L2 = std::sqrt(Y4[0]); o->dvy1_rel_L2 = rel(std::sqrt(Y4[0]), std::sqrt(Y4[2]));
  o->dpr1_abs_L2 = std::sqrt(P4[0]); o->dpr1_rel_L2 = rel(std::sqrt(P4[0]), std::sqrt(P4[2]));
  const double vi = std::max(X4[1], Y4[1]), vmax = std::max(X4[3], Y4[3]);
  o->dvxy_abs_inf = vi; o->dvxy_rel_inf = rel(vi, vmax);
  o->dvxy_abs_L2 = std::sqrt(X4[0] + Y4[0]); o->dvxy_rel_L2 = rel(std::sqrt(X4[0] + Y4[0]), std::sqrt(X4[2] + Y4[2]));
  o->resnl_L2 = std::sqrt(R4[2]);
  return EB_OK;
}

static double* vector_ptr(StokesSystem& s, int which) {
  switch (which) {
    case EB_SV_SOLUTION: return s.S;
    case EB_SV_RHS: return s.rhs;
    case EB_SV_SOLUTION_OLD: return s.S_old;
    case EB_SV_RESNL: return s.resnl;
    default: return nullptr;
  }
}

extern "C" int eb_stokes_vector_upload(eb_ctx* c, int which, const double* host) {
  int rc = need_system(c, false);
  if (rc) return rc;
  StokesSystem& s = c->st->sys;
  double* d = vector_ptr(s, which);
  if (!d || !host) return eb_fail(c, EB_BAD_INPUT, "bad Stokes vector id or null pointer");
  EB_CK(c, cudaMemcpyAsync(c->st->il, host, 3 * s.nc * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  EB_PROF(c, "k_interleave");
  k_deinterleave<<<nblk(s.nc), kB, 0, c->stream>>>(c->st->il, d, s.nc);
  EB_LAUNCHED(c);
  if (which == EB_SV_SOLUTION) s.S_pscale = s.pscale;  // an uploaded S is in the current system's scale
  EB_CK(c, cudaStreamSynchronize(c->stream));
  prof_resolve(c);
  return EB_OK;
}

extern "C" int eb_stokes_vector_download(eb_ctx* c, int which, double* host) {
  int rc = need_system(c, false);
  if (rc) return rc;
  StokesSystem& s = c->st->sys;
  double* d = vector_ptr(s, which);
  if (!d || !host) return eb_fail(c, EB_BAD_INPUT, "bad Stokes vector id or null pointer");
  EB_PROF(c, "k_interleave");
  k_interleave<<<nblk(s.nc), kB, 0, c->stream>>>(d, c->st->il, s.nc);
  EB_LAUNCHED(c);
  EB_CK(c, cudaMemcpyAsync(host, c->st->il, 3 * s.nc * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  prof_resolve(c);
  return EB_OK;
}

extern "C" int eb_stokes_apply(eb_ctx* c, const double* x, double* y) {
  int rc = need_system(c, true);
  if (rc) return rc;
  if (!x || !y) return eb_fail(c, EB_BAD_INPUT, "null vector");
  StokesSystem& s = c->st->sys;
  double* xin = c->st->tmp;
  EB_CK(c, cudaMemcpyAsync(c->st->il, x, 3 * s.nc * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  EB_PROF(c, "k_interleave");
  k_deinterleave<<<nblk(s.nc), kB, 0, c->stream>>>(c->st->il, xin, s.nc);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_apply64");
  k_apply64<<<nblk(s.nc), kB, 0, c->stream>>>(s.coef, xin, c->st->il, s.nx, s.ny, (int32_t)s.nc);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_interleave");
  k_interleave<<<nblk(s.nc), kB, 0, c->stream>>>(c->st->il, xin, s.nc);
  EB_LAUNCHED(c);
  EB_CK(c, cudaMemcpyAsync(y, xin, 3 * s.nc * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  prof_resolve(c);
  return EB_OK;
}

extern "C" int eb_stokes_export_coo(eb_ctx* c, int64_t* Li, int64_t* Lj, double* Lv, int64_t capacity, int64_t* nnz) {
  int rc = need_system(c, true);
  if (rc) return rc;
  return export_stokes_coo(c, &c->st->sys, Li, Lj, Lv, capacity, nnz);
}

extern "C" int eb_stokes_stencil_download(eb_ctx* c, double* host) {
  int rc = need_system(c, true);
  if (rc) return rc;
  if (!host) return eb_fail(c, EB_BAD_INPUT, "null pointer");
  StokesSystem& s = c->st->sys;
  EB_CK(c, cudaMemcpyAsync(host, s.coef, kStencilSlots * s.nc * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}

extern "C" double eb_stokes_pscale(const eb_ctx* c) { return (c && c->st) ? c->st->sys.pscale : 0.0; }
extern "C" int64_t eb_stokes_size(const eb_ctx* c) {
  return (c && c->have_grid) ? 3 * (int64_t)(c->xnum - 1) * (c->ynum - 1) : 0;
}

// ------------------------------------------- services of the learned preconditioner ---
int stokes_nn_ready(eb_ctx* c, int sweeps) {
  int rc = need_system(c, true);
  if (rc) return rc;
  StokesState* st = c->st;
  return prepare(c, st, sweeps, std::max(st->m, 1), false);
}
int stokes_nn_apply(eb_ctx* c, const double* x, double* y) { return apply_scaled(c, c->st, x, y); }
int stokes_nn_precondition(eb_ctx* c, const double* r, double* z) { return precondition(c, c->st, r, z, c->st->Z); }  // FP32 method
int stokes_nn_dot(eb_ctx* c, const double* a, const double* b, double* out) { return mdot(c, c->st, a, 0, 1, b, out); }
