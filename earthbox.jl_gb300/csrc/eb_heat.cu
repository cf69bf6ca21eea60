// eb_heat.cu -- the conductive heat step on the GPU.
//
// Reference: src/heat_solver.
//   RHS terms       HeatRhs.jl:5-80 (RT1 = hr1 + adiabatic + shear heating)
//   assembly        HeatBuildManager.build_system_of_equations (HeatBuildManager.jl:44-86),
//                   InternalNodes.jl:20-198, BoundaryNodes.jl:18-252, BuildStructs.jl:97-125
//   solve           SystemSolver.discretize_and_solve_conductive_heat_equation (SystemSolver.jl:32-66):
//                   MUMPS / UMFPACK, replaced here by multigrid-preconditioned conjugate gradients
//   residuals       HeatResiduals.compute_residuals_temp! (HeatResiduals.jl:12-162)
//   heat loop       HeatLoop.run_conductive_heat_solver_loop! (HeatLoop.jl:10-79)
//
// Built with -fmad=false: the assembly, RHS and residual kernels keep the Julia
// operand order and produce the reference's values bit for bit.
//
// Storage.  The assembled system is a stored 5-point stencil: slot 0 centre, 1 left
// (node - ynum), 2 right (node + ynum), 3 up (node - 1), 4 down (node + 1), node n =
// j*ynum + i (0-based), the reference's itk - 1 and the column-major offset of the
// basic grids.  A boundary row has a 1 in the centre slot and -b[.,2] in the slot of
// the one neighbour its BC names.
//
// Solve.  The BC rows T_b = b1 + b2 T_n are substituted into the internal rows, and
// each internal row is multiplied by its control-volume area dxC*dyC.  The internal
// system is then symmetric positive definite: diagonal m + sum of conductances
// (m = rhocp/dt * area, a boundary conductance counts with factor 1 - b2), off-diagonal
// -c with c = (kt_a + kt_b)/2 * (width across)/(step along).  It is solved by flexible
// conjugate gradients (Polak-Ribiere beta) in FP64, preconditioned by one FP32 V-cycle:
// red-black Gauss-Seidel, vertex coarsening (every other node; the last coarse interval
// takes three fine intervals when the count is odd), linear transfers in coordinates,
// coarse conductances from the fine ones (in series along an edge, summed with the
// prolongation weights across it), lumped mass, and a dense inverse on the coarsest
// level (at most kDenseMax unknowns).  The V-cycle is one CUDA graph.
#include "eb_internal.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

struct HeatLevel {
  int32_t ni = 0, nj = 0;                  // internal nodes: rows, columns
  float *cx = nullptr, *cy = nullptr;      // [ni*(nj-1)], [(ni-1)*nj] couplings
  float *d = nullptr, *rd = nullptr;       // diagonal, 1/diagonal
  float *m = nullptr, *gb = nullptr;       // lumped mass, boundary conductance (coarsening inputs)
  float *x = nullptr, *b = nullptr, *r = nullptr;
  // transfer to the next coarser level (absent on the coarsest)
  int32_t *py0 = nullptr, *px0 = nullptr;  // [ni], [nj] lower coarse parent
  float *wy = nullptr, *wx = nullptr;      // weight of that parent (1 - w for parent + 1)
  int32_t *cyi = nullptr, *cxi = nullptr;  // [ni_c + 1], [nj_c + 1] fine index of each coarse node (+ sentinel)
};

struct HeatState {
  int64_t N = 0;
  int32_t ni = 0, nj = 0;
  std::vector<void*> allocs;
  double* coef = nullptr;  // [5][N]
  double* rhs = nullptr;   // [N]
  double* res = nullptr;   // [N] residual of the reference's system
  bool built = false;
  double dt_built = 0.0;
  // level-0 FP64 operator on internal nodes
  double *cx = nullptr, *cy = nullptr, *d = nullptr, *b = nullptr;
  // flexible CG vectors
  double *x = nullptr, *r = nullptr, *rp = nullptr, *z = nullptr, *p = nullptr, *q = nullptr;
  double *partial = nullptr, *dots = nullptr;
  std::vector<HeatLevel> lv;
  float* Ainv = nullptr;
  int32_t n_dense = 0;
  int sweeps_graph = -1;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int64_t graph_kernels = 0;
};

namespace {

constexpr int kB = 256;
constexpr int kDenseMax = 48;  // Gauss-Jordan tableau 48 x 96 FP64 in shared memory
constexpr int kDotBlocks = 2 * 152;
unsigned nblk(int64_t n) { return (unsigned)((n + kB - 1) / kB); }

enum { H_C = 0, H_L, H_R, H_U, H_D };

// ------------------------------------------------------------ RHS terms ---
__global__ void k_heat_rhs(int32_t xnum, int32_t ynum, const double* __restrict__ hr1, const double* __restrict__ ha1,
                           const double* __restrict__ rho1, const double* __restrict__ vx1,
                           const double* __restrict__ vy1, const double* __restrict__ sxy2,
                           const double* __restrict__ etas1, const double* __restrict__ sxx2,
                           const double* __restrict__ etan1, double gravity_x, double gravity_y, int adiabatic,
                           int shear, double* __restrict__ RT1) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= (int64_t)xnum * ynum) return;
  const int32_t i = (int32_t)(n % ynum), j = (int32_t)(n / ynum);
  double rt = hr1[n];
  if (i > 0 && i < ynum - 1 && j > 0 && j < xnum - 1) {
    if (adiabatic) {
      const int64_t a = (int64_t)j * (ynum + 1) + i;    // vx1[i, j], vx1[i+1, j] (1-based)
      const int64_t v = (int64_t)j * ynum + i;          // vy1[i, j], vy1[i, j+1]
      rt += ha1[n] * rho1[n] * (gravity_x * (vx1[a] + vx1[a + 1]) + gravity_y * (vy1[v] + vy1[v + ynum])) / 2.0;
    }
    if (shear) {
      const double s = sxy2[n];
      rt += s * s / etas1[n];
      const int64_t rp = ynum - 1;
      const int64_t p00 = (int64_t)(j - 1) * rp + (i - 1), p10 = p00 + 1, p01 = p00 + rp, p11 = p01 + 1;
      const double a = sxx2[p00], b = sxx2[p10], c = sxx2[p01], d = sxx2[p11];
      rt += (a * a / etan1[p00] + b * b / etan1[p10] + c * c / etan1[p01] + d * d / etan1[p11]) / 4.0;
    }
  }
  RT1[n] = rt;
}

// ------------------------------------------------------------- assembly ---
struct HeatBC {
  const double *top, *bottom, *left, *right;  // (xnum, 2), (xnum, 2), (ynum, 2), (ynum, 2)
};

__global__ void k_heat_build(int32_t xnum, int32_t ynum, const double* __restrict__ gx, const double* __restrict__ gy,
                             const double* __restrict__ sx, const double* __restrict__ sy,
                             const double* __restrict__ tk, const double* __restrict__ rhocp,
                             const double* __restrict__ kt, const double* __restrict__ RT, HeatBC bc, double dt,
                             double* __restrict__ coef, double* __restrict__ R) {
  const int64_t N = (int64_t)xnum * ynum;
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int32_t i = (int32_t)(n % ynum), j = (int32_t)(n / ynum);
  double c[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  double r;
  if (i == 0 && j > 0 && j < xnum - 1) {
    r = bc.top[j];
    c[H_C] = 1.0;
    c[H_D] = -bc.top[xnum + j];
  } else if (i == ynum - 1 && j > 0 && j < xnum - 1) {
    r = bc.bottom[j];
    c[H_C] = 1.0;
    c[H_U] = -bc.bottom[xnum + j];
  } else if (j == 0) {
    r = bc.left[i];
    c[H_C] = 1.0;
    c[H_R] = -bc.left[ynum + i];
  } else if (j == xnum - 1) {
    r = bc.right[i];
    c[H_C] = 1.0;
    c[H_L] = -bc.right[ynum + i];
  } else {
    const double tkC = tk[n], rhocpC = rhocp[n];
    const double ktU = kt[n - 1], ktC = kt[n], ktD = kt[n + 1], ktL = kt[n - ynum], ktR = kt[n + ynum];
    const double dxL = sx[j - 1], dxR = sx[j], dxC = (gx[j + 1] - gx[j - 1]) / 2.0;
    const double dyU = sy[i - 1], dyD = sy[i], dyC = (gy[i + 1] - gy[i - 1]) / 2.0;
    r = RT[n] + tkC * rhocpC / dt;
    c[H_C] = rhocpC / dt + ((ktL + ktC) / dxL + (ktC + ktR) / dxR) / 2.0 / dxC +
             ((ktU + ktC) / dyU + (ktC + ktD) / dyD) / 2.0 / dyC;
    c[H_L] = -(ktL + ktC) / 2.0 / dxL / dxC;
    c[H_R] = -(ktC + ktR) / 2.0 / dxR / dxC;
    c[H_U] = -(ktU + ktC) / 2.0 / dyU / dyC;
    c[H_D] = -(ktC + ktD) / 2.0 / dyD / dyC;
  }
#pragma unroll
  for (int s = 0; s < 5; ++s) coef[(int64_t)s * N + n] = c[s];
  R[n] = r;
}

// HeatResiduals: rest from RT1, rhocp1, tk0 (old), tk2 (new), kt1.
__global__ void k_heat_residuals(int32_t xnum, int32_t ynum, const double* __restrict__ gx,
                                 const double* __restrict__ gy, const double* __restrict__ sx,
                                 const double* __restrict__ sy, const double* __restrict__ RT,
                                 const double* __restrict__ rhocp, const double* __restrict__ tk,
                                 const double* __restrict__ tn, const double* __restrict__ kt, double dt,
                                 double* __restrict__ rest) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= (int64_t)xnum * ynum) return;
  const int32_t i = (int32_t)(n % ynum), j = (int32_t)(n / ynum);
  if (i == 0 || i == ynum - 1 || j == 0 || j == xnum - 1) {
    rest[n] = 0.0;
    return;
  }
  double r = RT[n] + -rhocp[n] * (tn[n] - tk[n]) / dt;
  const double xc = (gx[j + 1] - gx[j - 1]) / 2.0, yc = (gy[i + 1] - gy[i - 1]) / 2.0;
  r += ((kt[n] + kt[n + ynum]) * (tn[n + ynum] - tn[n]) / sx[j] - (kt[n - ynum] + kt[n]) * (tn[n] - tn[n - ynum]) / sx[j - 1]) /
       2.0 / xc;
  r += ((kt[n] + kt[n + 1]) * (tn[n + 1] - tn[n]) / sy[i] - (kt[n - 1] + kt[n]) * (tn[n] - tn[n - 1]) / sy[i - 1]) / 2.0 /
       yc;
  rest[n] = r;
}

// ----------------------------------------------------------- COO export ---
// Entries before node n in the reference's order (columns j outer, rows i inner):
// boundary rows emit 2 entries, internal rows 5 (centre, left, right, up, down).
__host__ __device__ int64_t heat_coo_offset(int32_t xnum, int32_t ynum, int32_t i, int32_t j) {
  if (j == 0) return 2 * (int64_t)i;
  const int64_t col = 4 + 5 * (int64_t)(ynum - 2);  // entries of one middle column
  int64_t o = 2 * (int64_t)ynum + (int64_t)(j - 1) * col;
  if (j == xnum - 1) return o + 2 * (int64_t)i;
  if (i == 0) return o;
  if (i == ynum - 1) return o + 2 + 5 * (int64_t)(ynum - 2);
  return o + 2 + 5 * (int64_t)(i - 1);
}
__global__ void k_heat_coo(int32_t xnum, int32_t ynum, const double* __restrict__ coef, int64_t* __restrict__ Li,
                           int64_t* __restrict__ Lj, double* __restrict__ Lv) {
  const int64_t N = (int64_t)xnum * ynum;
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int32_t i = (int32_t)(n % ynum), j = (int32_t)(n / ynum);
  int64_t o = heat_coo_offset(xnum, ynum, i, j);
  const int64_t row = n + 1;
  auto put = [&](int s, int64_t col) {
    Li[o] = row;
    Lj[o] = col + 1;
    Lv[o] = coef[(int64_t)s * N + n];
    ++o;
  };
  if (i == 0 && j > 0 && j < xnum - 1) {
    put(H_C, n); put(H_D, n + 1);
  } else if (i == ynum - 1 && j > 0 && j < xnum - 1) {
    put(H_C, n); put(H_U, n - 1);
  } else if (j == 0) {
    put(H_C, n); put(H_R, n + ynum);
  } else if (j == xnum - 1) {
    put(H_C, n); put(H_L, n - ynum);
  } else {
    put(H_C, n); put(H_L, n - ynum); put(H_R, n + ynum); put(H_U, n - 1); put(H_D, n + 1);
  }
}

// --------------------------------------------- folded internal system ---
// Internal node (ii, jj), q = jj*ni + ii, is grid node (ii+1, jj+1) (0-based).
__device__ __forceinline__ double heat_cx(const double* kt, const double* sx, double dyC, int32_t ynum, int32_t i,
                                          int32_t j) {  // edge between grid columns j and j+1 at row i
  const int64_t n = (int64_t)j * ynum + i;
  return (kt[n] + kt[n + ynum]) / 2.0 * dyC / sx[j];
}
__device__ __forceinline__ double heat_cy(const double* kt, const double* sy, double dxC, int32_t ynum, int32_t i,
                                          int32_t j) {  // edge between grid rows i and i+1 at column j
  const int64_t n = (int64_t)j * ynum + i;
  return (kt[n] + kt[n + 1]) / 2.0 * dxC / sy[i];
}
__global__ void k_heat_fold(int32_t xnum, int32_t ynum, const double* __restrict__ gx, const double* __restrict__ gy,
                            const double* __restrict__ sx, const double* __restrict__ sy,
                            const double* __restrict__ rhocp, const double* __restrict__ kt,
                            const double* __restrict__ R, HeatBC bc, double dt, double* __restrict__ cx,
                            double* __restrict__ cy, double* __restrict__ d, double* __restrict__ b,
                            float* __restrict__ cx32, float* __restrict__ cy32, float* __restrict__ d32,
                            float* __restrict__ rd32, float* __restrict__ m32, float* __restrict__ gb32) {
  const int32_t ni = ynum - 2, nj = xnum - 2;
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (int64_t)ni * nj) return;
  const int32_t ii = (int32_t)(q % ni), jj = (int32_t)(q / ni);
  const int32_t i = ii + 1, j = jj + 1;
  const int64_t n = (int64_t)j * ynum + i;
  const double dxC = (gx[j + 1] - gx[j - 1]) / 2.0, dyC = (gy[i + 1] - gy[i - 1]) / 2.0;
  const double area = dxC * dyC;
  const double W = heat_cx(kt, sx, dyC, ynum, i, j - 1), E = heat_cx(kt, sx, dyC, ynum, i, j);
  const double Nn = heat_cy(kt, sy, dxC, ynum, i - 1, j), S = heat_cy(kt, sy, dxC, ynum, i, j);
  const double m = rhocp[n] / dt * area;
  double diag = m, gbnd = 0.0, rhs = area * R[n];
  // each neighbour: an internal coupling, or a boundary row T_b = b1 + b2 T_n folded in
  if (jj == 0) {
    gbnd += W * (1.0 - bc.left[ynum + i]);
    rhs += W * bc.left[i];
  } else {
    diag += W;
  }
  if (jj == nj - 1) {
    gbnd += E * (1.0 - bc.right[ynum + i]);
    rhs += E * bc.right[i];
  } else {
    diag += E;
  }
  if (ii == 0) {
    gbnd += Nn * (1.0 - bc.top[xnum + j]);
    rhs += Nn * bc.top[j];
  } else {
    diag += Nn;
  }
  if (ii == ni - 1) {
    gbnd += S * (1.0 - bc.bottom[xnum + j]);
    rhs += S * bc.bottom[j];
  } else {
    diag += S;
  }
  diag += gbnd;
  d[q] = diag;
  b[q] = rhs;
  d32[q] = (float)diag;
  rd32[q] = (float)(1.0 / diag);
  m32[q] = (float)m;
  gb32[q] = (float)gbnd;
  if (jj < nj - 1) {
    cx[(int64_t)jj * ni + ii] = E;
    cx32[(int64_t)jj * ni + ii] = (float)E;
  }
  if (ii < ni - 1) {
    cy[(int64_t)jj * (ni - 1) + ii] = S;
    cy32[(int64_t)jj * (ni - 1) + ii] = (float)S;
  }
}

// y = A x on the folded FP64 system
__global__ void k_heat_apply(int32_t ni, int32_t nj, const double* __restrict__ cx, const double* __restrict__ cy,
                             const double* __restrict__ d, const double* __restrict__ x, double* __restrict__ y) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (int64_t)ni * nj) return;
  const int32_t ii = (int32_t)(q % ni), jj = (int32_t)(q / ni);
  double s = d[q] * x[q];
  if (jj > 0) s -= cx[(int64_t)(jj - 1) * ni + ii] * x[q - ni];
  if (jj < nj - 1) s -= cx[(int64_t)jj * ni + ii] * x[q + ni];
  if (ii > 0) s -= cy[(int64_t)jj * (ni - 1) + ii - 1] * x[q - 1];
  if (ii < ni - 1) s -= cy[(int64_t)jj * (ni - 1) + ii] * x[q + 1];
  y[q] = s;
}

// ------------------------------------------------------ coarse levels ---
// 1-D weight of fine index f for coarse index k
__device__ __forceinline__ float w1(const int32_t* p0, const float* w, int32_t f, int32_t k) {
  const int32_t a = p0[f];
  return a == k ? w[f] : (a + 1 == k ? 1.f - w[f] : 0.f);
}
// coarse conductance of the edge from coarse column kj to kj+1 at coarse row ki
__device__ float coarse_cx(const HeatLevel& F, int32_t ki, int32_t kj) {
  const int32_t f0 = F.cyi[ki > 0 ? ki - 1 : 0] + (ki > 0 ? 1 : 0);
  const int32_t f1 = F.cyi[ki + 1] - 1 < F.ni - 1 ? F.cyi[ki + 1] - 1 : F.ni - 1;
  const int32_t q0 = F.cxi[kj], q1 = F.cxi[kj + 1];
  float s = 0.f;
  for (int32_t f = f0; f <= f1; ++f) {
    const float w = w1(F.py0, F.wy, f, ki);
    if (w == 0.f) continue;
    float res = 0.f;
    for (int32_t q = q0; q < q1; ++q) res += 1.f / F.cx[(int64_t)q * F.ni + f];
    s += w / res;
  }
  return s;
}
__device__ float coarse_cy(const HeatLevel& F, int32_t ki, int32_t kj) {
  const int32_t f0 = F.cxi[kj > 0 ? kj - 1 : 0] + (kj > 0 ? 1 : 0);
  const int32_t f1 = F.cxi[kj + 1] - 1 < F.nj - 1 ? F.cxi[kj + 1] - 1 : F.nj - 1;
  const int32_t q0 = F.cyi[ki], q1 = F.cyi[ki + 1];
  float s = 0.f;
  for (int32_t f = f0; f <= f1; ++f) {
    const float w = w1(F.px0, F.wx, f, kj);
    if (w == 0.f) continue;
    float res = 0.f;
    for (int32_t q = q0; q < q1; ++q) res += 1.f / F.cy[(int64_t)f * (F.ni - 1) + q];
    s += w / res;
  }
  return s;
}
__global__ void k_heat_coarsen(HeatLevel F, HeatLevel Cc) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (int64_t)Cc.ni * Cc.nj) return;
  const int32_t ki = (int32_t)(k % Cc.ni), kj = (int32_t)(k / Cc.ni);
  // children ranges along each axis
  const int32_t fi0 = ki > 0 ? F.cyi[ki - 1] + 1 : 0, fi1 = ki < Cc.ni - 1 ? F.cyi[ki + 1] - 1 : F.ni - 1;
  const int32_t fj0 = kj > 0 ? F.cxi[kj - 1] + 1 : 0, fj1 = kj < Cc.nj - 1 ? F.cxi[kj + 1] - 1 : F.nj - 1;
  float m = 0.f, gb = 0.f;
  for (int32_t fj = fj0; fj <= fj1; ++fj) {
    const float wj = w1(F.px0, F.wx, fj, kj);
    if (wj == 0.f) continue;
    for (int32_t fi = fi0; fi <= fi1; ++fi) {
      const float w = wj * w1(F.py0, F.wy, fi, ki);
      const int64_t q = (int64_t)fj * F.ni + fi;
      m += w * F.m[q];
      gb += w * F.gb[q];
    }
  }
  float diag = m + gb;
  if (kj < Cc.nj - 1) {
    const float e = coarse_cx(F, ki, kj);
    Cc.cx[(int64_t)kj * Cc.ni + ki] = e;
    diag += e;
  }
  if (kj > 0) diag += coarse_cx(F, ki, kj - 1);
  if (ki < Cc.ni - 1) {
    const float s = coarse_cy(F, ki, kj);
    Cc.cy[(int64_t)kj * (Cc.ni - 1) + ki] = s;
    diag += s;
  }
  if (ki > 0) diag += coarse_cy(F, ki - 1, kj);
  Cc.m[k] = m;
  Cc.gb[k] = gb;
  Cc.d[k] = diag;
  Cc.rd[k] = 1.f / diag;
}

// Dense inverse of the coarsest level (n <= kDenseMax) by Gauss-Jordan in FP64, one block.
__global__ void k_heat_dense_inverse(HeatLevel L, float* __restrict__ Ainv) {
  __shared__ double A[kDenseMax][2 * kDenseMax];
  const int n = L.ni * L.nj;
  for (int e = threadIdx.x; e < n * 2 * n; e += blockDim.x) {
    const int r = e / (2 * n), c = e % (2 * n);
    double v = 0.0;
    if (c >= n) {
      v = (c - n == r) ? 1.0 : 0.0;
    } else {
      const int ri = r % L.ni, rj = r / L.ni;
      if (c == r) v = L.d[r];
      else if (rj < L.nj - 1 && c == r + L.ni) v = -(double)L.cx[(int64_t)rj * L.ni + ri];
      else if (rj > 0 && c == r - L.ni) v = -(double)L.cx[(int64_t)(rj - 1) * L.ni + ri];
      else if (ri < L.ni - 1 && c == r + 1) v = -(double)L.cy[(int64_t)rj * (L.ni - 1) + ri];
      else if (ri > 0 && c == r - 1) v = -(double)L.cy[(int64_t)rj * (L.ni - 1) + ri - 1];
    }
    A[r][c] = v;
  }
  __syncthreads();
  // symmetric positive definite: no pivoting
  for (int k = 0; k < n; ++k) {
    const double piv = A[k][k];
    __syncthreads();
    for (int c = threadIdx.x; c < 2 * n; c += blockDim.x) A[k][c] /= piv;
    __syncthreads();
    for (int e = threadIdx.x; e < n * 2 * n; e += blockDim.x) {
      const int r = e / (2 * n), c = e % (2 * n);
      if (r != k) {
        const double f = A[r][k];
        if (c != k) A[r][c] -= f * A[k][c];
      }
    }
    __syncthreads();
    for (int r = threadIdx.x; r < n; r += blockDim.x)
      if (r != k) A[r][k] = 0.0;
    __syncthreads();
  }
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) Ainv[e] = (float)A[e / n][n + e % n];
}

// ------------------------------------------------------------ V-cycle ---
// One colour of red-black Gauss-Seidel: nodes with (ii + jj) % 2 == color, x from b.
__global__ void k_heat_rbgs(HeatLevel L, int color) {
  const int32_t half = (L.ni + 1) / 2;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)half * L.nj) return;
  const int32_t jj = (int32_t)(t / half);
  const int32_t ii = (int32_t)(t % half) * 2 + ((color + jj) & 1);
  if (ii >= L.ni) return;
  const int64_t q = (int64_t)jj * L.ni + ii;
  float s = L.b[q];
  if (jj > 0) s += L.cx[(int64_t)(jj - 1) * L.ni + ii] * L.x[q - L.ni];
  if (jj < L.nj - 1) s += L.cx[(int64_t)jj * L.ni + ii] * L.x[q + L.ni];
  if (ii > 0) s += L.cy[(int64_t)jj * (L.ni - 1) + ii - 1] * L.x[q - 1];
  if (ii < L.ni - 1) s += L.cy[(int64_t)jj * (L.ni - 1) + ii] * L.x[q + 1];
  L.x[q] = s * L.rd[q];
}
__global__ void k_heat_resid(HeatLevel L) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (int64_t)L.ni * L.nj) return;
  const int32_t ii = (int32_t)(q % L.ni), jj = (int32_t)(q / L.ni);
  float s = L.b[q] - L.d[q] * L.x[q];
  if (jj > 0) s += L.cx[(int64_t)(jj - 1) * L.ni + ii] * L.x[q - L.ni];
  if (jj < L.nj - 1) s += L.cx[(int64_t)jj * L.ni + ii] * L.x[q + L.ni];
  if (ii > 0) s += L.cy[(int64_t)jj * (L.ni - 1) + ii - 1] * L.x[q - 1];
  if (ii < L.ni - 1) s += L.cy[(int64_t)jj * (L.ni - 1) + ii] * L.x[q + 1];
  L.r[q] = s;
}
// coarse b = P^T r (gather over the children), coarse x = 0
__global__ void k_heat_restrict(HeatLevel F, HeatLevel Cc) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (int64_t)Cc.ni * Cc.nj) return;
  const int32_t ki = (int32_t)(k % Cc.ni), kj = (int32_t)(k / Cc.ni);
  const int32_t fi0 = ki > 0 ? F.cyi[ki - 1] + 1 : 0, fi1 = ki < Cc.ni - 1 ? F.cyi[ki + 1] - 1 : F.ni - 1;
  const int32_t fj0 = kj > 0 ? F.cxi[kj - 1] + 1 : 0, fj1 = kj < Cc.nj - 1 ? F.cxi[kj + 1] - 1 : F.nj - 1;
  float s = 0.f;
  for (int32_t fj = fj0; fj <= fj1; ++fj) {
    const float wj = w1(F.px0, F.wx, fj, kj);
    if (wj == 0.f) continue;
    float t = 0.f;
    for (int32_t fi = fi0; fi <= fi1; ++fi) t += w1(F.py0, F.wy, fi, ki) * F.r[(int64_t)fj * F.ni + fi];
    s += wj * t;
  }
  Cc.b[k] = s;
  Cc.x[k] = 0.f;
}
// fine x += P coarse x
__global__ void k_heat_prolong(HeatLevel F, HeatLevel Cc) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (int64_t)F.ni * F.nj) return;
  const int32_t ii = (int32_t)(q % F.ni), jj = (int32_t)(q / F.ni);
  const int32_t a = F.py0[ii], c = F.px0[jj];
  const float wa = F.wy[ii], wc = F.wx[jj];
  const bool a1 = a + 1 < Cc.ni && wa < 1.f, c1 = c + 1 < Cc.nj && wc < 1.f;
  float v = wa * wc * Cc.x[(int64_t)c * Cc.ni + a];
  if (a1) v += (1.f - wa) * wc * Cc.x[(int64_t)c * Cc.ni + a + 1];
  if (c1) v += wa * (1.f - wc) * Cc.x[(int64_t)(c + 1) * Cc.ni + a];
  if (a1 && c1) v += (1.f - wa) * (1.f - wc) * Cc.x[(int64_t)(c + 1) * Cc.ni + a + 1];
  F.x[q] += v;
}
__global__ void k_heat_dense_apply(HeatLevel L, const float* __restrict__ Ainv) {
  const int n = L.ni * L.nj;
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    float s = 0.f;
    for (int c = 0; c < n; ++c) s += Ainv[r * n + c] * L.b[c];
    L.x[r] = s;
  }
}

// ------------------------------------------------- flexible CG helpers ---
__global__ void k_heat_to32(const double* __restrict__ r, float* __restrict__ b, float* __restrict__ x, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  b[k] = (float)r[k];
  x[k] = 0.f;
}
__global__ void k_heat_to64(const float* __restrict__ x, double* __restrict__ z, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) z[k] = (double)x[k];
}
// up to three dot products in one pass: out[t] = a_t . b_t
struct Dots3 {
  const double *a[3], *b[3];
  int k;
};
__global__ void k_heat_dots(Dots3 D, int64_t n, double* __restrict__ partial) {
  double s[3] = {0.0, 0.0, 0.0};
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
#pragma unroll
    for (int t = 0; t < 3; ++t)
      if (t < D.k) s[t] += D.a[t][e] * D.b[t][e];
  __shared__ double sh[3][kB / 32];
#pragma unroll
  for (int t = 0; t < 3; ++t) {
    if (t >= D.k) break;
    double v = s[t];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[t][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if ((int)threadIdx.x < D.k) {
    double v = 0.0;
    for (int w = 0; w < kB / 32; ++w) v += sh[threadIdx.x][w];
    partial[(int64_t)threadIdx.x * gridDim.x + blockIdx.x] = v;
  }
}
__global__ void k_heat_dots_final(const double* __restrict__ partial, int nb, int k, double* __restrict__ out) {
  __shared__ double sh[kB];
  for (int t = 0; t < k; ++t) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += partial[(int64_t)t * nb + b];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = kB / 2; o > 0; o >>= 1) {
      if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[t] = sh[0];
    __syncthreads();
  }
}
__global__ void k_heat_sub(double* __restrict__ r, const double* __restrict__ b, const double* __restrict__ Ax,
                           int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) r[k] = b[k] - Ax[k];
}
__global__ void k_heat_p(double* __restrict__ p, const double* __restrict__ z, double beta, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) p[k] = z[k] + beta * p[k];
}
__global__ void k_heat_xr(double* __restrict__ x, double* __restrict__ r, double* __restrict__ rp,
                          const double* __restrict__ p, const double* __restrict__ q, double alpha, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  x[k] += alpha * p[k];
  const double rk = r[k];
  rp[k] = rk;
  r[k] = rk - alpha * q[k];
}
// internal initial guess from tk0 (or zero)
__global__ void k_heat_guess(int32_t ynum, int32_t ni, int32_t nj, const double* __restrict__ tk0,
                             double* __restrict__ x) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (int64_t)ni * nj) return;
  const int32_t ii = (int32_t)(q % ni), jj = (int32_t)(q / ni);
  x[q] = tk0 ? tk0[(int64_t)(jj + 1) * ynum + ii + 1] : 0.0;
}
// tk2: internal nodes from x, then the BC rows (top and bottom first: the side columns
// read them at the corners)
__global__ void k_heat_unpack(int32_t ynum, int32_t ni, int32_t nj, const double* __restrict__ x,
                              double* __restrict__ tk2) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (int64_t)ni * nj) return;
  const int32_t ii = (int32_t)(q % ni), jj = (int32_t)(q / ni);
  tk2[(int64_t)(jj + 1) * ynum + ii + 1] = x[q];
}
__global__ void k_heat_bc_tb(int32_t xnum, int32_t ynum, HeatBC bc, double* __restrict__ tk2) {
  const int32_t j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j >= xnum - 1) return;
  const int64_t c = (int64_t)j * ynum;
  tk2[c] = bc.top[j] + bc.top[xnum + j] * tk2[c + 1];
  tk2[c + ynum - 1] = bc.bottom[j] + bc.bottom[xnum + j] * tk2[c + ynum - 2];
}
__global__ void k_heat_bc_lr(int32_t xnum, int32_t ynum, HeatBC bc, double* __restrict__ tk2) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ynum) return;
  tk2[i] = bc.left[i] + bc.left[ynum + i] * tk2[ynum + i];
  const int64_t r = (int64_t)(xnum - 1) * ynum + i;
  tk2[r] = bc.right[i] + bc.right[ynum + i] * tk2[r - ynum];
}
// residual of the reference's system: res = R - L tk2
__global__ void k_heat_full_resid(int32_t xnum, int32_t ynum, const double* __restrict__ coef,
                                  const double* __restrict__ R, const double* __restrict__ t,
                                  double* __restrict__ res) {
  const int64_t N = (int64_t)xnum * ynum;
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  double s = coef[n] * t[n];
  const double cl = coef[N + n], cr = coef[2 * N + n], cu = coef[3 * N + n], cd = coef[4 * N + n];
  if (cl != 0.0) s += cl * t[n - ynum];
  if (cr != 0.0) s += cr * t[n + ynum];
  if (cu != 0.0) s += cu * t[n - 1];
  if (cd != 0.0) s += cd * t[n + 1];
  res[n] = R[n] - s;
}
// dtk1 = a - b and block maxima of |dtk1|
__global__ void k_heat_change(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out,
                              int64_t n, double* __restrict__ bmax) {
  double m = 0.0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const double v = a[k] - b[k];
    out[k] = v;
    m = fmax(m, fabs(v));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ double sh[kB / 32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0.0;
    for (int w = 0; w < kB / 32; ++w) v = fmax(v, sh[w]);
    bmax[blockIdx.x] = v;
  }
}
__global__ void k_heat_copy(double* __restrict__ dst, const double* __restrict__ src, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) dst[k] = src[k];
}

// ------------------------------------------------------------ host side ---
template <class T>
int halloc(eb_ctx* c, std::vector<void*>& owner, T** p, size_t n) {
  EB_CK(c, cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T)));
  owner.push_back(*p);
  return EB_OK;
}
template <class T>
int hupload(eb_ctx* c, std::vector<void*>& owner, T** p, const std::vector<T>& h) {
  int rc = halloc(c, owner, p, h.size());
  if (rc) return rc;
  if (!h.empty()) EB_CK(c, cudaMemcpyAsync(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, c->stream));
  return EB_OK;
}

HeatBC heat_bc(eb_ctx* c) {
  return HeatBC{c->gf[EB_G_BTOPT], c->gf[EB_G_BBOTTOMT], c->gf[EB_G_BLEFTT], c->gf[EB_G_BRIGHTT]};
}

int need_fields(eb_ctx* c, std::initializer_list<int> fs) {
  for (int f : fs) {
    int rc = ensure_grid_field(c, f);
    if (rc) return rc;
  }
  return EB_OK;
}

// every other index (ends kept; an odd interval count gives the last coarse interval three fine ones)
std::vector<int32_t> coarse_nodes(int32_t n) {
  std::vector<int32_t> cidx;
  if (n <= 2) {  // too short to coarsen: identity
    for (int32_t f = 0; f < n; ++f) cidx.push_back(f);
    return cidx;
  }
  for (int32_t f = 0; f < n; f += 2) cidx.push_back(f);
  if (cidx.back() != n - 1) cidx.back() = n - 1;
  return cidx;
}

// The state, its FP64 operator and the multigrid hierarchy for the current grid.
HeatState* heat_state(eb_ctx* c) {
  if (c->ht) return c->ht;
  auto* h = new HeatState();
  const int32_t X = c->xnum, Y = c->ynum;
  h->N = (int64_t)X * Y;
  h->ni = Y - 2;
  h->nj = X - 2;
  const int64_t ni = h->ni, nj = h->nj, nq = ni * nj;
  bool ok = halloc(c, h->allocs, &h->coef, 5 * h->N) == EB_OK && halloc(c, h->allocs, &h->rhs, h->N) == EB_OK &&
            halloc(c, h->allocs, &h->res, h->N) == EB_OK;
  if (ok && nq > 0) {
    ok = halloc(c, h->allocs, &h->cx, ni * std::max<int64_t>(nj - 1, 1)) == EB_OK &&
         halloc(c, h->allocs, &h->cy, std::max<int64_t>(ni - 1, 1) * nj) == EB_OK &&
         halloc(c, h->allocs, &h->d, nq) == EB_OK && halloc(c, h->allocs, &h->b, nq) == EB_OK &&
         halloc(c, h->allocs, &h->x, nq) == EB_OK && halloc(c, h->allocs, &h->r, nq) == EB_OK &&
         halloc(c, h->allocs, &h->rp, nq) == EB_OK && halloc(c, h->allocs, &h->z, nq) == EB_OK &&
         halloc(c, h->allocs, &h->p, nq) == EB_OK && halloc(c, h->allocs, &h->q, nq) == EB_OK &&
         halloc(c, h->allocs, &h->partial, 3 * kDotBlocks) == EB_OK && halloc(c, h->allocs, &h->dots, 4) == EB_OK;
    // levels: internal coordinates, coarsened until at most kDenseMax unknowns
    std::vector<double> ys(c->h_gy.begin() + 1, c->h_gy.end() - 1), xs(c->h_gx.begin() + 1, c->h_gx.end() - 1);
    int32_t li = h->ni, lj = h->nj;
    while (ok) {
      HeatLevel L;
      L.ni = li;
      L.nj = lj;
      const int64_t n = (int64_t)li * lj;
      ok = halloc(c, h->allocs, &L.cx, (int64_t)li * std::max(lj - 1, 1)) == EB_OK &&
           halloc(c, h->allocs, &L.cy, (int64_t)std::max(li - 1, 1) * lj) == EB_OK &&
           halloc(c, h->allocs, &L.d, n) == EB_OK && halloc(c, h->allocs, &L.rd, n) == EB_OK &&
           halloc(c, h->allocs, &L.m, n) == EB_OK && halloc(c, h->allocs, &L.gb, n) == EB_OK &&
           halloc(c, h->allocs, &L.x, n) == EB_OK && halloc(c, h->allocs, &L.b, n) == EB_OK &&
           halloc(c, h->allocs, &L.r, n) == EB_OK;
      if (!ok) break;
      if (n <= kDenseMax || (li <= 2 && lj <= 2)) {
        h->lv.push_back(L);
        break;
      }
      // transfer tables to the next level
      auto tables = [](const std::vector<double>& co, const std::vector<int32_t>& cidx, std::vector<int32_t>& p0,
                       std::vector<float>& w) {
        const int32_t nf = (int32_t)co.size();
        p0.assign(nf, 0);
        w.assign(nf, 1.f);
        for (size_t k = 0; k + 1 < cidx.size(); ++k)
          for (int32_t f = cidx[k]; f < cidx[k + 1]; ++f) {
            p0[f] = (int32_t)k;
            w[f] = (float)((co[cidx[k + 1]] - co[f]) / (co[cidx[k + 1]] - co[cidx[k]]));
          }
        p0[nf - 1] = (int32_t)cidx.size() - 1;
        w[nf - 1] = 1.f;
      };
      const std::vector<int32_t> ci = coarse_nodes(li), cj = coarse_nodes(lj);
      std::vector<int32_t> py0, px0;
      std::vector<float> wy, wx;
      tables(ys, ci, py0, wy);
      tables(xs, cj, px0, wx);
      std::vector<int32_t> cyi(ci), cxi(cj);
      cyi.push_back(li);  // sentinel: one past the last fine index
      cxi.push_back(lj);
      ok = hupload(c, h->allocs, &L.py0, py0) == EB_OK && hupload(c, h->allocs, &L.px0, px0) == EB_OK &&
           hupload(c, h->allocs, &L.wy, wy) == EB_OK && hupload(c, h->allocs, &L.wx, wx) == EB_OK &&
           hupload(c, h->allocs, &L.cyi, cyi) == EB_OK && hupload(c, h->allocs, &L.cxi, cxi) == EB_OK;
      h->lv.push_back(L);
      std::vector<double> ys2, xs2;
      for (int32_t f : ci) ys2.push_back(ys[f]);
      for (int32_t f : cj) xs2.push_back(xs[f]);
      ys.swap(ys2);
      xs.swap(xs2);
      li = (int32_t)ci.size();
      lj = (int32_t)cj.size();
    }
    if (ok) {
      h->n_dense = h->lv.back().ni * h->lv.back().nj;
      ok = h->n_dense <= kDenseMax && halloc(c, h->allocs, &h->Ainv, (int64_t)h->n_dense * h->n_dense) == EB_OK;
    }
  }
  if (!ok) {
    for (void* p : h->allocs) cudaFree(p);
    delete h;
    return nullptr;
  }
  c->ht = h;
  return h;
}

int vcycle_launch(eb_ctx* c, HeatState* h, int sweeps, int64_t* nk) {
  const int nl = (int)h->lv.size();
  auto rbgs = [&](HeatLevel& L, int color) -> int {
    const int64_t t = (int64_t)((L.ni + 1) / 2) * L.nj;
    k_heat_rbgs<<<nblk(t), kB, 0, c->stream>>>(L, color);
    ++*nk;
    EB_CK(c, cudaGetLastError());
    return EB_OK;
  };
  int rc;
  for (int l = 0; l < nl - 1; ++l) {
    HeatLevel &F = h->lv[l], &Cc = h->lv[l + 1];
    for (int s = 0; s < sweeps; ++s)
      if ((rc = rbgs(F, 0)) || (rc = rbgs(F, 1))) return rc;
    k_heat_resid<<<nblk((int64_t)F.ni * F.nj), kB, 0, c->stream>>>(F);
    k_heat_restrict<<<nblk((int64_t)Cc.ni * Cc.nj), kB, 0, c->stream>>>(F, Cc);
    *nk += 2;
    EB_CK(c, cudaGetLastError());
  }
  k_heat_dense_apply<<<1, kB, 0, c->stream>>>(h->lv[nl - 1], h->Ainv);
  ++*nk;
  for (int l = nl - 2; l >= 0; --l) {
    HeatLevel &F = h->lv[l], &Cc = h->lv[l + 1];
    k_heat_prolong<<<nblk((int64_t)F.ni * F.nj), kB, 0, c->stream>>>(F, Cc);
    ++*nk;
    EB_CK(c, cudaGetLastError());
    for (int s = 0; s < sweeps; ++s)
      if ((rc = rbgs(F, 1)) || (rc = rbgs(F, 0))) return rc;
  }
  return EB_OK;
}

int capture(eb_ctx* c, HeatState* h, int sweeps) {
  if (h->gexec && h->sweeps_graph == sweeps) return EB_OK;
  if (h->gexec) { cudaGraphExecDestroy(h->gexec); h->gexec = nullptr; }
  if (h->graph) { cudaGraphDestroy(h->graph); h->graph = nullptr; }
  const bool prof = c->prof.on;
  c->prof.on = false;
  int64_t nk = 0;
  EB_CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  int rc = vcycle_launch(c, h, sweeps, &nk);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  c->prof.on = prof;
  if (rc) return rc;
  if (e != cudaSuccess) return eb_cuda(c, e, "cudaStreamEndCapture");
  h->graph = g;
  EB_CK(c, cudaGraphInstantiate(&h->gexec, g, 0));
  h->graph_kernels = nk;
  h->sweeps_graph = sweeps;
  return EB_OK;
}

int dots(eb_ctx* c, HeatState* h, Dots3 D, int64_t n, double* out) {
  EB_PROF(c, "k_heat_dots");
  k_heat_dots<<<kDotBlocks, kB, 0, c->stream>>>(D, n, h->partial);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_heat_dots");
  k_heat_dots_final<<<1, kB, 0, c->stream>>>(h->partial, kDotBlocks, D.k, h->dots);
  EB_LAUNCHED(c);
  EB_CK(c, cudaMemcpyAsync(out, h->dots, D.k * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}
Dots3 dot1(const double* a, const double* b) { return Dots3{{a, nullptr, nullptr}, {b, nullptr, nullptr}, 1}; }

int build_system(eb_ctx* c, HeatState* h, double dt) {
  int rc;
  if ((rc = need_fields(c, {EB_G_TK0, EB_G_RHOCP1, EB_G_KT1, EB_G_RT1, EB_G_BTOPT, EB_G_BBOTTOMT, EB_G_BLEFTT,
                            EB_G_BRIGHTT})))
    return rc;
  EB_PROF(c, "k_heat_build");
  k_heat_build<<<nblk(h->N), kB, 0, c->stream>>>(c->xnum, c->ynum, c->g.gx, c->g.gy, c->g.sx, c->g.sy,
                                                 c->gf[EB_G_TK0], c->gf[EB_G_RHOCP1], c->gf[EB_G_KT1],
                                                 c->gf[EB_G_RT1], heat_bc(c), dt, h->coef, h->rhs);
  EB_LAUNCHED(c);
  h->built = true;
  h->dt_built = dt;
  return EB_OK;
}

int solve_system(eb_ctx* c, HeatState* h, const eb_solve_opts* o, eb_solve_report* rep) {
  const auto t0 = std::chrono::steady_clock::now();
  eb_solve_opts opt = o ? *o : eb_solve_opts{};
  if (!o) opt.use_initial_guess = 1;
  if (opt.rtol <= 0) opt.rtol = 1e-12;
  if (opt.max_iters <= 0) opt.max_iters = 500;
  if (opt.mg_sweeps <= 0) opt.mg_sweeps = 2;
  const int32_t X = c->xnum, Y = c->ynum, ni = h->ni, nj = h->nj;
  const int64_t nq = (int64_t)ni * nj;
  const double dt = h->dt_built;
  int rc, it = 0;
  double rel_s = 0.0;
  if (nq > 0) {
    HeatLevel& L0 = h->lv[0];
    EB_PROF(c, "k_heat_fold");
    k_heat_fold<<<nblk(nq), kB, 0, c->stream>>>(X, Y, c->g.gx, c->g.gy, c->g.sx, c->g.sy, c->gf[EB_G_RHOCP1],
                                                c->gf[EB_G_KT1], h->rhs, heat_bc(c), dt, h->cx, h->cy, h->d, h->b,
                                                L0.cx, L0.cy, L0.d, L0.rd, L0.m, L0.gb);
    EB_LAUNCHED(c);
    for (size_t l = 0; l + 1 < h->lv.size(); ++l) {
      EB_PROF(c, "k_heat_coarsen");
      k_heat_coarsen<<<nblk((int64_t)h->lv[l + 1].ni * h->lv[l + 1].nj), kB, 0, c->stream>>>(h->lv[l], h->lv[l + 1]);
      EB_LAUNCHED(c);
    }
    EB_PROF(c, "k_heat_dense_inverse");
    k_heat_dense_inverse<<<1, kB, 0, c->stream>>>(h->lv.back(), h->Ainv);
    EB_LAUNCHED(c);
    if ((rc = capture(c, h, opt.mg_sweeps))) return rc;
    // x0, r0 = b - A x0
    EB_PROF(c, "k_heat_axpy");
    k_heat_guess<<<nblk(nq), kB, 0, c->stream>>>(Y, ni, nj, opt.use_initial_guess ? c->gf[EB_G_TK0] : nullptr, h->x);
    EB_LAUNCHED(c);
    EB_PROF(c, "k_heat_apply");
    k_heat_apply<<<nblk(nq), kB, 0, c->stream>>>(ni, nj, h->cx, h->cy, h->d, h->x, h->q);
    EB_LAUNCHED(c);
    EB_PROF(c, "k_heat_axpy");
    k_heat_sub<<<nblk(nq), kB, 0, c->stream>>>(h->r, h->b, h->q, nq);
    EB_LAUNCHED(c);
    double nb[2];
    if ((rc = dots(c, h, Dots3{{h->b, h->r, nullptr}, {h->b, h->r, nullptr}, 2}, nq, nb))) return rc;
    const double bnorm = std::sqrt(nb[0]);
    if (!std::isfinite(bnorm) || !std::isfinite(nb[1])) return eb_fail(c, EB_NAN, "heat system has NaN/Inf");
    rel_s = bnorm > 0 ? std::sqrt(nb[1]) / bnorm : 0.0;
    double rho_prev = 0.0;
    while (rel_s > opt.rtol && it < opt.max_iters) {
      // z = M r
      EB_PROF(c, "k_heat_precond");
      k_heat_to32<<<nblk(nq), kB, 0, c->stream>>>(h->r, L0.b, L0.x, nq);
      EB_LAUNCHED(c);
      EB_PROF(c, "heat_vcycle_graph");
      EB_CK(c, cudaGraphLaunch(h->gexec, c->stream));
      c->launches += h->graph_kernels - 1;
      EB_LAUNCHED(c);
      EB_PROF(c, "k_heat_precond");
      k_heat_to64<<<nblk(nq), kB, 0, c->stream>>>(L0.x, h->z, nq);
      EB_LAUNCHED(c);
      double zr[2];
      double beta = 0.0, rho;
      if (it == 0) {
        if ((rc = dots(c, h, dot1(h->z, h->r), nq, zr))) return rc;
        rho = zr[0];
      } else {
        if ((rc = dots(c, h, Dots3{{h->z, h->z, nullptr}, {h->r, h->rp, nullptr}, 2}, nq, zr))) return rc;
        rho = zr[0];
        beta = (zr[0] - zr[1]) / rho_prev;  // Polak-Ribiere: z.(r - r_prev) / (z_prev . r_prev)
      }
      EB_PROF(c, "k_heat_axpy");
      k_heat_p<<<nblk(nq), kB, 0, c->stream>>>(h->p, h->z, beta, nq);
      EB_LAUNCHED(c);
      EB_PROF(c, "k_heat_apply");
      k_heat_apply<<<nblk(nq), kB, 0, c->stream>>>(ni, nj, h->cx, h->cy, h->d, h->p, h->q);
      EB_LAUNCHED(c);
      double pq;
      if ((rc = dots(c, h, dot1(h->p, h->q), nq, &pq))) return rc;
      if (!(pq > 0.0) || !std::isfinite(rho)) return eb_fail(c, EB_NAN, "heat CG breakdown (p.Ap <= 0 or NaN)");
      const double alpha = rho / pq;
      EB_PROF(c, "k_heat_axpy");
      k_heat_xr<<<nblk(nq), kB, 0, c->stream>>>(h->x, h->r, h->rp, h->p, h->q, alpha, nq);
      EB_LAUNCHED(c);
      double rr;
      if ((rc = dots(c, h, dot1(h->r, h->r), nq, &rr))) return rc;
      rho_prev = rho;
      ++it;
      rel_s = bnorm > 0 ? std::sqrt(rr) / bnorm : 0.0;
      if (!std::isfinite(rel_s)) return eb_fail(c, EB_NAN, "heat CG residual became NaN/Inf");
    }
    EB_PROF(c, "k_heat_unpack");
    k_heat_unpack<<<nblk(nq), kB, 0, c->stream>>>(Y, ni, nj, h->x, c->gf[EB_G_TK2]);
    EB_LAUNCHED(c);
  }
  EB_PROF(c, "k_heat_unpack");
  k_heat_bc_tb<<<nblk(X), kB, 0, c->stream>>>(X, Y, heat_bc(c), c->gf[EB_G_TK2]);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_heat_unpack");
  k_heat_bc_lr<<<nblk(Y), kB, 0, c->stream>>>(X, Y, heat_bc(c), c->gf[EB_G_TK2]);
  EB_LAUNCHED(c);
  // residual of the reference's (unscaled) system
  double* res = h->res;
  EB_PROF(c, "k_heat_resid_full");
  k_heat_full_resid<<<nblk(h->N), kB, 0, c->stream>>>(X, Y, h->coef, h->rhs, c->gf[EB_G_TK2], res);
  EB_LAUNCHED(c);
  double rn[2];
  if ((rc = dots(c, h, Dots3{{res, h->rhs, nullptr}, {res, h->rhs, nullptr}, 2}, h->N, rn))) return rc;
  prof_resolve(c);
  const double rel = rn[1] > 0 ? std::sqrt(rn[0] / rn[1]) : std::sqrt(rn[0]);
  if (rep) {
    rep->iterations = it;
    rep->levels = (int32_t)h->lv.size();
    rep->rel_residual = rel;
    rep->rel_residual_scaled = rel_s;
    rep->reorthogonalisations = 0;
    rep->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  if (!std::isfinite(rel)) return eb_fail(c, EB_NAN, "heat solution has NaN/Inf");
  if (rel_s > opt.rtol * 1.0000001)
    return eb_fail(c, EB_NOT_CONVERGED, "heat CG stopped at scaled relative residual " + std::to_string(rel_s) +
                                            " after " + std::to_string(it) + " iterations");
  return EB_OK;
}

int residuals(eb_ctx* c, double dt) {
  int rc;
  if ((rc = need_fields(c, {EB_G_RT1, EB_G_RHOCP1, EB_G_TK0, EB_G_TK2, EB_G_KT1, EB_G_REST}))) return rc;
  EB_PROF(c, "k_heat_residuals");
  k_heat_residuals<<<nblk((int64_t)c->xnum * c->ynum), kB, 0, c->stream>>>(
      c->xnum, c->ynum, c->g.gx, c->g.gy, c->g.sx, c->g.sy, c->gf[EB_G_RT1], c->gf[EB_G_RHOCP1], c->gf[EB_G_TK0],
      c->gf[EB_G_TK2], c->gf[EB_G_KT1], dt, c->gf[EB_G_REST]);
  EB_LAUNCHED(c);
  return EB_OK;
}

// dst = a - b over the basic grid; returns max |dst| on the host
int change(eb_ctx* c, HeatState* h, double* dst, const double* a, const double* b, double* maxabs) {
  const int64_t n = (int64_t)c->xnum * c->ynum;
  EB_PROF(c, "k_heat_change");
  k_heat_change<<<kDotBlocks, kB, 0, c->stream>>>(a, b, dst, n, h->partial);
  EB_LAUNCHED(c);
  std::vector<double> m(kDotBlocks);
  EB_CK(c, cudaMemcpyAsync(m.data(), h->partial, kDotBlocks * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  double v = 0.0;
  for (double t : m) v = std::max(v, t);
  if (maxabs) *maxabs = v;
  return EB_OK;
}

int need_heat(eb_ctx* c, HeatState** h) {
  if (!c) return EB_BAD_INPUT;
  if (!c->have_grid) return eb_fail(c, EB_NOT_READY, "eb_set_grid has not been called");
  if (c->xnum < 3 || c->ynum < 3) return eb_fail(c, EB_BAD_INPUT, "the heat step needs xnum, ynum >= 3");
  cudaSetDevice(c->device);
  *h = heat_state(c);
  if (!*h) return eb_fail(c, EB_CUDA_ERROR, "out of device memory for the heat system");
  return EB_OK;
}

}  // namespace

void heat_free(eb_ctx* c) {
  if (!c->ht) return;
  HeatState* h = c->ht;
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  if (h->graph) cudaGraphDestroy(h->graph);
  for (void* p : h->allocs) cudaFree(p);
  delete h;
  c->ht = nullptr;
}

// ------------------------------------------------------------ C-ABI ---
extern "C" int eb_calculate_heat_rhs_terms(eb_ctx* c, const eb_heat_params* hp) {
  HeatState* h;
  int rc = need_heat(c, &h);
  if (rc) return rc;
  if (!hp) return eb_fail(c, EB_BAD_INPUT, "eb_heat_params is null");
  if ((rc = need_fields(c, {EB_G_HR1, EB_G_HA1, EB_G_RHO1, EB_G_VX1, EB_G_VY1, EB_G_SXY2, EB_G_ETAS1, EB_G_SXX2,
                            EB_G_ETAN1, EB_G_RT1})))
    return rc;
  EB_PROF(c, "k_heat_rhs");
  k_heat_rhs<<<nblk(h->N), kB, 0, c->stream>>>(c->xnum, c->ynum, c->gf[EB_G_HR1], c->gf[EB_G_HA1], c->gf[EB_G_RHO1],
                                               c->gf[EB_G_VX1], c->gf[EB_G_VY1], c->gf[EB_G_SXY2], c->gf[EB_G_ETAS1],
                                               c->gf[EB_G_SXX2], c->gf[EB_G_ETAN1], hp->gravity_x, hp->gravity_y,
                                               hp->iuse_adiabatic_heating == 1, hp->iuse_shear_heating == 1,
                                               c->gf[EB_G_RT1]);
  EB_LAUNCHED(c);
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}

extern "C" int eb_initialize_old_temperature(eb_ctx* c) {
  HeatState* h;
  int rc = need_heat(c, &h);
  if (rc || (rc = need_fields(c, {EB_G_TK1, EB_G_TK0}))) return rc;
  EB_PROF(c, "k_heat_copy");
  k_heat_copy<<<nblk(h->N), kB, 0, c->stream>>>(c->gf[EB_G_TK0], c->gf[EB_G_TK1], h->N);
  EB_LAUNCHED(c);
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}

extern "C" int eb_build_heat_system(eb_ctx* c, double timestep_heat) {
  HeatState* h;
  int rc = need_heat(c, &h);
  if (rc) return rc;
  if (!(timestep_heat > 0.0)) return eb_fail(c, EB_BAD_INPUT, "timestep_heat must be positive");
  if ((rc = build_system(c, h, timestep_heat))) return rc;
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}

extern "C" int eb_solve_heat_system(eb_ctx* c, const eb_solve_opts* o, eb_solve_report* rep) {
  HeatState* h;
  int rc = need_heat(c, &h);
  if (rc) return rc;
  if (!h->built) return eb_fail(c, EB_NOT_READY, "eb_build_heat_system has not been called");
  if ((rc = need_fields(c, {EB_G_TK0, EB_G_TK2}))) return rc;
  return solve_system(c, h, o, rep);
}

extern "C" int eb_heat_residuals(eb_ctx* c, double timestep_heat) {
  HeatState* h;
  int rc = need_heat(c, &h);
  if (rc || (rc = residuals(c, timestep_heat))) return rc;
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}

extern "C" int eb_run_conductive_heat_solver_loop(eb_ctx* c, const eb_heat_params* hp, const eb_solve_opts* o,
                                                  eb_heat_loop_report* rep) {
  const auto t0 = std::chrono::steady_clock::now();
  HeatState* h;
  int rc = need_heat(c, &h);
  if (rc) return rc;
  if (!hp) return eb_fail(c, EB_BAD_INPUT, "eb_heat_params is null");
  if (!(hp->timestep > 0.0)) return eb_fail(c, EB_BAD_INPUT, "timestep must be positive");
  if ((rc = need_fields(c, {EB_G_TK0, EB_G_TK2, EB_G_DTK1}))) return rc;
  const double limit = hp->max_temp_change, start = hp->timestep;
  double loop = start, sum = 0.0, maxres = 0.0;
  int32_t substeps = 0, solves = 0, iters = 0;
  const int64_t n = h->N;
  auto solve = [&](double dt) -> int {
    eb_solve_report r{};
    int e;
    if ((e = build_system(c, h, dt)) || (e = solve_system(c, h, o, &r)) || (e = residuals(c, dt))) return e;
    ++solves;
    iters += r.iterations;
    maxres = std::max(maxres, r.rel_residual);
    return EB_OK;
  };
  while (sum < start) {
    if (substeps >= 100000) return eb_fail(c, EB_NOT_CONVERGED, "heat loop exceeded 100000 passes");
    if ((rc = solve(loop))) return rc;
    double dtkmax;
    if ((rc = change(c, h, c->gf[EB_G_DTK1], c->gf[EB_G_TK2], c->gf[EB_G_TK0], &dtkmax))) return rc;
    if (dtkmax > limit) {
      loop = loop * limit / dtkmax;
      if ((rc = solve(loop))) return rc;
    }
    sum = sum + loop;
    loop = std::min(loop, start - sum);
    EB_PROF(c, "k_heat_copy");
    k_heat_copy<<<nblk(n), kB, 0, c->stream>>>(c->gf[EB_G_TK0], c->gf[EB_G_TK2], n);
    EB_LAUNCHED(c);
    ++substeps;
  }
  EB_CK(c, cudaStreamSynchronize(c->stream));
  prof_resolve(c);
  if (rep) {
    rep->substeps = substeps;
    rep->solves = solves;
    rep->iterations = iters;
    rep->levels = (int32_t)h->lv.size();
    rep->timestep_sum = sum;
    rep->timestep_heat = loop;
    rep->max_rel_residual = maxres;
    rep->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  return EB_OK;
}

extern "C" int eb_calculate_grid_temp_change(eb_ctx* c) {
  HeatState* h;
  int rc = need_heat(c, &h);
  if (rc || (rc = need_fields(c, {EB_G_TK1, EB_G_TK2, EB_G_DTK1}))) return rc;
  return change(c, h, c->gf[EB_G_DTK1], c->gf[EB_G_TK2], c->gf[EB_G_TK1], nullptr);
}

extern "C" int eb_heat_export_coo(eb_ctx* c, int64_t* Li, int64_t* Lj, double* Lv, int64_t capacity, int64_t* nnz) {
  HeatState* h;
  int rc = need_heat(c, &h);
  if (rc) return rc;
  if (!h->built) return eb_fail(c, EB_NOT_READY, "eb_build_heat_system has not been called");
  const int64_t total = heat_coo_offset(c->xnum, c->ynum, c->ynum - 1, c->xnum - 1) + 2;
  if (nnz) *nnz = total;
  if (!Li || !Lj || !Lv) return EB_OK;
  if (capacity < total)
    return eb_fail(c, EB_BAD_INPUT, "COO arrays hold " + std::to_string(capacity) + " entries, the system has " +
                                        std::to_string(total));
  int64_t *d_li = nullptr, *d_lj = nullptr;
  double* d_lv = nullptr;
  cudaError_t e = cudaMalloc(&d_li, total * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMalloc(&d_lj, total * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMalloc(&d_lv, total * sizeof(double));
  if (e == cudaSuccess) {
    k_heat_coo<<<nblk(h->N), kB, 0, c->stream>>>(c->xnum, c->ynum, h->coef, d_li, d_lj, d_lv);
    c->launches++;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(Li, d_li, total * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(Lj, d_lj, total * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(Lv, d_lv, total * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d_li);
  cudaFree(d_lj);
  cudaFree(d_lv);
  if (e != cudaSuccess) return eb_cuda(c, e, "heat COO export");
  return EB_OK;
}

extern "C" int eb_heat_rhs_download(eb_ctx* c, double* host) {
  HeatState* h;
  int rc = need_heat(c, &h);
  if (rc) return rc;
  if (!host) return eb_fail(c, EB_BAD_INPUT, "host pointer is null");
  if (!h->built) return eb_fail(c, EB_NOT_READY, "eb_build_heat_system has not been called");
  EB_CK(c, cudaMemcpyAsync(host, h->rhs, h->N * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}

extern "C" int64_t eb_heat_size(const eb_ctx* c) {
  if (!c || !c->have_grid) return 0;
  return (int64_t)c->xnum * c->ynum;
}
