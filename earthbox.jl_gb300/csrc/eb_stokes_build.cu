// eb_stokes_build.cu -- Stokes-continuity system assembly on the GPU, FP64.
//
// Reference (paths under src/stokes_continuity_solver/):
//   solver/rhs/StokesViscoelasticTerms.jl:26-125   viscoelastic viscosity/stress terms
//   solver/rhs/StokesContinuityRhs.jl:30-190       RX1, RY1, RC1
//   solver/system_solver/SystemSolver.jl:99-115    initialize_solver!, pscale
//   solver/build_system/StokesBuildManager.jl:661-712 and the stencil modules
//     discretize_{x,y}_stokes_equation/, discretize_continuity_equation/
//   solver/system_solver/SystemSolver.jl:188-271   reload_solu_vel!, apply_vel_bc!
//
// The reference assembles a COO list (Li, Lj, Lv) row by row; here one thread
// per basic cell writes that cell's three rows into a stored 27-slot stencil.
// Every coefficient is computed with the reference's operand order and the
// boundary folds are added in the reference's order, and this file is built
// with -fmad=false, so each slot holds exactly the reference's Lv value (the
// sum of the reference's duplicate entries where a fold hits an existing one).
#include "eb_internal.h"

namespace {

// 1-based column-major access, as in Julia
#define A2(a, rows, i, j) (a)[((int64_t)(j) - 1) * (int64_t)(rows) + ((int64_t)(i) - 1)]

constexpr int kB = 256;

// ---- StokesViscoelasticTerms.jl:51-125 --------------------------------------
// Viscoelastic.calculate_viscoelastic_factor (utils/Viscoelastic.jl:26-38): eta / (eta + dt mu)
__global__ void k_ve_terms(const double* __restrict__ eta1, const double* __restrict__ mu1,
                           const double* __restrict__ s1, double* __restrict__ eta0, double* __restrict__ s0,
                           int64_t n, double dt) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double e = eta1[k];
  const double f = e / (e + dt * mu1[k]);
  eta0[k] = e * (1.0 - f);
  s0[k] = s1[k] * f;
}

// ---- StokesContinuityRhs.jl:63-157 ------------------------------------------
// One thread per basic node (i, j), i in 2..ynum, j in 2..xnum; RY1 then RX1 rules.
__global__ void k_rhs_xy(int32_t xnum, int32_t ynum, double gx, double gy, int32_t stab,
                         const double* __restrict__ xstp_b, const double* __restrict__ ystp_b,
                         const double* __restrict__ xstp_vy, const double* __restrict__ ystp_vx,
                         const double* __restrict__ rho1, const double* __restrict__ rho1_vy,
                         const double* __restrict__ sxx0, const double* __restrict__ sxy0,
                         double* __restrict__ RX1, double* __restrict__ RY1) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (int64_t)(xnum - 1) * (ynum - 1)) return;
  const int32_t i = (int32_t)(k % (ynum - 1)) + 2, j = (int32_t)(k / (ynum - 1)) + 2;
  const int32_t yp = ynum - 1;
  if (i != ynum) {  // Domain.basic_node_along_lower_boundary
    double r;
    if (stab == 1) r = -gy * A2(rho1_vy, ynum, i, j);
    else r = -gy * (A2(rho1, ynum, i, j) + A2(rho1, ynum, i, j - 1)) / 2;
    r += (A2(sxx0, yp, i, j - 1) - A2(sxx0, yp, i - 1, j - 1)) / ystp_vx[i - 1];
    r -= (A2(sxy0, ynum, i, j) - A2(sxy0, ynum, i, j - 1)) / xstp_b[j - 2];
    A2(RY1, ynum, i, j) = r;
  }
  if (j != xnum) {  // Domain.basic_node_on_right_boundary
    double r = -gx * (A2(rho1, ynum, i, j) + A2(rho1, ynum, i - 1, j)) / 2;
    r -= (A2(sxx0, yp, i - 1, j) - A2(sxx0, yp, i - 1, j - 1)) / xstp_vy[j - 1];
    r -= (A2(sxy0, ynum, i, j) - A2(sxy0, ynum, i - 1, j)) / ystp_b[i - 2];
    A2(RX1, ynum + 1, i, j) = r;
  }
}

// calc_plastic_volumetric_effect (StokesContinuityRhs.jl:159-190): 2 sin(dil pi/180) eii_plastic
__global__ void k_rhs_c(const double* __restrict__ dil, const double* __restrict__ eii, double* __restrict__ RC1,
                        int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double rad = dil[k] * 3.14159265358979323846 / 180.0;
  RC1[k] = 2.0 * sin(rad) * eii[k];
}

// ---- StokesBuildManager.jl:661-712 ------------------------------------------
struct BuildIn {
  int32_t xnum, ynum;
  double xstpavg, ystpavg, pscale, timestep, gravity_y, pressure_bc;
  int32_t stab, pressure_bc_mode;
  int64_t zone[8];
  double zvel[8];
  const double *xstp, *ystp, *xstpc, *ystpc;
  const double *btopx, *bbottomx, *btopy, *bbottomy, *bleftx, *brightx, *blefty, *brighty;
  const double *etan, *etas, *rho_vy, *RX, *RY, *RC;
};

// slot numbers inside each row
enum { X_C = 0, X_L, X_R, X_U, X_D, X_YUL, X_YUR, X_YLL, X_YLR, X_PL, X_PR };
enum { Y_C = 0, Y_U, Y_D, Y_L, Y_R, Y_XUL, Y_XUR, Y_XLL, Y_XLR, Y_PU, Y_PD };
enum { C_C = 0, C_XL, C_XR, C_YU, C_YD };

__global__ void k_build_system(BuildIn b, double* __restrict__ coef, double* __restrict__ rhs, int64_t nc) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const int32_t ny = b.ynum - 1;
  const int32_t i = (int32_t)(c % ny) + 1, j = (int32_t)(c / ny) + 1;  // 1-based cell (i, j)
  const double *xstp = b.xstp, *ystp = b.ystp, *xstpc = b.xstpc, *ystpc = b.ystpc;
#define ETAN(ii, jj) A2(b.etan, b.ynum - 1, ii, jj)
#define ETAS(ii, jj) A2(b.etas, b.ynum, ii, jj)
#define RHOVY(ii, jj) A2(b.rho_vy, b.ynum, ii, jj)
#define BX(a, k, col) A2(b.a, b.xnum, k, col)
#define BX1(a, k, col) A2(b.a, b.xnum + 1, k, col)
#define BY1(a, k, col) A2(b.a, b.ynum + 1, k, col)
#define BY(a, k, col) A2(b.a, b.ynum, k, col)
  double x[11] = {0}, y[11] = {0}, p[5] = {0};
  double Rx, Ry, Rc;
  const double kbond = 2.0 * b.pscale / (b.xstpavg + b.ystpavg);
  const bool top = (i == 1), left = (j == 1);
  // ---- x-Stokes (StencilForVxStokesUnknown.jl) ----
  const bool out_x = j != b.zone[0] || i < b.zone[1] || i > b.zone[2];
  if (!(j < b.xnum - 1 && out_x)) {  // boundary/BoundaryCells.jl:64-95
    x[X_C] = kbond;
    Rx = out_x ? 0.0 : 2.0 * b.pscale / (b.xstpavg + b.ystpavg) * b.zvel[3];
  } else {
    const bool bot = i >= b.ynum - 1, right2 = j >= b.xnum - 2;
    // CentralVelocityXNode.jl:6-45
    x[X_C] = -2.0 * (ETAN(i, j + 1) / xstp[j] + ETAN(i, j) / xstp[j - 1]) / xstpc[j] -
             (ETAS(i + 1, j + 1) / ystpc[i] + ETAS(i, j + 1) / ystpc[i - 1]) / ystp[i - 1];
    Rx = A2(b.RX, b.ynum + 1, i + 1, j + 1);
    // LeftVelocityXNode.jl:7-79
    if (!left) {
      x[X_L] = 2.0 * ETAN(i, j) / xstp[j - 1] / xstpc[j];
    } else {
      x[X_C] = x[X_C] + BY1(bleftx, i + 1, 2) * 2.0 * ETAN(i, j) / xstp[j - 1] / xstpc[j];
      Rx = Rx - BY1(bleftx, i + 1, 1) * 2.0 * ETAN(i, j) / xstp[j - 1] / xstpc[j];
    }
    // RightVelocityXNode.jl:7-59
    if (!right2) {
      x[X_R] = 2.0 * ETAN(i, j + 1) / xstp[j] / xstpc[j];
    } else {
      x[X_C] = x[X_C] + BY1(brightx, i + 1, 2) * 2.0 * ETAN(i, j + 1) / xstp[j] / xstpc[j];
      Rx = Rx - BY1(brightx, i + 1, 1) * 2.0 * ETAN(i, j + 1) / xstp[j] / xstpc[j];
    }
    // UpperVelocityXNode.jl:7-52
    if (!top) {
      x[X_U] = ETAS(i, j + 1) / ystpc[i - 1] / ystp[i - 1];
    } else {
      x[X_C] = x[X_C] + BX(btopx, j + 1, 2) * ETAS(i, j + 1) / ystpc[i - 1] / ystp[i - 1];
      Rx = Rx - BX(btopx, j + 1, 1) * ETAS(i, j + 1) / ystpc[i - 1] / ystp[i - 1];
    }
    // BottomVelocityXNode.jl:7-52
    if (!bot) {
      x[X_D] = ETAS(i + 1, j + 1) / ystpc[i] / ystp[i - 1];
    } else {
      x[X_C] = x[X_C] + BX(bbottomx, j + 1, 2) * ETAS(i + 1, j + 1) / ystpc[i] / ystp[i - 1];
      Rx = Rx - BX(bbottomx, j + 1, 1) * ETAS(i + 1, j + 1) / ystpc[i] / ystp[i - 1];
    }
    // UpperLeftVelocityYNode.jl:7-64, UpperRightVelocityYNode.jl:7-63
    if (!top) {
      x[X_YUL] = ETAS(i, j + 1) / xstpc[j] / ystp[i - 1];
      x[X_YUR] = -ETAS(i, j + 1) / xstpc[j] / ystp[i - 1];
    } else {
      x[X_YLL] = BX1(btopy, j + 1, 2) * ETAS(i, j + 1) / xstpc[j] / ystp[i - 1];
      Rx = Rx - BX1(btopy, j + 1, 1) * ETAS(i, j + 1) / xstpc[j] / ystp[i - 1];
      x[X_YLR] = -BX1(btopy, j + 2, 2) * ETAS(i, j + 1) / xstpc[j] / ystp[i - 1];
      Rx = Rx + BX1(btopy, j + 2, 1) * ETAS(i, j + 1) / xstpc[j] / ystp[i - 1];
    }
    // BottomLeftVelocityYNode.jl:8-72
    if (!bot) {
      if (!top) x[X_YLL] = -ETAS(i + 1, j + 1) / xstpc[j] / ystp[i - 1];
      else x[X_YLL] = x[X_YLL] - ETAS(i + 1, j + 1) / xstpc[j] / ystp[i - 1];
    } else {
      x[X_YUL] = x[X_YUL] - BX1(bbottomy, j + 1, 2) * ETAS(i + 1, j + 1) / xstpc[j] / ystp[i - 1];
      Rx = Rx + BX1(bbottomy, j + 1, 1) * ETAS(i + 1, j + 1) / xstpc[j] / ystp[i - 1];
    }
    // BottomRightVelocityYNode.jl:8-67
    if (!bot) {
      if (!top) x[X_YLR] = ETAS(i + 1, j + 1) / xstpc[j] / ystp[i - 1];
      else x[X_YLR] = x[X_YLR] + ETAS(i + 1, j + 1) / xstpc[j] / ystp[i - 1];
    } else {
      x[X_YUR] = x[X_YUR] + BX1(bbottomy, j + 2, 2) * ETAS(i + 1, j + 1) / xstpc[j] / ystp[i - 1];
      Rx = Rx - BX1(bbottomy, j + 2, 1) * ETAS(i + 1, j + 1) / xstpc[j] / ystp[i - 1];
    }
    // LeftAndRightPressureNodes.jl:6-54
    x[X_PL] = b.pscale / xstpc[j];
    x[X_PR] = -b.pscale / xstpc[j];
  }
  // ---- y-Stokes (StencilForVyStokesUnknown.jl) ----
  const bool out_y = j != b.zone[4] || i < b.zone[5] || i > b.zone[6];
  if (!(i < b.ynum - 1 && out_y)) {  // boundary/BoundaryCells.jl:68-99
    y[Y_C] = kbond;
    Ry = out_y ? 0.0 : 2.0 * b.pscale / (b.xstpavg + b.ystpavg) * b.zvel[7];
  } else {
    const bool bot2 = i >= b.ynum - 2, right = j >= b.xnum - 1;
    // InternalCells.calculate_stabilization_terms (:104-175)
    double dy = 0.0, dx = 0.0;
    if (b.stab == 1) {
      const double drhody = ((RHOVY(i + 2, j + 1) - RHOVY(i + 1, j + 1)) / ystp[i] +
                             (RHOVY(i + 1, j + 1) - RHOVY(i, j + 1)) / ystp[i - 1]) / 2.0;
      dy = drhody * b.gravity_y * b.timestep;
      const double drhodx = ((RHOVY(i + 1, j + 2) - RHOVY(i + 1, j + 1)) / xstpc[j] +
                             (RHOVY(i + 1, j + 1) - RHOVY(i + 1, j)) / xstpc[j - 1]) / 2.0;
      dx = drhodx * b.gravity_y * b.timestep;
    }
    // CentralVelocityYNode.jl:6-44
    y[Y_C] = -2 * (ETAN(i + 1, j) / ystp[i] + ETAN(i, j) / ystp[i - 1]) / ystpc[i] -
             (ETAS(i + 1, j + 1) / xstpc[j] + ETAS(i + 1, j) / xstpc[j - 1]) / xstp[j - 1] - dy;
    Ry = A2(b.RY, b.ynum, i + 1, j + 1);
    // UpperVelocityYNode.jl:7-51
    if (!top) {
      y[Y_U] = 2.0 * ETAN(i, j) / ystp[i - 1] / ystpc[i];
    } else {
      y[Y_C] = y[Y_C] + BX1(btopy, j + 1, 2) * 2.0 * ETAN(i, j) / ystp[i - 1] / ystpc[i];
      Ry = Ry - BX1(btopy, j + 1, 1) * 2.0 * ETAN(i, j) / ystp[i - 1] / ystpc[i];
    }
    // BottomVelocityYNode.jl:7-51
    if (!bot2) {
      y[Y_D] = 2.0 * ETAN(i + 1, j) / ystp[i] / ystpc[i];
    } else {
      y[Y_C] = y[Y_C] + BX1(bbottomy, j + 1, 2) * 2.0 * ETAN(i + 1, j) / ystp[i] / ystpc[i];
      Ry = Ry - BX1(bbottomy, j + 1, 1) * 2.0 * ETAN(i + 1, j) / ystp[i] / ystpc[i];
    }
    // LeftVelocityYNode.jl:7-46
    if (!left) {
      y[Y_L] = ETAS(i + 1, j) / xstpc[j - 1] / xstp[j - 1];
    } else {
      y[Y_C] = y[Y_C] + BY(blefty, i + 1, 2) * ETAS(i + 1, j) / xstpc[j - 1] / xstp[j - 1];
      Ry = Ry - BY(blefty, i + 1, 1) * ETAS(i + 1, j) / xstpc[j - 1] / xstp[j - 1];
    }
    // RightVelocityYNode.jl:7-47
    if (!right) {
      y[Y_R] = ETAS(i + 1, j + 1) / xstpc[j] / xstp[j - 1];
    } else {
      y[Y_C] += BY(brighty, i + 1, 2) * ETAS(i + 1, j + 1) / xstpc[j] / xstp[j - 1];
      Ry -= BY(brighty, i + 1, 1) * ETAS(i + 1, j + 1) / xstpc[j] / xstp[j - 1];
    }
    // UpperLeftVelocityXNode.jl:7-78
    if (!left) {
      y[Y_XUL] = ETAS(i + 1, j) / ystpc[i] / xstp[j - 1] - dx / 4.0;
    } else {
      y[Y_XUR] = BY1(bleftx, i + 1, 2) * (ETAS(i + 1, j) / ystpc[i] / xstp[j - 1] - dx / 4.0);
      Ry = Ry - BY1(bleftx, i + 1, 1) * (ETAS(i + 1, j) / ystpc[i] / xstp[j - 1] - dx / 4.0);
    }
    // BottomLeftVelocityXNode.jl:7-77
    if (!left) {
      y[Y_XLL] = -ETAS(i + 1, j) / ystpc[i] / xstp[j - 1] - dx / 4.0;
    } else {
      y[Y_XLR] = BY1(bleftx, i + 2, 2) * (-ETAS(i + 1, j) / ystpc[i] / xstp[j - 1] - dx / 4.0);
      Ry = Ry - BY1(bleftx, i + 2, 1) * (-ETAS(i + 1, j) / ystpc[i] / xstp[j - 1] - dx / 4.0);
    }
    // UpperRightVelocityXNode.jl:8-80
    if (!right) {
      if (!left) y[Y_XUR] = -ETAS(i + 1, j + 1) / ystpc[i] / xstp[j - 1] - dx / 4.0;
      else y[Y_XUR] = y[Y_XUR] - ETAS(i + 1, j + 1) / ystpc[i] / xstp[j - 1] - dx / 4.0;
    } else {
      y[Y_XUL] = y[Y_XUL] + BY1(brightx, i + 1, 2) * (-ETAS(i + 1, j + 1) / ystpc[i] / xstp[j - 1] - dx / 4.0);
      Ry = Ry - BY1(brightx, i + 1, 1) * (-ETAS(i + 1, j + 1) / ystpc[i] / xstp[j - 1] - dx / 4.0);
    }
    // BottomRightVelocityXNode.jl:8-80
    if (!right) {
      if (!left) y[Y_XLR] = ETAS(i + 1, j + 1) / ystpc[i] / xstp[j - 1] - dx / 4.0;
      else y[Y_XLR] = y[Y_XLR] + ETAS(i + 1, j + 1) / ystpc[i] / xstp[j - 1] - dx / 4.0;
    } else {
      y[Y_XLL] = y[Y_XLL] + BY1(brightx, i + 2, 2) * (ETAS(i + 1, j + 1) / ystpc[i] / xstp[j - 1] - dx / 4.0);
      Ry = Ry - BY1(brightx, i + 2, 1) * (ETAS(i + 1, j + 1) / ystpc[i] / xstp[j - 1] - dx / 4.0);
    }
    // UpperAndLowerPressureNodes.jl:6-43
    y[Y_PU] = b.pscale / ystpc[i];
    y[Y_PD] = -b.pscale / ystpc[i];
  }
  // ---- continuity (StencilForPContinuityUnknown.jl:31-52) ----
  bool internal;
  switch (b.pressure_bc_mode) {  // Domain.found_internal_cell_continuity
    case 0: internal = (j > 1 || i > 1); break;
    case 1: internal = (1 < i && i < b.ynum - 1); break;
    case 2: internal = (1 < j && j < b.xnum - 1); break;
    default: internal = false;
  }
  if (!internal) {  // boundary/BoundaryCells.jl:36-203
    const double rbc = 2.0 * b.pressure_bc / (b.xstpavg + b.ystpavg);
    Rc = 0.0;
    if (b.pressure_bc_mode >= 0 && b.pressure_bc_mode <= 2) {
      p[C_C] = kbond;
      Rc = (b.pressure_bc_mode == 0) ? rbc : (b.pressure_bc_mode == 1 ? (top ? rbc : 0.0) : (left ? rbc : 0.0));
    }
  } else {
    const double ps = b.pscale;
    const bool lower = i >= b.ynum - 1, rightb = j >= b.xnum - 1;
    Rc = A2(b.RC, b.ynum - 1, i, j) * ps;
    // internal/stencil_nodes/LeftVelocityXNode.jl:8-46
    if (!left) {
      p[C_XL] = -ps / xstp[j - 1];
      if (rightb) {
        p[C_XL] = p[C_XL] + BY1(brightx, i + 1, 2) * ps / xstp[j - 1];
        Rc = Rc - BY1(brightx, i + 1, 1) * ps / xstp[j - 1];
      }
    }
    // RightVelocityXNode.jl:8-45
    if (!rightb) {
      p[C_XR] = ps / xstp[j - 1];
      if (left) {
        p[C_XR] = p[C_XR] - BY1(bleftx, i + 1, 2) * ps / xstp[j - 1];
        Rc = Rc + BY1(bleftx, i + 1, 1) * ps / xstp[j - 1];
      }
    }
    // UpperVelocityYNode.jl:8-50
    if (!top) {
      p[C_YU] = -ps / ystp[i - 1];
      if (lower) {
        p[C_YU] = p[C_YU] + BX1(bbottomy, j + 1, 2) * ps / ystp[i - 1];
        Rc = Rc - BX1(bbottomy, j + 1, 1) * ps / ystp[i - 1];
      }
    }
    // BottomVelocityYNode.jl:8-44
    if (!lower) {
      p[C_YD] = ps / ystp[i - 1];
      if (top) {
        p[C_YD] = p[C_YD] - BX1(btopy, j + 1, 2) * ps / ystp[i - 1];
        Rc = Rc + BX1(btopy, j + 1, 1) * ps / ystp[i - 1];
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 11; ++k) coef[(int64_t)k * nc + c] = x[k];
#pragma unroll
  for (int k = 0; k < 11; ++k) coef[(int64_t)(11 + k) * nc + c] = y[k];
#pragma unroll
  for (int k = 0; k < 5; ++k) coef[(int64_t)(22 + k) * nc + c] = p[k];
  rhs[c] = Rx;
  rhs[nc + c] = Ry;
  rhs[2 * nc + c] = Rc;
#undef ETAN
#undef ETAS
#undef RHOVY
#undef BX
#undef BX1
#undef BY1
#undef BY
}

// ---- SystemSolver.reload_solu_vel! (:188-235) -------------------------------
__global__ void k_reload_solution(const double* __restrict__ S, int32_t xnum, int32_t ynum, double pscale,
                                  double* __restrict__ vx1, double* __restrict__ vy1, double* __restrict__ pr1) {
  const int64_t nc = (int64_t)(xnum - 1) * (ynum - 1);
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const int32_t i = (int32_t)(c % (ynum - 1)) + 1, j = (int32_t)(c / (ynum - 1)) + 1;
  if (j < xnum - 1) A2(vx1, ynum + 1, i + 1, j + 1) = S[c];
  if (i < ynum - 1) A2(vy1, ynum, i + 1, j + 1) = S[nc + c];
  A2(pr1, ynum - 1, i, j) = S[2 * nc + c] * pscale;
}

// ---- SystemSolver.apply_vel_bc! (:237-271), its four loops in order ---------
__global__ void k_bc_top_bottom_vx(double* vx1, const double* btopx, const double* bbottomx, int32_t xnum, int32_t ynum) {
  const int32_t j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > xnum) return;
  A2(vx1, ynum + 1, 1, j) = A2(btopx, xnum, j, 1) + A2(btopx, xnum, j, 2) * A2(vx1, ynum + 1, 2, j);
  A2(vx1, ynum + 1, ynum + 1, j) = A2(bbottomx, xnum, j, 1) + A2(bbottomx, xnum, j, 2) * A2(vx1, ynum + 1, ynum, j);
}
__global__ void k_bc_top_bottom_vy(double* vy1, const double* btopy, const double* bbottomy, int32_t xnum, int32_t ynum) {
  const int32_t j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > xnum + 1) return;
  A2(vy1, ynum, 1, j) = A2(btopy, xnum + 1, j, 1) + A2(btopy, xnum + 1, j, 2) * A2(vy1, ynum, 2, j);
  A2(vy1, ynum, ynum, j) = A2(bbottomy, xnum + 1, j, 1) + A2(bbottomy, xnum + 1, j, 2) * A2(vy1, ynum, ynum - 1, j);
}
__global__ void k_bc_left_right_vx(double* vx1, const double* bleftx, const double* brightx, int32_t xnum, int32_t ynum) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (i > ynum + 1) return;
  A2(vx1, ynum + 1, i, 1) = A2(bleftx, ynum + 1, i, 1) + A2(bleftx, ynum + 1, i, 2) * A2(vx1, ynum + 1, i, 2);
  A2(vx1, ynum + 1, i, xnum) = A2(brightx, ynum + 1, i, 1) + A2(brightx, ynum + 1, i, 2) * A2(vx1, ynum + 1, i, xnum - 1);
}
__global__ void k_bc_left_right_vy(double* vy1, const double* blefty, const double* brighty, int32_t xnum, int32_t ynum) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (i > ynum) return;
  A2(vy1, ynum, i, 1) = A2(blefty, ynum, i, 1) + A2(blefty, ynum, i, 2) * A2(vy1, ynum, i, 2);
  A2(vy1, ynum, i, xnum + 1) = A2(brighty, ynum, i, 1) + A2(brighty, ynum, i, 2) * A2(vy1, ynum, i, xnum);
}

// ---- post-solve grid kernels ---------------------------------------------
// GridStrainRate.jl:21-182: exx (pressure grid), exy and esp (basic grid); one thread per basic node.
__global__ void k_grid_strain_rate(int32_t xnum, int32_t ynum, const double* __restrict__ xstp_b,
                                   const double* __restrict__ ystp_b, const double* __restrict__ xstp_vy,
                                   const double* __restrict__ ystp_vx, const double* __restrict__ vx1,
                                   const double* __restrict__ vy1, double* __restrict__ exx, double* __restrict__ exy,
                                   double* __restrict__ esp) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (int64_t)xnum * ynum) return;
  const int32_t i = (int32_t)(k % ynum) + 1, j = (int32_t)(k / ynum) + 1;
  const int32_t yx = ynum + 1;
  if (i < ynum && j < xnum)
    A2(exx, ynum - 1, i, j) = 0.5 * ((A2(vx1, yx, i + 1, j + 1) - A2(vx1, yx, i + 1, j)) / xstp_b[j - 1] -
                                     (A2(vy1, ynum, i + 1, j + 1) - A2(vy1, ynum, i, j + 1)) / ystp_b[i - 1]);
  const double dvx = (A2(vx1, yx, i + 1, j) - A2(vx1, yx, i, j)) / ystp_vx[i - 1];
  const double dvy = (A2(vy1, ynum, i, j + 1) - A2(vy1, ynum, i, j)) / xstp_vy[j - 1];
  A2(exy, ynum, i, j) = 0.5 * (dvx + dvy);
  A2(esp, ynum, i, j) = 0.5 * (dvy - dvx);
}
// GridStrainRate.calculate_second_invariant! (:107-131); x^2.0 is x*x in Julia
__global__ void k_grid_eii(int32_t xnum, int32_t ynum, const double* __restrict__ exx, const double* __restrict__ exy,
                           double* __restrict__ eii) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (int64_t)(xnum - 1) * (ynum - 1)) return;
  const int32_t i = (int32_t)(k % (ynum - 1)) + 2, j = (int32_t)(k / (ynum - 1)) + 2;
  const double e = A2(exx, ynum - 1, i - 1, j - 1);
  const double a = A2(exy, ynum, i - 1, j - 1), b = A2(exy, ynum, i, j - 1);
  const double c = A2(exy, ynum, i - 1, j), d = A2(exy, ynum, i, j);
  A2(eii, ynum - 1, i - 1, j - 1) = sqrt(e * e + (a * a + b * b + c * c + d * d) / 4.0);
}
// GridStress.forecast_viscoelastic_{shear,normal}_stress! (:54-126)
__global__ void k_forecast_stress(const double* __restrict__ eta1, const double* __restrict__ mu1,
                                  const double* __restrict__ e, const double* __restrict__ s1,
                                  double* __restrict__ s2, int64_t n, double dt) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double eta = eta1[k];
  const double f = eta / (eta + dt * mu1[k]);
  s2[k] = (1.0 - f) * 2.0 * eta * e[k] + f * s1[k];
}
// GridStress.calculate_deviatoric_grid_stress_change! (:128-134)
__global__ void k_stress_change(const double* __restrict__ s2, const double* __restrict__ s1, double* __restrict__ ds,
                                int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) ds[k] = s2[k] - s1[k];
}
// StokesInterpolate.interpolate_stag_velocity_to_basic_grid! (:16-33)
__global__ void k_stag_to_basic(int32_t xnum, int32_t ynum, const double* __restrict__ vx1,
                                const double* __restrict__ vy1, double* __restrict__ vxb, double* __restrict__ vyb) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (int64_t)xnum * ynum) return;
  const int32_t i = (int32_t)(k % ynum) + 1, j = (int32_t)(k / ynum) + 1;
  A2(vxb, ynum, i, j) = (A2(vx1, ynum + 1, i, j) + A2(vx1, ynum + 1, i + 1, j)) / 2.0;
  A2(vyb, ynum, i, j) = (A2(vy1, ynum, i, j) + A2(vy1, ynum, i, j + 1)) / 2.0;
}

// HarmonicAverage.normal_viscosity_from_harmonic_avg_shear_viscosity! (HarmonicAverage.jl:20-51):
// cells that yield (CheckPlasticYield.plastic_yielding, tolerance 0) take the harmonic mean of
// their four corner etas1 (MathTools.harmonic4 with zero factors).
__global__ void k_harmonic_etan(int32_t xnum, int32_t ynum, const double* __restrict__ etas1,
                                const double* __restrict__ plastics, const double* __restrict__ plasticn,
                                const double* __restrict__ pyield, double* __restrict__ etan1) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (int64_t)(xnum - 1) * (ynum - 1)) return;
  const int32_t i = (int32_t)(k % (ynum - 1)) + 1, j = (int32_t)(k / (ynum - 1)) + 1;
  bool y = A2(plasticn, ynum - 1, i, j) > 0.0;
  y = y || A2(plastics, ynum, i, j) > 0.0 || A2(plastics, ynum, i, j + 1) > 0.0 ||
      A2(plastics, ynum, i + 1, j) > 0.0 || A2(plastics, ynum, i + 1, j + 1) > 0.0;
  y = y || A2(pyield, ynum, i, j) > 0.0 || A2(pyield, ynum, i, j + 1) > 0.0 || A2(pyield, ynum, i + 1, j) > 0.0 ||
      A2(pyield, ynum, i + 1, j + 1) > 0.0;
  if (!y) return;
  const double vinv = 1.0 / A2(etas1, ynum, i, j) + 1.0 / A2(etas1, ynum, i, j + 1) + 1.0 / A2(etas1, ynum, i + 1, j) +
                      1.0 / A2(etas1, ynum, i + 1, j + 1) + 0.0 + 0.0 + 0.0 + 0.0;
  if (vinv != 0.0) A2(etan1, ynum - 1, i, j) = 1.0 / (vinv / (4.0 + 0.0 + 0.0 + 0.0 + 0.0));
}

// ---- PlasticFailureNodes.jl:24-318 ------------------------------------------
struct NodalYieldIn {
  int32_t xnum, ynum;
  int64_t ntimestep;
  int32_t iuse_fluid, no_wall, no_plate;
  double dt, timesum, eta_min, eta_max, y_sealevel;
  double vix, xl, xr, yt, yb, pthick, pwidth;
  const double *gx, *gy, *pyield, *etas1, *eta_flow, *mus1, *coh, *fric, *sxy2, *sxx2, *pr1;
  double *yerr, *etavp, *psr, *pyield_new;
};
// interpolate_from_pressure_grid_to_basic_grid (:221-257)
__device__ double p_to_basic(int32_t i, int32_t j, int32_t ynum, int32_t xnum, const double* a) {
  const int32_t yp = ynum - 1;
  if (1 < i && i < ynum && 1 < j && j < xnum)
    return (A2(a, yp, i - 1, j - 1) + A2(a, yp, i, j - 1) + A2(a, yp, i - 1, j) + A2(a, yp, i, j)) / 4.0;
  if (i == 1 && j == 1) return A2(a, yp, i, j);
  if (i == ynum && j == 1) return A2(a, yp, i - 1, j);
  if (i == ynum && j == xnum) return A2(a, yp, i - 1, j - 1);
  if (i == 1 && j == xnum) return A2(a, yp, i, j - 1);
  if (j == 1) return (A2(a, yp, i, j) + A2(a, yp, i - 1, j)) / 2.0;
  if (j == xnum) return (A2(a, yp, i - 1, j - 1) + A2(a, yp, i, j - 1)) / 2.0;
  if (i == 1) return (A2(a, yp, i, j) + A2(a, yp, i, j - 1)) / 2.0;
  return (A2(a, yp, i - 1, j) + A2(a, yp, i - 1, j - 1)) / 2.0;
}
// One thread per basic node; per-block (count, sum err^2) in partial[2 * block].
__global__ void k_nodal_yield(NodalYieldIn q, double* __restrict__ partial) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double cnt = 0.0, esq = 0.0;
  if (k < (int64_t)q.xnum * q.ynum) {
    const int32_t i = (int32_t)(k % q.ynum) + 1, j = (int32_t)(k / q.ynum) + 1;
    const int32_t Y = q.ynum;
    const double vold = A2(q.etas1, Y, i, j), vflow = A2(q.eta_flow, Y, i, j), mu = A2(q.mus1, Y, i, j);
    const double coh = A2(q.coh, Y, i, j);
    const double fc = sin(A2(q.fric, Y, i, j) * (3.14159265358979323846 / 180.0));
    double etavp = vflow, ynew = 0.0, psr = 0.0;
    bool applicable = q.ntimestep > 0 && (coh > 0.0 || fc > 0.0);
    const double xs = q.vix * q.timesum;
    const double xn = q.gx[j - 1], yn = q.gy[i - 1];
    if (q.no_wall && (q.xl + xs) <= xn && xn <= (q.xr + xs) && q.yt <= yn && yn <= q.yb) applicable = false;
    if (q.no_plate) {
      const double xl = q.xl + xs;
      if (xl - q.pwidth <= xn && xn <= xl && q.yb - q.pthick <= yn && yn <= q.yb) applicable = false;
    }
    if (applicable) {
      const double p = p_to_basic(i, j, Y, q.xnum, q.pr1);
      const double sxx = p_to_basic(i, j, Y, q.xnum, q.sxx2), sxy = A2(q.sxy2, Y, i, j);
      const double sii = sqrt(sxy * sxy + sxx * sxx);
      const double sie = sii * (mu * q.dt + vold) / vold;
      const double cphi = cos(asin(fc));
      double sy;
      if (q.iuse_fluid == 0) {
        sy = coh * cphi + fc * p;
      } else {
        double depth = yn - q.y_sealevel;
        if (depth < 0.0) depth = 0.0;
        const double pf = 1000.0 * 9.81 * depth;
        sy = (p < pf) ? coh * cphi : coh * cphi + fc * (p - pf);
      }
      if (sy < 0.0) sy = 0.0;
      const bool at_yield = A2(q.pyield, Y, i, j) > 0;
      bool counted = false;
      if (at_yield) counted = true;
      if (sy < sie) {
        double vnew = q.dt * mu * sy / (sie - sy);
        if (vnew < vflow) {
          ynew = 1.0;
          vnew = vnew > q.eta_min ? vnew : q.eta_min;
          vnew = vnew < q.eta_max ? vnew : q.eta_max;
          etavp = vnew;
          psr = 0.5 * sii / vnew - 0.5 * sii / vflow;
          counted = true;
        }
      }
      if (counted) {
        const double err = sii - sy;
        A2(q.yerr, Y, i, j) = err;
        cnt = 1.0;
        esq = err * err;
      }
    }
    A2(q.etavp, Y, i, j) = etavp;
    A2(q.pyield_new, Y, i, j) = ynew;
    A2(q.psr, Y, i, j) = psr;
  }
  __shared__ double sc[kB], se[kB];
  sc[threadIdx.x] = cnt;
  se[threadIdx.x] = esq;
  __syncthreads();
  for (int o = kB / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) { sc[threadIdx.x] += sc[threadIdx.x + o]; se[threadIdx.x] += se[threadIdx.x + o]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) { partial[2 * blockIdx.x] = sc[0]; partial[2 * blockIdx.x + 1] = se[0]; }
}
// PlasticStrainRateInterpolation.interpolate_at_pressure_nodes! (:13-40)
__global__ void k_eii_plastic_pressure(int32_t xnum, int32_t ynum, const double* __restrict__ eb,
                                       double* __restrict__ ep) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (int64_t)(xnum - 1) * (ynum - 1)) return;
  const int32_t i = (int32_t)(k % (ynum - 1)) + 1, j = (int32_t)(k / (ynum - 1)) + 1;
  A2(ep, ynum - 1, i, j) = (A2(eb, ynum, i, j) + A2(eb, ynum, i, j + 1) + A2(eb, ynum, i + 1, j) +
                            A2(eb, ynum, i + 1, j + 1)) / 4.0;
}

// ---- the reference's COO entry order ------------------------------------------
// Which stencil slots StokesBuildManager emits for cell (i, j), in its order (the same
// branches as k_build_system; folds modify entries already emitted and add none).
struct CooIn {
  int32_t xnum, ynum, pressure_bc_mode;
  int64_t zone[8];
};
struct CooEntry { int8_t slot; int64_t col; };
__device__ int coo_entries(const CooIn& b, int32_t i, int32_t j, CooEntry* e) {
  const int64_t ny = b.ynum - 1;
  const int64_t c = (int64_t)(j - 1) * ny + (i - 1);
  const bool top = i == 1, left = j == 1;
  int n = 0;
  auto put = [&](int slot, int64_t col) { e[n].slot = (int8_t)slot; e[n].col = col; ++n; };
  // x-Stokes
  const bool out_x = j != b.zone[0] || i < b.zone[1] || i > b.zone[2];
  if (!(j < b.xnum - 1 && out_x)) {
    put(X_C, 3 * c);
  } else {
    const bool bot = i >= b.ynum - 1, right2 = j >= b.xnum - 2;
    put(X_C, 3 * c);
    if (!left) put(X_L, 3 * (c - ny));
    if (!right2) put(X_R, 3 * (c + ny));
    if (!top) put(X_U, 3 * (c - 1));
    if (!bot) put(X_D, 3 * (c + 1));
    if (!top) put(X_YUL, 3 * (c - 1) + 1); else put(X_YLL, 3 * c + 1);
    if (!top) put(X_YUR, 3 * (c - 1 + ny) + 1); else put(X_YLR, 3 * (c + ny) + 1);
    if (!bot && !top) put(X_YLL, 3 * c + 1);
    if (!bot && !top) put(X_YLR, 3 * (c + ny) + 1);
    put(X_PL, 3 * c + 2);
    put(X_PR, 3 * (c + ny) + 2);
  }
  // y-Stokes
  const bool out_y = j != b.zone[4] || i < b.zone[5] || i > b.zone[6];
  if (!(i < b.ynum - 1 && out_y)) {
    put(11 + Y_C, 3 * c + 1);
  } else {
    const bool bot2 = i >= b.ynum - 2, right = j >= b.xnum - 1;
    put(11 + Y_C, 3 * c + 1);
    if (!top) put(11 + Y_U, 3 * (c - 1) + 1);
    if (!bot2) put(11 + Y_D, 3 * (c + 1) + 1);
    if (!left) put(11 + Y_L, 3 * (c - ny) + 1);
    if (!right) put(11 + Y_R, 3 * (c + ny) + 1);
    if (!left) put(11 + Y_XUL, 3 * (c - ny)); else put(11 + Y_XUR, 3 * c);
    if (!left) put(11 + Y_XLL, 3 * (c + 1 - ny)); else put(11 + Y_XLR, 3 * (c + 1));
    if (!right && !left) put(11 + Y_XUR, 3 * c);
    if (!right && !left) put(11 + Y_XLR, 3 * (c + 1));
    put(11 + Y_PU, 3 * c + 2);
    put(11 + Y_PD, 3 * (c + 1) + 2);
  }
  // continuity
  bool internal;
  switch (b.pressure_bc_mode) {
    case 0: internal = (j > 1 || i > 1); break;
    case 1: internal = (1 < i && i < b.ynum - 1); break;
    case 2: internal = (1 < j && j < b.xnum - 1); break;
    default: internal = false;
  }
  if (!internal) {
    if (b.pressure_bc_mode >= 0 && b.pressure_bc_mode <= 2) put(22 + C_C, 3 * c + 2);
  } else {
    const bool lower = i >= b.ynum - 1, rightb = j >= b.xnum - 1;
    if (!left) put(22 + C_XL, 3 * (c - ny));
    if (!rightb) put(22 + C_XR, 3 * c);
    if (!top) put(22 + C_YU, 3 * (c - 1) + 1);
    if (!lower) put(22 + C_YD, 3 * c + 1);
  }
  return n;
}
// Cells in the reference's build order: r = (i-1) (xnum-1) + (j-1).
__global__ void k_coo_count(CooIn b, int32_t* __restrict__ count, int64_t nc) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nc) return;
  const int32_t i = (int32_t)(r / (b.xnum - 1)) + 1, j = (int32_t)(r % (b.xnum - 1)) + 1;
  CooEntry e[kStencilSlots];
  count[r] = coo_entries(b, i, j, e);
}
__global__ void k_coo_write(CooIn b, const int64_t* __restrict__ offset, const double* __restrict__ coef, int64_t nc,
                            int64_t* __restrict__ Li, int64_t* __restrict__ Lj, double* __restrict__ Lv) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nc) return;
  const int32_t i = (int32_t)(r / (b.xnum - 1)) + 1, j = (int32_t)(r % (b.xnum - 1)) + 1;
  const int64_t c = (int64_t)(j - 1) * (b.ynum - 1) + (i - 1);
  CooEntry e[kStencilSlots];
  const int n = coo_entries(b, i, j, e);
  int64_t o = offset[r];
  for (int k = 0; k < n; ++k, ++o) {
    const int row_kind = e[k].slot < 11 ? 0 : (e[k].slot < 22 ? 1 : 2);
    Li[o] = 3 * c + row_kind + 1;
    Lj[o] = e[k].col + 1;
    Lv[o] = coef[(int64_t)e[k].slot * nc + c];
  }
}

unsigned nblk(int64_t n) { return (unsigned)((n + kB - 1) / kB); }

}  // namespace

// The system as the reference's COO list (1-based Li, Lj; Lv), in StokesBuildManager's
// entry order.  Li/Lj/Lv null: only *nnz is returned.
int export_stokes_coo(eb_ctx* c, const StokesSystem* s, int64_t* Li, int64_t* Lj, double* Lv, int64_t capacity,
                      int64_t* nnz) {
  CooIn b{c->xnum, c->ynum, (int32_t)c->SP.pressure_bc_mode, {}};
  for (int k = 0; k < 8; ++k) b.zone[k] = c->SP.bintern_zone[k];
  const int64_t nc = s->nc;
  int32_t* d_count = nullptr;
  EB_CK(c, cudaMalloc(&d_count, nc * sizeof(int32_t)));
  k_coo_count<<<nblk(nc), kB, 0, c->stream>>>(b, d_count, nc);
  c->launches++;
  std::vector<int32_t> h(nc);
  cudaError_t e = cudaMemcpyAsync(h.data(), d_count, nc * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d_count);
  if (e != cudaSuccess) return eb_cuda(c, e, "COO entry count");
  std::vector<int64_t> off(nc);
  int64_t total = 0;
  for (int64_t r = 0; r < nc; ++r) { off[r] = total; total += h[r]; }
  if (nnz) *nnz = total;
  if (!Li || !Lj || !Lv) return EB_OK;
  if (capacity < total) return eb_fail(c, EB_BAD_INPUT, "COO arrays hold " + std::to_string(capacity) +
                                                            " entries, the system has " + std::to_string(total));
  int64_t *d_off = nullptr, *d_li = nullptr, *d_lj = nullptr;
  double* d_lv = nullptr;
  e = cudaMalloc(&d_off, nc * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMalloc(&d_li, total * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMalloc(&d_lj, total * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMalloc(&d_lv, total * sizeof(double));
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_off, off.data(), nc * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) {
    k_coo_write<<<nblk(nc), kB, 0, c->stream>>>(b, d_off, s->coef, nc, d_li, d_lj, d_lv);
    c->launches++;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(Li, d_li, total * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(Lj, d_lj, total * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(Lv, d_lv, total * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d_off); cudaFree(d_li); cudaFree(d_lj); cudaFree(d_lv);
  if (e != cudaSuccess) return eb_cuda(c, e, "COO export");
  return EB_OK;
}

int launch_nodal_yield(eb_ctx* c, const eb_mobile_wall* w, double* d_partial, int* nblocks) {
  double** g = c->gf;
  NodalYieldIn q{};
  q.xnum = c->xnum; q.ynum = c->ynum; q.ntimestep = c->P.ntimestep;
  q.iuse_fluid = (int32_t)c->P.iuse_fluid_pressure_for_yield; q.no_wall = (int32_t)(c->P.no_yielding_in_mobile_wall != 0);
  q.dt = c->P.timestep; q.eta_min = c->P.viscosity_min; q.eta_max = c->P.viscosity_max; q.y_sealevel = c->P.y_sealevel;
  if (w) {
    q.no_plate = (int32_t)(w->no_yielding_in_plate_extension != 0);
    q.timesum = w->timesum; q.vix = w->velocity_internal_x;
    q.xl = w->x_left_mobile_wall; q.xr = w->x_right_mobile_wall; q.yt = w->y_top_mobile_wall; q.yb = w->y_bottom_mobile_wall;
    q.pthick = w->plate_extension_thickness; q.pwidth = w->plate_extension_width;
  } else {
    q.no_wall = 0;
  }
  q.gx = c->g.gx; q.gy = c->g.gy;
  q.pyield = g[EB_G_PLASTIC_YIELD]; q.etas1 = g[EB_G_ETAS1]; q.eta_flow = g[EB_G_ETA_FLOW]; q.mus1 = g[EB_G_MUS1];
  q.coh = g[EB_G_COHESION]; q.fric = g[EB_G_FRIC_DEG]; q.sxy2 = g[EB_G_SXY2]; q.sxx2 = g[EB_G_SXX2]; q.pr1 = g[EB_G_PR1];
  q.yerr = g[EB_G_YIELD_ERROR]; q.etavp = g[EB_G_ETAVP_BUFFER]; q.psr = g[EB_G_PLASTIC_STRAIN_RATE_BUFFER];
  q.pyield_new = g[EB_G_PLASTIC_YIELD_BUFFER];
  *nblocks = (int)nblk((int64_t)c->xnum * c->ynum);
  EB_PROF(c, "k_nodal_yield");
  k_nodal_yield<<<*nblocks, kB, 0, c->stream>>>(q, d_partial);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_apply_nodal_yield(eb_ctx* c) {
  double** g = c->gf;
  const size_t nb = (size_t)c->xnum * c->ynum * sizeof(double);
  EB_CK(c, cudaMemcpyAsync(g[EB_G_ETAS1], g[EB_G_ETAVP_BUFFER], nb, cudaMemcpyDeviceToDevice, c->stream));
  EB_CK(c, cudaMemcpyAsync(g[EB_G_PLASTIC_YIELD], g[EB_G_PLASTIC_YIELD_BUFFER], nb, cudaMemcpyDeviceToDevice, c->stream));
  EB_CK(c, cudaMemcpyAsync(g[EB_G_EII_PLASTIC_BASIC], g[EB_G_PLASTIC_STRAIN_RATE_BUFFER], nb, cudaMemcpyDeviceToDevice,
                           c->stream));
  EB_PROF(c, "k_eii_plastic_pressure");
  k_eii_plastic_pressure<<<nblk((int64_t)(c->xnum - 1) * (c->ynum - 1)), kB, 0, c->stream>>>(
      c->xnum, c->ynum, g[EB_G_EII_PLASTIC_BASIC], g[EB_G_EII_PLASTIC_PRESSURE]);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_harmonic_etan(eb_ctx* c) {
  double** g = c->gf;
  EB_PROF(c, "k_harmonic_etan");
  k_harmonic_etan<<<nblk((int64_t)(c->xnum - 1) * (c->ynum - 1)), kB, 0, c->stream>>>(
      c->xnum, c->ynum, g[EB_G_ETAS1], g[EB_G_PLASTICS], g[EB_G_PLASTICN], g[EB_G_PLASTIC_YIELD], g[EB_G_ETAN1]);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_grid_strain_rate(eb_ctx* c) {
  double** g = c->gf;
  const int32_t X = c->xnum, Y = c->ynum;
  EB_PROF(c, "k_grid_strain_rate");
  k_grid_strain_rate<<<nblk((int64_t)X * Y), kB, 0, c->stream>>>(X, Y, c->g.sx, c->g.sy, c->g_xstp_vy, c->g_ystp_vx,
                                                                  g[EB_G_VX1], g[EB_G_VY1], g[EB_G_EXX], g[EB_G_EXY],
                                                                  g[EB_G_ESP]);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_grid_eii");
  k_grid_eii<<<nblk((int64_t)(X - 1) * (Y - 1)), kB, 0, c->stream>>>(X, Y, g[EB_G_EXX], g[EB_G_EXY], g[EB_G_EII]);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_forecast_stress(eb_ctx* c) {
  double** g = c->gf;
  const int64_t nb = (int64_t)c->xnum * c->ynum, np = (int64_t)(c->xnum - 1) * (c->ynum - 1);
  EB_PROF(c, "k_forecast_stress");
  k_forecast_stress<<<nblk(nb), kB, 0, c->stream>>>(g[EB_G_ETAS1], g[EB_G_MUS1], g[EB_G_EXY], g[EB_G_SXY1], g[EB_G_SXY2],
                                                    nb, c->P.timestep);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_forecast_stress");
  k_forecast_stress<<<nblk(np), kB, 0, c->stream>>>(g[EB_G_ETAN1], g[EB_G_MUN1], g[EB_G_EXX], g[EB_G_SXX1], g[EB_G_SXX2],
                                                    np, c->P.timestep);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_stress_change(eb_ctx* c) {
  double** g = c->gf;
  const int64_t nb = (int64_t)c->xnum * c->ynum, np = (int64_t)(c->xnum - 1) * (c->ynum - 1);
  EB_PROF(c, "k_stress_change");
  k_stress_change<<<nblk(nb), kB, 0, c->stream>>>(g[EB_G_SXY2], g[EB_G_SXY1], g[EB_G_DSXY], nb);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_stress_change");
  k_stress_change<<<nblk(np), kB, 0, c->stream>>>(g[EB_G_SXX2], g[EB_G_SXX1], g[EB_G_DSXX], np);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_stag_to_basic(eb_ctx* c) {
  double** g = c->gf;
  EB_PROF(c, "k_stag_to_basic");
  k_stag_to_basic<<<nblk((int64_t)c->xnum * c->ynum), kB, 0, c->stream>>>(c->xnum, c->ynum, g[EB_G_VX1], g[EB_G_VY1],
                                                                          g[EB_G_VXB], g[EB_G_VYB]);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_viscoelastic_terms(eb_ctx* c) {
  double** g = c->gf;
  const int64_t nb = (int64_t)c->xnum * c->ynum, np = (int64_t)(c->xnum - 1) * (c->ynum - 1);
  EB_PROF(c, "k_ve_terms");
  k_ve_terms<<<nblk(nb), kB, 0, c->stream>>>(g[EB_G_ETAS1], g[EB_G_MUS1], g[EB_G_SXY1], g[EB_G_ETAS0], g[EB_G_SXY0],
                                             nb, c->P.timestep);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_ve_terms");
  k_ve_terms<<<nblk(np), kB, 0, c->stream>>>(g[EB_G_ETAN1], g[EB_G_MUN1], g[EB_G_SXX1], g[EB_G_ETAN0], g[EB_G_SXX0],
                                             np, c->P.timestep);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_viscoelastic_rhs(eb_ctx* c) {
  double** g = c->gf;
  const int32_t X = c->xnum, Y = c->ynum;
  EB_CK(c, cudaMemsetAsync(g[EB_G_RX1], 0, sizeof(double) * (size_t)(Y + 1) * X, c->stream));
  EB_CK(c, cudaMemsetAsync(g[EB_G_RY1], 0, sizeof(double) * (size_t)Y * (X + 1), c->stream));
  const DevGrid& G = c->g;
  EB_PROF(c, "k_rhs_xy");
  k_rhs_xy<<<nblk((int64_t)(X - 1) * (Y - 1)), kB, 0, c->stream>>>(
      X, Y, c->SP.gravity_x, c->SP.gravity_y, (int32_t)c->SP.iuse_interface_stabilization, G.sx, G.sy,
      c->g_xstp_vy, c->g_ystp_vx, g[EB_G_RHO1], g[EB_G_RHO1_VY], g[EB_G_SXX0], g[EB_G_SXY0], g[EB_G_RX1], g[EB_G_RY1]);
  EB_LAUNCHED(c);
  const int64_t np = (int64_t)(X - 1) * (Y - 1);
  EB_PROF(c, "k_rhs_c");
  k_rhs_c<<<nblk(np), kB, 0, c->stream>>>(g[EB_G_DILAT], g[EB_G_EII_PLASTIC_PRESSURE], g[EB_G_RC1], np);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_build_stokes_system(eb_ctx* c, StokesSystem* s) {
  double** g = c->gf;
  BuildIn b{};
  b.xnum = c->xnum; b.ynum = c->ynum;
  b.xstpavg = c->g.xstpavg; b.ystpavg = c->g.ystpavg;
  b.pscale = s->pscale; b.timestep = c->P.timestep; b.gravity_y = c->SP.gravity_y; b.pressure_bc = c->SP.pressure_bc;
  b.stab = (int32_t)c->SP.iuse_interface_stabilization; b.pressure_bc_mode = (int32_t)c->SP.pressure_bc_mode;
  for (int k = 0; k < 8; ++k) { b.zone[k] = c->SP.bintern_zone[k]; b.zvel[k] = c->SP.bintern_velocity[k]; }
  b.xstp = c->g.sx; b.ystp = c->g.sy; b.xstpc = c->g_xstp_vy; b.ystpc = c->g_ystp_vx;
  b.btopx = g[EB_G_BTOPX]; b.bbottomx = g[EB_G_BBOTTOMX]; b.btopy = g[EB_G_BTOPY]; b.bbottomy = g[EB_G_BBOTTOMY];
  b.bleftx = g[EB_G_BLEFTX]; b.brightx = g[EB_G_BRIGHTX]; b.blefty = g[EB_G_BLEFTY]; b.brighty = g[EB_G_BRIGHTY];
  b.etan = g[EB_G_ETAN0]; b.etas = g[EB_G_ETAS0]; b.rho_vy = g[EB_G_RHO1_VY];
  b.RX = g[EB_G_RX1]; b.RY = g[EB_G_RY1]; b.RC = g[EB_G_RC1];
  EB_PROF(c, "k_build_system");
  k_build_system<<<nblk(s->nc), kB, 0, c->stream>>>(b, s->coef, s->rhs, s->nc);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_process_stokes_solution(eb_ctx* c, const StokesSystem* s) {
  double** g = c->gf;
  const int32_t X = c->xnum, Y = c->ynum;
  EB_CK(c, cudaMemsetAsync(g[EB_G_VX1], 0, sizeof(double) * (size_t)(Y + 1) * X, c->stream));
  EB_CK(c, cudaMemsetAsync(g[EB_G_VY1], 0, sizeof(double) * (size_t)Y * (X + 1), c->stream));
  EB_PROF(c, "k_reload_solution");
  k_reload_solution<<<nblk(s->nc), kB, 0, c->stream>>>(s->S, X, Y, s->pscale, g[EB_G_VX1], g[EB_G_VY1], g[EB_G_PR1]);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_apply_vel_bc");
  k_bc_top_bottom_vx<<<nblk(X), kB, 0, c->stream>>>(g[EB_G_VX1], g[EB_G_BTOPX], g[EB_G_BBOTTOMX], X, Y);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_apply_vel_bc");
  k_bc_top_bottom_vy<<<nblk(X + 1), kB, 0, c->stream>>>(g[EB_G_VY1], g[EB_G_BTOPY], g[EB_G_BBOTTOMY], X, Y);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_apply_vel_bc");
  k_bc_left_right_vx<<<nblk(Y + 1), kB, 0, c->stream>>>(g[EB_G_VX1], g[EB_G_BLEFTX], g[EB_G_BRIGHTX], X, Y);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_apply_vel_bc");
  k_bc_left_right_vy<<<nblk(Y), kB, 0, c->stream>>>(g[EB_G_VY1], g[EB_G_BLEFTY], g[EB_G_BRIGHTY], X, Y);
  EB_LAUNCHED(c);
  return EB_OK;
}
