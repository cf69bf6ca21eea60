/* heat_oracle.c -- CPU restatement of the reference's conductive heat step, test
 * infrastructure only (the product path never links it).
 *
 * Grids are the reference's column-major (rows, cols) Float64 matrices, node
 * (i, j) 1-based at [(j-1)*rows + (i-1)].  Operand order follows the Julia
 * source so that a build without FMA contraction reproduces it bit for bit.
 *
 *   o_heat_rhs_terms      HeatRhs.initialize_rhs_terms_array_for_heat!,
 *                         add_adiabatic_terms_to_rhs_grid!, add_friction_terms_to_rhs_grid!
 *                         (src/heat_solver/rhs/HeatRhs.jl:5-80)
 *   o_heat_build          HeatBuildManager.build_system_of_equations
 *                         (src/heat_solver/solver/build_system/HeatBuildManager.jl:44-86) with
 *                         InternalNodes.apply_stencil (internal/InternalNodes.jl:20-198),
 *                         BoundaryNodes.apply_stencil (boundary/BoundaryNodes.jl:18-252) and the
 *                         stencil data of BuildStructs.HeatStencilData (utils/BuildStructs.jl:97-125);
 *                         xstp_pr from PressureGridTools.spacing_loop!
 *                         (src/staggered_grid/utils/PressureGridTools.jl:34-42)
 *   o_heat_residuals      HeatResiduals.compute_residuals_temp!
 *                         (src/heat_solver/solver/residuals/HeatResiduals.jl:12-162)
 *
 * Julia's x^2.0 for Float64 x is the correctly rounded square, i.e. x*x.
 */
#include <stdint.h>

#define G(a, rows, i, j) (a)[((int64_t)(j) - 1) * (rows) + ((i) - 1)]

/* RT1 = hr1; + adiabatic and friction terms on internal nodes. */
void o_heat_rhs_terms(int64_t xnum, int64_t ynum, const double* hr1, const double* ha1, const double* rho1,
                      const double* vx1, const double* vy1, const double* sxy2, const double* etas1,
                      const double* sxx2, const double* etan1, double gravity_x, double gravity_y,
                      int64_t iuse_adiabatic, int64_t iuse_shear, double* RT1) {
  const int64_t n = xnum * ynum;
  for (int64_t k = 0; k < n; ++k) RT1[k] = hr1[k];
  const int64_t rvx = ynum + 1, rvy = ynum, rp = ynum - 1;
  if (iuse_adiabatic == 1)
    for (int64_t j = 2; j <= xnum - 1; ++j)
      for (int64_t i = 2; i <= ynum - 1; ++i)
        G(RT1, ynum, i, j) += G(ha1, ynum, i, j) * G(rho1, ynum, i, j) *
                              (gravity_x * (G(vx1, rvx, i, j) + G(vx1, rvx, i + 1, j)) +
                               gravity_y * (G(vy1, rvy, i, j) + G(vy1, rvy, i, j + 1))) /
                              2.0;
  if (iuse_shear == 1)
    for (int64_t j = 2; j <= xnum - 1; ++j)
      for (int64_t i = 2; i <= ynum - 1; ++i) {
        const double s = G(sxy2, ynum, i, j);
        G(RT1, ynum, i, j) += s * s / G(etas1, ynum, i, j);
        const double a = G(sxx2, rp, i - 1, j - 1), b = G(sxx2, rp, i, j - 1), c = G(sxx2, rp, i - 1, j),
                     d = G(sxx2, rp, i, j);
        G(RT1, ynum, i, j) += (a * a / G(etan1, rp, i - 1, j - 1) + b * b / G(etan1, rp, i, j - 1) +
                               c * c / G(etan1, rp, i - 1, j) + d * d / G(etan1, rp, i, j)) /
                              4.0;
      }
}

/* COO (1-based Li, Lj; Lv) and R of the heat system; returns nnz.  tk is tk0 (the
 * old temperature), dt the heat-loop time step.  BC arrays: btop, bbottom (xnum, 2),
 * bleft, bright (ynum, 2). */
int64_t o_heat_build(int64_t xnum, int64_t ynum, const double* gx, const double* gy, const double* xstp,
                     const double* ystp, const double* tk, const double* rhocp, const double* kt, const double* RT,
                     const double* btop, const double* bbottom, const double* bleft, const double* bright,
                     double dt, int64_t* Li, int64_t* Lj, double* Lv, double* R) {
  int64_t inz = 0;
#define PUT(row, col, val) (Li[inz] = (row), Lj[inz] = (col), Lv[inz] = (val), ++inz)
  for (int64_t j = 1; j <= xnum; ++j)
    for (int64_t i = 1; i <= ynum; ++i) {
      const int64_t itk = (j - 1) * ynum + i;
      if (j == 1 || j == xnum || i == 1 || i == ynum) {
        if (i == 1 && 1 < j && j < xnum) {
          R[itk - 1] = G(btop, xnum, j, 1);
          PUT(itk, itk, 1.0);
          PUT(itk, itk + 1, -G(btop, xnum, j, 2));
        }
        if (i == ynum && 1 < j && j < xnum) {
          R[itk - 1] = G(bbottom, xnum, j, 1);
          PUT(itk, itk, 1.0);
          PUT(itk, itk - 1, -G(bbottom, xnum, j, 2));
        }
        if (j == 1) {
          R[itk - 1] = G(bleft, ynum, i, 1);
          PUT(itk, itk, 1.0);
          PUT(itk, itk + ynum, -G(bleft, ynum, i, 2));
        }
        if (j == xnum) {
          R[itk - 1] = G(bright, ynum, i, 1);
          PUT(itk, itk, 1.0);
          PUT(itk, itk - ynum, -G(bright, ynum, i, 2));
        }
        continue;
      }
      const double tkC = G(tk, ynum, i, j), rhocpC = G(rhocp, ynum, i, j);
      const double ktU = G(kt, ynum, i - 1, j), ktC = G(kt, ynum, i, j), ktD = G(kt, ynum, i + 1, j);
      const double ktL = G(kt, ynum, i, j - 1), ktR = G(kt, ynum, i, j + 1);
      const double dxL = xstp[j - 2], dxR = xstp[j - 1], dxC = (gx[j] - gx[j - 2]) / 2.0;
      const double dyU = ystp[i - 2], dyD = ystp[i - 1], dyC = (gy[i] - gy[i - 2]) / 2.0;
      R[itk - 1] = G(RT, ynum, i, j) + tkC * rhocpC / dt;
      PUT(itk, itk,
          rhocpC / dt + ((ktL + ktC) / dxL + (ktC + ktR) / dxR) / 2.0 / dxC +
              ((ktU + ktC) / dyU + (ktC + ktD) / dyD) / 2.0 / dyC);
      PUT(itk, itk - ynum, -(ktL + ktC) / 2.0 / dxL / dxC);
      PUT(itk, itk + ynum, -(ktC + ktR) / 2.0 / dxR / dxC);
      PUT(itk, itk - 1, -(ktU + ktC) / 2.0 / dyU / dyC);
      PUT(itk, itk + 1, -(ktC + ktD) / 2.0 / dyD / dyC);
    }
#undef PUT
  return inz;
}

/* rest on the basic grid from tk0 (old), tk2 (new). */
void o_heat_residuals(int64_t xnum, int64_t ynum, const double* gx, const double* gy, const double* xstp,
                      const double* ystp, const double* RT, const double* rhocp, const double* tk,
                      const double* tknew, const double* kt, double dt, double* rest) {
  for (int64_t j = 1; j <= xnum; ++j)
    for (int64_t i = 1; i <= ynum; ++i) {
      if (j == 1 || j == xnum || i == 1 || i == ynum) {
        G(rest, ynum, i, j) = 0.0;
        continue;
      }
      double r = G(RT, ynum, i, j) +
                 -G(rhocp, ynum, i, j) * (G(tknew, ynum, i, j) - G(tk, ynum, i, j)) / dt;
      const double xc = (gx[j] - gx[j - 2]) / 2.0, yc = (gy[i] - gy[i - 2]) / 2.0;
      r += ((G(kt, ynum, i, j) + G(kt, ynum, i, j + 1)) * (G(tknew, ynum, i, j + 1) - G(tknew, ynum, i, j)) /
                xstp[j - 1] -
            (G(kt, ynum, i, j - 1) + G(kt, ynum, i, j)) * (G(tknew, ynum, i, j) - G(tknew, ynum, i, j - 1)) /
                xstp[j - 2]) /
           2.0 / xc;
      r += ((G(kt, ynum, i, j) + G(kt, ynum, i + 1, j)) * (G(tknew, ynum, i + 1, j) - G(tknew, ynum, i, j)) /
                ystp[i - 1] -
            (G(kt, ynum, i - 1, j) + G(kt, ynum, i, j)) * (G(tknew, ynum, i, j) - G(tknew, ynum, i - 1, j)) /
                ystp[i - 2]) /
           2.0 / yc;
      G(rest, ynum, i, j) = r;
    }
}
