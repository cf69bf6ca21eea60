/*
 * stokes_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY) for the Stokes-continuity step.
 *
 * A plain-C, FP64, serial restatement of the reference EarthBox.jl functions
 * that turn the marker-averaged grids into the Stokes-continuity system and
 * its solution into grid velocities and pressure:
 *   - viscoelastic viscosity and stress terms (StokesViscoelasticTerms.jl),
 *   - right-hand-side grids RX1, RY1, RC1 (StokesContinuityRhs.jl),
 *   - the pressure scaling pscale (SystemSolver.jl:110-115),
 *   - the COO system Li, Lj, Lv, R in the reference's entry order
 *     (StokesBuildManager.jl:661-712 and the stencil modules it calls),
 *   - reload_solu_vel! and apply_vel_bc! (SystemSolver.jl:188-271),
 *   - the COO product used by the residuals (StokesResiduals.jl:63-81).
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 *
 * Fidelity rules: compiled with -ffp-contract=off and without fast-math; every
 * floating-point expression keeps the reference's operand order, so the COO
 * values are bit-identical to what the reference computes; grids are
 * column-major (rows, cols) and all indices 1-based, as in Julia.
 * File paths are relative to src/stokes_continuity_solver/ of EarthBox.jl.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

/* Julia pi as a Float64 */
#define O_PI 3.14159265358979323846

#define A2(a, rows, i, j) (a)[((int64_t)(j) - 1) * (int64_t)(rows) + ((int64_t)(i) - 1)]

/* Viscoelastic.calculate_viscoelastic_factor (utils/Viscoelastic.jl:26-38) */
static double ve_factor(double eta, double mu, double dt) { return eta / (eta + dt * mu); }

/* StokesViscoelasticTerms.viscoelastic_shear_stress_and_viscosity_terms! (:51-87)
 * and viscoelastic_normal_stress_and_viscosity_terms! (:89-125). */
void o_viscoelastic_terms(int64_t xnum, int64_t ynum, double dt,
                          const double* etas1, const double* mus1, const double* sxy1,
                          const double* etan1, const double* mun1, const double* sxx1,
                          double* etas0, double* sxy0, double* etan0, double* sxx0) {
  for (int64_t j = 1; j <= xnum; ++j)
    for (int64_t i = 1; i <= ynum; ++i) {
      const double f = ve_factor(A2(etas1, ynum, i, j), A2(mus1, ynum, i, j), dt);
      A2(etas0, ynum, i, j) = A2(etas1, ynum, i, j) * (1.0 - f);
      A2(sxy0, ynum, i, j) = A2(sxy1, ynum, i, j) * f;
    }
  for (int64_t j = 1; j <= xnum - 1; ++j)
    for (int64_t i = 1; i <= ynum - 1; ++i) {
      const double f = ve_factor(A2(etan1, ynum - 1, i, j), A2(mun1, ynum - 1, i, j), dt);
      A2(etan0, ynum - 1, i, j) = A2(etan1, ynum - 1, i, j) * (1 - f);
      A2(sxx0, ynum - 1, i, j) = A2(sxx1, ynum - 1, i, j) * f;
    }
}

/* StokesContinuityRhs.viscoelastic_rhs! (:30-61): RX1 (ynum+1, xnum), RY1
 * (ynum, xnum+1), RC1 (ynum-1, xnum-1); zeroed first, then the y-Stokes
 * (:63-120), x-Stokes (:122-157) and continuity (:159-190) parts. */
void o_viscoelastic_rhs(int64_t xnum, int64_t ynum, double gravity_x, double gravity_y, int64_t stab,
                        const double* xstp_b, const double* ystp_b, const double* xstp_vy,
                        const double* ystp_vx, const double* rho1, const double* rho1_vy,
                        const double* sxx0, const double* sxy0, const double* dilatation_grid,
                        const double* eii_plastic_pressure, double* RX1, double* RY1, double* RC1) {
  memset(RX1, 0, sizeof(double) * (size_t)((ynum + 1) * xnum));
  memset(RY1, 0, sizeof(double) * (size_t)(ynum * (xnum + 1)));
  memset(RC1, 0, sizeof(double) * (size_t)((ynum - 1) * (xnum - 1)));
  const int64_t yv = ynum, yp = ynum - 1, yx = ynum + 1;
  for (int64_t j = 2; j <= xnum; ++j)
    for (int64_t i = 2; i <= ynum; ++i) {
      if (i == ynum) continue;  /* Domain.basic_node_along_lower_boundary */
      double r;
      if (stab == 1) r = -gravity_y * A2(rho1_vy, yv, i, j);
      else r = -gravity_y * (A2(rho1, ynum, i, j) + A2(rho1, ynum, i, j - 1)) / 2;
      r += (A2(sxx0, yp, i, j - 1) - A2(sxx0, yp, i - 1, j - 1)) / ystp_vx[i - 1];
      r -= (A2(sxy0, ynum, i, j) - A2(sxy0, ynum, i, j - 1)) / xstp_b[j - 2];
      A2(RY1, yv, i, j) = r;
    }
  for (int64_t j = 2; j <= xnum; ++j)
    for (int64_t i = 2; i <= ynum; ++i) {
      if (j == xnum) continue;  /* Domain.basic_node_on_right_boundary */
      double r = -gravity_x * (A2(rho1, ynum, i, j) + A2(rho1, ynum, i - 1, j)) / 2;
      r -= (A2(sxx0, yp, i - 1, j) - A2(sxx0, yp, i - 1, j - 1)) / xstp_vy[j - 1];
      r -= (A2(sxy0, ynum, i, j) - A2(sxy0, ynum, i - 1, j)) / ystp_b[i - 2];
      A2(RX1, yx, i, j) = r;
    }
  for (int64_t j = 1; j <= xnum - 1; ++j)
    for (int64_t i = 1; i <= ynum - 1; ++i) {
      /* calc_plastic_volumetric_effect (:184-190) */
      const double rad = A2(dilatation_grid, yp, i, j) * O_PI / 180.0;
      A2(RC1, yp, i, j) = 2.0 * sin(rad) * A2(eii_plastic_pressure, yp, i, j);
    }
}

/* Everything the system build reads (BuildStructs.jl: GridData, BCData, RhsData, StokesBuildData). */
typedef struct {
  int64_t xnum, ynum;
  double xstpavg, ystpavg;
  const double *xstp, *ystp, *xstpc, *ystpc;      /* xstp_b, ystp_b, xstp_vy, ystp_vx */
  const double *btopx, *bbottomx;                 /* (xnum, 2)   */
  const double *btopy, *bbottomy;                 /* (xnum+1, 2) */
  const double *bleftx, *brightx;                 /* (ynum+1, 2) */
  const double *blefty, *brighty;                 /* (ynum, 2)   */
  const int64_t* bintern_zone;                    /* [8] */
  const double* bintern_velocity;                 /* [8] */
  int64_t pressure_bc_mode;
  double pressure_bc;
  double timestep, gravity_y;
  int64_t iuse_interface_stabilization;
  double pscale;
  const double *etan, *etas, *rho1_vy, *RX, *RY, *RC;
} o_stokes_in;

typedef struct { int64_t *Li, *Lj; double* Lv; double* R; int64_t n; } coo_t;

static int64_t emit(coo_t* c, int64_t row, int64_t col, double v) {
  c->Li[c->n] = row; c->Lj[c->n] = col; c->Lv[c->n] = v;
  return c->n++;
}

/* src/utils/Domain.jl:41-99 predicates */
static int along_upper(int64_t i) { return i == 1; }
static int along_lower(int64_t i, int64_t ynum) { return i >= ynum - 1; }
static int along_left(int64_t j) { return j == 1; }
static int along_right(int64_t j, int64_t xnum) { return j >= xnum - 1; }
static int last_two_right(int64_t j, int64_t xnum) { return j >= xnum - 2; }
static int last_two_bottom(int64_t i, int64_t ynum) { return i >= ynum - 2; }
static int outside_zone_x(int64_t i, int64_t j, const int64_t* z) { return j != z[0] || i < z[1] || i > z[2]; }
static int outside_zone_y(int64_t i, int64_t j, const int64_t* z) { return j != z[4] || i < z[5] || i > z[6]; }

#define ETAN(i, j) A2(s->etan, s->ynum - 1, i, j)
#define ETAS(i, j) A2(s->etas, s->ynum, i, j)
#define RHOVY(i, j) A2(s->rho1_vy, s->ynum, i, j)
#define BX(a, k, c) A2(s->a, s->xnum, k, c)        /* btopx, bbottomx */
#define BX1(a, k, c) A2(s->a, s->xnum + 1, k, c)   /* btopy, bbottomy */
#define BY1(a, k, c) A2(s->a, s->ynum + 1, k, c)   /* bleftx, brightx */
#define BY(a, k, c) A2(s->a, s->ynum, k, c)        /* blefty, brighty */

/* x-Stokes equation of cell (i, j): discretize_x_stokes_equation/StencilForVxStokesUnknown.jl,
 * internal/InternalCells.jl:46-75 and internal/stencil_nodes/*.jl, boundary/BoundaryCells.jl:64-95. */
static void x_stokes(const o_stokes_in* s, coo_t* c, int64_t i, int64_t j, int64_t ivx, int64_t hs) {
  const double *xstp = s->xstp, *ystp = s->ystp, *xstpc = s->xstpc, *ystpc = s->ystpc;
  double* R = c->R;
  if (!(j < s->xnum - 1 && outside_zone_x(i, j, s->bintern_zone))) {
    emit(c, ivx, ivx, 2.0 * s->pscale / (s->xstpavg + s->ystpavg));
    R[ivx - 1] = outside_zone_x(i, j, s->bintern_zone)
                     ? 0.0 : 2.0 * s->pscale / (s->xstpavg + s->ystpavg) * s->bintern_velocity[3];
    return;
  }
  /* CentralVelocityXNode.jl:6-45 */
  const int64_t ic = emit(c, ivx, ivx,
      -2.0 * (ETAN(i, j + 1) / xstp[j] + ETAN(i, j) / xstp[j - 1]) / xstpc[j] -
      (ETAS(i + 1, j + 1) / ystpc[i] + ETAS(i, j + 1) / ystpc[i - 1]) / ystp[i - 1]);
  R[ivx - 1] = A2(s->RX, s->ynum + 1, i + 1, j + 1);
  /* LeftVelocityXNode.jl:7-79 */
  if (!along_left(j)) {
    emit(c, ivx, ivx - hs, 2.0 * ETAN(i, j) / xstp[j - 1] / xstpc[j]);
  } else {
    c->Lv[ic] = c->Lv[ic] + BY1(bleftx, i + 1, 2) * 2.0 * ETAN(i, j) / xstp[j - 1] / xstpc[j];
    R[ivx - 1] = R[ivx - 1] - BY1(bleftx, i + 1, 1) * 2.0 * ETAN(i, j) / xstp[j - 1] / xstpc[j];
  }
  /* RightVelocityXNode.jl:7-59 */
  if (!last_two_right(j, s->xnum)) {
    emit(c, ivx, ivx + hs, 2.0 * ETAN(i, j + 1) / xstp[j] / xstpc[j]);
  } else {
    c->Lv[ic] = c->Lv[ic] + BY1(brightx, i + 1, 2) * 2.0 * ETAN(i, j + 1) / xstp[j] / xstpc[j];
    R[ivx - 1] = R[ivx - 1] - BY1(brightx, i + 1, 1) * 2.0 * ETAN(i, j + 1) / xstp[j] / xstpc[j];
  }
  /* UpperVelocityXNode.jl:7-52 */
  if (!along_upper(i)) {
    emit(c, ivx, ivx - 3, ETAS(i, j + 1) / ystpc[i - 1] / ystp[i - 1]);
  } else {
    c->Lv[ic] = c->Lv[ic] + BX(btopx, j + 1, 2) * ETAS(i, j + 1) / ystpc[i - 1] / ystp[i - 1];
    R[ivx - 1] = R[ivx - 1] - BX(btopx, j + 1, 1) * ETAS(i, j + 1) / ystpc[i - 1] / ystp[i - 1];
  }
  /* BottomVelocityXNode.jl:7-52 */
  if (!along_lower(i, s->ynum)) {
    emit(c, ivx, ivx + 3, ETAS(i + 1, j + 1) / ystpc[i] / ystp[i - 1]);
  } else {
    c->Lv[ic] = c->Lv[ic] + BX(bbottomx, j + 1, 2) * ETAS(i + 1, j + 1) / ystpc[i] / ystp[i - 1];
    R[ivx - 1] = R[ivx - 1] - BX(bbottomx, j + 1, 1) * ETAS(i + 1, j + 1) / ystpc[i] / ystp[i - 1];
  }
  /* UpperLeftVelocityYNode.jl:7-64 */
  int64_t iUL = -1, iLL = -1, iUR = -1, iLR = -1;
  if (!along_upper(i)) {
    iUL = emit(c, ivx, ivx - 2, ETAS(i, j + 1) / xstpc[j] / ystp[i - 1]);
  } else {
    iLL = emit(c, ivx, ivx + 1, BX1(btopy, j + 1, 2) * ETAS(i, j + 1) / xstpc[j] / ystp[i - 1]);
    R[ivx - 1] = R[ivx - 1] - BX1(btopy, j + 1, 1) * ETAS(i, j + 1) / xstpc[j] / ystp[i - 1];
  }
  /* UpperRightVelocityYNode.jl:7-63 */
  if (!along_upper(i)) {
    iUR = emit(c, ivx, ivx - 2 + hs, -ETAS(i, j + 1) / xstpc[j] / ystp[i - 1]);
  } else {
    iLR = emit(c, ivx, ivx + 1 + hs, -BX1(btopy, j + 2, 2) * ETAS(i, j + 1) / xstpc[j] / ystp[i - 1]);
    R[ivx - 1] = R[ivx - 1] + BX1(btopy, j + 2, 1) * ETAS(i, j + 1) / xstpc[j] / ystp[i - 1];
  }
  /* BottomLeftVelocityYNode.jl:8-72 */
  if (!along_lower(i, s->ynum)) {
    if (!along_upper(i)) emit(c, ivx, ivx + 1, -ETAS(i + 1, j + 1) / xstpc[j] / ystp[i - 1]);
    else c->Lv[iLL] = c->Lv[iLL] - ETAS(i + 1, j + 1) / xstpc[j] / ystp[i - 1];
  } else {
    c->Lv[iUL] = c->Lv[iUL] - BX1(bbottomy, j + 1, 2) * ETAS(i + 1, j + 1) / xstpc[j] / ystp[i - 1];
    R[ivx - 1] = R[ivx - 1] + BX1(bbottomy, j + 1, 1) * ETAS(i + 1, j + 1) / xstpc[j] / ystp[i - 1];
  }
  /* BottomRightVelocityYNode.jl:8-67 */
  if (!along_lower(i, s->ynum)) {
    if (!along_upper(i)) emit(c, ivx, ivx + 1 + hs, ETAS(i + 1, j + 1) / xstpc[j] / ystp[i - 1]);
    else c->Lv[iLR] = c->Lv[iLR] + ETAS(i + 1, j + 1) / xstpc[j] / ystp[i - 1];
  } else {
    c->Lv[iUR] = c->Lv[iUR] + BX1(bbottomy, j + 2, 2) * ETAS(i + 1, j + 1) / xstpc[j] / ystp[i - 1];
    R[ivx - 1] = R[ivx - 1] - BX1(bbottomy, j + 2, 1) * ETAS(i + 1, j + 1) / xstpc[j] / ystp[i - 1];
  }
  /* LeftAndRightPressureNodes.jl:6-54 */
  emit(c, ivx, ivx + 2, s->pscale / xstpc[j]);
  emit(c, ivx, ivx + 2 + hs, -s->pscale / xstpc[j]);
}

/* y-Stokes equation of cell (i, j): discretize_y_stokes_equation/StencilForVyStokesUnknown.jl,
 * internal/InternalCells.jl:64-175 and internal/stencil_nodes/*.jl, boundary/BoundaryCells.jl:68-99. */
static void y_stokes(const o_stokes_in* s, coo_t* c, int64_t i, int64_t j, int64_t ivy, int64_t hs) {
  const double *xstp = s->xstp, *ystp = s->ystp, *xstpc = s->xstpc, *ystpc = s->ystpc;
  double* R = c->R;
  if (!(i < s->ynum - 1 && outside_zone_y(i, j, s->bintern_zone))) {
    emit(c, ivy, ivy, 2.0 * s->pscale / (s->xstpavg + s->ystpavg));
    R[ivy - 1] = outside_zone_y(i, j, s->bintern_zone)
                     ? 0.0 : 2.0 * s->pscale / (s->xstpavg + s->ystpavg) * s->bintern_velocity[7];
    return;
  }
  /* calculate_stabilization_terms (InternalCells.jl:104-175) */
  double dy = 0.0, dx = 0.0;
  if (s->iuse_interface_stabilization == 1) {
    const double drhody = ((RHOVY(i + 2, j + 1) - RHOVY(i + 1, j + 1)) / ystp[i] +
                           (RHOVY(i + 1, j + 1) - RHOVY(i, j + 1)) / ystp[i - 1]) / 2.0;
    dy = drhody * s->gravity_y * s->timestep;
    const double drhodx = ((RHOVY(i + 1, j + 2) - RHOVY(i + 1, j + 1)) / xstpc[j] +
                           (RHOVY(i + 1, j + 1) - RHOVY(i + 1, j)) / xstpc[j - 1]) / 2.0;
    dx = drhodx * s->gravity_y * s->timestep;
  }
  /* CentralVelocityYNode.jl:6-44 */
  const int64_t ic = emit(c, ivy, ivy,
      -2 * (ETAN(i + 1, j) / ystp[i] + ETAN(i, j) / ystp[i - 1]) / ystpc[i] -
      (ETAS(i + 1, j + 1) / xstpc[j] + ETAS(i + 1, j) / xstpc[j - 1]) / xstp[j - 1] - dy);
  R[ivy - 1] = A2(s->RY, s->ynum, i + 1, j + 1);
  /* UpperVelocityYNode.jl:7-51 */
  if (!along_upper(i)) {
    emit(c, ivy, ivy - 3, 2.0 * ETAN(i, j) / ystp[i - 1] / ystpc[i]);
  } else {
    c->Lv[ic] = c->Lv[ic] + BX1(btopy, j + 1, 2) * 2.0 * ETAN(i, j) / ystp[i - 1] / ystpc[i];
    R[ivy - 1] = R[ivy - 1] - BX1(btopy, j + 1, 1) * 2.0 * ETAN(i, j) / ystp[i - 1] / ystpc[i];
  }
  /* BottomVelocityYNode.jl:7-51 */
  if (!last_two_bottom(i, s->ynum)) {
    emit(c, ivy, ivy + 3, 2.0 * ETAN(i + 1, j) / ystp[i] / ystpc[i]);
  } else {
    c->Lv[ic] = c->Lv[ic] + BX1(bbottomy, j + 1, 2) * 2.0 * ETAN(i + 1, j) / ystp[i] / ystpc[i];
    R[ivy - 1] = R[ivy - 1] - BX1(bbottomy, j + 1, 1) * 2.0 * ETAN(i + 1, j) / ystp[i] / ystpc[i];
  }
  /* LeftVelocityYNode.jl:7-46 */
  if (!along_left(j)) {
    emit(c, ivy, ivy - hs, ETAS(i + 1, j) / xstpc[j - 1] / xstp[j - 1]);
  } else {
    c->Lv[ic] = c->Lv[ic] + BY(blefty, i + 1, 2) * ETAS(i + 1, j) / xstpc[j - 1] / xstp[j - 1];
    R[ivy - 1] = R[ivy - 1] - BY(blefty, i + 1, 1) * ETAS(i + 1, j) / xstpc[j - 1] / xstp[j - 1];
  }
  /* RightVelocityYNode.jl:7-47 */
  if (!along_right(j, s->xnum)) {
    emit(c, ivy, ivy + hs, ETAS(i + 1, j + 1) / xstpc[j] / xstp[j - 1]);
  } else {
    c->Lv[ic] += BY(brighty, i + 1, 2) * ETAS(i + 1, j + 1) / xstpc[j] / xstp[j - 1];
    R[ivy - 1] -= BY(brighty, i + 1, 1) * ETAS(i + 1, j + 1) / xstpc[j] / xstp[j - 1];
  }
  /* UpperLeftVelocityXNode.jl:7-78 */
  int64_t iUL = 0, iUR = 0, iLL = 0, iLR = 0;
  if (!along_left(j)) {
    iUL = emit(c, ivy, ivy - 1 - hs, ETAS(i + 1, j) / ystpc[i] / xstp[j - 1] - dx / 4.0);
  } else {
    iUR = emit(c, ivy, ivy - 1, BY1(bleftx, i + 1, 2) * (ETAS(i + 1, j) / ystpc[i] / xstp[j - 1] - dx / 4.0));
    R[ivy - 1] = R[ivy - 1] - BY1(bleftx, i + 1, 1) * (ETAS(i + 1, j) / ystpc[i] / xstp[j - 1] - dx / 4.0);
  }
  /* BottomLeftVelocityXNode.jl:7-77 */
  if (!along_left(j)) {
    iLL = emit(c, ivy, ivy + 2 - hs, -ETAS(i + 1, j) / ystpc[i] / xstp[j - 1] - dx / 4.0);
  } else {
    iLR = emit(c, ivy, ivy + 2, BY1(bleftx, i + 2, 2) * (-ETAS(i + 1, j) / ystpc[i] / xstp[j - 1] - dx / 4.0));
    R[ivy - 1] = R[ivy - 1] - BY1(bleftx, i + 2, 1) * (-ETAS(i + 1, j) / ystpc[i] / xstp[j - 1] - dx / 4.0);
  }
  /* UpperRightVelocityXNode.jl:8-80 */
  if (!along_right(j, s->xnum)) {
    if (!along_left(j)) emit(c, ivy, ivy - 1, -ETAS(i + 1, j + 1) / ystpc[i] / xstp[j - 1] - dx / 4.0);
    else c->Lv[iUR] = c->Lv[iUR] - ETAS(i + 1, j + 1) / ystpc[i] / xstp[j - 1] - dx / 4.0;
  } else {
    c->Lv[iUL] = c->Lv[iUL] + BY1(brightx, i + 1, 2) * (-ETAS(i + 1, j + 1) / ystpc[i] / xstp[j - 1] - dx / 4.0);
    R[ivy - 1] = R[ivy - 1] - BY1(brightx, i + 1, 1) * (-ETAS(i + 1, j + 1) / ystpc[i] / xstp[j - 1] - dx / 4.0);
  }
  /* BottomRightVelocityXNode.jl:8-80 */
  if (!along_right(j, s->xnum)) {
    if (!along_left(j)) emit(c, ivy, ivy + 2, ETAS(i + 1, j + 1) / ystpc[i] / xstp[j - 1] - dx / 4.0);
    else c->Lv[iLR] = c->Lv[iLR] + ETAS(i + 1, j + 1) / ystpc[i] / xstp[j - 1] - dx / 4.0;
  } else {
    c->Lv[iLL] = c->Lv[iLL] + BY1(brightx, i + 2, 2) * (ETAS(i + 1, j + 1) / ystpc[i] / xstp[j - 1] - dx / 4.0);
    R[ivy - 1] = R[ivy - 1] - BY1(brightx, i + 2, 1) * (ETAS(i + 1, j + 1) / ystpc[i] / xstp[j - 1] - dx / 4.0);
  }
  /* UpperAndLowerPressureNodes.jl:6-43 */
  emit(c, ivy, ivy + 1, s->pscale / ystpc[i]);
  emit(c, ivy, ivy + 4, -s->pscale / ystpc[i]);
}

/* Continuity equation of cell (i, j): discretize_continuity_equation/StencilForPContinuityUnknown.jl:31-52,
 * internal/InternalCells.jl:38-57 with stencil_nodes/*.jl, boundary/BoundaryCells.jl:36-203. */
static void continuity(const o_stokes_in* s, coo_t* c, int64_t i, int64_t j, int64_t ipr, int64_t hs) {
  const double *xstp = s->xstp, *ystp = s->ystp, ps = s->pscale;
  double* R = c->R;
  int internal;
  switch (s->pressure_bc_mode) {  /* Domain.found_internal_cell_continuity */
    case 0: internal = (j > 1 || i > 1); break;
    case 1: internal = (1 < i && i < s->ynum - 1); break;
    case 2: internal = (1 < j && j < s->xnum - 1); break;
    default: internal = 0;
  }
  if (!internal) {
    const double diag = 2.0 * ps / (s->xstpavg + s->ystpavg);
    const double rhs = 2.0 * s->pressure_bc / (s->xstpavg + s->ystpavg);
    if (s->pressure_bc_mode == 0) {
      emit(c, ipr, ipr, diag);
      R[ipr - 1] = rhs;
    } else if (s->pressure_bc_mode == 1) {
      emit(c, ipr, ipr, diag);
      R[ipr - 1] = along_upper(i) ? rhs : 0.0;
    } else if (s->pressure_bc_mode == 2) {
      emit(c, ipr, ipr, diag);
      R[ipr - 1] = along_left(j) ? rhs : 0.0;
    }
    return;
  }
  R[ipr - 1] = A2(s->RC, s->ynum - 1, i, j) * ps;
  /* LeftVelocityXNode.jl:8-46 */
  if (!along_left(j)) {
    const int64_t k = emit(c, ipr, ipr - 2 - hs, -ps / xstp[j - 1]);
    if (along_right(j, s->xnum)) {
      c->Lv[k] = c->Lv[k] + BY1(brightx, i + 1, 2) * ps / xstp[j - 1];
      R[ipr - 1] = R[ipr - 1] - BY1(brightx, i + 1, 1) * ps / xstp[j - 1];
    }
  }
  /* RightVelocityXNode.jl:8-45 */
  if (!along_right(j, s->xnum)) {
    const int64_t k = emit(c, ipr, ipr - 2, ps / xstp[j - 1]);
    if (along_left(j)) {
      c->Lv[k] = c->Lv[k] - BY1(bleftx, i + 1, 2) * ps / xstp[j - 1];
      R[ipr - 1] = R[ipr - 1] + BY1(bleftx, i + 1, 1) * ps / xstp[j - 1];
    }
  }
  /* UpperVelocityYNode.jl:8-50 */
  if (!along_upper(i)) {
    const int64_t k = emit(c, ipr, ipr - 4, -ps / ystp[i - 1]);
    if (along_lower(i, s->ynum)) {
      c->Lv[k] = c->Lv[k] + BX1(bbottomy, j + 1, 2) * ps / ystp[i - 1];
      R[ipr - 1] = R[ipr - 1] - BX1(bbottomy, j + 1, 1) * ps / ystp[i - 1];
    }
  }
  /* BottomVelocityYNode.jl:8-44 */
  if (!along_lower(i, s->ynum)) {
    const int64_t k = emit(c, ipr, ipr - 1, ps / ystp[i - 1]);
    if (along_upper(i)) {
      c->Lv[k] = c->Lv[k] - BX1(btopy, j + 1, 2) * ps / ystp[i - 1];
      R[ipr - 1] = R[ipr - 1] + BX1(btopy, j + 1, 1) * ps / ystp[i - 1];
    }
  }
}

/* StokesBuildManager.build_system_of_equations (:661-712): cells visited row by
 * row (i outer, j inner); per cell the x-Stokes, y-Stokes and continuity rows.
 * Li/Lj/Lv need room for 26 entries per cell; R has 3 (ynum-1)(xnum-1) entries.
 * Returns the number of entries (the reference's inz - 1). */
int64_t o_build_system(const o_stokes_in* s, int64_t* Li, int64_t* Lj, double* Lv, double* R) {
  coo_t c = {Li, Lj, Lv, R, 0};
  const int64_t ny = s->ynum - 1;
  const int64_t hs = 3 * ny;  /* hshift_to_vxR */
  for (int64_t i = 1; i <= s->ynum - 1; ++i)
    for (int64_t j = 1; j <= s->xnum - 1; ++j) {
      const int64_t cell = (j - 1) * ny + i;  /* GlobalIndices.jl:13-27 */
      const int64_t ivx = cell * 3 - 2, ivy = ivx + 1, ipr = ivx + 2;
      x_stokes(s, &c, i, j, ivx, hs);
      y_stokes(s, &c, i, j, ivy, hs);
      continuity(s, &c, i, j, ipr, hs);
    }
  return c.n;
}

/* StokesResiduals.stokes_calc_nonlinear_system_residual_optimized! (:63-81):
 * work = L x (COO order), minus R, absolute value. */
void o_coo_residual(int64_t nnz, const int64_t* Li, const int64_t* Lj, const double* Lv, const double* x,
                    const double* R, int64_t N, double* work, double* resnl) {
  for (int64_t k = 0; k < N; ++k) work[k] = 0.0;
  for (int64_t k = 0; k < nnz; ++k) work[Li[k] - 1] += Lv[k] * x[Lj[k] - 1];
  for (int64_t k = 0; k < N; ++k) {
    work[k] -= R[k];
    resnl[k] = fabs(work[k]);
  }
}

/* SystemSolver.reload_solu_vel! (:188-235) then apply_vel_bc! (:237-271). */
void o_process_stokes_solution(int64_t xnum, int64_t ynum, double pscale, const double* S,
                               const double* btopx, const double* bbottomx, const double* btopy,
                               const double* bbottomy, const double* bleftx, const double* brightx,
                               const double* blefty, const double* brighty,
                               double* vx1, double* vy1, double* pr1) {
  memset(vx1, 0, sizeof(double) * (size_t)((ynum + 1) * xnum));
  memset(vy1, 0, sizeof(double) * (size_t)(ynum * (xnum + 1)));
  memset(pr1, 0, sizeof(double) * (size_t)((ynum - 1) * (xnum - 1)));
  const int64_t ny = ynum - 1;
  for (int64_t j = 1; j <= xnum - 1; ++j)
    for (int64_t i = 1; i <= ynum - 1; ++i) {
      const int64_t cell = (j - 1) * ny + i;
      const int64_t ivx = cell * 3 - 2, ivy = ivx + 1, ipr = ivx + 2;
      if (j < xnum - 1) A2(vx1, ynum + 1, i + 1, j + 1) = S[ivx - 1];
      if (i < ynum - 1) A2(vy1, ynum, i + 1, j + 1) = S[ivy - 1];
      A2(pr1, ny, i, j) = S[ipr - 1] * pscale;
    }
  for (int64_t j = 1; j <= xnum; ++j) {
    A2(vx1, ynum + 1, 1, j) = A2(btopx, xnum, j, 1) + A2(btopx, xnum, j, 2) * A2(vx1, ynum + 1, 2, j);
    A2(vx1, ynum + 1, ynum + 1, j) = A2(bbottomx, xnum, j, 1) + A2(bbottomx, xnum, j, 2) * A2(vx1, ynum + 1, ynum, j);
  }
  for (int64_t j = 1; j <= xnum + 1; ++j) {
    A2(vy1, ynum, 1, j) = A2(btopy, xnum + 1, j, 1) + A2(btopy, xnum + 1, j, 2) * A2(vy1, ynum, 2, j);
    A2(vy1, ynum, ynum, j) = A2(bbottomy, xnum + 1, j, 1) + A2(bbottomy, xnum + 1, j, 2) * A2(vy1, ynum, ynum - 1, j);
  }
  for (int64_t i = 1; i <= ynum + 1; ++i) {
    A2(vx1, ynum + 1, i, 1) = A2(bleftx, ynum + 1, i, 1) + A2(bleftx, ynum + 1, i, 2) * A2(vx1, ynum + 1, i, 2);
    A2(vx1, ynum + 1, i, xnum) = A2(brightx, ynum + 1, i, 1) + A2(brightx, ynum + 1, i, 2) * A2(vx1, ynum + 1, i, xnum - 1);
  }
  for (int64_t i = 1; i <= ynum; ++i) {
    A2(vy1, ynum, i, 1) = A2(blefty, ynum, i, 1) + A2(blefty, ynum, i, 2) * A2(vy1, ynum, i, 2);
    A2(vy1, ynum, i, xnum + 1) = A2(brighty, ynum, i, 1) + A2(brighty, ynum, i, 2) * A2(vy1, ynum, i, xnum);
  }
}

/* ---- post-solve grid kernels (src/stokes_continuity_solver/utils/) ---------- */

/* GridStrainRate.update_grid_strain_rate_and_spin! (strain_rate/GridStrainRate.jl:6-182):
 * exx (ynum-1, xnum-1), exy (ynum, xnum), eii (ynum-1, xnum-1), esp (ynum, xnum). */
void o_grid_strain_rate_and_spin(int64_t xnum, int64_t ynum, const double* xstp_b, const double* ystp_b,
                                 const double* xstp_vy, const double* ystp_vx, const double* vx1,
                                 const double* vy1, double* exx, double* exy, double* eii, double* esp) {
  const int64_t yp = ynum - 1, yx = ynum + 1;
  memset(exx, 0, sizeof(double) * (size_t)(yp * (xnum - 1)));
  for (int64_t j = 1; j < xnum; ++j)
    for (int64_t i = 1; i < ynum; ++i)
      A2(exx, yp, i, j) = 0.5 * ((A2(vx1, yx, i + 1, j + 1) - A2(vx1, yx, i + 1, j)) / xstp_b[j - 1] -
                                 (A2(vy1, ynum, i + 1, j + 1) - A2(vy1, ynum, i, j + 1)) / ystp_b[i - 1]);
  for (int64_t j = 1; j <= xnum; ++j)
    for (int64_t i = 1; i <= ynum; ++i)
      A2(exy, ynum, i, j) = 0.5 * ((A2(vx1, yx, i + 1, j) - A2(vx1, yx, i, j)) / ystp_vx[i - 1] +
                                   (A2(vy1, ynum, i, j + 1) - A2(vy1, ynum, i, j)) / xstp_vy[j - 1]);
  memset(eii, 0, sizeof(double) * (size_t)(yp * (xnum - 1)));
  /* exx^2.0 etc.: Julia's x^2.0 is x*x */
  for (int64_t j = 2; j <= xnum; ++j)
    for (int64_t i = 2; i <= ynum; ++i) {
      const double e = A2(exx, yp, i - 1, j - 1);
      const double a = A2(exy, ynum, i - 1, j - 1), b = A2(exy, ynum, i, j - 1);
      const double c = A2(exy, ynum, i - 1, j), d = A2(exy, ynum, i, j);
      A2(eii, yp, i - 1, j - 1) = sqrt(e * e + (a * a + b * b + c * c + d * d) / 4.0);
    }
  for (int64_t j = 1; j <= xnum; ++j)
    for (int64_t i = 1; i <= ynum; ++i)
      A2(esp, ynum, i, j) = 0.5 * ((A2(vy1, ynum, i, j + 1) - A2(vy1, ynum, i, j)) / xstp_vy[j - 1] -
                                   (A2(vx1, yx, i + 1, j) - A2(vx1, yx, i, j)) / ystp_vx[i - 1]);
}

/* GridStress.forecast_viscoelastic_grid_stress! (GridStress.jl:30-126) and
 * calculate_deviatoric_grid_stress_change! (:128-134). */
void o_forecast_grid_stress(int64_t xnum, int64_t ynum, double dt, const double* etas1, const double* mus1,
                            const double* exy, const double* sxy1, const double* etan1, const double* mun1,
                            const double* exx, const double* sxx1, double* sxy2, double* sxx2, double* dsxy,
                            double* dsxx) {
  const int64_t nb = xnum * ynum, np = (xnum - 1) * (ynum - 1);
  for (int64_t k = 0; k < nb; ++k) {
    const double f = ve_factor(etas1[k], mus1[k], dt);
    sxy2[k] = (1.0 - f) * 2.0 * etas1[k] * exy[k] + f * sxy1[k];
  }
  for (int64_t k = 0; k < np; ++k) {
    const double f = ve_factor(etan1[k], mun1[k], dt);
    sxx2[k] = (1.0 - f) * 2.0 * etan1[k] * exx[k] + f * sxx1[k];
  }
  for (int64_t k = 0; k < nb; ++k) dsxy[k] = sxy2[k] - sxy1[k];
  for (int64_t k = 0; k < np; ++k) dsxx[k] = sxx2[k] - sxx1[k];
}

/* StokesInterpolate.interpolate_stag_velocity_to_basic_grid! (StokesInterpolate.jl:16-33). */
void o_stag_velocity_to_basic(int64_t xnum, int64_t ynum, const double* vx1, const double* vy1, double* vxb,
                              double* vyb) {
  for (int64_t j = 1; j <= xnum; ++j)
    for (int64_t i = 1; i <= ynum; ++i) {
      A2(vxb, ynum, i, j) = (A2(vx1, ynum + 1, i, j) + A2(vx1, ynum + 1, i + 1, j)) / 2.0;
      A2(vyb, ynum, i, j) = (A2(vy1, ynum, i, j) + A2(vy1, ynum, i, j + 1)) / 2.0;
    }
}

/* HarmonicAverage.normal_viscosity_from_harmonic_avg_shear_viscosity! (interpolation/utils/stokes_funcs/
 * HarmonicAverage.jl:20-51) with CheckPlasticYield.plastic_yielding (tolerance 0) and
 * MathTools.harmonic4 (zero factors): etan1 = 4 / sum(1 / etas1 corners) where the cell yields. */
void o_harmonic_normal_viscosity(int64_t xnum, int64_t ynum, const double* etas1, const double* plastics,
                                 const double* plasticn, const double* plastic_yield, double* etan1) {
  const int64_t yp = ynum - 1;
  for (int64_t i = 1; i <= ynum - 1; ++i)
    for (int64_t j = 1; j <= xnum - 1; ++j) {
      int yielding = A2(plasticn, yp, i, j) > 0.0;
      if (A2(plastics, ynum, i, j) > 0.0 || A2(plastics, ynum, i, j + 1) > 0.0 ||
          A2(plastics, ynum, i + 1, j) > 0.0 || A2(plastics, ynum, i + 1, j + 1) > 0.0) yielding = 1;
      if (A2(plastic_yield, ynum, i, j) > 0.0 || A2(plastic_yield, ynum, i, j + 1) > 0.0 ||
          A2(plastic_yield, ynum, i + 1, j) > 0.0 || A2(plastic_yield, ynum, i + 1, j + 1) > 0.0) yielding = 1;
      if (!yielding) continue;
      const double vinv = 1.0 / A2(etas1, ynum, i, j) + 1.0 / A2(etas1, ynum, i, j + 1) +
                          1.0 / A2(etas1, ynum, i + 1, j) + 1.0 / A2(etas1, ynum, i + 1, j + 1) + 0.0 + 0.0 + 0.0 + 0.0;
      if (vinv != 0.0) A2(etan1, yp, i, j) = 1.0 / (vinv / (4.0 + 0.0 + 0.0 + 0.0 + 0.0));
    }
}

/* ---- nodal Picard variant ---------------------------------------------------- */

/* PlasticFailureNodes.interpolate_from_pressure_grid_to_basic_grid (rheology/plastic_failure/nodes/
 * PlasticFailureNodes.jl:221-257): pressure-grid value at basic node (i, j). */
static double p_to_basic(int64_t i, int64_t j, int64_t ynum, int64_t xnum, const double* a) {
  const int64_t yp = ynum - 1;
  if (1 < i && i < ynum && 1 < j && j < xnum)
    return (A2(a, yp, i - 1, j - 1) + A2(a, yp, i, j - 1) + A2(a, yp, i - 1, j) + A2(a, yp, i, j)) / 4.0;
  if (i == 1 && j == 1) return A2(a, yp, i, j);
  if (i == ynum && j == 1) return A2(a, yp, i - 1, j);
  if (i == ynum && j == xnum) return A2(a, yp, i - 1, j - 1);
  if (i == 1 && j == xnum) return A2(a, yp, i, j - 1);
  if (j == 1) return (A2(a, yp, i, j) + A2(a, yp, i - 1, j)) / 2.0;
  if (j == xnum) return (A2(a, yp, i - 1, j - 1) + A2(a, yp, i, j - 1)) / 2.0;
  if (i == 1) return (A2(a, yp, i, j) + A2(a, yp, i, j - 1)) / 2.0;
  return (A2(a, yp, i - 1, j) + A2(a, yp, i - 1, j - 1)) / 2.0;  /* i == ynum */
}

typedef struct {
  int64_t ntimestep, iuse_fluid_pressure_for_yield, no_yielding_in_mobile_wall, no_yielding_in_plate_extension;
  double timestep, timesum, viscosity_min, viscosity_max, y_sealevel;
  double velocity_internal_x, x_left_mobile_wall, x_right_mobile_wall, y_top_mobile_wall, y_bottom_mobile_wall;
  double plate_extension_thickness, plate_extension_width;
} o_nodal_yield_in;

/* PlasticFailureNodes.update_nodes_for_plastic_yielding (PlasticFailureNodes.jl:24-184) with
 * CheckYield.check_yield_is_applicable, MobileWall.in_mobile_wall_transient /
 * in_plate_extension_transient (src/utils/MobileWall.jl), YieldStress.calc_yield_stress
 * (utils/YieldStress.jl:28-67, tension method 2) and the helpers :186-318.
 * viscosity_weight_factor is 0, so the weighted viscosity is the new one.
 * Returns nnode_yield; *gerr = sqrt(sum err^2 / nnode_yield) (0 when none). */
int64_t o_nodal_plastic_yielding(const o_nodal_yield_in* q, int64_t xnum, int64_t ynum, const double* gridx,
                                 const double* gridy, const double* plastic_yield, const double* etas1,
                                 const double* eta_flow, const double* mus1, const double* cohesion_grid,
                                 const double* fric_degrees_grid, const double* sxy2, const double* sxx2,
                                 const double* pr1, double* yield_error, double* etavp_new,
                                 double* plastic_strain_rate, double* plastic_yield_new, double* gerr) {
  const double pi_term = O_PI / 180.0;
  int64_t nnode = 0;
  double esum = 0.0;
  for (int64_t j = 1; j <= xnum; ++j)
    for (int64_t i = 1; i <= ynum; ++i) {
      const double vold = A2(etas1, ynum, i, j), vflow = A2(eta_flow, ynum, i, j), mu = A2(mus1, ynum, i, j);
      const double coh = A2(cohesion_grid, ynum, i, j);
      const double fc = sin(A2(fric_degrees_grid, ynum, i, j) * pi_term);
      A2(etavp_new, ynum, i, j) = vflow;
      A2(plastic_yield_new, ynum, i, j) = 0.0;
      A2(plastic_strain_rate, ynum, i, j) = 0.0;
      int applicable = q->ntimestep > 0 && (coh > 0.0 || fc > 0.0);
      const double xs = q->velocity_internal_x * q->timesum;
      if (q->no_yielding_in_mobile_wall) {
        const double xl = q->x_left_mobile_wall + xs, xr = q->x_right_mobile_wall + xs;
        if (xl <= gridx[j - 1] && gridx[j - 1] <= xr && q->y_top_mobile_wall <= gridy[i - 1] &&
            gridy[i - 1] <= q->y_bottom_mobile_wall)
          applicable = 0;
      }
      if (q->no_yielding_in_plate_extension) {
        const double xl = q->x_left_mobile_wall + xs;
        const double xmin = xl - q->plate_extension_width, ymin = q->y_bottom_mobile_wall - q->plate_extension_thickness;
        if (xmin <= gridx[j - 1] && gridx[j - 1] <= xl && ymin <= gridy[i - 1] && gridy[i - 1] <= q->y_bottom_mobile_wall)
          applicable = 0;
      }
      if (!applicable) continue;
      const double p = p_to_basic(i, j, ynum, xnum, pr1);
      const double sxx = p_to_basic(i, j, ynum, xnum, sxx2), sxy = A2(sxy2, ynum, i, j);
      const double sii = sqrt(sxy * sxy + sxx * sxx);
      const double sie = sii * (mu * q->timestep + vold) / vold;
      const double cphi = cos(asin(fc));
      double sy;
      if (q->iuse_fluid_pressure_for_yield == 0) {
        sy = coh * cphi + fc * p;
      } else {
        double depth = gridy[i - 1] - q->y_sealevel;
        if (depth < 0.0) depth = 0.0;
        const double pf = 1000.0 * 9.81 * depth;
        sy = (p < pf) ? coh * cphi : coh * cphi + fc * (p - pf);
      }
      if (sy < 0.0) sy = 0.0;
      const int at_yield = A2(plastic_yield, ynum, i, j) > 0;
      if (at_yield) {
        const double err = sii - sy;
        esum = esum + err * err;
        A2(yield_error, ynum, i, j) = err;
        ++nnode;
      }
      if (sy < sie) {
        double vnew = q->timestep * mu * sy / (sie - sy);
        if (vnew < vflow) {
          A2(plastic_yield_new, ynum, i, j) = 1.0;
          vnew = pow(vnew, 1.0 - 0.0) * pow(vold, 0.0);
          vnew = vnew > q->viscosity_min ? vnew : q->viscosity_min;
          vnew = vnew < q->viscosity_max ? vnew : q->viscosity_max;
          A2(etavp_new, ynum, i, j) = vnew;
          A2(plastic_strain_rate, ynum, i, j) = 0.5 * sii / vnew - 0.5 * sii / vflow;
          if (!at_yield) {
            const double err = sii - sy;
            esum = esum + err * err;
            A2(yield_error, ynum, i, j) = err;
            ++nnode;
          }
        }
      }
    }
  *gerr = nnode > 0 ? sqrt(esum / (double)nnode) : 0.0;
  return nnode;
}
