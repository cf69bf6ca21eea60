/*
 * mic_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY) for the marker-in-cell hot path.
 *
 * A plain-C, FP64, single-threaded restatement of the reference EarthBox.jl
 * functions on the per-timestep marker path.  It exists to check the CUDA
 * implementation: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it.  It is never part of the shipped product path.
 *
 * Fidelity rules
 *   - every loop over markers runs in increasing marker index, like the
 *     reference's serial scatters, so every grid sum is accumulated in the
 *     reference's order;
 *   - it is compiled with -ffp-contract=off and without fast-math, so
 *     a*b+c is never fused (Julia does not contract these expressions);
 *   - arrays use the reference's layout: column-major (rows, cols) grids,
 *     1-based Int32 cell indices, 1-based material ids.
 * Each function names the reference file:line it restates (paths relative to
 * the EarthBox.jl source tree).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Loops the reference runs with Threads.@threads carry "#pragma omp parallel for"
 * here; the scatter loops stay serial, as in the reference.  Each threaded loop
 * is independent per marker (or per grid column), so results do not depend on
 * the thread count. */
#define OMP_FOR _Pragma("omp parallel for schedule(static)")

int o_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

#define IDX(i, j, rows) ((size_t)((j) - 1) * (size_t)(rows) + (size_t)((i) - 1))
#define MAT(tab, nmat, m, k) ((tab)[(size_t)((k) - 1) * (size_t)(nmat) + (size_t)((m) - 1)])

static const double PA_TO_MPA = 1.0 / 1e6;

/* Julia's Float64^Float64 for the exponents used on this path: an integral 2
 * (compensated power-by-squaring rounds to fl(x*x)), 3 (Base.Math.pow_body
 * returns x*x*x) and 1; any other exponent goes to libm pow (both are
 * faithfully rounded, so the two can differ in the last bit). */
static inline double jl_pow(double x, double y) {
  if (y == 2.0) return x * x;
  if (y == 3.0) return x * x * x;
  if (y == 1.0) return x;
  return pow(x, y);
}

/* ---------------------------------------------------------------- mapping -- */

/* Julia searchsortedlast(v, x): index of the last element <= x, 0 if none. */
static int64_t searchsortedlast(const double* v, int64_t n, double x) {
  int64_t lo = 0, hi = n + 1; /* invariant: v[lo] <= x < v[hi] (1-based, sentinels) */
  while (hi - lo > 1) {
    int64_t mid = lo + ((hi - lo) >> 1);
    if (x < v[mid - 1]) hi = mid; else lo = mid;
  }
  return lo;
}

/* MarkerGridMapping.get_index_of_left_node (src/interpolation/mapping/MarkerGridMapping.jl:78-86) */
int32_t o_index_of_left_node(double x, const double* grid, int64_t n) {
  int64_t i = searchsortedlast(grid, n, x);
  if (i < 1) i = 1;
  if (i > n - 1) i = n - 1;
  return (int32_t)i;
}

/* GridFuncs.get_marker_inside_flags (src/utils/GridFuncs.jl:54-80) */
void o_inside_flags(int64_t M, const double* x, const double* y, double xmin, double xmax,
                    double ymin, double ymax, int8_t* flags) {
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    int in = xmin <= x[m] && x[m] <= xmax && ymin <= y[m] && y[m] <= ymax;
    flags[m] = in ? 1 : -1;
  }
}

/* calc_upper_left_basic_grid_cell_indices_for_markers! (MarkerGridMapping.jl:99-129),
 * calc_upper_left_vy_grid_cell_indices_for_markers!    (MarkerGridMapping.jl:142-173),
 * calc_normalized_distances_from_upper_left_basic_node! (MarkerGridMapping.jl:185-219),
 * calc_normalized_distances_from_upper_left_vy_node!    (MarkerGridMapping.jl:231-265),
 * MarkerGridNodeWeights.calc_marker_weights_for_basic_and_pressure_grids! (MarkerGridNodeWeights.jl:68-101),
 * MarkerGridNodeWeights.calc_marker_weights_for_vy_grid! (MarkerGridNodeWeights.jl:122-150).
 * w: 9 arrays of M: UL, LL, UR, LR, C (basic) and UL, LL, UR, LR (vy). */
void o_locate_and_weights(int64_t M, const int8_t* flags, const double* x, const double* y,
                          int64_t xnum, int64_t ynum, const double* gridx_b, const double* gridy_b,
                          const double* xstp_b, const double* ystp_b, const double* gridx_vy,
                          const double* xstp_vy, int32_t* xn, int32_t* yn, int32_t* xn_vy,
                          int32_t* yn_vy, double* dx, double* dy, double* dx_vy, double* dy_vy,
                          double* wUL, double* wLL, double* wUR, double* wLR, double* wC,
                          double* wULvy, double* wLLvy, double* wURvy, double* wLRvy) {
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    xn[m] = o_index_of_left_node(x[m], gridx_b, xnum);
    yn[m] = o_index_of_left_node(y[m], gridy_b, ynum);
  }
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    dx[m] = (x[m] - gridx_b[xn[m] - 1]) / xstp_b[xn[m] - 1];
    dy[m] = (y[m] - gridy_b[yn[m] - 1]) / ystp_b[yn[m] - 1];
  }
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    double a = dx[m], b = dy[m];
    wUL[m] = (1.0 - a) * (1.0 - b);
    wLL[m] = (1.0 - a) * b;
    wUR[m] = a * (1.0 - b);
    wLR[m] = a * b;
    wC[m] = (1.0 - fabs(0.5 - a)) * (1.0 - fabs(0.5 - b));
  }
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    xn_vy[m] = o_index_of_left_node(x[m], gridx_vy, xnum + 1);
    yn_vy[m] = o_index_of_left_node(y[m], gridy_b, ynum);
  }
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    dx_vy[m] = (x[m] - gridx_vy[xn_vy[m] - 1]) / xstp_vy[xn_vy[m] - 1];
    dy_vy[m] = (y[m] - gridy_b[yn_vy[m] - 1]) / ystp_b[yn_vy[m] - 1];
  }
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    double a = dx_vy[m], b = dy_vy[m];
    wULvy[m] = (1.0 - a) * (1.0 - b);
    wLLvy[m] = (1.0 - a) * b;
    wURvy[m] = a * (1.0 - b);
    wLRvy[m] = a * b;
  }
}

/* ---------------------------------------------------------- weight updates -- */

/* WeightFuncs.update_weight_inclusive! (src/interpolation/weights/WeightFuncs.jl:67-90) */
static inline void upd_incl(double* g, int64_t rows, int32_t iy, int32_t ix, double wul, double wll,
                            double wur, double wlr, double s) {
  g[IDX(iy, ix, rows)] += wul * s * 1.0;
  g[IDX(iy + 1, ix, rows)] += wll * s * 1.0;
  g[IDX(iy, ix + 1, rows)] += wur * s * 1.0;
  g[IDX(iy + 1, ix + 1, rows)] += wlr * s * 1.0;
}

/* WeightFuncs.update_weight_exclusive! (WeightFuncs.jl:122-155) */
static inline void upd_excl(double* g, int64_t rows, int32_t iy, int32_t ix, double wul, double wll,
                            double wur, double wlr, double dx, double dy, double s) {
  if (dx <= 0.5 && dy <= 0.5) g[IDX(iy, ix, rows)] += wul * s * 1.0;
  if (dx <= 0.5 && 0.5 <= dy) g[IDX(iy + 1, ix, rows)] += wll * s * 1.0;
  if (dx >= 0.5 && 0.5 >= dy) g[IDX(iy, ix + 1, rows)] += wur * s * 1.0;
  if (dx >= 0.5 && dy >= 0.5) g[IDX(iy + 1, ix + 1, rows)] += wlr * s * 1.0;
}

/* WeightFuncs.update_weight_central! (WeightFuncs.jl:178-191) */
static inline void upd_cent(double* g, int64_t rows, int32_t iy, int32_t ix, double wc, double s) {
  g[IDX(iy, ix, rows)] += wc * s * 1.0;
}

/* BilinearDenominator.calc_marker_weight_sums_for_basic_and_pressure_nodes!
 *   (src/interpolation/initialize/utils/BilinearDenominator.jl:34-100) and
 * calc_marker_weight_sums_for_vy_nodes! (BilinearDenominator.jl:116-157), after
 * clear_marker_weight_sums_on_grids! (BilinearDenominator.jl:184). */
void o_denominators(int64_t M, const int8_t* flags, int64_t xnum, int64_t ynum, const int32_t* xn,
                    const int32_t* yn, const int32_t* xn_vy, const int32_t* yn_vy, const double* dx,
                    const double* dy, const double* wUL, const double* wLL, const double* wUR,
                    const double* wLR, const double* wC, const double* wULvy, const double* wLLvy,
                    const double* wURvy, const double* wLRvy, double* wtnodes, double* wtetas,
                    double* wtetan, double* wtnodes_vy) {
  memset(wtnodes, 0, sizeof(double) * ynum * xnum);
  memset(wtetas, 0, sizeof(double) * ynum * xnum);
  memset(wtetan, 0, sizeof(double) * (ynum - 1) * (xnum - 1));
  memset(wtnodes_vy, 0, sizeof(double) * ynum * (xnum + 1));
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    upd_incl(wtnodes, ynum, yn[m], xn[m], wUL[m], wLL[m], wUR[m], wLR[m], 1.0);
    upd_excl(wtetas, ynum, yn[m], xn[m], wUL[m], wLL[m], wUR[m], wLR[m], dx[m], dy[m], 1.0);
    upd_cent(wtetan, ynum - 1, yn[m], xn[m], wC[m], 1.0);
  }
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    upd_incl(wtnodes_vy, ynum, yn_vy[m], xn_vy[m], wULvy[m], wLLvy[m], wURvy[m], wLRvy[m], 1.0);
  }
}

/* ---------------------------------------------------------------- averages -- */

/* BilinearAverage.calc_bilinear_average_arithmetic! (src/interpolation/utils/BilinearAverage.jl:276-294) */
void o_average_arith(int64_t n, double* avg, const double* old, const double* wsum) {
  OMP_FOR
  for (int64_t k = 0; k < n; ++k) avg[k] = (wsum[k] != 0) ? avg[k] / wsum[k] : old[k];
}

/* BilinearAverage.calc_bilinear_average_harmonic! (BilinearAverage.jl:304-322) */
void o_average_harm(int64_t n, double* avg, const double* old, const double* wsum) {
  OMP_FOR
  for (int64_t k = 0; k < n; ++k) avg[k] = (wsum[k] != 0) ? 1.0 / (avg[k] / wsum[k]) : old[k];
}

/* ------------------------------------------------------------ stokes scatter */

/* Stokes transport grids, in the order of BackupTransportArrays.jl:45-66. */
typedef struct o_stokes_grids {
  double *rho1, *rho0, *rho1_vy, *rho0_vy;           /* B, B, VY, VY */
  double *etas1, *etas0, *eta_flow, *eta_flow0;      /* B */
  double *mus1, *mus0, *sxy1, *sxy0;                 /* B */
  double *plastics, *plastics0, *cohesion, *cohesion0, *fric, *fric0; /* B */
  double *etan1, *etan0, *mun1, *mun0, *sxx1, *sxx0; /* P */
  double *plasticn, *plasticn0, *dilat, *dilat0, *melt, *melt0; /* P */
} o_stokes_grids;

/* MarkersToStokesArrays.interpolate_markers_to_transport_arrays!
 *   (src/interpolation/utils/MarkersToStokesArrays.jl:39-45):
 *   backup_and_clear_stokes_arrays!     (BackupTransportArrays.jl:33-98)
 *   calc_marker_weight_sums_for_basic_and_pressure_grids_stokes! (BilinearNumerator.jl:205-392)
 *   calc_marker_weight_sums_for_vy_grid_stokes!                  (BilinearNumerator.jl:408-454)
 *   calc_marker_average_at_staggered_nodes_stokes!               (BilinearAverage.jl:57-178)
 *   flatten_staggered_grid_density_in_sticky_air_layer!          (FlattenDensity.jl:29-89)
 * Returns 0, or the 1-based marker index of a zero shear modulus (the
 * reference raises an error there, BilinearNumerator.jl:158-163). */
int64_t o_scatter_stokes(int64_t M, const int8_t* flags, int64_t xnum, int64_t ynum,
                         const int32_t* xn, const int32_t* yn, const int32_t* xn_vy,
                         const int32_t* yn_vy, const double* dx, const double* dy,
                         const double* wUL, const double* wLL, const double* wUR, const double* wLR,
                         const double* wC, const double* wULvy, const double* wLLvy,
                         const double* wURvy, const double* wLRvy, const double* wtnodes,
                         const double* wtetas, const double* wtetan, const double* wtnodes_vy,
                         const int16_t* matid, const double* mat_mu, const double* m_rho,
                         const double* m_cohesion, const double* m_fric, const double* m_eta,
                         const double* m_eta_flow, const double* m_sxx, const double* m_sxy,
                         const float* m_pfailure, const float* m_dilat, const double* m_melt,
                         o_stokes_grids* g, int64_t iuse_topo, const double* gridy_b,
                         const double* hr1, double y_sealevel, double rho_sticky_air,
                         double rho_sticky_water) {
  const int64_t nb = ynum * xnum, np = (ynum - 1) * (xnum - 1), nvy = ynum * (xnum + 1);
  const int64_t rp = ynum - 1;
  /* backup then clear */
  memcpy(g->etas0, g->etas1, sizeof(double) * nb);
  memcpy(g->etan0, g->etan1, sizeof(double) * np);
  memcpy(g->eta_flow0, g->eta_flow, sizeof(double) * nb);
  memcpy(g->mus0, g->mus1, sizeof(double) * nb);
  memcpy(g->mun0, g->mun1, sizeof(double) * np);
  memcpy(g->sxy0, g->sxy1, sizeof(double) * nb);
  memcpy(g->sxx0, g->sxx1, sizeof(double) * np);
  memcpy(g->rho0, g->rho1, sizeof(double) * nb);
  memcpy(g->rho0_vy, g->rho1_vy, sizeof(double) * nvy);
  memcpy(g->plastics0, g->plastics, sizeof(double) * nb);
  memcpy(g->plasticn0, g->plasticn, sizeof(double) * np);
  memcpy(g->cohesion0, g->cohesion, sizeof(double) * nb);
  memcpy(g->fric0, g->fric, sizeof(double) * nb);
  memcpy(g->dilat0, g->dilat, sizeof(double) * np);
  memcpy(g->melt0, g->melt, sizeof(double) * np);
  double* clr_b[] = {g->etas1, g->eta_flow, g->mus1, g->sxy1, g->rho1, g->cohesion, g->fric, g->plastics};
  double* clr_p[] = {g->etan1, g->mun1, g->sxx1, g->plasticn, g->dilat, g->melt};
  for (int k = 0; k < 8; ++k) memset(clr_b[k], 0, sizeof(double) * nb);
  for (int k = 0; k < 6; ++k) memset(clr_p[k], 0, sizeof(double) * np);
  memset(g->rho1_vy, 0, sizeof(double) * nvy);

  const double pi = 3.14159265358979323846;
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    int32_t ix = xn[m], iy = yn[m];
    double a = dx[m], b = dy[m];
    double ul = wUL[m], ll = wLL[m], ur = wUR[m], lr = wLR[m], c = wC[m];
    int mt = matid[m];
    double mrho = m_rho[m];
    double mcoh = m_cohesion[m];
    double mfric = asin(m_fric[m]) * 180.0 / pi;
    double meta_flow = m_eta_flow[m];
    double meta = m_eta[m];
    double mshear = mat_mu[mt - 1];
    if (mshear == 0.0) return m + 1;
    double mmu_inv = 1 / mshear;
    double msxy = m_sxy[m];
    double plastyn = (double)m_pfailure[m];
    double mdil = (double)m_dilat[m];
    double mmelt = m_melt[m];
    double msxx = m_sxx[m];
    upd_incl(g->rho1, ynum, iy, ix, ul, ll, ur, lr, mrho);
    upd_excl(g->cohesion, ynum, iy, ix, ul, ll, ur, lr, a, b, mcoh);
    upd_excl(g->fric, ynum, iy, ix, ul, ll, ur, lr, a, b, mfric);
    upd_excl(g->eta_flow, ynum, iy, ix, ul, ll, ur, lr, a, b, meta_flow);
    upd_excl(g->etas1, ynum, iy, ix, ul, ll, ur, lr, a, b, meta);
    upd_cent(g->etan1, rp, iy, ix, c, meta);
    upd_excl(g->mus1, ynum, iy, ix, ul, ll, ur, lr, a, b, mmu_inv);
    upd_cent(g->mun1, rp, iy, ix, c, mmu_inv);
    upd_excl(g->sxy1, ynum, iy, ix, ul, ll, ur, lr, a, b, msxy);
    upd_excl(g->plastics, ynum, iy, ix, ul, ll, ur, lr, a, b, plastyn);
    upd_cent(g->plasticn, rp, iy, ix, c, plastyn);
    upd_cent(g->dilat, rp, iy, ix, c, mdil);
    upd_cent(g->melt, rp, iy, ix, c, mmelt);
    upd_cent(g->sxx1, rp, iy, ix, c, msxx);
  }
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    upd_incl(g->rho1_vy, ynum, yn_vy[m], xn_vy[m], wULvy[m], wLLvy[m], wURvy[m], wLRvy[m], m_rho[m]);
  }
  /* averages, in the order of BilinearAverage.jl:57-178 */
  o_average_arith(nb, g->rho1, g->rho0, wtnodes);
  o_average_arith(nvy, g->rho1_vy, g->rho0_vy, wtnodes_vy);
  o_average_harm(nb, g->mus1, g->mus0, wtetas);
  o_average_arith(nb, g->etas1, g->etas0, wtetas);
  o_average_arith(nb, g->sxy1, g->sxy0, wtetas);
  o_average_arith(nb, g->plastics, g->plastics0, wtetas);
  o_average_arith(nb, g->cohesion, g->cohesion0, wtetas);
  o_average_arith(nb, g->fric, g->fric0, wtetas);
  o_average_arith(nb, g->eta_flow, g->eta_flow0, wtetas);
  o_average_harm(np, g->mun1, g->mun0, wtetan);
  o_average_arith(np, g->etan1, g->etan0, wtetan);
  o_average_arith(np, g->sxx1, g->sxx0, wtetan);
  o_average_arith(np, g->plasticn, g->plasticn0, wtetan);
  o_average_arith(np, g->dilat, g->dilat0, wtetan);
  o_average_arith(np, g->melt, g->melt0, wtetan);
  /* FlattenDensity.flatten_staggered_grid_density_in_sticky_air_layer! (FlattenDensity.jl:29-89);
   * rho_sticky_* < 0 means the material type is absent (matid == -1). */
  if (iuse_topo == 1) {
    for (int64_t j = 1; j <= xnum; ++j)
      for (int64_t i = 1; i <= ynum; ++i) {
        double* r = &g->rho1[IDX(i, j, ynum)];
        double h = hr1[IDX(i, j, ynum)];
        if (*r <= 1100.0 && gridy_b[i - 1] < y_sealevel && h == 0.0 && rho_sticky_air >= 0) *r = rho_sticky_air;
        if (*r <= 1100.0 && gridy_b[i - 1] >= y_sealevel && h == 0.0 && rho_sticky_water >= 0) *r = rho_sticky_water;
      }
    for (int64_t j = 1; j <= xnum + 1; ++j)
      for (int64_t i = 1; i <= ynum; ++i) {
        double* r = &g->rho1_vy[IDX(i, j, ynum)];
        if (*r <= 1100.0 && gridy_b[i - 1] < y_sealevel && rho_sticky_air >= 0) *r = rho_sticky_air;
        if (*r <= 1100.0 && gridy_b[i - 1] >= y_sealevel && rho_sticky_water >= 0) *r = rho_sticky_water;
      }
  }
  return 0;
}

/* -------------------------------------------------------------- heat scatter */

/* MarkerToHeatArrays.interpolate_markers_to_transport_arrays! (MarkerToHeatArrays.jl:29-35):
 *   backup_and_clear_heat_transport_arrays! (BackupTransportArrays.jl:144-179; tk0 <- tk2)
 *   calc_marker_weight_sums_for_basic_grid_heat! (BilinearNumerator.jl:31-141)
 *   calc_marker_average_at_basic_nodes_heat!     (BilinearAverage.jl:10-50)
 *   apply_thermal_bc_along_boundaries!           (ApplyThermalBC.jl:20-44) */
void o_scatter_heat(int64_t M, const int8_t* flags, int64_t xnum, int64_t ynum, const int32_t* xn,
                    const int32_t* yn, const double* wUL, const double* wLL, const double* wUR,
                    const double* wLR, const double* wtnodes, const int16_t* matid,
                    const double* mat_hr, const double* m_tk, const double* m_kt,
                    const double* m_rhocp, const double* m_ha, const double* m_serp_hr,
                    int64_t iuse_serp, double* tk1, double* tk0, const double* tk2, double* kt1,
                    double* kt0, double* rhocp1, double* rhocp0, double* hr1, double* hr0,
                    double* ha1, double* ha0, const double* btopt, const double* bbottomt,
                    const double* bleftt, const double* brightt) {
  const int64_t nb = ynum * xnum;
  memcpy(tk0, tk2, sizeof(double) * nb);
  memcpy(rhocp0, rhocp1, sizeof(double) * nb);
  memcpy(kt0, kt1, sizeof(double) * nb);
  memcpy(hr0, hr1, sizeof(double) * nb);
  memcpy(ha0, ha1, sizeof(double) * nb);
  double* clr[] = {tk1, rhocp1, kt1, hr1, ha1};
  for (int k = 0; k < 5; ++k) memset(clr[k], 0, sizeof(double) * nb);
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    int32_t ix = xn[m], iy = yn[m];
    double ul = wUL[m], ll = wLL[m], ur = wUR[m], lr = wLR[m];
    double hr = mat_hr[matid[m] - 1];
    upd_incl(tk1, ynum, iy, ix, ul, ll, ur, lr, m_tk[m]);
    upd_incl(kt1, ynum, iy, ix, ul, ll, ur, lr, m_kt[m]);
    upd_incl(rhocp1, ynum, iy, ix, ul, ll, ur, lr, m_rhocp[m]);
    double total = (iuse_serp == 1) ? hr + m_serp_hr[m] : hr;
    upd_incl(hr1, ynum, iy, ix, ul, ll, ur, lr, total);
    upd_incl(ha1, ynum, iy, ix, ul, ll, ur, lr, m_ha[m]);
  }
  o_average_arith(nb, tk1, tk0, wtnodes);
  o_average_arith(nb, kt1, kt0, wtnodes);
  o_average_arith(nb, rhocp1, rhocp0, wtnodes);
  o_average_arith(nb, hr1, hr0, wtnodes);
  o_average_arith(nb, ha1, ha0, wtnodes);
  for (int64_t j = 2; j <= xnum - 1; ++j) {
    tk1[IDX(1, j, ynum)] = btopt[IDX(j, 1, xnum)] + btopt[IDX(j, 2, xnum)] * tk1[IDX(2, j, ynum)];
    tk1[IDX(ynum, j, ynum)] =
        bbottomt[IDX(j, 1, xnum)] + bbottomt[IDX(j, 2, xnum)] * tk1[IDX(ynum - 1, j, ynum)];
  }
  for (int64_t i = 1; i <= ynum; ++i) {
    tk1[IDX(i, 1, ynum)] = bleftt[IDX(i, 1, ynum)] + bleftt[IDX(i, 2, ynum)] * tk1[IDX(i, 2, ynum)];
    tk1[IDX(i, xnum, ynum)] =
        brightt[IDX(i, 1, ynum)] + brightt[IDX(i, 2, ynum)] * tk1[IDX(i, xnum - 1, ynum)];
  }
}

/* --------------------------------------------------------- viscosity scatter */

/* BackupTransportArrays.backup_and_clear_viscosity_transport_arrays! (BackupTransportArrays.jl:105-137) */
void o_backup_clear_viscosity(int64_t xnum, int64_t ynum, double* etas1, double* etas0, double* etan1,
                              double* etan0) {
  const int64_t nb = ynum * xnum, np = (ynum - 1) * (xnum - 1);
  memcpy(etas0, etas1, sizeof(double) * nb);
  memcpy(etan0, etan1, sizeof(double) * np);
  memset(etas1, 0, sizeof(double) * nb);
  memset(etan1, 0, sizeof(double) * np);
}

/* MarkersToStokesArrays.interpolate_viscosity_to_transport_arrays! (MarkersToStokesArrays.jl:60-64):
 *   calc_marker_weight_sums_viscosity!        (BilinearNumerator.jl:470-533)
 *   calc_marker_average_at_nodes_viscosity!   (BilinearAverage.jl:213-227) */
void o_scatter_viscosity(int64_t M, const int8_t* flags, int64_t xnum, int64_t ynum,
                         const int32_t* xn, const int32_t* yn, const double* dx, const double* dy,
                         const double* wUL, const double* wLL, const double* wUR, const double* wLR,
                         const double* wC, const double* wtetas, const double* wtetan,
                         const double* m_eta, double* etas1, const double* etas0, double* etan1,
                         const double* etan0) {
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    upd_excl(etas1, ynum, yn[m], xn[m], wUL[m], wLL[m], wUR[m], wLR[m], dx[m], dy[m], m_eta[m]);
    upd_cent(etan1, ynum - 1, yn[m], xn[m], wC[m], m_eta[m]);
  }
  o_average_arith(ynum * xnum, etas1, etas0, wtetas);
  o_average_arith((ynum - 1) * (xnum - 1), etan1, etan0, wtetan);
}

/* ------------------------------------------------------------------ gathers -- */

/* GridToMarker.get_marker_value (src/interpolation/utils/GridToMarker.jl:190-226) */
static inline double get_marker_value(int32_t yn, int32_t xn, double dy, double dx, const double* g,
                                      int64_t rows) {
  double wul = (1.0 - dx) * (1.0 - dy);
  double wll = (1.0 - dx) * dy;
  double wur = dx * (1.0 - dy);
  double wlr = dx * dy;
  double v = 0.0;
  v += wul * g[IDX(yn, xn, rows)];
  v += wll * g[IDX(yn + 1, xn, rows)];
  v += wur * g[IDX(yn, xn + 1, rows)];
  v += wlr * g[IDX(yn + 1, xn + 1, rows)];
  return v;
}

/* MarkerGridMapping.upr_left_index_pressure (MarkerGridMapping.jl:311-331) */
static inline int32_t upr_left_index_pressure(int64_t nnodes, int32_t ibasic, double loc,
                                              const double* gstag) {
  int32_t ip = (loc < gstag[ibasic]) ? ibasic - 1 : ibasic; /* gstag[ibasic+1] 1-based */
  if (ip < 1) ip = 1;
  if (ip > (int32_t)(nnodes - 2)) ip = (int32_t)(nnodes - 2);
  return ip;
}

/* MarkerGridMapping.upr_left_dist_pressure (MarkerGridMapping.jl:339-350) */
static inline double upr_left_dist_pressure(int32_t ip, double loc, const double* gstag,
                                            const double* stp) {
  return (loc - gstag[ip]) / stp[ip]; /* gstag[ip+1], stp[ip+1] 1-based */
}

/* GridToMarker.get_marker_value_from_pressure_grid_array (GridToMarker.jl:104-153) */
static inline double pressure_value(int64_t xnum, int64_t ynum, int32_t iy, int32_t ix, double y,
                                    double x, const double* gridy_vx, const double* ystp_vx,
                                    const double* gridx_vy, const double* xstp_vy, const double* pg) {
  int32_t yp = upr_left_index_pressure(ynum, iy, y, gridy_vx);
  int32_t xp = upr_left_index_pressure(xnum, ix, x, gridx_vy);
  double dyp = upr_left_dist_pressure(yp, y, gridy_vx, ystp_vx);
  double dxp = upr_left_dist_pressure(xp, x, gridx_vy, xstp_vy);
  return get_marker_value(yp, xp, dyp, dxp, pg, ynum - 1);
}

/* GridTemperatureToMarkers.interpolate! (GridTemperatureToMarkers.jl:18-45) */
void o_temperature_to_markers(int64_t M, const int8_t* flags, int64_t ynum, const int32_t* xn,
                              const int32_t* yn, const double* dx, const double* dy, const double* tk1,
                              double* m_tk) {
  OMP_FOR
  for (int64_t m = 0; m < M; ++m)
    if (flags[m] == 1) m_tk[m] = get_marker_value(yn[m], xn[m], dy[m], dx[m], tk1, ynum);
}

/* MarkerStrainRate.calculate_marker_strain_rate! (utils/strain_rate/MarkerStrainRate.jl:23-69),
 * MarkerStrainRateRatio.calculate_marker_strain_rate_ratio! (MarkerStrainRateRatio.jl:191-322),
 * MarkerPressure.calculate_marker_pressure! (utils/MarkerPressure.jl:17-54), in the order of
 * StokesContinuitySolver.execute_post_stokes_solver_steps! (StokesContinuitySolver.jl:283-290). */
void o_post_stokes_gathers(int64_t M, const int8_t* flags, int64_t xnum, int64_t ynum,
                           const double* x, const double* y, const int32_t* xn, const int32_t* yn,
                           const double* dx, const double* dy, const double* gridy_vx,
                           const double* ystp_vx, const double* gridx_vy, const double* xstp_vy,
                           const double* exx, const double* exy, const double* sxx2,
                           const double* sxy2, const double* dsxx, const double* dsxy,
                           const double* pr1, const int16_t* matid, const double* mat_mu,
                           const double* m_eta, double timestep, double* m_exx, double* m_exy,
                           double* m_sr_ratio, double* m_pr) {
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    m_exx[m] = pressure_value(xnum, ynum, yn[m], xn[m], y[m], x[m], gridy_vx, ystp_vx, gridx_vy, xstp_vy, exx);
    m_exy[m] = get_marker_value(yn[m], xn[m], dy[m], dx[m], exy, ynum);
  }
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    double sxx_m = pressure_value(xnum, ynum, yn[m], xn[m], y[m], x[m], gridy_vx, ystp_vx, gridx_vy, xstp_vy, sxx2);
    double sxy_m = get_marker_value(yn[m], xn[m], dy[m], dx[m], sxy2, ynum);
    double dsxx_m = pressure_value(xnum, ynum, yn[m], xn[m], y[m], x[m], gridy_vx, ystp_vx, gridx_vy, xstp_vy, dsxx);
    double dsxy_m = get_marker_value(yn[m], xn[m], dy[m], dx[m], dsxy, ynum);
    double mu = mat_mu[matid[m] - 1];
    double eta = m_eta[m];
    double exx_m = m_exx[m], exy_m = m_exy[m];
    double eii = sqrt(exx_m * exx_m + exy_m * exy_m);
    double r;
    if (eii > 0) {
      double tf = 1.0 / (timestep * mu);
      double a = 0.5 * (sxx_m / eta + dsxx_m * tf);
      double b = 0.5 * (sxy_m / eta + dsxy_m * tf);
      r = sqrt(a * a + b * b) / eii;
    } else {
      r = 1.0;
    }
    m_sr_ratio[m] = r;
  }
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    m_pr[m] = pressure_value(xnum, ynum, yn[m], xn[m], y[m], x[m], gridy_vx, ystp_vx, gridx_vy, xstp_vy, pr1);
  }
}

/* SubGridStress.Update.update_subgrid_stress! (subgrid_stress/update/Update.jl:69-87):
 *   SubgridShearStress.subgrid_shear_stress_changes!  (SubgridShearStress.jl:27-96)
 *   SubgridNormalStress.subgrid_normal_stress_changes! (SubgridNormalStress.jl:27-89)
 *   DiffusionTerm.calculate_subgrid_stress_diffusion_term (DiffusionTerm.jl:14-29)
 *   BilinearAverage.calc_marker_average_subgrid_stress_change! (BilinearAverage.jl:234-251)
 *   RemainingStress.calculate_remaining_stress_change! (RemainingStress.jl:18-26) */
static inline double stress_diffusion_term(double eta, double mu, double dt, double coef) {
  double maxwell = eta / mu;
  double s = -coef * dt / maxwell;
  if (s < -30.0) s = -30.0;
  return 1.0 - exp(s);
}
void o_subgrid_stress(int64_t M, const int8_t* flags, int64_t xnum, int64_t ynum, const double* x,
                      const double* y, const int32_t* xn, const int32_t* yn, const double* dx,
                      const double* dy, const double* wUL, const double* wLL, const double* wUR,
                      const double* wLR, const double* wC, const double* gridy_vx,
                      const double* ystp_vx, const double* gridx_vy, const double* xstp_vy,
                      const int16_t* matid, const double* mat_mu, const double* m_eta,
                      double timestep, double coef, const double* sxy1, const double* sxx1,
                      double* m_sxy, double* m_sxx, double* dsxyn, double* dsxxn, double* wtetas,
                      double* wtetan, double* dsxy, double* dsxx) {
  const int64_t nb = ynum * xnum, np = (ynum - 1) * (xnum - 1);
  memset(dsxyn, 0, sizeof(double) * nb);
  memset(dsxxn, 0, sizeof(double) * np);
  memset(wtetas, 0, sizeof(double) * nb);
  memset(wtetan, 0, sizeof(double) * np);
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    double mu = mat_mu[matid[m] - 1];
    double sdt = stress_diffusion_term(m_eta[m], mu, timestep, coef);
    double from_grid = get_marker_value(yn[m], xn[m], dy[m], dx[m], sxy1, ynum);
    double relax = (from_grid - m_sxy[m]) * sdt;
    m_sxy[m] += relax;
    upd_excl(dsxyn, ynum, yn[m], xn[m], wUL[m], wLL[m], wUR[m], wLR[m], dx[m], dy[m], relax);
    upd_excl(wtetas, ynum, yn[m], xn[m], wUL[m], wLL[m], wUR[m], wLR[m], dx[m], dy[m], 1.0);
  }
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    double mu = mat_mu[matid[m] - 1];
    double sdt = stress_diffusion_term(m_eta[m], mu, timestep, coef);
    double from_grid = pressure_value(xnum, ynum, yn[m], xn[m], y[m], x[m], gridy_vx, ystp_vx, gridx_vy, xstp_vy, sxx1);
    double relax = (from_grid - m_sxx[m]) * sdt;
    m_sxx[m] += relax;
    upd_cent(dsxxn, ynum - 1, yn[m], xn[m], wC[m], relax);
    upd_cent(wtetan, ynum - 1, yn[m], xn[m], wC[m], 1.0);
  }
  /* average against a copy of itself: empty nodes keep their (zero) sum */
  for (int64_t k = 0; k < nb; ++k) if (wtetas[k] != 0) dsxyn[k] = dsxyn[k] / wtetas[k];
  for (int64_t k = 0; k < np; ++k) if (wtetan[k] != 0) dsxxn[k] = dsxxn[k] / wtetan[k];
  for (int64_t k = 0; k < nb; ++k) dsxy[k] = dsxy[k] - dsxyn[k];
  for (int64_t k = 0; k < np; ++k) dsxx[k] = dsxx[k] - dsxxn[k];
}

/* Exclusive (basic grid) and central (pressure grid) weighted averages of per-marker values,
 * with the weights of the scatters above; nodes without markers get 0.  Test-side error
 * scales (the average of |contribution| bounds the rounding of a weighted sum). */
void o_excl_cent_average(int64_t M, const int8_t* flags, int64_t xnum, int64_t ynum, const int32_t* xn,
                         const int32_t* yn, const double* dx, const double* dy, const double* wUL,
                         const double* wLL, const double* wUR, const double* wLR, const double* wC,
                         const double* v_excl, const double* v_cent, double* avg_excl, double* avg_cent) {
  const int64_t nb = ynum * xnum, np = (ynum - 1) * (xnum - 1);
  double* we = (double*)calloc((size_t)nb, sizeof(double));
  double* wc = (double*)calloc((size_t)np, sizeof(double));
  memset(avg_excl, 0, sizeof(double) * nb);
  memset(avg_cent, 0, sizeof(double) * np);
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    upd_excl(avg_excl, ynum, yn[m], xn[m], wUL[m], wLL[m], wUR[m], wLR[m], dx[m], dy[m], v_excl[m]);
    upd_excl(we, ynum, yn[m], xn[m], wUL[m], wLL[m], wUR[m], wLR[m], dx[m], dy[m], 1.0);
    upd_cent(avg_cent, ynum - 1, yn[m], xn[m], wC[m], v_cent[m]);
    upd_cent(wc, ynum - 1, yn[m], xn[m], wC[m], 1.0);
  }
  for (int64_t k = 0; k < nb; ++k) if (we[k] != 0) avg_excl[k] /= we[k];
  for (int64_t k = 0; k < np; ++k) if (wc[k] != 0) avg_cent[k] /= wc[k];
  free(we);
  free(wc);
}

/* StressCorrection.apply_marker_stress_correction_for_remaining_grid_stress! (StressCorrection.jl:35-82) */
void o_stress_correction(int64_t M, const int8_t* flags, int64_t xnum, int64_t ynum, const double* x,
                         const double* y, const int32_t* xn, const int32_t* yn, const double* dx,
                         const double* dy, const double* gridy_vx, const double* ystp_vx,
                         const double* gridx_vy, const double* xstp_vy, const double* dsxy,
                         const double* dsxx, double* m_sxy, double* m_sxx) {
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    m_sxy[m] = m_sxy[m] + get_marker_value(yn[m], xn[m], dy[m], dx[m], dsxy, ynum);
    m_sxx[m] = m_sxx[m] + pressure_value(xnum, ynum, yn[m], xn[m], y[m], x[m], gridy_vx, ystp_vx, gridx_vy, xstp_vy, dsxx);
  }
}

/* SubgridDiffusion.subgrid_heat_diffusion_update! (heat_solver/subgrid_heat/SubgridDiffusion.jl:59-175)
 * and remove_subgrid_effects_from_grid_changes! (SubgridDiffusion.jl:191-195). */
void o_subgrid_heat(int64_t M, const int8_t* flags, int64_t xnum, int64_t ynum, const int32_t* xn,
                    const int32_t* yn, const double* dx, const double* dy, const double* wUL,
                    const double* wLL, const double* wUR, const double* wLR, double xstpavg,
                    double ystpavg, double timestep, double coef, const double* tk1,
                    const double* kt1, const double* rhocp1, double* m_tk, double* m_dt,
                    double* dtkn, double* wtnodes, double* dtk1) {
  const int64_t nb = ynum * xnum;
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) { m_dt[m] = 0.0; continue; }
    double tn = get_marker_value(yn[m], xn[m], dy[m], dx[m], tk1, ynum);
    double dtot = tn - m_tk[m];
    double k = get_marker_value(yn[m], xn[m], dy[m], dx[m], kt1, ynum);
    double rc = get_marker_value(yn[m], xn[m], dy[m], dx[m], rhocp1, ynum);
    double tsg = rc / k / (2.0 / (xstpavg * xstpavg) + 2.0 / (ystpavg * ystpavg));
    double term = -coef * timestep / tsg;
    if (term < -30.0) term = -30.0;
    double d = dtot * (1.0 - exp(term));
    m_dt[m] = d;
    m_tk[m] += d;
  }
  memset(dtkn, 0, sizeof(double) * nb);
  memset(wtnodes, 0, sizeof(double) * nb);
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    upd_incl(dtkn, ynum, yn[m], xn[m], wUL[m], wLL[m], wUR[m], wLR[m], m_dt[m]);
    upd_incl(wtnodes, ynum, yn[m], xn[m], wUL[m], wLL[m], wUR[m], wLR[m], 1.0);
  }
  for (int64_t k = 0; k < nb; ++k) if (wtnodes[k] != 0) dtkn[k] = dtkn[k] / wtnodes[k];
  for (int64_t k = 0; k < nb; ++k) dtk1[k] = dtk1[k] - dtkn[k];
}

/* MarkerTemperature.add_remaining_grid_change_to_marker_temperature! (MarkerTemperature.jl:18-45) */
void o_add_remaining_dt(int64_t M, const int8_t* flags, int64_t ynum, const int32_t* xn,
                        const int32_t* yn, const double* dx, const double* dy, const double* dtk1,
                        double* m_tk) {
  OMP_FOR
  for (int64_t m = 0; m < M; ++m)
    if (flags[m] == 1) m_tk[m] += get_marker_value(yn[m], xn[m], dy[m], dx[m], dtk1, ynum);
}

/* ---------------------------------------------------------------- advection -- */

/* VelocityAndSpin.interpolate_vx / interpolate_vy / interpolate_spin (VelocityAndSpin.jl:343-428)
 * with MarkerGridMapping.upr_left_{x,y}_mapping_{basic,vx,vy}_grid (MarkerGridMapping.jl:355-440). */
static inline void vel_spin(int64_t xnum, int64_t ynum, int32_t ixb, int32_t iyb, double x, double y,
                            const double* gridx_b, const double* gridy_b, const double* xstp_b,
                            const double* ystp_b, const double* gridx_vy, const double* xstp_vy,
                            const double* gridy_vx, const double* ystp_vx, const double* vx1,
                            const double* vy1, const double* esp, double* vx, double* vy, double* sp) {
  /* vx grid (ynum+1, xnum) */
  int32_t xi = ixb;
  double dxv = (x - gridx_b[ixb - 1]) / xstp_b[ixb - 1];
  int32_t yi = iyb;
  if (y > gridy_vx[yi]) yi += 1; /* gridy_vx[yi+1] 1-based */
  if (yi > (int32_t)ynum) yi -= 1;
  double dyv = (y - gridy_vx[yi - 1]) / ystp_vx[yi - 1];
  *vx = get_marker_value(yi, xi, dyv, dxv, vx1, ynum + 1);
  /* vy grid (ynum, xnum+1) */
  xi = ixb;
  if (x > gridx_vy[xi]) xi += 1;
  if (xi > (int32_t)xnum) xi = (int32_t)xnum;
  dxv = (x - gridx_vy[xi - 1]) / xstp_vy[xi - 1];
  yi = iyb;
  dyv = (y - gridy_b[iyb - 1]) / ystp_b[iyb - 1];
  *vy = get_marker_value(yi, xi, dyv, dxv, vy1, ynum);
  /* basic grid spin */
  dxv = (x - gridx_b[ixb - 1]) / xstp_b[ixb - 1];
  dyv = (y - gridy_b[iyb - 1]) / ystp_b[iyb - 1];
  *sp = get_marker_value(iyb, ixb, dyv, dxv, esp, ynum);
}

/* Advection.advect_markers_and_rotate_stress_tensor! (src/advection/Advection.jl:109-114):
 *   update_marker_velocity_and_spin_using_runge_kutta! (VelocityAndSpin.jl:45-129; RungeKutta.jl:9-69)
 *   MarkersLocation.update!                             (MarkersLocation.jl:11-39)
 *   MarkersStressRotation.update! / rotate_marker_stress (MarkersStressRotation.jl:15-75) */
void o_advect(int64_t M, const int8_t* flags, int64_t xnum, int64_t ynum, const double* gridx_b,
              const double* gridy_b, const double* xstp_b, const double* ystp_b,
              const double* gridx_vy, const double* xstp_vy, const double* gridy_vx,
              const double* ystp_vx, const double* vx1, const double* vy1, const double* esp,
              double timestep, int64_t rk_order_max, const int32_t* xn, const int32_t* yn,
              double* x, double* y, double* m_vx, double* m_vy, double* m_spin, double* m_sxx,
              double* m_sxy) {
  if (rk_order_max <= 0) return;
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) { m_vx[m] = 0.0; m_vy[m] = 0.0; m_spin[m] = 0.0; continue; }
    double x0 = x[m], y0 = y[m], xc = x0, yc = y0;
    double v[4][3];
    for (int r = 1; r <= 4; ++r) {
      int32_t ixb, iyb;
      if (r == 1) { ixb = xn[m]; iyb = yn[m]; }
      else { ixb = o_index_of_left_node(xc, gridx_b, xnum); iyb = o_index_of_left_node(yc, gridy_b, ynum); }
      vel_spin(xnum, ynum, ixb, iyb, xc, yc, gridx_b, gridy_b, xstp_b, ystp_b, gridx_vy, xstp_vy,
               gridy_vx, ystp_vx, vx1, vy1, esp, &v[r - 1][0], &v[r - 1][1], &v[r - 1][2]);
      if (r < 3) { xc = x0 + timestep / 2.0 * v[r - 1][0]; yc = y0 + timestep / 2.0 * v[r - 1][1]; }
      else if (r == 3) { xc = x0 + timestep * v[r - 1][0]; yc = y0 + timestep * v[r - 1][1]; }
      else { xc = x0; yc = y0; }
    }
    double vxm, vym, spm;
    if (rk_order_max == 4) {
      vxm = (v[0][0] + 2.0 * v[1][0] + 2.0 * v[2][0] + v[3][0]) / 6.0;
      vym = (v[0][1] + 2.0 * v[1][1] + 2.0 * v[2][1] + v[3][1]) / 6.0;
      spm = (v[0][2] + 2.0 * v[1][2] + 2.0 * v[2][2] + v[3][2]) / 6.0;
    } else {
      vxm = v[0][0]; vym = v[0][1]; spm = v[0][2];
    }
    m_vx[m] = vxm; m_vy[m] = vym; m_spin[m] = spm;
  }
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    x[m] = x[m] + timestep * m_vx[m];
    y[m] = y[m] + timestep * m_vy[m];
  }
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    double spin = m_spin[m], sxy = m_sxy[m], sxx = m_sxx[m];
    double t1 = 2.0 * spin * timestep, t2 = spin * timestep;
    double s1 = sin(t1), c1 = cos(t1), s2 = sin(t2), c2 = cos(t2);
    m_sxy[m] = sxx * s1 + sxy * c1;
    m_sxx[m] = sxx * (c2 * c2 - s2 * s2) - sxy * s1;
  }
}

/* MarkersStrain.update_total_strain! and update_plastic_strain! (src/advection/strain/MarkersStrain.jl:11-136) */
void o_update_strain(int64_t M, const int8_t* flags, double timestep, double healing,
                     const double* m_exx, const double* m_exy, double* m_gii, const double* m_sxx,
                     const double* m_sxy, const double* m_eta, const double* m_eta_flow,
                     const float* m_pfailure, double* m_sp, double* m_srp) {
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    m_gii[m] = m_gii[m] + timestep * sqrt(m_exx[m] * m_exx[m] + m_exy[m] * m_exy[m]);
  }
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1 || m_pfailure[m] != 1.0f) continue;
    double sii = sqrt(m_sxx[m] * m_sxx[m] + m_sxy[m] * m_sxy[m]);
    double rate = 0.5 * sii * (1.0 / m_eta[m] - 1.0 / m_eta_flow[m]);
    if (rate < 0.0) rate = 0.0;
    double s = m_sp[m] + timestep * rate - healing * timestep;
    if (s < 0.0) s = 0.0;
    m_sp[m] = s;
    m_srp[m] = rate;
  }
}

/* ---------------------------------------------------------------- rheology -- */

/* FailureProperties.calculate_failure_properties_loop! and helpers
 *   (src/rheology/plastic_failure/failure_properties/FailureProperties.jl:19-161) */
void o_failure_properties(int64_t M, const int8_t* flags, const int16_t* matid, int64_t nmat,
                          const double* mat_plastic, const double* m_sp, const double* m_fric_ini,
                          int64_t iuse_melt_damage, const double* m_melt_damage, double* m_coh,
                          double* m_fric) {
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    int mt = matid[m];
    double strain = m_sp[m], sfi_m = m_fric_ini[m];
    double ci = MAT(mat_plastic, nmat, mt, 1), cf = MAT(mat_plastic, nmat, mt, 2);
    double sfi_mat = MAT(mat_plastic, nmat, mt, 3), sff_mat = MAT(mat_plastic, nmat, mt, 4);
    double ei = MAT(mat_plastic, nmat, mt, 5), ef = MAT(mat_plastic, nmat, mt, 6);
    double sff;
    if (sfi_mat > 0.0 && sff_mat > 0.0) sff = sfi_m * (sff_mat / sfi_mat);
    else sff = sff_mat;
    double coh = ci, sf = sfi_m;
    if (strain >= ef) { coh = cf; sf = sff; }
    else if (ei <= strain && strain < ef) {
      coh = ci + (cf - ci) / (ef - ei) * (strain - ei);
      sf = sfi_m + (sff - sfi_m) / (ef - ei) * (strain - ei);
    }
    if (iuse_melt_damage == 1) { sf = sf / m_melt_damage[m]; coh = coh / m_melt_damage[m]; }
    m_coh[m] = coh;
    m_fric[m] = sf;
  }
}

/* CreepStrainRate.calculate_creep_strain_rate + ExponentialTerm (composite_creep/core/CreepStrainRate.jl, ExponentialTerm.jl) */
static inline double creep_rate(double p_mpa, double T, double R, double A, double Ea, double Va,
                                int use_old, double* expterm, double s_mpa, double n) {
  if (!use_old) {
    double fac1 = 1.0 / (R * T);
    double act = (Ea * 1000.0 + Va * p_mpa) * fac1;
    *expterm = exp(-act);
  }
  double st = (n == 1.0) ? s_mpa : jl_pow(s_mpa, n);
  return A * *expterm * st;
}

/* PeierlsCreep.calculate_peierls_creep_strain_rate (composite_creep/core/PeierlsCreep.jl:55-98) */
static inline double peierls_rate(double p_mpa, double T, double R, double A, double Ea, double Va,
                                  double m_exp, double n_exp, double s_p, int use_old, double* act,
                                  double s_mpa) {
  if (!use_old) {
    double fac1 = 1.0 / (R * T);
    *act = (Ea * 1000.0 + Va * p_mpa) * fac1;
  }
  double ratio = s_mpa / s_p;
  double tm = (m_exp == 1.0) ? 1.0 - ratio : 1.0 - jl_pow(ratio, m_exp);
  double inner = (n_exp == 2.0) ? tm * tm : jl_pow(tm, n_exp);
  double e = exp(-*act * inner);
  return A * e * (s_mpa * s_mpa);
}

/* CompositeCreep.calculate_composite_creep_viscosity_and_strain_rate (CompositeCreep.jl:18-144) */
static double composite_viscosity(double p_mpa, double T, double R, const double* fl, double preexp,
                                  double s_mpa, int use_old, double* e_disl, double* a_peierls,
                                  double* e_diff) {
  /* fl: flow-law row, fl[k-1] = mat_flow[mat, k] */
  double rd = creep_rate(p_mpa, T, R, preexp, fl[3], fl[4], use_old, e_disl, s_mpa, fl[2]);
  double rp = 0.0;
  if (fl[5] > 0.0 && T < 1200.0)
    rp = peierls_rate(p_mpa, T, R, fl[5], fl[3], fl[4], fl[6], fl[7], fl[8], use_old, a_peierls, s_mpa);
  double rf = 0.0;
  if (fl[9] > 0.0) rf = creep_rate(p_mpa, T, R, fl[9], fl[10], fl[11], use_old, e_diff, s_mpa, 1.0);
  double rate = ((rd > rp) ? rd : rp) + rf;
  return 0.5 * (s_mpa * 1e6) / rate;
}

static inline double forecast_ve(double dt, double mu, double srr, double sxx, double sxy, double exx,
                                 double exy, double smin, double eta) {
  /* CompositeViscosity.forecast_viscoelastic_stress (CompositeViscosity.jl:379-397) */
  double vef = eta / (mu * dt + eta);
  double fac1 = 2.0 * eta * srr;
  double om = 1.0 - vef;
  double nxx = fac1 * exx * om + sxx * vef;
  double nxy = fac1 * exy * om + sxy * vef;
  double s = sqrt(nxx * nxx + nxy * nxy);
  return (s > smin) ? s : smin;
}

/* The flow laws other than composite creep, selected as FlowViscosity.update_marker_flow_viscosity!
 * selects them (FlowViscosity.jl:21-44): option = the largest mat_flow_type of the model.
 *   0  Isoviscous.update_marker_flow_viscosity! (types/isoviscous/Isoviscous.jl):
 *      eta_flow = preexp = mat_flow[mat, 1];
 *   4  CouetteFlowBenchmark.update_marker_flow_viscosity! (types/couette_flow_benchmark/
 *      CouetteFlowBenchmark.jl): T = max(TK, T_left), eta = A exp(Ea 1000 / R / T_left
 *      (1 - (T - T_left) / T_left)) with A, Ea = mat_flow[mat, 13], [mat, 14]; preexp = A;
 *   5  Blankenback89.update_marker_flow_viscosity! (types/blankenbach89/Blankenback89.jl):
 *      T = max(TK, T_top), eta = eta0 exp(-b (T - T_top) / (T_bottom - T_top) + c y / ysize)
 *      with eta0, b, c = mat_flow[mat, 15:17]; preexp = eta0;
 *  -1  Xdependent.update_marker_flow_viscosity! (types/x_dependent/Xdependent.jl): the
 *      analytic viscosity of the 10 x 9.5 km non-Newtonian channel (n = 3, C = 1e-37,
 *      1e9 Pa), eta_max on the centre line; preexp = mat_flow[mat, 1].
 * mat_flow is the reference's nmat x 17 table.  Markers outside the domain are skipped. */
void o_flow_viscosity_other(int64_t M, const int8_t* flags, const int16_t* matid, int64_t nmat, int64_t option,
                            const double* mat_flow, double T_top, double T_bottom, double T_left, double R,
                            double ysize, double eta_max, const double* m_x, const double* m_y,
                            const double* m_tk, double* m_eta_flow, double* m_preexp) {
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    int mt = matid[m];
    double eta = 0.0, pre = 0.0;
    if (option == 0) {
      eta = MAT(mat_flow, nmat, mt, 1);
      pre = eta;
    } else if (option == 4) {
      double T = m_tk[m] > T_left ? m_tk[m] : T_left;
      pre = MAT(mat_flow, nmat, mt, 13);
      double ea = MAT(mat_flow, nmat, mt, 14);
      eta = pre * exp(ea * 1000.0 / R / T_left * (1.0 - (T - T_left) / T_left));
    } else if (option == 5) {
      double T = m_tk[m] > T_top ? m_tk[m] : T_top;
      pre = MAT(mat_flow, nmat, mt, 15);
      double b = MAT(mat_flow, nmat, mt, 16), cy = MAT(mat_flow, nmat, mt, 17);
      eta = pre * exp(-b * (T - T_top) / (T_bottom - T_top) + cy * m_y[m] / ysize);
    } else if (option == -1) {
      double pg = -1e9 / 9500.0, dx = m_x[m] - 10000.0 / 2.0;
      eta = fabs(dx) > 0.0 ? 1.0 / 1e-37 * pow(-pg, 1.0 - 3.0) * pow(dx, 1.0 - 3.0) : eta_max;
      pre = MAT(mat_flow, nmat, mt, 1);
    }
    m_eta_flow[m] = eta;
    m_preexp[m] = pre;
  }
}

/* CompositeViscosity.update_marker_flow_viscosity! (flow_viscosity/update/types/composite_viscosity/
 * CompositeViscosity.jl:133-284) incl. apply_strain_softening (:286-297, ViscousStrainSoftening.jl:14-39),
 * calc_initial_stress_invariant (:299-306), update_bisection_limits (:403-418).
 * iters_out (optional) receives the bisection iteration count per marker. */
void o_composite_viscosity(int64_t M, const int8_t* flags, const int16_t* matid, int64_t nmat,
                           const int64_t* mat_flow_type, const double* mat_flow,
                           const double* mat_plastic, const double* mat_mu, double timestep,
                           double T_top, double eta_min, double eta_max, double s_min, double R,
                           int64_t iuse_soft, double vsoftfac, const double* m_sxx,
                           const double* m_sxy, const double* m_exx, const double* m_exy,
                           const double* m_tk, const double* m_pr, const double* m_gii,
                           const double* m_srr, double* m_eta_flow, double* m_preexp,
                           int32_t* iters_out) {
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    int mt = matid[m];
    int64_t ft = mat_flow_type[mt - 1];
    double eta = 0.0;
    double A = MAT(mat_flow, nmat, mt, 2);
    int32_t iters = 0;
    if (ft == 0) {
      eta = MAT(mat_flow, nmat, mt, 1);
    } else if (ft == 1 || ft == 2) {
      double fl[12];
      for (int k = 1; k <= 12; ++k) fl[k - 1] = MAT(mat_flow, nmat, mt, k);
      double sxx = m_sxx[m], sxy = m_sxy[m], exx = m_exx[m], exy = m_exy[m];
      double strain = m_gii[m];
      double p_mpa = m_pr[m] * PA_TO_MPA;
      double srr = m_srr[m];
      double T = (m_tk[m] > T_top) ? m_tk[m] : T_top;
      double ei = MAT(mat_plastic, nmat, mt, 5), ef = MAT(mat_plastic, nmat, mt, 6);
      double mu = mat_mu[mt - 1];
      if (iuse_soft == 1) {
        double amin = A, amax = A * vsoftfac;
        if (ei < strain && strain < ef) A = amin + (amax - amin) / (ef - ei) * (strain - ei);
        if (strain >= ef) A = amax;
      }
      double s0 = sqrt(sxx * sxx + sxy * sxy);
      if (s0 < s_min) s0 = s_min;
      double e_disl = 0.0, a_p = 0.0, e_diff = 0.0;
      eta = composite_viscosity(p_mpa, T, R, fl, A, s0 * PA_TO_MPA, 0, &e_disl, &a_p, &e_diff);
      double sf = forecast_ve(timestep, mu, srr, sxx, sxy, exx, exy, s_min, eta);
      double delta = 1e39;
      int icount = 0;
      while (icount < 20 && delta > 1.0) {
        icount += 1;
        double savg = (s0 + sf) / 2.0;
        eta = composite_viscosity(p_mpa, T, R, fl, A, savg * PA_TO_MPA, 1, &e_disl, &a_p, &e_diff);
        double sfu = forecast_ve(timestep, mu, srr, sxx, sxy, exx, exy, s_min, eta);
        if ((sf > s0 && sfu > savg) || (sf < s0 && sfu < savg)) s0 = savg;
        else sf = savg;
        delta = fabs(sf - s0);
      }
      iters = icount;
      if (eta < eta_min) eta = eta_min;
      if (eta > eta_max) eta = eta_max;
    }
    m_eta_flow[m] = eta;
    m_preexp[m] = A;
    if (iters_out) iters_out[m] = iters;
  }
}

/* ViscoplasticViscosity.update_marker_viscoplastic_viscosity! (viscoplastic_viscosity/ViscoplasticViscosity.jl:21-60) */
void o_viscoplastic_viscosity(int64_t M, const int8_t* flags, int64_t ntimestep, int64_t itype_global,
                              const double* m_eta_flow, double* m_eta) {
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    double vf = m_eta_flow[m], vp = m_eta[m];
    if (itype_global == 0) vp = vf;
    else if (itype_global == 1) { if (ntimestep == 0 || vp == 0.0) vp = vf; }
    m_eta[m] = vp;
  }
}

/* ViscoelasticForecast.update_plastic_yielding! (plastic_failure/markers/update/types/ViscoelasticForecast.jl:11-181)
 * with CheckYield.check_yield_is_applicable (utils/CheckYield.jl:3-12), YieldStress.calc_yield_stress
 * (utils/YieldStress.jl:28-67), FluidPressure (utils/FluidPressure.jl:14-23), Limits (Limits.jl:3-21),
 * YieldCheck (YieldCheck.jl:3-63), Viscoelastic factor eta/(eta+mu*dt). */
void o_plastic_yielding(int64_t M, const int8_t* flags, int64_t ntimestep, double timestep,
                        int64_t iuse_fluid, double y_sealevel, double eta_min, double eta_max,
                        double sy_min, double sy_max, int64_t no_yield_mobile, int64_t id_air,
                        int64_t id_wall, int64_t id_plate, const double* y, const int16_t* matid,
                        const double* mat_mu, const double* m_coh, const double* m_fric,
                        const double* m_exx, const double* m_exy, const double* m_srr,
                        const double* m_pr, double* m_sxx, double* m_sxy, double* m_eta,
                        float* m_pfailure) {
  OMP_FOR
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    int mt = matid[m];
    double coh = m_coh[m], sf = m_fric[m];
    int applicable = (ntimestep > 0 && (coh > 0.0 || sf > 0.0));
    int yflag = 0;
    if (applicable) {
      double eta = m_eta[m], mu = mat_mu[mt - 1];
      double sxx = m_sxx[m], sxy = m_sxy[m], exx = m_exx[m], exy = m_exy[m];
      double srr = m_srr[m], p = m_pr[m];
      double cphi = cos(asin(sf));
      double sy;
      if (iuse_fluid == 0) {
        sy = coh * cphi + sf * p;
      } else {
        double depth = y[m] - y_sealevel;
        if (depth < 0.0) depth = 0.0;
        double pf = 1000.0 * 9.81 * depth;
        if (p < pf) sy = coh * cphi;
        else sy = coh * cphi + sf * (p - pf);
      }
      if (sy < 0.0) sy = 0.0;
      if (sy < sy_min) sy = sy_min;
      if (sy > sy_max) sy = sy_max;
      double vef = eta / (eta + mu * timestep);
      double nxx = sxx * vef + 2.0 * eta * exx * srr * (1.0 - vef);
      double nxy = sxy * vef + 2.0 * eta * exy * srr * (1.0 - vef);
      double sii = sqrt(nxx * nxx + nxy * nxy);
      int yielding = 0;
      if (no_yield_mobile) {
        if (sii > sy && mt != id_air && mt != id_wall && mt != id_plate) yielding = 1;
      } else if (sii > sy) {
        yielding = 1;
      }
      yflag = yielding;
      if (yielding) {
        double s_old = sqrt(sxx * sxx + sxy * sxy);
        if (s_old != 0.0) { sxx = sxx * sy / s_old; sxy = sxy * sy / s_old; }
        else { sxx = sy; sxy = sy; }
        double e_old = srr * sqrt(exx * exx + exy * exy);
        eta = sy / 2.0 / e_old;
        if (eta < eta_min) eta = eta_min;
        if (eta > eta_max) eta = eta_max;
        m_sxx[m] = sxx; m_sxy[m] = sxy; m_eta[m] = eta;
      }
    }
    if (m_pfailure[m] != 1.0f) m_pfailure[m] = (float)yflag;
  }
}

/* GridViscoplasticityToMarkers.calc_marker_viscoplastic_viscosity!
 * (src/rheology/plastic_failure/nodes/GridViscoplasticityToMarkers.jl:7-62), with
 * check_basic_grid_for_yielding (:64-74) and interpolate_grid_viscosity_to_marker (:76-118,
 * use_sum_for_numerator = true): markers of a cell with a yielding corner take the
 * plastic-flag-weighted harmonic average of etas1 when it is below their flow viscosity,
 * and are then marked as failed.  A serial marker loop, as in the reference. */
void o_marker_viscoplastic_viscosity_from_grid(int64_t M, const int8_t* flags, int64_t ynum,
                                               const int32_t* xn, const int32_t* yn, const double* mdx,
                                               const double* mdy, const double* plastic_yield,
                                               const double* etas1, const double* m_eta_flow, double* m_eta,
                                               float* m_pfailure) {
  for (int64_t m = 0; m < M; ++m) {
    if (flags[m] != 1) continue;
    const int32_t ix = xn[m], iy = yn[m];
    const double pul = plastic_yield[IDX(iy, ix, ynum)], pll = plastic_yield[IDX(iy + 1, ix, ynum)];
    const double pur = plastic_yield[IDX(iy, ix + 1, ynum)], plr = plastic_yield[IDX(iy + 1, ix + 1, ynum)];
    const int yielding = pul > 0.0 || pll > 0.0 || pur > 0.0 || plr > 0.0;
    const double vflow = m_eta_flow[m];
    if (!yielding) {
      m_eta[m] = vflow;
      continue;
    }
    const double dx = mdx[m], dy = mdy[m];
    const double wul = (1.0 - dx) * (1.0 - dy), wll = (1.0 - dx) * dy;
    const double wur = dx * (1.0 - dy), wlr = dx * dy;
    const double eul = etas1[IDX(iy, ix, ynum)], ell = etas1[IDX(iy + 1, ix, ynum)];
    const double eur = etas1[IDX(iy, ix + 1, ynum)], elr = etas1[IDX(iy + 1, ix + 1, ynum)];
    const double denom = pul / eul * wul + pll / ell * wll + pur / eur * wur + plr / elr * wlr;
    const double numer = pul * wul + pll * wll + pur * wur + plr * wlr;
    const double vvp = numer / denom;
    if (vvp >= vflow) {
      m_eta[m] = vflow;
    } else {
      m_eta[m] = vvp;
      m_pfailure[m] = 1.0f;
    }
  }
}
