/* boundary_oracle.c -- CPU restatement of the reference's step-boundary updates, test
 * infrastructure only (the product path never links it).
 *
 *   o_timestep_displacement_limit   time_step/update/Update.jl:16-219
 *       (update_model_time_step_using_displacement_limit: average-spacing and local
 *        staggered-node variants; returns the new time step)
 *   o_rock_properties               rock_properties/RockProperties.jl:99-125
 *       (update_marker_rock_properties!: density, rhocp, conductivity, adiabatic term,
 *        sediment porosity), with the model types of rock_properties/{density,rhocp,
 *        thermal_conductivity}/types/*.jl, UpdateAdiabaticTerm.jl:19-33 and
 *        porosity/{PorosityUpdate,SedimentPorosity}.jl; topography depth by
 *        MathTools.linear_interp (utils/MathTools.jl:160-198)
 *
 * Grids are column-major (rows, cols).  Julia's x^2 and x^3 of a Float64 literal power
 * are x*x and x*x*x.
 */
#include <math.h>
#include <stdint.h>

static double step_limit(double dt, double displ, double cell, double v) {
  if (v > 0) {
    const double lim = displ * cell / v;
    dt = dt < lim ? dt : lim;
  }
  return dt;
}

double o_timestep_displacement_limit(int64_t xnum, int64_t ynum, const double* vx1, const double* vy1,
                                     const double* xstp, const double* ystp, double xstpavg, double ystpavg,
                                     double displ, int64_t iuse_local, double dt_old) {
  const int64_t nvx = (ynum + 1) * xnum, nvy = ynum * (xnum + 1);
  if (iuse_local == 0) {
    double mx = vx1[0], mn = vx1[0];
    for (int64_t k = 1; k < nvx; ++k) { if (vx1[k] > mx) mx = vx1[k]; if (vx1[k] < mn) mn = vx1[k]; }
    const double vxmax = fabs(mx) > fabs(mn) ? fabs(mx) : fabs(mn);
    mx = vy1[0]; mn = vy1[0];
    for (int64_t k = 1; k < nvy; ++k) { if (vy1[k] > mx) mx = vy1[k]; if (vy1[k] < mn) mn = vy1[k]; }
    const double vymax = fabs(mx) > fabs(mn) ? fabs(mx) : fabs(mn);
    double dt = step_limit(dt_old, displ, xstpavg, vxmax);
    return step_limit(dt, displ, ystpavg, vymax);
  }
  double dt = dt_old;
  const int64_t jmax = xnum - 1, imax = ynum - 1;  /* length(xstp), length(ystp) */
  for (int64_t j = 1; j <= xnum; ++j)
    for (int64_t i = 1; i <= ynum + 1; ++i) {
      const double cell = j == 1 ? xstp[0] : (j == jmax + 1 ? xstp[jmax - 1] :
                          (xstp[j - 2] < xstp[j - 1] ? xstp[j - 2] : xstp[j - 1]));
      dt = step_limit(dt, displ, cell, fabs(vx1[(j - 1) * (ynum + 1) + (i - 1)]));
    }
  for (int64_t j = 1; j <= xnum + 1; ++j)
    for (int64_t i = 1; i <= ynum; ++i) {
      const double cell = i == 1 ? ystp[0] : (i == imax + 1 ? ystp[imax - 1] :
                          (ystp[i - 2] < ystp[i - 1] ? ystp[i - 2] : ystp[i - 1]));
      dt = step_limit(dt, displ, cell, fabs(vy1[(j - 1) * ynum + (i - 1)]));
    }
  return dt;
}

static double linear_interp(double x, const double* xc, const double* yv, int64_t n) {
  if (x <= xc[0]) return yv[0];
  if (x >= xc[n - 1]) return yv[n - 1];
  for (int64_t j = 1; j < n; ++j) {
    const double x1 = xc[j - 1], x2 = xc[j], y1 = yv[j - 1], y2 = yv[j];
    if (x == x1) return y1;
    if (x == x2) return y2;
    if (x1 < x && x < x2) return y1 + (y2 - y1) / (x2 - x1) * (x - x1);
  }
  return 0.0;
}

/* mat_rho (nmat, 3) column-major: standard density, expansivity, compressibility;
 * mat_kt (nmat, 2): reference conductivity, factor a. */
void o_rock_properties(int64_t M, const int8_t* inside, const int16_t* matid, const double* x, const double* y,
                       const double* pr, const double* tk, double* rho, double* rhocp, double* kt, double* ha,
                       int64_t nmat, const double* mat_rho, const double* mat_cp, const double* mat_kt,
                       int64_t density_model, int64_t rhocp_model, int64_t cond_model, double temperature_top,
                       double maximum_heat_capacity, int64_t iuse_por, const double* por0, const double* decay,
                       const double* burial, const double* topo_x, const double* topo_y, int64_t ntopo,
                       const int16_t* sed_ids, int64_t nsed, double k_water, double rho_water, double cp_water) {
  for (int64_t m = 0; m < M; ++m) {
    if (inside[m] != 1) continue;
    const int64_t id = matid[m] - 1;
    const double rho_s = mat_rho[id], alpha = mat_rho[nmat + id], beta = mat_rho[2 * nmat + id];
    const double T = tk[m];
    /* density: DensityLiao14.jl:92-104, DensityBlankenbach89.jl:95-102, DensityNaliboff17.jl */
    if (density_model == 0)
      rho[m] = rho_s * (1.0 - alpha * (T - 298.15)) * (1.0 + beta * (pr[m] - 1e5));
    else if (density_model == 1)
      rho[m] = rho_s * (1.0 - alpha * (T - temperature_top));
    else
      rho[m] = rho_s * (1.0 - alpha * (T - 830.0));
    /* rhocp: ConstantRhoCp.jl, TemperatureDependentWaples.jl (kelvin_to_celsius: T - 273) */
    const double cp20 = mat_cp[id];
    if (rhocp_model == 0) {
      rhocp[m] = rho[m] * cp20;
    } else {
      const double tc = T - 273.0;
      double cp = cp20 * (0.953 + 2.29e-3 * tc - 2.835e-6 * (tc * tc) + 1.191e-9 * (tc * tc * tc));
      cp = cp < maximum_heat_capacity ? cp : maximum_heat_capacity;
      rhocp[m] = rho[m] * cp;
    }
    /* conductivity: thermal_conductivity/types/*.jl */
    const double k0 = mat_kt[id], ka = mat_kt[nmat + id];
    double k;
    switch (cond_model) {
      case 0: k = (k0 + ka / (T + 77.0)) * exp(0.00004 * pr[m] / 1e6); break;
      case 1: k = k0; break;
      case 2: k = k0 / (1.0 + ka * (T - temperature_top) / temperature_top); break;
      case 3: k = y[m] > 110000.0 ? 39.25 : k0; break;
      case 4: k = y[m] > 100000.0 + 10000.0 ? (10000.0 / 100000.0) * 2.25 * (1330.0 - 0.0) / (1334.5 - 1330.0) : k0; break;
      default: k = k0 <= 20.0 ? 358.0 * (1.0227 * k0 - 1.882) * (1.0 / T - 0.00068) + 1.84 : k0; break;
    }
    kt[m] = k;
    /* adiabatic term (UpdateAdiabaticTerm.jl:19-33) */
    ha[m] = alpha * T;
    /* sediment porosity (PorosityUpdate.jl, SedimentPorosity.jl) */
    if (iuse_por == 1) {
      int sed = 0;
      for (int64_t s = 0; s < nsed; ++s) sed |= (sed_ids[s] == matid[m]);
      if (sed) {
        const double y_mud = linear_interp(x[m], topo_x, topo_y, ntopo);
        double ysub = y[m] - y_mud;
        ysub = ysub > burial[m] ? ysub : burial[m];
        const double phi = por0[m] * exp(-(1.0 / decay[m]) * ysub);
        const double kb = kt[m] * (1.0 - phi) + k_water * phi;
        const double rb = rho[m] * (1.0 - phi) + rho_water * phi;
        const double cb = cp20 * (1.0 - phi) + cp_water * phi;
        kt[m] = kb;
        rho[m] = rb;
        rhocp[m] = rb * cb;
      }
    }
  }
}
