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
 *   o_recycle_extension             boundary_conditions/marker_recycle/types/Extension.jl:14-129
 *       (recycle_markers! for the extension models: outside markers in marker order,
 *        InitializeMarkerRecycling.jl:26-108; positions, Coordinates.jl:60-153; property
 *        resets, ResetMarkers.jl:24-290; reset pressure, PressureReset.jl:20-26), with the
 *        reference's rand() replaced by the Philox-4x32-10 stream of o_recycle_uniforms
 *   o_recycle_no_bottom_inflow      marker_recycle/types/ExtensionNoBottomInflow.jl:25-123
 *   o_recycle_channel               marker_recycle/types/Channel.jl:20-54
 *   o_recycle_contraction           marker_recycle/types/ContractionViscoelastic.jl:20-134 with
 *       utils/ContractionRecycleLocations.jl:9-140, CountRecycle.jl:19-29, Coordinates.jl:223-293,
 *       marker_materials/init_manager/utils/{SevenLayerEarthModel2D.jl:20-62,StrongRegions.jl:24-80},
 *       markers/utils/Layers.jl:31-54
 *   o_recycle_side_inflow           marker_recycle/types/ExtensionInflowAndOutflowAlongSides.jl:20-237
 *       with boundary_velocity/utils/{InflowGeometry.jl,InflowRamp.jl}, Coordinates.jl:155-200
 *   o_recycle_fracture_zone         marker_recycle/types/ContractionFractureZone.jl:11-61 with
 *       utils/FractureZoneProperties.jl:17-55, marker_materials/init_manager/types/FractureZone.jl:
 *       63-299 and temperature/init_manager/types/FractureZone.jl:86-202 (erf from libm)
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

/* Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC 2011): round function
 * (c0,c1,c2,c3) -> (hi(M1 c2) ^ c1 ^ k0, lo(M1 c2), hi(M0 c0) ^ c3 ^ k1, lo(M0 c0)),
 * M0 = 0xD2511F53, M1 = 0xCD9E8D57, key bumped by (0x9E3779B9, 0xBB67AE85) between rounds. */
void o_philox4x32_10(uint32_t ctr[4], uint32_t k0, uint32_t k1) {
  for (int round = 0; round < 10; ++round) {
    if (round > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    const uint64_t a = (uint64_t)ctr[0] * 0xD2511F53u;
    const uint64_t b = (uint64_t)ctr[2] * 0xCD9E8D57u;
    const uint32_t out0 = (uint32_t)(b >> 32) ^ ctr[1] ^ k0;
    const uint32_t out2 = (uint32_t)(a >> 32) ^ ctr[3] ^ k1;
    ctr[1] = (uint32_t)b;
    ctr[3] = (uint32_t)a;
    ctr[0] = out0;
    ctr[2] = out2;
  }
}

/* counter (j lo, j hi, stream, step), key = seed; two doubles from the top 53 bits of
 * (w0:w1) and (w2:w3) */
void o_recycle_uniforms(uint64_t seed, int64_t step, uint32_t stream, int64_t j, double* u0, double* u1) {
  uint32_t ctr[4] = {(uint32_t)(uint64_t)j, (uint32_t)((uint64_t)j >> 32), stream, (uint32_t)(uint64_t)step};
  o_philox4x32_10(ctr, (uint32_t)seed, (uint32_t)(seed >> 32));
  const uint64_t a = ((uint64_t)ctr[0] << 32) | ctr[1], b = ((uint64_t)ctr[2] << 32) | ctr[3];
  *u0 = ldexp((double)(a >> 11), -53);
  *u1 = ldexp((double)(b >> 11), -53);
}

/* Marker fields the recycling writes, in this order (f[k] points to M doubles). */
enum { R_X, R_Y, R_TK, R_PR, R_SXX, R_SXY, R_EXX, R_EXY, R_ETA, R_SR_RATIO, R_GII, R_SP, R_SRP, R_MELT,
       R_FRIC_INI, R_FRIC, R_NF };

/* s[]: sticky_air, sticky_water, asthenosphere; d[]: xsize, ysize, vyu, vyl, timestep,
 * temperature_top, temperature_bottom, gridy_b[ynum], delta_fric_coef; mat_plastic (nmat, 6)
 * column-major.  Returns the number of recycled markers; list/flags (capacity M) get the
 * 1-based indices and flags in marker order, *n_air the sticky count. */
int64_t o_recycle_extension(int64_t M, const int8_t* inside, int16_t* matid, double** f, float* pfailure,
                            const int16_t* s, const double* d, int64_t nmat, const double* mat_plastic,
                            int64_t iuse_random_fric, uint64_t seed, int64_t step, int64_t* list, int8_t* flags,
                            int64_t* n_air) {
  const int16_t air = s[0], water = s[1], asth = s[2];
  const double xsize = d[0], ysize = d[1], dt = d[4];
  /* InitializeMarkerRecycling: outside indices in marker order, sticky count by material */
  int64_t nout = 0, nair = 0, nsub = 0;
  for (int64_t m = 0; m < M; ++m)
    if (inside[m] != 1) {
      list[nout++] = m;
      if (matid[m] == air || matid[m] == water) ++nair; else ++nsub;
    }
  /* Extension.calculate_recycled_locations: band widths |vyu dt| and -|vyl dt| */
  const double disp_upper = fabs(d[2] * dt), disp_lower = -fabs(d[3] * dt);
  int64_t ia = 0, is = 0;
  for (int64_t k = 0; k < nout; ++k) {
    const int64_t m = list[k];
    double u0, u1;
    int flag;
    if ((matid[m] == air || matid[m] == water) && nair > 0) {
      o_recycle_uniforms(seed, step, 0u, ia++, &u0, &u1);
      f[R_X][m] = 0.0 + u0 * xsize;
      f[R_Y][m] = 0.0 + u1 * disp_upper;
      flag = 0;
    } else {
      o_recycle_uniforms(seed, step, 1u, is++, &u0, &u1);
      f[R_X][m] = 0.0 + u0 * xsize;
      f[R_Y][m] = ysize + u1 * disp_lower;
      flag = 1;
    }
    flags[k] = (int8_t)flag;
    /* ResetMarkers.reset_marker!: sticky -> defaults (zero), subsurface -> asthenosphere */
    const int16_t id = flag == 0 ? air : asth;
    matid[m] = id;
    f[R_TK][m] = flag == 0 ? d[5] : d[6];
    f[R_PR][m] = flag == 0 ? 0.0 : 3300.0 * 9.81 * d[7];
    f[R_SXX][m] = f[R_SXY][m] = flag == 0 ? 0.0 : 1.96e6;
    f[R_EXX][m] = f[R_EXY][m] = flag == 0 ? 0.0 : 1e-14;
    f[R_SR_RATIO][m] = 0.0;
    f[R_GII][m] = f[R_SP][m] = f[R_SRP][m] = 0.0;
    f[R_MELT][m] = 0.0;
    f[R_ETA][m] = flag == 0 ? 0.0 : 1e20;
    pfailure[m] = 0.0f;
    double fric = mat_plastic[2 * nmat + (id - 1)];
    if (flag == 1 && iuse_random_fric == 1) {
      double r, unused;
      o_recycle_uniforms(seed, step, 2u, m, &r, &unused);
      if (r <= 0.5) fric = fric - d[8];
    }
    f[R_FRIC_INI][m] = fric;
    f[R_FRIC][m] = fric;
    list[k] = m + 1;
  }
  *n_air = nair;
  return nout;
}

/* ExtensionNoBottomInflow: every outside marker (marker order, rank j) re-enters at
 * y = u_j vyu dt, x = 0 + u_j xsize with ONE uniform u_j (stream 0, index j), and is reset as
 * sticky air at temperature_top (reset_marker! defaults: zero pressure, stress, strain rate,
 * strain, melt, viscosity; fric = mat_plastic[air, 3]).  d[]: xsize, vyu, dt, temperature_top. */
int64_t o_recycle_no_bottom_inflow(int64_t M, const int8_t* inside, int16_t* matid, double** f, float* pfailure,
                                   int16_t air, const double* d, int64_t nmat, const double* mat_plastic,
                                   uint64_t seed, int64_t step, int64_t* list, int8_t* flags) {
  const double displacement = d[1] * d[2];
  int64_t n = 0;
  for (int64_t m = 0; m < M; ++m) {
    if (inside[m] == 1) continue;
    double u, unused;
    o_recycle_uniforms(seed, step, 0u, n, &u, &unused);
    f[R_Y][m] = u * displacement;
    f[R_X][m] = 0.0 + u * d[0];
    matid[m] = air;
    f[R_TK][m] = d[3];
    f[R_PR][m] = 0.0;
    f[R_SXX][m] = f[R_SXY][m] = 0.0;
    f[R_EXX][m] = f[R_EXY][m] = 0.0;
    f[R_SR_RATIO][m] = 0.0;
    f[R_GII][m] = f[R_SP][m] = f[R_SRP][m] = 0.0;
    f[R_MELT][m] = 0.0;
    f[R_ETA][m] = 0.0;
    pfailure[m] = 0.0f;
    f[R_FRIC_INI][m] = f[R_FRIC][m] = mat_plastic[2 * nmat + (air - 1)];
    list[n] = m + 1;
    flags[n] = 0;
    ++n;
  }
  return n;
}

/* Channel: markers with y > gridy_b[ynum] move up by the grid height and their temperature
 * changes by temperature_top - temperature_bottom (evaluated as (T + T_top) - T_bottom). */
int64_t o_recycle_channel(int64_t M, double* y, double* tk, double gridy_min, double gridy_max, double t_top,
                          double t_bottom, int64_t* list) {
  const double ysize = gridy_max - gridy_min;
  int64_t n = 0;
  for (int64_t m = 0; m < M; ++m)
    if (y[m] > gridy_max) {
      y[m] = y[m] - ysize;
      tk[m] = tk[m] + t_top - t_bottom;
      list[n++] = m + 1;
    }
  return n;
}

/* SevenLayerEarthModel2D.define_material then StrongRegions.define_material with the layer
 * bases of Layers.calc_depths_for_layers (base[k] = base[k-1] + thick[k]).
 * ids: layers[0..6] (air, upper crust, lower crust, upper / middle / lower lithosphere,
 * asthenosphere), strong[0..2] (upper crust, lower crust, lithosphere). */
static int16_t contraction_define_material(double x, double y, const double* thick, double x_left, double x_right,
                                           const int16_t* layers, const int16_t* strong) {
  const double d1 = thick[0], d2 = d1 + thick[1], d3 = d2 + thick[2], d4 = d3 + thick[3], d5 = d4 + thick[4],
               d6 = d5 + thick[5];
  int16_t id = layers[6];
  if (y <= d1) id = layers[0];
  else if (y > d1 && y <= d2) id = layers[1];
  else if (y > d2 && y <= d3) id = layers[2];
  else if (y > d3 && y <= d4) id = layers[3];
  else if (y > d4 && y <= d5) id = layers[4];
  else if (y > d5 && y <= d6) id = layers[5];
  if (d1 < y && y <= d2) {
    if (x < x_left || x > x_right) id = strong[0];
  } else if (d2 < y && y <= d3) {
    if (x < x_left || x > x_right) id = strong[1];
  } else if (d3 < y && y <= d4) {
    if (x < x_left || x > x_right) id = strong[2];
  } else if (d4 < y && y <= d5) {
    if (x < x_left || x > x_right) id = strong[2];
  } else if (d5 < y && y <= d6) {
    if (x < x_left || x > x_right) id = strong[2];
  }
  return id;
}

/* ContractionRecycleLocations.calculate_recycled_*_locations for one group (n positions):
 * the first nleft = floor(n/2) (0 when asymmetric; CountRecycle.get_left_and_right_recycle_counts)
 * at the left side, the rest at the right; y = y0 + u_y height, x = x0 + u_x disp
 * (Coordinates.update_recycled_coordinates_vertical_boundary!).  Uniform pair j of `stream`. */
static void contraction_positions(int64_t n, int64_t asym, int air, double xsize, double ysize, double disp,
                                  double h_left, double h_right, uint64_t seed, int64_t step, uint32_t stream,
                                  double* newx, double* newy) {
  const int64_t nleft = asym ? 0 : n / 2;
  for (int64_t j = 0; j < n; ++j) {
    double ux, uy;
    o_recycle_uniforms(seed, step, stream, j, &ux, &uy);
    const int left = j < nleft;
    const double h = left ? h_left : h_right;
    const double y_initial = air ? 0.0 : h, y_height = air ? h : ysize - h;
    const double x_initial = left ? 0.0 : xsize, displacement_x = left ? disp : -disp;
    newy[j] = y_initial + uy * y_height;
    newx[j] = x_initial + ux * displacement_x;
  }
}

/* ContractionViscoelastic.execute_recycle_steps (marker_recycle/types/ContractionViscoelastic.jl:
 * 60-111): InitializeMarkerRecycling (outside markers in marker order, sticky by material),
 * ContractionRecycleLocations (sticky positions from stream 0, subsurface from stream 1),
 * Coordinates.reset_recycled_marker_coordinates (k-th marker of a group takes the k-th
 * position), get_subsurface_reset_properties_viscoelastic_contraction (material of the new
 * position, pressure PressureReset 3300 * 9.81 * y, temperature 0) and
 * ResetMarkers.reset_recycled_marker_properties!.
 * ids[]: sticky_air, sticky_water, layers[7], strong[3]; d[]: xsize, ysize,
 * full_velocity_contraction, timestep, sticky_thickness_left, sticky_thickness_right,
 * temperature_top, thick[6], x_left_strong, x_right_strong, delta_fric_coef.
 * newx/newy: scratch of M doubles each (positions of the sticky group, then the subsurface). */
int64_t o_recycle_contraction(int64_t M, const int8_t* inside, int16_t* matid, double** f, float* pfailure,
                              const int16_t* ids, const double* d, int64_t asym, int64_t nmat,
                              const double* mat_plastic, int64_t iuse_random_fric, uint64_t seed, int64_t step,
                              int64_t* list, int8_t* flags, double* newx, double* newy, int64_t* n_air) {
  const int16_t air = ids[0], water = ids[1];
  const double xsize = d[0], ysize = d[1];
  /* get_displacement_velocity: abs(v) * timestep * 0.5, or abs(v) * timestep */
  const double disp = asym ? fabs(d[2]) * d[3] : fabs(d[2]) * d[3] * 0.5;
  int64_t nout = 0, nair = 0, nsub = 0;
  for (int64_t m = 0; m < M; ++m)
    if (inside[m] != 1) {
      list[nout++] = m;
      if (matid[m] == air || matid[m] == water) ++nair; else ++nsub;
    }
  double *ax = newx, *ay = newy, *sx = newx + nair, *sy = newy + nair;
  contraction_positions(nair, asym, 1, xsize, ysize, disp, d[4], d[5], seed, step, 0u, ax, ay);
  contraction_positions(nsub, asym, 0, xsize, ysize, disp, d[4], d[5], seed, step, 1u, sx, sy);
  int64_t ia = 0, is = 0;
  for (int64_t k = 0; k < nout; ++k) {
    const int64_t m = list[k];
    const int sticky = (matid[m] == air || matid[m] == water) && nair > 0;
    if (sticky) { f[R_X][m] = ax[ia]; f[R_Y][m] = ay[ia]; ++ia; }
    else { f[R_X][m] = sx[is]; f[R_Y][m] = sy[is]; ++is; }
    flags[k] = (int8_t)(sticky ? 0 : 1);
    int16_t id;
    if (sticky) {
      id = air;
      f[R_TK][m] = d[6];
      f[R_PR][m] = 0.0;
      f[R_SXX][m] = f[R_SXY][m] = 0.0;
      f[R_EXX][m] = f[R_EXY][m] = 0.0;
      f[R_ETA][m] = 0.0;
    } else {
      id = contraction_define_material(f[R_X][m], f[R_Y][m], d + 7, d[13], d[14], ids + 2, ids + 9);
      f[R_TK][m] = 0.0;
      f[R_PR][m] = 3300.0 * 9.81 * f[R_Y][m];
      f[R_SXX][m] = f[R_SXY][m] = 1.96e6;
      f[R_EXX][m] = f[R_EXY][m] = 1e-14;
      f[R_ETA][m] = 1e20;
    }
    matid[m] = id;
    f[R_SR_RATIO][m] = 0.0;
    f[R_GII][m] = f[R_SP][m] = f[R_SRP][m] = 0.0;
    f[R_MELT][m] = 0.0;
    pfailure[m] = 0.0f;
    double fric = mat_plastic[2 * nmat + (id - 1)];
    if (!sticky && iuse_random_fric == 1) {
      double r, unused;
      o_recycle_uniforms(seed, step, 2u, m, &r, &unused);
      if (r <= 0.5) fric = fric - d[15];
    }
    f[R_FRIC_INI][m] = fric;
    f[R_FRIC][m] = fric;
    list[k] = m + 1;
  }
  *n_air = nair;
  return nout;
}

/* InflowRamp.calculate_ramp_factor: (y - top) / (bottom - top) inside [top, bottom), else 1 */
static double ramp_factor(double y, double top, double bottom) {
  return (top <= y && y < bottom) ? (y - top) / (bottom - top) : 1.0;
}

/* ExtensionInflowAndOutflowAlongSides.execute_recycling_steps (marker_recycle/types/
 * ExtensionInflowAndOutflowAlongSides.jl:20-237): sticky markers at the Extension top-band
 * positions (Extension.jl:58-73, stream 0), subsurface ones at the two sides (stream 1):
 * the first floor(n/2) at x0 = 0 with band |v_left| dt, the rest at x0 = xsize with band
 * -|v_right| dt; y0 = (sticky + plate) + smoothing of that side (InflowGeometry.jl), y = y0 +
 * u_y (ysize - y0) and x = x0 + u_x band f(y), f the ramp factor over [y0, y0 + smoothing)
 * (Coordinates.update_recycled_coordinates_vertical_inflow_outflow_boundary!).  Subsurface
 * properties: asthenosphere, 3300 * 9.81 * y, T_bottom - gradient ((ysize - y) / 1000).
 * d[]: xsize, ysize, vyu, timestep, temperature_top, temperature_bottom, sticky_left,
 * sticky_right, plate, smoothing, v_inflow_left, v_inflow_right, adiabatic_gradient,
 * delta_fric_coef; ids[]: sticky_air, sticky_water, asthenosphere. */
int64_t o_recycle_side_inflow(int64_t M, const int8_t* inside, int16_t* matid, double** f, float* pfailure,
                              const int16_t* ids, const double* d, int64_t nmat, const double* mat_plastic,
                              int64_t iuse_random_fric, uint64_t seed, int64_t step, int64_t* list, int8_t* flags,
                              double* newx, double* newy, int64_t* n_air) {
  const int16_t air = ids[0], water = ids[1], asth = ids[2];
  const double xsize = d[0], ysize = d[1], dt = d[3];
  int64_t nout = 0, nair = 0, nsub = 0;
  for (int64_t m = 0; m < M; ++m)
    if (inside[m] != 1) {
      list[nout++] = m;
      if (matid[m] == air || matid[m] == water) ++nair; else ++nsub;
    }
  double *ax = newx, *ay = newy, *sx = newx + nair, *sy = newy + nair;
  const double disp_upper = fabs(d[2] * dt);
  for (int64_t j = 0; j < nair; ++j) {
    double u0, u1;
    o_recycle_uniforms(seed, step, 0u, j, &u0, &u1);
    ay[j] = 0.0 + u1 * disp_upper;
    ax[j] = 0.0 + u0 * xsize;
  }
  const int64_t nleft = nsub / 2;
  for (int side = 0; side < 2; ++side) {
    const double sticky = side == 0 ? d[6] : d[7];
    const double y_initial = sticky + d[8] + d[9];           /* calculate_top_of_side_inflow */
    const double y_smooth_top = sticky + d[8] + d[9], y_smooth_bottom = y_smooth_top + d[9];
    const double y_height = ysize - y_initial;                /* get_y_height_of_inflow */
    const double x_initial = side == 0 ? 0.0 : xsize;
    const double displacement_x = side == 0 ? fabs(d[10]) * dt : -fabs(d[11]) * dt;
    const int64_t start = side == 0 ? 0 : nleft, count = side == 0 ? nleft : nsub - nleft;
    for (int64_t j = 0; j < count; ++j) {
      double ux, uy;
      o_recycle_uniforms(seed, step, 1u, start + j, &ux, &uy);
      sy[start + j] = y_initial + uy * y_height;
    }
    for (int64_t j = 0; j < count; ++j) {
      double ux, uy;
      o_recycle_uniforms(seed, step, 1u, start + j, &ux, &uy);
      const double rf = ramp_factor(sy[start + j], y_smooth_top, y_smooth_bottom);
      sx[start + j] = x_initial + ux * displacement_x * rf;
    }
  }
  int64_t ia = 0, is = 0;
  for (int64_t k = 0; k < nout; ++k) {
    const int64_t m = list[k];
    const int sticky = (matid[m] == air || matid[m] == water) && nair > 0;
    if (sticky) { f[R_X][m] = ax[ia]; f[R_Y][m] = ay[ia]; ++ia; }
    else { f[R_X][m] = sx[is]; f[R_Y][m] = sy[is]; ++is; }
    flags[k] = (int8_t)(sticky ? 0 : 1);
    const int16_t id = sticky ? air : asth;
    matid[m] = id;
    if (sticky) {
      f[R_TK][m] = d[4];
      f[R_PR][m] = 0.0;
      f[R_SXX][m] = f[R_SXY][m] = 0.0;
      f[R_EXX][m] = f[R_EXY][m] = 0.0;
      f[R_ETA][m] = 0.0;
    } else {
      const double dy_km = (ysize - f[R_Y][m]) / 1000.0;
      f[R_TK][m] = d[5] - d[12] * dy_km;
      f[R_PR][m] = 3300.0 * 9.81 * f[R_Y][m];
      f[R_SXX][m] = f[R_SXY][m] = 1.96e6;
      f[R_EXX][m] = f[R_EXY][m] = 1e-14;
      f[R_ETA][m] = 1e20;
    }
    f[R_SR_RATIO][m] = 0.0;
    f[R_GII][m] = f[R_SP][m] = f[R_SRP][m] = 0.0;
    f[R_MELT][m] = 0.0;
    pfailure[m] = 0.0f;
    double fric = mat_plastic[2 * nmat + (id - 1)];
    if (!sticky && iuse_random_fric == 1) {
      double r, unused;
      o_recycle_uniforms(seed, step, 2u, m, &r, &unused);
      if (r <= 0.5) fric = fric - d[13];
    }
    f[R_FRIC_INI][m] = fric;
    f[R_FRIC][m] = fric;
    list[k] = m + 1;
  }
  *n_air = nair;
  return nout;
}

/* FractureZone.define_material: the set_* rules in order, each overriding the previous id.
 * b[]: bases of sticky air, sediments, basaltic crust, gabbroic crust, younger, older and weak
 * lithosphere (define_geometry); id[]: air, sediment, basaltic, gabbroic, mantle lithosphere,
 * weak mantle lithosphere, asthenosphere. */
static int16_t fz_define_material(double x, double y, const double* b, double x_start, double x_end,
                                  const int16_t* id) {
  int16_t m = id[6];                                             /* set_asthenosphere */
  if (y <= b[0]) m = id[0];                                      /* set_sticky_air */
  if (b[0] < y && y <= b[1]) m = id[1];                          /* set_sediments */
  if (b[1] < y && y <= b[2]) m = id[2];                          /* set_basaltic_crust */
  if (b[2] < y && y <= b[3]) m = id[3];                          /* set_gabbroic_crust */
  const int younger = x < x_end && b[3] < y && y <= b[4];        /* in_younger_lithosphere */
  const int older = x >= x_end && b[3] < y && y <= b[5];         /* in_older_lithosphere */
  if (younger || older) m = id[4];                               /* set_lithosphere */
  const double x_weak_end = x_end + (b[3] - y) * 25.0;           /* get_x_end_of_weak_oceanic_crust */
  if (x_start < x && x < x_weak_end && (b[2] < y && y <= b[3])) m = id[2];
  if (x_start < x && x < x_end && b[3] < y && y <= b[6]) m = id[5];  /* set_weak_mantle_of_fracture_zone */
  return m;
}

/* calc_lithosphere_temperature with (kappa age)^0.5 as sqrt */
static double fz_lith_temp(double t_top, double t_bottom, double grad, double asth, double kappa, double depth,
                           double age) {
  const double t_base = t_bottom - grad * asth / 1000.0;
  return t_base + (t_top - t_base) * (1 - erf(depth / (2 * sqrt(kappa * age))));
}

/* exported for the known-answer test of the erf law (HalfSpaceCooling's form) */
double o_fz_lithosphere_temperature(double t_top, double t_bottom, double grad, double asth, double kappa,
                                    double depth, double age) {
  return fz_lith_temp(t_top, t_bottom, grad, asth, kappa, depth, age);
}

/* FractureZone.calculate_temperature(y, x, thermal_parameters); th[]: t_top, t_bottom, gradient,
 * x_end, age_left (s), age_right (s), sticky thickness, lithosphere depth left, right, kappa, ysize */
static double fz_calculate_temperature(double y, double x, const double* th) {
  const double t_top = th[0], t_bottom = th[1], grad = th[2], x_end = th[3], sticky = th[6];
  const double ysize = th[10], kappa = th[9];
  const double sub_sticky_depth = y - sticky;
  const double left_asth = ysize - th[7], right_asth = ysize - th[8];
  double t = t_bottom - (grad * (ysize - y) / 1000.0);
  if (y <= sticky) t = t_top;
  else if (0 < x && x < x_end && sticky < y && y < th[7])
    t = fz_lith_temp(t_top, t_bottom, grad, left_asth, kappa, sub_sticky_depth, th[4]);
  else if (x > x_end && sticky < y && y < th[8])
    t = fz_lith_temp(t_top, t_bottom, grad, right_asth, kappa, sub_sticky_depth, th[5]);
  return t;
}

/* ContractionFractureZone.execute_recycle_steps (marker_recycle/types/ContractionFractureZone.jl:
 * 11-61): positions as o_recycle_contraction, subsurface properties from
 * FractureZoneProperties.get_subsurface_reset_properties_fracture_zone (FractureZoneProperties.jl:
 * 17-55).  ids[]: sticky_air, sticky_water, fz ids[7]; d[]: xsize, ysize,
 * full_velocity_contraction, timestep, sticky_thickness_left, sticky_thickness_right,
 * temperature_top, temperature_bottom, adiabatic_gradient, fz thickness[7], x_fz_start, x_fz_end,
 * age_left (Myr), age_right (Myr), lithosphere depth left, right, kappa, delta_fric_coef. */
int64_t o_recycle_fracture_zone(int64_t M, const int8_t* inside, int16_t* matid, double** f, float* pfailure,
                                const int16_t* ids, const double* d, int64_t asym, int64_t nmat,
                                const double* mat_plastic, int64_t iuse_random_fric, uint64_t seed, int64_t step,
                                int64_t* list, int8_t* flags, double* newx, double* newy, int64_t* n_air) {
  const int16_t air = ids[0], water = ids[1];
  const double xsize = d[0], ysize = d[1];
  const double disp = asym ? fabs(d[2]) * d[3] : fabs(d[2]) * d[3] * 0.5;
  const double* t = d + 9;
  /* FractureZone.define_geometry */
  double b[7];
  b[0] = t[0];
  b[1] = b[0] + t[1];
  b[2] = b[1] + t[2];
  b[3] = b[2] + t[3];
  b[4] = b[3] + t[4];
  b[5] = b[3] + t[5];
  b[6] = b[3] + t[6];
  /* get_thermal_parameters (millions_of_years_to_seconds: (t 1e6) (365.25 24 3600)) */
  const double spy = 365.25 * 24.0 * 3600.0;
  const double th[11] = {d[6], d[7], d[8], d[17], (d[18] * 1e6) * spy, (d[19] * 1e6) * spy, t[0], d[20], d[21],
                         d[22], ysize};
  int64_t nout = 0, nair = 0, nsub = 0;
  for (int64_t m = 0; m < M; ++m)
    if (inside[m] != 1) {
      list[nout++] = m;
      if (matid[m] == air || matid[m] == water) ++nair; else ++nsub;
    }
  double *ax = newx, *ay = newy, *sx = newx + nair, *sy = newy + nair;
  contraction_positions(nair, asym, 1, xsize, ysize, disp, d[4], d[5], seed, step, 0u, ax, ay);
  contraction_positions(nsub, asym, 0, xsize, ysize, disp, d[4], d[5], seed, step, 1u, sx, sy);
  int64_t ia = 0, is = 0;
  for (int64_t k = 0; k < nout; ++k) {
    const int64_t m = list[k];
    const int sticky = (matid[m] == air || matid[m] == water) && nair > 0;
    if (sticky) { f[R_X][m] = ax[ia]; f[R_Y][m] = ay[ia]; ++ia; }
    else { f[R_X][m] = sx[is]; f[R_Y][m] = sy[is]; ++is; }
    flags[k] = (int8_t)(sticky ? 0 : 1);
    int16_t id;
    if (sticky) {
      id = air;
      f[R_TK][m] = d[6];
      f[R_PR][m] = 0.0;
      f[R_SXX][m] = f[R_SXY][m] = 0.0;
      f[R_EXX][m] = f[R_EXY][m] = 0.0;
      f[R_ETA][m] = 0.0;
    } else {
      id = fz_define_material(f[R_X][m], f[R_Y][m], b, d[16], d[17], ids + 2);
      f[R_TK][m] = fz_calculate_temperature(f[R_Y][m], f[R_X][m], th);
      f[R_PR][m] = 3300.0 * 9.81 * f[R_Y][m];
      f[R_SXX][m] = f[R_SXY][m] = 1.96e6;
      f[R_EXX][m] = f[R_EXY][m] = 1e-14;
      f[R_ETA][m] = 1e20;
    }
    matid[m] = id;
    f[R_SR_RATIO][m] = 0.0;
    f[R_GII][m] = f[R_SP][m] = f[R_SRP][m] = 0.0;
    f[R_MELT][m] = 0.0;
    pfailure[m] = 0.0f;
    double fric = mat_plastic[2 * nmat + (id - 1)];
    if (!sticky && iuse_random_fric == 1) {
      double r, unused;
      o_recycle_uniforms(seed, step, 2u, m, &r, &unused);
      if (r <= 0.5) fric = fric - d[23];
    }
    f[R_FRIC_INI][m] = fric;
    f[R_FRIC][m] = fric;
    list[k] = m + 1;
  }
  *n_air = nair;
  return nout;
}
