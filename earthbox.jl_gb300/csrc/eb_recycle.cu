// eb_recycle.cu -- recycling of markers that left the domain.
//
// Reference: MarkerRecycle.recycle_markers! (boundary_conditions/marker_recycle/MarkerRecycle.jl)
// for the extension models (LithosphericExtensionFixedBoundaries, ...Asymmetric,
// ...DepthDependent -> types/Extension.jl:14-129):
//   InitializeMarkerRecycling.initialize_recycling (utils/InitializeMarkerRecycling.jl): the
//     outside markers in marker order (GridFuncs.get_indices_of_markers_outside_domain),
//     split into sticky (air/water material) and subsurface;
//   Extension.calculate_recycled_locations (types/Extension.jl:53-97): sticky markers re-enter
//     at x = U xsize, y = U |vyu dt| (the top band), subsurface markers at x = U xsize,
//     y = ysize - U |vyl dt| (the bottom band);
//   Coordinates.reset_recycled_marker_coordinates (utils/Coordinates.jl): the k-th sticky
//     outside marker takes the k-th sticky position, likewise for subsurface;
//   ResetMarkers.reset_recycled_marker_properties! (utils/ResetMarkers.jl): sticky markers
//     become sticky air at temperature_top with zero pressure, stress, strain rate, strain,
//     melt and viscosity; subsurface markers become asthenosphere at temperature_bottom with
//     pressure 3300 * 9.81 * gridy_b[ynum] (PressureReset.jl), stress 1.96e6 Pa, strain rate
//     1e-14 1/s, viscosity 1e20 Pa s; both take fric_ini = fric = mat_plastic[matid, 3],
//     minus delta_fric_coef when random friction is on and the marker's random number is
//     <= 0.5 (FrictionRandomizer.randomize_initial_friction_coefficient).
//
// Random numbers.  The reference draws them from Julia's global generator (unseeded); here
// every uniform comes from Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC 2011) keyed by a caller seed, counter (j, stream, step):
// stream 0 gives the j-th sticky position, stream 1 the j-th subsurface position, stream 2
// marker j's friction number.  The same numbers in the oracle give the same results.
// Built with -fmad=false: ysize + u * (-|vyl dt|) is rounded twice, as Julia evaluates it.
#include "eb_internal.h"

#include <cmath>
#include <vector>

namespace {

constexpr int kB = 256;

// Philox-4x32-10: ten rounds of two 32x32->64 multiplies and a Weyl-sequence key schedule.
__host__ __device__ inline void philox4x32(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n1 = lo1, n2 = hi0 ^ c[3] ^ k1, n3 = lo0;
    c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}
// two uniforms in [0, 1) with 53 random bits each
__host__ __device__ inline void uniforms(uint64_t seed, int64_t step, uint32_t stream, int64_t j, double& u0,
                                        double& u1) {
  uint32_t c[4] = {(uint32_t)j, (uint32_t)((uint64_t)j >> 32), stream, (uint32_t)step};
  philox4x32(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  u0 = (double)((((uint64_t)c[0] << 32) | c[1]) >> 11) * 0x1p-53;
  u1 = (double)((((uint64_t)c[2] << 32) | c[3]) >> 11) * 0x1p-53;
}

struct RecycleK {
  int32_t type;                                 // 1 extension, 2 extension without bottom inflow, 3 channel,
                                                // 4 contraction
  int16_t sticky_air, sticky_water, asth;
  double xsize, ysize, disp_top, disp_bottom;  // disp_top = |vyu dt|, disp_bottom = -|vyl dt|
  double t_top, t_bottom, p_reset;
  double gridy_max, ysize_grid;                 // channel: gridy_b[ynum], gridy_b[ynum] - gridy_b[1]
  double fric_air, fric_asth;                   // mat_plastic[., 3]
  int32_t random_fric;
  double delta_fric;
  uint64_t seed;
  int64_t step;
  // contraction: side band, sticky thickness at the two sides, layer bases (cumulative
  // thicknesses), strong-zone limits and the seven-layer / strong-zone material ids
  int32_t asym;
  double disp_side, sticky_l, sticky_r;
  double depth[6];
  double x_left_strong, x_right_strong;
  int16_t layer_id[7], strong_id[3];
  // side inflow: top of the inflow zone (= top of the ramp) and base of the ramp per side,
  // inflow bands |v_left| dt and -|v_right| dt, adiabatic gradient (K/km)
  double in_top_l, in_top_r, ramp_bot_l, ramp_bot_r, disp_in_l, disp_in_r, adiabatic;
  // fracture zone: layer bases (sticky air, sediments, basaltic crust, gabbroic crust, younger,
  // older and weak lithosphere), zone limits, material ids, and the thermal model
  double fz_base[7], x_fz_start, x_fz_end;
  int16_t fz_id[7];  // air, sediment, basaltic, gabbroic, mantle lithosphere, weak mantle, asthenosphere
  double kappa, age_l, age_r, tld_l, tld_r, t_top_fz;
};

// FractureZone.define_material (marker_materials/init_manager/types/FractureZone.jl:103-299):
// asthenosphere, then each rule in turn overrides the id where it applies.
__device__ int16_t fz_material(double x, double y, const RecycleK& p) {
  const double* b = p.fz_base;
  int16_t id = p.fz_id[6];
  if (y <= b[0]) id = p.fz_id[0];
  if (b[0] < y && y <= b[1]) id = p.fz_id[1];
  if (b[1] < y && y <= b[2]) id = p.fz_id[2];
  if (b[2] < y && y <= b[3]) id = p.fz_id[3];
  const bool younger = x < p.x_fz_end && b[3] < y && y <= b[4];
  const bool older = x >= p.x_fz_end && b[3] < y && y <= b[5];
  if (younger || older) id = p.fz_id[4];
  // weak gabbroic crust: basaltic-crust material up to x_end + (base of gabbro - y) * 25
  const double x_weak_end = p.x_fz_end + (b[3] - y) * 25.0;
  if (p.x_fz_start < x && x < x_weak_end && b[2] < y && y <= b[3]) id = p.fz_id[2];
  if (p.x_fz_start < x && x < p.x_fz_end && b[3] < y && y <= b[6]) id = p.fz_id[5];
  return id;
}
// FractureZone.calculate_temperature (markers/temperature/init_manager/types/FractureZone.jl:
// 107-202): adiabat, T_top in the sticky layer, half-space cooling of the plate's age on either
// side of x_end (sqrt(kappa age) for the reference's (kappa age)^0.5)
__device__ double fz_lith_temperature(const RecycleK& p, double asth_thickness, double depth, double age) {
  const double t_base = p.t_bottom - p.adiabatic * asth_thickness / 1000.0;
  return t_base + (p.t_top_fz - t_base) * (1 - erf(depth / (2 * sqrt(p.kappa * age))));
}
__device__ double fz_temperature(double x, double y, const RecycleK& p) {
  const double sticky = p.fz_base[0];
  const double sub = y - sticky;
  double t = p.t_bottom - (p.adiabatic * (p.ysize - y) / 1000.0);
  if (y <= sticky) t = p.t_top_fz;
  else if (0 < x && x < p.x_fz_end && sticky < y && y < p.tld_l)
    t = fz_lith_temperature(p, p.ysize - p.tld_l, sub, p.age_l);
  else if (x > p.x_fz_end && sticky < y && y < p.tld_r)
    t = fz_lith_temperature(p, p.ysize - p.tld_r, sub, p.age_r);
  return t;
}

// SevenLayerEarthModel2D.define_material (marker_materials/init_manager/utils/
// SevenLayerEarthModel2D.jl:20-62) followed by StrongRegions.define_material
// (init_manager/utils/StrongRegions.jl:24-80), as ContractionViscoelastic.define_material
// applies them (types/ContractionViscoelastic.jl:113-134, strong zones on).
__device__ int16_t contraction_material(double x, double y, const RecycleK& p) {
  const double* d = p.depth;
  int16_t id = p.layer_id[6];
  if (y <= d[0]) id = p.layer_id[0];
  else if (y > d[0] && y <= d[1]) id = p.layer_id[1];
  else if (y > d[1] && y <= d[2]) id = p.layer_id[2];
  else if (y > d[2] && y <= d[3]) id = p.layer_id[3];
  else if (y > d[3] && y <= d[4]) id = p.layer_id[4];
  else if (y > d[4] && y <= d[5]) id = p.layer_id[5];
  const bool outside = x < p.x_left_strong || x > p.x_right_strong;
  if (d[0] < y && y <= d[1]) {
    if (outside) id = p.strong_id[0];
  } else if (d[1] < y && y <= d[2]) {
    if (outside) id = p.strong_id[1];
  } else if (d[2] < y && y <= d[3]) {
    if (outside) id = p.strong_id[2];
  } else if (d[3] < y && y <= d[4]) {
    if (outside) id = p.strong_id[2];
  } else if (d[4] < y && y <= d[5]) {
    if (outside) id = p.strong_id[2];
  }
  return id;
}

__device__ __forceinline__ bool sticky(int16_t m, const RecycleK& p) { return m == p.sticky_air || m == p.sticky_water; }
// the markers a recycling type moves: outside the domain, or (channel) below the grid
__device__ __forceinline__ bool selected(const DevMarkers& mk, int64_t m, const RecycleK& p) {
  if (m >= mk.M) return false;
  return p.type == 3 ? mk.y[m] > p.gridy_max : mk.inside[m] != 1;
}
// sticky rank (air/water positions): extension and contraction; the other types treat every
// marker alike
__device__ __forceinline__ bool sticky_sel(const DevMarkers& mk, int64_t m, const RecycleK& p) {
  return (p.type == 1 || p.type >= 4) && sticky(mk.matid[m], p);
}

// per block: number of outside markers and of outside sticky markers
__global__ void k_recycle_count(DevMarkers mk, RecycleK p, int32_t* __restrict__ counts, int32_t nblocks) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool out = selected(mk, m, p);
  const bool st = out && sticky_sel(mk, m, p);
  const int n_out = __syncthreads_count(out), n_st = __syncthreads_count(st);
  if (threadIdx.x == 0) {
    counts[blockIdx.x] = n_out;
    counts[nblocks + blockIdx.x] = n_st;
  }
}

// ranks in marker order, new positions and property resets; list[r] = 1-based index
__global__ void k_recycle_apply(DevMarkers mk, DevMats mt, RecycleK p, const int32_t* __restrict__ offsets,
                                int32_t nblocks, int64_t n_out, int64_t n_air, int64_t* __restrict__ list,
                                int8_t* __restrict__ flags) {
  __shared__ int32_t s_out[kB / 32], s_st[kB / 32];
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool out = selected(mk, m, p);
  const bool st = out && sticky_sel(mk, m, p);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned b_out = __ballot_sync(0xffffffffu, out), b_st = __ballot_sync(0xffffffffu, st);
  if (lane == 0) { s_out[w] = __popc(b_out); s_st[w] = __popc(b_st); }
  __syncthreads();
  if (!out) return;
  int32_t r_out = offsets[blockIdx.x], r_st = offsets[nblocks + blockIdx.x];
  for (int k = 0; k < w; ++k) { r_out += s_out[k]; r_st += s_st[k]; }
  const unsigned below = (1u << lane) - 1u;
  r_out += __popc(b_out & below);
  r_st += __popc(b_st & below);
  if (p.type == 3) {
    // Channel.execute_recycle_steps (types/Channel.jl:20-54): wrap to the top, shift T
    mk.y[m] = mk.y[m] - p.ysize_grid;
    mk.tk[m] = mk.tk[m] + p.t_top - p.t_bottom;
    list[r_out] = m + 1;
    flags[r_out] = 1;
    return;
  }
  double ux, uy;
  if (p.type == 2) {
    // ExtensionNoBottomInflow (types/ExtensionNoBottomInflow.jl:25-123): every outside marker
    // re-enters in the top band, one uniform for both coordinates, as sticky air
    uniforms(p.seed, p.step, 0u, r_out, ux, uy);
    mk.y[m] = ux * p.disp_top;
    mk.x[m] = 0.0 + ux * p.xsize;
    list[r_out] = m + 1;
    flags[r_out] = 0;
    mk.matid[m] = p.sticky_air;
    mk.tk[m] = p.t_top;
    mk.pr[m] = 0.0;
    mk.sxx[m] = 0.0; mk.sxy[m] = 0.0;
    mk.exx[m] = 0.0; mk.exy[m] = 0.0;
    mk.eta[m] = 0.0;
    mk.sr_ratio[m] = 0.0;
    mk.gii[m] = 0.0; mk.sp[m] = 0.0; mk.srp[m] = 0.0;
    mk.melt[m] = 0.0;
    mk.pfailure[m] = 0.0f;
    mk.fric_ini[m] = p.fric_air;
    mk.fric[m] = p.fric_air;
    return;
  }
  if (p.type == 4 || p.type == 6) {
    // ContractionViscoelastic / ContractionFractureZone .execute_recycle_steps (types/ContractionViscoelastic.jl:60-111):
    // the k-th sticky / subsurface marker takes the k-th position of its group; the first
    // floor(n/2) of a group (none when asymmetric) enter at the left side, x = 0 + u d,
    // the others at the right, x = xsize + u (-d) (ContractionRecycleLocations.jl:9-140);
    // sticky markers in y = 0 + u h, subsurface ones in y = h + u (ysize - h), h the sticky
    // thickness of that side.
    const bool air = st;
    const int64_t r = air ? (int64_t)r_st : (int64_t)r_out - r_st;
    const int64_t ngrp = air ? n_air : n_out - n_air;
    const int64_t nleft = p.asym ? 0 : ngrp / 2;
    uniforms(p.seed, p.step, air ? 0u : 1u, r, ux, uy);
    const bool left = r < nleft;
    const double h = left ? p.sticky_l : p.sticky_r;
    const double x = (left ? 0.0 : p.xsize) + ux * (left ? p.disp_side : -p.disp_side);
    const double y = air ? 0.0 + uy * h : h + uy * (p.ysize - h);
    mk.x[m] = x;
    mk.y[m] = y;
    list[r_out] = m + 1;
    flags[r_out] = air ? 0 : 1;
    double fric;
    if (air) {
      mk.matid[m] = p.sticky_air;
      mk.tk[m] = p.t_top;
      mk.pr[m] = 0.0;
      mk.sxx[m] = 0.0; mk.sxy[m] = 0.0;
      mk.exx[m] = 0.0; mk.exy[m] = 0.0;
      mk.eta[m] = 0.0;
      fric = p.fric_air;
    } else {
      // get_subsurface_reset_properties_viscoelastic_contraction (ContractionViscoelastic.jl:
      // 69-111): material at the new position, pressure 3300 * 9.81 * y, temperature 0
      // (fracture zone: FractureZoneProperties.jl:17-55, material and temperature of the
      // fracture-zone initial model)
      const int16_t id = p.type == 4 ? contraction_material(x, y, p) : fz_material(x, y, p);
      mk.matid[m] = id;
      mk.tk[m] = p.type == 4 ? 0.0 : fz_temperature(x, y, p);
      mk.pr[m] = 3300.0 * 9.81 * y;
      mk.sxx[m] = 1.96e6; mk.sxy[m] = 1.96e6;
      mk.exx[m] = 1e-14; mk.exy[m] = 1e-14;
      mk.eta[m] = 1e20;
      fric = __ldg(&mt.plastic[2 * (size_t)mt.nmat + (id - 1)]);  // mat_plastic[id, 3]
      if (p.random_fric == 1) {
        double r0, r1;
        uniforms(p.seed, p.step, 2u, m, r0, r1);
        if (r0 <= 0.5) fric = fric - p.delta_fric;
      }
    }
    mk.sr_ratio[m] = 0.0;
    mk.gii[m] = 0.0; mk.sp[m] = 0.0; mk.srp[m] = 0.0;
    mk.melt[m] = 0.0;
    mk.pfailure[m] = 0.0f;
    mk.fric_ini[m] = fric;
    mk.fric[m] = fric;
    return;
  }
  if (p.type == 5 && !st) {
    // ExtensionInflowAndOutflowAlongSides (types/ExtensionInflowAndOutflowAlongSides.jl:
    // 20-237): the first floor(n/2) subsurface markers enter at the left side, the others at
    // the right, y = y0 + u (ysize - y0) below the plate and smoothing layer
    // (InflowGeometry.jl), x = x0 + u d f with the ramp factor f of the new depth
    // (InflowRamp.calculate_ramp_factor; Coordinates.jl:155-200); asthenosphere at pressure
    // 3300 * 9.81 * y and T_bottom - gradient (ysize - y) / 1000.
    const int64_t r = (int64_t)r_out - r_st, nleft = (n_out - n_air) / 2;
    uniforms(p.seed, p.step, 1u, r, ux, uy);
    const bool left = r < nleft;
    const double y0 = left ? p.in_top_l : p.in_top_r, yb = left ? p.ramp_bot_l : p.ramp_bot_r;
    const double y = y0 + uy * (p.ysize - y0);
    const double f = (y0 <= y && y < yb) ? (y - y0) / (yb - y0) : 1.0;
    mk.x[m] = (left ? 0.0 : p.xsize) + ux * (left ? p.disp_in_l : p.disp_in_r) * f;
    mk.y[m] = y;
    list[r_out] = m + 1;
    flags[r_out] = 1;
    mk.matid[m] = p.asth;
    mk.tk[m] = p.t_bottom - p.adiabatic * ((p.ysize - y) / 1000.0);
    mk.pr[m] = 3300.0 * 9.81 * y;
    mk.sxx[m] = 1.96e6; mk.sxy[m] = 1.96e6;
    mk.exx[m] = 1e-14; mk.exy[m] = 1e-14;
    mk.eta[m] = 1e20;
    double fric = p.fric_asth;
    if (p.random_fric == 1) {
      double r0, r1;
      uniforms(p.seed, p.step, 2u, m, r0, r1);
      if (r0 <= 0.5) fric = fric - p.delta_fric;
    }
    mk.sr_ratio[m] = 0.0;
    mk.gii[m] = 0.0; mk.sp[m] = 0.0; mk.srp[m] = 0.0;
    mk.melt[m] = 0.0;
    mk.pfailure[m] = 0.0f;
    mk.fric_ini[m] = fric;
    mk.fric[m] = fric;
    return;
  }
  if (st && n_air > 0) {
    uniforms(p.seed, p.step, 0u, r_st, ux, uy);
    mk.x[m] = 0.0 + ux * p.xsize;
    mk.y[m] = 0.0 + uy * p.disp_top;
  } else {
    const int64_t r_sub = (int64_t)r_out - r_st;
    uniforms(p.seed, p.step, 1u, r_sub, ux, uy);
    mk.x[m] = 0.0 + ux * p.xsize;
    mk.y[m] = p.ysize + uy * p.disp_bottom;
  }
  list[r_out] = m + 1;
  flags[r_out] = st ? 0 : 1;
  double fric;
  if (st) {
    mk.matid[m] = p.sticky_air;
    mk.tk[m] = p.t_top;
    mk.pr[m] = 0.0;
    mk.sxx[m] = 0.0; mk.sxy[m] = 0.0;
    mk.exx[m] = 0.0; mk.exy[m] = 0.0;
    mk.eta[m] = 0.0;
    fric = p.fric_air;
  } else {
    mk.matid[m] = p.asth;
    mk.tk[m] = p.t_bottom;
    mk.pr[m] = p.p_reset;
    mk.sxx[m] = 1.96e6; mk.sxy[m] = 1.96e6;
    mk.exx[m] = 1e-14; mk.exy[m] = 1e-14;
    mk.eta[m] = 1e20;
    fric = p.fric_asth;
    if (p.random_fric == 1) {
      double r0, r1;
      uniforms(p.seed, p.step, 2u, m, r0, r1);
      if (r0 <= 0.5) fric = fric - p.delta_fric;
    }
  }
  mk.sr_ratio[m] = 0.0;
  mk.gii[m] = 0.0; mk.sp[m] = 0.0; mk.srp[m] = 0.0;
  mk.melt[m] = 0.0;
  mk.pfailure[m] = 0.0f;
  mk.fric_ini[m] = fric;
  mk.fric[m] = fric;
}

}  // namespace

// shared with the oracle test: the uniforms of (seed, step, stream, j)
extern "C" void eb_recycle_uniforms(uint64_t seed, int64_t step, uint32_t stream, int64_t j, double* u0, double* u1) {
  uniforms(seed, step, stream, j, *u0, *u1);
}

extern "C" int eb_recycle_markers(eb_ctx* c, const eb_recycle_params* rp, int64_t* nrecycle_air,
                                  int64_t* nrecycle_subsurface) {
  if (!c || !rp) return EB_BAD_INPUT;
  if (!c->have_grid || !c->have_params || !c->have_mats) return eb_fail(c, EB_NOT_READY, "grid, parameters and materials must be set");
  if (rp->recycle_type < 1 || rp->recycle_type > 6)
    return eb_fail(c, EB_BAD_INPUT, "recycle_type must be 1 (extension), 2 (extension without bottom inflow), "
                                    "3 (channel), 4 (contraction), 5 (extension with side inflow and outflow) "
                                    "or 6 (fracture-zone contraction)");
  const int64_t nmat = c->mats.nmat;
  std::vector<int64_t> ids = {rp->matid_sticky_air, rp->matid_sticky_water, rp->matid_asthenosphere};
  if (rp->recycle_type == 4) {
    ids.insert(ids.end(), rp->matid_layers, rp->matid_layers + 7);
    ids.insert(ids.end(), rp->matid_strong, rp->matid_strong + 3);
  }
  if (rp->recycle_type == 6) ids.insert(ids.end(), rp->matid_fz, rp->matid_fz + 7);
  for (int64_t id : ids)
    if (id < 1 || id > nmat) return eb_fail(c, EB_BAD_INPUT, "recycle material id outside the material table");
  if (c->M > 0 && c->matid_min < 1) return eb_fail(c, EB_NOT_READY, "marker_matid has not been uploaded");
  cudaSetDevice(c->device);
  int rc;
  const int need[] = {EB_M_INSIDE, EB_M_MATID, EB_M_X, EB_M_Y, EB_M_TK, EB_M_PR, EB_M_SXX, EB_M_SXY, EB_M_EXX, EB_M_EXY,
                      EB_M_ETA, EB_M_SR_RATIO, EB_M_GII, EB_M_STRAIN_PLASTIC, EB_M_STRAIN_RATE_PLASTIC, EB_M_MELTFRAC,
                      EB_M_PFAILURE, EB_M_FRIC_INI, EB_M_FRIC};
  for (int f : need)
    if ((rc = ensure_marker_field(c, f))) return rc;
  if (nrecycle_air) *nrecycle_air = 0;
  if (nrecycle_subsurface) *nrecycle_subsurface = 0;
  c->recycle_n = 0;
  if (c->M == 0) return EB_OK;
  const int32_t nblocks = (int32_t)((c->M + kB - 1) / kB);
  int32_t* d_counts = nullptr;
  EB_CK(c, cudaMalloc(&d_counts, 2 * (size_t)nblocks * sizeof(int32_t)));
  // mat_plastic[., 3] (sin of the initial friction angle) of the two reset materials
  std::vector<double>& mp = c->h_mat_plastic;
  // top band: |vyu dt| (extension), vyu dt with its sign (no bottom inflow)
  const double disp_top = rp->recycle_type == 2 ? rp->velocity_y_upper * c->P.timestep
                                                : std::fabs(rp->velocity_y_upper * c->P.timestep);
  RecycleK p{rp->recycle_type, (int16_t)rp->matid_sticky_air, (int16_t)rp->matid_sticky_water,
             (int16_t)rp->matid_asthenosphere, rp->xsize, rp->ysize, disp_top,
             -std::fabs(rp->velocity_y_lower * c->P.timestep), c->P.temperature_top, rp->temperature_bottom,
             3300.0 * 9.81 * c->h_gy.back(), c->h_gy.back(), c->h_gy.back() - c->h_gy.front(),
             mp[2 * nmat + rp->matid_sticky_air - 1], mp[2 * nmat + rp->matid_asthenosphere - 1],
             rp->iuse_random_fric, rp->delta_fric_coef, rp->seed, rp->counter};
  if (rp->recycle_type == 4 || rp->recycle_type == 6) {
    // ContractionRecycleLocations.get_displacement_velocity: |v| dt / 2, or |v| dt asymmetric
    p.asym = rp->asymmetric ? 1 : 0;
    p.disp_side = p.asym ? std::fabs(rp->full_velocity_contraction) * c->P.timestep
                         : std::fabs(rp->full_velocity_contraction) * c->P.timestep * 0.5;
    p.sticky_l = rp->sticky_thickness_left;
    p.sticky_r = rp->sticky_thickness_right;
    // Layers.calc_depths_for_layers (markers/utils/Layers.jl:31-54): running sums
    double base = rp->layer_thickness[0];
    p.depth[0] = base;
    for (int k = 1; k < 6; ++k) p.depth[k] = base = base + rp->layer_thickness[k];
    p.x_left_strong = rp->x_left_strong;
    p.x_right_strong = rp->x_right_strong;
    for (int k = 0; k < 7; ++k) p.layer_id[k] = (int16_t)rp->matid_layers[k];
    for (int k = 0; k < 3; ++k) p.strong_id[k] = (int16_t)rp->matid_strong[k];
  }
  if (rp->recycle_type == 6) {
    // FractureZone.define_geometry: bases as running sums from the sticky layer / gabbro base
    const double* t = rp->fz_thickness;
    p.fz_base[0] = t[0];
    p.fz_base[1] = p.fz_base[0] + t[1];
    p.fz_base[2] = p.fz_base[1] + t[2];
    p.fz_base[3] = p.fz_base[2] + t[3];
    p.fz_base[4] = p.fz_base[3] + t[4];
    p.fz_base[5] = p.fz_base[3] + t[5];
    p.fz_base[6] = p.fz_base[3] + t[6];
    p.x_fz_start = rp->x_fracture_zone_start;
    p.x_fz_end = rp->x_fracture_zone_end;
    for (int k = 0; k < 7; ++k) p.fz_id[k] = (int16_t)rp->matid_fz[k];
    // get_thermal_parameters: ages in Myr -> s (ConversionFuncs.millions_of_years_to_seconds)
    const double seconds_per_year = 365.25 * 24.0 * 3600.0;
    p.age_l = (rp->age_lithosphere_left * 1e6) * seconds_per_year;
    p.age_r = (rp->age_lithosphere_right * 1e6) * seconds_per_year;
    p.tld_l = rp->thermal_lithosphere_depth_left;
    p.tld_r = rp->thermal_lithosphere_depth_right;
    p.kappa = rp->thermal_diffusivity;
    p.adiabatic = rp->adiabatic_gradient;
    p.t_top_fz = c->P.temperature_top;
  }
  if (rp->recycle_type == 5) {
    // InflowGeometry.calculate_top_of_side_inflow / InflowRamp.get_top_and_bottom_of_inflow_ramp:
    // (sticky + plate) + smoothing, and that + smoothing
    p.in_top_l = rp->sticky_thickness_left + rp->plate_thickness + rp->smoothing_thickness;
    p.in_top_r = rp->sticky_thickness_right + rp->plate_thickness + rp->smoothing_thickness;
    p.ramp_bot_l = p.in_top_l + rp->smoothing_thickness;
    p.ramp_bot_r = p.in_top_r + rp->smoothing_thickness;
    p.disp_in_l = std::fabs(rp->velocity_inflow_left) * c->P.timestep;
    p.disp_in_r = -std::fabs(rp->velocity_inflow_right) * c->P.timestep;
    p.adiabatic = rp->adiabatic_gradient;
  }
  k_recycle_count<<<nblocks, kB, 0, c->stream>>>(dev_markers(c), p, d_counts, nblocks);
  c->launches++;
  std::vector<int32_t> h(2 * (size_t)nblocks);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), d_counts, h.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) { cudaFree(d_counts); return eb_cuda(c, e, "recycle count"); }
  int64_t n_out = 0, n_air = 0;
  for (int32_t b = 0; b < nblocks; ++b) {
    const int32_t o = h[b], s = h[nblocks + b];
    h[b] = (int32_t)n_out;
    h[nblocks + b] = (int32_t)n_air;
    n_out += o;
    n_air += s;
  }
  if (n_out > 0) {
    if ((size_t)n_out > c->recycle_cap) {
      cudaFree(c->recycle_list);
      cudaFree(c->recycle_flags);
      c->recycle_list = nullptr;
      c->recycle_flags = nullptr;
      c->recycle_cap = 0;
      e = cudaMalloc(&c->recycle_list, n_out * sizeof(int64_t));
      if (e == cudaSuccess) e = cudaMalloc(&c->recycle_flags, n_out * sizeof(int8_t));
      if (e != cudaSuccess) { cudaFree(d_counts); return eb_cuda(c, e, "recycle list"); }
      c->recycle_cap = (size_t)n_out;
    }
    e = cudaMemcpyAsync(d_counts, h.data(), h.size() * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
      EB_PROF(c, "k_recycle_apply");
      k_recycle_apply<<<nblocks, kB, 0, c->stream>>>(dev_markers(c), c->mats, p, d_counts, nblocks, n_out, n_air,
                                                     c->recycle_list, c->recycle_flags);
      c->launches++;
      prof_end(c);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  }
  cudaFree(d_counts);
  if (e != cudaSuccess) return eb_cuda(c, e, "marker recycling");
  c->recycle_n = n_out;
  c->located = false;  // markers moved
  if (rp->recycle_type == 2) n_air = n_out;  // every recycled marker becomes sticky air
  if (nrecycle_air) *nrecycle_air = n_air;
  if (nrecycle_subsurface) *nrecycle_subsurface = n_out - n_air;
  return EB_OK;
}

extern "C" int eb_recycled_markers(eb_ctx* c, int64_t* indices, int8_t* flags, int64_t capacity, int64_t* n) {
  if (!c) return EB_BAD_INPUT;
  if (n) *n = c->recycle_n;
  if (!indices || !flags || c->recycle_n == 0) return EB_OK;
  if (capacity < c->recycle_n) return eb_fail(c, EB_BAD_INPUT, "recycled-marker arrays too small");
  cudaSetDevice(c->device);
  EB_CK(c, cudaMemcpy(indices, c->recycle_list, c->recycle_n * sizeof(int64_t), cudaMemcpyDeviceToHost));
  EB_CK(c, cudaMemcpy(flags, c->recycle_flags, c->recycle_n * sizeof(int8_t), cudaMemcpyDeviceToHost));
  return EB_OK;
}
