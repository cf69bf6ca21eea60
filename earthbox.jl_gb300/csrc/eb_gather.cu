// eb_gather.cu -- grid -> marker bilinear gathers (coalesced SoA passes).
//
// Reference: GridToMarker.get_marker_value (src/interpolation/utils/GridToMarker.jl:190-226),
// GridTemperatureToMarkers.interpolate! (GridTemperatureToMarkers.jl:18-45),
// MarkerStrainRate.jl:23-69, MarkerStrainRateRatio.jl:191-322, MarkerPressure.jl:17-54,
// StressCorrection.jl:35-82, MarkerTemperature.jl:18-45.
// The post-Stokes marker gathers (strain rate, strain-rate ratio, pressure) are
// one pass here instead of three.  Weights and sums run in FP32 on FP64 grid
// values; results are stored in FP64.
#include "eb_internal.h"

namespace {

constexpr int kBlock = 256;


__global__ void k_gather_temperature(DevMarkers mk, DevGrid g, const float* __restrict__ tk1) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= mk.M || !(mk.mflags[m] & MF_INSIDE)) return;
  mk.tk[m] = f2d(gather4f(tk1, g.ynum, mk.yn[m], mk.xn[m], mk.fx[m], mk.fy[m]));
}

struct PostStokesGrids {
  const float *exx, *exy, *sxx2, *sxy2, *dsxx, *dsxy, *pr1;
  const double* mat_mu;
  float dt;
};

// The marker loads (flags, cell, offsets, material, viscosity) are all issued before the
// first store, which could alias them: one DRAM round trip per marker instead of three.
__global__ void k_post_stokes(DevMarkers mk, DevGrid g, PostStokesGrids G) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= mk.M) return;
  const uint8_t flags = __ldg(&mk.mflags[m]);
  const int32_t ix = __ldg(&mk.xn[m]), iy = __ldg(&mk.yn[m]);
  const float fx = __ldg(&mk.fx[m]), fy = __ldg(&mk.fy[m]);
  const int16_t matid = __ldg(&mk.matid[m]);
  const double eta64 = __ldg(&mk.eta[m]);
  if (!(flags & MF_INSIDE)) return;
  const float lx = fx * __ldg(&g.sxf[ix - 1]), ly = fy * __ldg(&g.syf[iy - 1]);
  // MarkerStrainRate.calculate_marker_strain_rate!
  const float exx = gather_p(G.exx, g, ix, iy, lx, ly);
  const float exy = gather4f(G.exy, g.ynum, iy, ix, fx, fy);
  mk.exx[m] = f2d(exx);
  mk.exy[m] = f2d(exy);
  // MarkerStrainRateRatio.calculate_marker_strain_rate_ratio! / marker_strain_rate_ratio
  const float sxx2 = gather_p(G.sxx2, g, ix, iy, lx, ly);
  const float sxy2 = gather4f(G.sxy2, g.ynum, iy, ix, fx, fy);
  const float dsxx = gather_p(G.dsxx, g, ix, iy, lx, ly);
  const float dsxy = gather4f(G.dsxy, g.ynum, iy, ix, fx, fy);
  const float mu = d2f(__ldg(&G.mat_mu[matid - 1]));
  const float eta = d2f(eta64);
  const float eii = hypotf(exx, exy);
  float r = 1.f;
  if (eii > 0.f) {
    const float tf = 1.f / (G.dt * mu);
    const float a = 0.5f * (sxx2 / eta + dsxx * tf);
    const float b = 0.5f * (sxy2 / eta + dsxy * tf);
    r = hypotf(a, b) / eii;
  }
  mk.sr_ratio[m] = f2d(r);
  // MarkerPressure.calculate_marker_pressure!
  mk.pr[m] = f2d(gather_p(G.pr1, g, ix, iy, lx, ly));
}

__global__ void k_stress_correction(DevMarkers mk, DevGrid g, const float* __restrict__ dsxy,
                                    const float* __restrict__ dsxx) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= mk.M || !(mk.mflags[m] & MF_INSIDE)) return;
  const int32_t ix = mk.xn[m], iy = mk.yn[m];
  const float fx = mk.fx[m], fy = mk.fy[m];
  const float lx = fx * __ldg(&g.sxf[ix - 1]), ly = fy * __ldg(&g.syf[iy - 1]);
  mk.sxy[m] = mk.sxy[m] + f2d(gather4f(dsxy, g.ynum, iy, ix, fx, fy));
  mk.sxx[m] = mk.sxx[m] + f2d(gather_p(dsxx, g, ix, iy, lx, ly));
}

__global__ void k_add_dt(DevMarkers mk, DevGrid g, const float* __restrict__ dtk1) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= mk.M || !(mk.mflags[m] & MF_INSIDE)) return;
  mk.tk[m] = mk.tk[m] + f2d(gather4f(dtk1, g.ynum, mk.yn[m], mk.xn[m], mk.fx[m], mk.fy[m]));
}

// GridViscoplasticityToMarkers.calc_marker_viscoplastic_viscosity!
// (src/rheology/plastic_failure/nodes/GridViscoplasticityToMarkers.jl:7-118): a marker whose
// basic cell has a yielding corner takes the harmonic average of etas1 over the yielding
// corners (weights plastic_yield x bilinear weight, numerator their sum) when that is below
// its flow viscosity, and is marked as failed; every other inside marker takes its flow
// viscosity.  Run once per time step of the nodal Picard variant, so it is done in FP64
// with the reference's normalised distances (MarkerGridMapping.jl:185-219): the harmonic
// average over corners whose viscosities differ by orders of magnitude amplifies an error in
// the weight of the weakest corner, and the comparison with the flow viscosity decides the
// failure flag.
__global__ void k_marker_eta_vp(DevMarkers mk, DevGrid g, const double* __restrict__ plastic_yield,
                                const double* __restrict__ etas1) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= mk.M || !(mk.mflags[m] & MF_INSIDE)) return;
  const int32_t ynum = g.ynum;
  const int32_t ix = mk.xn[m], iy = mk.yn[m];
  const size_t o = (size_t)(ix - 1) * ynum + (iy - 1);
  const double pul = __ldg(&plastic_yield[o]), pll = __ldg(&plastic_yield[o + 1]);
  const double pur = __ldg(&plastic_yield[o + ynum]), plr = __ldg(&plastic_yield[o + ynum + 1]);
  const double vflow = mk.eta_flow[m];
  if (!(pul > 0.0 || pll > 0.0 || pur > 0.0 || plr > 0.0)) {
    mk.eta[m] = vflow;
    return;
  }
  const double dx = (mk.x[m] - __ldg(&g.gx[ix - 1])) / __ldg(&g.sx[ix - 1]);
  const double dy = (mk.y[m] - __ldg(&g.gy[iy - 1])) / __ldg(&g.sy[iy - 1]);
  const double wul = (1.0 - dx) * (1.0 - dy), wll = (1.0 - dx) * dy, wur = dx * (1.0 - dy), wlr = dx * dy;
  const double denom = pul / __ldg(&etas1[o]) * wul + pll / __ldg(&etas1[o + 1]) * wll +
                       pur / __ldg(&etas1[o + ynum]) * wur + plr / __ldg(&etas1[o + ynum + 1]) * wlr;
  const double numer = pul * wul + pll * wll + pur * wur + plr * wlr;
  const double vvp = numer / denom;
  if (vvp >= vflow) {
    mk.eta[m] = vflow;
  } else {
    mk.eta[m] = vvp;
    mk.pfailure[m] = 1.0f;
  }
}

unsigned mblocks(const eb_ctx* c) { return (unsigned)((c->M + kBlock - 1) / kBlock); }

}  // namespace

int launch_gather_temperature(eb_ctx* c) {
  int rc;
  if ((rc = ensure_marker_field(c, EB_M_TK)) || (rc = ensure_grid_field(c, EB_G_TK1))) return rc;
  if (c->M == 0) return EB_OK;
  const float* tk1;
  if ((rc = grid_f32(c, {EB_G_TK1}, &tk1))) return rc;
  EB_PROF(c, "k_gather_temperature");
  k_gather_temperature<<<mblocks(c), kBlock, 0, c->stream>>>(dev_markers(c), c->g, tk1);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_post_stokes_gathers(eb_ctx* c) {
  int rc;
  const int mf[] = {EB_M_EXX, EB_M_EXY, EB_M_SR_RATIO, EB_M_PR, EB_M_ETA, EB_M_MATID};
  for (int f : mf) if ((rc = ensure_marker_field(c, f))) return rc;
  const int gfs[] = {EB_G_EXX, EB_G_EXY, EB_G_SXX2, EB_G_SXY2, EB_G_DSXX, EB_G_DSXY, EB_G_PR1};
  for (int f : gfs) if ((rc = ensure_grid_field(c, f))) return rc;
  if (c->M == 0) return EB_OK;
  const float* f[7];
  if ((rc = grid_f32(c, {EB_G_EXX, EB_G_EXY, EB_G_SXX2, EB_G_SXY2, EB_G_DSXX, EB_G_DSXY, EB_G_PR1}, f))) return rc;
  PostStokesGrids G{f[0], f[1], f[2], f[3], f[4], f[5], f[6], c->mats.mu, (float)c->P.timestep};
  EB_PROF(c, "k_post_stokes");
  k_post_stokes<<<mblocks(c), kBlock, 0, c->stream>>>(dev_markers(c), c->g, G);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_stress_correction(eb_ctx* c) {
  int rc;
  if ((rc = ensure_marker_field(c, EB_M_SXX)) || (rc = ensure_marker_field(c, EB_M_SXY)) ||
      (rc = ensure_grid_field(c, EB_G_DSXY)) || (rc = ensure_grid_field(c, EB_G_DSXX)))
    return rc;
  if (c->M == 0) return EB_OK;
  const float* f[2];
  if ((rc = grid_f32(c, {EB_G_DSXY, EB_G_DSXX}, f))) return rc;
  EB_PROF(c, "k_stress_correction");
  k_stress_correction<<<mblocks(c), kBlock, 0, c->stream>>>(dev_markers(c), c->g, f[0], f[1]);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_add_remaining_dt(eb_ctx* c) {
  int rc;
  if ((rc = ensure_marker_field(c, EB_M_TK)) || (rc = ensure_grid_field(c, EB_G_DTK1))) return rc;
  if (c->M == 0) return EB_OK;
  const float* dtk1;
  if ((rc = grid_f32(c, {EB_G_DTK1}, &dtk1))) return rc;
  EB_PROF(c, "k_add_dt");
  k_add_dt<<<mblocks(c), kBlock, 0, c->stream>>>(dev_markers(c), c->g, dtk1);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_marker_viscoplastic_viscosity(eb_ctx* c) {
  int rc;
  const int mf[] = {EB_M_ETA, EB_M_ETA_FLOW, EB_M_PFAILURE};
  for (int f : mf) if ((rc = ensure_marker_field(c, f))) return rc;
  if ((rc = ensure_grid_field(c, EB_G_PLASTIC_YIELD)) || (rc = ensure_grid_field(c, EB_G_ETAS1))) return rc;
  if (c->M == 0) return EB_OK;
  EB_PROF(c, "k_marker_eta_vp");
  k_marker_eta_vp<<<mblocks(c), kBlock, 0, c->stream>>>(dev_markers(c), c->g, c->gf[EB_G_PLASTIC_YIELD],
                                                         c->gf[EB_G_ETAS1]);
  EB_LAUNCHED(c);
  return EB_OK;
}
