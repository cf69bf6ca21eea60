// eb_advect.cu -- fused RK4 advection, stress rotation and strain update.
//
// Reference: Advection.advect_markers_and_rotate_stress_tensor! (src/advection/Advection.jl:109-114):
//   VelocityAndSpin.update_marker_velocity_and_spin_using_runge_kutta! (VelocityAndSpin.jl:45-129,
//     rk_update :131, interpolate_vx :343, interpolate_vy :373, interpolate_spin :402),
//   RungeKutta.jl:9-69, MarkersLocation.update! (MarkersLocation.jl:11-39),
//   MarkersStressRotation.rotate_marker_stress (MarkersStressRotation.jl:59-75);
// and MarkersStrain.update_total_strain! / update_plastic_strain! (MarkersStrain.jl:11-136).
// The reference runs three passes through marker_vx/vy/spin buffers; here one
// pass does all four RK stages, the move and the rotation.
//
// Precision: the intermediate RK positions are carried in FP32 relative to the
// marker's upper-left basic node (offsets below a few cells, so the FP32 error
// is ~1e-7 of a cell); the interpolated velocities are FP32; the final position
// update x + dt*v and the stress update are done in FP64.  A cell choice that
// differs from the reference at an intermediate stage (a point within FP32
// rounding of a grid line) does not change the velocity, because the bilinear
// interpolant is continuous across cell edges.
#include "eb_internal.h"

namespace {

constexpr int kBlock = 256;

struct VelGrids {
  const float *vx1, *vy1, *esp;
  float dt;
  double dtd;  // the same time step in FP64 for the position update
  int order;   // 1 or 4
};

// Locate a point given as an FP32 offset (px, py) from basic node (ix0, iy0):
// walk to the basic cell that contains it (searchsortedlast + clamp semantics)
// and return the offsets (ux, uy) from that cell's upper-left node.
__device__ __forceinline__ void walk_x(const DevGrid& g, int32_t ix0, float px, int32_t& j, float& u) {
  j = ix0;
  float o = 0.f;
  while (j < g.xnum - 1 && px >= o + __ldg(&g.sxf[j - 1])) { o += __ldg(&g.sxf[j - 1]); ++j; }
  while (j > 1 && px < o) { --j; o -= __ldg(&g.sxf[j - 1]); }
  u = px - o;
}
__device__ __forceinline__ void walk_y(const DevGrid& g, int32_t iy0, float py, int32_t& i, float& u) {
  i = iy0;
  float o = 0.f;
  while (i < g.ynum - 1 && py >= o + __ldg(&g.syf[i - 1])) { o += __ldg(&g.syf[i - 1]); ++i; }
  while (i > 1 && py < o) { --i; o -= __ldg(&g.syf[i - 1]); }
  u = py - o;
}

// sin(w) of the rotation angle w = spin dt, which is small on this path (spin ~1e-15/s, dt
// ~3e11 s): for |w| <= 0.25 the odd Taylor polynomial through w^7 is exact to FP32 rounding
// (the first omitted term, w^9 / 9!, is below 1e-10 of sin w), a few FMAs instead of sinf's
// range reduction; larger angles take sinf.
__device__ __forceinline__ float sin_rot(float w) {
  if (!(fabsf(w) <= 0.25f)) return sinf(w);
  const float w2 = w * w;
  return w * fmaf(w2, fmaf(w2, fmaf(w2, -1.f / 5040.f, 1.f / 120.f), -1.f / 6.f), 1.f);
}

// VelocityAndSpin.interpolate_vx / interpolate_vy / interpolate_spin at a point
// with offsets (ux, uy) inside basic cell (jx, jy).
__device__ __forceinline__ void vel_spin(const DevGrid& g, const VelGrids& V, int32_t jx, int32_t jy, float ux,
                                         float uy, float& vx, float& vy, float& sp) {
  const float4 cx0 = __ldg(&g.colx[2 * (jx - 1)]), cx1 = __ldg(&g.colx[2 * (jx - 1) + 1]);
  const float4 ry0 = __ldg(&g.rowy[2 * (jy - 1)]), ry1 = __ldg(&g.rowy[2 * (jy - 1) + 1]);
  const float dx = ux * cx0.y;
  const float dy = uy * ry0.y;
  // vx grid: x from the basic cell, y row yi = jy + (y > gridy_vx[jy+1])
  const bool ylo = !(uy > ry0.w);
  const int32_t yi = ylo ? jy : jy + 1;
  const float dyv = (uy - (ylo ? ry0.z : ry0.w)) * (ylo ? ry1.x : ry1.y);
  vx = gather4f(V.vx1, g.ynum + 1, yi, jx, dx, dyv);
  // vy grid: column xi = jx + (x > gridx_vy[jx+1]), y from the basic cell
  const bool xlo = !(ux > cx0.w);
  const int32_t xi = xlo ? jx : jx + 1;
  const float dxv = (ux - (xlo ? cx0.z : cx0.w)) * (xlo ? cx1.x : cx1.y);
  vy = gather4f(V.vy1, g.ynum, jy, xi, dxv, dy);
  // basic grid spin
  sp = gather4f(V.esp, g.ynum, jy, jx, dx, dy);
}

__global__ void k_advect(DevMarkers mk, DevGrid g, VelGrids V) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= mk.M) return;
  if (!(mk.mflags[m] & MF_INSIDE)) {
    mk.vx[m] = 0.0; mk.vy[m] = 0.0; mk.spin[m] = 0.0;
    return;
  }
  const int32_t ix0 = mk.xn[m], iy0 = mk.yn[m];
  const float lx0 = mk.fx[m] * __ldg(&g.sxf[ix0 - 1]);
  const float ly0 = mk.fy[m] * __ldg(&g.syf[iy0 - 1]);
  const float h = V.dt;
  float v1x, v1y, s1;
  vel_spin(g, V, ix0, iy0, lx0, ly0, v1x, v1y, s1);
  float vxm = v1x, vym = v1y, spm = s1;
  if (V.order == 4) {
    float v2x, v2y, s2, v3x, v3y, s3, v4x, v4y, s4, ux, uy;
    int32_t jx, jy;
    walk_x(g, ix0, lx0 + (h * 0.5f) * v1x, jx, ux);
    walk_y(g, iy0, ly0 + (h * 0.5f) * v1y, jy, uy);
    vel_spin(g, V, jx, jy, ux, uy, v2x, v2y, s2);
    walk_x(g, ix0, lx0 + (h * 0.5f) * v2x, jx, ux);
    walk_y(g, iy0, ly0 + (h * 0.5f) * v2y, jy, uy);
    vel_spin(g, V, jx, jy, ux, uy, v3x, v3y, s3);
    walk_x(g, ix0, lx0 + h * v3x, jx, ux);
    walk_y(g, iy0, ly0 + h * v3y, jy, uy);
    vel_spin(g, V, jx, jy, ux, uy, v4x, v4y, s4);
    // RungeKutta.apply_4th_order_runge_kutta
    vxm = (v1x + 2.f * v2x + 2.f * v3x + v4x) / 6.f;
    vym = (v1y + 2.f * v2y + 2.f * v3y + v4y) / 6.f;
    spm = (s1 + 2.f * s2 + 2.f * s3 + s4) / 6.f;
  }
  const double vxd = f2d(vxm), vyd = f2d(vym);
  mk.vx[m] = vxd;
  mk.vy[m] = vyd;
  mk.spin[m] = f2d(spm);
  // MarkersLocation.advect_marker: x + timestep * v (FP64)
  mk.x[m] = fma(V.dtd, vxd, mk.x[m]);
  mk.y[m] = fma(V.dtd, vyd, mk.y[m]);
  // MarkersStressRotation.rotate_marker_stress, written as increments:
  //   sxy' = sxy + sxx sin(2w) + sxy (cos(2w) - 1),  sxx' = sxx + sxx (cos(2w) - 1) - sxy sin(2w)
  // with cos(2w) - 1 = -2 sin(w)^2 evaluated without cancellation.
  const float w = spm * V.dt;
  const float s2w = sin_rot(2.f * w), sw = sin_rot(w);
  const float c2m1 = -2.f * sw * sw;
  const double sxx = mk.sxx[m], sxy = mk.sxy[m];
  const float fxx = d2f(sxx), fxy = d2f(sxy);
  mk.sxy[m] = sxy + f2d(fxx * s2w + fxy * c2m1);
  mk.sxx[m] = sxx + f2d(fxx * c2m1 - fxy * s2w);
}

// The last four steps of the marker cycle in one pass over the markers, each marker's
// fields read once and written once: StressCorrection (remaining grid stress change
// added to the marker stress, StressCorrection.jl:35-82), MarkerTemperature (remaining
// grid temperature change, MarkerTemperature.jl:18-45), the RK4 move and rotation of
// k_advect, and the strain update of k_strain.  Same arithmetic, same order: the
// correction precedes the rotation and the strain update reads the rotated stress, as
// when the four kernels run one after the other.
struct TailGrids {
  const float *dsxy, *dsxx, *dtk1;  // FP32 mirrors
  double healing;
};
// Every marker field the pass reads is loaded before its first store: the stores could
// alias the loads, so a load written after a store would wait for it and each marker
// would pay several DRAM round trips in sequence.  Loading first puts all of them in
// flight at once, and the plastic fields (10 % of markers or so) follow as soon as
// pfailure arrives, overlapping the RK4 gathers.
template <bool kMove>
__global__ void __launch_bounds__(kBlock) k_tail(DevMarkers mk, DevGrid g, VelGrids V, TailGrids T) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= mk.M) return;
  const uint8_t flags = __ldg(&mk.mflags[m]);
  const int32_t ix0 = __ldg(&mk.xn[m]), iy0 = __ldg(&mk.yn[m]);
  const float fx = __ldg(&mk.fx[m]), fy = __ldg(&mk.fy[m]);
  double sxy = mk.sxy[m], sxx = mk.sxx[m];
  const double tk = mk.tk[m], gii = mk.gii[m];
  const double exx = __ldg(&mk.exx[m]), exy = __ldg(&mk.exy[m]);
  const float pf = __ldg(&mk.pfailure[m]);
  double x = 0.0, y = 0.0;
  if (kMove) { x = mk.x[m]; y = mk.y[m]; }
  if (!(flags & MF_INSIDE)) {
    if (kMove) { mk.vx[m] = 0.0; mk.vy[m] = 0.0; mk.spin[m] = 0.0; }
    return;
  }
  const bool plastic = pf == 1.0f;
  double eta = 1.0, eta_flow = 1.0, sp0 = 0.0;
  if (plastic) { eta = __ldg(&mk.eta[m]); eta_flow = __ldg(&mk.eta_flow[m]); sp0 = mk.sp[m]; }
  const float lx0 = fx * __ldg(&g.sxf[ix0 - 1]);
  const float ly0 = fy * __ldg(&g.syf[iy0 - 1]);
  // stress correction
  sxy = sxy + f2d(gather4f(T.dsxy, g.ynum, iy0, ix0, fx, fy));
  sxx = sxx + f2d(gather_p(T.dsxx, g, ix0, iy0, lx0, ly0));
  // remaining temperature change
  mk.tk[m] = tk + f2d(gather4f(T.dtk1, g.ynum, iy0, ix0, fx, fy));
  if (kMove) {
    const float h = V.dt;
    float v1x, v1y, s1;
    vel_spin(g, V, ix0, iy0, lx0, ly0, v1x, v1y, s1);
    float vxm = v1x, vym = v1y, spm = s1;
    if (V.order == 4) {
      float v2x, v2y, s2, v3x, v3y, s3, v4x, v4y, s4, ux, uy;
      int32_t jx, jy;
      walk_x(g, ix0, lx0 + (h * 0.5f) * v1x, jx, ux);
      walk_y(g, iy0, ly0 + (h * 0.5f) * v1y, jy, uy);
      vel_spin(g, V, jx, jy, ux, uy, v2x, v2y, s2);
      walk_x(g, ix0, lx0 + (h * 0.5f) * v2x, jx, ux);
      walk_y(g, iy0, ly0 + (h * 0.5f) * v2y, jy, uy);
      vel_spin(g, V, jx, jy, ux, uy, v3x, v3y, s3);
      walk_x(g, ix0, lx0 + h * v3x, jx, ux);
      walk_y(g, iy0, ly0 + h * v3y, jy, uy);
      vel_spin(g, V, jx, jy, ux, uy, v4x, v4y, s4);
      vxm = (v1x + 2.f * v2x + 2.f * v3x + v4x) / 6.f;
      vym = (v1y + 2.f * v2y + 2.f * v3y + v4y) / 6.f;
      spm = (s1 + 2.f * s2 + 2.f * s3 + s4) / 6.f;
    }
    const double vxd = f2d(vxm), vyd = f2d(vym);
    mk.vx[m] = vxd;
    mk.vy[m] = vyd;
    mk.spin[m] = f2d(spm);
    mk.x[m] = fma(V.dtd, vxd, x);
    mk.y[m] = fma(V.dtd, vyd, y);
    const float w = spm * V.dt;
    const float s2w = sin_rot(2.f * w), sw = sin_rot(w);
    const float c2m1 = -2.f * sw * sw;
    const float fxx = d2f(sxx), fxy = d2f(sxy);
    const double nxy = sxy + f2d(fxx * s2w + fxy * c2m1);
    const double nxx = sxx + f2d(fxx * c2m1 - fxy * s2w);
    sxy = nxy;
    sxx = nxx;
  }
  mk.sxx[m] = sxx;
  mk.sxy[m] = sxy;
  // strain update (inside markers only, as k_strain)
  const float eii = hypotf(d2f(exx), d2f(exy));
  mk.gii[m] = fma(V.dtd, f2d(eii), gii);
  if (!plastic) return;
  const float sii = hypotf(d2f(sxx), d2f(sxy));
  const float d = d2f(eta_flow - eta);
  float rate = 0.5f * sii * ((d / d2f(eta)) / d2f(eta_flow));
  rate = fmaxf(0.f, rate);
  double sp = sp0 + V.dtd * f2d(rate) - T.healing * V.dtd;
  mk.sp[m] = sp > 0.0 ? sp : 0.0;
  mk.srp[m] = f2d(rate);
}

// MarkersStrain.update_total_strain! and update_plastic_strain!
__global__ void k_strain(DevMarkers mk, double dt, double healing) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= mk.M || mk.inside[m] != 1) return;
  const float eii = hypotf(d2f(mk.exx[m]), d2f(mk.exy[m]));
  mk.gii[m] = fma(dt, f2d(eii), mk.gii[m]);
  if (mk.pfailure[m] != 1.0f) return;
  const double eta = mk.eta[m], eta_flow = mk.eta_flow[m];
  const float sii = hypotf(d2f(mk.sxx[m]), d2f(mk.sxy[m]));
  // 0.5 sii (1/eta - 1/eta_flow) = 0.5 sii ((eta_flow - eta) / eta) / eta_flow
  const float d = d2f(eta_flow - eta);
  float rate = 0.5f * sii * ((d / d2f(eta)) / d2f(eta_flow));
  rate = fmaxf(0.f, rate);
  double sp = mk.sp[m] + dt * f2d(rate) - healing * dt;
  mk.sp[m] = sp > 0.0 ? sp : 0.0;
  mk.srp[m] = f2d(rate);
}

}  // namespace

int launch_advect(eb_ctx* c) {
  const int64_t order = c->P.runge_kutta_order;
  if (order <= 0) return EB_OK;  // NoMotion: markers fixed (Advection options)
  if (order != 1 && order != 4) return eb_fail(c, EB_BAD_INPUT, "runge_kutta_order must be 0, 1 or 4");
  int rc;
  const int mf[] = {EB_M_X, EB_M_Y, EB_M_VX, EB_M_VY, EB_M_SPIN, EB_M_SXX, EB_M_SXY};
  for (int f : mf) if ((rc = ensure_marker_field(c, f))) return rc;
  if ((rc = ensure_grid_field(c, EB_G_VX1)) || (rc = ensure_grid_field(c, EB_G_VY1)) || (rc = ensure_grid_field(c, EB_G_ESP)))
    return rc;
  if (c->M == 0) return EB_OK;
  const float* f[3];
  if ((rc = grid_f32(c, {EB_G_VX1, EB_G_VY1, EB_G_ESP}, f))) return rc;
  VelGrids V{f[0], f[1], f[2], (float)c->P.timestep, c->P.timestep, (int)order};
  EB_PROF(c, "k_advect");
  k_advect<<<(unsigned)((c->M + kBlock - 1) / kBlock), kBlock, 0, c->stream>>>(dev_markers(c), c->g, V);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_update_strain(eb_ctx* c) {
  int rc;
  const int mf[] = {EB_M_INSIDE, EB_M_EXX, EB_M_EXY, EB_M_GII, EB_M_PFAILURE, EB_M_ETA, EB_M_ETA_FLOW,
                    EB_M_SXX, EB_M_SXY, EB_M_STRAIN_PLASTIC, EB_M_STRAIN_RATE_PLASTIC};
  for (int f : mf) if ((rc = ensure_marker_field(c, f))) return rc;
  if (c->M == 0) return EB_OK;
  EB_PROF(c, "k_strain");
  k_strain<<<(unsigned)((c->M + kBlock - 1) / kBlock), kBlock, 0, c->stream>>>(dev_markers(c), c->P.timestep,
                                                                                c->P.plastic_healing_rate);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_marker_tail(eb_ctx* c) {
  const int64_t order = c->P.runge_kutta_order;
  if (order != 0 && order != 1 && order != 4) return eb_fail(c, EB_BAD_INPUT, "runge_kutta_order must be 0, 1 or 4");
  int rc;
  const int mf[] = {EB_M_X, EB_M_Y, EB_M_VX, EB_M_VY, EB_M_SPIN, EB_M_SXX, EB_M_SXY, EB_M_TK, EB_M_INSIDE, EB_M_EXX,
                    EB_M_EXY, EB_M_GII, EB_M_PFAILURE, EB_M_ETA, EB_M_ETA_FLOW, EB_M_STRAIN_PLASTIC,
                    EB_M_STRAIN_RATE_PLASTIC};
  for (int f : mf) if ((rc = ensure_marker_field(c, f))) return rc;
  for (int f : {EB_G_VX1, EB_G_VY1, EB_G_ESP, EB_G_DSXY, EB_G_DSXX, EB_G_DTK1})
    if ((rc = ensure_grid_field(c, f))) return rc;
  if (c->M == 0) return EB_OK;
  const float* f[6];
  if ((rc = grid_f32(c, {EB_G_VX1, EB_G_VY1, EB_G_ESP, EB_G_DSXY, EB_G_DSXX, EB_G_DTK1}, f))) return rc;
  VelGrids V{f[0], f[1], f[2], (float)c->P.timestep, c->P.timestep, (int)order};
  TailGrids T{f[3], f[4], f[5], c->P.plastic_healing_rate};
  EB_PROF(c, "k_tail");
  const unsigned blocks = (unsigned)((c->M + kBlock - 1) / kBlock);
  if (order > 0) k_tail<true><<<blocks, kBlock, 0, c->stream>>>(dev_markers(c), c->g, V, T);
  else k_tail<false><<<blocks, kBlock, 0, c->stream>>>(dev_markers(c), c->g, V, T);
  EB_LAUNCHED(c);
  return EB_OK;
}
