// eb_step_boundary.cu -- per-step updates at the boundary of the marker step: rock
// properties of the markers and the displacement-limited time step.
//
// Reference:
//   RockProperties.update_marker_rock_properties! (rock_properties/RockProperties.jl:99-125):
//     density (density/types/DensityLiao14.jl, DensityBlankenbach89.jl, DensityNaliboff17.jl),
//     rhocp (rhocp/types/ConstantRhoCp.jl, TemperatureDependentWaples.jl),
//     conductivity (thermal_conductivity/types/*.jl), the adiabatic term
//     (adiabatic_term/UpdateAdiabaticTerm.jl:19-33) and the sediment porosity correction
//     (porosity/PorosityUpdate.jl, SedimentPorosity.jl; the mudline depth by
//     MathTools.linear_interp, utils/MathTools.jl:160-198).
//   Update.update_model_time_step_using_displacement_limit (time_step/update/Update.jl:16-219).
//
// Built with -fmad=false: every formula keeps the Julia operand order, so the results are
// the reference's bit for bit (exp, in the Liao14 conductivity and the porosity law, is
// CUDA's, within an ulp of Julia's).  The time step is a minimum (and the velocity maxima
// are maxima): order-independent, so the parallel reduction is exact.
#include "eb_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace {

constexpr int kB = 256;

struct RockK {
  int64_t nmat;
  const double *rho, *cp, *kt;
  int32_t density_model, rhocp_model, cond_model, use_por;
  double temperature_top, max_cp;
  int64_t nsed, ntopo;
  const int16_t* sed;
  const double *tx, *ty;
  double kw, rhow, cpw;
};

// MathTools.linear_interp: the segment that holds x, found by bisection (the reference
// scans; both pick the same segment, the first j with x1 < x < x2 or an exact node)
__device__ double linear_interp(double x, const double* xc, const double* yv, int64_t n) {
  if (x <= xc[0]) return yv[0];
  if (x >= xc[n - 1]) return yv[n - 1];
  // largest lo with xc[lo] <= x (xc increasing), lo in [0, n-2]
  int64_t lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) / 2;
    if (xc[mid] <= x) lo = mid;
    else hi = mid;
  }
  const double x1 = xc[lo], x2 = xc[lo + 1], y1 = yv[lo], y2 = yv[lo + 1];
  if (x == x1) return y1;
  if (x == x2) return y2;
  return y1 + (y2 - y1) / (x2 - x1) * (x - x1);
}

__global__ void k_rock_properties(DevMarkers mk, RockK p) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= mk.M || mk.inside[m] != 1) return;
  const int64_t id = mk.matid[m] - 1;
  const double rho_s = p.rho[id], alpha = p.rho[p.nmat + id], beta = p.rho[2 * p.nmat + id];
  const double T = mk.tk[m];
  double rho;
  if (p.density_model == 0)
    rho = rho_s * (1.0 - alpha * (T - 298.15)) * (1.0 + beta * (mk.pr[m] - 1e5));
  else if (p.density_model == 1)
    rho = rho_s * (1.0 - alpha * (T - p.temperature_top));
  else
    rho = rho_s * (1.0 - alpha * (T - 830.0));
  const double cp20 = p.cp[id];
  double rhocp;
  if (p.rhocp_model == 0) {
    rhocp = rho * cp20;
  } else {
    const double tc = T - 273.0;  // ConversionFuncs.kelvin_to_celsius
    double cp = cp20 * (0.953 + 2.29e-3 * tc - 2.835e-6 * (tc * tc) + 1.191e-9 * (tc * tc * tc));
    cp = cp < p.max_cp ? cp : p.max_cp;
    rhocp = rho * cp;
  }
  const double k0 = p.kt[id], ka = p.kt[p.nmat + id];
  double k;
  switch (p.cond_model) {
    case 0: k = (k0 + ka / (T + 77.0)) * exp(0.00004 * mk.pr[m] / 1e6); break;
    case 1: k = k0; break;
    case 2: k = k0 / (1.0 + ka * (T - p.temperature_top) / p.temperature_top); break;
    case 3: k = mk.y[m] > 110000.0 ? 39.25 : k0; break;
    case 4: {  // Adiabatic.thermal_conductivity_simple_lithosphere_100km
      const double lith = 100000.0, air = 10000.0;
      k = mk.y[m] > lith + air ? (10000.0 / lith) * 2.25 * (1330.0 - 0.0) / (1334.5 - 1330.0) : k0;
      break;
    }
    default: k = k0 <= 20.0 ? 358.0 * (1.0227 * k0 - 1.882) * (1.0 / T - 0.00068) + 1.84 : k0; break;
  }
  const double ha = alpha * T;
  if (p.use_por == 1) {
    bool sed = false;
    for (int64_t s = 0; s < p.nsed; ++s) sed |= (p.sed[s] == mk.matid[m]);
    if (sed) {
      const double y_mud = linear_interp(mk.x[m], p.tx, p.ty, p.ntopo);
      double ysub = mk.y[m] - y_mud;
      ysub = ysub > mk.burial[m] ? ysub : mk.burial[m];
      const double phi = mk.por0[m] * exp(-(1.0 / mk.decay[m]) * ysub);
      k = k * (1.0 - phi) + p.kw * phi;
      rho = rho * (1.0 - phi) + p.rhow * phi;
      rhocp = rho * (cp20 * (1.0 - phi) + p.cpw * phi);
    }
  }
  mk.rho[m] = rho;
  mk.rhocp[m] = rhocp;
  mk.kt[m] = k;
  mk.ha[m] = ha;
}

// positive doubles order like their bit patterns: atomicMin/atomicMax on the bits
__device__ __forceinline__ void atomic_min_pos(unsigned long long* a, double v) {
  atomicMin(a, (unsigned long long)__double_as_longlong(v));
}
__device__ __forceinline__ void atomic_max_pos(unsigned long long* a, double v) {
  atomicMax(a, (unsigned long long)__double_as_longlong(v));
}

// out[0] = max |vx1|, out[1] = max |vy1|
__global__ void k_vmax(const double* __restrict__ vx, int64_t nvx, const double* __restrict__ vy, int64_t nvy,
                       unsigned long long* out) {
  double a = 0.0, b = 0.0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nvx || k < nvy;
       k += (int64_t)gridDim.x * blockDim.x) {
    if (k < nvx) a = fmax(a, fabs(vx[k]));
    if (k < nvy) b = fmax(b, fabs(vy[k]));
  }
  for (int o = 16; o > 0; o >>= 1) {
    a = fmax(a, __shfl_xor_sync(0xffffffffu, a, o));
    b = fmax(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomic_max_pos(&out[0], a);
    atomic_max_pos(&out[1], b);
  }
}

// out[0] = min over staggered nodes with |v| > 0 of displ * cell / |v| (vx then vy grids)
__global__ void k_dt_local(const double* __restrict__ vx, const double* __restrict__ vy,
                           const double* __restrict__ xstp, const double* __restrict__ ystp, int32_t xnum,
                           int32_t ynum, double displ, unsigned long long* out) {
  const int64_t nvx = (int64_t)(ynum + 1) * xnum, nvy = (int64_t)ynum * (xnum + 1);
  double best = INFINITY;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nvx + nvy;
       k += (int64_t)gridDim.x * blockDim.x) {
    double v, cell;
    if (k < nvx) {
      const int32_t j = (int32_t)(k / (ynum + 1)) + 1;  // 1-based column of vx1
      v = fabs(vx[k]);
      cell = j == 1 ? xstp[0] : (j == xnum ? xstp[xnum - 2] : (xstp[j - 2] < xstp[j - 1] ? xstp[j - 2] : xstp[j - 1]));
    } else {
      const int64_t q = k - nvx;
      const int32_t i = (int32_t)(q % ynum) + 1;       // 1-based row of vy1
      v = fabs(vy[q]);
      cell = i == 1 ? ystp[0] : (i == ynum ? ystp[ynum - 2] : (ystp[i - 2] < ystp[i - 1] ? ystp[i - 2] : ystp[i - 1]));
    }
    if (v > 0) {
      const double lim = displ * cell / v;
      best = best < lim ? best : lim;
    }
  }
  for (int o = 16; o > 0; o >>= 1) best = fmin(best, __shfl_xor_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0 && best < INFINITY) atomic_min_pos(&out[0], best);
}

template <class T>
int upload_table(eb_ctx* c, std::vector<void*>& owner, const T* host, size_t n, const T** dev) {
  if (n == 0) { *dev = nullptr; return EB_OK; }
  if (!host) return eb_fail(c, EB_BAD_INPUT, "null table pointer");
  void* p = nullptr;
  EB_CK(c, cudaMalloc(&p, n * sizeof(T)));
  owner.push_back(p);
  EB_CK(c, cudaMemcpyAsync(p, host, n * sizeof(T), cudaMemcpyHostToDevice, c->stream));
  *dev = (const T*)p;
  return EB_OK;
}

}  // namespace

extern "C" int eb_set_rock_tables(eb_ctx* c, const eb_rock_desc* t) {
  if (!c || !t) return EB_BAD_INPUT;
  if (t->nmat < 1) return eb_fail(c, EB_BAD_INPUT, "eb_rock_desc.nmat must be >= 1");
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (void* p : c->rock_allocs) cudaFree(p);
  c->rock_allocs.clear();
  c->rock_nmat = 0;
  int rc;
  const size_t n = (size_t)t->nmat;
  if ((rc = upload_table(c, c->rock_allocs, t->mat_rho, 3 * n, &c->rock_rho)) ||
      (rc = upload_table(c, c->rock_allocs, t->mat_cp, n, &c->rock_cp)) ||
      (rc = upload_table(c, c->rock_allocs, t->mat_kt, 2 * n, &c->rock_kt)))
    return rc;
  EB_CK(c, cudaStreamSynchronize(c->stream));
  c->rock_nmat = t->nmat;
  return EB_OK;
}

extern "C" int eb_set_sediment_porosity(eb_ctx* c, const eb_sediment_desc* d) {
  if (!c || !d) return EB_BAD_INPUT;
  if (d->nsed < 0 || d->ntopo < 1) return eb_fail(c, EB_BAD_INPUT, "eb_sediment_desc: nsed >= 0 and ntopo >= 1");
  for (int64_t k = 1; k < d->ntopo; ++k)
    if (!(d->topo_x[k] > d->topo_x[k - 1])) return eb_fail(c, EB_BAD_INPUT, "topo_x must increase");
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (void* p : c->sed_allocs) cudaFree(p);
  c->sed_allocs.clear();
  c->have_sed = false;
  int rc;
  if ((rc = upload_table(c, c->sed_allocs, d->matids_sediments, (size_t)d->nsed, &c->sed_ids)) ||
      (rc = upload_table(c, c->sed_allocs, d->topo_x, (size_t)d->ntopo, &c->sed_tx)) ||
      (rc = upload_table(c, c->sed_allocs, d->topo_y, (size_t)d->ntopo, &c->sed_ty)))
    return rc;
  EB_CK(c, cudaStreamSynchronize(c->stream));
  c->sed_n = d->nsed;
  c->sed_ntopo = d->ntopo;
  c->sed_kw = d->conductivity_water;
  c->sed_rhow = d->density_water;
  c->sed_cpw = d->heat_capacity_water;
  c->have_sed = true;
  return EB_OK;
}

extern "C" int eb_update_marker_rock_properties(eb_ctx* c, const eb_rock_params* p) {
  if (!c || !p) return EB_BAD_INPUT;
  if (!c->have_params) return eb_fail(c, EB_NOT_READY, "eb_set_params has not been called");
  if (c->rock_nmat < 1) return eb_fail(c, EB_NOT_READY, "eb_set_rock_tables has not been called");
  if (p->density_model < 0 || p->density_model > 2 || p->rhocp_model < 0 || p->rhocp_model > 1 ||
      p->conductivity_model < 0 || p->conductivity_model > 5)
    return eb_fail(c, EB_BAD_INPUT, "rock-property model id out of range");
  if (p->iuse_sed_porosity == 1 && !c->have_sed) return eb_fail(c, EB_NOT_READY, "eb_set_sediment_porosity has not been called");
  if (c->M > 0 && (c->matid_min < 1 || c->matid_max > c->rock_nmat))
    return eb_fail(c, EB_BAD_INPUT, "marker_matid outside the rock tables (or not uploaded)");
  cudaSetDevice(c->device);
  int rc;
  const int need[] = {EB_M_INSIDE, EB_M_MATID, EB_M_X, EB_M_Y, EB_M_PR, EB_M_TK, EB_M_RHO, EB_M_RHOCP, EB_M_KT, EB_M_HA};
  for (int f : need)
    if ((rc = ensure_marker_field(c, f))) return rc;
  if (p->iuse_sed_porosity == 1)
    for (int f : {EB_M_POROSITY_INITIAL, EB_M_DECAY_DEPTH, EB_M_MAX_BURIAL_DEPTH})
      if ((rc = ensure_marker_field(c, f))) return rc;
  if (c->M == 0) return EB_OK;
  RockK k{c->rock_nmat, c->rock_rho, c->rock_cp, c->rock_kt, p->density_model, p->rhocp_model,
          p->conductivity_model, p->iuse_sed_porosity, c->P.temperature_top, p->maximum_heat_capacity,
          c->sed_n, c->sed_ntopo, c->sed_ids, c->sed_tx, c->sed_ty, c->sed_kw, c->sed_rhow, c->sed_cpw};
  EB_PROF(c, "k_rock_properties");
  k_rock_properties<<<(unsigned)((c->M + kB - 1) / kB), kB, 0, c->stream>>>(dev_markers(c), k);
  EB_LAUNCHED(c);
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}

extern "C" int eb_update_model_time_step_using_displacement_limit(eb_ctx* c, double displ, int32_t iuse_local,
                                                                  double* timestep, int32_t* updated) {
  if (!c || !timestep) return EB_BAD_INPUT;
  if (!c->have_grid) return eb_fail(c, EB_NOT_READY, "eb_set_grid has not been called");
  cudaSetDevice(c->device);
  int rc;
  if ((rc = ensure_grid_field(c, EB_G_VX1)) || (rc = ensure_grid_field(c, EB_G_VY1))) return rc;
  unsigned long long* d = nullptr;
  EB_CK(c, cudaMalloc(&d, 2 * sizeof(unsigned long long)));
  const int64_t nvx = (int64_t)(c->ynum + 1) * c->xnum, nvy = (int64_t)c->ynum * (c->xnum + 1);
  const unsigned blocks = (unsigned)std::min<int64_t>((std::max(nvx, nvy) + kB - 1) / kB, 4 * 152);
  unsigned long long h[2];
  cudaError_t e;
  if (iuse_local == 0) {
    e = cudaMemsetAsync(d, 0, 2 * sizeof(unsigned long long), c->stream);  // +0.0
    if (e == cudaSuccess) {
      k_vmax<<<blocks, kB, 0, c->stream>>>(c->gf[EB_G_VX1], nvx, c->gf[EB_G_VY1], nvy, d);
      c->launches++;
      e = cudaGetLastError();
    }
  } else {
    const double inf_d = INFINITY;
    unsigned long long inf;
    std::memcpy(&inf, &inf_d, sizeof(inf));
    e = cudaMemcpyAsync(d, &inf, sizeof(inf), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
      k_dt_local<<<(unsigned)std::min<int64_t>((nvx + nvy + kB - 1) / kB, 4 * 152), kB, 0, c->stream>>>(
          c->gf[EB_G_VX1], c->gf[EB_G_VY1], c->g.sx, c->g.sy, c->xnum, c->ynum, displ, d);
      c->launches++;
      e = cudaGetLastError();
    }
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d);
  if (e != cudaSuccess) return eb_cuda(c, e, "time-step reduction");
  auto as_double = [](unsigned long long b) { double v; std::memcpy(&v, &b, 8); return v; };
  const double old = *timestep;
  double dt = old;
  auto limit = [&](double cell, double v) {  // Update.calculate_new_time_step_for_cell
    if (v > 0) {
      const double lim = displ * cell / v;
      dt = std::min(dt, lim);
    }
  };
  if (iuse_local == 0) {
    limit(c->g.xstpavg, as_double(h[0]));
    limit(c->g.ystpavg, as_double(h[1]));
  } else {
    const double best = as_double(h[0]);
    if (best < INFINITY) dt = std::min(dt, best);
  }
  *timestep = dt;
  if (updated) *updated = dt != old ? 1 : 0;
  return EB_OK;
}
