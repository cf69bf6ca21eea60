// eb_rheology.cu -- per-marker failure properties, composite creep viscosity and
// Drucker-Prager marker yielding.
//
// Reference (src/rheology):
//   FailureProperties.calculate_failure_properties_loop!   plastic_failure/failure_properties/FailureProperties.jl:19-161
//   CompositeViscosity.update_marker_flow_viscosity!        flow_viscosity/update/types/composite_viscosity/CompositeViscosity.jl:133-418
//   CompositeCreep / CreepStrainRate / ExponentialTerm / PeierlsCreep   composite_creep/*.jl
//   ViscousStrainSoftening                                   viscous_strain_softening/ViscousStrainSoftening.jl:14-39
//   ViscoplasticViscosity.update_marker_viscoplastic_viscosity!  viscoplastic_viscosity/ViscoplasticViscosity.jl:21-60
//   ViscoelasticForecast.update_plastic_yielding!            plastic_failure/markers/update/types/ViscoelasticForecast.jl:11-181
//   YieldStress / FluidPressure / Limits / YieldCheck / CheckYield   plastic_failure/utils/*.jl, markers/update/utils/*.jl
// The arithmetic is FP64 where results are formed: the bisection's stopping test
// (|dsigma| <= 1 Pa), its midpoints and its final viscosity follow the reference's FP64
// path.  Its branch decisions come from the root of the decision function, found once per
// marker (FP32 search, two FP64 Newton steps), with the reference's FP64 test wherever a
// midpoint lies too close to that root to decide by comparison.
#include "eb_internal.h"

namespace {

constexpr int kBlock = 128;
constexpr double kPaToMPa = 1.0 / 1e6;

__device__ __forceinline__ double MATV(const double* t, int32_t nmat, int32_t m, int k) {
  return __ldg(&t[(size_t)(k - 1) * nmat + (m - 1)]);
}

// Julia Float64^Float64 for the exponents on this path (2 -> x*x, 3 -> x*x*x, 1 -> x).
// The flow-viscosity bisection evaluates a power law up to 20 times per marker and the FP64
// pipe bounds the kernel (ncu: 86 % busy), so the other common exponents of the flow laws
// (4, 3.5, 2.5, 1.5) are products and square roots, and any other exponent is
// exp(y log x): within a few ulps of the correctly rounded power, like pow itself.
__device__ __forceinline__ double jl_pow(double x, double y) {
  if (y == 2.0) return x * x;
  if (y == 3.0) return x * x * x;
  if (y == 1.0) return x;
  if (x > 0.0 && x < INFINITY) {
    if (y == 4.0) {
      const double x2 = x * x;
      return x2 * x2;
    }
    if (y == 3.5) return x * x * x * sqrt(x);
    if (y == 2.5) return x * x * sqrt(x);
    if (y == 1.5) return x * sqrt(x);
    return exp(y * log(x));
  }
  return pow(x, y);
}

__device__ __forceinline__ void d_failure(const DevMarkers& mk, const DevMats& mt, int melt_damage, int64_t m) {
  const int32_t id = mk.matid[m];
  const double strain = mk.sp[m], sfi_m = mk.fric_ini[m];
  const double ci = MATV(mt.plastic, mt.nmat, id, 1), cf = MATV(mt.plastic, mt.nmat, id, 2);
  const double sfi_mat = MATV(mt.plastic, mt.nmat, id, 3), sff_mat = MATV(mt.plastic, mt.nmat, id, 4);
  const double ei = MATV(mt.plastic, mt.nmat, id, 5), ef = MATV(mt.plastic, mt.nmat, id, 6);
  // update_final_friction_angle
  const double sff = (sfi_mat > 0.0 && sff_mat > 0.0) ? sfi_m * (sff_mat / sfi_mat) : sff_mat;
  // strain_weakening_or_hardening
  double coh = ci, sf = sfi_m;
  if (strain >= ef) {
    coh = cf;
    sf = sff;
  } else if (ei <= strain && strain < ef) {
    coh = ci + (cf - ci) / (ef - ei) * (strain - ei);
    sf = sfi_m + (sff - sfi_m) / (ef - ei) * (strain - ei);
  }
  if (melt_damage) {
    sf = sf / mk.melt_damage[m];
    coh = coh / mk.melt_damage[m];
  }
  mk.cohesion[m] = coh;
  mk.fric[m] = sf;
}
__global__ void k_failure(DevMarkers mk, DevMats mt, int melt_damage) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= mk.M || mk.inside[m] != 1) return;
  d_failure(mk, mt, melt_damage, m);
}

struct CreepRow {
  double A_disl, n_disl, Ea_disl, Va_disl, A_p, m_p, n_p, s_p, A_diff, Ea_diff, Va_diff;
};

// CompositeCreep.calculate_composite_creep_viscosity_and_strain_rate: the total creep strain
// rate at s_mpa (the viscosity is 0.5 s / rate); inv_sp = 1 / s_p of the Peierls law.
__device__ double creep_rate(const CreepRow& r, double p_mpa, double T, double R, double preexp, double s_mpa,
                             bool use_old, double inv_sp, double& e_disl, double& a_p, double& e_diff) {
  if (!use_old) e_disl = exp(-((r.Ea_disl * 1000.0 + r.Va_disl * p_mpa) * (1.0 / (R * T))));
  const double rd = preexp * e_disl * ((r.n_disl == 1.0) ? s_mpa : jl_pow(s_mpa, r.n_disl));
  double rp = 0.0;
  if (r.A_p > 0.0 && T < 1200.0) {
    if (!use_old) a_p = (r.Ea_disl * 1000.0 + r.Va_disl * p_mpa) * (1.0 / (R * T));
    const double ratio = s_mpa * inv_sp;
    const double tm = (r.m_p == 1.0) ? 1.0 - ratio : 1.0 - jl_pow(ratio, r.m_p);
    const double inner = (r.n_p == 2.0) ? tm * tm : jl_pow(tm, r.n_p);
    rp = r.A_p * exp(-a_p * inner) * (s_mpa * s_mpa);
  }
  double rf = 0.0;
  if (r.A_diff > 0.0) {
    if (!use_old) e_diff = exp(-((r.Ea_diff * 1000.0 + r.Va_diff * p_mpa) * (1.0 / (R * T))));
    rf = r.A_diff * e_diff * s_mpa;
  }
  return ((rd > rp) ? rd : rp) + rf;
}

__device__ __forceinline__ double forecast_ve(double dt, double mu, double srr, double sxx, double sxy, double exx,
                                              double exy, double smin, double eta) {
  const double vef = eta / (mu * dt + eta);
  const double fac1 = 2.0 * eta * srr;
  const double om = 1.0 - vef;
  const double nxx = fac1 * exx * om + sxx * vef;
  const double nxy = fac1 * exy * om + sxy * vef;
  const double s = sqrt(nxx * nxx + nxy * nxy);
  return (s > smin) ? s : smin;
}

struct RheoParams {
  double dt, T_top, eta_min, eta_max, s_min, R, vsoftfac;
  int soft;
  double T_bottom, T_left, ysize;  // the Blankenbach and Couette flow laws
};

// ---- root-guided bisection --------------------------------------------------------------
// Each step of the reference's bisection (CompositeViscosity.jl:133-284) asks on which side of
// the visco-elastic forecast the midpoint savg lies.  With a = savg / 2 (the reference's
// 0.5 (s_mpa 1e6)) and D = mu dt rate(savg) + a, the forecast exceeds savg exactly when
//   phi(savg) = 2 mu dt rate(savg) + savg - |c| < 0,   c = 2 srr mu dt (exx, exy) + (sxx, sxy),
// and phi increases with the stress (every creep rate does), so every decision is "savg below
// the root s* of phi".  s* is found once: a bracketed search on log(s) in FP32, then two FP64
// Newton steps on phi.  The bisection then runs with its exact FP64 midpoints, deciding each
// step by comparing the midpoint's bit pattern with s*'s (both positive, so integer order is
// numeric order); a midpoint within kBandUlps of s* (relative 3e-11, far above the ~1e-15 of
// either evaluation) takes the reference's own FP64 test.  The decisions, the step count and
// the final midpoint are therefore those of the plain FP64 loop, with one FP64 creep-rate
// evaluation at the end instead of one per step.  A marker whose Newton steps do not settle
// (a kink of max(dislocation, Peierls) at the root) runs the plain loop.
constexpr int64_t kBandUlps = 1 << 17;

struct FlowLaw {
  CreepRow r;
  double A, p_mpa, T, R, inv_sp, e_disl, a_p, e_diff;
};

__device__ __forceinline__ double rate_at(const FlowLaw& f, double s_mpa) {
  double ed = f.e_disl, ap = f.a_p, ef = f.e_diff;
  return creep_rate(f.r, f.p_mpa, f.T, f.R, f.A, s_mpa, true, f.inv_sp, ed, ap, ef);
}

// rate and d rate / d s (s in Pa) of the reference's composite law at s
__device__ double rate_and_slope(const FlowLaw& f, double s, double& slope) {
  const double s_mpa = s * kPaToMPa;
  const double inv_s = 1.0 / s;
  const double rd = f.A * f.e_disl * ((f.r.n_disl == 1.0) ? s_mpa : jl_pow(s_mpa, f.r.n_disl));
  const double drd = f.r.n_disl * rd * inv_s;
  double rp = 0.0, drp = 0.0;
  if (f.r.A_p > 0.0 && f.T < 1200.0) {
    const double ratio = s_mpa * f.inv_sp;
    const double rm = (f.r.m_p == 1.0) ? ratio : jl_pow(ratio, f.r.m_p);
    const double tm = 1.0 - rm;
    const double inner = (f.r.n_p == 2.0) ? tm * tm : jl_pow(tm, f.r.n_p);
    rp = f.r.A_p * exp(-f.a_p * inner) * (s_mpa * s_mpa);
    const double tpow = (f.r.n_p == 2.0) ? tm : jl_pow(tm, f.r.n_p - 1.0);
    drp = rp * (2.0 + f.a_p * f.r.n_p * tpow * f.r.m_p * rm) * inv_s;
  }
  double rf = 0.0, drf = 0.0;
  if (f.r.A_diff > 0.0) {
    rf = f.r.A_diff * f.e_diff * s_mpa;
    drf = rf * inv_s;
  }
  slope = ((rd > rp) ? drd : drp) + drf;
  return ((rd > rp) ? rd : rp) + rf;
}

// psi(u) = log(2 mdt rate(e^u)) - log(|c| - e^u) in FP32 (increasing in u); +inf past |c|
struct LogLaw {
  float ld, lp, lf, n, a_p, m_p, n_p, inv_sp, l2mdt, cabs;
  bool peierls, diff;
  __device__ float psi(float u) const {
    const float e = __expf(u);
    if (!(e < cabs)) return INFINITY;
    const float lsm = u - 13.815510558f;  // log(s_mpa) = log(s) - log(1e6)
    float L = ld + n * lsm;
    if (peierls) {
      const float ratio = __expf(lsm) * inv_sp;
      const float rm = (m_p == 1.f) ? ratio : __powf(ratio, m_p);
      const float tm = 1.f - rm;
      const float inner = (n_p == 2.f) ? tm * tm : __powf(tm, n_p);
      L = fmaxf(L, lp - a_p * inner + 2.f * lsm);
    }
    if (diff) {
      const float lrf = lf + lsm;
      const float hi = fmaxf(L, lrf), lo = fminf(L, lrf);
      L = hi + log1pf(__expf(lo - hi));
    }
    return l2mdt + L - __logf(cabs - e);
  }
};

// The root s* of phi (see above); false when the Newton steps do not settle.  Roots far
// outside [lo, hi] (every midpoint on one side by a wide margin) return 0 or +inf.
__device__ bool flow_root(const FlowLaw& f, double mdt, double cabs, double lo, double hi, double& sstar) {
  if (!(cabs > 0.0)) {  // phi > 0 everywhere: every midpoint lies above the root
    sstar = 0.0;
    return true;
  }
  // FP32 copies by integer conversion (d2f): the F2F instructions would issue on the FP64 pipe
  // that bounds this kernel
  LogLaw g;
  const float inv_rt = 1.f / (d2f(f.R) * d2f(f.T));  // FP32: this stage only brackets the root
  const float p32 = d2f(f.p_mpa);
  g.ld = __logf(d2f(f.A)) - (d2f(f.r.Ea_disl) * 1000.f + d2f(f.r.Va_disl) * p32) * inv_rt;
  g.n = d2f(f.r.n_disl);
  g.peierls = f.r.A_p > 0.0 && f.T < 1200.0;
  g.lp = g.peierls ? __logf(d2f(f.r.A_p)) : 0.f;
  g.a_p = d2f(f.a_p);
  g.m_p = d2f(f.r.m_p);
  g.n_p = d2f(f.r.n_p);
  g.inv_sp = d2f(f.inv_sp);
  g.diff = f.r.A_diff > 0.0;
  g.lf = g.diff ? __logf(d2f(f.r.A_diff)) - (d2f(f.r.Ea_diff) * 1000.f + d2f(f.r.Va_diff) * p32) * inv_rt : 0.f;
  g.l2mdt = __logf(2.f * d2f(mdt));
  g.cabs = d2f(cabs);
  // The shortcuts below trust psi's sign only where |c| - s does not cancel in FP32 (s at
  // least 1 % below |c|; at or above |c|, phi > 0 holds exactly).
  constexpr float kMargin = 1e-3f;  // far above the FP32 evaluation error of psi there
  float ul = __logf(d2f(lo)), uh = __logf(d2f(hi));
  const float pl = g.psi(ul), ph = g.psi(uh);
  if (lo >= cabs || (lo < 0.99 * cabs && pl > kMargin)) { sstar = 0.0; return true; }  // root well below lo
  if (hi < 0.99 * cabs && ph < -kMargin) { sstar = INFINITY; return true; }           // ... well above hi
  ul -= 1e-3f;
  uh = fminf(uh + 1e-3f, __logf(g.cabs) - 1e-6f);
  if (!(g.psi(ul) <= 0.f)) ul -= 0.1f;
  for (int k = 0; k < 26; ++k) {
    const float um = 0.5f * (ul + uh);
    if (g.psi(um) > 0.f) uh = um; else ul = um;
  }
  double s = f2d(__expf(0.5f * (ul + uh)));
  double step = 0.0;
  for (int k = 0; k < 2; ++k) {
    double slope;
    const double rate = rate_and_slope(f, s, slope);
    const double phi = 2.0 * mdt * rate + s - cabs;
    step = phi / (2.0 * mdt * slope + 1.0);
    s -= step;
  }
  sstar = s;
  return isfinite(s) && s > 0.0 && fabs(step) <= 1e-9 * s;
}

// The bisection's bookkeeping on positive finite doubles in integer form, decided exactly as
// the FP64 operations would be: the comparisons compare bit patterns (integer order is numeric
// order for positive doubles), halving a sum subtracts one from its exponent, and
// |b - a| > 1 uses the exact difference (Sterbenz: within a factor of 2 the FP64 difference is
// exact; farther apart it exceeds b / 2, above 1 once b >= 4).  Comparisons, multiplications
// and differences of doubles all issue on the FP64 pipe, which bounds this kernel.
__device__ __forceinline__ int64_t dbits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ bool gap_above_one(double a, double b) {
  int64_t ia = dbits(a), ib = dbits(b);
  if (ia > ib) {
    const int64_t t = ia; ia = ib; ib = t;
  }
  // below Sterbenz's range (2a < b) the difference exceeds b / 2
  if (ia + ((int64_t)1 << 52) < ib) return ib >= 0x4010000000000000LL /* 4.0 */ || fabs(b - a) > 1.0;
  const int32_t ea = (int32_t)(ia >> 52), eb = (int32_t)(ib >> 52);
  const int64_t one = (int64_t)1 << 52;
  const int64_t ma = (ia & (one - 1)) | one, mb = (ib & (one - 1)) | one;
  const int64_t D = (mb << (eb - ea)) - ma;  // b - a in units of 2^(ea - 1075), exact
  const int sh = 1075 - ea;                  // D 2^-sh > 1  <=>  D > 2^sh
  if (sh < 0) return D > 0;
  if (sh >= 62) return false;
  return D > ((int64_t)1 << sh);
}
__device__ __forceinline__ bool pos_normal(double x) {
  const int64_t b = dbits(x);
  return b >= ((int64_t)1 << 52) && b < 0x7FF0000000000000LL;
}

// The flow laws other than composite creep; the model's law is its largest mat_flow_type
// (FlowViscosity.jl:21-44, UpdateManager.jl).  Each sets eta_flow and preexp as the
// reference's module does, with the same operations in the same order.
__device__ __forceinline__ bool d_flow_viscosity_other(const DevMarkers& mk, const DevMats& mt, const RheoParams& P,
                                                       int64_t m) {
  const int32_t id = mk.matid[m];
  double eta, pre;
  switch (mt.option) {
    case 0:  // Isoviscous.jl
      eta = MATV(mt.flow, mt.nmat, id, 1);
      pre = eta;
      break;
    case 4: {  // CouetteFlowBenchmark.jl: temperature limited below by the left wall's
      const double T = fmax(mk.tk[m], P.T_left);
      pre = MATV(mt.flow, mt.nmat, id, 13);
      const double ea = MATV(mt.flow, mt.nmat, id, 14);
      eta = pre * exp(ea * 1000.0 / P.R / P.T_left * (1.0 - (T - P.T_left) / P.T_left));
      break;
    }
    case 5: {  // Blankenback89.jl: temperature limited below by the top's
      const double T = fmax(mk.tk[m], P.T_top);
      pre = MATV(mt.flow, mt.nmat, id, 15);
      const double b = MATV(mt.flow, mt.nmat, id, 16), cy = MATV(mt.flow, mt.nmat, id, 17);
      eta = pre * exp(-b * (T - P.T_top) / (P.T_bottom - P.T_top) + cy * mk.y[m] / P.ysize);
      break;
    }
    case -1: {  // Xdependent.jl: the analytic viscosity of the non-Newtonian channel
      const double pgrad = -1e9 / 9500.0, dx = mk.x[m] - 10000.0 / 2.0;
      eta = fabs(dx) > 0.0 ? 1.0 / 1e-37 * pow(-pgrad, 1.0 - 3.0) * pow(dx, 1.0 - 3.0) : P.eta_max;
      pre = MATV(mt.flow, mt.nmat, id, 1);
      break;
    }
    default:
      return false;
  }
  mk.eta_flow[m] = eta;
  mk.preexp[m] = pre;
  return true;
}

__device__ __forceinline__ void d_flow_viscosity(const DevMarkers& mk, const DevMats& mt, const RheoParams& P, int64_t m) {
  if (d_flow_viscosity_other(mk, mt, P, m)) return;
  const int32_t id = mk.matid[m];
  const int32_t ft = __ldg(&mt.flow_type[id - 1]);
  double eta = 0.0;
  double A = MATV(mt.flow, mt.nmat, id, 2);
  if (ft == 0) {
    eta = MATV(mt.flow, mt.nmat, id, 1);
  } else if (ft == 1 || ft == 2) {
    CreepRow r;
    r.n_disl = MATV(mt.flow, mt.nmat, id, 3); r.Ea_disl = MATV(mt.flow, mt.nmat, id, 4);
    r.Va_disl = MATV(mt.flow, mt.nmat, id, 5); r.A_p = MATV(mt.flow, mt.nmat, id, 6);
    r.m_p = MATV(mt.flow, mt.nmat, id, 7); r.n_p = MATV(mt.flow, mt.nmat, id, 8);
    r.s_p = MATV(mt.flow, mt.nmat, id, 9); r.A_diff = MATV(mt.flow, mt.nmat, id, 10);
    r.Ea_diff = MATV(mt.flow, mt.nmat, id, 11); r.Va_diff = MATV(mt.flow, mt.nmat, id, 12);
    const double sxx = mk.sxx[m], sxy = mk.sxy[m], exx = mk.exx[m], exy = mk.exy[m];
    const double strain = mk.gii[m];
    const double p_mpa = mk.pr[m] * kPaToMPa;
    const double srr = mk.sr_ratio[m];
    const double T = fmax(mk.tk[m], P.T_top);
    const double ei = MATV(mt.plastic, mt.nmat, id, 5), ef = MATV(mt.plastic, mt.nmat, id, 6);
    const double mu = __ldg(&mt.mu[id - 1]);
    if (P.soft) {  // ViscousStrainSoftening.update_pre_exponential_for_viscous_strain_softening
      const double amin = A, amax = A * P.vsoftfac;
      if (ei < strain && strain < ef) A = amin + (amax - amin) / (ef - ei) * (strain - ei);
      if (strain >= ef) A = amax;
    }
    double s0 = sqrt(sxx * sxx + sxy * sxy);
    if (s0 < P.s_min) s0 = P.s_min;
    double e_disl = 0.0, a_p = 0.0, e_diff = 0.0;
    const double inv_sp = (r.A_p > 0.0 && T < 1200.0) ? 1.0 / r.s_p : 0.0;  // Peierls creep only
    double s_mpa = s0 * kPaToMPa;
    double rate = creep_rate(r, p_mpa, T, P.R, A, s_mpa, false, inv_sp, e_disl, a_p, e_diff);
    eta = 0.5 * (s_mpa * 1e6) / rate;
    double sf = forecast_ve(P.dt, mu, srr, sxx, sxy, exx, exy, P.s_min, eta);
    double delta = 1e39;
    int icount = 0;
    // Each step needs only the side of savg the forecast falls on.  With eta = a / rate
    // (a = s / 2) and D = mu dt rate + a, the forecast components are (a / D) c with
    // c = 2 srr mu dt (exx, exy) + (sxx, sxy), fixed over the loop, and
    // max(|forecast|, s_min) > savg >= s_min compares as a^2 |c|^2 > savg^2 D^2: no
    // division or square root per step.  The viscosity of the last step is formed after
    // the loop.
    const double mdt = mu * P.dt;
    const double cxx = 2.0 * srr * mdt * exx + sxx, cxy = 2.0 * srr * mdt * exy + sxy;
    const double cc = cxx * cxx + cxy * cxy;
    FlowLaw fl{r, A, p_mpa, T, P.R, inv_sp, e_disl, a_p, e_diff};
    double sstar;
    if (pos_normal(s0) && pos_normal(sf) && P.s_min >= 0.0 &&
        flow_root(fl, mdt, sqrt(cc), fmin(s0, sf), fmax(s0, sf), sstar)) {
      const int64_t kr = dbits(sstar), kmin = dbits(P.s_min);
      int64_t i0 = dbits(s0), i1 = dbits(sf);
      bool more = true;  // delta = 1e39 > 1 before the first step
      int64_t iavg = i0;
      while (icount < 20 && more) {
        ++icount;
        // (s0 + sf) / 2: the sum in FP64, halved exactly in the exponent
        iavg = dbits(__longlong_as_double(i0) + __longlong_as_double(i1)) - ((int64_t)1 << 52);
        const int64_t dist = iavg - kr;
        bool above, below;
        if (dist > kBandUlps) {
          above = false;
          below = kmin < iavg;
        } else if (dist < -kBandUlps) {
          above = true;
          below = false;
        } else {  // within the band: the reference's own test
          const double savg = __longlong_as_double(iavg);
          s_mpa = savg * kPaToMPa;
          rate = rate_at(fl, s_mpa);
          const double a = 0.5 * (s_mpa * 1e6);
          const double d = mdt * rate + a;
          const double lhs = (a * a) * cc, rhs = (savg * savg) * (d * d);
          above = lhs > rhs;
          below = lhs < rhs && P.s_min < savg;
        }
        if ((i1 > i0 && above) || (i1 < i0 && below)) i0 = iavg;
        else i1 = iavg;
        more = gap_above_one(__longlong_as_double(i0), __longlong_as_double(i1));
      }
      s_mpa = __longlong_as_double(iavg) * kPaToMPa;
      rate = rate_at(fl, s_mpa);
    } else while (icount < 20 && delta > 1.0) {
      ++icount;
      const double savg = (s0 + sf) / 2.0;
      s_mpa = savg * kPaToMPa;
      rate = creep_rate(r, p_mpa, T, P.R, A, s_mpa, true, inv_sp, e_disl, a_p, e_diff);
      const double a = 0.5 * (s_mpa * 1e6);
      const double d = mdt * rate + a;
      const double lhs = (a * a) * cc, rhs = (savg * savg) * (d * d);
      const bool above = lhs > rhs, below = lhs < rhs && P.s_min < savg;
      if ((sf > s0 && above) || (sf < s0 && below)) s0 = savg;
      else sf = savg;
      delta = fabs(sf - s0);
    }
    if (icount > 0) eta = 0.5 * (s_mpa * 1e6) / rate;
    eta = fmin(fmax(eta, P.eta_min), P.eta_max);
  }
  mk.eta_flow[m] = eta;
  mk.preexp[m] = A;
}
__global__ void k_flow_viscosity(DevMarkers mk, DevMats mt, RheoParams P) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= mk.M || mk.inside[m] != 1) return;
  d_flow_viscosity(mk, mt, P, m);
}

__device__ __forceinline__ void d_viscoplastic(const DevMarkers& mk, int64_t ntimestep, int64_t itype_global, int64_t m) {
  const double vf = mk.eta_flow[m];
  double vp = mk.eta[m];
  if (itype_global == 0) vp = vf;
  else if (itype_global == 1 && (ntimestep == 0 || vp == 0.0)) vp = vf;
  mk.eta[m] = vp;
}
__global__ void k_viscoplastic(DevMarkers mk, int64_t ntimestep, int64_t itype_global) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= mk.M || mk.inside[m] != 1) return;
  d_viscoplastic(mk, ntimestep, itype_global, m);
}

struct YieldParams {
  int64_t ntimestep;
  double dt, y_sealevel, eta_min, eta_max, sy_min, sy_max;
  int fluid, no_yield_mobile;
  int32_t id_air, id_wall, id_plate;
};

__device__ __forceinline__ void d_yield(const DevMarkers& mk, const DevMats& mt, const YieldParams& P, int64_t m) {
  const int32_t id = mk.matid[m];
  const double coh = mk.cohesion[m], sf = mk.fric[m];
  int yflag = 0;
  if (P.ntimestep > 0 && (coh > 0.0 || sf > 0.0)) {
    double eta = mk.eta[m];
    const double mu = __ldg(&mt.mu[id - 1]);
    double sxx = mk.sxx[m], sxy = mk.sxy[m];
    const double exx = mk.exx[m], exy = mk.exy[m], srr = mk.sr_ratio[m], p = mk.pr[m];
    // cos(asin(sf)) of YieldStress.calc_yield_stress, as the identity sqrt(1 - sf^2) for
    // sf in [-1, 1]: one square root instead of two FP64 transcendentals (they differ by a few
    // ulps of cos(phi), which moves the yield test only for a stress within ~1e-16 of yield)
    const double cphi = sqrt(fmax(0.0, 1.0 - sf * sf));
    double sy;
    if (P.fluid == 0) {
      sy = coh * cphi + sf * p;
    } else {
      const double depth = fmax(0.0, mk.y[m] - P.y_sealevel);
      const double pf = 1000.0 * 9.81 * depth;
      sy = (p < pf) ? coh * cphi : coh * cphi + sf * (p - pf);
    }
    sy = fmax(sy, 0.0);
    sy = fmin(fmax(sy, P.sy_min), P.sy_max);
    const double vef = eta / (eta + P.dt * mu);
    const double nxx = sxx * vef + 2.0 * eta * exx * srr * (1.0 - vef);
    const double nxy = sxy * vef + 2.0 * eta * exy * srr * (1.0 - vef);
    const double sii = sqrt(nxx * nxx + nxy * nxy);
    bool yielding = sii > sy;
    if (P.no_yield_mobile && (id == P.id_air || id == P.id_wall || id == P.id_plate)) yielding = false;
    if (yielding) {
      yflag = 1;
      const double s_old = sqrt(sxx * sxx + sxy * sxy);
      if (s_old != 0.0) {
        sxx = sxx * sy / s_old;
        sxy = sxy * sy / s_old;
      } else {
        sxx = sy;
        sxy = sy;
      }
      const double e_old = srr * sqrt(exx * exx + exy * exy);
      eta = sy / 2.0 / e_old;
      eta = fmin(fmax(eta, P.eta_min), P.eta_max);
      mk.sxx[m] = sxx;
      mk.sxy[m] = sxy;
      mk.eta[m] = eta;
    }
  }
  if (mk.pfailure[m] != 1.0f) mk.pfailure[m] = (float)yflag;
}
__global__ void k_yield(DevMarkers mk, DevMats mt, YieldParams P) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= mk.M || mk.inside[m] != 1) return;
  d_yield(mk, mt, P, m);
}

// Rheology.update_marker_rheology! followed by update_marker_viscoplastic_viscosity!
// (TimeLoop.jl:222-223) in one pass: failure properties, flow viscosity, viscoplastic
// viscosity and (marker plasticity) yielding of each marker, the same steps in the same order
// as the four kernels above; the fields a step writes are read back by the next from L1.
__global__ void k_rheology(DevMarkers mk, DevMats mt, int melt_damage, RheoParams R, int64_t ntimestep,
                           int64_t itype_global, int yield, YieldParams Y) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= mk.M || mk.inside[m] != 1) return;
  d_failure(mk, mt, melt_damage, m);
  d_flow_viscosity(mk, mt, R, m);
  d_viscoplastic(mk, ntimestep, itype_global, m);
  if (yield) d_yield(mk, mt, Y, m);
}

unsigned mblocks(const eb_ctx* c) { return (unsigned)((c->M + kBlock - 1) / kBlock); }

int ensure(eb_ctx* c, std::initializer_list<int> fs) {
  for (int f : fs) {
    int rc = ensure_marker_field(c, f);
    if (rc) return rc;
  }
  return EB_OK;
}

YieldParams yield_params(const eb_params& p) {
  return YieldParams{p.ntimestep, p.timestep, p.y_sealevel, p.viscosity_min, p.viscosity_max, p.yield_stress_min,
                     p.yield_stress_max, (int)(p.iuse_fluid_pressure_for_yield != 0),
                     (int)(p.no_yielding_in_mobile_wall != 0), (int32_t)p.matid_sticky_air,
                     (int32_t)p.matid_mobile_wall, (int32_t)p.matid_plate_extension};
}
RheoParams rheo_params(const eb_ctx* c) {
  const eb_params& p = c->P;
  const double ysize = c->h_gy.empty() ? 0.0 : c->h_gy.back() - c->h_gy.front();
  return RheoParams{p.timestep, p.temperature_top, p.viscosity_min, p.viscosity_max, p.powerlaw_stress_min,
                    p.gas_constant, p.vsoftfac, (int)(p.iuse_viscous_strain_soft == 1), p.temperature_bottom,
                    p.temperature_left, ysize};
}

int yield_launch(eb_ctx* c) {
  int rc = ensure(c, {EB_M_INSIDE, EB_M_MATID, EB_M_COHESION, EB_M_FRIC, EB_M_ETA, EB_M_SXX, EB_M_SXY, EB_M_EXX,
                      EB_M_EXY, EB_M_SR_RATIO, EB_M_PR, EB_M_Y, EB_M_PFAILURE});
  if (rc) return rc;
  if (c->M == 0) return EB_OK;
  const YieldParams Y = yield_params(c->P);
  EB_PROF(c, "k_yield");
  k_yield<<<mblocks(c), kBlock, 0, c->stream>>>(dev_markers(c), c->mats, Y);
  EB_LAUNCHED(c);
  return EB_OK;
}

}  // namespace

int launch_rheology(eb_ctx* c) {
  int rc = ensure(c, {EB_M_INSIDE, EB_M_MATID, EB_M_STRAIN_PLASTIC, EB_M_FRIC_INI, EB_M_COHESION, EB_M_FRIC,
                      EB_M_SXX, EB_M_SXY, EB_M_EXX, EB_M_EXY, EB_M_TK, EB_M_PR, EB_M_GII, EB_M_SR_RATIO,
                      EB_M_ETA_FLOW, EB_M_PREEXP, EB_M_X, EB_M_Y});
  if (rc) return rc;
  const int melt = c->P.iuse_melt_damage == 1;
  if (melt && (rc = ensure_marker_field(c, EB_M_MELT_DAMAGE))) return rc;
  if (c->M == 0) return EB_OK;
  EB_PROF(c, "k_failure");
  k_failure<<<mblocks(c), kBlock, 0, c->stream>>>(dev_markers(c), c->mats, melt);
  EB_LAUNCHED(c);
  const RheoParams R = rheo_params(c);
  EB_PROF(c, "k_flow_viscosity");
  k_flow_viscosity<<<mblocks(c), kBlock, 0, c->stream>>>(dev_markers(c), c->mats, R);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_viscoplastic(eb_ctx* c, int use_marker_plasticity) {
  int rc = ensure(c, {EB_M_INSIDE, EB_M_ETA, EB_M_ETA_FLOW});
  if (rc) return rc;
  if (c->M == 0) return EB_OK;
  EB_PROF(c, "k_viscoplastic");
  k_viscoplastic<<<mblocks(c), kBlock, 0, c->stream>>>(dev_markers(c), c->P.ntimestep, c->P.itype_global);
  EB_LAUNCHED(c);
  if (use_marker_plasticity) return yield_launch(c);
  return EB_OK;
}

int launch_plastic_yielding(eb_ctx* c) { return yield_launch(c); }

int launch_rheology_fused(eb_ctx* c, int use_marker_plasticity) {
  int rc = ensure(c, {EB_M_INSIDE, EB_M_MATID, EB_M_STRAIN_PLASTIC, EB_M_FRIC_INI, EB_M_COHESION, EB_M_FRIC,
                      EB_M_SXX, EB_M_SXY, EB_M_EXX, EB_M_EXY, EB_M_TK, EB_M_PR, EB_M_GII, EB_M_SR_RATIO,
                      EB_M_ETA_FLOW, EB_M_PREEXP, EB_M_ETA, EB_M_X, EB_M_Y, EB_M_PFAILURE});
  if (rc) return rc;
  const int melt = c->P.iuse_melt_damage == 1;
  if (melt && (rc = ensure_marker_field(c, EB_M_MELT_DAMAGE))) return rc;
  if (c->M == 0) return EB_OK;
  EB_PROF(c, "k_rheology");
  k_rheology<<<mblocks(c), kBlock, 0, c->stream>>>(dev_markers(c), c->mats, melt, rheo_params(c), c->P.ntimestep,
                                                  c->P.itype_global, use_marker_plasticity ? 1 : 0, yield_params(c->P));
  EB_LAUNCHED(c);
  return EB_OK;
}
