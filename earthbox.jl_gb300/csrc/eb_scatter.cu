// eb_scatter.cu -- marker -> grid bilinear averaging as a deterministic cell-sorted reduction.
//
// Reference (src/interpolation): BilinearDenominator.jl:34-157 (weight sums),
// BilinearNumerator.jl:31-533 (numerators), BilinearAverage.jl:10-322 (averages),
// BackupTransportArrays.jl:33-179 (backup + clear), FlattenDensity.jl:29-89,
// ApplyThermalBC.jl:20-44, and the subgrid scatters
// subgrid_stress/update/stress_change/*.jl and heat_solver/subgrid_heat/SubgridDiffusion.jl:126-195.
//
// The reference folds every marker into the grid serially in marker order.
// Here each block owns 32 consecutive basic cells (column-major cell id); it
// stages its markers' weights and values in shared memory (markers come from
// the cell-sorted list, so they are read in cell order) and one warp per
// "role" (a corner, a quadrant, the cell centre, a vy half-cell) folds the
// markers of one cell per lane, in increasing marker index, with FP32
// compensated sums.  The per-cell partial sums are then combined per node in
// a fixed order.  The result is deterministic: it does not depend on thread
// scheduling, and there are no floating-point atomics.
#include "eb_internal.h"

namespace {

constexpr int kChunk = 288;  // staging slots per pass (32 cells x 9)
constexpr float kRad2Deg = 57.295779513082320876798f;

enum { C_UL = 0, C_LL = 1, C_UR = 2, C_LR = 3 };

__device__ __forceinline__ int32_t cell_id(int32_t ci, int32_t cj, int32_t ynum) {
  return (cj - 1) * (ynum - 1) + (ci - 1);
}

// Geometry of one basic-cell column ix (1-based), loaded once per staging thread: every
// marker of a cell lies in the cell's column, so the cell-sorted folds need no per-marker
// xn load and no per-marker geometry gathers.
struct ColW { float vlo, vhi, sx, r0, r1; };  // vyoff_lo/hi[ix-1], sxf[ix-1], rsxvyf[ix-1], rsxvyf[ix]
__device__ __forceinline__ ColW col_weights(const DevGrid& g, int32_t ix) {
  const float4 c0 = __ldg(&g.colx[2 * (ix - 1)]), c1 = __ldg(&g.colx[2 * (ix - 1) + 1]);
  return ColW{c0.z, c0.w, c0.x, c1.x, c1.y};
}

// Weights of one marker from its stored FP32 normalised offsets.
struct MW {
  W4 b;       // basic UL, LL, UR, LR
  float wc;   // central (pressure) node
  W4 vy;      // vy-grid corners
  int half;   // 0: vy cell = xn, 1: vy cell = xn + 1
};
__device__ __forceinline__ MW marker_weights(const ColW& c, float fx, float fy, uint8_t fl) {
  MW w;
  w.b = wts(fx, fy);
  w.wc = (1.f - fabsf(0.5f - fx)) * (1.f - fabsf(0.5f - fy));
  w.half = (fl & MF_VYRIGHT) ? 1 : 0;
  const float off = w.half ? c.vhi : c.vlo;
  const float dxv = (fx * c.sx - off) * (w.half ? c.r1 : c.r0);
  w.vy = wts(dxv, fy);
  return w;
}

// Bit q set when the marker belongs to exclusive quadrant q (UL, LL, UR, LR).
// A marker exactly on a half line belongs to two (or four) quadrants.
__device__ __forceinline__ uint32_t quadrant_mask(uint8_t fl) {
  const bool xl = fl & MF_XLE, xg = fl & MF_XGE, yl = fl & MF_YLE, yg = fl & MF_YGE;
  return (xl && yl ? 1u : 0u) | (xl && yg ? 2u : 0u) | (xg && yl ? 4u : 0u) | (xg && yg ? 8u : 0u);
}

// Compensated accumulators in shared memory, indexed per lane: slot k of lane j is
// the float4 (s0, s1, c0, c1) at a[k*32 + j] -- one accumulator pair, or one
// accumulator in the .x/.z halves.  The 32 lanes of a warp read 32 consecutive
// float4 whichever slot each lane picks (a lane's slot can depend on its marker,
// e.g. on the marker's quadrant), so an add is one 128-bit load and one store.
struct SAcc {
  float4* a;
  __device__ __forceinline__ void add2(int k, int lane, float2 v) const {
    float4* p = a + k * 32 + lane;
    const float4 q = *p;
    float2 sv = make_float2(q.x, q.y), cv = make_float2(q.z, q.w);
    two_sum2(sv, cv, v);
    *p = make_float4(sv.x, sv.y, cv.x, cv.y);
  }
  __device__ __forceinline__ void add1(int k, int lane, float v) const {
    float4* p = a + k * 32 + lane;
    const float4 q = *p;
    KSum t{q.x, q.z};
    t.add(v);
    p->x = t.s;
    p->z = t.c;
  }
  __device__ __forceinline__ float get0(int k, int lane) const { const float4 q = a[k * 32 + lane]; return q.x + q.z; }
  __device__ __forceinline__ float get1(int k, int lane) const { const float4 q = a[k * 32 + lane]; return q.y + q.w; }
};

// ---------------------------------------------------------------- staging ---
// Stage layout indices (rows of the shared-memory table).
enum { S_UL = 0, S_LL, S_UR, S_LR, S_WC, S_VUL, S_VLL, S_VUR, S_VLR, S_HALF, S_V0 };

__device__ __forceinline__ void stage_weights(float (*sv)[kChunk], int t, const MW& w) {
  sv[S_UL][t] = w.b.ul; sv[S_LL][t] = w.b.ll; sv[S_UR][t] = w.b.ur; sv[S_LR][t] = w.b.lr;
  sv[S_WC][t] = w.wc;
  sv[S_VUL][t] = w.vy.ul; sv[S_VLL][t] = w.vy.ll; sv[S_VUR][t] = w.vy.ur; sv[S_VLR][t] = w.vy.lr;
  sv[S_HALF][t] = (float)w.half;
}

// ------------------------------------------------------------------ specs ---
// Each spec defines: kRoles (folding warps, <= 8), kNV (staged rows), kAcc
// (register accumulator pairs KSum2 per folding thread), kSlots (shared-memory
// accumulator slots, SAcc, each a pair), a Cell record of per-cell constants and
// cell() that loads them (once per staging thread: a thread stages the same cell in
// every pass), a Raw record of the marker fields it reads, load() (the global loads
// only, issued one pass ahead), put() (arithmetic on a loaded Raw and the cell's
// constants, marker write-backs, staging), accum() and store().  Every
// accumulator receives its cell's markers in slot (marker) order; accumulators
// travel in pairs through packed FP32x2 arithmetic where two share a role.

// Denominators: wtnodes (incl), wtetas (excl), wtetan (central), wtnodes_vy.
// part slots: 0-3 incl corners, 4-7 excl quadrants, 8 central, 9-16 vy half*4+corner
struct DenomSpec {
  static constexpr const char* kName = "k_cells<denominators>";
  // roles: 0-1 inclusive corners {0,1} / {2,3} (registers), 2 exclusive quadrants (shared
  //        slot q), 3 central node (registers), 4-5 vy corners {0,1} / {2,3} (shared pair
  //        slot 4 + 2*half + pair)
  static constexpr int kRoles = 6, kNV = S_V0, kAcc = 1, kSlots = 8;
  using Cell = ColW;
  __device__ Cell cell(const DevGrid& g, int32_t, int32_t ix) const { return col_weights(g, ix); }
  struct Raw { float fx, fy; uint8_t fl; };
  __device__ Raw load(const DevMarkers& mk, int32_t m) const {
    return Raw{mk.fx[m], mk.fy[m], mk.mflags[m]};
  }
  __device__ void put(const Raw& r, const Cell& cc, const DevMarkers&, const DevGrid&, int t, float (*sv)[kChunk],
                      uint8_t* sfl) const {
    stage_weights(sv, t, marker_weights(cc, r.fx, r.fy, r.fl));
    sfl[t] = r.fl;
  }
  __device__ void accum(int role, int lane, int t, float (*sv)[kChunk], const uint8_t* sfl, KSum2* a, SAcc sa) const {
    if (role < 2) {
      a[0].add(make_float2(sv[S_UL + 2 * role][t], sv[S_UL + 2 * role + 1][t]));
    } else if (role == 2) {
      for (uint32_t m = quadrant_mask(sfl[t]); m; m &= m - 1) {
        const int q = __ffs(m) - 1;
        sa.add1(q, lane, sv[S_UL + q][t]);
      }
    } else if (role == 3) {
      a[0].add(make_float2(sv[S_WC][t], 0.f));
    } else {
      const int h = (int)sv[S_HALF][t], p = role - 4;
      sa.add2(4 + 2 * h + p, lane, make_float2(sv[S_VUL + 2 * p][t], sv[S_VUL + 2 * p + 1][t]));
    }
  }
  __device__ void store(int role, int lane, int32_t cell, int32_t nc, const KSum2* a, SAcc sa, float* part) const {
    if (role < 2) {
      part[(size_t)(2 * role) * nc + cell] = a[0].x();
      part[(size_t)(2 * role + 1) * nc + cell] = a[0].y();
    } else if (role == 2) {
      for (int q = 0; q < 4; ++q) part[(size_t)(4 + q) * nc + cell] = sa.get0(q, lane);
    } else if (role == 3) {
      part[(size_t)8 * nc + cell] = a[0].x();
    } else {
      const int p = role - 4;
      for (int h = 0; h < 2; ++h) {
        part[(size_t)(9 + 4 * h + 2 * p) * nc + cell] = sa.get0(4 + 2 * h + p, lane);
        part[(size_t)(9 + 4 * h + 2 * p + 1) * nc + cell] = sa.get1(4 + 2 * h + p, lane);
      }
    }
  }
};

// Stokes numerators (BilinearNumerator.jl:205-454).
// values: rho, coh, fric_deg, eta_flow, eta, mu_inv, sxy, plast, dil, melt, sxx
enum { V_RHO = S_V0, V_COH, V_FRIC, V_ETAF, V_ETA, V_MUI, V_SXY, V_PLAST, V_DIL, V_MELT, V_SXX, V_END };
// part slots: 0-3 incl rho; 4 + 7*q + f excl (f: coh, fric, eta_flow, eta, mu_inv, sxy, plast);
//             32-37 central (eta, mu_inv, plast, dil, melt, sxx); 38-45 vy rho half*4+corner
struct StokesSpec {
  static constexpr const char* kName = "k_cells<stokes>";
  // Eight roles of about equal work:
  //   0 inclusive rho, corner pairs {UL, LL}, {UR, LR} (registers)
  //   1-3 exclusive field pairs {coh, fric}, {eta_flow, eta}, {mu_inv, sxy} (shared pair slot 4(role-1) + q)
  //   4 exclusive plast (shared slot 12 + q) + central {eta, mu_inv} (registers)
  //   5 central {plast, dil}, {melt, sxx} (registers)
  //   6-7 vy rho corner pairs {0, 1}, {2, 3} (shared pair slot 16 + 2*half + pair)
  static constexpr int kRoles = 8, kNV = V_END, kAcc = 2, kSlots = 20;
  const double* mat_mu;
  int32_t* dflag;
  // (the column geometry is loaded per marker here: held per cell it costs this fold its
  // fourth resident block at 64 registers)
  struct Cell {};
  __device__ Cell cell(const DevGrid&, int32_t, int32_t) const { return Cell{}; }
  struct Raw {
    double rho, coh, fric, etaf, eta, sxy, melt, sxx;
    float fx, fy, plast, dil;
    int32_t xn, mt;
    uint8_t fl;
  };
  __device__ Raw load(const DevMarkers& mk, int32_t m) const {
    Raw r;
    r.fl = mk.mflags[m]; r.xn = mk.xn[m]; r.fx = mk.fx[m]; r.fy = mk.fy[m]; r.mt = mk.matid[m];
    r.rho = mk.rho[m]; r.coh = mk.cohesion[m]; r.fric = mk.fric[m]; r.etaf = mk.eta_flow[m];
    r.eta = mk.eta[m]; r.sxy = mk.sxy[m]; r.plast = mk.pfailure[m]; r.dil = mk.dilat[m];
    r.melt = mk.melt[m]; r.sxx = mk.sxx[m];
    return r;
  }
  __device__ void put(const Raw& r, const Cell&, const DevMarkers&, const DevGrid& g, int t, float (*sv)[kChunk],
                      uint8_t* sfl) const {
    stage_weights(sv, t, marker_weights(col_weights(g, r.xn), r.fx, r.fy, r.fl));
    sfl[t] = r.fl;
    const double mu = __ldg(&mat_mu[r.mt - 1]);
    if ((__double_as_longlong(mu) << 1) == 0) atomicOr(dflag, 2);  // reference raises on a zero shear modulus
    sv[V_RHO][t] = d2f(r.rho);
    sv[V_COH][t] = d2f(r.coh);
    sv[V_FRIC][t] = asinf(d2f(r.fric)) * kRad2Deg;
    sv[V_ETAF][t] = d2f(r.etaf);
    sv[V_ETA][t] = d2f(r.eta);
    sv[V_MUI][t] = 1.f / d2f(mu);
    sv[V_SXY][t] = d2f(r.sxy);
    sv[V_PLAST][t] = r.plast;
    sv[V_DIL][t] = r.dil;
    sv[V_MELT][t] = d2f(r.melt);
    sv[V_SXX][t] = d2f(r.sxx);
  }
  __device__ void accum(int role, int lane, int t, float (*sv)[kChunk], const uint8_t* sfl, KSum2* a, SAcc sa) const {
    if (role == 0) {
      const float2 r = make_float2(sv[V_RHO][t], sv[V_RHO][t]);
      a[0].add(__fmul2_rn(make_float2(sv[S_UL][t], sv[S_LL][t]), r));
      a[1].add(__fmul2_rn(make_float2(sv[S_UR][t], sv[S_LR][t]), r));
    } else if (role <= 4) {
      const int f0 = 2 * (role - 1);  // exclusive fields f0, f0 + 1 (role 4: plast only)
      for (uint32_t m = quadrant_mask(sfl[t]); m; m &= m - 1) {
        const int q = __ffs(m) - 1;
        const float w = sv[S_UL + q][t];
        if (role < 4) {
          sa.add2(4 * (role - 1) + q, lane,
                  __fmul2_rn(make_float2(w, w), make_float2(sv[V_COH + f0][t], sv[V_COH + f0 + 1][t])));
        } else {
          sa.add1(12 + q, lane, w * sv[V_PLAST][t]);
        }
      }
      if (role == 4) {
        const float w = sv[S_WC][t];
        a[0].add(__fmul2_rn(make_float2(w, w), make_float2(sv[V_ETA][t], sv[V_MUI][t])));
      }
    } else if (role == 5) {
      const float2 w = make_float2(sv[S_WC][t], sv[S_WC][t]);
      a[0].add(__fmul2_rn(w, make_float2(sv[V_PLAST][t], sv[V_DIL][t])));
      a[1].add(__fmul2_rn(w, make_float2(sv[V_MELT][t], sv[V_SXX][t])));
    } else {
      const int h = (int)sv[S_HALF][t], p = role - 6;
      const float r = sv[V_RHO][t];
      sa.add2(16 + 2 * h + p, lane,
              __fmul2_rn(make_float2(sv[S_VUL + 2 * p][t], sv[S_VUL + 2 * p + 1][t]), make_float2(r, r)));
    }
  }
  __device__ void store(int role, int lane, int32_t cell, int32_t nc, const KSum2* a, SAcc sa, float* part) const {
    if (role == 0) {
      part[(size_t)0 * nc + cell] = a[0].x();
      part[(size_t)1 * nc + cell] = a[0].y();
      part[(size_t)2 * nc + cell] = a[1].x();
      part[(size_t)3 * nc + cell] = a[1].y();
    } else if (role < 4) {
      const int f0 = 2 * (role - 1);
      for (int q = 0; q < 4; ++q) {
        part[(size_t)(4 + 7 * q + f0) * nc + cell] = sa.get0(4 * (role - 1) + q, lane);
        part[(size_t)(4 + 7 * q + f0 + 1) * nc + cell] = sa.get1(4 * (role - 1) + q, lane);
      }
    } else if (role == 4) {
      for (int q = 0; q < 4; ++q) part[(size_t)(4 + 7 * q + 6) * nc + cell] = sa.get0(12 + q, lane);
      part[(size_t)32 * nc + cell] = a[0].x();
      part[(size_t)33 * nc + cell] = a[0].y();
    } else if (role == 5) {
      part[(size_t)34 * nc + cell] = a[0].x();
      part[(size_t)35 * nc + cell] = a[0].y();
      part[(size_t)36 * nc + cell] = a[1].x();
      part[(size_t)37 * nc + cell] = a[1].y();
    } else {
      const int p = role - 6;
      for (int h = 0; h < 2; ++h) {
        part[(size_t)(38 + 4 * h + 2 * p) * nc + cell] = sa.get0(16 + 2 * h + p, lane);
        part[(size_t)(38 + 4 * h + 2 * p + 1) * nc + cell] = sa.get1(16 + 2 * h + p, lane);
      }
    }
  }
};

// Heat numerators (BilinearNumerator.jl:31-141): tk, kt, rhocp, hr(+serp), ha; part slots 5*corner + f.
// With kDen the same fold also sums the weight denominators of DenomSpec (BilinearDenominator.jl:34-157)
// into part slots kDenBase + DenomSpec's slot: the bilinear set-up and the heat scatter of a marker
// cycle then walk the cell lists once.  Every sum receives the same terms in the same order as in
// DenomSpec (a term of 0 leaves a compensated sum unchanged), so the denominators are bit-identical.
constexpr int kDenBase = 20;
template <bool kDen>
struct HeatSpecT {
  static constexpr const char* kName = kDen ? "k_cells<heat+denominators>" : "k_cells<heat>";
  // roles: corner (role & 3) x field pairs {tk, kt} + {ha, incl weight} (role < 4) or {rhocp, hr}
  //        (role >= 4); with kDen roles >= 4 also sum {excl weight of quadrant k, vy weight half 0}
  //        and {vy weight half 1, central weight (role 4)}
  static constexpr int kRoles = 8, kNV = S_V0 + 5, kAcc = kDen ? 3 : 2, kSlots = 0;
  const double* mat_hr;
  int use_serp;
  struct Cell { ColW col; };
  __device__ Cell cell(const DevGrid& g, int32_t, int32_t ix) const {
    Cell c{};
    if (kDen) c.col = col_weights(g, ix);
    return c;
  }
  struct Raw { double tk, kt, rhocp, ha, serp; float fx, fy; int32_t mt; uint8_t fl; };
  __device__ Raw load(const DevMarkers& mk, int32_t m) const {
    Raw r;
    r.fx = mk.fx[m]; r.fy = mk.fy[m]; r.mt = mk.matid[m];
    r.tk = mk.tk[m]; r.kt = mk.kt[m]; r.rhocp = mk.rhocp[m]; r.ha = mk.ha[m];
    r.serp = use_serp ? mk.serp_hr[m] : 0.0;
    if (kDen) r.fl = mk.mflags[m];
    return r;
  }
  __device__ void put(const Raw& r, const Cell& cc, const DevMarkers&, const DevGrid&, int t, float (*sv)[kChunk],
                      uint8_t* sfl) const {
    if (kDen) {
      stage_weights(sv, t, marker_weights(cc.col, r.fx, r.fy, r.fl));
      sfl[t] = r.fl;
    } else {
      const W4 w = wts(r.fx, r.fy);
      sv[S_UL][t] = w.ul; sv[S_LL][t] = w.ll; sv[S_UR][t] = w.ur; sv[S_LR][t] = w.lr;
    }
    double hr = __ldg(&mat_hr[r.mt - 1]);
    if (use_serp) hr = hr + r.serp;
    sv[S_V0 + 0][t] = d2f(r.tk);
    sv[S_V0 + 1][t] = d2f(r.kt);
    sv[S_V0 + 2][t] = d2f(r.rhocp);
    sv[S_V0 + 3][t] = d2f(hr);
    sv[S_V0 + 4][t] = d2f(r.ha);
  }
  __device__ void accum(int role, int, int t, float (*sv)[kChunk], const uint8_t* sfl, KSum2* a, SAcc) const {
    const int k = role & 3;
    const float w = sv[S_UL + k][t];
    const float2 w2 = make_float2(w, w);
    if (role < 4) {
      a[0].add(__fmul2_rn(w2, make_float2(sv[S_V0 + 0][t], sv[S_V0 + 1][t])));
      a[1].add(make_float2(w * sv[S_V0 + 4][t], kDen ? w : 0.f));
    } else {
      a[0].add(__fmul2_rn(w2, make_float2(sv[S_V0 + 2][t], sv[S_V0 + 3][t])));
      if (kDen) {
        const float wv = sv[S_VUL + k][t];
        const bool h1 = sv[S_HALF][t] != 0.f;
        a[1].add(make_float2(((quadrant_mask(sfl[t]) >> k) & 1u) ? w : 0.f, h1 ? 0.f : wv));
        a[2].add(make_float2(h1 ? wv : 0.f, k == 0 ? sv[S_WC][t] : 0.f));
      }
    }
  }
  __device__ void store(int role, int, int32_t cell, int32_t nc, const KSum2* a, SAcc, float* part) const {
    const int k = role & 3;
    if (role < 4) {
      part[(size_t)(5 * k + 0) * nc + cell] = a[0].x();
      part[(size_t)(5 * k + 1) * nc + cell] = a[0].y();
      part[(size_t)(5 * k + 4) * nc + cell] = a[1].x();
      if (kDen) part[(size_t)(kDenBase + k) * nc + cell] = a[1].y();
    } else {
      part[(size_t)(5 * k + 2) * nc + cell] = a[0].x();
      part[(size_t)(5 * k + 3) * nc + cell] = a[0].y();
      if (kDen) {
        part[(size_t)(kDenBase + 4 + k) * nc + cell] = a[1].x();
        part[(size_t)(kDenBase + 9 + k) * nc + cell] = a[1].y();
        part[(size_t)(kDenBase + 13 + k) * nc + cell] = a[2].x();
        if (k == 0) part[(size_t)(kDenBase + 8) * nc + cell] = a[2].y();
      }
    }
  }
};
using HeatSpec = HeatSpecT<false>;

// Viscosity re-scatter (BilinearNumerator.jl:470-533): part slots 0-3 excl eta, 4 central eta
// roles: 0 exclusive quadrants (shared slot q), 1 central node (registers)
struct ViscSpec {
  static constexpr const char* kName = "k_cells<viscosity>";
  // roles 0-3: the exclusive quadrant of that index (registers), 4: the central node; one warp
  // per quadrant keeps the fold short (a marker usually lies in one quadrant)
  static constexpr int kRoles = 5, kNV = S_V0 + 1, kAcc = 1, kSlots = 0;
  struct Cell {};
  __device__ Cell cell(const DevGrid&, int32_t, int32_t) const { return Cell{}; }
  struct Raw { double eta; float fx, fy; uint8_t fl; };
  __device__ Raw load(const DevMarkers& mk, int32_t m) const {
    return Raw{mk.eta[m], mk.fx[m], mk.fy[m], mk.mflags[m]};
  }
  __device__ void put(const Raw& r, const Cell&, const DevMarkers&, const DevGrid&, int t, float (*sv)[kChunk],
                      uint8_t* sfl) const {
    const W4 w = wts(r.fx, r.fy);
    sv[S_UL][t] = w.ul; sv[S_LL][t] = w.ll; sv[S_UR][t] = w.ur; sv[S_LR][t] = w.lr;
    sv[S_WC][t] = (1.f - fabsf(0.5f - r.fx)) * (1.f - fabsf(0.5f - r.fy));
    sfl[t] = r.fl;
    sv[S_V0][t] = d2f(r.eta);
  }
  __device__ void accum(int role, int lane, int t, float (*sv)[kChunk], const uint8_t* sfl, KSum2* a, SAcc sa) const {
    const float e = sv[S_V0][t];
    if (role < 4) {
      if ((quadrant_mask(sfl[t]) >> role) & 1u) a[0].add(make_float2(sv[S_UL + role][t] * e, 0.f));
    } else {
      a[0].add(make_float2(sv[S_WC][t] * e, 0.f));
    }
  }
  __device__ void store(int role, int, int32_t cell, int32_t nc, const KSum2* a, SAcc, float* part) const {
    part[(size_t)role * nc + cell] = a[0].x();
  }
};


// Pressure-grid bilinear gather of one marker (GridToMarker.jl:104-153 with
// MarkerGridMapping.upr_left_index_pressure / upr_left_dist_pressure, :311-350).
__device__ __forceinline__ float gather_pressure_grid(const float* __restrict__ pg, const DevGrid& g, int32_t ix,
                                                      int32_t iy, float fx, float fy) {
  const float lx = fx * __ldg(&g.sxf[ix - 1]);
  const float ly = fy * __ldg(&g.syf[iy - 1]);
  const float hx = __ldg(&g.vyoff_hi[ix - 1]), hy = __ldg(&g.vxoff_hi[iy - 1]);
  int32_t xp = (lx < hx) ? ix - 1 : ix;
  int32_t yp = (ly < hy) ? iy - 1 : iy;
  xp = clamp_i(xp, 1, g.xnum - 2);
  yp = clamp_i(yp, 1, g.ynum - 2);
  // staggered node xp+1 lies at offset vyoff_lo (== ix) or vyoff_hi (== ix+1) from gx[ix]
  const float ox = (xp + 1 == ix) ? __ldg(&g.vyoff_lo[ix - 1]) : hx;
  const float oy = (yp + 1 == iy) ? __ldg(&g.vxoff_lo[iy - 1]) : hy;
  const float dxp = (lx - ox) * __ldg(&g.rsxvyf[xp]);
  const float dyp = (ly - oy) * __ldg(&g.rsyvxf[yp]);
  return gather4f(pg, g.ynum - 1, yp, xp, dxp, dyp);
}

// Subgrid stress (SubgridShearStress.jl:27-96, SubgridNormalStress.jl:27-89):
// put() relaxes the marker stress, writes it back and stages the relaxed change.
// part slots: 0-3 excl relax_xy*w, 4-7 excl w, 8 central relax_xx*wc, 9 central wc
// roles 0-3: the exclusive quadrant of that index ({relax_xy*w, w} in registers), 4: the central
// node; one warp per quadrant keeps the fold, which the staging warps wait for, short
struct SubgridStressSpec {
  static constexpr const char* kName = "k_cells<subgrid_stress>";
  static constexpr int kRoles = 5, kNV = S_V0 + 2, kAcc = 1, kSlots = 0;
  const float *sxy1, *sxx1;  // FP32 mirrors
  const double* mat_mu;
  float dt, coef;
  // the cell's basic indices and its four sxy1 nodes (UL, LL, UR, LR)
  struct Cell { int32_t iy, ix; float n0, n1, n2, n3; };
  __device__ Cell cell(const DevGrid& g, int32_t iy, int32_t ix) const {
    const float* p = sxy1 + ((ix - 1) * g.ynum + (iy - 1));
    return Cell{iy, ix, __ldg(p), __ldg(p + 1), __ldg(p + g.ynum), __ldg(p + g.ynum + 1)};
  }
  struct Raw { double eta, sxy, sxx; int32_t m, mt; float fx, fy; uint8_t fl; };
  __device__ Raw load(const DevMarkers& mk, int32_t m) const {
    Raw r;
    r.m = m; r.fl = mk.mflags[m]; r.fx = mk.fx[m]; r.fy = mk.fy[m];
    r.mt = mk.matid[m]; r.eta = mk.eta[m]; r.sxy = mk.sxy[m]; r.sxx = mk.sxx[m];
    return r;
  }
  __device__ void put(const Raw& r, const Cell& cc, const DevMarkers& mk, const DevGrid& g, int t, float (*sv)[kChunk],
                      uint8_t* sfl) const {
    const W4 w = wts(r.fx, r.fy);
    sv[S_UL][t] = w.ul; sv[S_LL][t] = w.ll; sv[S_UR][t] = w.ur; sv[S_LR][t] = w.lr;
    sv[S_WC][t] = (1.f - fabsf(0.5f - r.fx)) * (1.f - fabsf(0.5f - r.fy));
    sfl[t] = r.fl;
    // DiffusionTerm.calculate_subgrid_stress_diffusion_term (DiffusionTerm.jl:14-29)
    const float mu = d2f(__ldg(&mat_mu[r.mt - 1]));
    const float maxwell = d2f(r.eta) / mu;
    const float sdif = fmaxf(-coef * dt / maxwell, -30.f);
    const float term = -expm1f(sdif);  // 1 - exp(sdif), accurate for small |sdif|
    const float sxy_g = gather4v(cc.n0, cc.n1, cc.n2, cc.n3, r.fx, r.fy);
    const float rxy = (sxy_g - d2f(r.sxy)) * term;
    mk.sxy[r.m] = r.sxy + f2d(rxy);
    const float sxx_g = gather_pressure_grid(sxx1, g, cc.ix, cc.iy, r.fx, r.fy);
    const float rxx = (sxx_g - d2f(r.sxx)) * term;
    mk.sxx[r.m] = r.sxx + f2d(rxx);
    sv[S_V0][t] = rxy;
    sv[S_V0 + 1][t] = rxx;
  }
  __device__ void accum(int role, int lane, int t, float (*sv)[kChunk], const uint8_t* sfl, KSum2* a, SAcc sa) const {
    if (role < 4) {
      if ((quadrant_mask(sfl[t]) >> role) & 1u) {
        const float w = sv[S_UL + role][t];
        a[0].add(make_float2(w * sv[S_V0][t], w));
      }
    } else {
      const float w = sv[S_WC][t];
      a[0].add(make_float2(w * sv[S_V0 + 1][t], w));
    }
  }
  __device__ void store(int role, int, int32_t cell, int32_t nc, const KSum2* a, SAcc, float* part) const {
    const int q = role < 4 ? role : 8;
    part[(size_t)q * nc + cell] = a[0].x();
    part[(size_t)(q < 4 ? 4 + q : 9) * nc + cell] = a[0].y();
  }
};

// Subgrid heat diffusion (SubgridDiffusion.jl:67-175): part slots 0-3 dT*w, 4-7 w
// roles 0-3: one corner each, {dT*w, w} packed
struct SubgridHeatSpec {
  static constexpr const char* kName = "k_cells<subgrid_heat>";
  static constexpr int kRoles = 4, kNV = S_V0 + 1, kAcc = 1, kSlots = 0;
  const float *tk1, *kt1, *rhocp1;  // FP32 mirrors
  float dt, coef, inv_ts;  // inv_ts = 2/xstpavg^2 + 2/ystpavg^2
  // the four nodes (UL, LL, UR, LR) of the cell in tk1, kt1 and rhocp1
  struct Cell { float4 tk, kt, rc; };
  __device__ static float4 nodes(const float* f, const DevGrid& g, int32_t iy, int32_t ix) {
    const float* p = f + ((ix - 1) * g.ynum + (iy - 1));
    return make_float4(__ldg(p), __ldg(p + 1), __ldg(p + g.ynum), __ldg(p + g.ynum + 1));
  }
  __device__ Cell cell(const DevGrid& g, int32_t iy, int32_t ix) const {
    return Cell{nodes(tk1, g, iy, ix), nodes(kt1, g, iy, ix), nodes(rhocp1, g, iy, ix)};
  }
  struct Raw { double tk; int32_t m; float fx, fy; };
  __device__ Raw load(const DevMarkers& mk, int32_t m) const {
    return Raw{mk.tk[m], m, mk.fx[m], mk.fy[m]};
  }
  __device__ void put(const Raw& r, const Cell& cc, const DevMarkers& mk, const DevGrid&, int t, float (*sv)[kChunk],
                      uint8_t*) const {
    const W4 w = wts(r.fx, r.fy);
    sv[S_UL][t] = w.ul; sv[S_LL][t] = w.ll; sv[S_UR][t] = w.ur; sv[S_LR][t] = w.lr;
    const float tn = gather4v(cc.tk.x, cc.tk.y, cc.tk.z, cc.tk.w, r.fx, r.fy);
    const float k = gather4v(cc.kt.x, cc.kt.y, cc.kt.z, cc.kt.w, r.fx, r.fy);
    const float rc = gather4v(cc.rc.x, cc.rc.y, cc.rc.z, cc.rc.w, r.fx, r.fy);
    const float tsg = rc / k / inv_ts;
    const float term = fmaxf(-coef * dt / tsg, -30.f);
    const float d = (tn - d2f(r.tk)) * (-expm1f(term));
    mk.subgrid_dt[r.m] = f2d(d);
    mk.tk[r.m] = r.tk + f2d(d);
    sv[S_V0][t] = d;
  }
  __device__ void accum(int role, int, int t, float (*sv)[kChunk], const uint8_t*, KSum2* a, SAcc) const {
    const float w = sv[S_UL + role][t];
    a[0].add(make_float2(w * sv[S_V0][t], w));
  }
  __device__ void store(int role, int, int32_t cell, int32_t nc, const KSum2* a, SAcc, float* part) const {
    part[(size_t)role * nc + cell] = a[0].x();
    part[(size_t)(4 + role) * nc + cell] = a[0].y();
  }
};


// ------------------------------------------------------- per-cell kernel ---
// Block = 256 threads = 32 consecutive cells.  Pass p stages markers
// [8p, 8p+8) of every cell: thread t owns marker 8p + (t & 7) of cell t >> 3,
// so eight consecutive threads read eight consecutive entries of one cell's
// list (coalesced), and stage it to slot (t >> 3) * 9 + (t & 7).  The global
// loads of pass p+1 are issued into registers before the fold of pass p, so
// their latency hides behind the fold.  Warp `role` < kRoles, lane j folds
// cell j's slots j*9 .. j*9+7 in order (stride 9 keeps the 32 lanes on 32
// different banks), so each cell is folded in its marker order.
constexpr int kThreads = 256;
constexpr int kPer = 8;             // markers per cell per pass
constexpr int kSlotStride = kPer + 1;
static_assert(kChunk >= 32 * kSlotStride, "staging table too small");
static_assert(kThreads == 32 * kPer, "one staged marker per thread per pass");

template <class S>
__global__ void __launch_bounds__(kThreads, 4) k_cells(S spec, DevMarkers mk, DevGrid g,
                                                    const int32_t* __restrict__ start,
                                                    const int32_t* __restrict__ perm, int32_t nc,
                                                    float* __restrict__ part) {
  static_assert(S::kRoles <= kThreads / 32, "one warp per role");
  __shared__ float sv[S::kNV][kChunk];
  __shared__ uint8_t sfl[kChunk];
  __shared__ int32_t s_beg[32], s_cnt[32], s_max;
  __shared__ float4 s_acc[S::kSlots > 0 ? S::kSlots * 32 : 1];
  for (int k = threadIdx.x; k < S::kSlots * 32; k += blockDim.x) s_acc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
  const SAcc sa{s_acc};
  const int lane = threadIdx.x & 31, role = threadIdx.x >> 5;
  const int sj = threadIdx.x >> 3, si = threadIdx.x & 7;  // staging cell / marker of this thread
  const int32_t c0 = blockIdx.x * 32;
  if (threadIdx.x < 32) {
    const int32_t cell = c0 + lane;
    const int32_t b = cell < nc ? start[cell] : 0;
    const int32_t n = cell < nc ? start[cell + 1] - b : 0;
    s_beg[lane] = b;
    s_cnt[lane] = n;
    int32_t mx = n;
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) s_max = mx;
  }
  __syncthreads();
  const int32_t nmax = s_max;
  const int32_t my_cnt = s_cnt[lane];
  const int32_t st_beg = s_beg[sj], st_cnt = s_cnt[sj];
  // constants of this thread's staging cell (basic indices iy, ix; markers of the cell-sorted
  // list of a cell carry exactly these indices)
  typename S::Cell cc{};
  if (st_cnt > 0) {
    const int32_t cell = c0 + sj, rows = g.ynum - 1;
    cc = spec.cell(g, cell % rows + 1, cell / rows + 1);
  }
  KSum2 acc[S::kAcc];
#pragma unroll
  for (int k = 0; k < S::kAcc; ++k) acc[k].init();
  // The marker index of a staged entry is read one pass before its fields: the field
  // loads of pass p+1 then wait for one memory latency, not for a perm load and then them.
  typename S::Raw r;
  bool have = si < st_cnt;
  int32_t m_next = kPer + si < st_cnt ? __ldg(&perm[st_beg + kPer + si]) : -1;
  if (have) r = spec.load(mk, __ldg(&perm[st_beg + si]));
  for (int32_t base = 0; base < nmax; base += kPer) {
    __syncthreads();
    if (have) spec.put(r, cc, mk, g, sj * kSlotStride + si, sv, sfl);
    __syncthreads();
    have = m_next >= 0;
    if (have) r = spec.load(mk, m_next);
    const int32_t nxt2 = base + 2 * kPer + si;
    m_next = nxt2 < st_cnt ? __ldg(&perm[st_beg + nxt2]) : -1;
    if (role < S::kRoles) {
      const int n = min(kPer, my_cnt - base);
      for (int i = 0; i < n; ++i) spec.accum(role, lane, lane * kSlotStride + i, sv, sfl, acc, sa);
    }
  }
  if (role < S::kRoles && c0 + lane < nc) spec.store(role, lane, c0 + lane, nc, acc, sa, part);
}

template <class S>
int run_cells(eb_ctx* c, const S& spec) {
  const int32_t nc = c->cs.ncells;
  const unsigned blocks = (unsigned)((nc + 31) / 32);
  EB_PROF(c, S::kName);
  k_cells<S><<<blocks, kThreads, 0, c->stream>>>(spec, dev_markers(c), c->g, c->cs.start, c->cs.perm, nc, c->part);
  EB_LAUNCHED(c);
  return EB_OK;
}

// ---------------------------------------------------- node combination ---
struct NodeCtx {
  const float* part;
  int32_t nc, ynum, xnum;
  __device__ float p(int slot, int32_t ci, int32_t cj) const {
    return part[(size_t)slot * nc + cell_id(ci, cj, ynum)];
  }
  // Sum over the cells around basic node (i, j): LR of (i-1, j-1), UR of (i, j-1),
  // LL of (i-1, j), UL of (i, j).  slot(k) = base + stride * k.
  __device__ float basic(int32_t i, int32_t j, int base, int stride) const {
    KSum s; s.init();
    if (i > 1 && j > 1) s.add(p(base + stride * C_LR, i - 1, j - 1));
    if (i < ynum && j > 1) s.add(p(base + stride * C_UR, i, j - 1));
    if (i > 1 && j < xnum) s.add(p(base + stride * C_LL, i - 1, j));
    if (i < ynum && j < xnum) s.add(p(base + stride * C_UL, i, j));
    return s.get();
  }
  // vy node (i, jv): vy cells (ci, cjv) are the left half of basic cell (ci, cjv)
  // plus the right half of basic cell (ci, cjv-1).  slot = base + half*4 + corner.
  __device__ void vycell(KSum& s, int32_t ci, int32_t cjv, int k, int base) const {
    if (ci < 1 || ci > ynum - 1 || cjv < 1 || cjv > xnum) return;
    if (cjv <= xnum - 1) s.add(p(base + k, ci, cjv));
    if (cjv >= 2) s.add(p(base + 4 + k, ci, cjv - 1));
  }
  __device__ float vy(int32_t i, int32_t jv, int base) const {
    KSum s; s.init();
    vycell(s, i - 1, jv - 1, C_LR, base);
    vycell(s, i, jv - 1, C_UR, base);
    vycell(s, i - 1, jv, C_LL, base);
    vycell(s, i, jv, C_UL, base);
    return s.get();
  }
};

__global__ void k_finish_denoms(NodeCtx n, int base, double* wtnodes, double* wtetas, double* wtetan,
                                double* wtnodes_vy) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nb = (int64_t)n.ynum * n.xnum, np = (int64_t)(n.ynum - 1) * (n.xnum - 1),
                nv = (int64_t)n.ynum * (n.xnum + 1);
  if (t < nb) {
    const int32_t i = (int32_t)(t % n.ynum) + 1, j = (int32_t)(t / n.ynum) + 1;
    wtnodes[t] = f2d(n.basic(i, j, base + 0, 1));
    wtetas[t] = f2d(n.basic(i, j, base + 4, 1));
  }
  if (t < np) wtetan[t] = f2d(n.part[(size_t)(base + 8) * n.nc + t]);
  if (t < nv) {
    const int32_t i = (int32_t)(t % n.ynum) + 1, jv = (int32_t)(t / n.ynum) + 1;
    wtnodes_vy[t] = f2d(n.vy(i, jv, base + 9));
  }
}

// average with backup: den != 0 -> num/den, else the backup value
// (weight sums are FP32 sums stored in FP64, so d2f(den) is exact)
__device__ __forceinline__ double avg_or(float num, double den, double backup) {
  const float d = d2f(den);
  return d != 0.f ? f2d(num / d) : backup;
}
__device__ __forceinline__ double harm_or(float num, double den, double backup) {
  const float d = d2f(den);
  return d != 0.f ? f2d(d / num) : backup;
}

struct StokesGrids {
  double *rho1, *rho0, *etas1, *etas0, *eta_flow, *eta_flow0, *mus1, *mus0, *sxy1, *sxy0;
  double *plastics, *plastics0, *coh, *coh0, *fric, *fric0;
  double *etan1, *etan0, *mun1, *mun0, *sxx1, *sxx0, *plasticn, *plasticn0, *dil, *dil0, *melt, *melt0;
  double *rho1_vy, *rho0_vy;
  const double *wtnodes, *wtetas, *wtetan, *wtnodes_vy, *hr1, *gy;
  int iuse_topo;
  double y_sealevel, rho_air, rho_water;
};

__global__ void k_finish_stokes(NodeCtx n, StokesGrids G) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nb = (int64_t)n.ynum * n.xnum, np = (int64_t)(n.ynum - 1) * (n.xnum - 1),
                nv = (int64_t)n.ynum * (n.xnum + 1);
  if (t < nb) {
    const int32_t i = (int32_t)(t % n.ynum) + 1, j = (int32_t)(t / n.ynum) + 1;
    const double dn = G.wtnodes[t], ds = G.wtetas[t];
    // backups (BackupTransportArrays.backup_stokes_transport_arrays!)
    const double o_rho = G.rho1[t], o_etas = G.etas1[t], o_etaf = G.eta_flow[t], o_mus = G.mus1[t],
                 o_sxy = G.sxy1[t], o_pl = G.plastics[t], o_coh = G.coh[t], o_fr = G.fric[t];
    G.rho0[t] = o_rho; G.etas0[t] = o_etas; G.eta_flow0[t] = o_etaf; G.mus0[t] = o_mus;
    G.sxy0[t] = o_sxy; G.plastics0[t] = o_pl; G.coh0[t] = o_coh; G.fric0[t] = o_fr;
    double rho = avg_or(n.basic(i, j, 0, 1), dn, o_rho);
    // FlattenDensity.flatten_staggered_grid_density_in_sticky_air_layer! (FlattenDensity.jl:48-66)
    if (G.iuse_topo == 1 && G.hr1[t] == 0.0 && rho <= 1100.0) {
      const bool above = G.gy[i - 1] < G.y_sealevel;
      if (above && G.rho_air >= 0.0) rho = G.rho_air;
      else if (!above && G.rho_water >= 0.0) rho = G.rho_water;
    }
    G.rho1[t] = rho;
    G.coh[t] = avg_or(n.basic(i, j, 4 + 0, 7), ds, o_coh);
    G.fric[t] = avg_or(n.basic(i, j, 4 + 1, 7), ds, o_fr);
    G.eta_flow[t] = avg_or(n.basic(i, j, 4 + 2, 7), ds, o_etaf);
    G.etas1[t] = avg_or(n.basic(i, j, 4 + 3, 7), ds, o_etas);
    G.mus1[t] = harm_or(n.basic(i, j, 4 + 4, 7), ds, o_mus);
    G.sxy1[t] = avg_or(n.basic(i, j, 4 + 5, 7), ds, o_sxy);
    G.plastics[t] = avg_or(n.basic(i, j, 4 + 6, 7), ds, o_pl);
  }
  if (t < np) {
    const double dc = G.wtetan[t];
    const double o_etan = G.etan1[t], o_mun = G.mun1[t], o_pl = G.plasticn[t], o_dil = G.dil[t],
                 o_melt = G.melt[t], o_sxx = G.sxx1[t];
    G.etan0[t] = o_etan; G.mun0[t] = o_mun; G.plasticn0[t] = o_pl; G.dil0[t] = o_dil;
    G.melt0[t] = o_melt; G.sxx0[t] = o_sxx;
    const float* P = n.part;
    const size_t nc = n.nc;
    G.etan1[t] = avg_or(P[32 * nc + t], dc, o_etan);
    G.mun1[t] = harm_or(P[33 * nc + t], dc, o_mun);
    G.plasticn[t] = avg_or(P[34 * nc + t], dc, o_pl);
    G.dil[t] = avg_or(P[35 * nc + t], dc, o_dil);
    G.melt[t] = avg_or(P[36 * nc + t], dc, o_melt);
    G.sxx1[t] = avg_or(P[37 * nc + t], dc, o_sxx);
  }
  if (t < nv) {
    const int32_t i = (int32_t)(t % n.ynum) + 1, jv = (int32_t)(t / n.ynum) + 1;
    const double o = G.rho1_vy[t];
    G.rho0_vy[t] = o;
    double rho = avg_or(n.vy(i, jv, 38), G.wtnodes_vy[t], o);
    if (G.iuse_topo == 1 && rho <= 1100.0) {
      const bool above = G.gy[i - 1] < G.y_sealevel;
      if (above && G.rho_air >= 0.0) rho = G.rho_air;
      else if (!above && G.rho_water >= 0.0) rho = G.rho_water;
    }
    G.rho1_vy[t] = rho;
  }
}

struct HeatGrids {
  double *tk1, *tk0, *kt1, *kt0, *rhocp1, *rhocp0, *hr1, *hr0, *ha1, *ha0;
  const double *tk2, *wtnodes;
};
__global__ void k_finish_heat(NodeCtx n, HeatGrids G) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n.ynum * n.xnum) return;
  const int32_t i = (int32_t)(t % n.ynum) + 1, j = (int32_t)(t / n.ynum) + 1;
  const double dn = G.wtnodes[t];
  const double b_tk = G.tk2[t], b_kt = G.kt1[t], b_rc = G.rhocp1[t], b_hr = G.hr1[t], b_ha = G.ha1[t];
  G.tk0[t] = b_tk; G.kt0[t] = b_kt; G.rhocp0[t] = b_rc; G.hr0[t] = b_hr; G.ha0[t] = b_ha;
  G.tk1[t] = avg_or(n.basic(i, j, 0, 5), dn, b_tk);
  G.kt1[t] = avg_or(n.basic(i, j, 1, 5), dn, b_kt);
  G.rhocp1[t] = avg_or(n.basic(i, j, 2, 5), dn, b_rc);
  G.hr1[t] = avg_or(n.basic(i, j, 3, 5), dn, b_hr);
  G.ha1[t] = avg_or(n.basic(i, j, 4, 5), dn, b_ha);
}

// ApplyThermalBC.apply_thermal_bc_along_boundaries! (ApplyThermalBC.jl:20-44): top/bottom rows
// for j in 2:xnum-1, then left/right columns for every i (the column pass runs second).
__global__ void k_thermal_bc_rows(double* tk1, const double* btop, const double* bbot, int32_t ynum, int32_t xnum) {
  const int32_t j = blockIdx.x * blockDim.x + threadIdx.x + 2;
  if (j > xnum - 1) return;
  const size_t col = (size_t)(j - 1) * ynum;
  tk1[col] = btop[j - 1] + btop[xnum + j - 1] * tk1[col + 1];
  tk1[col + ynum - 1] = bbot[j - 1] + bbot[xnum + j - 1] * tk1[col + ynum - 2];
}
__global__ void k_thermal_bc_cols(double* tk1, const double* bl, const double* br, int32_t ynum, int32_t xnum) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (i > ynum) return;
  tk1[i - 1] = bl[i - 1] + bl[ynum + i - 1] * tk1[(size_t)ynum + i - 1];
  tk1[(size_t)(xnum - 1) * ynum + i - 1] = br[i - 1] + br[ynum + i - 1] * tk1[(size_t)(xnum - 2) * ynum + i - 1];
}

__global__ void k_finish_visc(NodeCtx n, double* etas1, const double* etas0, double* etan1, const double* etan0,
                              const double* wtetas, const double* wtetan) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (int64_t)n.ynum * n.xnum) {
    const int32_t i = (int32_t)(t % n.ynum) + 1, j = (int32_t)(t / n.ynum) + 1;
    etas1[t] = avg_or(n.basic(i, j, 0, 1), wtetas[t], etas0[t]);
  }
  if (t < (int64_t)(n.ynum - 1) * (n.xnum - 1)) etan1[t] = avg_or(n.part[(size_t)4 * n.nc + t], wtetan[t], etan0[t]);
}

// BilinearAverage.calc_marker_average_subgrid_stress_change! + RemainingStress (Update.jl:69-87)
__global__ void k_finish_subgrid_stress(NodeCtx n, double* dsxyn, double* dsxxn, double* wtetas, double* wtetan,
                                        double* dsxy, double* dsxx) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (int64_t)n.ynum * n.xnum) {
    const int32_t i = (int32_t)(t % n.ynum) + 1, j = (int32_t)(t / n.ynum) + 1;
    const float num = n.basic(i, j, 0, 1), den = n.basic(i, j, 4, 1);
    const double v = f2d(den != 0.f ? num / den : num);
    dsxyn[t] = v;
    wtetas[t] = f2d(den);
    dsxy[t] = dsxy[t] - v;
  }
  if (t < (int64_t)(n.ynum - 1) * (n.xnum - 1)) {
    const float num = n.part[(size_t)8 * n.nc + t], den = n.part[(size_t)9 * n.nc + t];
    const double v = f2d(den != 0.f ? num / den : num);
    dsxxn[t] = v;
    wtetan[t] = f2d(den);
    dsxx[t] = dsxx[t] - v;
  }
}

// SubgridDiffusion.interpolate_subgrid_temperature_change_to_grid! + remove_subgrid_effects_from_grid_changes!
__global__ void k_finish_subgrid_heat(NodeCtx n, double* dtkn, double* wtnodes, double* dtk1) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n.ynum * n.xnum) return;
  const int32_t i = (int32_t)(t % n.ynum) + 1, j = (int32_t)(t / n.ynum) + 1;
  const float num = n.basic(i, j, 0, 1), den = n.basic(i, j, 4, 1);
  const double v = f2d(den != 0.f ? num / den : num);
  dtkn[t] = v;
  wtnodes[t] = f2d(den);
  dtk1[t] = dtk1[t] - v;
}

NodeCtx node_ctx(eb_ctx* c) { return NodeCtx{c->part, c->cs.ncells, c->ynum, c->xnum}; }
unsigned node_blocks(eb_ctx* c, int64_t n) { return (unsigned)((n + 255) / 256); }

int ensure_grids(eb_ctx* c, std::initializer_list<int> fields) {
  for (int f : fields) {
    int rc = ensure_grid_field(c, f);
    if (rc) return rc;
  }
  return EB_OK;
}
int ensure_markers(eb_ctx* c, std::initializer_list<int> fields) {
  for (int f : fields) {
    int rc = ensure_marker_field(c, f);
    if (rc) return rc;
  }
  return EB_OK;
}

}  // namespace

namespace {
int finish_denominators(eb_ctx* c, int base) {
  const int64_t n = (int64_t)c->ynum * (c->xnum + 1);
  EB_PROF(c, "k_finish_denoms");
  k_finish_denoms<<<node_blocks(c, n), 256, 0, c->stream>>>(node_ctx(c), base, c->gf[EB_G_WTNODES],
                                                            c->gf[EB_G_WTETAS], c->gf[EB_G_WTETAN],
                                                            c->gf[EB_G_WTNODES_VY]);
  EB_LAUNCHED(c);
  return EB_OK;
}
}  // namespace

int launch_denominators(eb_ctx* c) {
  if (c->M > 0) {
    int rc = run_cells(c, DenomSpec{});
    if (rc) return rc;
  } else {
    EB_CK(c, cudaMemsetAsync(c->part, 0, (size_t)kMaxSlots * c->cs.ncells * sizeof(float), c->stream));
  }
  return finish_denominators(c, 0);
}

int launch_scatter_stokes(eb_ctx* c) {
  int rc = ensure_markers(c, {EB_M_MATID, EB_M_RHO, EB_M_COHESION, EB_M_FRIC, EB_M_ETA_FLOW, EB_M_ETA, EB_M_SXY,
                              EB_M_SXX, EB_M_PFAILURE, EB_M_DILATATION, EB_M_MELTFRAC});
  if (rc) return rc;
  rc = ensure_grids(c, {EB_G_RHO1, EB_G_RHO0, EB_G_ETAS1, EB_G_ETAS0, EB_G_ETA_FLOW, EB_G_ETA_FLOW0, EB_G_MUS1,
                        EB_G_MUS0, EB_G_SXY1, EB_G_SXY0, EB_G_PLASTICS, EB_G_PLASTICS0, EB_G_COHESION,
                        EB_G_COHESION0, EB_G_FRIC_DEG, EB_G_FRIC_DEG0, EB_G_ETAN1, EB_G_ETAN0, EB_G_MUN1, EB_G_MUN0,
                        EB_G_SXX1, EB_G_SXX0, EB_G_PLASTICN, EB_G_PLASTICN0, EB_G_DILAT, EB_G_DILAT0, EB_G_MELTFRAC,
                        EB_G_MELTFRAC0, EB_G_RHO1_VY, EB_G_RHO0_VY, EB_G_HR1});
  if (rc) return rc;
  EB_CK(c, cudaMemsetAsync(c->dflag, 0, sizeof(int32_t), c->stream));
  if (c->M > 0) {
    rc = run_cells(c, StokesSpec{c->mats.mu, c->dflag});
    if (rc) return rc;
  } else {
    EB_CK(c, cudaMemsetAsync(c->part, 0, (size_t)kMaxSlots * c->cs.ncells * sizeof(float), c->stream));
  }
  StokesGrids G{};
  double** gf = c->gf;
  G.rho1 = gf[EB_G_RHO1]; G.rho0 = gf[EB_G_RHO0]; G.etas1 = gf[EB_G_ETAS1]; G.etas0 = gf[EB_G_ETAS0];
  G.eta_flow = gf[EB_G_ETA_FLOW]; G.eta_flow0 = gf[EB_G_ETA_FLOW0]; G.mus1 = gf[EB_G_MUS1]; G.mus0 = gf[EB_G_MUS0];
  G.sxy1 = gf[EB_G_SXY1]; G.sxy0 = gf[EB_G_SXY0]; G.plastics = gf[EB_G_PLASTICS]; G.plastics0 = gf[EB_G_PLASTICS0];
  G.coh = gf[EB_G_COHESION]; G.coh0 = gf[EB_G_COHESION0]; G.fric = gf[EB_G_FRIC_DEG]; G.fric0 = gf[EB_G_FRIC_DEG0];
  G.etan1 = gf[EB_G_ETAN1]; G.etan0 = gf[EB_G_ETAN0]; G.mun1 = gf[EB_G_MUN1]; G.mun0 = gf[EB_G_MUN0];
  G.sxx1 = gf[EB_G_SXX1]; G.sxx0 = gf[EB_G_SXX0]; G.plasticn = gf[EB_G_PLASTICN]; G.plasticn0 = gf[EB_G_PLASTICN0];
  G.dil = gf[EB_G_DILAT]; G.dil0 = gf[EB_G_DILAT0]; G.melt = gf[EB_G_MELTFRAC]; G.melt0 = gf[EB_G_MELTFRAC0];
  G.rho1_vy = gf[EB_G_RHO1_VY]; G.rho0_vy = gf[EB_G_RHO0_VY];
  G.wtnodes = gf[EB_G_WTNODES]; G.wtetas = gf[EB_G_WTETAS]; G.wtetan = gf[EB_G_WTETAN]; G.wtnodes_vy = gf[EB_G_WTNODES_VY];
  G.hr1 = gf[EB_G_HR1]; G.gy = c->g.gy;
  G.iuse_topo = (int)c->P.iuse_topo;
  G.y_sealevel = c->P.y_sealevel;
  auto mrho = [&](int64_t id) -> double {
    if (id < 1 || id > (int64_t)c->h_mat_rho.size()) return -1.0;
    return c->h_mat_rho[id - 1];
  };
  G.rho_air = c->P.iuse_topo == 1 ? mrho(c->P.matid_sticky_air_rho) : -1.0;
  G.rho_water = c->P.iuse_topo == 1 ? mrho(c->P.matid_sticky_water_rho) : -1.0;
  const int64_t n = (int64_t)c->ynum * (c->xnum + 1);
  EB_PROF(c, "k_finish_stokes");
  k_finish_stokes<<<node_blocks(c, n), 256, 0, c->stream>>>(node_ctx(c), G);
  EB_LAUNCHED(c);
  int32_t flag = 0;
  EB_CK(c, cudaMemcpyAsync(&flag, c->dflag, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  if (flag & 2) return eb_fail(c, EB_BAD_INPUT, "Shear modulus for marker material is zero");
  return EB_OK;
}

int launch_scatter_heat(eb_ctx* c, bool with_denominators) {
  int rc = ensure_markers(c, {EB_M_MATID, EB_M_TK, EB_M_KT, EB_M_RHOCP, EB_M_HA, EB_M_SERP_HR});
  if (rc) return rc;
  rc = ensure_grids(c, {EB_G_TK1, EB_G_TK0, EB_G_TK2, EB_G_KT1, EB_G_KT0, EB_G_RHOCP1, EB_G_RHOCP0, EB_G_HR1, EB_G_HR0,
                        EB_G_HA1, EB_G_HA0, EB_G_BTOPT, EB_G_BBOTTOMT, EB_G_BLEFTT, EB_G_BRIGHTT});
  if (rc) return rc;
  if (c->M > 0) {
    const int serp = (int)(c->P.iuse_serpentinization == 1);
    rc = with_denominators ? run_cells(c, HeatSpecT<true>{c->mats.hr, serp}) : run_cells(c, HeatSpec{c->mats.hr, serp});
    if (rc) return rc;
  } else {
    EB_CK(c, cudaMemsetAsync(c->part, 0, (size_t)kMaxSlots * c->cs.ncells * sizeof(float), c->stream));
  }
  if (with_denominators && (rc = finish_denominators(c, kDenBase))) return rc;  // k_finish_heat reads wtnodes
  double** gf = c->gf;
  HeatGrids G{gf[EB_G_TK1], gf[EB_G_TK0], gf[EB_G_KT1], gf[EB_G_KT0], gf[EB_G_RHOCP1], gf[EB_G_RHOCP0],
              gf[EB_G_HR1], gf[EB_G_HR0], gf[EB_G_HA1], gf[EB_G_HA0], gf[EB_G_TK2], gf[EB_G_WTNODES]};
  const int64_t n = (int64_t)c->ynum * c->xnum;
  EB_PROF(c, "k_finish_heat");
  k_finish_heat<<<node_blocks(c, n), 256, 0, c->stream>>>(node_ctx(c), G);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_thermal_bc_rows");
  k_thermal_bc_rows<<<(c->xnum + 255) / 256, 256, 0, c->stream>>>(gf[EB_G_TK1], gf[EB_G_BTOPT], gf[EB_G_BBOTTOMT], c->ynum, c->xnum);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_thermal_bc_cols");
  k_thermal_bc_cols<<<(c->ynum + 255) / 256, 256, 0, c->stream>>>(gf[EB_G_TK1], gf[EB_G_BLEFTT], gf[EB_G_BRIGHTT], c->ynum, c->xnum);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_scatter_viscosity(eb_ctx* c) {
  int rc = ensure_markers(c, {EB_M_ETA});
  if (rc) return rc;
  rc = ensure_grids(c, {EB_G_ETAS1, EB_G_ETAS0, EB_G_ETAN1, EB_G_ETAN0});
  if (rc) return rc;
  if (c->M > 0) {
    rc = run_cells(c, ViscSpec{});
    if (rc) return rc;
  } else {
    EB_CK(c, cudaMemsetAsync(c->part, 0, (size_t)kMaxSlots * c->cs.ncells * sizeof(float), c->stream));
  }
  double** gf = c->gf;
  EB_PROF(c, "k_finish_visc");
  k_finish_visc<<<node_blocks(c, (int64_t)c->ynum * c->xnum), 256, 0, c->stream>>>(
      node_ctx(c), gf[EB_G_ETAS1], gf[EB_G_ETAS0], gf[EB_G_ETAN1], gf[EB_G_ETAN0], gf[EB_G_WTETAS], gf[EB_G_WTETAN]);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_subgrid_stress(eb_ctx* c) {
  if (!(c->P.subgrid_diff_coef_stress > 0)) return EB_OK;  // StokesContinuitySolver.jl:371-373
  int rc = ensure_markers(c, {EB_M_MATID, EB_M_ETA, EB_M_SXY, EB_M_SXX});
  if (rc) return rc;
  rc = ensure_grids(c, {EB_G_SXY1, EB_G_SXX1, EB_G_DSXYN, EB_G_DSXXN, EB_G_DSXY, EB_G_DSXX});
  if (rc) return rc;
  double** gf = c->gf;
  if (c->M > 0) {
    const float* f[2];
    if ((rc = grid_f32(c, {EB_G_SXY1, EB_G_SXX1}, f))) return rc;
    SubgridStressSpec s{f[0], f[1], c->mats.mu, (float)c->P.timestep, (float)c->P.subgrid_diff_coef_stress};
    rc = run_cells(c, s);
    if (rc) return rc;
  } else {
    EB_CK(c, cudaMemsetAsync(c->part, 0, (size_t)kMaxSlots * c->cs.ncells * sizeof(float), c->stream));
  }
  EB_PROF(c, "k_finish_subgrid_stress");
  k_finish_subgrid_stress<<<node_blocks(c, (int64_t)c->ynum * c->xnum), 256, 0, c->stream>>>(
      node_ctx(c), gf[EB_G_DSXYN], gf[EB_G_DSXXN], gf[EB_G_WTETAS], gf[EB_G_WTETAN], gf[EB_G_DSXY], gf[EB_G_DSXX]);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_subgrid_heat(eb_ctx* c) {
  int rc = ensure_markers(c, {EB_M_TK, EB_M_SUBGRID_DT});
  if (rc) return rc;
  rc = ensure_grids(c, {EB_G_TK1, EB_G_KT1, EB_G_RHOCP1, EB_G_DTKN, EB_G_DTK1});
  if (rc) return rc;
  double** gf = c->gf;
  // markers outside the domain get a zero subgrid change (SubgridDiffusion.jl:119-121)
  EB_CK(c, cudaMemsetAsync(c->mf[EB_M_SUBGRID_DT], 0, c->M * sizeof(double), c->stream));
  if (c->M > 0) {
    const double its = 2.0 / (c->g.xstpavg * c->g.xstpavg) + 2.0 / (c->g.ystpavg * c->g.ystpavg);
    const float* f[3];
    if ((rc = grid_f32(c, {EB_G_TK1, EB_G_KT1, EB_G_RHOCP1}, f))) return rc;
    SubgridHeatSpec s{f[0], f[1], f[2], (float)c->P.timestep, (float)c->P.subgrid_diff_coef_temp, (float)its};
    rc = run_cells(c, s);
    if (rc) return rc;
  } else {
    EB_CK(c, cudaMemsetAsync(c->part, 0, (size_t)kMaxSlots * c->cs.ncells * sizeof(float), c->stream));
  }
  EB_PROF(c, "k_finish_subgrid_heat");
  k_finish_subgrid_heat<<<node_blocks(c, (int64_t)c->ynum * c->xnum), 256, 0, c->stream>>>(
      node_ctx(c), gf[EB_G_DTKN], gf[EB_G_WTNODES], gf[EB_G_DTK1]);
  EB_LAUNCHED(c);
  return EB_OK;
}
