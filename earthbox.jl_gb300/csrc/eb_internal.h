// eb_internal.h -- context layout and kernel launchers shared by the .cu files.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <map>
#include <string>
#include <vector>
#include "../../include/ebgpu.h"
#include "eb_common.cuh"

// Device-side grid tables (all pointers are device pointers).
struct DevGrid {
  int32_t xnum, ynum;
  const double *gx, *gy, *sx, *sy;       // basic coordinates / spacings (FP64)
  const double *rsx, *rsy;                // 1/xstp_b, 1/ystp_b (FP64)
  Axis ax, ay, axvy;                      // exact search tables
  // FP32 per-basic-index tables, index j-1 for 1-based j
  const float *sxf, *rsxf;                // [xnum-1] xstp_b, 1/xstp_b
  const float *syf, *rsyf;                // [ynum-1]
  const float *vyoff_lo, *vyoff_hi;       // [xnum-1] gridx_vy[j]-gx[j], gridx_vy[j+1]-gx[j]
  const float *vxoff_lo, *vxoff_hi;       // [ynum-1] gridy_vx[i]-gy[i], gridy_vx[i+1]-gy[i]
  const float *rsxvyf;                    // [xnum]   1/xstp_vy
  const float *rsyvxf;                    // [ynum]   1/ystp_vx
  // the same FP32 tables packed per basic index j (1-based, entry 2(j-1) and 2(j-1)+1):
  // {xstp_b, 1/xstp_b, vyoff_lo, vyoff_hi}, {1/xstp_vy[j], 1/xstp_vy[j+1], 0, 0}; rowy likewise
  // for y with the vx-grid offsets: one cell's geometry in two 16-byte loads
  const float4 *colx, *rowy;
  uint64_t kxmin, kxmax, kymin, kymax;    // order keys of the domain limits
  double xstpavg, ystpavg;
};

// Pressure-grid bilinear gather (GridToMarker.jl:104-153, MarkerGridMapping.jl:311-350)
// on an FP32 mirror of the grid; (lx, ly) is the marker's offset from basic node (ix, iy).
// xp is ix-1 or ix (after the clamp), so its staggered spacing is one of the pair at ix-1.
__device__ __forceinline__ float gather_p(const float* __restrict__ pg, const DevGrid& g, int32_t ix, int32_t iy,
                                          float lx, float ly) {
  const float4 c0 = __ldg(&g.colx[2 * (ix - 1)]), c1 = __ldg(&g.colx[2 * (ix - 1) + 1]);
  const float4 r0 = __ldg(&g.rowy[2 * (iy - 1)]), r1 = __ldg(&g.rowy[2 * (iy - 1) + 1]);
  const float hx = c0.w, hy = r0.w;
  const int32_t xp = clamp_i((lx < hx) ? ix - 1 : ix, 1, g.xnum - 2);
  const int32_t yp = clamp_i((ly < hy) ? iy - 1 : iy, 1, g.ynum - 2);
  const bool xl = xp + 1 == ix, yl = yp + 1 == iy;
  const float ox = xl ? c0.z : hx;
  const float oy = yl ? r0.z : hy;
  return gather4f(pg, g.ynum - 1, yp, xp, (lx - ox) * (xl ? c1.x : c1.y), (ly - oy) * (yl ? r1.x : r1.y));
}

constexpr int kFlowCols = 17;  // columns of the reference's mat_flow table
struct DevMats {
  int32_t nmat;
  int32_t option;  // the model's flow law: the largest mat_flow_type (FlowViscosity.jl:21-44)
  const double *mu, *hr, *flow, *plastic, *rho;
  const int32_t* flow_type;
};

// Marker SoA pointers handed to kernels.
struct DevMarkers {
  int64_t M;
  double *x, *y;
  int16_t* matid;  // the reference's Vector{Int16}
  double *rho, *cohesion, *fric, *fric_ini, *eta, *eta_flow, *preexp;
  double *sxx, *sxy, *exx, *exy, *pr, *sr_ratio, *gii, *sp, *srp;
  double *tk, *kt, *rhocp, *ha, *melt, *melt_damage, *serp_hr;
  float *pfailure, *dilat;
  double *vx, *vy, *spin, *subgrid_dt;
  int32_t *xn, *yn;
  int8_t* inside;
  double *por0, *decay, *burial;  // sediment porosity (Athy's law) inputs
  float *fx, *fy;   // FP32 normalised distances from the upper-left basic node
  uint8_t* mflags;  // MF_* bits
};

struct CellSort {
  int32_t ncells;        // (ynum-1)*(xnum-1)
  int32_t* count;        // [ncells+1]
  int32_t* start;        // [ncells+1] exclusive scan of count
  int32_t* perm;         // [M] marker indices grouped by cell, ascending within a cell
  int32_t* perm_tmp;     // [M] placement buffer before the per-cell sort
  int32_t* scan_tmp;     // block sums for the scan
  int32_t scan_blocks;
};

// Per-kernel timing with CUDA events on the context's stream (off by default).
struct Profiler {
  bool on = false;
  std::vector<cudaEvent_t> pool;                 // reused event pairs
  size_t used = 0;                               // events handed out since the last resolve
  std::vector<std::pair<std::string, size_t>> pending;  // (kernel, index of its start event)
  std::map<std::string, std::pair<double, int64_t>> acc;  // kernel -> (total ms, launches)
  const char* open_name = nullptr;
};

struct StokesState;  // eb_stokes_solve.cu
struct HeatState;    // eb_heat.cu
namespace nn { struct Net; }  // eb_nn_net.cu: the learned preconditioner

struct eb_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  int64_t launches = 0;
  eb_params P{};
  bool have_params = false, have_grid = false, have_mats = false, located = false;
  // grid
  int32_t xnum = 0, ynum = 0;
  std::vector<void*> grid_allocs;  // coordinate tables
  DevGrid g{};
  const double *g_xstp_vy = nullptr, *g_ystp_vx = nullptr;  // FP64 staggered spacings (device)
  std::vector<double> h_gx, h_gy;                             // basic coordinates (host)
  double* gf[EB_G_NFIELDS] = {};
  float* gf32[EB_G_NFIELDS] = {};  // FP32 mirrors of grids read by the gathers
  // materials
  std::vector<void*> mat_allocs;
  DevMats mats{};
  std::vector<double> h_mat_rho, h_mat_plastic;  // host copies used by launch set-up
  // markers
  int64_t M = 0;
  int32_t matid_min = 0, matid_max = 0;  // range of the uploaded marker_matid (checked before use)
  int32_t* d_minmax = nullptr;            // device scratch of the range check
  void* h_pinned = nullptr;               // 64 pinned host bytes for small async read-backs
  // copy streams and events of eb_marker_cycle_host
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  std::vector<cudaEvent_t> pipe_events;
  void* mf[EB_M_NFIELDS] = {};
  float *fx = nullptr, *fy = nullptr;
  uint8_t* mflags = nullptr;
  // cell sort and per-cell partial sums
  CellSort cs{};
  float* part = nullptr;     // [kMaxSlots * ncells]
  int32_t* dflag = nullptr;  // device status word written by kernels (0 = ok)
  Profiler prof;
  // Stokes-continuity step
  eb_stokes_params SP{};
  bool have_stokes_params = false;
  StokesState* st = nullptr;
  // conductive heat step
  HeatState* ht = nullptr;
  nn::Net* net = nullptr;
  // rock-property tables and sediment porosity inputs (eb_step_boundary.cu)
  std::vector<void*> rock_allocs;
  int64_t rock_nmat = 0;
  const double *rock_rho = nullptr, *rock_cp = nullptr, *rock_kt = nullptr;  // [nmat x 3], [nmat], [nmat x 2]
  std::vector<void*> sed_allocs;
  int64_t sed_n = 0, sed_ntopo = 0;
  const int16_t* sed_ids = nullptr;
  const double *sed_tx = nullptr, *sed_ty = nullptr;
  double sed_kw = 0.0, sed_rhow = 0.0, sed_cpw = 0.0;
  bool have_sed = false;
  // the markers recycled by the last eb_recycle_markers (eb_recycle.cu)
  int64_t* recycle_list = nullptr;
  int8_t* recycle_flags = nullptr;
  size_t recycle_cap = 0;
  int64_t recycle_n = 0;
};

// Stokes system storage shared by the assembly (eb_stokes_build.cu) and the
// solver (eb_stokes_solve.cu).  Vectors are SoA blocks [vx | vy | p] of nc
// cells each, cell c = j*ny + i (0-based column j, row i), i.e. the
// reference's interleaved index 3c + {0, 1, 2}.
constexpr int kStencilSlots = 27;  // 11 x-Stokes, 11 y-Stokes, 5 continuity
struct StokesSystem {
  int32_t nx = 0, ny = 0;  // cells: xnum-1, ynum-1
  int64_t nc = 0;          // nx * ny
  double* coef = nullptr;  // [27][nc]
  double* rhs = nullptr;   // [3][nc]
  double* S = nullptr;     // [3][nc] solution
  double* S_old = nullptr; // [3][nc]
  double* resnl = nullptr; // [3][nc]
  double pscale = 0.0;
  double S_pscale = 0.0;   // pscale of the system S was solved for (its pressure unknowns are p / S_pscale)
  bool built = false;
};
StokesSystem* stokes_system(eb_ctx* c);            // allocated on first use for the current grid
void stokes_free(eb_ctx* c);
int launch_viscoelastic_terms(eb_ctx* c);
int launch_viscoelastic_rhs(eb_ctx* c);
int launch_build_stokes_system(eb_ctx* c, StokesSystem* s);
int launch_process_stokes_solution(eb_ctx* c, const StokesSystem* s);
int launch_grid_strain_rate(eb_ctx* c);
int launch_forecast_stress(eb_ctx* c);
int launch_stress_change(eb_ctx* c);
int launch_stag_to_basic(eb_ctx* c);
int launch_harmonic_etan(eb_ctx* c);
int launch_nodal_yield(eb_ctx* c, const eb_mobile_wall* w, double* d_partial, int* nblocks);
int launch_apply_nodal_yield(eb_ctx* c);
int export_stokes_coo(eb_ctx* c, const StokesSystem* s, int64_t* Li, int64_t* Lj, double* Lv, int64_t capacity,
                      int64_t* nnz);

void heat_free(eb_ctx* c);  // eb_heat.cu
// learned preconditioner (eb_nn_net.cu)
void nn_free(eb_ctx* c);
bool nn_trained(const eb_ctx* c);
int nn_correction(eb_ctx* c, const double* t, double s, double* z_add);  // z_add = s kappa NN(t / s)
// one learned-stage application: kept or not, its time, and the fraction of the squared
// preconditioner residual it removed
void nn_count(eb_ctx* c, bool accepted, double seconds, double removed);
int launch_matid_range(eb_ctx* c, cudaStream_t s);  // eb_ctx.cu: marker_matid range check
int finish_matid_range(eb_ctx* c);

constexpr int kMaxSlots = 48;

// error helpers
int eb_fail(eb_ctx* c, int code, const std::string& msg);
int eb_cuda(eb_ctx* c, cudaError_t e, const char* what);
#define EB_CK(ctx, call)                                  \
  do {                                                    \
    cudaError_t _e = (call);                              \
    if (_e != cudaSuccess) return eb_cuda(ctx, _e, #call); \
  } while (0)
// Every kernel launch is bracketed by EB_PROF(ctx, "name") before and EB_LAUNCHED(ctx) after.
void prof_begin(eb_ctx* c, const char* name);
void prof_end(eb_ctx* c);
void prof_resolve(eb_ctx* c);
#define EB_PROF(ctx, name) prof_begin(ctx, name)
#define EB_LAUNCHED(ctx)                                                    \
  do {                                                                      \
    (ctx)->launches++;                                                      \
    prof_end(ctx);                                                          \
    cudaError_t _e = cudaGetLastError();                                    \
    if (_e != cudaSuccess) return eb_cuda(ctx, _e, "kernel launch");        \
  } while (0)

// field helpers (eb_ctx.cu)
int ensure_grid_field(eb_ctx* c, int f);
int ensure_marker_field(eb_ctx* c, int f);
DevMarkers dev_markers(eb_ctx* c);
size_t grid_field_count(const eb_ctx* c, int f);

// FP32 mirrors: convert the listed grid fields (up to 8) in one launch and
// return their device pointers in `out` (same order).
int grid_f32(eb_ctx* c, std::initializer_list<int> fields, const float** out);

// launchers
int launch_inside_flags(eb_ctx* c);
int launch_locate_and_sort(eb_ctx* c);
int launch_denominators(eb_ctx* c);
int launch_scatter_stokes(eb_ctx* c);
// with_denominators: the same fold also sums the weight denominators (wtnodes, wtetas, wtetan,
// wtnodes_vy) that launch_denominators would (bit-identical), for a heat scatter that directly
// follows the bilinear set-up
int launch_scatter_heat(eb_ctx* c, bool with_denominators = false);
int launch_scatter_viscosity(eb_ctx* c);
int launch_subgrid_stress(eb_ctx* c);
int launch_subgrid_heat(eb_ctx* c);
int launch_gather_temperature(eb_ctx* c);
int launch_post_stokes_gathers(eb_ctx* c);
int launch_marker_viscoplastic_viscosity(eb_ctx* c);
int launch_stress_correction(eb_ctx* c);
int launch_add_remaining_dt(eb_ctx* c);
int launch_advect(eb_ctx* c);
int launch_update_strain(eb_ctx* c);
// stress correction, remaining temperature change, advection + rotation and the strain
// update in one marker pass (the four steps in that order; eb_advect.cu)
int launch_marker_tail(eb_ctx* c);
// The bilinear set-up without its denominator pass and the heat scatter that sums them; run
// back to back they equal eb_initialize_bilinear_interpolation followed by
// eb_interpolate_marker_heat_parameters_to_grid (eb_ctx.cu; the host pipeline runs them as two
// steps so the heat fields' upload can overlap the locate and sort).
int cycle_bilinear_setup(eb_ctx* c);
int cycle_heat_and_denominators(eb_ctx* c);
int launch_rheology(eb_ctx* c);
int launch_viscoplastic(eb_ctx* c, int use_marker_plasticity);
int launch_rheology_fused(eb_ctx* c, int use_marker_plasticity);
int launch_plastic_yielding(eb_ctx* c);
