// eb_ctx.cu -- context, memory and the C-ABI entry points of libebgpu.
//
// Every allocation happens in the set-up calls (eb_set_grid, eb_set_materials,
// eb_resize_markers, eb_*_upload) or on a field's first use; the per-step entry
// points only launch kernels on the context's stream and synchronise before
// returning, mirroring the synchronous Julia calls they replace.
#include <cstdio>
#include <cstring>
#include <algorithm>
#include "eb_internal.h"

int eb_fail(eb_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}
int eb_cuda(eb_ctx* c, cudaError_t e, const char* what) {
  return eb_fail(c, EB_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
}

// ---------------------------------------------------------------- shapes ---
enum Shape { SH_B, SH_P, SH_VX, SH_VY, SH_BCX, SH_BCY, SH_BCX1, SH_BCY1 };
static Shape grid_shape(int f) {
  if (f <= EB_G_PLASTIC_YIELD) return SH_B;
  if (f <= EB_G_PR1) return SH_P;
  if (f == EB_G_VX1 || f == EB_G_RX1 || f == EB_G_VX1_OLD) return SH_VX;
  if (f <= EB_G_WTNODES_VY || f == EB_G_RY1 || f == EB_G_VY1_OLD) return SH_VY;
  if (f == EB_G_RC1 || f == EB_G_EII_PLASTIC_PRESSURE || f == EB_G_EII || f == EB_G_PR1_OLD) return SH_P;
  if (f == EB_G_VXB || f == EB_G_VYB || (f >= EB_G_ETAVP_BUFFER && f <= EB_G_EII_PLASTIC_BASIC)) return SH_B;
  if (f == EB_G_RT1 || f == EB_G_REST) return SH_B;
  if (f == EB_G_BTOPT || f == EB_G_BBOTTOMT || f == EB_G_BTOPX || f == EB_G_BBOTTOMX) return SH_BCX;
  if (f == EB_G_BTOPY || f == EB_G_BBOTTOMY) return SH_BCX1;
  if (f == EB_G_BLEFTX || f == EB_G_BRIGHTX) return SH_BCY1;
  return SH_BCY;  // bleftt, brightt, blefty, brighty
}
size_t grid_field_count(const eb_ctx* c, int f) {
  const size_t X = c->xnum, Y = c->ynum;
  switch (grid_shape(f)) {
    case SH_B: return Y * X;
    case SH_P: return (Y - 1) * (X - 1);
    case SH_VX: return (Y + 1) * X;
    case SH_VY: return Y * (X + 1);
    case SH_BCX: return X * 2;
    case SH_BCX1: return (X + 1) * 2;
    case SH_BCY1: return (Y + 1) * 2;
    default: return Y * 2;
  }
}

int ensure_grid_field(eb_ctx* c, int f) {
  if (f < 0 || f >= EB_G_NFIELDS) return eb_fail(c, EB_BAD_INPUT, "grid field id out of range");
  if (!c->have_grid) return eb_fail(c, EB_NOT_READY, "eb_set_grid has not been called");
  if (!c->gf[f]) {
    size_t n = grid_field_count(c, f);
    EB_CK(c, cudaMalloc(&c->gf[f], n * sizeof(double)));
    EB_CK(c, cudaMemsetAsync(c->gf[f], 0, n * sizeof(double), c->stream));
  }
  return EB_OK;
}

// min and max of the uploaded marker_matid
__global__ void k_matid_range(const int16_t* __restrict__ m, int64_t n, int32_t* __restrict__ mm);

int launch_matid_range(eb_ctx* c, cudaStream_t s) {
  if (!c->d_minmax) EB_CK(c, cudaMalloc(&c->d_minmax, 2 * sizeof(int32_t)));
  const int32_t init[2] = {INT32_MAX, INT32_MIN};
  if (!c->h_pinned) EB_CK(c, cudaMallocHost(&c->h_pinned, 64));
  std::memcpy(c->h_pinned, init, sizeof(init));
  EB_CK(c, cudaMemcpyAsync(c->d_minmax, c->h_pinned, sizeof(init), cudaMemcpyHostToDevice, s));
  k_matid_range<<<(unsigned)std::min<int64_t>((c->M + 255) / 256, 4 * 152), 256, 0, s>>>(
      (const int16_t*)c->mf[EB_M_MATID], c->M, c->d_minmax);
  c->launches++;
  EB_CK(c, cudaGetLastError());
  EB_CK(c, cudaMemcpyAsync((char*)c->h_pinned + 8, c->d_minmax, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  return EB_OK;
}

// after the stream of launch_matid_range has reached it: accept or reject the range
int finish_matid_range(eb_ctx* c) {
  int32_t mm[2];
  std::memcpy(mm, (const char*)c->h_pinned + 8, sizeof(mm));
  if (mm[0] < 1 || (c->have_mats && mm[1] > c->mats.nmat)) return eb_fail(c, EB_BAD_INPUT, "marker_matid out of range");
  c->matid_min = mm[0];
  c->matid_max = mm[1];
  return EB_OK;
}

__global__ void k_matid_range(const int16_t* __restrict__ m, int64_t n, int32_t* __restrict__ mm) {
  int32_t lo = INT32_MAX, hi = INT32_MIN;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t v = m[k];
    lo = min(lo, v);
    hi = max(hi, v);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&mm[0], lo);
    atomicMax(&mm[1], hi);
  }
}

static size_t marker_elem_size(int f) {
  switch (f) {
    case EB_M_MATID: return 2;
    case EB_M_XN: case EB_M_YN: case EB_M_XN_VY: case EB_M_YN_VY: return 4;
    case EB_M_PFAILURE: case EB_M_DILATATION: return 4;
    case EB_M_INSIDE: return 1;
    default: return 8;
  }
}

int ensure_marker_field(eb_ctx* c, int f) {
  if (f < 0 || f >= EB_M_NFIELDS) return eb_fail(c, EB_BAD_INPUT, "marker field id out of range");
  if (f == EB_M_XN_VY || f == EB_M_YN_VY) return EB_OK;  // derived from xn/yn + flags
  if (c->M <= 0) return EB_OK;  // no markers: nothing to allocate, no marker kernel runs
  if (!c->mf[f]) {
    size_t bytes = (size_t)c->M * marker_elem_size(f);
    EB_CK(c, cudaMalloc(&c->mf[f], bytes));
    EB_CK(c, cudaMemsetAsync(c->mf[f], 0, bytes, c->stream));
  }
  return EB_OK;
}

DevMarkers dev_markers(eb_ctx* c) {
  DevMarkers d{};
  d.M = c->M;
  auto D = [&](int f) { return (double*)c->mf[f]; };
  d.x = D(EB_M_X); d.y = D(EB_M_Y);
  d.matid = (int16_t*)c->mf[EB_M_MATID];
  d.rho = D(EB_M_RHO); d.cohesion = D(EB_M_COHESION); d.fric = D(EB_M_FRIC); d.fric_ini = D(EB_M_FRIC_INI);
  d.eta = D(EB_M_ETA); d.eta_flow = D(EB_M_ETA_FLOW); d.preexp = D(EB_M_PREEXP);
  d.sxx = D(EB_M_SXX); d.sxy = D(EB_M_SXY); d.exx = D(EB_M_EXX); d.exy = D(EB_M_EXY);
  d.pr = D(EB_M_PR); d.sr_ratio = D(EB_M_SR_RATIO); d.gii = D(EB_M_GII);
  d.sp = D(EB_M_STRAIN_PLASTIC); d.srp = D(EB_M_STRAIN_RATE_PLASTIC);
  d.tk = D(EB_M_TK); d.kt = D(EB_M_KT); d.rhocp = D(EB_M_RHOCP); d.ha = D(EB_M_HA);
  d.melt = D(EB_M_MELTFRAC); d.melt_damage = D(EB_M_MELT_DAMAGE); d.serp_hr = D(EB_M_SERP_HR);
  d.pfailure = (float*)c->mf[EB_M_PFAILURE]; d.dilat = (float*)c->mf[EB_M_DILATATION];
  d.vx = D(EB_M_VX); d.vy = D(EB_M_VY); d.spin = D(EB_M_SPIN); d.subgrid_dt = D(EB_M_SUBGRID_DT);
  d.xn = (int32_t*)c->mf[EB_M_XN]; d.yn = (int32_t*)c->mf[EB_M_YN];
  d.inside = (int8_t*)c->mf[EB_M_INSIDE];
  d.por0 = D(EB_M_POROSITY_INITIAL); d.decay = D(EB_M_DECAY_DEPTH); d.burial = D(EB_M_MAX_BURIAL_DEPTH);
  d.fx = c->fx; d.fy = c->fy; d.mflags = c->mflags;
  return d;
}

// ------------------------------------------------------------ FP32 mirrors ---
namespace {
struct ConvJob {
  const double* src[8];
  float* dst[8];
  int64_t n[8];
  int count;
};
__global__ void k_grids_to_f32(ConvJob j) {
  const int g = blockIdx.y;
  if (g >= j.count) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < j.n[g]; i += (int64_t)gridDim.x * blockDim.x)
    j.dst[g][i] = d2f(j.src[g][i]);
}
}  // namespace

int grid_f32(eb_ctx* c, std::initializer_list<int> fields, const float** out) {
  ConvJob job{};
  int64_t nmax = 0;
  for (int f : fields) {
    if (job.count == 8) return eb_fail(c, EB_BAD_INPUT, "too many grids for one conversion");
    int rc = ensure_grid_field(c, f);
    if (rc) return rc;
    const int64_t n = (int64_t)grid_field_count(c, f);
    if (!c->gf32[f]) EB_CK(c, cudaMalloc(&c->gf32[f], n * sizeof(float)));
    job.src[job.count] = c->gf[f];
    job.dst[job.count] = c->gf32[f];
    job.n[job.count] = n;
    out[job.count] = c->gf32[f];
    nmax = n > nmax ? n : nmax;
    ++job.count;
  }
  const unsigned bx = (unsigned)((nmax + 255) / 256 < 1184 ? (nmax + 255) / 256 : 1184);
  EB_PROF(c, "k_grids_to_f32");
  k_grids_to_f32<<<dim3(bx, job.count), 256, 0, c->stream>>>(job);
  EB_LAUNCHED(c);
  return EB_OK;
}

// -------------------------------------------------------------- profiler ---
void prof_begin(eb_ctx* c, const char* name) {
  Profiler& p = c->prof;
  if (!p.on) return;
  if (p.used + 2 > p.pool.size()) {
    for (int k = 0; k < 64; ++k) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) return;
      p.pool.push_back(e);
    }
  }
  cudaEventRecord(p.pool[p.used], c->stream);
  p.pending.emplace_back(name, p.used);
  p.used += 2;
  p.open_name = name;
}

void prof_end(eb_ctx* c) {
  Profiler& p = c->prof;
  if (!p.on || !p.open_name) return;
  cudaEventRecord(p.pool[p.pending.back().second + 1], c->stream);
  p.open_name = nullptr;
}

void prof_resolve(eb_ctx* c) {
  Profiler& p = c->prof;
  for (auto& pr : p.pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.pool[pr.second], p.pool[pr.second + 1]) == cudaSuccess) {
      auto& a = p.acc[pr.first];
      a.first += ms;
      a.second += 1;
    }
  }
  p.pending.clear();
  p.used = 0;
}

extern "C" int eb_profile_enable(eb_ctx* c, int on) {
  if (!c) return EB_BAD_INPUT;
  cudaStreamSynchronize(c->stream);
  prof_resolve(c);
  c->prof.acc.clear();
  c->prof.on = on != 0;
  return EB_OK;
}

extern "C" int eb_profile_count(const eb_ctx* c) { return c ? (int)c->prof.acc.size() : 0; }

extern "C" int eb_profile_entry(const eb_ctx* c, int i, char* name, int name_len, double* total_ms, int64_t* launches) {
  if (!c || i < 0 || i >= (int)c->prof.acc.size() || !name || name_len < 1) return EB_BAD_INPUT;
  auto it = c->prof.acc.begin();
  std::advance(it, i);
  std::snprintf(name, (size_t)name_len, "%s", it->first.c_str());
  if (total_ms) *total_ms = it->second.first;
  if (launches) *launches = it->second.second;
  return EB_OK;
}

// ------------------------------------------------------------ lifecycle ---
extern "C" int eb_create(eb_ctx** out, int device) {
  if (!out) return EB_BAD_INPUT;
  *out = nullptr;
  eb_ctx* c = new eb_ctx();
  c->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return EB_CUDA_ERROR;
  }
  if (cudaMalloc(&c->dflag, sizeof(int32_t)) != cudaSuccess) {
    cudaStreamDestroy(c->stream);
    delete c;
    return EB_CUDA_ERROR;
  }
  cudaMemset(c->dflag, 0, sizeof(int32_t));
  *out = c;
  return EB_OK;
}

static void free_grid_tables(eb_ctx* c) {
  for (void* p : c->grid_allocs) cudaFree(p);
  c->grid_allocs.clear();
  for (int f = 0; f < EB_G_NFIELDS; ++f) {
    cudaFree(c->gf[f]);
    cudaFree(c->gf32[f]);
    c->gf[f] = nullptr;
    c->gf32[f] = nullptr;
  }
  cudaFree(c->cs.count); cudaFree(c->cs.start); cudaFree(c->cs.scan_tmp);
  cudaFree(c->part);
  c->cs.count = c->cs.start = c->cs.scan_tmp = nullptr;
  c->part = nullptr;
}

static void free_markers(eb_ctx* c) {
  for (int f = 0; f < EB_M_NFIELDS; ++f) { cudaFree(c->mf[f]); c->mf[f] = nullptr; }
  cudaFree(c->fx); cudaFree(c->fy); cudaFree(c->mflags); cudaFree(c->cs.perm); cudaFree(c->cs.perm_tmp);
  c->fx = c->fy = nullptr; c->mflags = nullptr; c->cs.perm = c->cs.perm_tmp = nullptr;
}

extern "C" int eb_destroy(eb_ctx* c) {
  if (!c) return EB_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  free_grid_tables(c);
  free_markers(c);
  stokes_free(c);
  heat_free(c);
  nn_free(c);
  for (void* p : c->mat_allocs) cudaFree(p);
  for (void* p : c->rock_allocs) cudaFree(p);
  for (void* p : c->sed_allocs) cudaFree(p);
  for (cudaEvent_t e : c->prof.pool) cudaEventDestroy(e);
  cudaFree(c->dflag);
  cudaFree(c->d_minmax);
  cudaFree(c->recycle_list);
  cudaFree(c->recycle_flags);
  if (c->h_pinned) cudaFreeHost(c->h_pinned);
  if (c->copy_in) cudaStreamDestroy(c->copy_in);
  if (c->copy_out) cudaStreamDestroy(c->copy_out);
  for (cudaEvent_t e : c->pipe_events) cudaEventDestroy(e);
  cudaStreamDestroy(c->stream);
  delete c;
  return EB_OK;
}

extern "C" const char* eb_last_error(const eb_ctx* c) { return c ? c->err.c_str() : "null context"; }
extern "C" void* eb_stream(eb_ctx* c) { return c ? (void*)c->stream : nullptr; }
extern "C" int64_t eb_launch_count(const eb_ctx* c) { return c ? c->launches : 0; }

template <class T>
static int upload_vec(eb_ctx* c, std::vector<void*>& owner, const std::vector<T>& h, const T** out) {
  T* d = nullptr;
  EB_CK(c, cudaMalloc(&d, std::max<size_t>(h.size(), 1) * sizeof(T)));
  owner.push_back(d);
  if (!h.empty()) EB_CK(c, cudaMemcpyAsync(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, c->stream));
  *out = d;
  return EB_OK;
}

static int64_t host_searchsortedlast(const double* v, int64_t n, double x) {
  return std::upper_bound(v, v + n, x) - v;  // count of elements <= x
}

static int build_axis(eb_ctx* c, const double* v, int32_t n, Axis* a) {
  std::vector<uint64_t> keys(n);
  for (int32_t i = 0; i < n; ++i) keys[i] = dkey(v[i]);
  const int32_t nb = std::max(4 * (n - 1), 1);
  const double v0 = v[0], v1 = v[n - 1];
  const double h = (v1 - v0) / nb;
  std::vector<int32_t> bucket(nb + 1);
  for (int32_t b = 0; b <= nb; ++b) bucket[b] = (int32_t)host_searchsortedlast(v, n, v0 + b * h);
  const uint64_t* dk;
  const int32_t* db;
  int rc = upload_vec(c, c->grid_allocs, keys, &dk);
  if (rc) return rc;
  rc = upload_vec(c, c->grid_allocs, bucket, &db);
  if (rc) return rc;
  a->key = dk; a->bucket = db; a->n = n; a->nb = nb;
  a->v0 = (float)v0;
  a->inv_h = (v1 > v0) ? (float)(nb / (v1 - v0)) : 0.f;
  return EB_OK;
}

extern "C" int eb_set_grid(eb_ctx* c, const eb_grid_desc* G) {
  if (!c || !G) return EB_BAD_INPUT;
  if (G->xnum < 3 || G->ynum < 3 || G->xnum > (1 << 20) || G->ynum > (1 << 20))
    return eb_fail(c, EB_BAD_INPUT, "grid needs 3 <= xnum, ynum <= 2^20");
  if ((G->xnum - 1) * (G->ynum - 1) >= (int64_t)INT32_MAX / 2)
    return eb_fail(c, EB_BAD_INPUT, "too many cells");
  const double* arrs[] = {G->gridx_b, G->gridy_b, G->xstp_b, G->ystp_b, G->gridx_vy, G->xstp_vy, G->gridy_vx, G->ystp_vx};
  for (const double* p : arrs) if (!p) return eb_fail(c, EB_BAD_INPUT, "null grid array");
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  free_grid_tables(c);
  const int32_t X = (int32_t)G->xnum, Y = (int32_t)G->ynum;
  for (int32_t j = 1; j < X; ++j)
    if (!(G->gridx_b[j] > G->gridx_b[j - 1]) || !(G->xstp_b[j - 1] > 0)) return eb_fail(c, EB_BAD_INPUT, "gridx_b must increase");
  for (int32_t i = 1; i < Y; ++i)
    if (!(G->gridy_b[i] > G->gridy_b[i - 1]) || !(G->ystp_b[i - 1] > 0)) return eb_fail(c, EB_BAD_INPUT, "gridy_b must increase");
  c->xnum = X; c->ynum = Y;
  DevGrid& g = c->g;
  g.xnum = X; g.ynum = Y;
  auto up = [&](const double* h, size_t n, const double** out) {
    return upload_vec(c, c->grid_allocs, std::vector<double>(h, h + n), out);
  };
  int rc;
  if ((rc = up(G->gridx_b, X, &g.gx)) || (rc = up(G->gridy_b, Y, &g.gy)) || (rc = up(G->xstp_b, X - 1, &g.sx)) ||
      (rc = up(G->ystp_b, Y - 1, &g.sy)))
    return rc;
  {
    std::vector<double> rsx(X - 1), rsy(Y - 1);
    for (int32_t j = 0; j < X - 1; ++j) rsx[j] = 1.0 / G->xstp_b[j];
    for (int32_t i = 0; i < Y - 1; ++i) rsy[i] = 1.0 / G->ystp_b[i];
    if ((rc = upload_vec(c, c->grid_allocs, rsx, &g.rsx)) || (rc = upload_vec(c, c->grid_allocs, rsy, &g.rsy))) return rc;
  }
  if ((rc = up(G->xstp_vy, X, &c->g_xstp_vy)) || (rc = up(G->ystp_vx, Y, &c->g_ystp_vx))) return rc;
  c->h_gx.assign(G->gridx_b, G->gridx_b + X);
  c->h_gy.assign(G->gridy_b, G->gridy_b + Y);
  stokes_free(c);  // the Stokes system and its multigrid hierarchy follow the grid
  heat_free(c);
  if ((rc = build_axis(c, G->gridx_b, X, &g.ax)) || (rc = build_axis(c, G->gridy_b, Y, &g.ay)) ||
      (rc = build_axis(c, G->gridx_vy, X + 1, &g.axvy)))
    return rc;
  std::vector<float> sxf(X - 1), rsxf(X - 1), vylo(X - 1), vyhi(X - 1), rsxvy(X);
  std::vector<float> syf(Y - 1), rsyf(Y - 1), vxlo(Y - 1), vxhi(Y - 1), rsyvx(Y);
  for (int32_t j = 0; j < X - 1; ++j) {
    sxf[j] = (float)G->xstp_b[j];
    rsxf[j] = (float)(1.0 / G->xstp_b[j]);
    vylo[j] = (float)(G->gridx_vy[j] - G->gridx_b[j]);
    vyhi[j] = (float)(G->gridx_vy[j + 1] - G->gridx_b[j]);
  }
  for (int32_t j = 0; j < X; ++j) rsxvy[j] = (float)(1.0 / G->xstp_vy[j]);
  for (int32_t i = 0; i < Y - 1; ++i) {
    syf[i] = (float)G->ystp_b[i];
    rsyf[i] = (float)(1.0 / G->ystp_b[i]);
    vxlo[i] = (float)(G->gridy_vx[i] - G->gridy_b[i]);
    vxhi[i] = (float)(G->gridy_vx[i + 1] - G->gridy_b[i]);
  }
  for (int32_t i = 0; i < Y; ++i) rsyvx[i] = (float)(1.0 / G->ystp_vx[i]);
  auto upf = [&](const std::vector<float>& h, const float** out) { return upload_vec(c, c->grid_allocs, h, out); };
  if ((rc = upf(sxf, &g.sxf)) || (rc = upf(rsxf, &g.rsxf)) || (rc = upf(vylo, &g.vyoff_lo)) || (rc = upf(vyhi, &g.vyoff_hi)) ||
      (rc = upf(rsxvy, &g.rsxvyf)) || (rc = upf(syf, &g.syf)) || (rc = upf(rsyf, &g.rsyf)) || (rc = upf(vxlo, &g.vxoff_lo)) ||
      (rc = upf(vxhi, &g.vxoff_hi)) || (rc = upf(rsyvx, &g.rsyvxf)))
    return rc;
  std::vector<float> colx(8 * (size_t)(X - 1), 0.f), rowy(8 * (size_t)(Y - 1), 0.f);
  for (int32_t j = 0; j < X - 1; ++j) {
    float* e = &colx[8 * (size_t)j];
    e[0] = sxf[j]; e[1] = rsxf[j]; e[2] = vylo[j]; e[3] = vyhi[j]; e[4] = rsxvy[j]; e[5] = rsxvy[j + 1];
  }
  for (int32_t i = 0; i < Y - 1; ++i) {
    float* e = &rowy[8 * (size_t)i];
    e[0] = syf[i]; e[1] = rsyf[i]; e[2] = vxlo[i]; e[3] = vxhi[i]; e[4] = rsyvx[i]; e[5] = rsyvx[i + 1];
  }
  const float *pcx = nullptr, *pry = nullptr;
  if ((rc = upf(colx, &pcx)) || (rc = upf(rowy, &pry))) return rc;
  g.colx = reinterpret_cast<const float4*>(pcx);  // cudaMalloc storage: 256-byte aligned
  g.rowy = reinterpret_cast<const float4*>(pry);
  // cell sort tables and partial-sum buffer
  CellSort& s = c->cs;
  s.ncells = (X - 1) * (Y - 1);
  s.scan_blocks = (s.ncells + 1 + 1023) / 1024;
  EB_CK(c, cudaMalloc(&s.count, (s.ncells + 1) * sizeof(int32_t)));
  EB_CK(c, cudaMalloc(&s.start, (s.ncells + 1) * sizeof(int32_t)));
  EB_CK(c, cudaMalloc(&s.scan_tmp, (s.scan_blocks + 1) * sizeof(int32_t)));
  EB_CK(c, cudaMalloc(&c->part, (size_t)kMaxSlots * s.ncells * sizeof(float)));
  g.kxmin = dkey(G->xmin); g.kxmax = dkey(G->xmax);
  g.kymin = dkey(G->ymin); g.kymax = dkey(G->ymax);
  g.xstpavg = G->xstpavg; g.ystpavg = G->ystpavg;
  c->have_grid = true;
  c->located = false;
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}

extern "C" int eb_set_materials(eb_ctx* c, const eb_material_desc* m) {
  if (!c || !m) return EB_BAD_INPUT;
  if (m->nmat < 1 || m->nmat > 32767) return eb_fail(c, EB_BAD_INPUT, "nmat out of range");
  if (!m->mat_mu || !m->mat_hr || !m->mat_flow_type || !m->mat_flow || !m->mat_plastic)
    return eb_fail(c, EB_BAD_INPUT, "null material array");
  int64_t option = m->mat_flow_type[0];
  for (int64_t i = 1; i < m->nmat; ++i) option = std::max<int64_t>(option, m->mat_flow_type[i]);
  if (!(option == -1 || option == 0 || option == 1 || option == 2 || option == 4 || option == 5))
    return eb_fail(c, EB_BAD_INPUT, "flow law type (largest mat_flow_type) must be -1, 0, 1, 2, 4 or 5");
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (void* p : c->mat_allocs) cudaFree(p);
  for (void* p : c->rock_allocs) cudaFree(p);
  for (void* p : c->sed_allocs) cudaFree(p);
  c->mat_allocs.clear();
  const int32_t n = (int32_t)m->nmat;
  DevMats& d = c->mats;
  d.nmat = n;
  std::vector<int32_t> ft(n);
  for (int32_t i = 0; i < n; ++i) ft[i] = (int32_t)m->mat_flow_type[i];
  d.option = (int32_t)option;
  std::vector<double> rho(n, -1.0);
  if (m->mat_rho) rho.assign(m->mat_rho, m->mat_rho + n);
  int rc;
  if ((rc = upload_vec(c, c->mat_allocs, std::vector<double>(m->mat_mu, m->mat_mu + n), &d.mu)) ||
      (rc = upload_vec(c, c->mat_allocs, std::vector<double>(m->mat_hr, m->mat_hr + n), &d.hr)) ||
      (rc = upload_vec(c, c->mat_allocs, std::vector<double>(m->mat_flow, m->mat_flow + (size_t)kFlowCols * n), &d.flow)) ||
      (rc = upload_vec(c, c->mat_allocs, std::vector<double>(m->mat_plastic, m->mat_plastic + 6 * (size_t)n), &d.plastic)) ||
      (rc = upload_vec(c, c->mat_allocs, rho, &d.rho)) || (rc = upload_vec(c, c->mat_allocs, ft, &d.flow_type)))
    return rc;
  c->h_mat_rho = rho;
  c->h_mat_plastic.assign(m->mat_plastic, m->mat_plastic + 6 * (size_t)n);
  c->have_mats = true;
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}

extern "C" int eb_set_params(eb_ctx* c, const eb_params* p) {
  if (!c || !p) return EB_BAD_INPUT;
  c->P = *p;
  c->have_params = true;
  return EB_OK;
}

extern "C" int eb_resize_markers(eb_ctx* c, int64_t M) {
  if (!c) return EB_BAD_INPUT;
  if (M < 0 || M >= (int64_t)INT32_MAX) return eb_fail(c, EB_BAD_INPUT, "marknum must be in [0, 2^31-1)");
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  free_markers(c);
  c->M = M;
  c->matid_min = 0;
  c->matid_max = 0;
  c->located = false;
  if (M == 0) return EB_OK;
  EB_CK(c, cudaMalloc(&c->fx, M * sizeof(float)));
  EB_CK(c, cudaMalloc(&c->fy, M * sizeof(float)));
  EB_CK(c, cudaMalloc(&c->mflags, M));
  EB_CK(c, cudaMalloc(&c->cs.perm, M * sizeof(int32_t)));
  EB_CK(c, cudaMalloc(&c->cs.perm_tmp, M * sizeof(int32_t)));
  EB_CK(c, cudaMemsetAsync(c->mflags, 0, M, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}

// ---------------------------------------------------------------- copies ---
extern "C" int eb_marker_upload(eb_ctx* c, int f, const void* host) {
  if (!c || !host) return EB_BAD_INPUT;
  if (f == EB_M_XN || f == EB_M_YN || f == EB_M_XN_VY || f == EB_M_YN_VY)
    return eb_fail(c, EB_BAD_INPUT, "cell indices are computed on the device (download only)");
  int rc = ensure_marker_field(c, f);
  if (rc) return rc;
  cudaSetDevice(c->device);
  if (c->M == 0) return EB_OK;
  if (f == EB_M_MATID) {
    // copied as is (Int16, as the reference stores it); its range is checked on the device
    c->matid_min = 0;  // unusable until the check passes
    c->matid_max = 0;
    EB_CK(c, cudaMemcpyAsync(c->mf[f], host, c->M * 2, cudaMemcpyHostToDevice, c->stream));
    if ((rc = launch_matid_range(c, c->stream))) return rc;
    EB_CK(c, cudaStreamSynchronize(c->stream));
    return finish_matid_range(c);
  }
  EB_CK(c, cudaMemcpyAsync(c->mf[f], host, c->M * marker_elem_size(f), cudaMemcpyHostToDevice, c->stream));
  if (f == EB_M_X || f == EB_M_Y) c->located = false;
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}

extern "C" int eb_marker_download(eb_ctx* c, int f, void* host) {
  if (!c || !host) return EB_BAD_INPUT;
  cudaSetDevice(c->device);
  if (c->M == 0) return EB_OK;
  if (f == EB_M_XN_VY || f == EB_M_YN_VY) {
    if (!c->mf[EB_M_XN]) return eb_fail(c, EB_NOT_READY, "markers have not been located");
    std::vector<int32_t> idx(c->M);
    EB_CK(c, cudaMemcpyAsync(idx.data(), c->mf[f == EB_M_XN_VY ? EB_M_XN : EB_M_YN], c->M * 4, cudaMemcpyDeviceToHost, c->stream));
    std::vector<uint8_t> fl(c->M);
    EB_CK(c, cudaMemcpyAsync(fl.data(), c->mflags, c->M, cudaMemcpyDeviceToHost, c->stream));
    EB_CK(c, cudaStreamSynchronize(c->stream));
    int32_t* out = (int32_t*)host;
    for (int64_t i = 0; i < c->M; ++i) out[i] = idx[i] + ((f == EB_M_XN_VY && (fl[i] & MF_VYRIGHT)) ? 1 : 0);
    return EB_OK;
  }
  int rc = ensure_marker_field(c, f);
  if (rc) return rc;
  if (f == EB_M_MATID) {
    EB_CK(c, cudaMemcpyAsync(host, c->mf[f], c->M * 2, cudaMemcpyDeviceToHost, c->stream));
    EB_CK(c, cudaStreamSynchronize(c->stream));
    return EB_OK;
  }
  EB_CK(c, cudaMemcpyAsync(host, c->mf[f], c->M * marker_elem_size(f), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}

extern "C" int eb_grid_upload(eb_ctx* c, int f, const double* host) {
  if (!c || !host) return EB_BAD_INPUT;
  int rc = ensure_grid_field(c, f);
  if (rc) return rc;
  cudaSetDevice(c->device);
  EB_CK(c, cudaMemcpyAsync(c->gf[f], host, grid_field_count(c, f) * 8, cudaMemcpyHostToDevice, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}

extern "C" int eb_grid_download(eb_ctx* c, int f, double* host) {
  if (!c || !host) return EB_BAD_INPUT;
  int rc = ensure_grid_field(c, f);
  if (rc) return rc;
  cudaSetDevice(c->device);
  EB_CK(c, cudaMemcpyAsync(host, c->gf[f], grid_field_count(c, f) * 8, cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}

extern "C" int eb_marker_device_ptr(eb_ctx* c, int f, void** d) {
  if (!c || !d) return EB_BAD_INPUT;
  int rc = ensure_marker_field(c, f);
  if (rc) return rc;
  *d = c->mf[f];
  return EB_OK;
}

extern "C" int eb_grid_device_ptr(eb_ctx* c, int f, double** d) {
  if (!c || !d) return EB_BAD_INPUT;
  int rc = ensure_grid_field(c, f);
  if (rc) return rc;
  *d = c->gf[f];
  return EB_OK;
}

// ------------------------------------------------------------ entry points --
static int ready(eb_ctx* c, bool need_mats, bool need_located) {
  if (!c) return EB_BAD_INPUT;
  if (!c->have_grid) return eb_fail(c, EB_NOT_READY, "eb_set_grid has not been called");
  if (!c->have_params) return eb_fail(c, EB_NOT_READY, "eb_set_params has not been called");
  if (need_mats && !c->have_mats) return eb_fail(c, EB_NOT_READY, "eb_set_materials has not been called");
  if (need_mats && c->M > 0 && c->matid_min < 1)
    return eb_fail(c, EB_NOT_READY, "marker_matid has not been uploaded (or held values below 1)");
  if (need_mats && c->matid_max > c->mats.nmat) return eb_fail(c, EB_BAD_INPUT, "marker_matid exceeds the material count");
  if (need_located && !c->located)
    return eb_fail(c, EB_NOT_READY, "eb_initialize_bilinear_interpolation must run after markers move");
  cudaSetDevice(c->device);
  return EB_OK;
}

static int finish(eb_ctx* c, int rc) {
  if (rc) return rc;
  EB_CK(c, cudaStreamSynchronize(c->stream));
  prof_resolve(c);
  return EB_OK;
}

extern "C" int eb_get_marker_inside_flags(eb_ctx* c) {
  int rc = ready(c, false, false);
  if (rc) return rc;
  if (c->M == 0) return EB_OK;
  if ((rc = ensure_marker_field(c, EB_M_X)) || (rc = ensure_marker_field(c, EB_M_Y)) ||
      (rc = ensure_marker_field(c, EB_M_INSIDE)))
    return rc;
  return finish(c, launch_inside_flags(c));
}

// cell location and the cell-sorted list: eb_initialize_bilinear_interpolation without its
// denominator pass
static int bilinear_locate(eb_ctx* c) {
  int rc;
  const int need[] = {EB_M_X, EB_M_Y, EB_M_INSIDE, EB_M_XN, EB_M_YN};
  for (int f : need) if ((rc = ensure_marker_field(c, f))) return rc;
  const int grids[] = {EB_G_WTNODES, EB_G_WTETAS, EB_G_WTETAN, EB_G_WTNODES_VY};
  for (int f : grids) if ((rc = ensure_grid_field(c, f))) return rc;
  if (c->M > 0 && (rc = launch_locate_and_sort(c))) return rc;
  c->located = true;
  return EB_OK;
}

extern "C" int eb_initialize_bilinear_interpolation(eb_ctx* c) {
  int rc = ready(c, false, false);
  if (rc) return rc;
  if ((rc = bilinear_locate(c))) return rc;
  return finish(c, launch_denominators(c));
}

int cycle_bilinear_setup(eb_ctx* c) {
  int rc = ready(c, false, false);
  if (rc) return rc;
  return finish(c, bilinear_locate(c));
}

int cycle_heat_and_denominators(eb_ctx* c) {
  int rc = ready(c, true, true);
  if (rc) return rc;
  return finish(c, launch_scatter_heat(c, true));
}

extern "C" int eb_initialize_bilinear_interpolation_and_heat_scatter(eb_ctx* c) {
  int rc = ready(c, true, false);
  if (rc) return rc;
  if ((rc = bilinear_locate(c))) return rc;
  return finish(c, launch_scatter_heat(c, true));
}

extern "C" int eb_interpolate_marker_stokes_parameters_to_grid(eb_ctx* c) {
  int rc = ready(c, true, true);
  if (rc) return rc;
  return finish(c, launch_scatter_stokes(c));
}
extern "C" int eb_interpolate_marker_heat_parameters_to_grid(eb_ctx* c) {
  int rc = ready(c, true, true);
  if (rc) return rc;
  return finish(c, launch_scatter_heat(c));
}
extern "C" int eb_backup_and_clear_viscosity_transport_arrays(eb_ctx* c) {
  int rc = ready(c, false, false);
  if (rc) return rc;
  if ((rc = ensure_grid_field(c, EB_G_ETAS1)) || (rc = ensure_grid_field(c, EB_G_ETAS0)) ||
      (rc = ensure_grid_field(c, EB_G_ETAN1)) || (rc = ensure_grid_field(c, EB_G_ETAN0)))
    return rc;
  const size_t nb = grid_field_count(c, EB_G_ETAS1) * 8, np = grid_field_count(c, EB_G_ETAN1) * 8;
  EB_CK(c, cudaMemcpyAsync(c->gf[EB_G_ETAS0], c->gf[EB_G_ETAS1], nb, cudaMemcpyDeviceToDevice, c->stream));
  EB_CK(c, cudaMemcpyAsync(c->gf[EB_G_ETAN0], c->gf[EB_G_ETAN1], np, cudaMemcpyDeviceToDevice, c->stream));
  EB_CK(c, cudaMemsetAsync(c->gf[EB_G_ETAS1], 0, nb, c->stream));
  EB_CK(c, cudaMemsetAsync(c->gf[EB_G_ETAN1], 0, np, c->stream));
  return finish(c, EB_OK);
}
extern "C" int eb_interpolate_viscosity_to_transport_arrays(eb_ctx* c) {
  int rc = ready(c, false, true);
  if (rc) return rc;
  return finish(c, launch_scatter_viscosity(c));
}
extern "C" int eb_interpolate_temperature_to_markers(eb_ctx* c) {
  int rc = ready(c, false, true);
  if (rc) return rc;
  return finish(c, launch_gather_temperature(c));
}
extern "C" int eb_update_marker_rheology(eb_ctx* c) {
  int rc = ready(c, true, false);
  if (rc) return rc;
  return finish(c, launch_rheology(c));
}
extern "C" int eb_update_marker_viscoplastic_viscosity(eb_ctx* c, int use_marker_plasticity) {
  int rc = ready(c, true, false);
  if (rc) return rc;
  return finish(c, launch_viscoplastic(c, use_marker_plasticity));
}
extern "C" int eb_update_marker_rheology_and_viscoplastic_viscosity(eb_ctx* c, int use_marker_plasticity) {
  int rc = ready(c, true, false);
  if (rc) return rc;
  return finish(c, launch_rheology_fused(c, use_marker_plasticity));
}
extern "C" int eb_update_plastic_yielding(eb_ctx* c) {
  int rc = ready(c, true, false);
  if (rc) return rc;
  return finish(c, launch_plastic_yielding(c));
}
extern "C" int eb_post_stokes_marker_gathers(eb_ctx* c) {
  int rc = ready(c, true, true);
  if (rc) return rc;
  return finish(c, launch_post_stokes_gathers(c));
}
extern "C" int eb_calc_marker_viscoplastic_viscosity(eb_ctx* c) {
  int rc = ready(c, false, true);
  if (rc) return rc;
  return finish(c, launch_marker_viscoplastic_viscosity(c));
}
extern "C" int eb_update_subgrid_stress(eb_ctx* c) {
  int rc = ready(c, true, true);
  if (rc) return rc;
  return finish(c, launch_subgrid_stress(c));
}
extern "C" int eb_apply_marker_stress_correction(eb_ctx* c) {
  int rc = ready(c, false, true);
  if (rc) return rc;
  return finish(c, launch_stress_correction(c));
}
extern "C" int eb_subgrid_heat_diffusion_update(eb_ctx* c) {
  int rc = ready(c, false, true);
  if (rc) return rc;
  return finish(c, launch_subgrid_heat(c));
}
extern "C" int eb_add_remaining_grid_change_to_marker_temperature(eb_ctx* c) {
  int rc = ready(c, false, true);
  if (rc) return rc;
  return finish(c, launch_add_remaining_dt(c));
}
extern "C" int eb_advect_markers_and_rotate_stress(eb_ctx* c) {
  int rc = ready(c, false, true);
  if (rc) return rc;
  rc = launch_advect(c);
  if (rc) return rc;
  c->located = false;  // markers moved: indices must be recomputed
  return finish(c, EB_OK);
}
extern "C" int eb_update_marker_strain(eb_ctx* c) {
  int rc = ready(c, false, false);
  if (rc) return rc;
  return finish(c, launch_update_strain(c));
}

extern "C" int eb_correct_advect_and_update_strain(eb_ctx* c) {
  int rc = ready(c, false, true);
  if (rc) return rc;
  return finish(c, launch_marker_tail(c));
}

// ------------------------------------------------------------ checkpoints ---
// File layout (little-endian host words): "EBGPUCK1", int64 version (1), xnum, ynum,
// marknum, entry count; then per entry int32 kind (0 marker field, 1 grid field), int32
// field id, int64 byte count and the bytes of the field in the layout eb_marker_download /
// eb_grid_download return.  Every field the context holds is written; derived state (the
// cell sort, FP32 mirrors, solver workspaces) is rebuilt by the next steps.
namespace {
constexpr char kCkMagic[8] = {'E', 'B', 'G', 'P', 'U', 'C', 'K', '1'};
}  // namespace

extern "C" int eb_checkpoint_write(eb_ctx* c, const char* path) {
  if (!c || !path) return EB_BAD_INPUT;
  if (!c->have_grid) return eb_fail(c, EB_NOT_READY, "eb_set_grid has not been called");
  cudaSetDevice(c->device);
  EB_CK(c, cudaStreamSynchronize(c->stream));
  std::FILE* fp = std::fopen(path, "wb");
  if (!fp) return eb_fail(c, EB_BAD_INPUT, std::string("cannot open ") + path + " for writing");
  std::vector<std::pair<int, int>> entries;
  for (int f = 0; f < EB_M_NFIELDS; ++f)
    if (c->mf[f] && c->M > 0) entries.push_back({0, f});
  for (int f = 0; f < EB_G_NFIELDS; ++f)
    if (c->gf[f]) entries.push_back({1, f});
  const int64_t head[5] = {1, c->xnum, c->ynum, c->M, (int64_t)entries.size()};
  bool ok = std::fwrite(kCkMagic, 1, 8, fp) == 8 && std::fwrite(head, sizeof(head), 1, fp) == 1;
  std::vector<char> buf;
  for (auto [kind, f] : entries) {
    if (!ok) break;
    const int64_t bytes = kind == 0 ? c->M * (int64_t)marker_elem_size(f) : (int64_t)(grid_field_count(c, f) * sizeof(double));
    buf.resize((size_t)bytes);
    cudaError_t e = cudaMemcpy(buf.data(), kind == 0 ? c->mf[f] : (void*)c->gf[f], (size_t)bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      std::fclose(fp);
      return eb_cuda(c, e, "checkpoint read-back");
    }
    const int32_t kf[2] = {kind, f};
    ok = std::fwrite(kf, sizeof(kf), 1, fp) == 1 && std::fwrite(&bytes, sizeof(bytes), 1, fp) == 1 &&
         std::fwrite(buf.data(), 1, (size_t)bytes, fp) == (size_t)bytes;
  }
  if (std::fclose(fp) != 0) ok = false;
  return ok ? EB_OK : eb_fail(c, EB_BAD_INPUT, std::string("writing ") + path + " failed");
}

extern "C" int eb_checkpoint_read(eb_ctx* c, const char* path) {
  if (!c || !path) return EB_BAD_INPUT;
  if (!c->have_grid) return eb_fail(c, EB_NOT_READY, "eb_set_grid has not been called");
  cudaSetDevice(c->device);
  std::FILE* fp = std::fopen(path, "rb");
  if (!fp) return eb_fail(c, EB_BAD_INPUT, std::string("cannot open ") + path);
  auto fail = [&](const std::string& m) { std::fclose(fp); return eb_fail(c, EB_BAD_INPUT, m); };
  char magic[8];
  int64_t head[5];
  if (std::fread(magic, 1, 8, fp) != 8 || std::memcmp(magic, kCkMagic, 8) != 0 || std::fread(head, sizeof(head), 1, fp) != 1)
    return fail(std::string(path) + " is not an eb checkpoint");
  if (head[0] != 1) return fail("unsupported checkpoint version");
  if (head[1] != c->xnum || head[2] != c->ynum) return fail("checkpoint grid differs from the context's grid");
  // Validate every entry header and size before the context changes: a truncated or
  // mismatched file then leaves the context as it was.
  if (std::fseek(fp, 0, SEEK_END) != 0) return fail("cannot read the checkpoint");
  const long fsize = std::ftell(fp);
  const long data0 = 8 + (long)sizeof(head);
  if (fsize < data0 || std::fseek(fp, data0, SEEK_SET) != 0) return fail("truncated checkpoint");
  const int64_t Mck = head[3];
  if (Mck < 0) return fail("bad checkpoint marker count");
  for (int64_t k = 0; k < head[4]; ++k) {
    int32_t kf[2];
    int64_t bytes;
    if (std::fread(kf, sizeof(kf), 1, fp) != 1 || std::fread(&bytes, sizeof(bytes), 1, fp) != 1)
      return fail("truncated checkpoint");
    const int kind = kf[0], f = kf[1];
    if (kind != 0 && kind != 1) return fail("bad checkpoint entry");
    if ((kind == 0 && (f < 0 || f >= EB_M_NFIELDS)) || (kind == 1 && (f < 0 || f >= EB_G_NFIELDS)))
      return fail("checkpoint field id out of range");
    const int64_t want = kind == 0 ? Mck * (int64_t)marker_elem_size(f) : (int64_t)(grid_field_count(c, f) * sizeof(double));
    if (bytes != want) return fail("checkpoint field size differs from the context's");
    const long pos = std::ftell(fp);
    if (pos < 0 || bytes > (int64_t)(fsize - pos) || std::fseek(fp, (long)bytes, SEEK_CUR) != 0)
      return fail("truncated checkpoint");
  }
  if (head[3] != c->M) {
    int rc = eb_resize_markers(c, head[3]);
    if (rc) { std::fclose(fp); return rc; }
  }
  if (std::fseek(fp, data0, SEEK_SET) != 0) return fail("cannot reread the checkpoint");
  std::vector<char> buf;
  bool matid = false;
  for (int64_t k = 0; k < head[4]; ++k) {
    int32_t kf[2];
    int64_t bytes;
    if (std::fread(kf, sizeof(kf), 1, fp) != 1 || std::fread(&bytes, sizeof(bytes), 1, fp) != 1)
      return fail("truncated checkpoint");
    const int kind = kf[0], f = kf[1];
    if (kind != 0 && kind != 1) return fail("bad checkpoint entry");
    if ((kind == 0 && (f < 0 || f >= EB_M_NFIELDS)) || (kind == 1 && (f < 0 || f >= EB_G_NFIELDS)))
      return fail("checkpoint field id out of range");
    const int64_t want = kind == 0 ? c->M * (int64_t)marker_elem_size(f) : (int64_t)(grid_field_count(c, f) * sizeof(double));
    if (bytes != want) return fail("checkpoint field size differs from the context's");
    buf.resize((size_t)bytes);
    if (std::fread(buf.data(), 1, (size_t)bytes, fp) != (size_t)bytes) return fail("truncated checkpoint");
    int rc = kind == 0 ? ensure_marker_field(c, f) : ensure_grid_field(c, f);
    if (rc) { std::fclose(fp); return rc; }
    cudaError_t e = cudaMemcpyAsync(kind == 0 ? c->mf[f] : (void*)c->gf[f], buf.data(), (size_t)bytes,
                                    cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) { std::fclose(fp); return eb_cuda(c, e, "checkpoint upload"); }
    if (kind == 0 && f == EB_M_MATID) matid = true;
  }
  std::fclose(fp);
  c->located = false;  // the cell sort is rebuilt by the next bilinear set-up
  if (matid && c->M > 0) {
    c->matid_min = 0;
    c->matid_max = 0;
    int rc = launch_matid_range(c, c->stream);
    if (rc) return rc;
    EB_CK(c, cudaStreamSynchronize(c->stream));
    return finish_matid_range(c);
  }
  return EB_OK;
}
