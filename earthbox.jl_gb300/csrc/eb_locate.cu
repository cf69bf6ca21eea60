// eb_locate.cu -- inside flags, upper-left cell indices and the cell-sorted marker list.
//
// Reference: GridFuncs.get_marker_inside_flags (src/utils/GridFuncs.jl:54-80) and
// MarkerGridMapping (src/interpolation/mapping/MarkerGridMapping.jl:78-265).
// The marker->cell list replaces the reference's serial marker-order scatter
// loops: markers are grouped by basic cell (column-major cell id, as Julia's
// Matrix layout) and ordered by marker index inside each cell, so every
// per-cell sum below is accumulated in the reference's marker order.
#include "eb_internal.h"

namespace {

constexpr int kBlock = 256;

// GridFuncs.check_in_domain_optimized: xmin <= x <= xmax && ymin <= y <= ymax,
// evaluated on order keys (integer compares; NaN is outside as in IEEE).
__global__ void k_inside_flags(const double* __restrict__ x, const double* __restrict__ y, int64_t M,
                               uint64_t kx0, uint64_t kx1, uint64_t ky0, uint64_t ky1,
                               int8_t* __restrict__ inside) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  uint64_t kx = dkey(x[m]), ky = dkey(y[m]);
  bool in = kx0 <= kx && kx <= kx1 && ky0 <= ky && ky <= ky1;
  // NaN keys sort above +inf (positive NaN) or below -inf (negative NaN): outside.
  inside[m] = in ? 1 : -1;
}

// Exact decision of fl(d / s) <= 0.5 and >= 0.5 for the exclusive quadrant
// tests (WeightFuncs.update_weight_exclusive!, WeightFuncs.jl:122-155).
// fl rounds to nearest even: fl(q) <= 0.5 <=> q <= 0.5 + 2^-54 and
// fl(q) >= 0.5 <=> q >= 0.5 - 2^-55.  With t = d - 0.5 s (exact near the
// boundary by Sterbenz's lemma) these become t <= s 2^-54 and t >= -s 2^-55.
// Kept out of line: only markers within 1e-7 of the half line reach it, and
// an inlined copy would be if-converted and run on every marker's FP64 pipe.
__device__ __noinline__ uint32_t exact_half_bits(double d, double s) {
  const double t = d - 0.5 * s;
  return (t <= s * 0x1p-54 ? 1u : 0u) | (t >= -s * 0x1p-55 ? 2u : 0u);
}
// bit 0: fl(d/s) <= 0.5, bit 1: fl(d/s) >= 0.5; the FP32 offset f errs by < 3e-8
__device__ __forceinline__ uint32_t half_bits(float f, double d,
                                              const double* __restrict__ s_tab, int32_t k) {
  if (fabsf(f - 0.5f) > 1e-7f) return f < 0.5f ? 1u : 2u;
  return exact_half_bits(d, __ldg(&s_tab[k]));
}

// rank[m]: the marker's slot within its cell's segment, from the histogram's own atomics (the
// order of the warps' groups within a cell is the atomics' order; k_sort_segments restores
// marker order).
__global__ void k_locate_count(DevMarkers mk, DevGrid g, int32_t* __restrict__ count,
                               int32_t* __restrict__ dflag, int32_t* __restrict__ rank) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int32_t key = -1;
  if (m < mk.M) {
    uint8_t fl = 0;
    if (mk.inside[m] == 1) {
      const double x = mk.x[m], y = mk.y[m];
      const int32_t ix = clamp_i(axis_search(g.ax, x), 1, g.xnum - 1);
      const int32_t iy = clamp_i(axis_search(g.ay, y), 1, g.ynum - 1);
      const int32_t ivy = clamp_i(axis_search(g.axvy, x), 1, g.xnum);
      fl = MF_INSIDE;
      if (ivy == ix + 1) fl |= MF_VYRIGHT;
      else if (ivy != ix) atomicOr(dflag, 1);  // vy grid is not staggered inside the basic cell
      const double dxd = x - __ldg(&g.gx[ix - 1]);
      const double dyd = y - __ldg(&g.gy[iy - 1]);
      // one FP64 multiply by the reciprocal spacing, rounded once to FP32:
      // |fx - fl64(dx)| <= 2^-25 fx + 2^-52, i.e. below 3e-8 on [0, 1]
      const float fx = d2f(dxd * __ldg(&g.rsx[ix - 1]));
      const float fy = d2f(dyd * __ldg(&g.rsy[iy - 1]));
      const uint32_t hx = half_bits(fx, dxd, g.sx, ix - 1);
      const uint32_t hy = half_bits(fy, dyd, g.sy, iy - 1);
      if (hx & 1u) fl |= MF_XLE;
      if (hx & 2u) fl |= MF_XGE;
      if (hy & 1u) fl |= MF_YLE;
      if (hy & 2u) fl |= MF_YGE;
      mk.xn[m] = ix;
      mk.yn[m] = iy;
      mk.fx[m] = fx;
      mk.fy[m] = fy;
      key = (ix - 1) * (g.ynum - 1) + (iy - 1);
    }
    mk.mflags[m] = fl;
  }
  // warp-aggregated histogram: one atomic per distinct cell per warp
  const unsigned peers = __match_any_sync(0xffffffffu, key);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  int32_t base = 0;
  if (key >= 0 && lane == leader) base = atomicAdd(&count[key], __popc(peers));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (key >= 0) rank[m] = base + __popc(peers & ((1u << lane) - 1u));
}

__global__ void k_place(const int32_t* __restrict__ xn, const int32_t* __restrict__ yn,
                        const uint8_t* __restrict__ mflags, int64_t M, int32_t ynum,
                        const int32_t* __restrict__ start, const int32_t* __restrict__ rank,
                        int32_t* __restrict__ perm_tmp) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M || !(mflags[m] & MF_INSIDE)) return;
  const int32_t key = (xn[m] - 1) * (ynum - 1) + (yn[m] - 1);
  perm_tmp[start[key] + rank[m]] = (int32_t)m;
}

// One warp per cell: order the cell's marker indices ascending.  Up to 32 markers: a bitonic
// network across the warp's lanes (15 compare-exchange stages; the padding INT32_MAX sorts last
// and every index is distinct); more: rank by count.
__global__ void k_sort_segments(const int32_t* __restrict__ start, int32_t ncells,
                                const int32_t* __restrict__ perm_tmp, int32_t* __restrict__ perm) {
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= ncells) return;
  const int32_t beg = start[warp], n = start[warp + 1] - beg;
  if (n <= 32) {
    int32_t v = lane < n ? perm_tmp[beg + lane] : INT32_MAX;
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
      for (int j = k >> 1; j > 0; j >>= 1) {
        const int32_t o = __shfl_xor_sync(0xffffffffu, v, j);
        const bool keep_min = ((lane & j) == 0) == ((lane & k) == 0);
        v = keep_min ? min(v, o) : max(v, o);
      }
    }
    if (lane < n) perm[beg + lane] = v;
  } else {
    for (int i = lane; i < n; i += 32) {
      const int32_t v = perm_tmp[beg + i];
      int r = 0;
      for (int j = 0; j < n; ++j) r += (perm_tmp[beg + j] < v);
      perm[beg + r] = v;
    }
  }
}

// ---- exclusive scan of int32 counts (three passes) ---------------------------
__device__ __forceinline__ int32_t block_exclusive_scan(int32_t v, int32_t* total) {
  __shared__ int32_t warp_sums[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) warp_sums[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    int32_t s = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int32_t t = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += t;
    }
    if (lane < nw) warp_sums[lane] = s;  // inclusive warp prefix
  }
  __syncthreads();
  const int32_t warp_off = wid ? warp_sums[wid - 1] : 0;
  *total = warp_sums[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_off + inc - v;
}

__global__ void k_scan_blocks(const int32_t* __restrict__ in, int32_t n, int32_t* __restrict__ out,
                              int32_t* __restrict__ bsum) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  int32_t total;
  const int32_t e = block_exclusive_scan(i < n ? in[i] : 0, &total);
  if (i < n) out[i] = e;
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

__global__ void k_scan_top(int32_t* __restrict__ bsum, int32_t nb) {
  __shared__ int32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int32_t base = 0; base < nb; base += blockDim.x) {
    const int32_t i = base + threadIdx.x;
    int32_t total;
    const int32_t e = block_exclusive_scan(i < nb ? bsum[i] : 0, &total);
    const int32_t c0 = carry;
    __syncthreads();
    if (i < nb) bsum[i] = e + c0;
    if (threadIdx.x == 0) carry = c0 + total;
    __syncthreads();
  }
}

__global__ void k_scan_add(int32_t* __restrict__ out, int32_t n, const int32_t* __restrict__ bsum) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += bsum[blockIdx.x];
}

}  // namespace

int launch_inside_flags(eb_ctx* c) {
  DevMarkers mk = dev_markers(c);
  const DevGrid& g = c->g;
  const unsigned blocks = (unsigned)((c->M + kBlock - 1) / kBlock);
  EB_PROF(c, "k_inside_flags");
  k_inside_flags<<<blocks, kBlock, 0, c->stream>>>(mk.x, mk.y, c->M, g.kxmin, g.kxmax, g.kymin, g.kymax, mk.inside);
  EB_LAUNCHED(c);
  return EB_OK;
}

int launch_locate_and_sort(eb_ctx* c) {
  DevMarkers mk = dev_markers(c);
  CellSort& s = c->cs;
  const int32_t n = s.ncells + 1;
  EB_CK(c, cudaMemsetAsync(s.count, 0, n * sizeof(int32_t), c->stream));
  EB_CK(c, cudaMemsetAsync(c->dflag, 0, sizeof(int32_t), c->stream));
  const unsigned mblocks = (unsigned)((c->M + kBlock - 1) / kBlock);
  EB_PROF(c, "k_locate_count");
  // s.perm holds each marker's slot in its cell until k_sort_segments writes the sorted list
  k_locate_count<<<mblocks, kBlock, 0, c->stream>>>(mk, c->g, s.count, c->dflag, s.perm);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_scan_blocks");
  k_scan_blocks<<<s.scan_blocks, 1024, 0, c->stream>>>(s.count, n, s.start, s.scan_tmp);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_scan_top");
  k_scan_top<<<1, 1024, 0, c->stream>>>(s.scan_tmp, s.scan_blocks);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_scan_add");
  k_scan_add<<<s.scan_blocks, 1024, 0, c->stream>>>(s.start, n, s.scan_tmp);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_place");
  k_place<<<mblocks, kBlock, 0, c->stream>>>(mk.xn, mk.yn, mk.mflags, c->M, c->ynum, s.start, s.perm, s.perm_tmp);
  EB_LAUNCHED(c);
  const unsigned sblocks = (unsigned)(((int64_t)s.ncells * 32 + kBlock - 1) / kBlock);
  EB_PROF(c, "k_sort_segments");
  k_sort_segments<<<sblocks, kBlock, 0, c->stream>>>(s.start, s.ncells, s.perm_tmp, s.perm);
  EB_LAUNCHED(c);
  int32_t flag = 0;
  EB_CK(c, cudaMemcpyAsync(&flag, c->dflag, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  if (flag) return eb_fail(c, EB_BAD_INPUT, "gridx_vy does not interleave gridx_b (marker_xn_vy not in {xn, xn+1})");
  return EB_OK;
}
