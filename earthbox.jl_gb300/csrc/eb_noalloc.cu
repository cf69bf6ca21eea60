// eb_noalloc.cu -- marker -> basic-grid bilinear average that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a host program whose device memory is
// owned by another allocator (a Julia or Python memory pool handing out
// buffers), a code path that runs while allocation is forbidden or would
// stall (a stream-ordered pipeline, a tight real-time loop), or a process
// whose device-memory budget is fixed up front.  This entry point serves them:
// the caller passes every input and output as device pointers, and the only
// working memory is a file-scope static __device__ array of kNoAllocScratchBytes
// (16 MiB).  Every GPU that loads the library holds that array until the
// process exits.
//
// It computes one inclusive bilinear average on the basic grid, the operation
// of BilinearNumerator (update_weight_inclusive!) + BilinearAverage
// (calc_bilinear_average_arithmetic!) for a field such as density or
// temperature, in FP64 and deterministically: markers are grouped by cell with
// their marker order kept, each cell folds its markers in that order, and nodes
// sum their four cells in a fixed order.
#include <cstdio>
#include <cstring>
#include <mutex>
#include "eb_internal.h"

namespace {

constexpr int64_t kMaxMarkers = 1 << 19;  // 524,288 markers
constexpr int64_t kMaxCells = 1 << 17;    // 131,072 basic cells
// Stable LSD radix sort of the markers by cell key: two passes of 9 bits cover keys
// 0..nc (nc <= 2^17; key nc marks a marker outside the grid), 2048-marker tiles.
constexpr int kDigitBits = 9;
constexpr int kDigits = 1 << kDigitBits;
constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kTile = kSortThreads * kSortItems;
constexpr int64_t kMaxTiles = (kMaxMarkers + kTile - 1) / kTile;
// Scratch layout (bytes): per marker key/perm_tmp/perm (3 x 4); per cell count/start (2 x 4,
// plus one) and 8 FP64 partial sums (8 x 8).  The radix sort's second key buffer and its
// per-tile digit counts live in the partial-sum region, which is written only after the sort.
constexpr size_t kMarkerBytes = (size_t)kMaxMarkers * 3 * 4;
constexpr size_t kCellBytes = (size_t)(kMaxCells + 1) * 2 * 4 + (size_t)kMaxCells * 8 * 8;
constexpr size_t kNoAllocScratchBytes = 16u << 20;
static_assert(kMarkerBytes + kCellBytes + 2048 <= kNoAllocScratchBytes, "scratch layout exceeds the array");
static_assert((size_t)kMaxMarkers * 4 + 256 + (size_t)kDigits * kMaxTiles * 4 + 4 <= (size_t)kMaxCells * 8 * 8,
              "radix buffers exceed the partial-sum region they share");

static __device__ __align__(256) unsigned char g_scratch[kNoAllocScratchBytes];

struct Scratch {
  int32_t *key, *perm_tmp, *perm, *count, *start;
  int32_t *key2, *hist;  // alias `part` (used only before the cell folds)
  double* part;
};

Scratch carve(unsigned char* base) {
  Scratch s;
  size_t o = 0;
  auto take = [&](size_t bytes) { unsigned char* p = base + o; o += (bytes + 255) & ~size_t(255); return p; };
  s.key = (int32_t*)take(kMaxMarkers * 4);
  s.perm_tmp = (int32_t*)take(kMaxMarkers * 4);
  s.perm = (int32_t*)take(kMaxMarkers * 4);
  s.count = (int32_t*)take((kMaxCells + 1) * 4);
  s.start = (int32_t*)take((kMaxCells + 1) * 4);
  s.part = (double*)take(kMaxCells * 8 * 8);
  s.key2 = (int32_t*)s.part;
  s.hist = (int32_t*)((unsigned char*)s.part + (((size_t)kMaxMarkers * 4 + 255) & ~size_t(255)));
  return s;
}

// searchsortedlast on a device coordinate array by order keys (exact).
__device__ int32_t search(const double* __restrict__ v, int32_t n, double x) {
  const uint64_t kx = dkey(x);
  int32_t lo = 0, hi = n + 1;
  while (hi - lo > 1) {
    const int32_t mid = (lo + hi) >> 1;
    if (kx < dkey(__ldg(&v[mid - 1]))) hi = mid; else lo = mid;
  }
  return lo;
}

// Cell key (column-major basic cell, 0-based; nc for a marker outside the grid) and the
// per-cell marker counts.
__global__ void k_na_locate(const double* __restrict__ x, const double* __restrict__ y, int32_t M,
                            const double* __restrict__ gx, int32_t xnum, const double* __restrict__ gy, int32_t ynum,
                            Scratch s) {
  const int32_t m = blockIdx.x * blockDim.x + threadIdx.x;
  const int32_t nc = (xnum - 1) * (ynum - 1);
  int32_t key = nc;
  if (m < M) {
    const double xm = x[m], ym = y[m];
    const uint64_t kx = dkey(xm), ky = dkey(ym);
    const bool in = dkey(gx[0]) <= kx && kx <= dkey(gx[xnum - 1]) && dkey(gy[0]) <= ky && ky <= dkey(gy[ynum - 1]);
    if (in) {
      const int32_t ix = clamp_i(search(gx, xnum, xm), 1, xnum - 1);
      const int32_t iy = clamp_i(search(gy, ynum, ym), 1, ynum - 1);
      key = (ix - 1) * (ynum - 1) + (iy - 1);
    }
    s.key[m] = key;
  }
  const unsigned peers = __match_any_sync(0xffffffffu, key);
  if (key < nc && (int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&s.count[key], __popc(peers));
}

// Exclusive scan of in[0..n) into out[0..n] by one block; in and out may be the same array
// (each thread reads in[i] before it writes out[i], and no other thread reads index i).
__global__ void k_na_scan(const int32_t* in, int32_t* out, int32_t n) {
  __shared__ int32_t warp_sums[32];
  __shared__ int32_t carry;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int32_t base = 0; base < n; base += blockDim.x) {
    const int32_t i = base + threadIdx.x;
    const int32_t v = i < n ? in[i] : 0;
    int32_t inc = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) warp_sums[wid] = inc;
    __syncthreads();
    if (wid == 0) {
      int32_t w = lane < nw ? warp_sums[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const int32_t t = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += t;
      }
      if (lane < nw) warp_sums[lane] = w;
    }
    __syncthreads();
    const int32_t c0 = carry;
    if (i < n) out[i] = c0 + (wid ? warp_sums[wid - 1] : 0) + inc - v;
    __syncthreads();
    if (threadIdx.x == 0) carry = c0 + warp_sums[nw - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = carry;
}

// Radix pass, step 1: digit counts of one tile of kTile markers, stored digit-major
// (hist[d * ntiles + tile]) so that one exclusive scan gives every (digit, tile) its offset.
__global__ void __launch_bounds__(kSortThreads) k_na_digit_count(const int32_t* __restrict__ key, int32_t M,
                                                                 int shift, int32_t ntiles,
                                                                 int32_t* __restrict__ hist) {
  __shared__ int32_t cnt[kDigits];
  for (int d = threadIdx.x; d < kDigits; d += kSortThreads) cnt[d] = 0;
  __syncthreads();
  const int32_t base = blockIdx.x * kTile;
  for (int r = 0; r < kSortItems; ++r) {
    const int32_t i = base + r * kSortThreads + threadIdx.x;
    if (i < M) atomicAdd(&cnt[(key[i] >> shift) & (kDigits - 1)], 1);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kDigits; d += kSortThreads) hist[(size_t)d * ntiles + blockIdx.x] = cnt[d];
}

// Radix pass, step 2: stable scatter.  A marker's place is its (digit, tile) offset plus the
// markers of its tile with the same digit that come before it: those of earlier rounds
// (cnt), of earlier warps of its round (wcnt) and of lower lanes of its warp.  Pass 0 reads
// the markers in index order (val_in == nullptr: the value is the index itself).
__global__ void __launch_bounds__(kSortThreads) k_na_digit_scatter(const int32_t* __restrict__ key_in,
                                                                   const int32_t* __restrict__ val_in, int32_t M,
                                                                   int shift, int32_t ntiles,
                                                                   const int32_t* __restrict__ hoff,
                                                                   int32_t* __restrict__ key_out,
                                                                   int32_t* __restrict__ val_out) {
  constexpr int kWarps = kSortThreads / 32;
  __shared__ int32_t cnt[kDigits];
  __shared__ int32_t wcnt[kWarps][kDigits];
  for (int d = threadIdx.x; d < kDigits; d += kSortThreads) {
    cnt[d] = 0;
    for (int w = 0; w < kWarps; ++w) wcnt[w][d] = 0;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int32_t base = blockIdx.x * kTile;
  for (int r = 0; r < kSortItems; ++r) {
    const int32_t i = base + r * kSortThreads + threadIdx.x;
    const bool valid = i < M;
    const int32_t k = valid ? key_in[i] : 0;
    const int d = valid ? (k >> shift) & (kDigits - 1) : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    if (valid && lane == __ffs(peers) - 1) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    if (valid) {
      int32_t pre = cnt[d];
      for (int w = 0; w < warp; ++w) pre += wcnt[w][d];
      const int32_t pos = hoff[(size_t)d * ntiles + blockIdx.x] + pre + __popc(peers & ((1u << lane) - 1u));
      if (key_out) key_out[pos] = k;
      val_out[pos] = val_in ? val_in[i] : i;
    }
    __syncthreads();
    for (int dd = threadIdx.x; dd < kDigits; dd += kSortThreads) {
      int32_t add = 0;
      for (int w = 0; w < kWarps; ++w) {
        add += wcnt[w][dd];
        wcnt[w][dd] = 0;
      }
      cnt[dd] += add;
    }
    __syncthreads();
  }
}

// One thread per cell: fold the cell's markers in marker order into the four corners'
// w*value and w sums.  Offsets and weights are the reference's FP64 expressions
// (MarkerGridMapping.jl:185-219, MarkerGridNodeWeights.jl:68-101): a marker within an FP32
// rounding of the far grid line still gives that node its (tiny) weight, as in the reference.
__global__ void k_na_cells(const double* __restrict__ x, const double* __restrict__ y,
                           const double* __restrict__ value, const double* __restrict__ gx,
                           const double* __restrict__ gy, int32_t ynum, int32_t nc, Scratch s) {
  const int32_t cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= nc) return;
  const int32_t ix = cell / (ynum - 1) + 1, iy = cell % (ynum - 1) + 1;
  const double x0 = gx[ix - 1], hx = gx[ix] - x0, y0 = gy[iy - 1], hy = gy[iy] - y0;
  double a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int32_t k = s.start[cell]; k < s.start[cell + 1]; ++k) {
    const int32_t m = s.perm[k];
    const double dx = (x[m] - x0) / hx, dy = (y[m] - y0) / hy;
    const double wul = (1.0 - dx) * (1.0 - dy), wll = (1.0 - dx) * dy, wur = dx * (1.0 - dy), wlr = dx * dy;
    const double v = value[m];
    a[0] += wul * v; a[1] += wll * v; a[2] += wur * v; a[3] += wlr * v;
    a[4] += wul; a[5] += wll; a[6] += wur; a[7] += wlr;
  }
  for (int k = 0; k < 8; ++k) s.part[(size_t)k * nc + cell] = a[k];
}

// Node (i, j) is UL of cell (i, j), LL of (i-1, j), UR of (i, j-1), LR of (i-1, j-1).
__global__ void k_na_finish(int32_t xnum, int32_t ynum, Scratch s, double* __restrict__ avg,
                            double* __restrict__ wsum) {
  const int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= xnum * ynum) return;
  const int32_t i = t % ynum + 1, j = t / ynum + 1, nc = (xnum - 1) * (ynum - 1);
  double n = 0.0, d = 0.0;
  auto add = [&](int32_t ci, int32_t cj, int corner) {
    const int32_t c = (cj - 1) * (ynum - 1) + (ci - 1);
    n += s.part[(size_t)corner * nc + c];
    d += s.part[(size_t)(4 + corner) * nc + c];
  };
  if (i > 1 && j > 1) add(i - 1, j - 1, 3);
  if (i < ynum && j > 1) add(i, j - 1, 2);
  if (i > 1 && j < xnum) add(i - 1, j, 1);
  if (i < ynum && j < xnum) add(i, j, 0);
  wsum[t] = d;
  if (d != 0.0) avg[t] = n / d;  // else: keep the caller's previous value (the backup)
}

std::mutex g_mutex;
void* g_scratch_ptr[256];  // per device, resolved once with that device current

}  // namespace

// Documented in include/ebgpu.h.
extern "C" int eb_marker_to_basic_grid_average_noalloc(const double* d_marker_x, const double* d_marker_y,
                                                       const double* d_marker_value, int64_t marknum,
                                                       const double* d_gridx_b, int64_t xnum,
                                                       const double* d_gridy_b, int64_t ynum, double* d_avg,
                                                       double* d_wsum, void* stream, char* errbuf,
                                                       size_t errlen) {
  auto fail = [&](int code, const char* msg) {
    if (errbuf && errlen) std::snprintf(errbuf, errlen, "%s", msg);
    return code;
  };
  if (marknum < 0 || marknum > kMaxMarkers) return fail(EB_BAD_INPUT, "marknum exceeds the no-alloc limit of 524288 markers");
  if (xnum < 2 || ynum < 2) return fail(EB_BAD_INPUT, "xnum and ynum must be >= 2");
  if ((xnum - 1) * (ynum - 1) > kMaxCells) return fail(EB_BAD_INPUT, "(xnum-1)*(ynum-1) exceeds the no-alloc limit of 131072 cells");
  if (!d_gridx_b || !d_gridy_b || !d_avg || !d_wsum || (marknum > 0 && (!d_marker_x || !d_marker_y || !d_marker_value)))
    return fail(EB_BAD_INPUT, "null device pointer");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return fail(EB_CUDA_ERROR, "cudaGetDevice failed");
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_ptr[dev]) {  // first call on this device: resolve the array's device address
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
      if (e != cudaSuccess) return fail(EB_CUDA_ERROR, cudaGetErrorString(e));
      g_scratch_ptr[dev] = p;
    }
    base = g_scratch_ptr[dev];
  }
  const Scratch s = carve((unsigned char*)base);
  cudaStream_t st = (cudaStream_t)stream;
  const int32_t M = (int32_t)marknum, X = (int32_t)xnum, Y = (int32_t)ynum, nc = (X - 1) * (Y - 1);
  // the array keeps the previous call's contents: clear the counters this call accumulates into
  if (cudaMemsetAsync(s.count, 0, (nc + 1) * sizeof(int32_t), st) != cudaSuccess)
    return fail(EB_CUDA_ERROR, "cudaMemsetAsync failed");
  const unsigned mb = (unsigned)((M + 255) / 256);
  if (M > 0) k_na_locate<<<mb, 256, 0, st>>>(d_marker_x, d_marker_y, M, d_gridx_b, X, d_gridy_b, Y, s);
  k_na_scan<<<1, 1024, 0, st>>>(s.count, s.start, nc);
  if (M > 0) {
    // markers ordered by (cell, marker index): two stable passes over the cell key
    const int32_t ntiles = (M + kTile - 1) / kTile;
    k_na_digit_count<<<ntiles, kSortThreads, 0, st>>>(s.key, M, 0, ntiles, s.hist);
    k_na_scan<<<1, 1024, 0, st>>>(s.hist, s.hist, kDigits * ntiles);
    k_na_digit_scatter<<<ntiles, kSortThreads, 0, st>>>(s.key, nullptr, M, 0, ntiles, s.hist, s.key2, s.perm_tmp);
    k_na_digit_count<<<ntiles, kSortThreads, 0, st>>>(s.key2, M, kDigitBits, ntiles, s.hist);
    k_na_scan<<<1, 1024, 0, st>>>(s.hist, s.hist, kDigits * ntiles);
    k_na_digit_scatter<<<ntiles, kSortThreads, 0, st>>>(s.key2, s.perm_tmp, M, kDigitBits, ntiles, s.hist, nullptr,
                                                        s.perm);
  }
  k_na_cells<<<(unsigned)((nc + 255) / 256), 256, 0, st>>>(d_marker_x, d_marker_y, d_marker_value, d_gridx_b,
                                                          d_gridy_b, Y, nc, s);
  k_na_finish<<<(unsigned)((X * Y + 255) / 256), 256, 0, st>>>(X, Y, s, d_avg, d_wsum);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(EB_CUDA_ERROR, cudaGetErrorString(e));
  return EB_OK;
}
