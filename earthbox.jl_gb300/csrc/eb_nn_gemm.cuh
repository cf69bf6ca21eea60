// eb_nn_gemm.cuh -- BF16 x BF16 -> FP32 GEMM on the fifth-generation tensor cores (tcgen05).
//
// D[M x N] = A[M x K] . B[N x K]^T, both operands K-major (K contiguous).  One CTA of 128
// threads owns a 128-row tile of D and BN (16..256, multiple of 16) columns:
//   * every thread stages 16-byte chunks of the next K-chunk (64 BF16 = 128 B per row) into
//     shared memory with cp.async, in the 128-byte-swizzled K-major layout the tensor core
//     reads (chunk c of row r stored at chunk position c ^ (r mod 8), 8-row atoms of
//     1024 B, atoms 1024-B aligned);
//   * one thread issues four tcgen05.mma (K = 16 each) per K-chunk into an FP32 accumulator
//     in tensor memory and commits them to an mbarrier; two shared-memory stages let the
//     loads of chunk k+1 overlap the MMAs of chunk k;
//   * the epilogue reads the accumulator with tcgen05.ld (warp w owns lanes 32w..32w+31,
//     i.e. rows 32w..32w+31 of the tile) and hands each thread 16 consecutive columns of
//     its row.
// Every mbarrier wait is bounded: after kSpinLimit polls the CTA records an error in
// *err, stops issuing work and still frees its tensor memory.
//
// The A operand comes from a loader functor (plain matrix or implicit 3x3 convolution),
// so the same kernel serves the forward convolution, the input gradient and the weight
// gradient of the learned preconditioner (eb_nn.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace nn {

constexpr int kGemmThreads = 128;
constexpr int kTileM = 128;
constexpr int kChunkK = 64;                       // BF16 elements per row per stage (128 B)
constexpr uint32_t kSpinLimit = 1u << 24;

// ---- PTX wrappers ---------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, bool valid) {
  const int n = valid ? 16 : 0;  // 0: the 16 bytes are zero-filled and nothing is read
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}
// true when the phase of parity `parity` has completed, within kSpinLimit polls
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (uint32_t it = 0; it < kSpinLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(dst_smem), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar) : "memory");
}
// 16 consecutive FP32 columns of this thread's accumulator row
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

// ---- descriptors ------------------------------------------------------------------
// Shared-memory matrix descriptor (tcgen05): start address >> 4 in bits 0-13, leading-
// dimension byte offset >> 4 in 16-29 (unused for K-major 128-B swizzle), stride byte
// offset >> 4 in 32-45 (1024 B between 8-row atoms), the fixed value 1 in bits 46-48,
// base offset 0 (atoms 1024-B aligned), swizzle mode 2 (128 B) in bits 61-63.
__host__ __device__ constexpr uint64_t smem_desc_sw128(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}
// Instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B BF16 (bits 7-9 and
// 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(uint32_t m, uint32_t n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}
// byte offset of 16-byte chunk c of row r inside a swizzled tile
__host__ __device__ constexpr uint32_t sw128_offset(uint32_t r, uint32_t c) { return r * 128u + ((c ^ (r & 7u)) << 4); }

__host__ __device__ constexpr uint32_t tmem_cols(uint32_t bn) {
  return bn <= 32 ? 32u : (bn <= 64 ? 64u : (bn <= 128 ? 128u : 256u));
}
__host__ __device__ constexpr size_t gemm_smem_bytes(int bn) {
  return 1024 + 2 * (size_t)(kTileM + bn) * 128 + 64;
}

// ---- operand loaders ----------------------------------------------------------------
// A thread stages the same 16-byte chunk column (tid mod 8) of fixed tile rows in every
// K-chunk, so each loader splits the address into a per-row part (computed once per CTA)
// and a per-column part (once per K-chunk).
struct RowAt {
  int64_t pix;  // row index (matrix) or pixel index (convolution)
  int32_t y, x;
  bool ok;
};
struct ColAt {
  int64_t k;    // column (matrix) or channel (convolution)
  int32_t off;  // pixel offset of the tap (convolution)
  int32_t dy, dx;
  bool ok;
};
// Plain K-major matrix: row r at base + r * ld (elements), rows >= rows_valid and
// columns >= k_valid read as zero.
struct MatLoader {
  const uint16_t* base;
  int64_t ld;
  int64_t rows_valid;
  int64_t k_valid;
  __device__ __forceinline__ RowAt row(int64_t r) const { return RowAt{r, 0, 0, r < rows_valid}; }
  __device__ __forceinline__ ColAt col(int64_t k) const { return ColAt{k, 0, 0, 0, k < k_valid}; }
  __device__ __forceinline__ const void* at(const RowAt& R, const ColAt& K, bool& ok) const {
    ok = R.ok && K.ok;
    return ok ? (const void*)(base + R.pix * ld + K.k) : (const void*)base;
  }
};
// Implicit 3x3 (or 1x1) convolution, NHWC input [B][H][W][C] with C a multiple of 8:
// row r = output pixel (b, y, x); column k = tap * C + c, tap = 3 (dy + 1) + (dx + 1);
// taps outside the image read zero.  With flip, tap t reads offset -d(t) (input gradient).
struct ConvLoader {
  const uint16_t* x;
  int32_t B, H, W, C, taps;  // taps 9 or 1
  int32_t flip;
  __device__ __forceinline__ RowAt row(int64_t r) const {
    const int64_t P = (int64_t)B * H * W;
    if (r >= P) return RowAt{0, 0, 0, false};
    const int32_t rem = (int32_t)(r % ((int64_t)H * W));
    return RowAt{r, rem / W, rem % W, true};
  }
  __device__ __forceinline__ ColAt col(int64_t k) const {
    if (k >= (int64_t)taps * C) return ColAt{0, 0, 0, 0, false};
    const int32_t tap = (int32_t)(k / C), c = (int32_t)(k - (int64_t)tap * C);
    int32_t dy = 0, dx = 0;
    if (taps == 9) { dy = tap / 3 - 1; dx = tap % 3 - 1; if (flip) { dy = -dy; dx = -dx; } }
    return ColAt{c, dy * W + dx, dy, dx, true};
  }
  __device__ __forceinline__ const void* at(const RowAt& R, const ColAt& K, bool& ok) const {
    ok = R.ok && K.ok && R.y + K.dy >= 0 && R.y + K.dy < H && R.x + K.dx >= 0 && R.x + K.dx < W;
    return ok ? (const void*)(x + (R.pix + K.off) * C + K.k) : (const void*)x;
  }
};

// Epilogue: out[row][col] (row < M, col < N) from the FP32 accumulator.
//   mode 0: FP32 store           out32[row * ldo + col0 + col]
//   mode 1: BF16, + bias, ReLU   out16[row * ldo + col0 + col]
//   mode 2: BF16, + bias         (no activation)
struct Epilogue {
  float* out32;
  uint16_t* out16;
  const float* bias;  // [N] or null
  int64_t ldo;
  int32_t col0;
  int32_t mode;
};

__device__ __forceinline__ uint16_t f32_to_bf16_rne(float f) { return __bfloat16_as_ushort(__float2bfloat16_rn(f)); }

// grid: (ceil(M / 128), ceil(N / BN), splits); split s handles K chunks [s*kc_per, (s+1)*kc_per)
// and, with splits > 1, writes its partial sums to out32 + s * M * ldo (mode 0 only).
template <class ALoad>
__global__ void __launch_bounds__(kGemmThreads) k_gemm_bf16(ALoad A, MatLoader Bm, int64_t M, int32_t N, int32_t BN,
                                                             int64_t K, int32_t kc_per, Epilogue ep,
                                                             int32_t* __restrict__ err) {
  extern __shared__ __align__(16) uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  uint8_t* const gbase = smem_raw + (base - raw);
  const uint32_t a_bytes = kTileM * 128, b_bytes = (uint32_t)BN * 128;
  const uint32_t stage_bytes = a_bytes + b_bytes;
  const uint32_t bar0 = base + 2 * stage_bytes;  // two mbarriers, then the TMEM address word
  const uint32_t tslot = bar0 + 16;
  volatile uint32_t* tslot_ptr = reinterpret_cast<volatile uint32_t*>(gbase + 2 * stage_bytes + 16);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t m0 = (int64_t)blockIdx.x * kTileM;
  const int64_t n0 = (int64_t)blockIdx.y * BN;
  const int64_t nchunks_total = (K + kChunkK - 1) / kChunkK;
  const int64_t kc0 = (int64_t)blockIdx.z * kc_per;
  const int64_t kc1 = min(nchunks_total, kc0 + kc_per);
  const int32_t nk = (int32_t)max((int64_t)0, kc1 - kc0);
  const uint32_t ncols = tmem_cols((uint32_t)BN);

  if (warp == 0) {
    tmem_alloc(tslot, ncols);
    tmem_relinquish();
  }
  if (tid == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar0 + 8, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot_ptr;

  // this thread's chunk column and rows: tile rows tid/8 + 16 i
  const int cc = tid & 7, r0 = tid >> 3;
  RowAt arow[kTileM / 16];
#pragma unroll
  for (int i = 0; i < kTileM / 16; ++i) arow[i] = A.row(m0 + r0 + 16 * i);
  auto load_stage = [&](int32_t j, int buf) {
    const int64_t k = (kc0 + j) * kChunkK + 8 * cc;
    const uint32_t sa = base + (uint32_t)buf * stage_bytes, sb = sa + a_bytes;
    const ColAt ka = A.col(k), kb = Bm.col(k);
#pragma unroll
    for (int i = 0; i < kTileM / 16; ++i) {
      bool ok;
      const void* src = A.at(arow[i], ka, ok);
      cp_async16(sa + sw128_offset(r0 + 16 * i, cc), src, ok);
    }
    for (int r = r0; r < BN; r += 16) {
      bool ok;
      const void* src = Bm.at(Bm.row(n0 + r), kb, ok);
      cp_async16(sb + sw128_offset(r, cc), src, ok);
    }
    cp_async_commit();
  };

  bool failed = false;
  const uint32_t idesc = idesc_bf16_f32(kTileM, (uint32_t)BN);
  if (nk > 0) load_stage(0, 0);
  for (int32_t j = 0; j < nk; ++j) {
    const int buf = j & 1;
    bool f = false;
    if (j + 1 < nk) {
      // buffer (j+1)&1 was last read by the MMAs of chunk j-1
      if (j >= 1 && !mbar_wait(bar0 + 8 * ((j - 1) & 1), ((j - 1) >> 1) & 1)) f = true;
      if (!f) load_stage(j + 1, (j + 1) & 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    fence_async_smem();
    if (__syncthreads_or(f)) {  // block-uniform: every thread leaves the loop together
      failed = true;
      break;
    }
    if (tid == 0) {
      tc_fence_after();
      const uint32_t sa = base + (uint32_t)buf * stage_bytes, sb = sa + a_bytes;
#pragma unroll
      for (int kk = 0; kk < kChunkK / 16; ++kk)
        mma_bf16(tmem, smem_desc_sw128(sa + 32u * kk), smem_desc_sw128(sb + 32u * kk), idesc,
                 (j > 0 || kk > 0) ? 1u : 0u);
      mma_commit(bar0 + 8 * buf);
    }
  }
  cp_async_wait<0>();
  // the last commit arrives once every MMA issued before it has completed
  if (!failed && nk > 0 && !mbar_wait(bar0 + 8 * ((nk - 1) & 1), ((nk - 1) >> 1) & 1)) failed = true;
  failed = __syncthreads_or(failed);
  tc_fence_after();
  if (failed) {
    if (tid == 0) atomicExch(err, 1);
  } else {
    const int64_t row = m0 + warp * 32 + lane;
    const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
    for (int32_t c0 = 0; c0 < BN; c0 += 16) {
      float v[16];
      if (nk > 0) {
        tmem_ld16(lane_addr + (uint32_t)c0, v);
      } else {
#pragma unroll
        for (int k = 0; k < 16; ++k) v[k] = 0.f;
      }
      if (row >= M) continue;
      const int64_t col = n0 + c0;
      if (ep.mode == 0) {
        float* o = ep.out32 + (int64_t)blockIdx.z * M * ep.ldo + row * ep.ldo + ep.col0 + col;
#pragma unroll
        for (int k = 0; k < 16; ++k)
          if (col + k < N) o[k] = v[k];
      } else {
        uint16_t* o = ep.out16 + row * ep.ldo + ep.col0 + col;
#pragma unroll
        for (int k = 0; k < 16; ++k)
          if (col + k < N) {
            float t = v[k] + (ep.bias ? ep.bias[col + k] : 0.f);
            if (ep.mode == 1) t = fmaxf(t, 0.f);
            o[k] = f32_to_bf16_rne(t);
          }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, ncols);
}

}  // namespace nn
