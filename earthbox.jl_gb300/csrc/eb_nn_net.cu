// eb_nn_net.cu -- the learned preconditioner stage of the Stokes solve: a BF16 convolutional
// U-Net (FP32 accumulation on the tcgen05 tensor cores), trained on the GPU by its own
// forward and backward kernels on correction pairs that the plain solver generates, and
// applied inside FGMRES after the multigrid V-cycle.
//
// Network (cells of the Stokes grid as pixels, column j as image row, row i as image column):
//   level 0 (32 ch) -> pool -> level 1 (64) -> pool -> level 2 (128) -> pool -> level 3 (128),
//   two 3x3 convolutions + ReLU per level on the way down, nearest-neighbour upsampling,
//   concatenation with the skip tensor and two 3x3 convolutions + ReLU on the way up, and a
//   1x1 output convolution to the three correction channels (vx, vy, p): 1.1M parameters.
//   Inputs: standardised log10 of the cell viscosity (etan0), standardised density (rho1 at
//   the cell's upper-left node) and the three components of a residual r divided by its RMS s.
//   Output: the correction e with A e = r, divided by s * kappa (kappa: RMS(e) / RMS(r) of the
//   training data), so the stage is z = s kappa NN(r / s) and scales with r.
//
// Layout: activations BF16 NHWC [batch][H][W][C] (the skip half of each concatenation is
// written by its encoder convolution straight into the concatenated tensor), gradients FP32.
// Convolution forward / input gradient: implicit GEMM (eb_nn_gemm.cuh) over (pixel) x
// (tap, channel); weight gradient: GEMM of the transposed im2col matrix and the transposed
// output gradient over the pixels (K), split across CTAs and reduced in a fixed order.
//
// Training pairs (scaled system A = W L W of the current Stokes system): z_true = P(xi) for
// Philox normal noise xi, v = A z_true, z1 = P(v) (P: the block multigrid preconditioner),
// e = z_true - z1 is the preconditioner's error and r = v - A z1 = A e its residual; the
// network learns r -> e on patches cut from the grid.
#include "eb_internal.h"
#include "eb_nn.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <random>
#include <vector>

namespace nn {
namespace {

constexpr int kT = 256;
unsigned blocks(int64_t n) { return (unsigned)((n + kT - 1) / kT); }

struct LayerSpec {
  int cin, cout, taps;
  bool relu;
  int level;
};
enum { E0A, E0B, E1A, E1B, E2A, E2B, E3A, E3B, D2A, D2B, D1A, D1B, D0A, D0B, OUT, kNL };
constexpr LayerSpec kLayers[kNL] = {
    {8, 32, 9, true, 0},    {32, 32, 9, true, 0},   {32, 64, 9, true, 1},   {64, 64, 9, true, 1},
    {64, 128, 9, true, 2},  {128, 128, 9, true, 2}, {128, 128, 9, true, 3}, {128, 128, 9, true, 3},
    {256, 128, 9, true, 2}, {128, 128, 9, true, 2}, {192, 64, 9, true, 1},  {64, 64, 9, true, 1},
    {96, 32, 9, true, 0},   {32, 32, 9, true, 0},   {32, 16, 1, false, 0}};
constexpr int kInC = 8, kOutC = 16, kOutUsed = 3;

// ---- elementwise kernels -------------------------------------------------------------
__device__ __forceinline__ float bf2f(uint16_t b) { return __uint_as_float((uint32_t)b << 16); }

// 2x2 average pool of channels [c0, c0+C) of src (ld lds) -> dense dst [B][H/2][W/2][C];
// one thread per 8 channels (16-byte loads and stores: C, c0 and lds are multiples of 8)
__global__ void k_pool(const uint16_t* __restrict__ src, int64_t lds, int32_t c0, int32_t C, int32_t B, int32_t H,
                       int32_t W, uint16_t* __restrict__ dst) {
  const int32_t C8 = C / 8;
  const int64_t n = (int64_t)B * (H / 2) * (W / 2) * C8;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int32_t c = (int32_t)(t % C8) * 8;
  const int64_t q = t / C8;
  const int32_t x = (int32_t)(q % (W / 2)), y = (int32_t)((q / (W / 2)) % (H / 2));
  const int32_t b = (int32_t)(q / ((int64_t)(W / 2) * (H / 2)));
  const int64_t p00 = ((int64_t)b * H + 2 * y) * W + 2 * x;
  const uint4 a = *reinterpret_cast<const uint4*>(src + p00 * lds + c0 + c);
  const uint4 b1 = *reinterpret_cast<const uint4*>(src + (p00 + 1) * lds + c0 + c);
  const uint4 b2 = *reinterpret_cast<const uint4*>(src + (p00 + W) * lds + c0 + c);
  const uint4 b3 = *reinterpret_cast<const uint4*>(src + (p00 + W + 1) * lds + c0 + c);
  const uint16_t *pa = reinterpret_cast<const uint16_t*>(&a), *p1 = reinterpret_cast<const uint16_t*>(&b1),
                 *p2 = reinterpret_cast<const uint16_t*>(&b2), *p3 = reinterpret_cast<const uint16_t*>(&b3);
  uint4 o;
  uint16_t* po = reinterpret_cast<uint16_t*>(&o);
#pragma unroll
  for (int k = 0; k < 8; ++k) po[k] = f32_to_bf16_rne(0.25f * (((bf2f(pa[k]) + bf2f(p1[k])) + bf2f(p2[k])) + bf2f(p3[k])));
  *reinterpret_cast<uint4*>(dst + q * C + c) = o;
}
// nearest upsampling of dense src [B][H/2][W/2][C] into channels [0, C) of dst (ld ldd);
// one thread per 8 channels
__global__ void k_up(const uint16_t* __restrict__ src, int32_t C, int32_t B, int32_t H, int32_t W,
                     uint16_t* __restrict__ dst, int64_t ldd) {
  const int32_t C8 = C / 8;
  const int64_t n = (int64_t)B * H * W * C8;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int32_t c = (int32_t)(t % C8) * 8;
  const int64_t p = t / C8;
  const int32_t x = (int32_t)(p % W), y = (int32_t)((p / W) % H), b = (int32_t)(p / ((int64_t)W * H));
  const int64_t q = ((int64_t)b * (H / 2) + y / 2) * (W / 2) + x / 2;
  *reinterpret_cast<uint4*>(dst + p * ldd + c) = *reinterpret_cast<const uint4*>(src + q * C + c);
}
// gradient of the upsampling: g_src[q][c] = sum of the four children's gcat[child][c], c < C
__global__ void k_up_bwd(const float* __restrict__ gcat, int64_t ldc, int32_t C, int32_t B, int32_t H, int32_t W,
                         float* __restrict__ gsrc) {
  const int64_t n = (int64_t)B * (H / 2) * (W / 2) * C;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int32_t c = (int32_t)(t % C);
  const int64_t q = t / C;
  const int32_t x = (int32_t)(q % (W / 2)), y = (int32_t)((q / (W / 2)) % (H / 2));
  const int32_t b = (int32_t)(q / ((int64_t)(W / 2) * (H / 2)));
  const int64_t p00 = ((int64_t)b * H + 2 * y) * W + 2 * x;
  gsrc[t] = (gcat[p00 * ldc + c] + gcat[(p00 + 1) * ldc + c]) + (gcat[(p00 + W) * ldc + c] + gcat[(p00 + W + 1) * ldc + c]);
}
// gradient of an encoder output that feeds both a concatenation (channels [c0, c0+C) of gcat)
// and the pool below: g[p][c] = gcat[p][c0 + c] + gx[parent(p)][c] / 4
__global__ void k_skip_grad(const float* __restrict__ gcat, int64_t ldc, int32_t c0, int32_t C,
                            const float* __restrict__ gx, int32_t B, int32_t H, int32_t W, float* __restrict__ g) {
  const int64_t n = (int64_t)B * H * W * C;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int32_t c = (int32_t)(t % C);
  const int64_t p = t / C;
  const int32_t x = (int32_t)(p % W), y = (int32_t)((p / W) % H), b = (int32_t)(p / ((int64_t)W * H));
  const int64_t q = ((int64_t)b * (H / 2) + y / 2) * (W / 2) + x / 2;
  g[t] = gcat[p * ldc + c0 + c] + 0.25f * gx[q * C + c];
}
// D = bf16(g * (a > 0)) (a: the layer's ReLU output, channels [c0, c0+C) of ld lda; null: no mask)
__global__ void k_mask(const float* __restrict__ g, const uint16_t* __restrict__ a, int64_t lda, int32_t c0,
                       int32_t C, int64_t P, uint16_t* __restrict__ d) {
  const int64_t n = P * C;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  float v = g[t];
  if (a) {
    const int64_t p = t / C;
    const int32_t c = (int32_t)(t % C);
    if (!(bf2f(a[p * lda + c0 + c]) > 0.f)) v = 0.f;
  }
  d[t] = f32_to_bf16_rne(v);
}
// out[c][p] = in[p * ld + c0 + c] for c < C, p < P, zero for P <= p < ldo (rows of ldo
// elements, a multiple of 8, so that every row starts on a 16-byte boundary for the GEMM);
// 32 x 32 tiles through shared memory
__global__ void k_transpose(const uint16_t* __restrict__ in, int64_t ld, int32_t c0, int32_t C, int64_t P,
                            int64_t ldo, uint16_t* __restrict__ out) {
  __shared__ uint16_t tile[32][33];
  const int64_t p0 = (int64_t)blockIdx.x * 32;
  const int32_t cb = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t p = p0 + r;
    const int32_t c = cb + threadIdx.x;
    tile[r][threadIdx.x] = (p < P && c < C) ? in[p * ld + c0 + c] : (uint16_t)0;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int32_t c = cb + r;
    const int64_t p = p0 + threadIdx.x;
    if (c < C && p < ldo) out[(int64_t)c * ldo + p] = tile[threadIdx.x][r];
  }
}
// transposed im2col of a 3x3 convolution: out[(t C + c)][p] = xt[c][p + d(t)] (zero outside
// the image and for P <= p < ldp); rows of ldp elements in both
__global__ void k_im2colT(const uint16_t* __restrict__ xt, int32_t C, int32_t B, int32_t H, int32_t W, int64_t ldp,
                          uint16_t* __restrict__ out) {
  const int64_t P = (int64_t)B * H * W;
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int32_t row = blockIdx.y;  // t * C + c
  if (p >= ldp) return;
  const int32_t t = row / C, c = row - t * C;
  const int32_t dy = t / 3 - 1, dx = t % 3 - 1;
  uint16_t v = 0;
  if (p < P) {
    const int32_t x = (int32_t)(p % W), y = (int32_t)((p / W) % H);
    if (y + dy >= 0 && y + dy < H && x + dx >= 0 && x + dx < W) v = xt[(int64_t)c * ldp + p + (int64_t)dy * W + dx];
  }
  out[(int64_t)row * ldp + p] = v;
}
// gb[c] = sum_p dt[c][p] in a fixed order (one block per channel; rows of ldp elements)
__global__ void k_bias_grad(const uint16_t* __restrict__ dt, int64_t P, int64_t ldp, float* __restrict__ gb) {
  __shared__ float s[kT];
  const int32_t c = blockIdx.x;
  float a = 0.f;
  for (int64_t p = threadIdx.x; p < P; p += kT) a += bf2f(dt[(int64_t)c * ldp + p]);
  s[threadIdx.x] = a;
  __syncthreads();
  for (int w = kT / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) gb[c] = s[0];
}
// gW[co][r] = sum_s part[s][r][co] (splits in order)
__global__ void k_reduce_splits(const float* __restrict__ part, int32_t S, int32_t M, int32_t N,
                                float* __restrict__ gw) {
  const int64_t n = (int64_t)M * N;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int32_t co = (int32_t)(t / M), r = (int32_t)(t % M);
  float a = 0.f;
  for (int32_t s = 0; s < S; ++s) a += part[((int64_t)s * M + r) * N + co];
  gw[t] = a;
}
// loss = sum (y - t)^2 / n over the used channels; g = 2 (y - t) / n; one partial per block
__global__ void k_loss(const float* __restrict__ y, const float* __restrict__ tgt, int64_t P, double inv_n,
                       float* __restrict__ g, double* __restrict__ partial) {
  __shared__ double s[kT];
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double a = 0.0;
  if (t < P * kOutC) {
    const int64_t p = t / kOutC;
    const int32_t c = (int32_t)(t % kOutC);
    float gv = 0.f;
    if (c < kOutUsed) {
      const double d = (double)y[t] - (double)tgt[p * kOutUsed + c];
      a = d * d;
      gv = (float)(2.0 * d * inv_n);
    }
    g[t] = gv;
  }
  s[threadIdx.x] = a;
  __syncthreads();
  for (int w = kT / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = s[0] * inv_n;
}
__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, int64_t n, float lr, float b1, float b2, float eps, float bc1,
                       float bc2) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float gt = g[t];
  const float mt = b1 * m[t] + (1.f - b1) * gt;
  const float vt = b2 * v[t] + (1.f - b2) * gt * gt;
  m[t] = mt;
  v[t] = vt;
  w[t] -= lr * (mt / bc1) / (sqrtf(vt / bc2) + eps);
}
// BF16 copies of one layer's FP32 weights [cout][taps][cin]: w16 [cout][taps cin] and the
// input-gradient operand wt16 [cin][taps cout]
__global__ void k_pack(const float* __restrict__ w, int32_t cin, int32_t cout, int32_t taps, uint16_t* __restrict__ w16,
                       uint16_t* __restrict__ wt16) {
  const int64_t n = (int64_t)cout * taps * cin;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int32_t ci = (int32_t)(t % cin), tap = (int32_t)((t / cin) % taps), co = (int32_t)(t / ((int64_t)cin * taps));
  const uint16_t b = f32_to_bf16_rne(w[t]);
  w16[t] = b;
  wt16[((int64_t)ci * taps + tap) * cout + co] = b;
}
// host FP32 NHWC [P][kInC] -> BF16
__global__ void k_to_bf16(const float* __restrict__ a, int64_t n, uint16_t* __restrict__ b) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) b[t] = f32_to_bf16_rne(a[t]);
}

// ---- network inputs from the Stokes grid ---------------------------------------------------
struct GridIn {
  const double* etan;   // [nx][ny] cell viscosity (pressure grid, column-major)
  const double* rho;    // basic grid [(nx+1)][(ny+1)]
  int32_t nx, ny;
  float eta_mean, eta_inv_std, rho_mean, rho_inv_std;
};
// batch b: pixel (y, x) of a ph x pw patch at cell offset (oj[b], oi[b]); cells outside the
// grid (padding of the full-grid image) get zeros.  r and e are SoA [3][nc]; e may be null.
__global__ void k_gather_patch(GridIn G, const double* __restrict__ r, const double* __restrict__ e, double r_scale,
                               double e_scale, const int32_t* __restrict__ oj, const int32_t* __restrict__ oi,
                               int32_t B, int32_t ph, int32_t pw, uint16_t* __restrict__ x0, float* __restrict__ tgt) {
  const int64_t P = (int64_t)B * ph * pw;
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const int32_t xx = (int32_t)(p % pw), yy = (int32_t)((p / pw) % ph), b = (int32_t)(p / ((int64_t)pw * ph));
  const int32_t j = oj[b] + yy, i = oi[b] + xx;
  float v[kInC] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  float tv[kOutUsed] = {0.f, 0.f, 0.f};
  if (j < G.nx && i < G.ny) {
    const int64_t nc = (int64_t)G.nx * G.ny;
    const int64_t c = (int64_t)j * G.ny + i;
    v[0] = ((float)log10(G.etan[c]) - G.eta_mean) * G.eta_inv_std;
    v[1] = ((float)G.rho[(int64_t)j * (G.ny + 1) + i] - G.rho_mean) * G.rho_inv_std;
    for (int k = 0; k < 3; ++k) v[2 + k] = (float)(r[k * nc + c] / r_scale);
    if (e)
      for (int k = 0; k < 3; ++k) tv[k] = (float)(e[k * nc + c] / e_scale);
  }
  for (int k = 0; k < kInC; ++k) x0[p * kInC + k] = f32_to_bf16_rne(v[k]);
  if (tgt)
    for (int k = 0; k < kOutUsed; ++k) tgt[p * kOutUsed + k] = tv[k];
}
// z[k][c] = scale * y[p][k] for the cells of the (padded) full-grid image
__global__ void k_scatter_out(const float* __restrict__ y, int32_t nx, int32_t ny, int32_t pw, double scale,
                              double* __restrict__ z) {
  const int64_t nc = (int64_t)nx * ny;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const int32_t i = (int32_t)(c % ny), j = (int32_t)(c / ny);
  const int64_t p = (int64_t)j * pw + i;
  for (int k = 0; k < 3; ++k) z[k * nc + c] = scale * (double)y[p * kOutC + k];
}
// Philox-4x32-10 normals (Box-Muller) for the training noise
__device__ __forceinline__ void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    c[1] = (uint32_t)p1;
    c[3] = (uint32_t)p0;
    c[0] = n0;
    c[2] = n2;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}
__global__ void k_noise(double* __restrict__ x, int64_t n, uint64_t seed, uint32_t step) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  uint32_t c[4] = {(uint32_t)t, (uint32_t)((uint64_t)t >> 32), step, 0x4E4Eu};
  philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  const double u1 = ((double)((((uint64_t)c[0] << 32) | c[1]) >> 11) + 0.5) * 0x1p-53;
  const double u2 = (double)((((uint64_t)c[2] << 32) | c[3]) >> 11) * 0x1p-53;
  x[t] = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}
__global__ void k_axpby(double* y, const double* a, const double* b, double beta, int64_t n) {  // y = a + beta b (y may be b)
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) y[t] = a[t] + beta * b[t];
}

}  // namespace

// ------------------------------------------------------------------ the network ---
struct Net {
  int64_t woff[kNL], boff[kNL], w16off[kNL];
  int64_t nparam = 0, nw16 = 0;
  float *w32 = nullptr, *m = nullptr, *v = nullptr, *g = nullptr;
  uint16_t *w16 = nullptr, *wt16 = nullptr;
  int32_t* err = nullptr;
  int64_t adam_t = 0;
  bool trained = false;
  float eta_mean = 0.f, eta_inv_std = 1.f, rho_mean = 0.f, rho_inv_std = 1.f;
  double kappa = 1.0;
  std::vector<void*> base_allocs;
  // workspace for one (B, H, W)
  int32_t B = 0, H = 0, W = 0;
  std::vector<void*> ws;
  uint16_t *X0 = nullptr, *X1 = nullptr, *X2 = nullptr, *X3 = nullptr, *CAT0 = nullptr, *CAT1 = nullptr, *CAT2 = nullptr;
  uint16_t* A[kNL] = {};
  float* Y = nullptr;
  float* G[kNL] = {};
  float *GY = nullptr, *GCAT0 = nullptr, *GCAT1 = nullptr, *GCAT2 = nullptr, *GX1 = nullptr, *GX2 = nullptr,
        *GX3 = nullptr, *T = nullptr, *part = nullptr;
  size_t part_cap = 0;
  uint16_t *D16 = nullptr, *DT16 = nullptr, *XT16 = nullptr, *IM = nullptr;
  double* lpart = nullptr;
  int32_t *d_oj = nullptr, *d_oi = nullptr;
  // solver-side full-grid buffers (scaled system, 3 nc each)
  int64_t n3 = 0;
  double *gz = nullptr, *gv = nullptr, *gz1 = nullptr, *ge = nullptr, *gr = nullptr;
  std::vector<void*> grid_allocs;
  // statistics of the stage inside FGMRES
  int64_t accepted = 0, rejected = 0;
  double seconds = 0.0, removed = 0.0;
};

namespace {

int nalloc(eb_ctx* c, std::vector<void*>& owner, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes + 16);
  if (e != cudaSuccess) return eb_cuda(c, e, "learned preconditioner buffer");
  owner.push_back(*p);
  return EB_OK;
}
template <class T>
int nalloc(eb_ctx* c, std::vector<void*>& owner, T** p, size_t n) {
  return nalloc(c, owner, reinterpret_cast<void**>(p), n * sizeof(T));
}
void free_all(std::vector<void*>& v) {
  for (void* p : v) cudaFree(p);
  v.clear();
}

int64_t level_pixels(const Net* n, int l) { return (int64_t)n->B * (n->H >> l) * (n->W >> l); }

int ensure_net(eb_ctx* c) {
  if (c->net) return EB_OK;
  Net* n = new Net();
  int64_t off = 0, off16 = 0;
  for (int l = 0; l < kNL; ++l) {
    const LayerSpec& L = kLayers[l];
    n->woff[l] = off;
    off += (int64_t)L.cout * L.taps * L.cin;
    n->boff[l] = off;
    off += L.cout;
    n->w16off[l] = off16;
    off16 += (int64_t)L.cout * L.taps * L.cin;
  }
  n->nparam = off;
  n->nw16 = off16;
  c->net = n;
  int rc;
  if ((rc = nalloc(c, n->base_allocs, &n->w32, off)) || (rc = nalloc(c, n->base_allocs, &n->m, off)) ||
      (rc = nalloc(c, n->base_allocs, &n->v, off)) || (rc = nalloc(c, n->base_allocs, &n->g, off)) ||
      (rc = nalloc(c, n->base_allocs, &n->w16, off16)) || (rc = nalloc(c, n->base_allocs, &n->wt16, off16)) ||
      (rc = nalloc(c, n->base_allocs, &n->err, 1)))
    return rc;
  cudaMemsetAsync(n->m, 0, off * sizeof(float), c->stream);
  cudaMemsetAsync(n->v, 0, off * sizeof(float), c->stream);
  cudaMemsetAsync(n->err, 0, sizeof(int32_t), c->stream);
  return EB_OK;
}

int pack(eb_ctx* c, Net* n) {
  for (int l = 0; l < kNL; ++l) {
    const LayerSpec& L = kLayers[l];
    EB_PROF(c, "k_nn_pack");
    k_pack<<<blocks((int64_t)L.cout * L.taps * L.cin), kT, 0, c->stream>>>(
        n->w32 + n->woff[l], L.cin, L.cout, L.taps, n->w16 + n->w16off[l], n->wt16 + n->w16off[l]);
    EB_LAUNCHED(c);
  }
  return EB_OK;
}

// He-normal weights, zero biases; the output rows beyond the three used channels are zero
int init_weights(eb_ctx* c, Net* n, uint64_t seed) {
  std::vector<float> h(n->nparam, 0.f);
  std::mt19937_64 gen(seed);
  for (int l = 0; l < kNL; ++l) {
    const LayerSpec& L = kLayers[l];
    const double sd = std::sqrt(2.0 / ((double)L.taps * L.cin)) * (l == OUT ? 0.1 : 1.0);
    std::normal_distribution<double> nd(0.0, sd);
    for (int co = 0; co < L.cout; ++co)
      for (int k = 0; k < L.taps * L.cin; ++k) {
        const double w = nd(gen);
        if (l == OUT && co >= kOutUsed) continue;
        h[n->woff[l] + (int64_t)co * L.taps * L.cin + k] = (float)w;
      }
  }
  EB_CK(c, cudaMemcpyAsync(n->w32, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  EB_CK(c, cudaMemsetAsync(n->m, 0, n->nparam * sizeof(float), c->stream));
  EB_CK(c, cudaMemsetAsync(n->v, 0, n->nparam * sizeof(float), c->stream));
  n->adam_t = 0;
  n->trained = false;
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return pack(c, n);
}

int ensure_workspace(eb_ctx* c, Net* n, int32_t B, int32_t H, int32_t W) {
  if (n->B == B && n->H == H && n->W == W) return EB_OK;
  free_all(n->ws);
  n->B = B;
  n->H = H;
  n->W = W;
  const int64_t P0 = level_pixels(n, 0), P1 = level_pixels(n, 1), P2 = level_pixels(n, 2), P3 = level_pixels(n, 3);
  int rc;
  auto A16 = [&](uint16_t** p, int64_t cnt) { return nalloc(c, n->ws, p, (size_t)cnt); };
  auto A32 = [&](float** p, int64_t cnt) { return nalloc(c, n->ws, p, (size_t)cnt); };
  if ((rc = A16(&n->X0, P0 * kInC)) || (rc = A16(&n->X1, P1 * 32)) || (rc = A16(&n->X2, P2 * 64)) ||
      (rc = A16(&n->X3, P3 * 128)) || (rc = A16(&n->CAT0, P0 * 96)) || (rc = A16(&n->CAT1, P1 * 192)) ||
      (rc = A16(&n->CAT2, P2 * 256)) || (rc = A32(&n->Y, P0 * kOutC)) || (rc = A32(&n->GY, P0 * kOutC)) ||
      (rc = A32(&n->GCAT0, P0 * 96)) || (rc = A32(&n->GCAT1, P1 * 192)) || (rc = A32(&n->GCAT2, P2 * 256)) ||
      (rc = A32(&n->GX1, P1 * 32)) || (rc = A32(&n->GX2, P2 * 64)) || (rc = A32(&n->GX3, P3 * 128)) ||
      (rc = A32(&n->T, P0 * kOutUsed)) || (rc = A16(&n->D16, P0 * 128)) || (rc = A16(&n->DT16, (P0 + 8) * 128)) ||
      (rc = A16(&n->XT16, (P0 + 8) * 256)) || (rc = A16(&n->IM, (P0 + 8) * 9 * 96)) ||
      (rc = nalloc(c, n->ws, &n->lpart, (size_t)blocks(P0 * kOutC))) || (rc = nalloc(c, n->ws, &n->d_oj, 64)) ||
      (rc = nalloc(c, n->ws, &n->d_oi, 64)))
    return rc;
  // the largest per-level products bound the im2col and transposed buffers (rows padded to a
  // multiple of 8 pixels): level 0: 9 x 96 x P0, level 1: 9 x 192 x P0/4, level 2: 9 x 256 x P0/16,
  // level 3: 9 x 128 x P0/64; transposed inputs at most 96 x P0, transposed gradients 32 x P0
  for (int l = 0; l < kNL; ++l) {
    if (l == E0B || l == E1B || l == E2B || l == OUT) continue;  // written into a concatenation / Y
    if ((rc = A16(&n->A[l], level_pixels(n, kLayers[l].level) * kLayers[l].cout))) return rc;
  }
  for (int l = 0; l < kNL; ++l)
    if ((rc = A32(&n->G[l], level_pixels(n, kLayers[l].level) * kLayers[l].cout))) return rc;
  n->part_cap = 0;
  return EB_OK;
}

struct Act {
  const uint16_t* p;
  int64_t ld;
  int32_t c0;
};
Act layer_in(const Net* n, int l) {
  switch (l) {
    case E0A: return {n->X0, kInC, 0};
    case E1A: return {n->X1, 32, 0};
    case E2A: return {n->X2, 64, 0};
    case E3A: return {n->X3, 128, 0};
    case D2A: return {n->CAT2, 256, 0};
    case D1A: return {n->CAT1, 192, 0};
    case D0A: return {n->CAT0, 96, 0};
    default: return {n->A[l - 1], kLayers[l - 1].cout, 0};
  }
}
Act layer_out(const Net* n, int l) {
  switch (l) {
    case E0B: return {n->CAT0, 96, 64};
    case E1B: return {n->CAT1, 192, 128};
    case E2B: return {n->CAT2, 256, 128};
    default: return {n->A[l], kLayers[l].cout, 0};
  }
}

int conv_forward(eb_ctx* c, Net* n, int l) {
  const LayerSpec& L = kLayers[l];
  const int lv = L.level;
  const Act in = layer_in(n, l);
  const ConvLoader a{in.p, n->B, n->H >> lv, n->W >> lv, L.cin, L.taps, 0};
  const int64_t K = (int64_t)L.taps * L.cin;
  const MatLoader b{n->w16 + n->w16off[l], K, L.cout, K};
  Epilogue ep{};
  if (l == OUT) {
    ep = Epilogue{n->Y, nullptr, n->w32 + n->boff[l], kOutC, 0, 0};
  } else {
    const Act o = layer_out(n, l);
    ep = Epilogue{nullptr, const_cast<uint16_t*>(o.p), n->w32 + n->boff[l], o.ld, o.c0, L.relu ? 1 : 2};
  }
  EB_PROF(c, "k_gemm_bf16<conv>");
  const cudaError_t e = launch_gemm(a, b, level_pixels(n, lv), L.cout, K, ep, 1, c->stream, n->err);
  if (e != cudaSuccess) return eb_cuda(c, e, "tensor-core convolution");
  prof_end(c);
  c->launches++;
  return EB_OK;
}

// ep for the output layer adds the bias through the FP32 path: mode 0 has no bias, so add it
__global__ void k_add_bias(float* __restrict__ y, const float* __restrict__ b, int64_t P, int32_t C) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < P * C) y[t] += b[t % C];
}

int forward(eb_ctx* c, Net* n) {
  int rc;
  const int32_t B = n->B, H = n->H, W = n->W;
  auto pool = [&](const uint16_t* src, int64_t lds, int32_t c0, int32_t C, int lv, uint16_t* dst) {
    const int32_t h = H >> lv, w = W >> lv;
    EB_PROF(c, "k_nn_pool");
    k_pool<<<blocks((int64_t)B * (h / 2) * (w / 2) * (C / 8)), kT, 0, c->stream>>>(src, lds, c0, C, B, h, w, dst);
    EB_LAUNCHED(c);
    return EB_OK;
  };
  auto up = [&](const uint16_t* src, int32_t C, int lv, uint16_t* dst, int64_t ldd) {
    const int32_t h = H >> lv, w = W >> lv;  // destination level
    EB_PROF(c, "k_nn_up");
    k_up<<<blocks((int64_t)B * h * w * (C / 8)), kT, 0, c->stream>>>(src, C, B, h, w, dst, ldd);
    EB_LAUNCHED(c);
    return EB_OK;
  };
  if ((rc = conv_forward(c, n, E0A)) || (rc = conv_forward(c, n, E0B)) || (rc = pool(n->CAT0, 96, 64, 32, 0, n->X1)) ||
      (rc = conv_forward(c, n, E1A)) || (rc = conv_forward(c, n, E1B)) || (rc = pool(n->CAT1, 192, 128, 64, 1, n->X2)) ||
      (rc = conv_forward(c, n, E2A)) || (rc = conv_forward(c, n, E2B)) ||
      (rc = pool(n->CAT2, 256, 128, 128, 2, n->X3)) || (rc = conv_forward(c, n, E3A)) ||
      (rc = conv_forward(c, n, E3B)) || (rc = up(n->A[E3B], 128, 2, n->CAT2, 256)) || (rc = conv_forward(c, n, D2A)) ||
      (rc = conv_forward(c, n, D2B)) || (rc = up(n->A[D2B], 128, 1, n->CAT1, 192)) || (rc = conv_forward(c, n, D1A)) ||
      (rc = conv_forward(c, n, D1B)) || (rc = up(n->A[D1B], 64, 0, n->CAT0, 96)) || (rc = conv_forward(c, n, D0A)) ||
      (rc = conv_forward(c, n, D0B)) || (rc = conv_forward(c, n, OUT)))
    return rc;
  const int64_t P0 = level_pixels(n, 0);
  EB_PROF(c, "k_nn_bias");
  k_add_bias<<<blocks(P0 * kOutC), kT, 0, c->stream>>>(n->Y, n->w32 + n->boff[OUT], P0, kOutC);
  EB_LAUNCHED(c);
  return EB_OK;
}

// weight, bias and (when gin is non-null) input gradient of layer l from its output gradient
int layer_backward(eb_ctx* c, Net* n, int l, const float* gout, float* gin) {
  const LayerSpec& L = kLayers[l];
  const int lv = L.level;
  const int32_t h = n->H >> lv, w = n->W >> lv;
  const int64_t P = level_pixels(n, lv);
  const int64_t ldP = (P + 7) / 8 * 8;  // row stride of the transposed operands
  const Act o = layer_out(n, l);
  EB_PROF(c, "k_nn_mask");
  k_mask<<<blocks(P * L.cout), kT, 0, c->stream>>>(gout, L.relu ? o.p : nullptr, o.ld, o.c0, L.cout, P, n->D16);
  EB_LAUNCHED(c);
  const dim3 tb(32, 8);
  EB_PROF(c, "k_nn_transpose");
  k_transpose<<<dim3((unsigned)((ldP + 31) / 32), (unsigned)((L.cout + 31) / 32)), tb, 0, c->stream>>>(
      n->D16, L.cout, 0, L.cout, P, ldP, n->DT16);
  EB_LAUNCHED(c);
  EB_PROF(c, "k_nn_bias_grad");
  k_bias_grad<<<L.cout, kT, 0, c->stream>>>(n->DT16, P, ldP, n->g + n->boff[l]);
  EB_LAUNCHED(c);
  const Act in = layer_in(n, l);
  EB_PROF(c, "k_nn_transpose");
  k_transpose<<<dim3((unsigned)((ldP + 31) / 32), (unsigned)((L.cin + 31) / 32)), tb, 0, c->stream>>>(
      in.p, in.ld, in.c0, L.cin, P, ldP, n->XT16);
  EB_LAUNCHED(c);
  const uint16_t* amat = n->XT16;
  if (L.taps == 9) {
    EB_PROF(c, "k_nn_im2col");
    k_im2colT<<<dim3(blocks(ldP), (unsigned)(9 * L.cin)), kT, 0, c->stream>>>(n->XT16, L.cin, n->B, h, w, ldP, n->IM);
    EB_LAUNCHED(c);
    amat = n->IM;
  }
  // weight gradient: part[s][r][co] = sum over this split's pixels of im2colT[r][p] D[p][co]
  const int32_t M = L.taps * L.cin;
  const int64_t mtiles = (M + kTileM - 1) / kTileM, kchunks = (P + kChunkK - 1) / kChunkK;
  const int32_t S = (int32_t)std::max<int64_t>(1, std::min<int64_t>(kchunks, 304 / mtiles));
  const size_t need = (size_t)S * M * L.cout;
  if (need > n->part_cap) {
    for (auto it = n->ws.begin(); it != n->ws.end(); ++it)
      if (*it == n->part) { cudaFree(n->part); n->ws.erase(it); break; }
    n->part = nullptr;
    int rc = nalloc(c, n->ws, &n->part, need);
    if (rc) return rc;
    n->part_cap = need;
  }
  const MatLoader a{amat, ldP, M, P}, b{n->DT16, ldP, L.cout, P};
  const Epilogue ep{n->part, nullptr, nullptr, L.cout, 0, 0};
  EB_PROF(c, "k_gemm_bf16<wgrad>");
  cudaError_t e = launch_gemm(a, b, M, L.cout, P, ep, S, c->stream, n->err);
  if (e != cudaSuccess) return eb_cuda(c, e, "tensor-core weight gradient");
  prof_end(c);
  c->launches++;
  EB_PROF(c, "k_nn_reduce");
  k_reduce_splits<<<blocks((int64_t)M * L.cout), kT, 0, c->stream>>>(n->part, S, M, L.cout, n->g + n->woff[l]);
  EB_LAUNCHED(c);
  if (gin) {
    const ConvLoader da{n->D16, n->B, h, w, L.cout, L.taps, 1};
    const int64_t K = (int64_t)L.taps * L.cout;
    const MatLoader db{n->wt16 + n->w16off[l], K, L.cin, K};
    const Epilogue dep{gin, nullptr, nullptr, L.cin, 0, 0};
    EB_PROF(c, "k_gemm_bf16<dgrad>");
    e = launch_gemm(da, db, P, L.cin, K, dep, 1, c->stream, n->err);
    if (e != cudaSuccess) return eb_cuda(c, e, "tensor-core input gradient");
    prof_end(c);
    c->launches++;
  }
  return EB_OK;
}

// loss of the current Y against T and all gradients (n->g); returns the loss
int loss_backward(eb_ctx* c, Net* n, double* loss) {
  const int32_t B = n->B, H = n->H, W = n->W;
  const int64_t P0 = level_pixels(n, 0);
  const unsigned nb = blocks(P0 * kOutC);
  EB_PROF(c, "k_nn_loss");
  k_loss<<<nb, kT, 0, c->stream>>>(n->Y, n->T, P0, 1.0 / ((double)P0 * kOutUsed), n->GY, n->lpart);
  EB_LAUNCHED(c);
  auto upb = [&](const float* gcat, int64_t ldc, int32_t C, int lv_dst, float* g) {
    const int32_t h = H >> (lv_dst - 1), w = W >> (lv_dst - 1);  // the finer level
    EB_PROF(c, "k_nn_up_bwd");
    k_up_bwd<<<blocks((int64_t)B * (h / 2) * (w / 2) * C), kT, 0, c->stream>>>(gcat, ldc, C, B, h, w, g);
    EB_LAUNCHED(c);
    return EB_OK;
  };
  auto skip = [&](const float* gcat, int64_t ldc, int32_t c0, int32_t C, const float* gx, int lv, float* g) {
    const int32_t h = H >> lv, w = W >> lv;
    EB_PROF(c, "k_nn_skip_grad");
    k_skip_grad<<<blocks((int64_t)B * h * w * C), kT, 0, c->stream>>>(gcat, ldc, c0, C, gx, B, h, w, g);
    EB_LAUNCHED(c);
    return EB_OK;
  };
  int rc;
  if ((rc = layer_backward(c, n, OUT, n->GY, n->G[D0B])) || (rc = layer_backward(c, n, D0B, n->G[D0B], n->G[D0A])) ||
      (rc = layer_backward(c, n, D0A, n->G[D0A], n->GCAT0)) || (rc = upb(n->GCAT0, 96, 64, 1, n->G[D1B])) ||
      (rc = layer_backward(c, n, D1B, n->G[D1B], n->G[D1A])) || (rc = layer_backward(c, n, D1A, n->G[D1A], n->GCAT1)) ||
      (rc = upb(n->GCAT1, 192, 128, 2, n->G[D2B])) || (rc = layer_backward(c, n, D2B, n->G[D2B], n->G[D2A])) ||
      (rc = layer_backward(c, n, D2A, n->G[D2A], n->GCAT2)) || (rc = upb(n->GCAT2, 256, 128, 3, n->G[E3B])) ||
      (rc = layer_backward(c, n, E3B, n->G[E3B], n->G[E3A])) || (rc = layer_backward(c, n, E3A, n->G[E3A], n->GX3)) ||
      (rc = skip(n->GCAT2, 256, 128, 128, n->GX3, 2, n->G[E2B])) ||
      (rc = layer_backward(c, n, E2B, n->G[E2B], n->G[E2A])) || (rc = layer_backward(c, n, E2A, n->G[E2A], n->GX2)) ||
      (rc = skip(n->GCAT1, 192, 128, 64, n->GX2, 1, n->G[E1B])) ||
      (rc = layer_backward(c, n, E1B, n->G[E1B], n->G[E1A])) || (rc = layer_backward(c, n, E1A, n->G[E1A], n->GX1)) ||
      (rc = skip(n->GCAT0, 96, 64, 32, n->GX1, 0, n->G[E0B])) ||
      (rc = layer_backward(c, n, E0B, n->G[E0B], n->G[E0A])) || (rc = layer_backward(c, n, E0A, n->G[E0A], nullptr)))
    return rc;
  std::vector<double> h(nb);
  EB_CK(c, cudaMemcpyAsync(h.data(), n->lpart, nb * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  double s = 0.0;
  for (double v : h) s += v;
  *loss = s;
  return EB_OK;
}

int check_err(eb_ctx* c, Net* n) {
  int32_t h = 0;
  EB_CK(c, cudaMemcpyAsync(&h, n->err, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  if (h) return eb_fail(c, EB_CUDA_ERROR, "tensor-core kernel gave up waiting on its MMA barrier");
  return EB_OK;
}

int adam_step(eb_ctx* c, Net* n, float lr) {
  n->adam_t++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = 1.f - std::pow(b1, (float)n->adam_t), bc2 = 1.f - std::pow(b2, (float)n->adam_t);
  EB_PROF(c, "k_nn_adam");
  k_adam<<<blocks(n->nparam), kT, 0, c->stream>>>(n->w32, n->m, n->v, n->g, n->nparam, lr, b1, b2, 1e-8f, bc1, bc2);
  EB_LAUNCHED(c);
  return pack(c, n);
}

}  // namespace
}  // namespace nn

using namespace nn;

void nn_free(eb_ctx* c) {
  if (!c || !c->net) return;
  free_all(c->net->ws);
  free_all(c->net->grid_allocs);
  free_all(c->net->base_allocs);
  delete c->net;
  c->net = nullptr;
}

bool nn_trained(const eb_ctx* c) { return c && c->net && c->net->trained; }

// ------------------------------------------------------------------ solver side ---
namespace {
// grid statistics of the two physical input channels
int grid_stats(eb_ctx* c, Net* n, const StokesSystem& s) {
  const int64_t nc = s.nc, nb = (int64_t)(s.nx + 1) * (s.ny + 1);
  std::vector<double> eta(nc), rho(nb);
  EB_CK(c, cudaMemcpyAsync(eta.data(), c->gf[EB_G_ETAN0], nc * 8, cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaMemcpyAsync(rho.data(), c->gf[EB_G_RHO1], nb * 8, cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  double m1 = 0, m2 = 0, r1 = 0, r2 = 0;
  for (double e : eta) { const double l = std::log10(std::max(e, 1e-300)); m1 += l; m2 += l * l; }
  for (double r : rho) { r1 += r; r2 += r * r; }
  m1 /= nc; m2 /= nc; r1 /= nb; r2 /= nb;
  n->eta_mean = (float)m1;
  n->eta_inv_std = (float)(1.0 / std::sqrt(std::max(m2 - m1 * m1, 1e-12)));
  n->rho_mean = (float)r1;
  n->rho_inv_std = (float)(1.0 / std::sqrt(std::max(r2 - r1 * r1, 1e-12)));
  return EB_OK;
}
GridIn grid_in(eb_ctx* c, const Net* n, const StokesSystem& s) {
  return GridIn{c->gf[EB_G_ETAN0], c->gf[EB_G_RHO1], s.nx, s.ny, n->eta_mean, n->eta_inv_std, n->rho_mean,
                n->rho_inv_std};
}
int ensure_grid_buffers(eb_ctx* c, Net* n, int64_t n3) {
  if (n->n3 == n3 && n->gz) return EB_OK;
  free_all(n->grid_allocs);
  n->n3 = n3;
  int rc;
  if ((rc = nalloc(c, n->grid_allocs, &n->gz, n3)) || (rc = nalloc(c, n->grid_allocs, &n->gv, n3)) ||
      (rc = nalloc(c, n->grid_allocs, &n->gz1, n3)) || (rc = nalloc(c, n->grid_allocs, &n->ge, n3)) ||
      (rc = nalloc(c, n->grid_allocs, &n->gr, n3)))
    return rc;
  return EB_OK;
}
int32_t ceil8(int32_t v) { return (v + 7) / 8 * 8; }
}  // namespace

// z_add = s kappa NN(t / s) on the full grid (t, z_add: scaled-system SoA vectors)
int nn_correction(eb_ctx* c, const double* t, double s, double* z_add) {
  Net* n = c->net;
  const StokesSystem& sys = *stokes_system(c);
  if (!c->gf[EB_G_ETAN0] || !c->gf[EB_G_RHO1])
    return eb_fail(c, EB_NOT_READY, "etan0 and rho1 (network inputs) are not on the device");
  int rc;
  if ((rc = ensure_workspace(c, n, 1, ceil8(sys.nx), ceil8(sys.ny)))) return rc;
  const int32_t zero = 0;
  EB_CK(c, cudaMemcpyAsync(n->d_oj, &zero, 4, cudaMemcpyHostToDevice, c->stream));
  EB_CK(c, cudaMemcpyAsync(n->d_oi, &zero, 4, cudaMemcpyHostToDevice, c->stream));
  EB_PROF(c, "k_nn_gather");
  k_gather_patch<<<blocks(level_pixels(n, 0)), kT, 0, c->stream>>>(grid_in(c, n, sys), t, nullptr, s, 1.0, n->d_oj,
                                                                    n->d_oi, 1, n->H, n->W, n->X0, nullptr);
  EB_LAUNCHED(c);
  if ((rc = forward(c, n))) return rc;
  EB_PROF(c, "k_nn_scatter");
  k_scatter_out<<<blocks(sys.nc), kT, 0, c->stream>>>(n->Y, sys.nx, sys.ny, n->W, s * n->kappa, z_add);
  EB_LAUNCHED(c);
  return EB_OK;
}

void nn_count(eb_ctx* c, bool accepted, double seconds, double removed) {
  if (!c->net) return;
  (accepted ? c->net->accepted : c->net->rejected)++;
  c->net->seconds += seconds;
  c->net->removed += removed;
}

// ------------------------------------------------------------------ C-ABI ---
extern "C" int eb_learned_init(eb_ctx* c, uint64_t seed) {
  if (!c) return EB_BAD_INPUT;
  cudaSetDevice(c->device);
  int rc;
  if ((rc = ensure_net(c))) return rc;
  return init_weights(c, c->net, seed);
}

extern "C" int eb_learned_params(eb_ctx* c, float* host, int64_t capacity, int64_t* n, int32_t set) {
  if (!c || !n) return EB_BAD_INPUT;
  cudaSetDevice(c->device);
  int rc;
  if ((rc = ensure_net(c))) return rc;
  Net* net = c->net;
  *n = net->nparam;
  if (!host) return EB_OK;
  if (capacity < net->nparam) return eb_fail(c, EB_BAD_INPUT, "parameter array too small");
  if (set) {
    EB_CK(c, cudaMemcpyAsync(net->w32, host, net->nparam * 4, cudaMemcpyHostToDevice, c->stream));
    EB_CK(c, cudaStreamSynchronize(c->stream));
    if ((rc = pack(c, net))) return rc;
  } else {
    EB_CK(c, cudaMemcpyAsync(host, net->w32, net->nparam * 4, cudaMemcpyDeviceToHost, c->stream));
  }
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return EB_OK;
}

extern "C" int eb_learned_state(eb_ctx* c, double* state, int32_t set) {
  // state: eta_mean, eta_inv_std, rho_mean, rho_inv_std, kappa, trained
  if (!c || !state) return EB_BAD_INPUT;
  int rc;
  if ((rc = ensure_net(c))) return rc;
  Net* n = c->net;
  if (set) {
    n->eta_mean = (float)state[0];
    n->eta_inv_std = (float)state[1];
    n->rho_mean = (float)state[2];
    n->rho_inv_std = (float)state[3];
    n->kappa = state[4];
    n->trained = state[5] != 0.0;
  } else {
    state[0] = n->eta_mean;
    state[1] = n->eta_inv_std;
    state[2] = n->rho_mean;
    state[3] = n->rho_inv_std;
    state[4] = n->kappa;
    state[5] = n->trained ? 1.0 : 0.0;
  }
  return EB_OK;
}

extern "C" int eb_learned_forward(eb_ctx* c, int32_t B, int32_t H, int32_t W, const float* x, float* y) {
  if (!c || !x || !y || B <= 0 || H <= 0 || W <= 0 || H % 8 || W % 8) return EB_BAD_INPUT;
  cudaSetDevice(c->device);
  int rc;
  if ((rc = ensure_net(c)) || (rc = ensure_workspace(c, c->net, B, H, W))) return rc;
  Net* n = c->net;
  const int64_t P0 = level_pixels(n, 0);
  float* dx = nullptr;
  EB_CK(c, cudaMalloc(&dx, P0 * kInC * sizeof(float)));
  cudaError_t e = cudaMemcpyAsync(dx, x, P0 * kInC * sizeof(float), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) {
    k_to_bf16<<<blocks(P0 * kInC), kT, 0, c->stream>>>(dx, P0 * kInC, n->X0);
    c->launches++;
  }
  if (e == cudaSuccess && (rc = forward(c, n))) { cudaFree(dx); return rc; }
  if (e == cudaSuccess) e = cudaMemcpyAsync(y, n->Y, P0 * kOutC * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(dx);
  if (e != cudaSuccess) return eb_cuda(c, e, "learned forward");
  return check_err(c, n);
}

extern "C" int eb_learned_loss_grad(eb_ctx* c, int32_t B, int32_t H, int32_t W, const float* x, const float* t,
                                    double* loss, float* grad) {
  if (!c || !x || !t || !loss || B <= 0 || H <= 0 || W <= 0 || H % 8 || W % 8) return EB_BAD_INPUT;
  cudaSetDevice(c->device);
  int rc;
  if ((rc = ensure_net(c)) || (rc = ensure_workspace(c, c->net, B, H, W))) return rc;
  Net* n = c->net;
  const int64_t P0 = level_pixels(n, 0);
  float* dx = nullptr;
  EB_CK(c, cudaMalloc(&dx, P0 * kInC * sizeof(float)));
  cudaError_t e = cudaMemcpyAsync(dx, x, P0 * kInC * sizeof(float), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(n->T, t, P0 * kOutUsed * sizeof(float), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) {
    k_to_bf16<<<blocks(P0 * kInC), kT, 0, c->stream>>>(dx, P0 * kInC, n->X0);
    c->launches++;
  }
  if (e != cudaSuccess) { cudaFree(dx); return eb_cuda(c, e, "learned loss input"); }
  if ((rc = forward(c, n)) || (rc = loss_backward(c, n, loss))) { cudaFree(dx); return rc; }
  cudaFree(dx);
  if (grad) EB_CK(c, cudaMemcpyAsync(grad, n->g, n->nparam * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  EB_CK(c, cudaStreamSynchronize(c->stream));
  return check_err(c, n);
}

// Services of the Stokes solver on its diagonally scaled system (eb_stokes_solve.cu).
int stokes_nn_ready(eb_ctx* c, int sweeps);
int stokes_nn_apply(eb_ctx* c, const double* x, double* y);
int stokes_nn_precondition(eb_ctx* c, const double* r, double* z);
int stokes_nn_dot(eb_ctx* c, const double* a, const double* b, double* out);

extern "C" int eb_learned_train(eb_ctx* c, const eb_learned_opts* o, eb_learned_report* rep) {
  if (!c || !o) return EB_BAD_INPUT;
  if (o->batch <= 0 || o->batch > 16 || o->steps <= 0 || o->patch < 8 || o->patch % 8 || o->lr <= 0)
    return eb_fail(c, EB_BAD_INPUT, "eb_learned_opts: batch 1..16, steps > 0, patch a positive multiple of 8, lr > 0");
  cudaSetDevice(c->device);
  const auto t0 = std::chrono::steady_clock::now();
  int rc;
  if ((rc = ensure_net(c)) || (rc = stokes_nn_ready(c, o->mg_sweeps > 0 ? o->mg_sweeps : 3))) return rc;
  Net* n = c->net;
  const StokesSystem& s = *stokes_system(c);
  const int64_t n3 = 3 * s.nc;
  if (!c->gf[EB_G_ETAN0] || !c->gf[EB_G_RHO1])
    return eb_fail(c, EB_NOT_READY, "etan0 and rho1 (network inputs) are not on the device");
  if ((rc = ensure_grid_buffers(c, n, n3)) || (rc = grid_stats(c, n, s))) return rc;
  const int32_t ph = std::min(o->patch, s.nx / 8 * 8), pw = std::min(o->patch, s.ny / 8 * 8);
  if (ph < 8 || pw < 8) return eb_fail(c, EB_BAD_INPUT, "grid smaller than one 8 x 8 patch");
  if ((rc = ensure_workspace(c, n, o->batch, ph, pw))) return rc;
  std::mt19937_64 gen(o->seed ^ 0x5DEECE66DULL);
  double first = 0.0, last = 0.0, rs = 1.0;
  const int avg = std::max(1, std::min(8, o->steps / 2));
  const int per_sample = std::max(1, o->patches_per_sample);
  std::uniform_int_distribution<int32_t> dj(0, s.nx - ph), di(0, s.ny - pw);
  std::vector<int32_t> oj(o->batch), oi(o->batch);
  for (int step = 0; step < o->steps; ++step) {
    if (step % per_sample == 0) {
      // a new full-grid sample: z_true = P(xi), v = A z_true, z1 = P(v), e = z_true - z1,
      // r = v - A z1 (= A e)
      EB_PROF(c, "k_nn_noise");
      k_noise<<<blocks(n3), kT, 0, c->stream>>>(n->gv, n3, o->seed, (uint32_t)step);
      EB_LAUNCHED(c);
      if ((rc = stokes_nn_precondition(c, n->gv, n->gz)) || (rc = stokes_nn_apply(c, n->gz, n->gv)) ||
          (rc = stokes_nn_precondition(c, n->gv, n->gz1)) || (rc = stokes_nn_apply(c, n->gz1, n->gr)))
        return rc;
      EB_PROF(c, "k_nn_axpby");
      k_axpby<<<blocks(n3), kT, 0, c->stream>>>(n->ge, n->gz, n->gz1, -1.0, n3);
      EB_LAUNCHED(c);
      EB_PROF(c, "k_nn_axpby");
      k_axpby<<<blocks(n3), kT, 0, c->stream>>>(n->gr, n->gv, n->gr, -1.0, n3);
      EB_LAUNCHED(c);
      double rr, ee;
      if ((rc = stokes_nn_dot(c, n->gr, n->gr, &rr)) || (rc = stokes_nn_dot(c, n->ge, n->ge, &ee))) return rc;
      if (!(rr > 0.0) || !std::isfinite(rr) || !std::isfinite(ee))
        return eb_fail(c, EB_NAN, "training sample has a zero or non-finite residual");
      rs = std::sqrt(rr / n3);
      // the output scale is fixed by the first sample an untrained network sees
      if (step == 0 && !n->trained) n->kappa = std::sqrt(ee / n3) / rs;
    }
    for (int b = 0; b < o->batch; ++b) { oj[b] = dj(gen); oi[b] = di(gen); }
    EB_CK(c, cudaMemcpyAsync(n->d_oj, oj.data(), o->batch * 4, cudaMemcpyHostToDevice, c->stream));
    EB_CK(c, cudaMemcpyAsync(n->d_oi, oi.data(), o->batch * 4, cudaMemcpyHostToDevice, c->stream));
    EB_PROF(c, "k_nn_gather");
    k_gather_patch<<<blocks(level_pixels(n, 0)), kT, 0, c->stream>>>(grid_in(c, n, s), n->gr, n->ge, rs, rs * n->kappa,
                                                                      n->d_oj, n->d_oi, o->batch, ph, pw, n->X0, n->T);
    EB_LAUNCHED(c);
    double loss;
    if ((rc = forward(c, n)) || (rc = loss_backward(c, n, &loss)) || (rc = adam_step(c, n, (float)o->lr))) return rc;
    if (!std::isfinite(loss)) return eb_fail(c, EB_NAN, "training loss became NaN/Inf");
    // mean loss of the first and of the last `avg` steps
    if (step < avg) first += loss / avg;
    if (step >= o->steps - avg) last += loss / avg;
  }
  if ((rc = check_err(c, n))) return rc;
  n->trained = true;
  prof_resolve(c);
  if (rep) {
    rep->steps = o->steps;
    rep->loss_first = first;
    rep->loss_last = last;
    rep->kappa = n->kappa;
    rep->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    rep->patch_h = ph;
    rep->patch_w = pw;
  }
  return EB_OK;
}

extern "C" int eb_learned_stats(eb_ctx* c, int64_t* accepted, int64_t* rejected, double* seconds,
                                double* mean_removed) {
  if (!c) return EB_BAD_INPUT;
  Net* n = c->net;
  const int64_t calls = n ? n->accepted + n->rejected : 0;
  if (accepted) *accepted = n ? n->accepted : 0;
  if (rejected) *rejected = n ? n->rejected : 0;
  if (seconds) *seconds = n ? n->seconds : 0.0;
  if (mean_removed) *mean_removed = calls ? n->removed / calls : 0.0;
  if (n) { n->accepted = 0; n->rejected = 0; n->seconds = 0.0; n->removed = 0.0; }
  return EB_OK;
}
