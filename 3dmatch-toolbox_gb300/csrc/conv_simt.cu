// FP32 CUDA-core convolution path (the drop-in form of the net) plus the
// layers every precision shares: conv1 (1 input channel) and 2^3 max-pool.
//
// Replaces Marvin's cuDNN calls (core/marvin.hpp:4639 cudnnConvolutionForward
// with CUDNN_CROSS_CORRELATION, :4656 cudnnAddTensor, :5486 ReLU in place,
// :5580 max-pool).  Activations are channels-last, [B][D][D][D][C] float.
#include "common.cuh"
#include "internal.h"

namespace tdm {
namespace {

// conv1: 1 -> 64 channels, 30^3 -> 28^3, bias + ReLU.  Thread = (4
// consecutive x positions, group of 16 channels): per tap, 16 weights read
// from shared memory as float4 feed 64 FMAs.  Weights [27][64] in shared memory.
template <bool BF16_OUT>
__global__ __launch_bounds__(256) void conv1_kernel(const float* __restrict__ patches, int64_t n_quads,
                                                    const float* __restrict__ w, const float* __restrict__ bias,
                                                    void* __restrict__ out, int64_t out_cs) {
  __shared__ __align__(16) float sw[27 * 64];
  __shared__ float sb[64];
  for (int i = threadIdx.x; i < 27 * 64; i += 256) sw[i] = w[i];
  if (threadIdx.x < 64) sb[threadIdx.x] = bias[threadIdx.x];
  __syncthreads();
  const int64_t q = (int64_t)blockIdx.x * 64 + threadIdx.x / 4;  // x-quad index
  const int g = threadIdx.x & 3;
  if (q >= n_quads) return;
  const int64_t b = q / 5488;  // 28 * 28 * 7 quads per patch
  const int r = (int)(q - b * 5488);
  const int z = r / 196, y = (r / 7) % 28, x0 = (r % 7) * 4;
  const float* p = patches + b * 27000 + z * 900 + y * 30 + x0;
  float acc[4][16];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int k = 0; k < 16; ++k) acc[i][k] = sb[g * 16 + k];
#pragma unroll
  for (int zy = 0; zy < 9; ++zy) {
    const float* row = p + (zy / 3) * 900 + (zy % 3) * 30;
    float v[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) v[j] = __ldg(row + j);
#pragma unroll
    for (int dx = 0; dx < 3; ++dx) {
      const float4* wt = reinterpret_cast<const float4*>(sw + (zy * 3 + dx) * 64 + g * 16);
      float wk[16];
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        float4 t = wt[h];
        wk[4 * h] = t.x; wk[4 * h + 1] = t.y; wk[4 * h + 2] = t.z; wk[4 * h + 3] = t.w;
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 16; ++k) acc[i][k] = fmaf(v[i + dx], wk[k], acc[i][k]);
    }
  }
  const int64_t pos0 = b * 21952 + (int64_t)(z * 28 + y) * 28 + x0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) acc[i][k] = fmaxf(acc[i][k], 0.0f);
    const int64_t pos = pos0 + i;
    if (BF16_OUT) {
      // chunk-planar layout: chunk j at out + j*out_cs, row pos at +pos*16
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        __nv_bfloat162 t[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) t[e] = __floats2bfloat162_rn(acc[i][8 * h + 2 * e], acc[i][8 * h + 2 * e + 1]);
        uint8_t* dst = static_cast<uint8_t*>(out) + (int64_t)(2 * g + h) * out_cs + pos * 16;
        *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<uint4*>(t);
      }
    } else {
      float4* dst = reinterpret_cast<float4*>(static_cast<float*>(out) + pos * 64 + g * 16);
#pragma unroll
      for (int h = 0; h < 4; ++h)
        dst[h] = make_float4(acc[i][4 * h], acc[i][4 * h + 1], acc[i][4 * h + 2], acc[i][4 * h + 3]);
    }
  }
}

// Implicit-GEMM convolution on CUDA cores: M = B*Do^3 output positions,
// N = K output channels, K-loop over taps x input channels (BK = 16 channels of
// one tap per step).  Weights are [T*C][K] (row = tap*C + c).  Tile 128 x BN,
// 256 threads, each 8 x BN/16 accumulators, double-buffered shared memory.
template <int BN>
__global__ __launch_bounds__(256) void conv_f32_kernel(const float* __restrict__ in, int D, int C, int ks,
                                                       const float* __restrict__ w, const float* __restrict__ bias,
                                                       int K, int relu, int64_t M, int Do, float* __restrict__ out) {
  constexpr int BM = 128, BK = 16, TN = BN / 16, NB4 = BN / 64;
  __shared__ __align__(16) float As[2][BK][BM + 4];
  __shared__ __align__(16) float Bs[2][BK][BN];
  const int tid = threadIdx.x;
  const int64_t m0 = (int64_t)blockIdx.x * BM;
  const int n0 = blockIdx.y * BN;
  const int lq = tid & 3;
  const int64_t Do3 = (int64_t)Do * Do * Do;
  int64_t base[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    int64_t m = m0 + (tid >> 2) + 64 * h;
    if (m >= M) m = M - 1;
    int64_t b = m / Do3;
    int r = (int)(m - b * Do3);
    int z = r / (Do * Do), y = (r / Do) % Do, x = r % Do;
    base[h] = (((b * D + z) * D + y) * D + x) * (int64_t)C + lq * 4;
  }
  const int csteps = C / BK;
  const int ksteps = ks * ks * ks * csteps;
  float4 ra[2], rb[NB4];
  auto load = [&](int s) {
    int t = s / csteps, c0 = (s - t * csteps) * BK;
    int tz = t / (ks * ks), ty = (t / ks) % ks, tx = t % ks;
    int64_t toff = ((int64_t)(tz * D + ty) * D + tx) * C + c0;
    ra[0] = __ldg(reinterpret_cast<const float4*>(in + base[0] + toff));
    ra[1] = __ldg(reinterpret_cast<const float4*>(in + base[1] + toff));
    int64_t krow = (int64_t)t * C + c0;
#pragma unroll
    for (int h = 0; h < NB4; ++h) {
      int idx = tid + h * 256, r = idx / (BN / 4), c4 = idx % (BN / 4);
      rb[h] = __ldg(reinterpret_cast<const float4*>(w + (krow + r) * K + n0 + c4 * 4));
    }
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      int row = (tid >> 2) + 64 * h;
      As[buf][lq * 4 + 0][row] = ra[h].x;
      As[buf][lq * 4 + 1][row] = ra[h].y;
      As[buf][lq * 4 + 2][row] = ra[h].z;
      As[buf][lq * 4 + 3][row] = ra[h].w;
    }
#pragma unroll
    for (int h = 0; h < NB4; ++h) {
      int idx = tid + h * 256, r = idx / (BN / 4), c4 = idx % (BN / 4);
      *reinterpret_cast<float4*>(&Bs[buf][r][c4 * 4]) = rb[h];
    }
  };
  float acc[8][TN];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = 0.0f;
  load(0);
  store(0);
  __syncthreads();
  const int ty = tid >> 4, tx = tid & 15;
  for (int s = 0; s < ksteps; ++s) {
    const int cur = s & 1;
    if (s + 1 < ksteps) load(s + 1);
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      float4 a0 = *reinterpret_cast<const float4*>(&As[cur][k][ty * 4]);
      float4 a1 = *reinterpret_cast<const float4*>(&As[cur][k][64 + ty * 4]);
      float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      float bb[TN];
#pragma unroll
      for (int h = 0; h < TN / 4; ++h) {
        float4 b4 = *reinterpret_cast<const float4*>(&Bs[cur][k][h * 64 + tx * 4]);
        bb[4 * h] = b4.x; bb[4 * h + 1] = b4.y; bb[4 * h + 2] = b4.z; bb[4 * h + 3] = b4.w;
      }
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fmaf(a[i], bb[j], acc[i][j]);
    }
    if (s + 1 < ksteps) store(cur ^ 1);
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    int64_t m = m0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + i - 4);
    if (m >= M) continue;
#pragma unroll
    for (int h = 0; h < TN / 4; ++h) {
      int n = n0 + h * 64 + tx * 4;
      float4 v;
      v.x = acc[i][4 * h + 0] + __ldg(bias + n + 0);
      v.y = acc[i][4 * h + 1] + __ldg(bias + n + 1);
      v.z = acc[i][4 * h + 2] + __ldg(bias + n + 2);
      v.w = acc[i][4 * h + 3] + __ldg(bias + n + 3);
      if (relu) {
        v.x = fmaxf(v.x, 0.0f); v.y = fmaxf(v.y, 0.0f); v.z = fmaxf(v.z, 0.0f); v.w = fmaxf(v.w, 0.0f);
      }
      *reinterpret_cast<float4*>(out + m * K + n) = v;
    }
  }
}

// 2^3 max-pool, stride 2, channels-last float.  Thread = (position, 4 channels).
__global__ __launch_bounds__(256) void pool_f32_kernel(const float* __restrict__ in, int D, int C, int64_t n_out,
                                                       float* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x;
  const int c4n = C / 4;
  if (i >= n_out * c4n) return;
  int c4 = (int)(i % c4n);
  int64_t q = i / c4n;
  const int Do = D / 2;
  const int64_t Do3 = (int64_t)Do * Do * Do;
  int64_t b = q / Do3;
  int r = (int)(q - b * Do3);
  int z = r / (Do * Do), y = (r / Do) % Do, x = r % Do;
  float4 best = make_float4(-INFINITY, -INFINITY, -INFINITY, -INFINITY);
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    int zz = 2 * z + (t >> 2), yy = 2 * y + ((t >> 1) & 1), xx = 2 * x + (t & 1);
    float4 v = __ldg(reinterpret_cast<const float4*>(in + (((b * D + zz) * D + yy) * D + xx) * (int64_t)C) + c4);
    best.x = fmaxf(best.x, v.x); best.y = fmaxf(best.y, v.y); best.z = fmaxf(best.z, v.z); best.w = fmaxf(best.w, v.w);
  }
  reinterpret_cast<float4*>(out + q * C)[c4] = best;
}

// Same pool on the BF16 chunk-planar layout (8 channels per 16-byte row).
// XP: the input is already max-pooled along x (x extent D/2, written so by
// the dx-fused conv2), so only the four (z, y) taps remain; ZP (with XP):
// also along z (the CTA-pair conv2), so only the two y taps remain.
template <bool XP, bool ZP = false>
__global__ __launch_bounds__(256) void pool_c8_kernel(const uint8_t* __restrict__ in, int64_t in_cs, int D,
                                                      int nchunks, int64_t n_out, uint8_t* __restrict__ out,
                                                      int64_t out_cs) {
  int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x;
  if (i >= n_out * nchunks) return;
  int j = (int)(i / n_out);
  int64_t q = i - (int64_t)j * n_out;
  const int Do = D / 2, XW = XP ? Do : D;
  const int64_t Do3 = (int64_t)Do * Do * Do;
  int64_t b = q / Do3;
  int r = (int)(q - b * Do3);
  int z = r / (Do * Do), y = (r / Do) % Do, x = r % Do;
  __nv_bfloat162 best[4];
  const uint8_t* src = in + (int64_t)j * in_cs;
  constexpr int TAPS = ZP ? 2 : XP ? 4 : 8;
  const int ZW = ZP ? Do : D;
#pragma unroll
  for (int t = 0; t < TAPS; ++t) {
    const int zz = ZP ? z : XP ? 2 * z + (t >> 1) : 2 * z + (t >> 2);
    const int yy = ZP ? 2 * y + t : XP ? 2 * y + (t & 1) : 2 * y + ((t >> 1) & 1);
    const int xx = XP ? x : 2 * x + (t & 1);
    uint4 v = __ldg(reinterpret_cast<const uint4*>(src + (((b * ZW + zz) * D + yy) * XW + xx) * 16));
    __nv_bfloat162 e[4];
    memcpy(e, &v, 16);
#pragma unroll
    for (int h = 0; h < 4; ++h) best[h] = t == 0 ? e[h] : __hmax2(best[h], e[h]);
  }
  uint4 o;
  memcpy(&o, best, 16);
  *reinterpret_cast<uint4*>(out + (int64_t)j * out_cs + q * 16) = o;
}

// Same pool on the E4M3 chunk-planar layout (16 channels per 16-byte row).
// Inputs are ReLU outputs (>= 0), whose E4M3 bytes order like the values, so
// a byte-wise unsigned max is the max-pool.
template <bool XP, bool ZP = false>
__global__ __launch_bounds__(256) void pool_c16_u8_kernel(const uint8_t* __restrict__ in, int64_t in_cs, int D,
                                                          int nchunks, int64_t n_out, uint8_t* __restrict__ out,
                                                          int64_t out_cs) {
  int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x;
  if (i >= n_out * nchunks) return;
  int j = (int)(i / n_out);
  int64_t q = i - (int64_t)j * n_out;
  const int Do = D / 2, XW = XP ? Do : D;
  const int64_t Do3 = (int64_t)Do * Do * Do;
  int64_t b = q / Do3;
  int r = (int)(q - b * Do3);
  int z = r / (Do * Do), y = (r / Do) % Do, x = r % Do;
  const uint8_t* src = in + (int64_t)j * in_cs;
  uint4 best = make_uint4(0, 0, 0, 0);
  constexpr int TAPS = ZP ? 2 : XP ? 4 : 8;
  const int ZW = ZP ? Do : D;
#pragma unroll
  for (int t = 0; t < TAPS; ++t) {
    const int zz = ZP ? z : XP ? 2 * z + (t >> 1) : 2 * z + (t >> 2);
    const int yy = ZP ? 2 * y + t : XP ? 2 * y + (t & 1) : 2 * y + ((t >> 1) & 1);
    const int xx = XP ? x : 2 * x + (t & 1);
    uint4 v = __ldg(reinterpret_cast<const uint4*>(src + (((b * ZW + zz) * D + yy) * XW + xx) * 16));
    best.x = __vmaxu4(best.x, v.x);
    best.y = __vmaxu4(best.y, v.y);
    best.z = __vmaxu4(best.z, v.z);
    best.w = __vmaxu4(best.w, v.w);
  }
  *reinterpret_cast<uint4*>(out + (int64_t)j * out_cs + q * 16) = best;
}

}  // namespace

tdm_status launch_pool_c16_u8(const uint8_t* in, int64_t in_cs, int B, int D, int nchunks, uint8_t* out,
                              int64_t out_cs, cudaStream_t s, bool x_pooled, bool z_pooled) {
  int Do = D / 2;
  int64_t n_out = (int64_t)B * Do * Do * Do;
  int64_t n = n_out * nchunks;
  TDM_REQUIRE(!z_pooled || x_pooled, "pool: a z-pooled input is x-pooled too");
  if (z_pooled)
    pool_c16_u8_kernel<true, true><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, in_cs, D, nchunks, n_out, out, out_cs);
  else if (x_pooled)
    pool_c16_u8_kernel<true><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, in_cs, D, nchunks, n_out, out, out_cs);
  else
    pool_c16_u8_kernel<false><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, in_cs, D, nchunks, n_out, out, out_cs);
  TDM_CHECK_LAUNCH("pool_c16_u8_kernel");
  return TDM_OK;
}

tdm_status launch_conv1(const float* patches, int B, const float* w, const float* bias, bool bf16_out, void* out,
                        int64_t out_cs, cudaStream_t s) {
  int64_t n_quads = (int64_t)B * 5488;
  unsigned blocks = (unsigned)((n_quads + 63) / 64);
  if (bf16_out) conv1_kernel<true><<<blocks, 256, 0, s>>>(patches, n_quads, w, bias, out, out_cs);
  else conv1_kernel<false><<<blocks, 256, 0, s>>>(patches, n_quads, w, bias, out, out_cs);
  TDM_CHECK_LAUNCH("conv1_kernel");
  return TDM_OK;
}

tdm_status launch_conv_f32(const float* in, int B, int D, int C, int ks, const float* w, const float* bias, int K,
                           bool relu, float* out, cudaStream_t s) {
  TDM_REQUIRE(C % 16 == 0 && K % 64 == 0, "conv_f32: C must be a multiple of 16 and K of 64");
  int Do = D - ks + 1;
  int64_t M = (int64_t)B * Do * Do * Do;
  if (K % 128 == 0) {
    dim3 grid((unsigned)((M + 127) / 128), K / 128);
    conv_f32_kernel<128><<<grid, 256, 0, s>>>(in, D, C, ks, w, bias, K, relu ? 1 : 0, M, Do, out);
  } else {
    dim3 grid((unsigned)((M + 127) / 128), K / 64);
    conv_f32_kernel<64><<<grid, 256, 0, s>>>(in, D, C, ks, w, bias, K, relu ? 1 : 0, M, Do, out);
  }
  TDM_CHECK_LAUNCH("conv_f32_kernel");
  return TDM_OK;
}

tdm_status launch_pool_f32(const float* in, int B, int D, int C, float* out, cudaStream_t s) {
  int Do = D / 2;
  int64_t n_out = (int64_t)B * Do * Do * Do;
  int64_t n = n_out * (C / 4);
  pool_f32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, D, C, n_out, out);
  TDM_CHECK_LAUNCH("pool_f32_kernel");
  return TDM_OK;
}

tdm_status launch_pool_c8(const uint8_t* in, int64_t in_cs, int B, int D, int nchunks, uint8_t* out, int64_t out_cs,
                          cudaStream_t s, bool x_pooled, bool z_pooled) {
  int Do = D / 2;
  int64_t n_out = (int64_t)B * Do * Do * Do;
  int64_t n = n_out * nchunks;
  TDM_REQUIRE(!z_pooled || x_pooled, "pool: a z-pooled input is x-pooled too");
  if (z_pooled)
    pool_c8_kernel<true, true><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, in_cs, D, nchunks, n_out, out, out_cs);
  else if (x_pooled)
    pool_c8_kernel<true><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, in_cs, D, nchunks, n_out, out, out_cs);
  else
    pool_c8_kernel<false><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, in_cs, D, nchunks, n_out, out, out_cs);
  TDM_CHECK_LAUNCH("pool_c8_kernel");
  return TDM_OK;
}

}  // namespace tdm
