// The 3DMatch descriptor net (core/3dmatch-net-test.json): conv1..conv8 3x3x3
// valid convolutions with ReLU, 2^3 max-pool after conv2, then `feat`, a
// 1x1x1 512->512 convolution without ReLU.  30^3 TDF patch -> 512-d.
//
// Replaces marvin::Net as demo.cu drives it (core/demo.cu:179-231): weights
// are found by layer name in a .marvin file (Layer::setWeights,
// core/marvin.hpp:3321-3370), buffers are owned by the handle, and forward
// runs the layer sequence.  Precisions:
//   FP32: CUDA-core implicit GEMM for every layer (the drop-in form).
//   BF16: conv1 on CUDA cores (K = 27), conv2..feat on tcgen05 with BF16
//         operands, FP32 accumulation, BF16 activations between layers.
#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "marvin_io.h"

#include <cuda_fp8.h>

using namespace tdm;

namespace {
const char* kNames[9] = {"conv1", "conv2", "conv3", "conv4", "conv5", "conv6", "conv7", "conv8", "feat"};
const int kCout[9] = {64, 64, 128, 128, 256, 256, 512, 512, 512};
const int kCin[9] = {1, 64, 64, 128, 128, 256, 256, 512, 512};
const int kKs[9] = {3, 3, 3, 3, 3, 3, 3, 3, 1};
const int kDin[9] = {30, 28, 13, 11, 9, 7, 5, 3, 1};  // input extent of each layer (pool after conv2)
constexpr int kDefaultMaxBatch = 2048;
// Response ids: layer index 0..8 (conv1..conv8, feat) = that layer's output
// (after its in-place ReLU); kPool = pool1.  -1 = the full forward.
constexpr int kPool = 100;
// timed layer ids: 0..8 = conv1..feat, 9 = pool1
constexpr int kTimedLayers = 10;

// Chunk-planar BF16 -> channels-last float (responses of the BF16 form).
// taps_layout: rows are patches and chunk = tap*(C/8) + c/8 (conv7's output).
__global__ void c8_to_f32_kernel(const uint8_t* __restrict__ in, int64_t cs, int64_t npos, int C, int taps_layout,
                                 int ntaps, float* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npos * C) return;
  int c = (int)(i % C);
  int64_t p = i / C;
  int64_t chunk, row;
  if (taps_layout) {
    int64_t b = p / ntaps;
    int t = (int)(p - b * ntaps);
    chunk = (int64_t)t * (C / 8) + c / 8;
    row = b;
  } else {
    chunk = c / 8;
    row = p;
  }
  __nv_bfloat16 v = *reinterpret_cast<const __nv_bfloat16*>(in + chunk * cs + row * 16 + (c % 8) * 2);
  out[i] = __bfloat162float(v);
}
// Chunk-planar E4M3 (16 channels per 16-byte row) -> float, times `scale`.
__global__ void c16_to_f32_kernel(const uint8_t* __restrict__ in, int64_t cs, int64_t npos, int C, int taps_layout,
                                  int ntaps, float scale, float* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npos * C) return;
  int c = (int)(i % C);
  int64_t p = i / C;
  int64_t chunk, row;
  if (taps_layout) {
    int64_t b = p / ntaps;
    int t = (int)(p - b * ntaps);
    chunk = (int64_t)t * (C / 16) + c / 16;
    row = b;
  } else {
    chunk = c / 16;
    row = p;
  }
  __nv_fp8_e4m3 v;
  v.__x = in[chunk * cs + row * 16 + (c % 16)];
  out[i] = (float)v * scale;
}

// max over non-negative floats (ReLU responses) for FP8 calibration
__global__ void amax_kernel(const float* __restrict__ x, int64_t n, unsigned int* __restrict__ out) {
  float m = 0.0f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, x[i]);
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}
}  // namespace

struct tdm_net {
  tdm_precision prec = TDM_FP32;
  int use_feat = 1;
  int device = 0;
  std::vector<float> hw[9], hb[9];  // Marvin layout: [K][C][taps], [K]
  float* d_b[9] = {};
  float* d_w1 = nullptr;  // conv1 [27][64]
  float* d_w32[9] = {};   // FP32 path: [taps*C][K]
  TcLayer tc[9];          // BF16 tcgen05 layers (conv1 GEMM at 0, conv2..feat at 1..8)
  TcLayer tc8[9];         // FP8 form: conv2 (BF16 in, E4M3 out) at 1, conv3..conv8 (E4M3 in) at 2..7
  float act_scale[9] = {};  // FP8 form: dequantisation scale of the E4M3 input of layer l (2..7)
  bool calibrated = false;
  std::vector<void*> allocs;
  // packed tcgen05 weights per (form, layer, N tile), filled as tiles change
  std::map<int, uint8_t*> packed;
  uint8_t* ws = nullptr;
  size_t ws_bytes = 0;
  // bumped whenever a buffer or tile a captured forward refers to changes
  uint64_t generation = 0;
  int max_batch = kDefaultMaxBatch;
  // optional per-layer timing: CUDA events recorded on the launching stream
  bool timing = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pool;
  std::vector<std::pair<int, size_t>> ev_pending;  // (layer id, pool slot)
  double layer_ms[kTimedLayers] = {};
  int64_t layer_n[kTimedLayers] = {};

  ~tdm_net() {
    for (void* p : allocs) cudaFree(p);
    if (ws) cudaFree(ws);
    for (auto& e : ev_pool) {
      cudaEventDestroy(e.first);
      cudaEventDestroy(e.second);
    }
  }
  // Folds recorded event pairs into the per-layer totals (synchronizes).
  cudaError_t drain() {
    for (auto& pe : ev_pending) {
      auto& e = ev_pool[pe.second];
      cudaError_t r = cudaEventSynchronize(e.second);
      if (r != cudaSuccess) return r;
      float t = 0.0f;
      r = cudaEventElapsedTime(&t, e.first, e.second);
      if (r != cudaSuccess) return r;
      layer_ms[pe.first] += t;
      layer_n[pe.first] += 1;
    }
    ev_pending.clear();
    return cudaSuccess;
  }
  // Brackets one layer launch with events when timing is on.
  cudaEvent_t begin(int id, cudaStream_t s) {
    if (!timing) return nullptr;
    if (ev_pending.size() >= 1024 && drain() != cudaSuccess) return nullptr;
    size_t slot = ev_pending.size();
    if (slot >= ev_pool.size()) {
      cudaEvent_t a, b;
      if (cudaEventCreate(&a) != cudaSuccess) return nullptr;
      if (cudaEventCreate(&b) != cudaSuccess) { cudaEventDestroy(a); return nullptr; }
      ev_pool.emplace_back(a, b);
    }
    ev_pending.emplace_back(id, slot);
    cudaEventRecord(ev_pool[slot].first, s);
    return ev_pool[slot].second;
  }
  void end(cudaEvent_t e, cudaStream_t s) {
    if (e) cudaEventRecord(e, s);
  }
  template <typename T>
  tdm_status upload(const T* h, size_t n, T** d) {
    void* p = nullptr;
    TDM_CHECK_CUDA(cudaMalloc(&p, n * sizeof(T)));
    allocs.push_back(p);
    TDM_CHECK_CUDA(cudaMemcpy(p, h, n * sizeof(T), cudaMemcpyHostToDevice));
    *d = static_cast<T*>(p);
    return TDM_OK;
  }
};

namespace {

int64_t round16(int64_t x) { return (x + 15) & ~(int64_t)15; }

constexpr int kConv8Splits = 4;  // conv8's K splits (divides its 216 BF16 / 108 E4M3 K groups)

TcLayer make_tc_layer(int l, bool use_feat) {
  TcLayer L{};
  L.cin = kCin[l];
  L.cout = kCout[l];
  L.relu = l < 8 ? 1 : 0;
  L.fp8_in = L.fp8_out = false;
  if (l <= 6) {  // 3x3x3 conv on a grid
    L.D = kDin[l];
    L.Do = L.D - 2;
    L.nz = 3;
    L.nyx = 9;
    L.kgroups = L.cin / 64;
    L.out_mode = l == 6 ? TC_OUT_C8_TAPS : TC_OUT_C8_CONV;
  } else {  // conv8 (K = 27*512, flattened) and feat (K = 512) as GEMMs over patches
    L.D = 1;
    L.Do = 1;
    L.nz = 1;
    L.nyx = 1;
    L.kgroups = (l == 7 ? 27 * 512 : 512) / 64;
    L.out_mode = (l == 7 && use_feat) ? TC_OUT_C8_ROWS : TC_OUT_F32_ROWS;
    L.ksplit = l == 7 ? kConv8Splits : 1;  // conv8: K = 13,824 over only cout/nt x rows/128 tiles
  }
  // N tile and M sub-tiles per CTA; two accumulator buffers of msub*nt TMEM
  // columns each must fit in 512 columns.
  if (L.cout == 64) { L.nt = 64; L.msub = 4; }
  else if (L.cout == 128) { L.nt = 128; L.msub = 2; }
  else { L.nt = 256; L.msub = 1; }
  if (l == 1) {  // conv2: the dx taps share one MMA; a CTA pair covers both halves of the outputs
    L.dxf = true;
    L.pair = true;
    L.nt = 32;
    L.msub = 2;
  }
  if (l >= 2 && l <= 6) {  // conv3..conv7: M over the valid output positions (conv3..conv6: whole x runs)
    L.gather = true;
    L.xrun = l <= 5;
    L.wt = L.cout == 128;  // conv3, conv4: weights as the MMA's A operand
    L.nt = L.cout == 128 ? 128 : 256;
    L.msub = 2;
  }
  return L;
}

tdm_status setup_weights(tdm_net* net) {
  // biases and conv1 (all precisions)
  for (int l = 0; l < 9; ++l) {
    tdm_status st = net->upload(net->hb[l].data(), net->hb[l].size(), &net->d_b[l]);
    if (st != TDM_OK) return st;
  }
  std::vector<float> w1(27 * 64);
  for (int k = 0; k < 64; ++k)
    for (int t = 0; t < 27; ++t) w1[t * 64 + k] = net->hw[0][k * 27 + t];
  tdm_status st = net->upload(w1.data(), w1.size(), &net->d_w1);
  if (st != TDM_OK) return st;
  if (net->prec == TDM_FP32) {
    for (int l = 1; l < 9; ++l) {
      int K = kCout[l], C = kCin[l], T = kKs[l] * kKs[l] * kKs[l];
      std::vector<float> wt((size_t)T * C * K);
      for (int k = 0; k < K; ++k)
        for (int c = 0; c < C; ++c)
          for (int t = 0; t < T; ++t) wt[((size_t)t * C + c) * K + k] = net->hw[l][((size_t)k * C + c) * T + t];
      st = net->upload(wt.data(), wt.size(), &net->d_w32[l]);
      if (st != TDM_OK) return st;
    }
    return TDM_OK;
  }
  if (net->prec == TDM_BF16 || net->prec == TDM_FP8) {
    // conv1 on the tensor cores: a GEMM over output positions with K = 27
    // taps padded to 32 (im2col operand), N = 64.
    {
      TcLayer L{};
      L.cin = 32;
      L.cout = 64;
      L.D = L.Do = 1;
      L.nz = L.nyx = 1;
      L.kgroups = 1;
      L.nt = 64;
      L.msub = 4;
      L.out_mode = TC_OUT_C8_ROWS;
      L.relu = 1;
      std::vector<uint8_t> pk((size_t)4 * 64 * 16, 0);
      for (int j = 0; j < 4; ++j)
        for (int n = 0; n < 64; ++n)
          for (int e = 0; e < 8; ++e) {
            int t = 8 * j + e;
            __nv_bfloat16 h = __float2bfloat16_rn(t < 27 ? net->hw[0][(size_t)n * 27 + t] : 0.0f);
            std::memcpy(&pk[((size_t)j * 64 + n) * 16 + 2 * e], &h, 2);
          }
      st = net->upload(pk.data(), pk.size(), &L.wpk);
      if (st != TDM_OK) return st;
      L.bias = net->d_b[0];
      net->tc[0] = L;
    }
    for (int l = 1; l < 9; ++l) {
      TcLayer L = make_tc_layer(l, net->use_feat != 0);
      std::vector<uint8_t> pk;
      std::vector<float> sc;
      if (L.dxf) pack_dxf_weights(L, net->hw[l].data(), &pk);
      else pack_tc_weights(L, net->hw[l].data(), l == 7 ? 27 : 1, &pk, &sc);
      st = net->upload(pk.data(), pk.size(), &L.wpk);
      if (st != TDM_OK) return st;
      L.bias = net->d_b[l];
      L.wscale = nullptr;
      net->tc[l] = L;
    }
    if (net->prec == TDM_BF16) return TDM_OK;
    // FP8 form: conv2 keeps BF16 operands but writes E4M3; conv3..conv8 take
    // E4M3 operands with per-output-channel weight scales.
    net->tc8[1] = net->tc[1];
    net->tc8[1].fp8_out = true;
    for (int l = 2; l < 8; ++l) {
      TcLayer L = make_tc_layer(l, net->use_feat != 0);
      L.fp8_in = true;
      L.fp8_out = l < 7;
      const int k_total = l <= 6 ? kCin[l] : 27 * 512;  // K elements per tap (conv) or in total (conv8)
      const int chunks = k_total / 16;
      L.kgroups = chunks < 8 ? 1 : chunks / 8;
      std::vector<uint8_t> pk;
      std::vector<float> sc;
      pack_tc_weights(L, net->hw[l].data(), l == 7 ? 27 : 1, &pk, &sc);
      st = net->upload(pk.data(), pk.size(), &L.wpk);
      if (st != TDM_OK) return st;
      st = net->upload(sc.data(), sc.size(), &L.wscale);
      if (st != TDM_OK) return st;
      L.bias = net->d_b[l];
      net->tc8[l] = L;
    }
    net->tc8[8] = net->tc[8];
    return TDM_OK;
  }
  return fail(TDM_ERR_UNSUPPORTED, "unknown precision");
}

tdm_status create_common(tdm_net* net, tdm_precision prec, int32_t use_feat) {
  net->prec = prec;
  net->use_feat = use_feat ? 1 : 0;
  TDM_CHECK_CUDA(cudaGetDevice(&net->device));
  return setup_weights(net);
}

// ---------------------------------------------------------------------------
// FP32 forward of one chunk: buffers hold channels-last float activations.
// ---------------------------------------------------------------------------
// Output extent and channels of each response.
void response_shape(int id, int* D, int* C) {
  static const int Dout[9] = {28, 26, 11, 9, 7, 5, 3, 1, 1};
  if (id == kPool) { *D = 13; *C = 64; return; }
  *D = Dout[id];
  *C = kCout[id];
}

tdm_status copy_response_f32(const float* src, int B, int id, float* out, cudaStream_t s) {
  int D, C;
  response_shape(id, &D, &C);
  TDM_CHECK_CUDA(cudaMemcpyAsync(out, src, sizeof(float) * (size_t)B * D * D * D * C, cudaMemcpyDeviceToDevice, s));
  return TDM_OK;
}

tdm_status forward_f32(tdm_net* net, const float* patches, int B, float* desc, int stop, cudaStream_t s) {
  float* b0 = reinterpret_cast<float*>(net->ws);
  float* b1 = b0 + (size_t)B * 1404928;  // 28^3 * 64
  cudaEvent_t ev = net->begin(0, s);
  tdm_status st = launch_conv1(patches, B, net->d_w1, net->d_b[0], false, b0, 0, s);
  net->end(ev, s);
  if (st) return st;
  if (stop == 0) return copy_response_f32(b0, B, 0, desc, s);
  float* in = b0;
  float* out = b1;
  for (int l = 1; l < 9; ++l) {
    if (l == 8 && !net->use_feat) break;
    bool last = stop < 0 && ((l == 8) || (l == 7 && !net->use_feat));
    float* dst = last ? desc : out;
    ev = net->begin(l, s);
    st = launch_conv_f32(in, B, kDin[l], kCin[l], kKs[l], net->d_w32[l], net->d_b[l], kCout[l], l < 8, dst, s);
    net->end(ev, s);
    if (st) return st;
    if (stop == l) return copy_response_f32(dst, B, l, desc, s);
    if (l == 1) {  // 2^3 max-pool after conv2 (26^3 -> 13^3)
      ev = net->begin(9, s);
      st = launch_pool_f32(dst, B, 26, 64, in, s);
      net->end(ev, s);
      if (st) return st;
      if (stop == kPool) return copy_response_f32(in, B, kPool, desc, s);
      continue;  // pooled result is back in `in`
    }
    std::swap(in, out);
  }
  return TDM_OK;
}

size_t f32_ws_bytes(int B) { return (size_t)B * (1404928 + 1124864) * sizeof(float); }

// ---------------------------------------------------------------------------
// BF16 forward of one chunk (chunk-planar BF16 activations).
// ---------------------------------------------------------------------------
struct Bf16Plan {
  int64_t rows_alloc[9];  // rows allocated per chunk for the input of layer l
  int64_t rows[9];        // live rows of the input of layer l
  size_t off1;            // byte offset of buffer 1
  size_t off_part;        // conv8's split-K partial sums
  size_t total;
};

Bf16Plan bf16_plan(const tdm_net* net, int B) {
  Bf16Plan P{};
  // inputs: l=1 conv2 (28^3), pool input (26^3) handled separately, l=2 conv3 (13^3) ...
  for (int l = 1; l < 9; ++l) {
    int64_t rows = l <= 6 ? (int64_t)B * kDin[l] * kDin[l] * kDin[l] : B;
    P.rows[l] = rows;
    int64_t tail = tc_tail_rows(net->tc[l]);
    if (net->prec == TDM_FP8 && l <= 7) tail = std::max(tail, tc_tail_rows(net->tc8[l]));
    P.rows_alloc[l] = rows + tail;
  }
  // buffer 0 holds inputs of l = 1, 2(pooled), 4, 6, 8; buffer 1: conv2 output (pool input), 3, 5, 7
  auto chunks = [](int l) { return kCin[l] / 8; };
  size_t b0 = 0, b1 = 0;
  for (int l : {1, 2, 4, 6, 8}) b0 = std::max(b0, (size_t)(l == 7 ? 1728 : chunks(l)) * P.rows_alloc[l] * 16);
  // conv2 output (pre-pool, 26^3 rows per chunk); the CTA-pair form uses the
  // first quarter for x- and z-pooled rows and writes conv3's pooled input
  // (plus conv3's tail rows) after them
  b1 = std::max(b1, (size_t)8 * ((int64_t)B * 17576 + 8) * 16);
  for (int l : {3, 5}) b1 = std::max(b1, (size_t)chunks(l) * P.rows_alloc[l] * 16);
  b1 = std::max(b1, (size_t)1728 * P.rows_alloc[7] * 16);  // conv7 -> conv8 flattened operand
  P.off1 = round16((int64_t)b0) + 4096;
  P.off_part = P.off1 + round16((int64_t)b1) + 4096;
  P.total = P.off_part + (size_t)kConv8Splits * B * 512 * sizeof(float) + 4096;
  return P;
}

tdm_status c8_response(const uint8_t* src, int64_t cs, int B, int id, bool taps, float* out, cudaStream_t s) {
  int D, C;
  response_shape(id, &D, &C);
  int64_t npos = (int64_t)B * D * D * D;
  c8_to_f32_kernel<<<(unsigned)((npos * C + 255) / 256), 256, 0, s>>>(src, cs, npos, C, taps ? 1 : 0, D * D * D, out);
  TDM_CHECK_LAUNCH("c8_to_f32_kernel");
  return TDM_OK;
}

tdm_status c16_response(const uint8_t* src, int64_t cs, int B, int id, bool taps, float scale, float* out,
                        cudaStream_t s) {
  int D, C;
  response_shape(id, &D, &C);
  int64_t npos = (int64_t)B * D * D * D;
  c16_to_f32_kernel<<<(unsigned)((npos * C + 255) / 256), 256, 0, s>>>(src, cs, npos, C, taps ? 1 : 0, D * D * D,
                                                                        scale, out);
  TDM_CHECK_LAUNCH("c16_to_f32_kernel");
  return TDM_OK;
}

// Tensor-core forward of one chunk.  BF16 form: BF16 activations between all
// layers.  FP8 form (fp8 = true): conv2 writes E4M3, conv3..conv7 read and
// write E4M3 with per-tensor activation scales, conv8 reads E4M3 and writes
// BF16 for feat.
tdm_status forward_tc(tdm_net* net, const float* patches, int B, float* desc, int stop, bool fp8, cudaStream_t s) {
  Bf16Plan P = bf16_plan(net, B);
  uint8_t* b0 = net->ws;
  uint8_t* b1 = net->ws + P.off1;
  // conv1 on tcgen05, its im2col operand built in shared memory -> chunk-planar BF16 input of conv2
  int64_t cs = P.rows_alloc[1] * 16;
  cudaEvent_t ev = net->begin(0, s);
  tdm_status st = launch_conv1_tc(patches, B, net->tc[0], b0, cs, s);
  net->end(ev, s);
  if (st) return st;
  if (stop == 0) return c8_response(b0, cs, B, 0, false, desc, s);
  uint8_t* cur = b0;
  int64_t cur_cs = cs;
  for (int l = 1; l < 9; ++l) {
    if (l == 8 && !net->use_feat) break;
    const bool l_fp8 = fp8 && l <= 7;
    const TcLayer& L = l_fp8 ? net->tc8[l] : net->tc[l];
    bool last = (l == 8) || (l == 7 && !net->use_feat);
    uint8_t* dst = (cur == b0) ? b1 : b0;
    TcArgs a{};
    a.act = cur;
    a.act_cs = cur_cs;
    a.rows = P.rows[l];
    a.in_scale = L.fp8_in ? net->act_scale[l] : 1.0f;
    a.out_qinv = L.fp8_out ? 1.0f / net->act_scale[l + 1] : 1.0f;
    a.part = reinterpret_cast<float*>(net->ws + P.off_part);
    int64_t out_cs = 0;
    if (last) {
      a.out = reinterpret_cast<uint8_t*>(desc);
      a.out_cs = 0;
    } else if (l == 1) {
      out_cs = ((int64_t)B * 17576 + 8) * 16;  // conv2 output, read by the pool
      a.out = dst;
      a.out_cs = out_cs;
      // the epilogue takes the pool's x-pair max unless conv2's own response is wanted
      a.xpool = stop != 1 && L.dxf;
      // the CTA-pair form also takes the z-pair max (z extent 13) and, for y
      // pairs within one CTA, the y-pair max: the pooled rows (conv3's input)
      // go after the x- and z-pooled ones in conv2's output buffer, which is
      // sized for the unpooled 26^3 rows (conv2 still reads buffer 0 while it
      // writes them)
      a.zpool = a.xpool && tc_pair_form_applies(L, a.rows);
      if (a.zpool) {
        const int64_t xz_rows = ((int64_t)B * 13 * 26 * 13 + 15) / 16 * 16;
        a.out2 = dst + xz_rows * 16;
      }
    } else {
      out_cs = P.rows_alloc[l + 1] * 16;
      a.out = dst;
      a.out_cs = out_cs;
    }
    ev = net->begin(l, s);
    st = launch_tc_layer(L, a, s);
    net->end(ev, s);
    if (st) return st;
    if (last) break;
    if (stop == l) {
      const bool taps = L.out_mode == TC_OUT_C8_TAPS;
      if (L.fp8_out) return c16_response(dst, out_cs, B, l, taps, net->act_scale[l + 1], desc, s);
      return c8_response(dst, out_cs, B, l, taps, desc, s);
    }
    if (l == 1 && a.out2) {  // finish the y pairs that crossed CTA halves; conv3 reads a.out2
      ev = net->begin(9, s);
      st = launch_pool_ycross(L, dst, out_cs, B, a.out2, s);
      net->end(ev, s);
      if (st) return st;
      if (stop == kPool) {
        if (fp8) return c16_response(a.out2, out_cs, B, kPool, false, net->act_scale[2], desc, s);
        return c8_response(a.out2, out_cs, B, kPool, false, desc, s);
      }
      cur = a.out2;
      cur_cs = out_cs;
      continue;
    }
    if (l == 1) {  // pool 26^3 -> 13^3 back into buffer 0 as conv3's input
      int64_t pcs = P.rows_alloc[2] * 16;
      ev = net->begin(9, s);
      st = fp8 ? launch_pool_c16_u8(dst, out_cs, B, 26, 4, cur, pcs, s, a.xpool, a.zpool)
               : launch_pool_c8(dst, out_cs, B, 26, 8, cur, pcs, s, a.xpool, a.zpool);
      net->end(ev, s);
      if (st) return st;
      if (stop == kPool) {
        if (fp8) return c16_response(cur, pcs, B, kPool, false, net->act_scale[2], desc, s);
        return c8_response(cur, pcs, B, kPool, false, desc, s);
      }
      cur_cs = pcs;
      continue;
    }
    cur = dst;
    cur_cs = out_cs;
  }
  return TDM_OK;
}

// The zero fill runs on the caller's stream: a plain cudaMemset would be
// queued on the legacy stream, which a non-blocking caller stream does not
// wait for, and could land after the forward's first writes.
tdm_status ensure_ws(tdm_net* net, size_t bytes, cudaStream_t s) {
  if (net->ws_bytes >= bytes) return TDM_OK;
  if (net->ws) {
    TDM_CHECK_CUDA(cudaDeviceSynchronize());
    cudaFree(net->ws);
    net->ws = nullptr;
    net->ws_bytes = 0;
  }
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) return cuda_status(e, "net workspace");
  net->ws = static_cast<uint8_t*>(p);
  net->ws_bytes = 0;
  ++net->generation;
  TDM_CHECK_CUDA(cudaMemsetAsync(p, 0, bytes, s));
  net->ws_bytes = bytes;
  return TDM_OK;
}

tdm_status load_host_weights(tdm_net* net, const float* const* w, const float* const* b) {
  for (int l = 0; l < 9; ++l) {
    size_t n = (size_t)kCout[l] * kCin[l] * kKs[l] * kKs[l] * kKs[l];
    if (!w[l] || !b[l]) return fail(TDM_ERR_INVALID_ARG, std::string("missing weights for ") + kNames[l]);
    net->hw[l].assign(w[l], w[l] + n);
    net->hb[l].assign(b[l], b[l] + kCout[l]);
  }
  return TDM_OK;
}

}  // namespace

extern "C" tdm_status tdm_net_create_from_host(const float* const* w, const float* const* b, tdm_precision prec,
                                               int32_t use_feat, tdm_net** out) {
  TDM_REQUIRE(w && b && out, "tdm_net_create_from_host: null pointer");
  TDM_REQUIRE(prec == TDM_FP32 || prec == TDM_BF16 || prec == TDM_FP8, "tdm_net_create_from_host: bad precision");
  tdm_net* net = new tdm_net();
  tdm_status st = load_host_weights(net, w, b);
  if (st == TDM_OK) st = create_common(net, prec, use_feat);
  // cudaMemcpy from pageable memory may return before its DMA lands; the
  // handle is used next on streams that do not wait for the legacy stream
  if (st == TDM_OK && cudaDeviceSynchronize() != cudaSuccess) st = fail(TDM_ERR_DEVICE, "weight upload failed");
  if (st != TDM_OK) {
    delete net;
    return st;
  }
  *out = net;
  return TDM_OK;
}

extern "C" tdm_status tdm_net_create(const char* path, tdm_precision prec, int32_t use_feat, tdm_net** out) {
  TDM_REQUIRE(path && out, "tdm_net_create: null pointer");
  std::map<std::string, MarvinTensor> t;
  std::string err;
  tdm_status st = read_marvin(path, &t, &err);
  if (st != TDM_OK) return fail(st, err);
  const float* w[9];
  const float* b[9];
  for (int l = 0; l < 9; ++l) {
    auto iw = t.find(std::string(kNames[l]) + ".weight");
    auto ib = t.find(std::string(kNames[l]) + ".bias");
    if (iw == t.end() || ib == t.end()) return fail(TDM_ERR_FORMAT, std::string("weight file lacks ") + kNames[l]);
    size_t n = (size_t)kCout[l] * kCin[l] * kKs[l] * kKs[l] * kKs[l];
    if (iw->second.data.size() != n || ib->second.data.size() != (size_t)kCout[l])
      return fail(TDM_ERR_FORMAT, std::string("element count mismatch for ") + kNames[l]);
    w[l] = iw->second.data.data();
    b[l] = ib->second.data.data();
  }
  return tdm_net_create_from_host(w, b, prec, use_feat, out);
}

// form: the precision to run (an FP8 net can also run its BF16 form, which
// calibration uses).
static tdm_status net_run(tdm_net* net, const float* patches, int32_t b, float* out, int stop, tdm_stream s,
                          tdm_precision form) {
  if (b == 0) return TDM_OK;
  TDM_REQUIRE(patches && out, "tdm_net_forward: null pointer");
  TDM_REQUIRE(form != TDM_FP8 || net->calibrated,
              "FP8 net has no activation scales yet: call tdm_net_calibrate first");
  const int chunk = std::min<int>(b, net->max_batch);
  size_t need = net->prec == TDM_FP32 ? f32_ws_bytes(chunk) : bf16_plan(net, chunk).total;
  tdm_status st = ensure_ws(net, need, s);
  if (st) return st;
  size_t per = 512;
  if (stop >= 0) {
    int D, C;
    response_shape(stop, &D, &C);
    per = (size_t)D * D * D * C;
  }
  for (int i = 0; i < b; i += chunk) {
    int n = std::min(chunk, b - i);
    const float* p = patches + (size_t)i * 27000;
    float* d = out + (size_t)i * per;
    st = form == TDM_FP32 ? forward_f32(net, p, n, d, stop, s)
                          : forward_tc(net, p, n, d, stop, form == TDM_FP8, s);
    if (st) return st;
  }
  return TDM_OK;
}

extern "C" tdm_status tdm_net_forward(tdm_net* net, const float* patches, int32_t b, float* desc, tdm_stream s) {
  TDM_REQUIRE(net && b >= 0, "tdm_net_forward: bad arguments");
  return net_run(net, patches, b, desc, -1, s, net->prec);
}

extern "C" tdm_status tdm_net_response(tdm_net* net, const char* name, const float* patches, int32_t b, float* out,
                                       tdm_stream s) {
  TDM_REQUIRE(net && name && b >= 0, "tdm_net_response: bad arguments");
  std::string n(name);
  int id = -2;
  for (int l = 0; l < 9; ++l)
    if (n == kNames[l]) id = l;
  if (n == "pool1") id = kPool;
  TDM_REQUIRE(id != -2, "tdm_net_response: unknown response name");
  TDM_REQUIRE(!(id == 8 && !net->use_feat), "tdm_net_response: net built without feat");
  return net_run(net, patches, b, out, id, s, net->prec);
}

extern "C" tdm_status tdm_net_calibrate(tdm_net* net, const float* patches, int32_t b, tdm_stream s) {
  TDM_REQUIRE(net && patches && b > 0, "tdm_net_calibrate: bad arguments");
  if (net->prec != TDM_FP8) return TDM_OK;
  // Largest activation of conv2..conv7 over the calibration patches in the
  // BF16 form; the E4M3 scale maps it to 448 (the largest finite E4M3).
  int64_t maxn = (int64_t)b * 26 * 26 * 26 * 64;
  float* buf = nullptr;
  unsigned int* amax = nullptr;
  TDM_CHECK_CUDA(cudaMalloc(&buf, sizeof(float) * maxn));
  cudaError_t e = cudaMalloc(&amax, sizeof(unsigned int) * 8);
  if (e != cudaSuccess) {
    cudaFree(buf);
    return cuda_status(e, "calibration buffer");
  }
  tdm_status st = TDM_OK;
  for (int l = 1; l <= 6 && st == TDM_OK; ++l) {
    st = net_run(net, patches, b, buf, l, s, TDM_BF16);
    if (st) break;
    int D, C;
    response_shape(l, &D, &C);
    int64_t n = (int64_t)b * D * D * D * C;
    if (cudaMemsetAsync(amax + l, 0, sizeof(unsigned int), s) != cudaSuccess) { st = TDM_ERR_DEVICE; break; }
    amax_kernel<<<1216, 256, 0, s>>>(buf, n, amax + l);
    if (cudaGetLastError() != cudaSuccess) st = fail(TDM_ERR_DEVICE, "amax_kernel launch failed");
    note_launches(1);
  }
  unsigned int h[8] = {};
  if (st == TDM_OK) {
    e = cudaMemcpyAsync(h, amax, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = cuda_status(e, "calibration readback");
  }
  cudaFree(buf);
  cudaFree(amax);
  if (st) return st;
  for (int l = 1; l <= 6; ++l) {
    float m;
    std::memcpy(&m, &h[l], 4);
    net->act_scale[l + 1] = (m > 0.0f ? m : 1.0f) / 448.0f;
  }
  net->calibrated = true;
  return TDM_OK;
}

extern "C" tdm_status tdm_net_act_scales(tdm_net* net, float* scales) {
  TDM_REQUIRE(net && scales, "tdm_net_act_scales: null pointer");
  for (int l = 0; l < 9; ++l) scales[l] = net->act_scale[l];
  return TDM_OK;
}

extern "C" tdm_status tdm_net_set_max_batch(tdm_net* net, int32_t max_batch) {
  TDM_REQUIRE(net && max_batch > 0, "tdm_net_set_max_batch: bad arguments");
  net->max_batch = max_batch;
  return TDM_OK;
}

extern "C" tdm_status tdm_net_set_timing(tdm_net* net, int32_t enable) {
  TDM_REQUIRE(net, "tdm_net_set_timing: null net");
  net->timing = enable != 0;
  return TDM_OK;
}

extern "C" tdm_status tdm_net_layer_times(tdm_net* net, double* ms, int64_t* launches, int32_t reset) {
  TDM_REQUIRE(net && ms && launches, "tdm_net_layer_times: null pointer");
  TDM_CHECK_CUDA(net->drain());
  for (int i = 0; i < kTimedLayers; ++i) {
    ms[i] = net->layer_ms[i];
    launches[i] = net->layer_n[i];
    if (reset) {
      net->layer_ms[i] = 0.0;
      net->layer_n[i] = 0;
    }
  }
  return TDM_OK;
}

namespace tdm {
int net_max_batch(const tdm_net* net) { return net->max_batch; }
tdm_precision net_precision(const tdm_net* net) { return net->prec; }
uint64_t net_generation(const tdm_net* net) { return net->generation; }
}  // namespace tdm

namespace {

struct Tile {
  int nt, msub, form;  // form: TDM_CONV_GRID, TDM_CONV_DXF or TDM_CONV_GATHER
};
constexpr Tile kTiles[] = {{64, 4, TDM_CONV_GRID},   {64, 2, TDM_CONV_GRID},    {128, 2, TDM_CONV_GRID},
                           {128, 1, TDM_CONV_GRID},  {256, 1, TDM_CONV_GRID},   {256, 2, TDM_CONV_GATHER},
                           {256, 1, TDM_CONV_GATHER}, {128, 2, TDM_CONV_GATHER}, {256, 2, TDM_CONV_XRUN},
                           {256, 1, TDM_CONV_XRUN},   {128, 2, TDM_CONV_XRUN},   {128, 2, TDM_CONV_GATHER_WT},
                           {128, 2, TDM_CONV_XRUN_WT}};

bool form_gathers(int f) {
  return f == TDM_CONV_GATHER || f == TDM_CONV_XRUN || f == TDM_CONV_GATHER_WT || f == TDM_CONV_XRUN_WT;
}
bool form_xrun(int f) { return f == TDM_CONV_XRUN || f == TDM_CONV_XRUN_WT; }
bool form_wt(int f) { return f == TDM_CONV_GATHER_WT || f == TDM_CONV_XRUN_WT; }

int form_of(const TcLayer& L) {
  if (L.dxf) return L.pair ? TDM_CONV_DXF_PAIR : TDM_CONV_DXF;
  if (!L.gather) return TDM_CONV_GRID;
  if (L.wt) return L.xrun ? TDM_CONV_XRUN_WT : TDM_CONV_GATHER_WT;
  return L.xrun ? TDM_CONV_XRUN : TDM_CONV_GATHER;
}

// The tcgen05 layer a forward of `net` runs for layer l.
TcLayer& active_layer(tdm_net* net, int l) {
  return (net->prec == TDM_FP8 && l >= 1 && l <= 7) ? net->tc8[l] : net->tc[l];
}

// Tiles layer l can run: the N tile divides cout and the plan fits; conv1's
// im2col GEMM has one weight packing (N = 64).
std::vector<Tile> tile_candidates(tdm_net* net, int l) {
  std::vector<Tile> out;
  if (active_layer(net, l).dxf) {  // the dx-fused conv2: on a CTA pair, or 32 channels per CTA
    TcLayer L = active_layer(net, l);
    L.msub = 2;
    L.pair = true;
    if (tc_layer_fits(L)) out.push_back(Tile{32, 2, TDM_CONV_DXF_PAIR});
    for (int ms : {2, 1}) {
      L.msub = ms;
      L.pair = false;
      if (tc_layer_fits(L)) out.push_back(Tile{32, ms, TDM_CONV_DXF});
    }
    return out;
  }
  if (l == 0) return {Tile{64, 4, TDM_CONV_GRID}};  // conv1's fused im2col kernel has one tile shape
  for (const Tile& t : kTiles) {
    TcLayer L = active_layer(net, l);
    L.nt = t.nt;
    L.msub = t.msub;
    L.gather = form_gathers(t.form);
    L.xrun = form_xrun(t.form);
    L.wt = form_wt(t.form);
    if (tc_layer_fits(L)) out.push_back(t);
  }
  return out;
}

// Switches layer l to tile t, packing its weights for t.nt once per form.
tdm_status set_tile(tdm_net* net, int l, Tile t) {
  TcLayer& L = active_layer(net, l);
  const int form = (net->prec == TDM_FP8 && l >= 1 && l <= 7) ? 1 : 0;
  auto key = [&](int nt) { return (form * 16 + l) * 1024 + nt; };
  if (L.nt != t.nt) {
    net->packed[key(L.nt)] = L.wpk;
    auto it = net->packed.find(key(t.nt));
    if (it != net->packed.end()) {
      L.wpk = it->second;
    } else {
      TcLayer T = L;
      T.nt = t.nt;
      std::vector<uint8_t> pk;
      std::vector<float> sc;
      pack_tc_weights(T, net->hw[l].data(), l == 7 ? 27 : 1, &pk, &sc);
      uint8_t* d = nullptr;
      tdm_status st = net->upload(pk.data(), pk.size(), &d);
      if (st) return st;
      TDM_CHECK_CUDA(cudaDeviceSynchronize());
      net->packed[key(t.nt)] = d;
      L.wpk = d;
    }
  }
  if (L.nt != t.nt || L.msub != t.msub || form_of(L) != t.form) ++net->generation;
  L.nt = t.nt;
  L.msub = t.msub;
  if (L.dxf) {
    L.pair = t.form == TDM_CONV_DXF_PAIR;
  } else {
    L.gather = form_gathers(t.form);
    L.xrun = form_xrun(t.form);
    L.wt = form_wt(t.form);
  }
  return TDM_OK;
}

}  // namespace

extern "C" tdm_status tdm_net_autotune(tdm_net* net, const float* patches, int32_t b, int32_t reps, tdm_stream s) {
  TDM_REQUIRE(net && patches && b > 0 && reps > 0, "tdm_net_autotune: bad arguments");
  if (net->prec == TDM_FP32) return TDM_OK;  // the CUDA-core form has a single tile shape
  TDM_REQUIRE(net->prec != TDM_FP8 || net->calibrated, "FP8 net has no activation scales yet: call tdm_net_calibrate first");
  const int B = std::min<int>(b, net->max_batch);
  const int nl = net->use_feat ? 9 : 8;
  std::vector<std::vector<Tile>> cand(nl);
  size_t rounds = 0;
  for (int l = 0; l < nl; ++l) {
    cand[l] = tile_candidates(net, l);
    TDM_REQUIRE(!cand[l].empty(), "tdm_net_autotune: a layer has no tile that fits");
    rounds = std::max(rounds, cand[l].size());
  }
  float* out = nullptr;
  TDM_CHECK_CUDA(cudaMalloc(&out, (size_t)B * 512 * sizeof(float)));
  const bool timing = net->timing;
  net->timing = true;
  std::vector<double> best(nl, 1e30);
  std::vector<Tile> pick(nl);
  tdm_status st = TDM_OK;
  // Round r runs every layer on its r-th candidate (its first when it has
  // fewer); per-layer CUDA events attribute the time.
  for (size_t r = 0; r < rounds && st == TDM_OK; ++r) {
    for (int l = 0; l < nl && st == TDM_OK; ++l) st = set_tile(net, l, cand[l][r < cand[l].size() ? r : 0]);
    if (st) break;
    st = net_run(net, patches, B, out, -1, s, net->prec);  // warm-up (and workspace growth)
    if (st) break;
    if (net->drain() != cudaSuccess) { st = fail(TDM_ERR_DEVICE, "autotune timing"); break; }
    for (int i = 0; i < kTimedLayers; ++i) { net->layer_ms[i] = 0.0; net->layer_n[i] = 0; }
    for (int k = 0; k < reps && st == TDM_OK; ++k) st = net_run(net, patches, B, out, -1, s, net->prec);
    if (st) break;
    if (net->drain() != cudaSuccess) { st = fail(TDM_ERR_DEVICE, "autotune timing"); break; }
    for (int l = 0; l < nl; ++l) {
      if (r >= cand[l].size()) continue;
      if (net->layer_ms[l] < best[l]) { best[l] = net->layer_ms[l]; pick[l] = cand[l][r]; }
    }
  }
  for (int l = 0; l < nl && st == TDM_OK; ++l) st = set_tile(net, l, pick[l]);
  for (int i = 0; i < kTimedLayers; ++i) { net->layer_ms[i] = 0.0; net->layer_n[i] = 0; }
  net->timing = timing;
  cudaStreamSynchronize(s);
  cudaFree(out);
  return st;
}

extern "C" tdm_status tdm_net_tiles(const tdm_net* net, int32_t nt[9], int32_t msub[9]) {
  TDM_REQUIRE(net && nt && msub, "tdm_net_tiles: null pointer");
  for (int l = 0; l < 9; ++l) {
    const TcLayer& L = (net->prec == TDM_FP8 && l >= 1 && l <= 7) ? net->tc8[l] : net->tc[l];
    nt[l] = net->prec == TDM_FP32 ? 0 : L.nt;
    msub[l] = net->prec == TDM_FP32 ? 0 : L.msub;
  }
  return TDM_OK;
}

extern "C" tdm_status tdm_net_tile_forms(const tdm_net* net, int32_t form[9]) {
  TDM_REQUIRE(net && form, "tdm_net_tile_forms: null pointer");
  for (int l = 0; l < 9; ++l) {
    const TcLayer& L = (net->prec == TDM_FP8 && l >= 1 && l <= 7) ? net->tc8[l] : net->tc[l];
    form[l] = net->prec == TDM_FP32 ? TDM_CONV_GRID : form_of(L);
  }
  return TDM_OK;
}

extern "C" tdm_status tdm_net_set_tile_form(tdm_net* net, int32_t layer, int32_t nt, int32_t msub, int32_t form) {
  TDM_REQUIRE(net && layer >= 0 && layer < 9, "tdm_net_set_tile: bad arguments");
  TDM_REQUIRE(net->prec != TDM_FP32, "tdm_net_set_tile: the FP32 form has no tile choice");
  // an explicit form first; else the layer's current form, then any form with this tile
  const int cur = form_of(active_layer(net, layer));
  const std::vector<Tile> cand = tile_candidates(net, layer);
  for (int pass = 0; pass < 2; ++pass)
    for (const Tile& t : cand) {
      if (t.nt != nt || t.msub != msub) continue;
      if (form >= 0 ? t.form != form : (pass == 0 && t.form != cur)) continue;
      TDM_CHECK_CUDA(cudaDeviceSynchronize());  // no forward may still read the old packing's tile
      return set_tile(net, layer, t);
    }
  return fail(TDM_ERR_INVALID_ARG, "tdm_net_set_tile: tile not available for this layer");
}

extern "C" tdm_status tdm_net_set_tile(tdm_net* net, int32_t layer, int32_t nt, int32_t msub) {
  return tdm_net_set_tile_form(net, layer, nt, msub, -1);
}

extern "C" tdm_status tdm_net_destroy(tdm_net* net) {
  delete net;
  return TDM_OK;
}

extern "C" tdm_status tdm_write_seeded_weights(const char* path, uint64_t seed) {
  TDM_REQUIRE(path, "tdm_write_seeded_weights: null path");
  std::string err;
  tdm_status st = write_marvin_f32(path, seeded_weights(seed), &err);
  if (st != TDM_OK) return fail(st, err);
  return TDM_OK;
}

extern "C" tdm_status tdm_net_clone(const tdm_net* src, tdm_net** out) {
  TDM_REQUIRE(src && out, "tdm_net_clone: null pointer");
  const float* w[9];
  const float* b[9];
  for (int l = 0; l < 9; ++l) {
    w[l] = src->hw[l].data();
    b[l] = src->hb[l].data();
  }
  tdm_net* net = nullptr;
  tdm_status st = tdm_net_create_from_host(w, b, src->prec, src->use_feat, &net);
  if (st) return st;
  for (int l = 0; l < 9; ++l) net->act_scale[l] = src->act_scale[l];
  net->calibrated = src->calibrated;
  net->max_batch = src->max_batch;
  *out = net;
  return TDM_OK;
}

extern "C" size_t tdm_net_workspace_bytes(const tdm_net* net, int32_t b) {
  if (!net || b <= 0) return 0;
  const int chunk = std::min<int>(b, net->max_batch);
  return net->prec == TDM_FP32 ? f32_ws_bytes(chunk) : bf16_plan(net, chunk).total;
}
