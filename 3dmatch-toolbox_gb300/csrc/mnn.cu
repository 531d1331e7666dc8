// Mutual nearest neighbours in descriptor space (core/demo.m:51-57):
//   nn_ab[i] = argmin_j |a_i - b_j|,  nn_ba[j] = argmin_i |a_i - b_j|,
//   pairs (nn_ba[j], j) for every j with nn_ab[nn_ba[j]] == j, increasing j.
// The reference uses MATLAB KD-trees in double precision (exact NN).
//
// Dot products a_i . b_j come from a GEMM: FP32 CUDA cores (FP32 form) or the
// tcgen05 BF16 tensor-core GEMM (BF16 form).  Each row / column keeps its 4
// best candidates of |a|^2 + |b|^2 - 2 a.b, which are then re-scored exactly:
// sum_k (double)(a_k - b_k)^2 accumulated in k order with fma, the same
// expression the CPU oracle uses.  In the FP32 form a candidate list whose
// spread is below twice the FP32 error bound is replaced by a full FP64 scan
// of that row/column, so the indices equal the exact double-precision NN.
#include <cfloat>

#include "common.cuh"
#include "internal.h"

namespace tdm {
namespace {

constexpr int TOPK = 4;

__device__ __forceinline__ bool better(float d, int j, float bd, int bj) { return d < bd || (d == bd && j < bj); }

__device__ __forceinline__ double exact_sqdist(const float* __restrict__ a, const float* __restrict__ b, int dim) {
  double s = 0.0;
  for (int k = 0; k < dim; ++k) {
    double d = (double)a[k] - (double)b[k];
    s = fma(d, d, s);
  }
  return s;
}

__global__ void sqnorm_kernel(const float* __restrict__ x, int n, int dim, float* __restrict__ out) {
  int i = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  int lane = threadIdx.x & 31;
  if (i >= n) return;
  float s = 0.0f;
  for (int k = lane; k < dim; k += 32) s = fmaf(x[(int64_t)i * dim + k], x[(int64_t)i * dim + k], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[i] = s;
}

// bT[k][j] = b[j][k], zero for j >= nb (FP32 GEMM operand, row length nbp)
__global__ void transpose_pad_kernel(const float* __restrict__ b, int nb, int nbp, int dim, float* __restrict__ bT) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)dim * nbp) return;
  int k = (int)(t / nbp), j = (int)(t % nbp);
  bT[t] = j < nb ? b[(int64_t)j * dim + k] : 0.0f;
}

// BF16 chunk-planar copy of a: chunk c/8, row i (tensor-core A operand)
__global__ void to_c8_kernel(const float* __restrict__ a, int n, int dim, uint8_t* __restrict__ out, int64_t cs) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * (dim / 8)) return;
  int i = (int)(t / (dim / 8)), c = (int)(t % (dim / 8));
  const float* src = a + (int64_t)i * dim + c * 8;
  __nv_bfloat162 v[4];
  for (int h = 0; h < 4; ++h) v[h] = __floats2bfloat162_rn(src[2 * h], src[2 * h + 1]);
  *reinterpret_cast<uint4*>(out + (int64_t)c * cs + (int64_t)i * 16) = *reinterpret_cast<uint4*>(v);
}

// b packed as the tensor-core B operand: blocks (ntile, K group) of
// [chunk j][row n in 256][8 BF16]; rows beyond nb are zero.
__global__ void pack_b_kernel(const float* __restrict__ b, int nb, int nbp, int dim, uint8_t* __restrict__ out) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int kgroups = dim / 64;
  if (t >= (int64_t)nbp * (dim / 8)) return;
  int row = (int)(t / (dim / 8)), c = (int)(t % (dim / 8));
  int nt = row / 256, n = row % 256, cg = c / 8, j = c % 8;
  __nv_bfloat162 v[4];
  for (int h = 0; h < 4; ++h) {
    float x0 = row < nb ? b[(int64_t)row * dim + c * 8 + 2 * h] : 0.0f;
    float x1 = row < nb ? b[(int64_t)row * dim + c * 8 + 2 * h + 1] : 0.0f;
    v[h] = __floats2bfloat162_rn(x0, x1);
  }
  int64_t off = ((((int64_t)nt * kgroups + cg) * 8 + j) * 256 + n) * 16;
  *reinterpret_cast<uint4*>(out + off) = *reinterpret_cast<uint4*>(v);
}

struct Cand {
  float d[TOPK];
  int j[TOPK];
};

__device__ __forceinline__ void cand_init(Cand& c) {
#pragma unroll
  for (int q = 0; q < TOPK; ++q) { c.d[q] = FLT_MAX; c.j[q] = INT_MAX; }
}

__device__ __forceinline__ void cand_push(Cand& c, float d, int j) {
  if (!better(d, j, c.d[TOPK - 1], c.j[TOPK - 1])) return;
  int q = TOPK - 1;
  while (q > 0 && better(d, j, c.d[q - 1], c.j[q - 1])) {
    c.d[q] = c.d[q - 1];
    c.j[q] = c.j[q - 1];
    --q;
  }
  c.d[q] = d;
  c.j[q] = j;
}

// Warp-wide merge of per-lane candidate lists into lane 0's (ordered) list.
__device__ __forceinline__ Cand warp_merge(const Cand& mine) {
  Cand out;
  cand_init(out);
  int head = 0;
  for (int q = 0; q < TOPK; ++q) {
    float d = head < TOPK ? mine.d[head] : FLT_MAX;
    int j = head < TOPK ? mine.j[head] : INT_MAX;
    float bd = d;
    int bj = j;
    for (int o = 16; o > 0; o >>= 1) {
      float od = __shfl_xor_sync(0xffffffffu, bd, o);
      int oj = __shfl_xor_sync(0xffffffffu, bj, o);
      if (better(od, oj, bd, bj)) { bd = od; bj = oj; }
    }
    out.d[q] = bd;
    out.j[q] = bj;
    if (j == bj && bj != INT_MAX) ++head;  // the winning lane advances
  }
  return out;
}

// Row pass: warp per query row i of `dot` [nq][ld]; distances d = nq_i + nr_j - 2 dot.
// Candidates re-scored in FP64; `fallback` rows scanned completely in FP64.
__global__ void nn_rows_kernel(const float* __restrict__ dot, int64_t ld, int nq, int nr,
                               const float* __restrict__ qn, const float* __restrict__ rn,
                               const float* __restrict__ rn_max_ptr,
                               const float* __restrict__ q, const float* __restrict__ r, int dim, int transposed,
                               int exact, int32_t* __restrict__ nn) {
  const int warps = blockDim.x / 32, lane = threadIdx.x & 31;
  const int i = blockIdx.x * warps + threadIdx.x / 32;
  if (i >= nq) return;
  Cand c;
  cand_init(c);
  for (int j = lane; j < nr; j += 32) {
    float dp = transposed ? dot[(int64_t)j * ld + i] : dot[(int64_t)i * ld + j];
    float d = qn[i] + rn[j] - 2.0f * dp;
    cand_push(c, d, j);
  }
  Cand m = warp_merge(c);
  // error bound of the FP32 expansion (dot of length dim, sequential fma)
  const float sq = sqrtf(qn[i]) + sqrtf(*rn_max_ptr);
  const float E = 2.0f * (float)(dim + 8) * 5.97e-8f * sq * sq;
  const bool full = exact && (m.d[TOPK - 1] - m.d[0] < 2.0f * E) && nr > TOPK;
  const float* qi = q + (int64_t)i * dim;
  double best = DBL_MAX;
  int bj = INT_MAX;
  if (!full) {
    if (lane < TOPK && m.j[lane] < nr) {
      best = exact_sqdist(qi, r + (int64_t)m.j[lane] * dim, dim);
      bj = m.j[lane];
    }
  } else {
    for (int j = lane; j < nr; j += 32) {
      double d = exact_sqdist(qi, r + (int64_t)j * dim, dim);
      if (d < best || (d == best && j < bj)) { best = d; bj = j; }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    double od = __shfl_xor_sync(0xffffffffu, best, o);
    int oj = __shfl_xor_sync(0xffffffffu, bj, o);
    if (od < best || (od == best && oj < bj)) { best = od; bj = oj; }
  }
  if (lane == 0) nn[i] = bj;
}

// Mutual check and ordered compaction (one block): pairs (nn_ba[j], j).
__global__ void mutual_kernel(const int32_t* __restrict__ nn_ab, const int32_t* __restrict__ nn_ba, int na, int nb,
                              int32_t* __restrict__ pairs, int32_t* __restrict__ n_pairs) {
  __shared__ int s_warp[32];
  __shared__ int s_base;
  if (threadIdx.x == 0) s_base = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j0 = 0; j0 < nb; j0 += blockDim.x) {
    int j = j0 + threadIdx.x;
    int f = 0, i = 0;
    if (j < nb) {
      i = nn_ba[j];
      f = (i >= 0 && i < na && nn_ab[i] == j) ? 1 : 0;
    }
    unsigned bal = __ballot_sync(0xffffffffu, f);
    int pre = __popc(bal & ((1u << lane) - 1));
    if (lane == 31) s_warp[w] = pre + f;
    __syncthreads();
    if (threadIdx.x == 0) {
      int acc = 0;
      for (int q = 0; q < nw; ++q) { int t = s_warp[q]; s_warp[q] = acc; acc += t; }
      s_warp[31] = acc;  // block total (nw <= 31 warps used below)
    }
    __syncthreads();
    if (f) {
      int pos = s_base + s_warp[w] + pre;
      pairs[2 * pos] = i;
      pairs[2 * pos + 1] = j;
    }
    __syncthreads();
    if (threadIdx.x == 0) s_base += s_warp[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) *n_pairs = s_base;
}

__global__ void max_kernel(const float* __restrict__ x, int n, float* __restrict__ out) {
  float m = 0.0f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmaxf(m, x[i]);
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ float s[32];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, s[w]);
    *out = m;
  }
}

struct MnnLayout {
  int nbp;
  size_t dot, bT, na_n, nb_n, maxes, a8, bpk, zeros, total;
  int64_t a8_cs;
};

MnnLayout mnn_layout(int na, int nb, int dim) {
  MnnLayout L{};
  L.nbp = ((nb + 255) / 256) * 256;
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~(size_t)255; return o; };
  L.dot = take((size_t)na * L.nbp * 4);
  L.bT = take((size_t)dim * L.nbp * 4);
  L.na_n = take((size_t)na * 4);
  L.nb_n = take((size_t)nb * 4);
  L.maxes = take(64);
  L.a8_cs = ((int64_t)na + 256 + 16) * 16;
  L.a8 = take((size_t)(dim / 8) * L.a8_cs);
  L.bpk = take((size_t)L.nbp * (dim / 8) * 16);
  L.zeros = take((size_t)L.nbp * 4);
  L.total = off;
  return L;
}

}  // namespace
}  // namespace tdm

using namespace tdm;

extern "C" size_t tdm_mnn_workspace_bytes(int32_t na, int32_t nb, int32_t dim) {
  if (na <= 0 || nb <= 0 || dim <= 0) return 0;
  return mnn_layout(na, nb, dim).total;
}

extern "C" tdm_status tdm_match_mnn(const float* da, int32_t na, const float* db, int32_t nb, int32_t dim,
                                    tdm_precision prec, int32_t* nn_ab, int32_t* nn_ba, int32_t* pairs,
                                    int32_t* n_pairs, void* ws, size_t ws_bytes, tdm_stream s) {
  TDM_REQUIRE(da && db && nn_ab && nn_ba && pairs && n_pairs && ws, "tdm_match_mnn: null pointer");
  TDM_REQUIRE(na > 0 && nb > 0, "tdm_match_mnn: empty descriptor set");
  TDM_REQUIRE(dim % 64 == 0, "tdm_match_mnn: dim must be a multiple of 64");
  TDM_REQUIRE(prec == TDM_FP32 || prec == TDM_BF16, "tdm_match_mnn: precision must be FP32 or BF16");
  MnnLayout L = mnn_layout(na, nb, dim);
  TDM_REQUIRE(ws_bytes >= L.total, "tdm_match_mnn: workspace too small");
  uint8_t* w = static_cast<uint8_t*>(ws);
  float* dot = reinterpret_cast<float*>(w + L.dot);
  float* an = reinterpret_cast<float*>(w + L.na_n);
  float* bn = reinterpret_cast<float*>(w + L.nb_n);
  float* maxes = reinterpret_cast<float*>(w + L.maxes);
  sqnorm_kernel<<<(na + 7) / 8, 256, 0, s>>>(da, na, dim, an);
  sqnorm_kernel<<<(nb + 7) / 8, 256, 0, s>>>(db, nb, dim, bn);
  max_kernel<<<1, 1024, 0, s>>>(an, na, maxes);
  max_kernel<<<1, 1024, 0, s>>>(bn, nb, maxes + 1);
  note_launches(3);
  TDM_CHECK_LAUNCH("mnn norms");
  float* zeros = reinterpret_cast<float*>(w + L.zeros);
  TDM_CHECK_CUDA(cudaMemsetAsync(zeros, 0, (size_t)L.nbp * 4, s));
  if (prec == TDM_FP32) {
    float* bT = reinterpret_cast<float*>(w + L.bT);
    int64_t n = (int64_t)dim * L.nbp;
    transpose_pad_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(db, nb, L.nbp, dim, bT);
    TDM_CHECK_LAUNCH("transpose_pad_kernel");
    // dot[i][j] = sum_k a[i][k] * bT[k][j]: the CUDA-core GEMM with a 1x1x1 "conv"
    tdm_status st = launch_conv_f32(da, na, 1, dim, 1, bT, zeros, L.nbp, false, dot, s);
    if (st) return st;
  } else {
    uint8_t* a8 = w + L.a8;
    uint8_t* bpk = w + L.bpk;
    int64_t n = (int64_t)na * (dim / 8);
    to_c8_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(da, na, dim, a8, L.a8_cs);
    n = (int64_t)L.nbp * (dim / 8);
    pack_b_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(db, nb, L.nbp, dim, bpk);
    note_launches(1);
    TDM_CHECK_LAUNCH("mnn bf16 packing");
    TcLayer T{};
    T.cin = dim;
    T.cout = L.nbp;
    T.D = T.Do = 1;
    T.nz = T.nyx = 1;
    T.kgroups = dim / 64;
    T.nt = 256;
    T.msub = 1;
    T.out_mode = TC_OUT_F32_ROWS;
    T.relu = 0;
    T.wpk = bpk;
    T.bias = zeros;
    TcArgs a{};
    a.act = a8;
    a.act_cs = L.a8_cs;
    a.rows = na;
    a.out = reinterpret_cast<uint8_t*>(dot);
    a.in_scale = a.out_qinv = 1.0f;
    tdm_status st = launch_tc_layer(T, a, s);
    if (st) return st;
  }
  const int exact = prec == TDM_FP32 ? 1 : 0;
  // rows: a -> b ; columns: b -> a (dot read transposed)
  nn_rows_kernel<<<(na + 7) / 8, 256, 0, s>>>(dot, L.nbp, na, nb, an, bn, maxes + 1, da, db, dim, 0, exact, nn_ab);
  nn_rows_kernel<<<(nb + 7) / 8, 256, 0, s>>>(dot, L.nbp, nb, na, bn, an, maxes, db, da, dim, 1, exact, nn_ba);
  note_launches(1);
  TDM_CHECK_LAUNCH("nn_rows_kernel");
  mutual_kernel<<<1, 992, 0, s>>>(nn_ab, nn_ba, na, nb, pairs, n_pairs);
  TDM_CHECK_LAUNCH("mutual_kernel");
  return TDM_OK;
}
