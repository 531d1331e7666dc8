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

// float -> double by moving the fields (exact, integer pipe); zeros,
// subnormals, infinities and NaNs take the hardware conversion.
__device__ __forceinline__ double f2d(float x) {
  const uint32_t u = __float_as_uint(x), e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return (double)x;
  const uint64_t bits = ((uint64_t)(u >> 31) << 63) | ((uint64_t)(e + 896u) << 52) | ((uint64_t)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)bits);
}

// sum_k (a_k - b_k)^2 in double, k in order, one fma per term (the oracle's
// expression).  GB300 issues an FP64 warp instruction at a small fraction of
// the FP32 rate whatever the number of active lanes, so callers keep all 32
// lanes busy with independent (query, candidate) pairs.
__device__ __forceinline__ double exact_sqdist(const float* __restrict__ a, const float* __restrict__ b, int dim) {
  double s = 0.0;
#pragma unroll 4
  for (int k = 0; k < dim; k += 4) {
    const float4 x = *reinterpret_cast<const float4*>(a + k);
    const float4 y = *reinterpret_cast<const float4*>(b + k);
    double d = f2d(x.x) - f2d(y.x);
    s = fma(d, d, s);
    d = f2d(x.y) - f2d(y.y);
    s = fma(d, d, s);
    d = f2d(x.z) - f2d(y.z);
    s = fma(d, d, s);
    d = f2d(x.w) - f2d(y.w);
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

// Candidate lists: cand[g][0..3] for query g (rows of a first, then the
// columns, i.e. the rows of b).  cand[g][0] == -1 marks a query whose list is
// closer than twice the FP32 error bound of the expansion (FP32 form only);
// such a query is appended to `full` and scanned completely in FP64.
__device__ __forceinline__ void put_candidates(const Cand& m, float qn, float rn_max, int nr, int dim, int exact,
                                               int g, int32_t* __restrict__ cand, int32_t* __restrict__ full,
                                               int32_t* __restrict__ n_full) {
  const float sq = sqrtf(qn) + sqrtf(rn_max);
  const float E = 2.0f * (float)(dim + 8) * 5.97e-8f * sq * sq;
  if (exact && nr > TOPK && m.d[TOPK - 1] - m.d[0] < 2.0f * E) {
    cand[4 * g] = -1;
    full[atomicAdd(n_full, 1)] = g;
    return;
  }
#pragma unroll
  for (int t = 0; t < TOPK; ++t) cand[4 * g + t] = m.j[t];
}

// Row scan: warp per query row i of `dot` [nq][ld]; d = qn_i + rn_j - 2 dot.
__global__ void nn_rows_kernel(const float* __restrict__ dot, int64_t ld, int nq, int nr,
                               const float* __restrict__ qn, const float* __restrict__ rn,
                               const float* __restrict__ rn_max_ptr, int dim, int exact, int32_t* __restrict__ cand,
                               int32_t* __restrict__ full, int32_t* __restrict__ n_full) {
  const int warps = blockDim.x / 32, lane = threadIdx.x & 31;
  const int i = blockIdx.x * warps + threadIdx.x / 32;
  if (i >= nq) return;
  Cand c;
  cand_init(c);
  const float qi = qn[i];
  // four columns per lane per step: one 512-byte coalesced read per warp
  const float* row = dot + (int64_t)i * ld;
  for (int j = 4 * lane; j < nr; j += 128) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(row + j));
    const float4 n = __ldg(reinterpret_cast<const float4*>(rn + j));
    cand_push(c, qi + n.x - 2.0f * v.x, j);
    if (j + 1 < nr) cand_push(c, qi + n.y - 2.0f * v.y, j + 1);
    if (j + 2 < nr) cand_push(c, qi + n.z - 2.0f * v.z, j + 2);
    if (j + 3 < nr) cand_push(c, qi + n.w - 2.0f * v.w, j + 3);
  }
  Cand m = warp_merge(c);
  if (lane == 0) put_candidates(m, qi, *rn_max_ptr, nr, dim, exact, i, cand, full, n_full);
}

// Column scan over `dot` [nr][ld]: query j is a column, candidates are the
// rows i.  A block owns 8 consecutive columns: lane = (row group lane / 8,
// column lane % 8), so one warp load reads 4 rows x 32 bytes (one sector
// each), and the 16 warps split the rows; 8 columns per block give 1,000
// columns 125 blocks.  A warp's four row-group lists are merged with
// shuffles, the warps' lists in shared memory.  The top 4 of a set under the
// (distance, index) order does not depend on the merge order.  Query index
// g = goff + j.
constexpr int COL_WARPS = 16, COL_COLS = 8, COL_GROUPS = 32 / COL_COLS;

__global__ void __launch_bounds__(COL_WARPS * 32)
nn_cols_kernel(const float* __restrict__ dot, int64_t ld, int nq, int nr, const float* __restrict__ qn,
               const float* __restrict__ rn, const float* __restrict__ rn_max_ptr, int dim, int exact, int goff,
               int32_t* __restrict__ cand, int32_t* __restrict__ full, int32_t* __restrict__ n_full) {
  __shared__ float s_d[COL_WARPS][TOPK][COL_COLS];
  __shared__ int s_j[COL_WARPS][TOPK][COL_COLS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int col = lane % COL_COLS, grp = lane / COL_COLS;
  const int j = blockIdx.x * COL_COLS + col;
  const bool live = j < nq;
  Cand c;
  cand_init(c);
  if (live) {
    constexpr int STEP = COL_WARPS * COL_GROUPS;  // rows per pass of the block
    const float qj = qn[j];
    int i = w * COL_GROUPS + grp;
    for (; i + 3 * STEP < nr; i += 4 * STEP) {  // four rows in flight
      float v[4], n[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        v[u] = __ldg(dot + (int64_t)(i + u * STEP) * ld + j);
        n[u] = __ldg(rn + i + u * STEP);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) cand_push(c, qj + n[u] - 2.0f * v[u], i + u * STEP);
    }
    for (; i < nr; i += STEP) cand_push(c, qj + __ldg(rn + i) - 2.0f * __ldg(dot + (int64_t)i * ld + j), i);
  }
  // lanes col, col + 8, col + 16, col + 24 scanned disjoint rows of one column
#pragma unroll
  for (int o = COL_COLS; o < 32; o <<= 1) {
    float od[TOPK];
    int oj[TOPK];
#pragma unroll
    for (int t = 0; t < TOPK; ++t) {
      od[t] = __shfl_xor_sync(0xffffffffu, c.d[t], o);
      oj[t] = __shfl_xor_sync(0xffffffffu, c.j[t], o);
    }
#pragma unroll
    for (int t = 0; t < TOPK; ++t) cand_push(c, od[t], oj[t]);
  }
  if (grp == 0) {
#pragma unroll
    for (int t = 0; t < TOPK; ++t) { s_d[w][t][col] = c.d[t]; s_j[w][t][col] = c.j[t]; }
  }
  __syncthreads();
  if (w == 0 && grp == 0 && live) {
    Cand m;
    cand_init(m);
    for (int v = 0; v < COL_WARPS; ++v)
#pragma unroll
      for (int t = 0; t < TOPK; ++t) cand_push(m, s_d[v][t][col], s_j[v][t][col]);
    put_candidates(m, qn[j], *rn_max_ptr, nr, dim, exact, goff + j, cand, full, n_full);
  }
}

// Query g < na: a_g against the rows of b (result nn_ab[g]); otherwise
// b_{g-na} against the rows of a (nn_ba[g-na]).
struct Query {
  const float* q;
  const float* r;
  int nr;
  int32_t* out;
};

__device__ __forceinline__ Query query_of(int g, const float* a, const float* b, int na, int nb, int dim,
                                          int32_t* nn_ab, int32_t* nn_ba) {
  if (g < na) return Query{a + (int64_t)g * dim, b, nb, nn_ab + g};
  return Query{b + (int64_t)(g - na) * dim, a, na, nn_ba + (g - na)};
}

// Re-scoring: four consecutive lanes hold the four candidates of one query;
// the exact minimum (ties -> lower index) is reduced over those lanes.
__global__ void rescore_kernel(const float* __restrict__ a, const float* __restrict__ b, int na, int nb, int dim,
                               const int32_t* __restrict__ cand, int32_t* __restrict__ nn_ab,
                               int32_t* __restrict__ nn_ba) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int g = (int)(t >> 2);
  double best = DBL_MAX;
  int bj = INT_MAX;
  bool skip = true;
  Query Q{};
  if (g < na + nb) {
    Q = query_of(g, a, b, na, nb, dim, nn_ab, nn_ba);
    skip = cand[4 * g] == -1;
    const int j = cand[t];
    if (!skip && j >= 0 && j < Q.nr) {
      best = exact_sqdist(Q.q, Q.r + (int64_t)j * dim, dim);
      bj = j;
    }
  }
  for (int o = 1; o < 4; o <<= 1) {
    const double od = __shfl_xor_sync(0xffffffffu, best, o);
    const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
    if (od < best || (od == best && oj < bj)) { best = od; bj = oj; }
  }
  if (!skip && (t & 3) == 0) *Q.out = bj;
}

// Re-scoring of the BF16 form, one warp per query: lane l takes dims
// [l*dim/32, (l+1)*dim/32) of the query and of its four candidates (coalesced
// reads), sums (a_k - b_k)^2 in double over its slice, and a shuffle tree adds
// the 32 slices; the minimum (ties -> lower index) wins.  The sums differ from
// the oracle's k-ordered ones only in the last bits of double, far below the
// BF16 candidates' own error; the FP32 form keeps rescore_kernel.
//
// The same sums are first taken in FP32.  Every term is non-negative, so an
// FP32 sum lies within REL * sum + ABS of the exact one: a lane's slice and
// the tree round at most dim/32 + 5 times, each square and difference adds
// two roundings (2^-24 each, ~1.4e-6 for dim 512; REL = 4e-6 leaves a margin
// of ~3), and squares below the normal range lose at most 2^-150 each (ABS).
// When the best candidate's interval lies below every other candidate's, the
// exact sums and the FP64 ones (whose own error is ~1e-15 relative) pick that
// candidate too, and the FP64 pass is skipped; otherwise (near-ties, NaN,
// overflow) the query takes the FP64 pass.  So the chosen index is the FP64
// pass's in every case.  The FP32 sums and the decision are identical in all
// lanes (xor butterflies: each add's operands are swapped, not regrouped), so
// the branch is warp-uniform.
__global__ void __launch_bounds__(256) rescore_warp_kernel(const float* __restrict__ a, const float* __restrict__ b,
                                                           int na, int nb, int dim, const int32_t* __restrict__ cand,
                                                           int32_t* __restrict__ nn_ab, int32_t* __restrict__ nn_ba) {
  const int g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (g >= na + nb) return;
  const Query Q = query_of(g, a, b, na, nb, dim, nn_ab, nn_ba);
  if (cand[TOPK * g] == -1) return;
  const int per = dim >> 5, k0 = lane * per;  // dim is a multiple of 64: per is even
  double part[TOPK];
  int cj[TOPK];
#pragma unroll
  for (int c = 0; c < TOPK; ++c) {
    const int j = cand[TOPK * g + c];
    cj[c] = (j >= 0 && j < Q.nr) ? j : -1;
    part[c] = 0.0;
  }
  {
    float pf[TOPK];
#pragma unroll
    for (int c = 0; c < TOPK; ++c) pf[c] = 0.0f;
    for (int k = k0; k < k0 + per; k += 2) {
      const float2 x = *reinterpret_cast<const float2*>(Q.q + k);
#pragma unroll
      for (int c = 0; c < TOPK; ++c) {
        if (cj[c] < 0) continue;
        const float2 y = *reinterpret_cast<const float2*>(Q.r + (int64_t)cj[c] * dim + k);
        float d = x.x - y.x;
        pf[c] = fmaf(d, d, pf[c]);
        d = x.y - y.y;
        pf[c] = fmaf(d, d, pf[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < TOPK; ++c)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) pf[c] += __shfl_xor_sync(0xffffffffu, pf[c], o);
    constexpr float REL = 4e-6f, ABS = 1e-40f;
    int bc = -1;
#pragma unroll
    for (int c = 0; c < TOPK; ++c)
      if (cj[c] >= 0 && (bc < 0 || pf[c] < pf[bc])) bc = c;
    bool decided = bc >= 0 && pf[bc] == pf[bc];
    if (decided) {
      const float hi = pf[bc] + (REL * pf[bc] + ABS);
#pragma unroll
      for (int c = 0; c < TOPK; ++c)
        if (c != bc && cj[c] >= 0 && !(pf[c] - (REL * pf[c] + ABS) > hi)) decided = false;
    }
    if (decided) {
      if (lane == 0) *Q.out = cj[bc];
      return;
    }
  }
  for (int k = k0; k < k0 + per; k += 2) {
    const float2 x = *reinterpret_cast<const float2*>(Q.q + k);
#pragma unroll
    for (int c = 0; c < TOPK; ++c) {
      if (cj[c] < 0) continue;
      const float2 y = *reinterpret_cast<const float2*>(Q.r + (int64_t)cj[c] * dim + k);
      double d = f2d(x.x) - f2d(y.x);
      part[c] = fma(d, d, part[c]);
      d = f2d(x.y) - f2d(y.y);
      part[c] = fma(d, d, part[c]);
    }
  }
#pragma unroll
  for (int c = 0; c < TOPK; ++c)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part[c] += __shfl_xor_sync(0xffffffffu, part[c], o);
  if (lane == 0) {
    double best = DBL_MAX;
    int bj = INT_MAX;
#pragma unroll
    for (int c = 0; c < TOPK; ++c)
      if (cj[c] >= 0 && (part[c] < best || (part[c] == best && cj[c] < bj))) {
        best = part[c];
        bj = cj[c];
      }
    if (bj != INT_MAX) *Q.out = bj;
  }
}

// Full FP64 scan of the listed queries, one block per query at a time.
__global__ void full_scan_kernel(const float* __restrict__ a, const float* __restrict__ b, int na, int nb, int dim,
                                 const int32_t* __restrict__ full, const int32_t* __restrict__ n_full,
                                 int32_t* __restrict__ nn_ab, int32_t* __restrict__ nn_ba) {
  __shared__ double s_d[32];
  __shared__ int s_i[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int n = *n_full;
  for (int e = blockIdx.x; e < n; e += gridDim.x) {
    const Query Q = query_of(full[e], a, b, na, nb, dim, nn_ab, nn_ba);
    double best = DBL_MAX;
    int bi = INT_MAX;
    for (int i = threadIdx.x; i < Q.nr; i += blockDim.x) {
      const double d = exact_sqdist(Q.q, Q.r + (int64_t)i * dim, dim);
      if (d < best) { best = d; bi = i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double od = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (od < best || (od == best && oi < bi)) { best = od; bi = oi; }
    }
    if (lane == 0) { s_d[w] = best; s_i[w] = bi; }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int v = 1; v < nw; ++v)
        if (s_d[v] < best || (s_d[v] == best && s_i[v] < bi)) { best = s_d[v]; bi = s_i[v]; }
      *Q.out = bi;
    }
    __syncthreads();
  }
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

// Block 0: max of x0[0..n0), block 1: max of x1[0..n1) (into out[0], out[1]).
__global__ void max2_kernel(const float* __restrict__ x0, int n0, const float* __restrict__ x1, int n1,
                            float* __restrict__ out) {
  const float* x = blockIdx.x == 0 ? x0 : x1;
  const int n = blockIdx.x == 0 ? n0 : n1;
  float m = 0.0f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmaxf(m, x[i]);
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ float s[32];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, s[w]);
    out[blockIdx.x] = m;
  }
}

struct MnnLayout {
  int nbp;
  size_t dot, bT, na_n, nb_n, maxes, a8, bpk, zeros, cand, full, total;
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
  L.zeros = take((size_t)L.nbp * 4 + 16);  // zero bias row, then the full-scan counter
  L.cand = take((size_t)(na + nb) * TOPK * 4);
  L.full = take((size_t)(na + nb) * 4);
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
  TDM_REQUIRE(((uintptr_t)da | (uintptr_t)db) % 16 == 0, "tdm_match_mnn: descriptors must be 16-byte aligned");
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
  max2_kernel<<<2, 1024, 0, s>>>(an, na, bn, nb, maxes);
  note_launches(2);
  TDM_CHECK_LAUNCH("mnn norms");
  float* zeros = reinterpret_cast<float*>(w + L.zeros);
  int32_t* n_full = reinterpret_cast<int32_t*>(zeros + L.nbp);
  int32_t* cand = reinterpret_cast<int32_t*>(w + L.cand);
  int32_t* full = reinterpret_cast<int32_t*>(w + L.full);
  TDM_CHECK_CUDA(cudaMemsetAsync(zeros, 0, (size_t)L.nbp * 4 + 16, s));
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
  // candidates: rows a -> b (warp per row), columns b -> a (8 columns per block)
  nn_rows_kernel<<<(na + 7) / 8, 256, 0, s>>>(dot, L.nbp, na, nb, an, bn, maxes + 1, dim, exact, cand, full, n_full);
  nn_cols_kernel<<<(nb + COL_COLS - 1) / COL_COLS, COL_WARPS * 32, 0, s>>>(dot, L.nbp, nb, na, bn, an, maxes, dim, exact, na, cand,
                                                          full, n_full);
  const int64_t lanes = (int64_t)(na + nb) * TOPK;
  if (exact) {
    // one warp per block: the FP64 work of 8 queries per warp spreads over every
    // SM's FP64 pipe instead of packing four warps onto a quarter of the SMs
    rescore_kernel<<<(unsigned)((lanes + 31) / 32), 32, 0, s>>>(da, db, na, nb, dim, cand, nn_ab, nn_ba);
  } else {
    rescore_warp_kernel<<<(unsigned)((na + nb + 7) / 8), 256, 0, s>>>(da, db, na, nb, dim, cand, nn_ab, nn_ba);
  }
  note_launches(2);
  if (exact) {
    full_scan_kernel<<<256, 256, 0, s>>>(da, db, na, nb, dim, full, n_full, nn_ab, nn_ba);
    note_launches(1);
  }
  TDM_CHECK_LAUNCH("mnn candidate scans / re-scoring");
  mutual_kernel<<<1, 992, 0, s>>>(nn_ab, nn_ba, na, nb, pairs, n_pairs);
  TDM_CHECK_LAUNCH("mutual_kernel");
  return TDM_OK;
}
