// Rigid ICP refinement of a registered pair: the step register2Fragments.m
// keeps commented out at lines 70-78 (pcregrigid on pcdownsample(...,
// 'gridAverage', 0.01) clouds, 'InlierRatio' 0.3, 'Tolerance' [1e-4, 9e-5],
// 'MaxIterations' 50).  Point-to-point:
//   1. both clouds averaged per grid cell (exact 2^-24 m fixed-point sums);
//   2. per iteration every moved moving point takes its nearest fixed point
//      within max_dist (hashed grid; ties go to the lexicographically smaller
//      point), the closest inlier_ratio of the pairs are kept (a 4,096-bin
//      quantile of d^2), and their Kabsch fit updates the transform;
//   3. stop when the update moves less than tol_translation and turns less
//      than tol_rotation_deg.
// The Kabsch sums are exact 128-bit integer sums of fixed-point coordinates,
// reduced per block on the device and across blocks on the host, so the
// result does not depend on thread order: a pair gives the same bits every
// run.  (pcregrigid's 'Extrapolate' quaternion step is not reproduced.)
//
// Compiled with -fmad=false.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "hashgrid.cuh"
#include "kabsch.cuh"

namespace tdm {
namespace {

constexpr int kHist = 4096;
constexpr int kSums = 17;  // sx[3], sy[3], syx[9] (y_a x_b at 3a+b), n, sum d2
constexpr int kSumBlocks = 512;
constexpr float kQ = 16777216.0f;  // 2^24 fixed-point scale

// Downsampling table: a cell's key, point count and fixed-point sums.
struct AvgTable {
  uint64_t* keys;
  int32_t* count;
  unsigned long long* sum;  // 3 per slot
  int32_t* pos;             // output position of an occupied slot
  int64_t H;
};

__global__ void avg_clear_kernel(AvgTable T) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < T.H; i += (int64_t)gridDim.x * blockDim.x) {
    T.keys[i] = kEmpty;
    T.count[i] = 0;
    T.sum[3 * i] = T.sum[3 * i + 1] = T.sum[3 * i + 2] = 0ull;
  }
}

__device__ __forceinline__ long long q24(float v) { return __float2ll_rn(__fmul_rn(v, kQ)); }

__global__ void avg_insert_kernel(const float* __restrict__ p, int n, float cell, float lim, AvgTable T,
                                  int* __restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float x = p[3 * (int64_t)i], y = p[3 * (int64_t)i + 1], z = p[3 * (int64_t)i + 2];
  if (!(fabsf(x) < lim && fabsf(y) < lim && fabsf(z) < lim)) {
    atomicExch(err, 1);
    return;
  }
  int c[3];
  cell_of(x, y, z, cell, c);
  const uint64_t key = cell_key(c[0], c[1], c[2]);
  uint32_t s = slot_of(key, T.H);
  for (int64_t probe = 0; probe < T.H; ++probe) {
    const unsigned long long prev =
        atomicCAS(reinterpret_cast<unsigned long long*>(T.keys + s), (unsigned long long)kEmpty, key);
    if (prev == kEmpty || prev == key) {
      atomicAdd(T.count + s, 1);
      atomicAdd(T.sum + 3 * s, (unsigned long long)q24(x));
      atomicAdd(T.sum + 3 * s + 1, (unsigned long long)q24(y));
      atomicAdd(T.sum + 3 * s + 2, (unsigned long long)q24(z));
      return;
    }
    s = (uint32_t)((s + 1) & (T.H - 1));
  }
  atomicExch(err, 2);
}

__global__ void avg_flag_kernel(AvgTable T) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < T.H; i += (int64_t)gridDim.x * blockDim.x)
    T.pos[i] = T.count[i] > 0 ? 1 : 0;
}

// centroids of the occupied cells, at their scanned positions
__global__ void avg_write_kernel(AvgTable T, const int32_t* __restrict__ scanned, float* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < T.H; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t c = T.count[i];
    if (c == 0) continue;
    const int32_t at = scanned[i];
    for (int a = 0; a < 3; ++a)
      out[3 * (int64_t)at + a] = (float)((double)(long long)T.sum[3 * i + a] / ((double)c * (double)kQ));
  }
}

__device__ __forceinline__ bool lex_less(float ax, float ay, float az, float bx, float by, float bz) {
  return ax < bx || (ax == bx && (ay < by || (ay == by && az < bz)));
}

// Nearest fixed point within max_dist of each moved moving point.
__global__ void nn_kernel(const float* __restrict__ mv, int n, const float* __restrict__ Rt, float cell, float lim,
                          float max_d2, Table T, float* __restrict__ moved, float* __restrict__ match,
                          float* __restrict__ d2out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float x0 = mv[3 * (int64_t)i], y0 = mv[3 * (int64_t)i + 1], z0 = mv[3 * (int64_t)i + 2];
  float m[3];
  for (int r = 0; r < 3; ++r)
    m[r] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(Rt[4 * r], x0), __fmul_rn(Rt[4 * r + 1], y0)),
                               __fmul_rn(Rt[4 * r + 2], z0)),
                     Rt[4 * r + 3]);
  moved[3 * (int64_t)i] = m[0];
  moved[3 * (int64_t)i + 1] = m[1];
  moved[3 * (int64_t)i + 2] = m[2];
  float best = INFINITY, bx = 0.f, by = 0.f, bz = 0.f;
  if (fabsf(m[0]) < lim && fabsf(m[1]) < lim && fabsf(m[2]) < lim) {
    int c[3];
    cell_of(m[0], m[1], m[2], cell, c);
    for (int d = 0; d < 27; ++d) {
      const uint64_t key = cell_key(c[0] + d / 9 - 1, c[1] + (d / 3) % 3 - 1, c[2] + d % 3 - 1);
      uint32_t s = slot_of(key, T.H);
      for (int64_t probe = 0; probe < T.H; ++probe) {
        const uint64_t k = T.keys[s];
        if (k == kEmpty) break;
        if (k == key) {
          const int32_t a = T.start[s], e = a + T.count[s];
          for (int32_t j = a; j < e; ++j) {
            const float qx = T.pts[3 * (int64_t)j], qy = T.pts[3 * (int64_t)j + 1], qz = T.pts[3 * (int64_t)j + 2];
            const float dx = __fsub_rn(m[0], qx), dy = __fsub_rn(m[1], qy), dz = __fsub_rn(m[2], qz);
            const float e2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            if (e2 < max_d2 && (e2 < best || (e2 == best && lex_less(qx, qy, qz, bx, by, bz)))) {
              best = e2;
              bx = qx;
              by = qy;
              bz = qz;
            }
          }
          break;
        }
        s = (uint32_t)((s + 1) & (T.H - 1));
      }
    }
  }
  match[3 * (int64_t)i] = bx;
  match[3 * (int64_t)i + 1] = by;
  match[3 * (int64_t)i + 2] = bz;
  d2out[i] = best;
}

__device__ __forceinline__ int d2_bin(float d2, float max_d2) {
  return min(kHist - 1, (int)(__fdiv_rn(d2, max_d2) * (float)kHist));
}

__global__ void hist_kernel(const float* __restrict__ d2, int n, float max_d2, int32_t* __restrict__ hist) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && d2[i] < max_d2) atomicAdd(hist + d2_bin(d2[i], max_d2), 1);
}

__device__ __forceinline__ __int128 shfl_down_i128(__int128 v, int o) {
  const unsigned long long lo = (unsigned long long)v;
  const long long hi = (long long)(v >> 64);
  const unsigned long long l2 = __shfl_down_sync(0xffffffffu, lo, o);
  const long long h2 = __shfl_down_sync(0xffffffffu, hi, o);
  return ((__int128)h2 << 64) | (__int128)l2;
}

// Exact sums over the kept pairs (bin <= bmax): x = matched fixed point,
// y = moved moving point; one partial of kSums values per block.
__global__ void __launch_bounds__(256) sums_kernel(const float* __restrict__ moved, const float* __restrict__ match,
                                                   const float* __restrict__ d2, int n, float max_d2, int bmax,
                                                   __int128* __restrict__ part) {
  __shared__ __int128 s_warp[8][kSums];
  __int128 acc[kSums];
  for (int k = 0; k < kSums; ++k) acc[k] = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float e = d2[i];
    if (!(e < max_d2) || d2_bin(e, max_d2) > bmax) continue;
    long long X[3], Y[3];
    for (int a = 0; a < 3; ++a) {
      X[a] = q24(match[3 * (int64_t)i + a]);
      Y[a] = q24(moved[3 * (int64_t)i + a]);
      acc[a] += X[a];
      acc[3 + a] += Y[a];
    }
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) acc[6 + 3 * a + b] += (__int128)Y[a] * X[b];
    acc[15] += 1;
    acc[16] += q24(e);
  }
  for (int k = 0; k < kSums; ++k)
    for (int o = 16; o > 0; o >>= 1) acc[k] += shfl_down_i128(acc[k], o);
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0)
    for (int k = 0; k < kSums; ++k) s_warp[w][k] = acc[k];
  __syncthreads();
  if (threadIdx.x < kSums) {
    __int128 t = 0;
    for (int v = 0; v < (int)(blockDim.x >> 5); ++v) t += s_warp[v][threadIdx.x];
    part[(int64_t)blockIdx.x * kSums + threadIdx.x] = t;
  }
}

struct IcpLayout {
  int64_t Hf, Hm;
  size_t avg[2][4], down[2], tab[5], moved, match, d2, hist, part, sums, flag, total;
  int64_t Ht;
};

IcpLayout icp_layout(int nf, int nm) {
  IcpLayout L{};
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~(size_t)255; return o; };
  const int n[2] = {nf, nm};
  L.Hf = table_slots(nf);
  L.Hm = table_slots(nm);
  const int64_t H[2] = {L.Hf, L.Hm};
  for (int t = 0; t < 2; ++t) {
    L.avg[t][0] = take((size_t)H[t] * 8);
    L.avg[t][1] = take((size_t)H[t] * 4);
    L.avg[t][2] = take((size_t)H[t] * 24);
    L.avg[t][3] = take((size_t)H[t] * 4);
    L.down[t] = take((size_t)n[t] * 12);
  }
  L.Ht = table_slots(nf);
  L.tab[0] = take((size_t)L.Ht * 8);
  L.tab[1] = take((size_t)L.Ht * 4);
  L.tab[2] = take((size_t)L.Ht * 4);
  L.tab[3] = take((size_t)L.Ht * 4);
  L.tab[4] = take((size_t)nf * 16);  // pslot (4) + grouped points (12)
  L.moved = take((size_t)nm * 12);
  L.match = take((size_t)nm * 12);
  L.d2 = take((size_t)nm * 4);
  L.hist = take(kHist * 4);
  L.part = take((size_t)kSumBlocks * kSums * 16 + 16);
  L.sums = take(kScanBlock * 4);
  L.flag = take(16 + 12 * 4);  // error word, then the transform as floats
  L.total = off;
  return L;
}

// Grid-average of n points into `out`; returns the number of cells.
tdm_status downsample(const float* p, int n, float cell, float lim, AvgTable T, int32_t* sums, int* err, float* out,
                      int* n_out, cudaStream_t s) {
  const unsigned g = (unsigned)std::min<int64_t>((T.H + 255) / 256, 4096);
  avg_clear_kernel<<<g, 256, 0, s>>>(T);
  avg_insert_kernel<<<(n + 255) / 256, 256, 0, s>>>(p, n, cell, lim, T, err);
  avg_flag_kernel<<<g, 256, 0, s>>>(T);
  const int nblk = (int)((T.H + kScanBlock - 1) / kScanBlock);
  // inclusive count = exclusive scan + flag of the last slot
  scan_block_kernel<<<nblk, kScanBlock, 0, s>>>(T.pos, T.H, T.pos, sums);
  scan_sums_kernel<<<1, kScanBlock, 0, s>>>(sums, nblk);
  scan_add_kernel<<<nblk, kScanBlock, 0, s>>>(T.pos, T.H, sums);
  avg_write_kernel<<<g, 256, 0, s>>>(T, T.pos, out);
  note_launches(7);
  TDM_CHECK_LAUNCH("icp downsample");
  int32_t last_pos = 0, last_cnt = 0;
  TDM_CHECK_CUDA(cudaMemcpyAsync(&last_pos, T.pos + T.H - 1, 4, cudaMemcpyDeviceToHost, s));
  TDM_CHECK_CUDA(cudaMemcpyAsync(&last_cnt, T.count + T.H - 1, 4, cudaMemcpyDeviceToHost, s));
  TDM_CHECK_CUDA(cudaStreamSynchronize(s));
  *n_out = last_pos + (last_cnt > 0 ? 1 : 0);
  return TDM_OK;
}

void compose(const double a[12], const double b[12], double out[12]) {  // out = a o b (3x4 affine)
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) out[4 * r + c] = a[4 * r] * b[c] + a[4 * r + 1] * b[4 + c] + a[4 * r + 2] * b[8 + c];
    out[4 * r + 3] = a[4 * r] * b[3] + a[4 * r + 1] * b[7] + a[4 * r + 2] * b[11] + a[4 * r + 3];
  }
}

}  // namespace
}  // namespace tdm

using namespace tdm;

extern "C" size_t tdm_icp_workspace_bytes(int32_t nf, int32_t nm) {
  if (nf <= 0 || nm <= 0 || nf > (1 << 19) || nm > (1 << 19)) return 0;
  return icp_layout(nf, nm).total;
}

extern "C" tdm_status tdm_icp(const float* fixed, int32_t nf, const float* moving, int32_t nm, const double init[12],
                              const tdm_icp_params* prm, tdm_icp_result* res, void* ws, size_t ws_bytes,
                              tdm_stream s) {
  TDM_REQUIRE(fixed && moving && init && prm && res && ws, "tdm_icp: null pointer");
  TDM_REQUIRE(nf > 0 && nm > 0 && nf <= (1 << 19) && nm <= (1 << 19), "tdm_icp: 1 .. 524288 points per cloud");
  TDM_REQUIRE(prm->grid > 0.0f && prm->max_dist > 0.0f && prm->max_dist < 1.0e3f && prm->inlier_ratio > 0.0f &&
                  prm->inlier_ratio <= 1.0f && prm->max_iterations >= 0,
              "tdm_icp: bad parameters");
  const IcpLayout L = icp_layout(nf, nm);
  TDM_REQUIRE(ws_bytes >= L.total, "tdm_icp: workspace too small");
  uint8_t* w = static_cast<uint8_t*>(ws);
  int* err = reinterpret_cast<int*>(w + L.flag);
  float* d_rt = reinterpret_cast<float*>(w + L.flag + 16);
  int32_t* sums = reinterpret_cast<int32_t*>(w + L.sums);
  AvgTable A[2];
  const int64_t H[2] = {L.Hf, L.Hm};
  for (int t = 0; t < 2; ++t)
    A[t] = AvgTable{reinterpret_cast<uint64_t*>(w + L.avg[t][0]), reinterpret_cast<int32_t*>(w + L.avg[t][1]),
                    reinterpret_cast<unsigned long long*>(w + L.avg[t][2]), reinterpret_cast<int32_t*>(w + L.avg[t][3]),
                    H[t]};
  float* df = reinterpret_cast<float*>(w + L.down[0]);
  float* dm = reinterpret_cast<float*>(w + L.down[1]);
  TDM_CHECK_CUDA(cudaMemsetAsync(err, 0, 16, s));
  const float glim = prm->grid * kMaxCells;
  int nf2 = 0, nm2 = 0;
  tdm_status st = downsample(fixed, nf, prm->grid, glim, A[0], sums, err, df, &nf2, s);
  if (!st) st = downsample(moving, nm, prm->grid, glim, A[1], sums, err, dm, &nm2, s);
  if (st) return st;
  Table T{reinterpret_cast<uint64_t*>(w + L.tab[0]), reinterpret_cast<int32_t*>(w + L.tab[1]),
          reinterpret_cast<int32_t*>(w + L.tab[2]), reinterpret_cast<int32_t*>(w + L.tab[3]),
          reinterpret_cast<int32_t*>(w + L.tab[4]), reinterpret_cast<float*>(w + L.tab[4] + (size_t)nf * 4), L.Ht};
  const float cell = prm->max_dist * kCellScale, lim = cell * kMaxCells, max_d2 = prm->max_dist * prm->max_dist;
  st = build_table(df, nf2, cell, lim, T, sums, err, s);
  if (st) return st;
  int h_err = 0;
  TDM_CHECK_CUDA(cudaMemcpyAsync(&h_err, err, 4, cudaMemcpyDeviceToHost, s));
  TDM_CHECK_CUDA(cudaStreamSynchronize(s));
  TDM_REQUIRE(h_err == 0, "tdm_icp: a coordinate is non-finite or too far from the origin for the grids");

  float* moved = reinterpret_cast<float*>(w + L.moved);
  float* match = reinterpret_cast<float*>(w + L.match);
  float* d2 = reinterpret_cast<float*>(w + L.d2);
  int32_t* hist = reinterpret_cast<int32_t*>(w + L.hist);
  __int128* part = reinterpret_cast<__int128*>(w + L.part);
  const int sblocks = std::min(kSumBlocks, std::max(1, (nm2 + 255) / 256));
  double T_cur[12];
  for (int i = 0; i < 12; ++i) T_cur[i] = init[i];
  std::vector<int32_t> h_hist(kHist);
  std::vector<__int128> h_part((size_t)sblocks * kSums);
  res->iterations = 0;
  res->converged = 0;
  res->correspondences = 0;
  res->rmse = 0.0f;
  for (int it = 0; it < prm->max_iterations; ++it) {
    float frt[12];
    for (int i = 0; i < 12; ++i) frt[i] = (float)T_cur[i];
    TDM_CHECK_CUDA(cudaMemcpyAsync(d_rt, frt, sizeof(frt), cudaMemcpyHostToDevice, s));
    TDM_CHECK_CUDA(cudaMemsetAsync(hist, 0, kHist * 4, s));
    nn_kernel<<<(nm2 + 127) / 128, 128, 0, s>>>(dm, nm2, d_rt, cell, lim, max_d2, T, moved, match, d2);
    hist_kernel<<<(nm2 + 255) / 256, 256, 0, s>>>(d2, nm2, max_d2, hist);
    note_launches(2);
    TDM_CHECK_LAUNCH("icp nn / histogram");
    TDM_CHECK_CUDA(cudaMemcpyAsync(h_hist.data(), hist, kHist * 4, cudaMemcpyDeviceToHost, s));
    TDM_CHECK_CUDA(cudaStreamSynchronize(s));
    int64_t total = 0;
    for (int b = 0; b < kHist; ++b) total += h_hist[b];
    if (total < 3) break;  // too few pairs within max_dist to fit
    const int64_t want = std::max<int64_t>(3, (int64_t)std::ceil((double)prm->inlier_ratio * (double)total));
    int bmax = 0;
    for (int64_t c = 0; bmax < kHist; ++bmax) {
      c += h_hist[bmax];
      if (c >= want) break;
    }
    sums_kernel<<<sblocks, 256, 0, s>>>(moved, match, d2, nm2, max_d2, bmax, part);
    note_launches(1);
    TDM_CHECK_LAUNCH("icp sums");
    TDM_CHECK_CUDA(cudaMemcpyAsync(h_part.data(), part, h_part.size() * 16, cudaMemcpyDeviceToHost, s));
    TDM_CHECK_CUDA(cudaStreamSynchronize(s));
    __int128 S[kSums] = {};
    for (int b = 0; b < sblocks; ++b)
      for (int k = 0; k < kSums; ++k) S[k] += h_part[(size_t)b * kSums + k];
    const __int128 n = S[15];
    // n * sum (y - cy)(x - cx)^T = n * syx - sy sx^T, exactly
    double Hm[3][3], cx[3], cy[3];
    const double q2 = (double)kQ * (double)kQ, nd = (double)n;
    for (int a = 0; a < 3; ++a) {
      cx[a] = (double)S[a] / (nd * (double)kQ);
      cy[a] = (double)S[3 + a] / (nd * (double)kQ);
      for (int b = 0; b < 3; ++b) Hm[a][b] = (double)(n * S[6 + 3 * a + b] - S[3 + a] * S[b]) / (nd * q2);
    }
    double R[9], t[3];
    if (!kabsch_from_h(Hm, cx, cy, R, t)) break;
    const double D[12] = {R[0], R[1], R[2], t[0], R[3], R[4], R[5], t[1], R[6], R[7], R[8], t[2]};
    double Tn[12];
    compose(D, T_cur, Tn);
    for (int i = 0; i < 12; ++i) T_cur[i] = Tn[i];
    res->iterations = it + 1;
    res->correspondences = (int32_t)n;
    res->rmse = (float)std::sqrt((double)S[16] / (nd * (double)kQ));
    const double dt = std::sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    const double ca = std::max(-1.0, std::min(1.0, (R[0] + R[4] + R[8] - 1.0) / 2.0));
    const double dr = std::acos(ca) * (180.0 / 3.14159265358979323846);
    if (dt < prm->tol_translation && dr < prm->tol_rotation_deg) {
      res->converged = 1;
      break;
    }
  }
  for (int i = 0; i < 12; ++i) res->rt[i] = T_cur[i];
  return TDM_OK;
}
