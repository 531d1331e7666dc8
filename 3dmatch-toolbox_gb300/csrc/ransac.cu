// RANSAC rigid registration with Kabsch refit.
//
// Replaces ransacfitRt.m (core/external/sfm/ransacfitRt.m:20-38), ransac.m
// (core/external/peter/ransac.m:113-232) and estimateRt.m.  Model x = R y + t
// (x: fragment-1 keypoints, y: fragment-2 keypoints).  Every trial h draws 3
// distinct correspondences from a counter-based stream (splitmix64 keyed by
// seed and 3h+j), fits R,t with Kabsch in FP32 (covariance, SVD through the
// Jacobi eigen-decomposition of H^T H; the model is used in FP32 for the
// inlier tests, and FP32 issues far faster than FP64), and counts inliers with the
// strict |x - (R y + t)| < threshold of euc3Ddist.  The best count wins and
// ties go to the later trial (ransac.m:194 uses >=).  The final model is the
// FP64 Kabsch refit on the winner's inliers (ransacfitRt.m:37).
//
// This translation unit is compiled with -fmad=false: the CPU oracle performs
// the same operations in the same order, so trial counts and inlier sets are
// identical on both.
#include <cfloat>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "kabsch.cuh"

namespace tdm {
namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__device__ __forceinline__ uint32_t bounded(uint64_t seed, uint64_t ctr, uint32_t n) {
  return (uint32_t)__umul64hi(mix64(seed + (ctr + 1) * 0x9E3779B97F4A7C15ULL), (uint64_t)n);
}

__device__ void sample3(uint64_t seed, uint32_t h, int m, int s[3]) {
  uint32_t i0 = bounded(seed, 3ull * h + 0, (uint32_t)m);
  uint32_t i1 = bounded(seed, 3ull * h + 1, (uint32_t)(m - 1));
  uint32_t i2 = bounded(seed, 3ull * h + 2, (uint32_t)(m - 2));
  if (i1 >= i0) i1++;
  uint32_t lo = i0 < i1 ? i0 : i1, hi = i0 < i1 ? i1 : i0;
  if (i2 >= lo) i2++;
  if (i2 >= hi) i2++;
  s[0] = (int)i0; s[1] = (int)i1; s[2] = (int)i2;
}

// FP64 Kabsch refit on the listed correspondences, run by one whole warp.
// The one-thread form is: centroids cx, cy summed in list order and divided
// by n; H[a][b] = sum over the list of (y[a] - cy[a]) (x[b] - cx[b]); then
// kabsch_from_h (kabsch.cuh; the host ICP and the oracle use the same steps).
// GB300 issues an FP64 warp instruction at a fixed cost whatever the number of
// active lanes, so a one-thread refit pays for 32 lanes per operation; here
// values that do not depend on one another (the six centroid sums, the nine
// covariance sums, the rows of each Jacobi rotation, R and t) are computed by
// different lanes with one instruction stream.  Each value goes through the
// same operations in the same order as in the one-thread form (the
// translation unit is built without contraction), so every bit is the same.
// Every lane returns the fit.
__device__ __forceinline__ double pick3(int i, double a0, double a1, double a2) {
  return i == 0 ? a0 : (i == 1 ? a1 : a2);
}

__device__ void jacobi3_warp(double A[3][3], double V[3][3], double ev[3]) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int k = lane < 3 ? lane : (lane < 6 ? lane - 3 : 0);  // row of A (lanes 0-2) or of V (lanes 3-5)
  const bool vrow = lane >= 3 && lane < 6;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) V[i][j] = (i == j) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 24; ++sweep) {
    double off = fabs(A[0][1]) + fabs(A[0][2]) + fabs(A[1][2]);
    double scale = fabs(A[0][0]) + fabs(A[1][1]) + fabs(A[2][2]);
    if (off <= 1e-300 || off <= 1e-18 * scale) break;
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
      for (int q = p + 1; q < 3; ++q) {
        double apq = A[p][q];
        if (apq == 0.0) continue;  // A is the same in every lane: a uniform branch
        double theta = (A[q][q] - A[p][p]) / (2.0 * apq);
        double t = 1.0 / (fabs(theta) + sqrt(theta * theta + 1.0));
        if (theta < 0.0) t = -t;
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        // columns p, q of row k of A (lanes 0-2) and of V (lanes 3-5)
        {
          const double u = vrow ? pick3(k, V[0][p], V[1][p], V[2][p]) : pick3(k, A[0][p], A[1][p], A[2][p]);
          const double v = vrow ? pick3(k, V[0][q], V[1][q], V[2][q]) : pick3(k, A[0][q], A[1][q], A[2][q]);
          const double np = c * u - s * v, nq = s * u + c * v;
#pragma unroll
          for (int r = 0; r < 3; ++r) {
            A[r][p] = __shfl_sync(full, np, r);
            A[r][q] = __shfl_sync(full, nq, r);
            V[r][p] = __shfl_sync(full, np, 3 + r);
            V[r][q] = __shfl_sync(full, nq, 3 + r);
          }
        }
        // rows p, q of column k of A (lanes 0-2), from the updated columns
        {
          const double u = pick3(k, A[p][0], A[p][1], A[p][2]);
          const double v = pick3(k, A[q][0], A[q][1], A[q][2]);
          const double np = c * u - s * v, nq = s * u + c * v;
#pragma unroll
          for (int r = 0; r < 3; ++r) {
            A[p][r] = __shfl_sync(full, np, r);
            A[q][r] = __shfl_sync(full, nq, r);
          }
        }
      }
  }
  for (int i = 0; i < 3; ++i) ev[i] = A[i][i];
}

__device__ bool kabsch_warp(const float* x, const float* y, const int* idx, int n, double R[9], double t[3]) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  // centroids: lanes 0-2 sum x[.][lane], lanes 3-5 sum y[.][lane - 3], in list order
  const float* src = lane < 3 ? x : y;
  const int comp = lane < 3 ? lane : (lane < 6 ? lane - 3 : 0);
  double acc = 0.0;
  for (int i = 0; i < n; ++i) acc += (double)src[3 * idx[i] + comp];
  acc /= (double)n;
  double cx[3], cy[3];
  for (int a = 0; a < 3; ++a) {
    cx[a] = __shfl_sync(full, acc, a);
    cy[a] = __shfl_sync(full, acc, 3 + a);
  }
  // covariance H[a][b] = sum dy[a] dx[b]: lane 3a + b, in list order
  const int ha = lane < 9 ? lane / 3 : 0, hb = lane < 9 ? lane % 3 : 0;
  const double cya = pick3(ha, cy[0], cy[1], cy[2]), cxb = pick3(hb, cx[0], cx[1], cx[2]);
  double hs = 0.0;
  for (int i = 0; i < n; ++i) {
    const int k = idx[i];
    const double dy = (double)y[3 * k + ha] - cya;
    const double dx = (double)x[3 * k + hb] - cxb;
    hs += dy * dx;
  }
  double H[3][3];
  for (int r = 0; r < 9; ++r) H[r / 3][r % 3] = __shfl_sync(full, hs, r);
  // M = H^T H: lane 3i + j
  double ms = 0.0;
  for (int kk = 0; kk < 3; ++kk)
    ms += pick3(ha, H[kk][0], H[kk][1], H[kk][2]) * pick3(hb, H[kk][0], H[kk][1], H[kk][2]);
  double M[3][3], V[3][3], ev[3];
  for (int r = 0; r < 9; ++r) M[r / 3][r % 3] = __shfl_sync(full, ms, r);
  jacobi3_warp(M, V, ev);
  // the rest as in kabsch_from_h, the same in every lane
  int o[3] = {0, 1, 2};
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2 - i; ++j)
      if (ev[o[j]] < ev[o[j + 1]]) { int tmp = o[j]; o[j] = o[j + 1]; o[j + 1] = tmp; }
  double v[3][3], u[3][3];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) v[c][r] = V[r][o[c]];
  v[2][0] = v[0][1] * v[1][2] - v[0][2] * v[1][1];
  v[2][1] = v[0][2] * v[1][0] - v[0][0] * v[1][2];
  v[2][2] = v[0][0] * v[1][1] - v[0][1] * v[1][0];
  for (int c = 0; c < 2; ++c) {
    double hv[3], nn = 0.0;
    for (int r = 0; r < 3; ++r) {
      hv[r] = H[r][0] * v[c][0] + H[r][1] * v[c][1] + H[r][2] * v[c][2];
      nn += hv[r] * hv[r];
    }
    nn = sqrt(nn);
    if (!(nn > 1e-300)) return false;
    for (int r = 0; r < 3; ++r) u[c][r] = hv[r] / nn;
  }
  {
    double d = u[0][0] * u[1][0] + u[0][1] * u[1][1] + u[0][2] * u[1][2], nn = 0.0;
    for (int r = 0; r < 3; ++r) { u[1][r] = u[1][r] - d * u[0][r]; nn += u[1][r] * u[1][r]; }
    nn = sqrt(nn);
    if (!(nn > 1e-300)) return false;
    for (int r = 0; r < 3; ++r) u[1][r] = u[1][r] / nn;
  }
  u[2][0] = u[0][1] * u[1][2] - u[0][2] * u[1][1];
  u[2][1] = u[0][2] * u[1][0] - u[0][0] * u[1][2];
  u[2][2] = u[0][0] * u[1][1] - u[0][1] * u[1][0];
  // R[3i + j]: lane 3i + j
  const double rr = pick3(ha, v[0][0], v[0][1], v[0][2]) * pick3(hb, u[0][0], u[0][1], u[0][2]) +
                    pick3(ha, v[1][0], v[1][1], v[1][2]) * pick3(hb, u[1][0], u[1][1], u[1][2]) +
                    pick3(ha, v[2][0], v[2][1], v[2][2]) * pick3(hb, u[2][0], u[2][1], u[2][2]);
  for (int r = 0; r < 9; ++r) R[r] = __shfl_sync(full, rr, r);
  // t[i]: lane i
  const int ti = lane < 3 ? lane : 0;
  const double tt = pick3(ti, cx[0], cx[1], cx[2]) -
                    (pick3(ti, R[0], R[3], R[6]) * cy[0] + pick3(ti, R[1], R[4], R[7]) * cy[1] +
                     pick3(ti, R[2], R[5], R[8]) * cy[2]);
  for (int r = 0; r < 3; ++r) t[r] = __shfl_sync(full, tt, r);
  return true;
}

__device__ __forceinline__ bool is_inlier(const float* xi, const float* yi, const float Rf[9], const float tf[3],
                                          float thr2) {
  float px = Rf[0] * yi[0] + Rf[1] * yi[1] + Rf[2] * yi[2] + tf[0];
  float py = Rf[3] * yi[0] + Rf[4] * yi[1] + Rf[5] * yi[2] + tf[1];
  float pz = Rf[6] * yi[0] + Rf[7] * yi[1] + Rf[8] * yi[2] + tf[2];
  float ex = xi[0] - px, ey = xi[1] - py, ez = xi[2] - pz;
  float d2 = ex * ex + ey * ey + ez * ez;
  return d2 < thr2;
}

// Trial model for h, fitted in FP32 (false when the sample is degenerate).
__device__ bool trial_model(const float* x, const float* y, int m, uint64_t seed, uint32_t h, float Rf[9],
                            float tf[3]) {
  int s[3];
  sample3(seed, h, m, s);
  return kabsch3f(x, y, s, Rf, tf);
}

// One thread per trial; correspondences staged in shared memory (x then y).
__global__ __launch_bounds__(256) void trials_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                                     const int32_t* __restrict__ m_dev, int m_max, int smem_pts,
                                                     uint64_t seed, int iters, float thr, int32_t* __restrict__ counts,
                                                     float* __restrict__ models,
                                                     unsigned long long* __restrict__ best) {
  extern __shared__ float sp[];
  int m = *m_dev;
  m = m < m_max ? m : m_max;
  const bool staged = m <= smem_pts;
  if (staged) {
    for (int i = threadIdx.x; i < 3 * m; i += blockDim.x) {
      sp[i] = x[i];
      sp[3 * smem_pts + i] = y[i];
    }
  }
  __syncthreads();
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  // (count, trial) key of this thread's trial; threads past the last trial
  // hold 0, which no trial's key is below
  unsigned long long key = 0;
  if (h < iters) {
    int c = 0;
    if (m >= 3) {
      const float* xs = staged ? sp : x;
      const float* ys = staged ? sp + 3 * smem_pts : y;
      float Rf[9], tf[3];
      if (trial_model(xs, ys, m, seed, (uint32_t)h, Rf, tf)) {
        // kept for the winner: the finalize step reads it instead of refitting
        float4* mo = reinterpret_cast<float4*>(models + 12 * (int64_t)h);
        mo[0] = make_float4(Rf[0], Rf[1], Rf[2], Rf[3]);
        mo[1] = make_float4(Rf[4], Rf[5], Rf[6], Rf[7]);
        mo[2] = make_float4(Rf[8], tf[0], tf[1], tf[2]);
        const float thr2 = thr * thr;
        for (int i = 0; i < m; ++i) c += is_inlier(xs + 3 * i, ys + 3 * i, Rf, tf, thr2) ? 1 : 0;
      }
    }
    counts[h] = c;
    key = ((unsigned long long)(uint32_t)c << 32) | (unsigned long long)(uint32_t)h;
  }
  // the block's largest key takes one atomic (100k same-word atomics would
  // queue at one L2 slice); the max is order-free, so the winner is unchanged
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long other = __shfl_xor_sync(0xffffffffu, key, o);
    key = other > key ? other : key;
  }
  __shared__ unsigned long long s_key[8];
  if ((threadIdx.x & 31) == 0) s_key[threadIdx.x >> 5] = key;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) key = s_key[w] > key ? s_key[w] : key;
    atomicMax(best, key);
  }
}

// Winner, ordered inlier list and FP64 refit (one block).
__global__ __launch_bounds__(1024) void finalize_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                                        const int32_t* __restrict__ m_dev, int m_max, uint64_t seed,
                                                        int iters, float thr, int adaptive, int max_trials,
                                                        const int32_t* __restrict__ counts,
                                                        const float* __restrict__ models,
                                                        const unsigned long long* __restrict__ best,
                                                        double* __restrict__ rt, int32_t* __restrict__ inliers,
                                                        int32_t* __restrict__ info) {
  __shared__ int s_h, s_trials, s_ok;
  __shared__ float sR[9], st[3];
  __shared__ int s_warp[32];
  __shared__ int s_base, s_round;
  int m = *m_dev;
  m = m < m_max ? m : m_max;
  if (threadIdx.x == 0) {
    int h = -1, trials = iters;
    if (m >= 3 && iters > 0) {
      if (adaptive) {
        // ransac.m:139-221 loop replayed over the scored trials
        double N = 1.0, p = 0.99, eps = 2.220446049250313e-16;
        int bestscore = 0, tc = 0;
        while (N > (double)tc && tc < iters) {
          int c = counts[tc];
          if (c >= bestscore) {
            // a tie keeps N: it is a function of the count alone (the FP64
            // logarithms are the loop's slow part on this GPU)
            const bool grew = c > bestscore || h < 0;
            bestscore = c;
            h = tc;
            if (grew) {
              double w = (double)c / (double)m;
              double pno = 1.0 - w * w * w;
              if (pno < eps) pno = eps;
              if (pno > 1.0 - eps) pno = 1.0 - eps;
              N = log(1.0 - p) / log(pno);
              if (N < 10.0) N = 10.0;
            }
          }
          tc++;
          if (tc > max_trials) break;
        }
        trials = tc;
      } else {
        h = (int)(uint32_t)(*best & 0xFFFFFFFFull);
      }
    }
    s_h = h;
    s_trials = trials;
    s_ok = 0;
    if (h >= 0 && counts[h] > 0) {  // a positive count implies a valid trial model, stored by trials_kernel
      for (int i = 0; i < 9; ++i) sR[i] = models[12 * (int64_t)h + i];
      for (int i = 0; i < 3; ++i) st[i] = models[12 * (int64_t)h + 9 + i];
      s_ok = 1;
    }
    s_base = 0;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (s_ok) {
    const float thr2 = thr * thr;
    for (int i0 = 0; i0 < m; i0 += blockDim.x) {
      int i = i0 + threadIdx.x;
      int f = (i < m) && is_inlier(x + 3 * i, y + 3 * i, sR, st, thr2) ? 1 : 0;
      unsigned bal = __ballot_sync(0xffffffffu, f);
      int pre = __popc(bal & ((1u << lane) - 1));
      if (lane == 31) s_warp[w] = pre + f;
      __syncthreads();
      if (threadIdx.x == 0) {
        int acc = 0;
        for (int q = 0; q < nw; ++q) { int t = s_warp[q]; s_warp[q] = acc; acc += t; }
        s_round = acc;  // all 32 warps hold data: the total needs its own slot
      }
      __syncthreads();
      if (f) inliers[s_base + s_warp[w] + pre] = i;
      __syncthreads();
      if (threadIdx.x == 0) s_base += s_round;
      __syncthreads();
    }
  }
  if (threadIdx.x < 32) {  // warp 0: the refit (s_ok and s_base are block-uniform)
    int n = s_ok ? s_base : 0;
    double R[9], t[3];
    bool fit = n >= 3 && kabsch_warp(x, y, inliers, n, R, t);
    if (threadIdx.x != 0) return;
    for (int i = 0; i < 3; ++i) {
      for (int j = 0; j < 3; ++j) rt[4 * i + j] = fit ? R[3 * i + j] : (i == j ? 1.0 : 0.0);
      rt[4 * i + 3] = fit ? t[i] : 0.0;
    }
    info[0] = n;
    info[1] = s_h;
    info[2] = s_h >= 0 ? counts[s_h] : 0;
    info[3] = s_trials;
  }
}

__global__ void pairs_to_points_kernel(const float* __restrict__ ka, const float* __restrict__ kb,
                                       const int32_t* __restrict__ pairs, const int32_t* __restrict__ n_dev, int mx,
                                       float* __restrict__ x, float* __restrict__ y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int n = *n_dev;
  if (i >= mx || i >= n) return;
  int a = pairs[2 * i], b = pairs[2 * i + 1];
  for (int q = 0; q < 3; ++q) {
    x[3 * i + q] = ka[3 * a + q];
    y[3 * i + q] = kb[3 * b + q];
  }
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Raises trials_kernel's dynamic shared-memory cap (once per device).
cudaError_t trials_smem_cap() {
  return raise_smem_cap(reinterpret_cast<const void*>(trials_kernel), 6 * 4096 * 4);
}

}  // namespace
}  // namespace tdm

using namespace tdm;

// Workspace: best-trial word, one inlier count and one FP32 model (R, t:
// 12 floats) per trial.
extern "C" size_t tdm_ransac_workspace_bytes(int32_t m_max, int32_t iterations) {
  (void)m_max;
  if (iterations < 0) return 0;
  const size_t n = (size_t)(iterations > 0 ? iterations : 1);
  return align256(8) + align256(n * 4) + n * 48;
}

extern "C" tdm_status tdm_ransac(const float* x, const float* y, const int32_t* m_dev, int32_t m_max,
                                 const tdm_ransac_params* prm, double* rt, int32_t* inliers, int32_t* info, void* ws,
                                 size_t ws_bytes, tdm_stream s) {
  TDM_REQUIRE(x && y && m_dev && prm && rt && inliers && info && ws, "tdm_ransac: null pointer");
  TDM_REQUIRE(m_max >= 0 && prm->iterations >= 0 && prm->threshold > 0.0f, "tdm_ransac: bad parameters");
  TDM_REQUIRE(ws_bytes >= tdm_ransac_workspace_bytes(m_max, prm->iterations), "tdm_ransac: workspace too small");
  uint8_t* w = static_cast<uint8_t*>(ws);
  unsigned long long* best = reinterpret_cast<unsigned long long*>(w);
  int32_t* counts = reinterpret_cast<int32_t*>(w + align256(8));
  float* models = reinterpret_cast<float*>(w + align256(8) + align256((size_t)(prm->iterations > 0 ? prm->iterations : 1) * 4));
  TDM_CHECK_CUDA(cudaMemsetAsync(best, 0, 8, s));
  const int iters = prm->iterations;
  if (iters > 0) {
    int smem_pts = m_max <= 4096 ? m_max : 0;  // 96 KB of correspondences at most
    size_t smem = (size_t)6 * smem_pts * sizeof(float);
    TDM_CHECK_CUDA(trials_smem_cap());
    trials_kernel<<<(iters + 255) / 256, 256, smem, s>>>(x, y, m_dev, m_max, smem_pts, prm->seed, iters,
                                                          prm->threshold, counts, models, best);
    TDM_CHECK_LAUNCH("trials_kernel");
  }
  finalize_kernel<<<1, 1024, 0, s>>>(x, y, m_dev, m_max, prm->seed, iters, prm->threshold, prm->adaptive ? 1 : 0,
                                     prm->max_trials, counts, models, best, rt, inliers, info);
  TDM_CHECK_LAUNCH("finalize_kernel");
  return TDM_OK;
}

extern "C" tdm_status tdm_pairs_to_points(const float* ka, const float* kb, const int32_t* pairs,
                                          const int32_t* n_pairs, int32_t max_pairs, float* x, float* y,
                                          tdm_stream s) {
  TDM_REQUIRE(ka && kb && pairs && n_pairs && x && y && max_pairs >= 0, "tdm_pairs_to_points: bad arguments");
  if (max_pairs == 0) return TDM_OK;
  pairs_to_points_kernel<<<(max_pairs + 255) / 256, 256, 0, s>>>(ka, kb, pairs, n_pairs, max_pairs, x, y);
  TDM_CHECK_LAUNCH("pairs_to_points_kernel");
  return TDM_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free RANSAC.
//
// tdm_ransac needs a caller-provided device workspace (the best-trial word and
// one inlier count per trial).  Some callers cannot provide one: bindings that
// reach this library through a foreign-function layer holding no device
// allocator (a MATLAB loadlibrary/calllib binding, a scripting FFI that passes
// only pointers it was given), and serving loops that forbid cudaMalloc after
// start-up because it synchronizes the device and can fail under a memory
// budget.  For them this variant keeps its scratch in a fixed device array of
// this file, sized for kNoAllocMaxTrials trials (about 6.8 MB, held by every
// GPU that loads the library until the process exits).
//
// The array is shared by every call: the best-trial word is cleared at the
// start of each call and every trial count is rewritten, so a call never sees
// the previous call's results, but two calls whose work overlaps on the GPU
// (different streams, or different host threads) race on it and must be
// serialized by the caller.
// ---------------------------------------------------------------------------
namespace tdm {
namespace {

constexpr int kNoAllocMaxTrials = 131072;
constexpr size_t kNoAllocCountsOffset = 256;  // best word, padded; then counts
constexpr size_t kNoAllocModelsOffset = kNoAllocCountsOffset + 4 * (size_t)kNoAllocMaxTrials;  // then 12 floats per trial
static __device__ __align__(256) unsigned char g_ransac_scratch[kNoAllocModelsOffset + 48 * (size_t)kNoAllocMaxTrials];

// Device address of g_ransac_scratch, resolved once per device with that
// device current (the host-side symbol is only a stand-in, never a device
// address).
tdm_status noalloc_scratch(void** out) {
  static std::mutex mu;
  static std::vector<void*> addr;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  std::lock_guard<std::mutex> lk(mu);
  if ((int)addr.size() <= dev) addr.resize(dev + 1, nullptr);
  if (!addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_ransac_scratch);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_ransac_scratch)");
    addr[dev] = p;
  }
  *out = addr[dev];
  return TDM_OK;
}

}  // namespace
}  // namespace tdm

extern "C" tdm_status tdm_ransac_noalloc(const float* x, const float* y, const int32_t* m_dev, int32_t m_max,
                                         const tdm_ransac_params* prm, double* rt, int32_t* inliers,
                                         int32_t* info, tdm_stream s) {
  TDM_REQUIRE(x && y && m_dev && prm && rt && inliers && info, "tdm_ransac_noalloc: null pointer");
  TDM_REQUIRE(m_max >= 0 && prm->iterations >= 0 && prm->threshold > 0.0f, "tdm_ransac_noalloc: bad parameters");
  if (prm->iterations > kNoAllocMaxTrials)
    return fail(TDM_ERR_INVALID_ARG, "tdm_ransac_noalloc: iterations " + std::to_string(prm->iterations) +
                                         " exceed the fixed scratch of " + std::to_string(kNoAllocMaxTrials) +
                                         " trials; use tdm_ransac with a workspace");
  void* scratch = nullptr;
  tdm_status st = noalloc_scratch(&scratch);
  if (st) return st;
  uint8_t* w = static_cast<uint8_t*>(scratch);
  unsigned long long* best = reinterpret_cast<unsigned long long*>(w);
  int32_t* counts = reinterpret_cast<int32_t*>(w + kNoAllocCountsOffset);
  float* models = reinterpret_cast<float*>(w + kNoAllocModelsOffset);
  TDM_CHECK_CUDA(cudaMemsetAsync(best, 0, 8, s));  // the best word must start at zero
  const int iters = prm->iterations;
  if (iters > 0) {
    int smem_pts = m_max <= 4096 ? m_max : 0;
    size_t smem = (size_t)6 * smem_pts * sizeof(float);
    TDM_CHECK_CUDA(trials_smem_cap());
    trials_kernel<<<(iters + 255) / 256, 256, smem, s>>>(x, y, m_dev, m_max, smem_pts, prm->seed, iters,
                                                          prm->threshold, counts, models, best);
    TDM_CHECK_LAUNCH("trials_kernel (noalloc)");
  }
  finalize_kernel<<<1, 1024, 0, s>>>(x, y, m_dev, m_max, prm->seed, iters, prm->threshold, prm->adaptive ? 1 : 0,
                                     prm->max_trials, counts, models, best, rt, inliers, info);
  TDM_CHECK_LAUNCH("finalize_kernel (noalloc)");
  return TDM_OK;
}
