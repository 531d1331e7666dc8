/*
 * oracle.c -- CPU restatement of the 3DMatch registration hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA product is
 * compared against (tests/, __graft_entry__.smoke() and the CPU-baseline leg of
 * bench.py).  Nothing in the product links or calls it.
 *
 * Every function restates the reference's arithmetic from its source (paths are
 * relative to the andyzeng/3dmatch-toolbox tree):
 *   grid setup + occupancy ...... core/demo.cu:97-135
 *   TDF (per-voxel 11^3 loop) ... core/demo.cu:22-57 (both index decodes)
 *   keypoint grid coordinates ... core/demo.cu:164-177
 *   30^3 patch gather ........... core/demo.cu:195-218
 *   conv3d / ReLU / max-pool .... core/marvin.hpp:4634-4700, 5483, 5561-5587
 *                                 with the net of core/3dmatch-net-test.json
 *   mutual nearest neighbours ... core/demo.m:51-57
 *   RANSAC loop ................. core/external/peter/ransac.m:113-232,
 *                                 core/external/sfm/ransacfitRt.m:20-73
 *   TSDF integration ............ depth-fusion/demo.cu:18-68
 *   surface extraction .......... core/utils.hpp:23-65
 *
 * Compile with -ffp-contract=off: the float expressions must round exactly as
 * written (no fused multiply-add), on x86-64 and on aarch64 alike.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* Deterministic random streams (splitmix64, Steele/Lea/Flood 2014).          */
/* The product implements the same published generator; both sides derive    */
/* keypoint indices and RANSAC samples from (seed, counter) only.             */
/* ------------------------------------------------------------------------ */
static uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static uint64_t stream_u64(uint64_t seed, uint64_t counter) {
  return mix64(seed + (counter + 1) * 0x9E3779B97F4A7C15ULL);
}
static uint32_t bounded(uint64_t r, uint32_t n) { /* floor(r * n / 2^64) */
  return (uint32_t)(((unsigned __int128)r * n) >> 64);
}

/* Keypoint index stream: idx_i = floor(u_i * n_pts).  Replaces the
 * random_device-seeded GetRandomFloat of core/utils.hpp:15-20 (which cannot be
 * replayed) with a seeded stream. */
void orc_keypoint_indices(uint64_t seed, int n_pts, int k, int32_t* idx) {
  for (int i = 0; i < k; ++i) idx[i] = (int32_t)bounded(stream_u64(seed, (uint64_t)i), (uint32_t)n_pts);
}

/* Three distinct sample indices for RANSAC trial h (randsample(npts,3) in
 * ransac.m:153 draws without replacement). */
void orc_ransac_sample(uint64_t seed, uint32_t h, int m, int32_t out[3]) {
  uint32_t i0 = bounded(stream_u64(seed, 3ULL * h + 0), (uint32_t)m);
  uint32_t i1 = bounded(stream_u64(seed, 3ULL * h + 1), (uint32_t)(m - 1));
  uint32_t i2 = bounded(stream_u64(seed, 3ULL * h + 2), (uint32_t)(m - 2));
  if (i1 >= i0) i1++;
  uint32_t lo = i0 < i1 ? i0 : i1, hi = i0 < i1 ? i1 : i0;
  if (i2 >= lo) i2++;
  if (i2 >= hi) i2++;
  out[0] = (int32_t)i0; out[1] = (int32_t)i1; out[2] = (int32_t)i2;
}

/* ------------------------------------------------------------------------ */
/* Grid setup and occupancy: core/demo.cu:97-135                              */
/* ------------------------------------------------------------------------ */
void orc_grid_setup(const float* pts, int n, float voxel_size, int pad, int dim[3], float origin[3]) {
  float mn[3] = {pts[0], pts[1], pts[2]}, mx[3] = {pts[0], pts[1], pts[2]};
  for (int i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) {
      float v = pts[3 * i + a];
      if (v < mn[a]) mn[a] = v;
      if (v > mx[a]) mx[a] = v;
    }
  for (int a = 0; a < 3; ++a) {
    dim[a] = (int)roundf((mx[a] - mn[a]) / voxel_size) + 1 + pad * 2;
    origin[a] = mn[a] - (float)pad * voxel_size + voxel_size / 2.0f;
  }
}

/* occ[z*dy*dx + y*dx + x] = 1 with x = round((p - o) / vs).  Points that land
 * outside the grid, or have a non-finite coordinate, are skipped (the
 * reference has no check; with its padding and finite clouds neither occurs). */
void orc_occupancy(const float* pts, int n, const int dim[3], const float origin[3], float vs, uint8_t* occ) {
  size_t V = (size_t)dim[0] * dim[1] * dim[2];
  memset(occ, 0, V);
  for (int i = 0; i < n; ++i) {
    int g[3];
    if (!(isfinite(pts[3 * i]) && isfinite(pts[3 * i + 1]) && isfinite(pts[3 * i + 2]))) continue;
    for (int a = 0; a < 3; ++a) g[a] = (int)roundf((pts[3 * i + a] - origin[a]) / vs);
    if (g[0] < 0 || g[1] < 0 || g[2] < 0 || g[0] >= dim[0] || g[1] >= dim[1] || g[2] >= dim[2]) continue;
    occ[(size_t)g[2] * dim[1] * dim[0] + (size_t)g[1] * dim[0] + g[0]] = 1;
  }
}

/* Index decode of ComputeTDF (core/demo.cu:32-34).
 *  mode 0: exact integer decode (what the kernel means);
 *  mode 1: the reference's float32 expressions, evaluated without contraction;
 *  mode 2: the same expressions with nvcc's default multiply-add contraction
 *          (fmad=true), i.e. a - b*c evaluated as fma(-b, c, a). */
static void decode_voxel(int64_t idx, int dx, int dy, int mode, int* x, int* y, int* z) {
  if (mode == 0) {
    int64_t plane = (int64_t)dx * dy;
    *z = (int)(idx / plane);
    int64_t r = idx - (int64_t)(*z) * plane;
    *y = (int)(r / dx);
    *x = (int)(r - (int64_t)(*y) * dx);
    return;
  }
  float fi = (float)idx, fx = (float)dx, fy = (float)dy;
  int zz = (int)floorf(fi / (fx * fy));
  float zp = (float)zz * fx; /* ((float)z * (float)dx) */
  float u;
  if (mode == 1) u = fi - zp * fy;
  else u = fmaf(-zp, fy, fi);
  int yy = (int)floorf(u / fx);
  float xr;
  if (mode == 1) xr = u - (float)yy * fx;
  else xr = fmaf(-(float)yy, fx, u);
  *z = zz; *y = yy; *x = (int)xr;
}

/* Number of voxels whose decode under `mode` differs from the exact one. */
int64_t orc_count_misdecoded(const int dim[3], int mode) {
  int64_t V = (int64_t)dim[0] * dim[1] * dim[2], bad = 0;
#pragma omp parallel for reduction(+ : bad) schedule(static)
  for (int64_t i = 0; i < V; ++i) {
    int x0, y0, z0, x1, y1, z1;
    decode_voxel(i, dim[0], dim[1], 0, &x0, &y0, &z0);
    decode_voxel(i, dim[0], dim[1], mode, &x1, &y1, &z1);
    bad += (x0 != x1 || y0 != y1 || z0 != z1);
  }
  return bad;
}

/* The ComputeTDF loop (core/demo.cu:22-57) for voxels [v0, v1): occupied -> 1,
 * otherwise max(0, max over occupied voxels in the clipped (2r+1)^3 cube of
 * 1 - sqrtf(d^2)/r), r = round(trunc/vs). */
void orc_tdf_range(const uint8_t* occ, const int dim[3], float vs, float trunc, int mode,
                   int64_t v0, int64_t v1, float* tdf) {
  int dx = dim[0], dy = dim[1], dz = dim[2];
  int r = (int)roundf(trunc / vs);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t idx = v0; idx < v1; ++idx) {
    int x, y, z;
    decode_voxel(idx, dx, dy, mode, &x, &y, &z);
    if (occ[idx]) { tdf[idx - v0] = 1.0f; continue; }
    float best = 0.0f;
    int x0 = x - r > 0 ? x - r : 0, x1 = x + r + 1 < dx ? x + r + 1 : dx;
    int y0 = y - r > 0 ? y - r : 0, y1 = y + r + 1 < dy ? y + r + 1 : dy;
    int z0 = z - r > 0 ? z - r : 0, z1 = z + r + 1 < dz ? z + r + 1 : dz;
    for (int ix = x0; ix < x1; ++ix)
      for (int iy = y0; iy < y1; ++iy)
        for (int iz = z0; iz < z1; ++iz) {
          if (occ[(int64_t)iz * dx * dy + (int64_t)iy * dx + ix]) {
            float xd = (float)(x - ix), yd = (float)(y - iy), zd = (float)(z - iz);
            float dist = sqrtf(xd * xd + yd * yd + zd * zd) / (float)r;
            if (1.0f - dist > best) best = 1.0f - dist;
          }
        }
    tdf[idx - v0] = best;
  }
}

void orc_tdf(const uint8_t* occ, const int dim[3], float vs, float trunc, int mode, float* tdf) {
  orc_tdf_range(occ, dim, vs, trunc, mode, 0, (int64_t)dim[0] * dim[1] * dim[2], tdf);
}

/* Keypoints (core/demo.cu:168-176): keypts = pts[idx], grid = round((p-o)/vs). */
void orc_keypoints(const float* pts, const int32_t* idx, int k, const float origin[3], float vs,
                   float* keypts, int32_t* kp_grid) {
  for (int i = 0; i < k; ++i)
    for (int a = 0; a < 3; ++a) {
      float p = pts[3 * (int64_t)idx[i] + a];
      keypts[3 * i + a] = p;
      kp_grid[3 * i + a] = (int32_t)roundf((p - origin[a]) / vs);
    }
}

/* Patch gather (core/demo.cu:206-217): z,y,x in [k-15, k+14], x fastest.
 * Voxels outside the grid read as 0 (the reference reads out of bounds). */
void orc_gather(const float* tdf, const int dim[3], const int32_t* kp_grid, int k, float* patches) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < k; ++i) {
    float* out = patches + (int64_t)i * 27000;
    int n = 0;
    for (int z = kp_grid[3 * i + 2] - 15; z < kp_grid[3 * i + 2] + 15; ++z)
      for (int y = kp_grid[3 * i + 1] - 15; y < kp_grid[3 * i + 1] + 15; ++y)
        for (int x = kp_grid[3 * i + 0] - 15; x < kp_grid[3 * i + 0] + 15; ++x) {
          int in = x >= 0 && y >= 0 && z >= 0 && x < dim[0] && y < dim[1] && z < dim[2];
          out[n++] = in ? tdf[(int64_t)z * dim[0] * dim[1] + (int64_t)y * dim[0] + x] : 0.0f;
        }
  }
}

/* ------------------------------------------------------------------------ */
/* 3D ConvNet (core/3dmatch-net-test.json, Marvin ConvolutionLayer semantics) */
/* Activations channels-last [B][D][D][D][C]; weights as Marvin stores them,  */
/* [K][C][3][3][3] (dims z,y,x), cross-correlation, stride 1, no padding.      */
/* ------------------------------------------------------------------------ */
#define DEFINE_CONV(T, NAME)                                                                        \
  void NAME(const T* in, int B, int D, int C, const float* w, const float* bias, int K, int ks,     \
            int relu, T* out) {                                                                     \
    int Do = D - ks + 1, taps = ks * ks * ks;                                                       \
    /* transpose weights to [tap][c][k] so the k loop is contiguous */                              \
    T* wt = (T*)malloc(sizeof(T) * (size_t)taps * C * K);                                           \
    for (int k = 0; k < K; ++k)                                                                     \
      for (int c = 0; c < C; ++c)                                                                   \
        for (int t = 0; t < taps; ++t) wt[((size_t)t * C + c) * K + k] = (T)w[((size_t)k * C + c) * taps + t]; \
    int64_t M = (int64_t)B * Do * Do * Do;                                                          \
    _Pragma("omp parallel")                                                                         \
    {                                                                                               \
      T* acc = (T*)malloc(sizeof(T) * K);                                                           \
      _Pragma("omp for schedule(static)")                                                           \
      for (int64_t m = 0; m < M; ++m) {                                                             \
        int x = (int)(m % Do), y = (int)((m / Do) % Do), z = (int)((m / Do / Do) % Do);             \
        int64_t b = m / ((int64_t)Do * Do * Do);                                                    \
        for (int k = 0; k < K; ++k) acc[k] = 0;                                                     \
        for (int t = 0; t < taps; ++t) {                                                            \
          int tz = t / (ks * ks), ty = (t / ks) % ks, tx = t % ks;                                  \
          const T* row = in + ((((b * D + z + tz) * D + y + ty) * D + x + tx) * (int64_t)C);        \
          const T* wtt = wt + (size_t)t * C * K;                                                    \
          for (int c = 0; c < C; ++c) {                                                             \
            T a = row[c];                                                                           \
            const T* wk = wtt + (size_t)c * K;                                                      \
            for (int k = 0; k < K; ++k) acc[k] += a * wk[k];                                        \
          }                                                                                         \
        }                                                                                           \
        T* o = out + m * K;                                                                         \
        for (int k = 0; k < K; ++k) {                                                               \
          T v = acc[k] + (T)bias[k];                                                                \
          o[k] = (relu && v < 0) ? (T)0 : v;                                                        \
        }                                                                                           \
      }                                                                                             \
      free(acc);                                                                                    \
    }                                                                                               \
    free(wt);                                                                                       \
  }

DEFINE_CONV(float, orc_conv3d_f32)
DEFINE_CONV(double, orc_conv3d_f64)

/* Max-pool 2^3 stride 2 (core/marvin.hpp:5561-5587); D even in this net. */
#define DEFINE_POOL(T, NAME)                                                                        \
  void NAME(const T* in, int B, int D, int C, T* out) {                                             \
    int Do = (D + 1) / 2;                                                                           \
    int64_t M = (int64_t)B * Do * Do * Do;                                                          \
    _Pragma("omp parallel for schedule(static)")                                                    \
    for (int64_t m = 0; m < M; ++m) {                                                               \
      int x = (int)(m % Do), y = (int)((m / Do) % Do), z = (int)((m / Do / Do) % Do);               \
      int64_t b = m / ((int64_t)Do * Do * Do);                                                      \
      for (int c = 0; c < C; ++c) {                                                                 \
        T best = -INFINITY;                                                                         \
        for (int dz = 0; dz < 2; ++dz)                                                              \
          for (int dy = 0; dy < 2; ++dy)                                                            \
            for (int dx = 0; dx < 2; ++dx) {                                                        \
              int zz = 2 * z + dz, yy = 2 * y + dy, xx = 2 * x + dx;                                \
              if (zz >= D || yy >= D || xx >= D) continue;                                          \
              T v = in[(((b * D + zz) * D + yy) * D + xx) * (int64_t)C + c];                        \
              if (v > best) best = v;                                                               \
            }                                                                                       \
        out[m * C + c] = best;                                                                      \
      }                                                                                             \
    }                                                                                               \
  }

DEFINE_POOL(float, orc_pool_f32)
DEFINE_POOL(double, orc_pool_f64)

/* Layer table of core/3dmatch-net-test.json: conv1..conv8 (+ReLU), pool after
 * conv2, then feat (1x1x1, 512->512, no ReLU). */
static const int NET_COUT[9] = {64, 64, 128, 128, 256, 256, 512, 512, 512};
static const int NET_KS[9] = {3, 3, 3, 3, 3, 3, 3, 3, 1};

/* Forward B patches [B][30^3] -> desc [B][512].  weights[l] is [K][C][ks^3]
 * float, biases[l] is [K]; use_feat=0 stops after conv8 (+ReLU). */
#define DEFINE_NET(T, NAME, CONV, POOL)                                                              \
  void NAME(const float* patches, int B, const float* const* weights, const float* const* biases,   \
            int use_feat, T* desc) {                                                                \
    int D = 30, C = 1;                                                                              \
    T* cur = (T*)malloc(sizeof(T) * (size_t)B * 27000);                                             \
    for (int64_t i = 0; i < (int64_t)B * 27000; ++i) cur[i] = (T)patches[i];                        \
    int nl = use_feat ? 9 : 8;                                                                      \
    for (int l = 0; l < nl; ++l) {                                                                  \
      int K = NET_COUT[l], ks = NET_KS[l], Do = D - ks + 1;                                         \
      T* nxt = (T*)malloc(sizeof(T) * (size_t)B * Do * Do * Do * K);                                \
      CONV(cur, B, D, C, weights[l], biases[l], K, ks, l < 8, nxt);                                 \
      free(cur); cur = nxt; D = Do; C = K;                                                          \
      if (l == 1) {                                                                                 \
        int Dp = (D + 1) / 2;                                                                       \
        T* p = (T*)malloc(sizeof(T) * (size_t)B * Dp * Dp * Dp * C);                                \
        POOL(cur, B, D, C, p);                                                                      \
        free(cur); cur = p; D = Dp;                                                                 \
      }                                                                                             \
    }                                                                                               \
    memcpy(desc, cur, sizeof(T) * (size_t)B * 512);                                                 \
    free(cur);                                                                                      \
  }

DEFINE_NET(float, orc_net_forward_f32, orc_conv3d_f32, orc_pool_f32)
DEFINE_NET(double, orc_net_forward_f64, orc_conv3d_f64, orc_pool_f64)

/* ------------------------------------------------------------------------ */
/* Mutual nearest neighbours (core/demo.m:51-57), exact in double.            */
/* dist(i,j) = sum_k (double)(a_ik - b_jk)^2, summed in k order with fma.     */
/* Ties go to the lowest index.                                               */
/* ------------------------------------------------------------------------ */
static double sqdist_f64(const float* a, const float* b, int dim) {
  double s = 0.0;
  for (int k = 0; k < dim; ++k) {
    double d = (double)a[k] - (double)b[k];
    s = fma(d, d, s);
  }
  return s;
}

/* Eight reference rows at a time: independent accumulation chains, each one
 * still summed in k order, so every distance equals sqdist_f64's. */
void orc_nn(const float* q, int nq, const float* ref, int nr, int dim, int32_t* nn) {
#pragma omp parallel for schedule(dynamic, 8)
  for (int i = 0; i < nq; ++i) {
    const float* a = q + (int64_t)i * dim;
    double best = INFINITY;
    int bj = 0;
    int j = 0;
    for (; j + 8 <= nr; j += 8) {
      double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      for (int k = 0; k < dim; ++k) {
        double ak = (double)a[k];
        for (int u = 0; u < 8; ++u) {
          double d = ak - (double)ref[(int64_t)(j + u) * dim + k];
          s[u] = fma(d, d, s[u]);
        }
      }
      for (int u = 0; u < 8; ++u)
        if (s[u] < best) { best = s[u]; bj = j + u; }
    }
    for (; j < nr; ++j) {
      double d = sqdist_f64(a, ref + (int64_t)j * dim, dim);
      if (d < best) { best = d; bj = j; }
    }
    nn[i] = bj;
  }
}

/* pairs[2*m] = (index into A, index into B), in increasing B index. */
int orc_mutual_nn(const float* da, int na, const float* db, int nb, int dim, int32_t* nn_ab, int32_t* nn_ba,
                  int32_t* pairs) {
  orc_nn(da, na, db, nb, dim, nn_ab);
  orc_nn(db, nb, da, na, dim, nn_ba);
  int m = 0;
  for (int j = 0; j < nb; ++j)
    if (nn_ab[nn_ba[j]] == j) { pairs[2 * m] = nn_ba[j]; pairs[2 * m + 1] = j; ++m; }
  return m;
}

/* ------------------------------------------------------------------------ */
/* Rigid fit, x = R y + t, least squares (Kabsch): FP64 covariance, SVD of the */
/* 3x3 cross-covariance through the Jacobi eigen-decomposition of H^T H.       */
/* The CUDA product performs the same operation sequence so RANSAC trials     */
/* score identically.                                                         */
/* ------------------------------------------------------------------------ */
static void jacobi3(double A[3][3], double V[3][3], double ev[3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) V[i][j] = (i == j) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 24; ++sweep) {
    double off = fabs(A[0][1]) + fabs(A[0][2]) + fabs(A[1][2]);
    double scale = fabs(A[0][0]) + fabs(A[1][1]) + fabs(A[2][2]);
    if (off <= 1e-300 || off <= 1e-18 * scale) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        double apq = A[p][q];
        if (apq == 0.0) continue;
        double theta = (A[q][q] - A[p][p]) / (2.0 * apq);
        double t = 1.0 / (fabs(theta) + sqrt(theta * theta + 1.0));
        if (theta < 0.0) t = -t;
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; ++k) { /* A <- A J (columns p,q) */
          double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - s * akq;
          A[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) { /* A <- J^T A (rows p,q) */
          double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - s * aqk;
          A[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          double vkp = V[k][p], vkq = V[k][q];
          V[k][p] = c * vkp - s * vkq;
          V[k][q] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < 3; ++i) ev[i] = A[i][i];
}

/* R (row-major 3x3) and t from centred cross-covariance H = sum (y-cy)(x-cx)^T.
 * Returns 0 on success, -1 when the fit is degenerate (rank < 2). */
static int kabsch_from_h(const double H[3][3], const double cx[3], const double cy[3], double R[9], double t[3]) {
  double M[3][3], V[3][3], ev[3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s += H[k][i] * H[k][j];
      M[i][j] = s;
    }
  jacobi3(M, V, ev);
  /* order eigenpairs by decreasing eigenvalue (stable) */
  int o[3] = {0, 1, 2};
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2 - i; ++j)
      if (ev[o[j]] < ev[o[j + 1]]) { int tmp = o[j]; o[j] = o[j + 1]; o[j + 1] = tmp; }
  double v[3][3], u[3][3]; /* columns */
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) v[c][r] = V[r][o[c]];
  /* v3 = v1 x v2 keeps V right-handed */
  v[2][0] = v[0][1] * v[1][2] - v[0][2] * v[1][1];
  v[2][1] = v[0][2] * v[1][0] - v[0][0] * v[1][2];
  v[2][2] = v[0][0] * v[1][1] - v[0][1] * v[1][0];
  for (int c = 0; c < 2; ++c) {
    double hv[3], n = 0.0;
    for (int r = 0; r < 3; ++r) {
      hv[r] = H[r][0] * v[c][0] + H[r][1] * v[c][1] + H[r][2] * v[c][2];
      n += hv[r] * hv[r];
    }
    n = sqrt(n);
    if (!(n > 1e-300)) return -1;
    for (int r = 0; r < 3; ++r) u[c][r] = hv[r] / n;
  }
  /* u2 <- u2 - (u1.u2) u1, renormalised (guards tiny eigen-gaps) */
  {
    double d = u[0][0] * u[1][0] + u[0][1] * u[1][1] + u[0][2] * u[1][2], n = 0.0;
    for (int r = 0; r < 3; ++r) { u[1][r] = u[1][r] - d * u[0][r]; n += u[1][r] * u[1][r]; }
    n = sqrt(n);
    if (!(n > 1e-300)) return -1;
    for (int r = 0; r < 3; ++r) u[1][r] = u[1][r] / n;
  }
  u[2][0] = u[0][1] * u[1][2] - u[0][2] * u[1][1];
  u[2][1] = u[0][2] * u[1][0] - u[0][0] * u[1][2];
  u[2][2] = u[0][0] * u[1][1] - u[0][1] * u[1][0];
  /* With both bases right-handed, R = V U^T is the proper rotation that
   * Kabsch's diag(1,1,sign det) correction selects. */
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[3 * i + j] = v[0][i] * u[0][j] + v[1][i] * u[1][j] + v[2][i] * u[2][j];
  for (int i = 0; i < 3; ++i) t[i] = cx[i] - (R[3 * i] * cy[0] + R[3 * i + 1] * cy[1] + R[3 * i + 2] * cy[2]);
  return 0;
}

/* Fit x = R y + t on the listed correspondences (idx == NULL: all n). */
int orc_kabsch(const float* x, const float* y, const int32_t* idx, int n, double R[9], double t[3]) {
  double cx[3] = {0, 0, 0}, cy[3] = {0, 0, 0};
  for (int i = 0; i < n; ++i) {
    int k = idx ? idx[i] : i;
    for (int a = 0; a < 3; ++a) { cx[a] += (double)x[3 * k + a]; cy[a] += (double)y[3 * k + a]; }
  }
  for (int a = 0; a < 3; ++a) { cx[a] /= (double)n; cy[a] /= (double)n; }
  double H[3][3] = {{0}};
  for (int i = 0; i < n; ++i) {
    int k = idx ? idx[i] : i;
    double dx[3], dy[3];
    for (int a = 0; a < 3; ++a) { dx[a] = (double)x[3 * k + a] - cx[a]; dy[a] = (double)y[3 * k + a] - cy[a]; }
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) H[a][b] += dy[a] * dx[b];
  }
  return kabsch_from_h(H, cx, cy, R, t);
}

/* RANSAC trial fit in FP32 on the three sampled correspondences: the same
 * steps as jacobi3 / kabsch_from_h in single precision (16 sweeps at most,
 * stop when the off-diagonal sum is below 1e-6 of the diagonal).  The trial
 * model is used in FP32 for the inlier tests; the final refit stays FP64
 * (estimateRt.m in ransacfitRt.m:37). */
static void jacobi3f(float A[3][3], float V[3][3], float ev[3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) V[i][j] = (i == j) ? 1.0f : 0.0f;
  for (int sweep = 0; sweep < 16; ++sweep) {
    float off = fabsf(A[0][1]) + fabsf(A[0][2]) + fabsf(A[1][2]);
    float scale = fabsf(A[0][0]) + fabsf(A[1][1]) + fabsf(A[2][2]);
    if (off <= 1e-30f || off <= 1e-6f * scale) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        float apq = A[p][q];
        if (apq == 0.0f) continue;
        float theta = (A[q][q] - A[p][p]) / (2.0f * apq);
        float t = 1.0f / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
        if (theta < 0.0f) t = -t;
        float c = 1.0f / sqrtf(t * t + 1.0f), s = t * c;
        for (int k = 0; k < 3; ++k) {
          float akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - s * akq;
          A[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {
          float apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - s * aqk;
          A[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          float vkp = V[k][p], vkq = V[k][q];
          V[k][p] = c * vkp - s * vkq;
          V[k][q] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < 3; ++i) ev[i] = A[i][i];
}

static int kabsch3f(const float* x, const float* y, const int32_t s[3], float R[9], float t[3]) {
  float cx[3], cy[3];
  for (int a = 0; a < 3; ++a) {
    cx[a] = ((x[3 * s[0] + a] + x[3 * s[1] + a]) + x[3 * s[2] + a]) / 3.0f;
    cy[a] = ((y[3 * s[0] + a] + y[3 * s[1] + a]) + y[3 * s[2] + a]) / 3.0f;
  }
  float H[3][3] = {{0.0f}};
  for (int i = 0; i < 3; ++i) {
    float dx[3], dy[3];
    for (int a = 0; a < 3; ++a) { dx[a] = x[3 * s[i] + a] - cx[a]; dy[a] = y[3 * s[i] + a] - cy[a]; }
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) H[a][b] += dy[a] * dx[b];
  }
  float M[3][3], V[3][3], ev[3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      float acc = 0.0f;
      for (int k = 0; k < 3; ++k) acc += H[k][i] * H[k][j];
      M[i][j] = acc;
    }
  jacobi3f(M, V, ev);
  int o[3] = {0, 1, 2};
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2 - i; ++j)
      if (ev[o[j]] < ev[o[j + 1]]) { int tmp = o[j]; o[j] = o[j + 1]; o[j + 1] = tmp; }
  float v[3][3], u[3][3];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) v[c][r] = V[r][o[c]];
  v[2][0] = v[0][1] * v[1][2] - v[0][2] * v[1][1];
  v[2][1] = v[0][2] * v[1][0] - v[0][0] * v[1][2];
  v[2][2] = v[0][0] * v[1][1] - v[0][1] * v[1][0];
  for (int c = 0; c < 2; ++c) {
    float hv[3], n = 0.0f;
    for (int r = 0; r < 3; ++r) {
      hv[r] = H[r][0] * v[c][0] + H[r][1] * v[c][1] + H[r][2] * v[c][2];
      n += hv[r] * hv[r];
    }
    n = sqrtf(n);
    if (!(n > 1e-30f)) return -1;
    for (int r = 0; r < 3; ++r) u[c][r] = hv[r] / n;
  }
  {
    float d = u[0][0] * u[1][0] + u[0][1] * u[1][1] + u[0][2] * u[1][2], n = 0.0f;
    for (int r = 0; r < 3; ++r) { u[1][r] = u[1][r] - d * u[0][r]; n += u[1][r] * u[1][r]; }
    n = sqrtf(n);
    if (!(n > 1e-30f)) return -1;
    for (int r = 0; r < 3; ++r) u[1][r] = u[1][r] / n;
  }
  u[2][0] = u[0][1] * u[1][2] - u[0][2] * u[1][1];
  u[2][1] = u[0][2] * u[1][0] - u[0][0] * u[1][2];
  u[2][2] = u[0][0] * u[1][1] - u[0][1] * u[1][0];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[3 * i + j] = v[0][i] * u[0][j] + v[1][i] * u[1][j] + v[2][i] * u[2][j];
  for (int i = 0; i < 3; ++i) t[i] = cx[i] - (R[3 * i] * cy[0] + R[3 * i + 1] * cy[1] + R[3 * i + 2] * cy[2]);
  return 0;
}

/* Exported for the tests: the FP32 trial fit on the listed three correspondences. */
int orc_kabsch3f(const float* x, const float* y, const int32_t s[3], float R[9], float t[3]) {
  return kabsch3f(x, y, s, R, t);
}

/* Inlier count of model (R,t) in float: |x - (R y + t)|^2 < thr^2, strict as
 * euc3Ddist in ransacfitRt.m:51-61. */
static int count_inliers(const float* x, const float* y, int m, const float Rf[9], const float tf[3], float thr2,
                         int32_t* list) {
  int cnt = 0;
  for (int i = 0; i < m; ++i) {
    float px = Rf[0] * y[3 * i] + Rf[1] * y[3 * i + 1] + Rf[2] * y[3 * i + 2] + tf[0];
    float py = Rf[3] * y[3 * i] + Rf[4] * y[3 * i + 1] + Rf[5] * y[3 * i + 2] + tf[1];
    float pz = Rf[6] * y[3 * i] + Rf[7] * y[3 * i + 1] + Rf[8] * y[3 * i + 2] + tf[2];
    float ex = x[3 * i] - px, ey = x[3 * i + 1] - py, ez = x[3 * i + 2] - pz;
    float d2 = ex * ex + ey * ey + ez * ez;
    if (d2 < thr2) { if (list) list[cnt] = i; ++cnt; }
  }
  return cnt;
}

/* One RANSAC trial: sample, fit, score.  Returns the inlier count (0 when the
 * sample is degenerate). */
int orc_ransac_trial(const float* x, const float* y, int m, uint64_t seed, uint32_t h, float thr, float Rf[9],
                     float tf[3]) {
  int32_t s[3];
  orc_ransac_sample(seed, h, m, s);
  if (kabsch3f(x, y, s, Rf, tf) != 0) return 0;
  return count_inliers(x, y, m, Rf, tf, thr * thr, NULL);
}

/* Fixed-trial RANSAC: every trial h in [0, iters) is scored; the best count
 * wins and ties go to the later trial (ransac.m:194 uses >=).  counts[] (may
 * be NULL) receives every trial's count.  The final model is the FP64 Kabsch
 * refit on the winner's inliers (ransacfitRt.m:37).  Returns #inliers. */
int orc_ransac(const float* x, const float* y, int m, uint64_t seed, int iters, float thr, int32_t* counts,
               int32_t* best_trial, int32_t* inliers, double Rt[12]) {
  int best = -1, bh = -1;
#pragma omp parallel
  {
    int lbest = -1, lbh = -1;
#pragma omp for schedule(static)
    for (int h = 0; h < iters; ++h) {
      float Rf[9], tf[3];
      int c = orc_ransac_trial(x, y, m, seed, (uint32_t)h, thr, Rf, tf);
      if (counts) counts[h] = c;
      if (c > lbest || (c == lbest && h > lbh)) { lbest = c; lbh = h; }
    }
#pragma omp critical
    {
      if (lbest > best || (lbest == best && lbh > bh)) { best = lbest; bh = lbh; }
    }
  }
  *best_trial = bh;
  float Rf[9], tf[3];
  int32_t s[3];
  orc_ransac_sample(seed, (uint32_t)bh, m, s);
  double R[9], t[3];
  int n = 0;
  if (best > 0 && kabsch3f(x, y, s, Rf, tf) == 0) n = count_inliers(x, y, m, Rf, tf, thr * thr, inliers);
  if (n >= 3 && orc_kabsch(x, y, inliers, n, R, t) == 0) {
    for (int i = 0; i < 3; ++i) {
      for (int j = 0; j < 3; ++j) Rt[4 * i + j] = R[3 * i + j];
      Rt[4 * i + 3] = t[i];
    }
  } else {
    for (int i = 0; i < 12; ++i) Rt[i] = (i % 5 == 0) ? 1.0 : 0.0;
  }
  return n;
}

/* Reference-compatible stopping rule of ransac.m:139-221 replayed over a
 * precomputed count sequence: N = log(1-p)/log(1-w^3) refreshed whenever a
 * trial ties or beats the best, at least 10, at most max_trials + 1 trials.
 * Returns the number of trials the adaptive loop runs; *best_trial gets the
 * trial whose model it keeps. */
int orc_ransac_adaptive_stop(const int32_t* counts, int n_trials, int m, int max_trials, int32_t* best_trial) {
  double N = 1.0, p = 0.99, eps = 2.220446049250313e-16;
  int bestscore = 0, trialcount = 0, bh = -1;
  while (N > (double)trialcount && trialcount < n_trials) {
    int c = counts[trialcount];
    if (c >= bestscore) {
      bestscore = c; bh = trialcount;
      double w = (double)c / (double)m;
      double pno = 1.0 - w * w * w;
      if (pno < eps) pno = eps;
      if (pno > 1.0 - eps) pno = 1.0 - eps;
      N = log(1.0 - p) / log(pno);
      if (N < 10.0) N = 10.0;
    }
    trialcount++;
    if (trialcount > max_trials) break;
  }
  *best_trial = bh;
  return trialcount;
}

/* ------------------------------------------------------------------------ */
/* TSDF integration, depth-fusion/demo.cu:18-68, one frame.                   */
/* ------------------------------------------------------------------------ */
/* Voxels with z in [z0, z1) only (z1 <= 0 means all); tsdf/weight are the
 * full grid arrays. */
void orc_tsdf_integrate_z(const float K[9], const float c2b[16], const float* depth, int H, int W, const int dim[3],
                          const float origin[3], float vs, float trunc, int z0, int z1, float* tsdf, float* weight) {
  int dx = dim[0], dy = dim[1], dz = dim[2];
  if (z1 <= 0 || z1 > dz) z1 = dz;
#pragma omp parallel for schedule(static)
  for (int z = z0; z < z1; ++z)
    for (int y = 0; y < dy; ++y)
      for (int x = 0; x < dx; ++x) {
        float bx = origin[0] + (float)x * vs, by = origin[1] + (float)y * vs, bz = origin[2] + (float)z * vs;
        float t0 = bx - c2b[3], t1 = by - c2b[7], t2 = bz - c2b[11];
        float cx = c2b[0] * t0 + c2b[4] * t1 + c2b[8] * t2;
        float cy = c2b[1] * t0 + c2b[5] * t1 + c2b[9] * t2;
        float cz = c2b[2] * t0 + c2b[6] * t1 + c2b[10] * t2;
        if (cz <= 0) continue;
        int px = (int)roundf(K[0] * (cx / cz) + K[2]);
        int py = (int)roundf(K[4] * (cy / cz) + K[5]);
        if (px < 0 || px >= W || py < 0 || py >= H) continue;
        float d = depth[py * W + px];
        if (d <= 0 || d > 6) continue;
        float qx = cx / cz, qy = cy / cz;
        float diff = (d - cz) * sqrtf(1 + qx * qx + qy * qy);
        if (diff <= -trunc) continue;
        int64_t v = (int64_t)z * dy * dx + (int64_t)y * dx + x;
        float dist = fminf(1.0f, diff / trunc);
        float wo = weight[v], wn = wo + 1.0f;
        weight[v] = wn;
        tsdf[v] = (tsdf[v] * wo + dist) / wn;
      }
}

void orc_tsdf_integrate(const float K[9], const float c2b[16], const float* depth, int H, int W, const int dim[3],
                        const float origin[3], float vs, float trunc, float* tsdf, float* weight) {
  orc_tsdf_integrate_z(K, c2b, depth, H, W, dim, origin, vs, trunc, 0, 0, tsdf, weight);
}

/* Surface points (core/utils.hpp:23-65): voxel centres o + i*vs where
 * |tsdf| < tsdf_thr and weight > w_thr, in linear index order.  Returns the
 * count; pts may be NULL to count only. */
int64_t orc_extract_surface(const float* tsdf, const float* weight, const int dim[3], const float origin[3], float vs,
                            float tsdf_thr, float w_thr, float* pts) {
  int64_t V = (int64_t)dim[0] * dim[1] * dim[2], n = 0;
  for (int64_t i = 0; i < V; ++i) {
    if (fabsf(tsdf[i]) < tsdf_thr && weight[i] > w_thr) {
      if (pts) {
        int64_t z = i / ((int64_t)dim[0] * dim[1]);
        int64_t y = (i - z * dim[0] * dim[1]) / dim[0];
        int64_t x = i - z * dim[0] * dim[1] - y * dim[0];
        pts[3 * n + 0] = origin[0] + (float)x * vs;
        pts[3 * n + 1] = origin[1] + (float)y * vs;
        pts[3 * n + 2] = origin[2] + (float)z * vs;
      }
      ++n;
    }
  }
  return n;
}

/* Surface overlap (core/demo.m:66-72, register2Fragments.m:90-97): counts[0]
 * = points of a with a point of Rt*b closer than radius, counts[1] = points
 * of Rt*b with a point of a closer than radius, by brute force.  b is moved
 * in float with R, t rounded from double: ((R0 x + R1 y) + R2 z) + t;
 * d2 = (dx dx + dy dy) + dz dz < radius * radius in float. */
void orc_overlap(const float* a, int na, const float* b, int nb, const double rt[12], float radius, int32_t counts[2]) {
  float R[9] = {(float)rt[0], (float)rt[1], (float)rt[2], (float)rt[4], (float)rt[5],
                (float)rt[6], (float)rt[8], (float)rt[9], (float)rt[10]};
  float t[3] = {(float)rt[3], (float)rt[7], (float)rt[11]};
  float* bt = (float*)malloc(sizeof(float) * 3 * (size_t)nb);
  for (int i = 0; i < nb; ++i)
    for (int r = 0; r < 3; ++r) {
      float v = R[3 * r] * b[3 * i];
      v = v + R[3 * r + 1] * b[3 * i + 1];
      v = v + R[3 * r + 2] * b[3 * i + 2];
      bt[3 * i + r] = v + t[r];
    }
  const float r2 = radius * radius;
  const float* q[2] = {a, bt};
  const float* ref[2] = {bt, a};
  const int nq[2] = {na, nb}, nr[2] = {nb, na};
  for (int dir = 0; dir < 2; ++dir) {
    int32_t cnt = 0;
#pragma omp parallel for reduction(+ : cnt) schedule(dynamic, 256)
    for (int i = 0; i < nq[dir]; ++i) {
      const float* p = q[dir] + 3 * (size_t)i;
      for (int j = 0; j < nr[dir]; ++j) {
        const float* s = ref[dir] + 3 * (size_t)j;
        float dx = p[0] - s[0], dy = p[1] - s[1], dz = p[2] - s[2];
        float d2 = dx * dx + dy * dy;
        d2 = d2 + dz * dz;
        if (d2 < r2) {
          ++cnt;
          break;
        }
      }
    }
    counts[dir] = cnt;
  }
  free(bt);
}

/* Exact TDF (evaluation/model-fitting-apc/pointCloud2TDF.m): for every voxel
 * centre c = o + i vs (double), d = distance to the nearest point (double,
 * brute force over the points), tdf = 1 - min(d / trunc, 1). */
void orc_tdf_exact(const float* pts, int n, const int dim[3], const float origin[3], float vs, float trunc, float* tdf) {
  const int64_t V = (int64_t)dim[0] * dim[1] * dim[2];
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t v = 0; v < V; ++v) {
    const int64_t z = v / ((int64_t)dim[0] * dim[1]);
    const int64_t y = (v / dim[0]) % dim[1];
    const int64_t x = v % dim[0];
    const double c[3] = {(double)origin[0] + x * (double)vs, (double)origin[1] + y * (double)vs,
                         (double)origin[2] + z * (double)vs};
    double best = INFINITY;
    for (int i = 0; i < n; ++i) {
      const double ex = c[0] - pts[3 * i], ey = c[1] - pts[3 * i + 1], ez = c[2] - pts[3 * i + 2];
      const double d2 = ex * ex + ey * ey + ez * ez;
      if (d2 < best) best = d2;
    }
    const double t = sqrt(best) / trunc;
    tdf[v] = (float)(1.0 - (t < 1.0 ? t : 1.0));
  }
}
