// Per-voxel, per-tile and per-keypoint arithmetic shared by the single-fragment
// entry points (tdf.cu) and the batched form (batch.cu), so both give the same
// bits by construction.  Geometry follows core/demo.cu:97-135, keypoints
// core/demo.cu:164-177, the patch gather core/demo.cu:206-217.
#pragma once

#include <cmath>
#include <cstdint>

#include "tdm.h"

namespace tdm {

// Grid axis, core/demo.cu:109-118: dim = round(ext / vs) + 1 + 2 pad,
// origin = min - pad * vs + vs / 2.  Plain IEEE float operations: host code is
// compiled without contraction and device callers with -fmad=false, so host
// and device give identical bits.  Returns 0, or 1 for a non-finite or too
// large extent.
__host__ __device__ inline int grid_axis(float mn, float mx, float vs, int32_t pad, int32_t* dim, float* origin) {
  if (!(mn - mn == 0.0f) || !(mx - mx == 0.0f)) return 1;  // NaN or infinity
  const float ext = roundf((mx - mn) / vs);
  if (ext > 1.0e6f) return 1;
  *dim = (int32_t)ext + 1 + pad * 2;
  *origin = mn - (float)pad * vs + vs / 2.0f;
  return 0;
}

#ifdef __CUDACC__

// Order-preserving float <-> int map for atomicMin/atomicMax on floats.
__device__ __forceinline__ int float_to_ordered(float f) {
  int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__host__ __device__ __forceinline__ float ordered_to_float(int i) {
  int b = i >= 0 ? i : i ^ 0x7FFFFFFF;
  float f;
  memcpy(&f, &b, sizeof(f));
  return f;
}

// Voxel coordinate of a point along one axis: round((p - o) / vs).
__device__ __forceinline__ int voxel_coord(float p, float o, float vs) {
  return (int)roundf(__fdiv_rn(__fsub_rn(p, o), vs));
}

// In-plane pass of the separable TDF on one tile of one z-plane:
// g2[z][y][x] = min over the in-plane (2R+1)^2 window of dx^2 + dy^2 over
// occupied voxels (kNone8 = none).  The occupancy rows of a PA_TY-row band
// (plus halo) are staged in shared memory, scanned along x, then along y.
// 256 threads; the caller synchronises before reusing the shared arrays.
constexpr int PA_TY = 16, PA_TX = 512;
constexpr uint8_t kNone8 = 0xFF;

template <int R>
struct PlaneSmem {
  uint8_t occ[PA_TY + 2 * R][PA_TX + 2 * R];
  uint8_t g1[PA_TY + 2 * R][PA_TX];
};

template <int R>
__device__ __forceinline__ void plane_tile(const uint8_t* __restrict__ occ, int dx, int dy, uint8_t* __restrict__ g2,
                                           int x0, int y0, int z, PlaneSmem<R>& sm) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t plane = (int64_t)dx * dy;
  const uint8_t* src = occ + (int64_t)z * plane;
  const int tx = min(PA_TX, dx - x0);
  for (int ly = warp; ly < PA_TY + 2 * R; ly += 8) {
    const int gy = y0 - R + ly;
    const bool row_in = gy >= 0 && gy < dy;
    for (int lx = lane; lx < tx + 2 * R; lx += 32) {
      const int gx = x0 - R + lx;
      sm.occ[ly][lx] = (row_in && gx >= 0 && gx < dx) ? src[(int64_t)gy * dx + gx] : 0;
    }
  }
  __syncthreads();
  for (int ly = warp; ly < PA_TY + 2 * R; ly += 8)
    for (int lx = lane; lx < tx; lx += 32) {
      int best = kNone8;
#pragma unroll
      for (int d = -R; d <= R; ++d)
        if (sm.occ[ly][lx + R + d]) best = min(best, d * d);
      sm.g1[ly][lx] = (uint8_t)best;
    }
  __syncthreads();
  const int ny = min(PA_TY, dy - y0);
  uint8_t* dst = g2 + (int64_t)z * plane;
  for (int ly = warp; ly < ny; ly += 8)
    for (int lx = lane; lx < tx; lx += 32) {
      int best = kNone8;
#pragma unroll
      for (int d = -R; d <= R; ++d) {
        int v = sm.g1[ly + R + d][lx];
        if (v != kNone8) best = min(best, v + d * d);
      }
      dst[(int64_t)(y0 + ly) * dx + x0 + lx] = (uint8_t)best;
    }
}

// Pass along z for voxel v (z = v / plane), then the TDF value.  Distance 0
// is the voxel's own occupancy, so 1 - sqrtf(0)/R = 1 reproduces the
// reference's "occupied -> 1" (core/demo.cu:40-43).
template <int R>
__device__ __forceinline__ float z_voxel(const uint8_t* __restrict__ g2, int64_t plane, int dz, int64_t v) {
  const int z = (int)(v / plane);
  int best = 0xFFFF;
#pragma unroll
  for (int d = -R; d <= R; ++d) {
    const int zz = z + d;
    if (zz < 0 || zz >= dz) continue;
    const int g = __ldg(g2 + v + (int64_t)d * plane);
    if (g != kNone8) best = min(best, g + d * d);
  }
  if (best == 0xFFFF) return 0.0f;
  const float val = __fsub_rn(1.0f, __fdiv_rn(__fsqrt_rn((float)best), (float)R));
  return val > 0.0f ? val : 0.0f;
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// Keypoint i of a fragment of n_pts points: a splitmix64 counter stream
// mapped to [0, n_pts) by a 64x64 high multiply (stands in for the
// reference's mt19937 + uniform_real, core/utils.hpp:15-20).
__device__ __forceinline__ int32_t keypoint_index(uint64_t seed, uint32_t n_pts, int i) {
  const uint64_t r = mix64(seed + (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ULL);
  return (int32_t)__umul64hi(r, (uint64_t)n_pts);
}

// patch[z][y][x] = tdf[kz-15+z][ky-15+y][kx-15+x], zero outside the grid;
// the 256 threads of a block write one 30^3 patch.
__device__ __forceinline__ void gather_patch(const float* __restrict__ tdf, int dx, int dy, int dz, int bx, int by,
                                             int bz, float* __restrict__ out) {
  for (int i = threadIdx.x; i < 27000; i += 256) {
    const int x = i % 30, y = (i / 30) % 30, z = i / 900;
    const int gx = bx + x, gy = by + y, gz = bz + z;
    float v = 0.0f;
    if (gx >= 0 && gy >= 0 && gz >= 0 && gx < dx && gy < dy && gz < dz)
      v = __ldg(tdf + ((int64_t)gz * dy + gy) * dx + gx);
    out[i] = v;
  }
}

#endif  // __CUDACC__

}  // namespace tdm
