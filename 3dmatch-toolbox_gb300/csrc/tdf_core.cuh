// Per-voxel, per-tile and per-keypoint arithmetic shared by the single-fragment
// entry points (tdf.cu) and the batched form (batch.cu), so both give the same
// bits by construction.  Geometry follows core/demo.cu:97-135, keypoints
// core/demo.cu:164-177, the patch gather core/demo.cu:206-217.
#pragma once

#include <cmath>
#include <cstdint>
#ifdef __CUDACC__
#include <cuda_fp16.h>
#endif

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

// The occupancy and in-plane distance arrays are stored with each x row
// padded to a multiple of 4 bytes (pitch X = occ_pitch(dx), index
// (z*dy + y)*X + x, padding bytes zero), so 4 voxels of a row are one aligned
// 32-bit word.  Squared distances are bytes: in-plane values are <= 2 R^2 <=
// 200, "none" is 0xFF, and sums saturate at 0xFF (__vaddus4), which maps every
// distance above R^2 to the same value 0 as the reference.
__host__ __device__ inline int64_t occ_pitch(int dx) { return ((int64_t)dx + 3) & ~(int64_t)3; }

// Min-plus on packed squared distances.  The saturating byte form
//   best = min_k min(255, g_k + d_k^2)
// is computed as min(255, min_k (g_k + d_k^2)) in half2 lanes holding 1024 + g
// (bytes placed under the FP16 exponent of 1024, whose ulp is 1): every value
// stays an integer below 2048, exact in FP16, so the bytes are the byte form's,
// with two voxels per HADD2/HMNMX2 instead of the byte-SIMD emulation.
__device__ __forceinline__ void bytes_to_h2(uint32_t w, uint32_t& lo, uint32_t& hi) {
  lo = __byte_perm(w, 0x64646464u, 0x4140);  // (1024 + b0, 1024 + b1)
  hi = __byte_perm(w, 0x64646464u, 0x4342);  // (1024 + b2, 1024 + b3)
}
__device__ __forceinline__ uint32_t h2_add(uint32_t a, uint32_t b) {
  __half2 r = __hadd2(*reinterpret_cast<const __half2*>(&a), *reinterpret_cast<const __half2*>(&b));
  return *reinterpret_cast<uint32_t*>(&r);
}
__device__ __forceinline__ uint32_t h2_min(uint32_t a, uint32_t b) {
  __half2 r = __hmin2(*reinterpret_cast<const __half2*>(&a), *reinterpret_cast<const __half2*>(&b));
  return *reinterpret_cast<uint32_t*>(&r);
}
// FP16 bits of an integer 0 <= n < 2048 (exact: 11 significant bits)
__host__ __device__ constexpr uint32_t fp16_bits_of_int(int n) {
  int e = 0;
  while (e < 10 && (n >> (e + 1)) != 0) ++e;
  return n == 0 ? 0u : (uint32_t)(((e + 15) << 10) | ((n - (1 << e)) << (10 - e)));
}
static_assert(fp16_bits_of_int(1024) == 0x6400u && fp16_bits_of_int(25) == 0x4E40u, "FP16 integer encoding");
// the squared offset k^2 in both lanes (k^2 <= 100)
__device__ __forceinline__ constexpr uint32_t h2_sq(int k) { return fp16_bits_of_int(k * k) * 0x10001u; }
// min(255, value - 1024) of both lanes of lo and hi, packed back into 4 bytes
__device__ __forceinline__ uint32_t h2_to_bytes(uint32_t lo, uint32_t hi) {
  constexpr uint32_t kCap = 0x64FF64FFu;  // (1024 + 255) in both lanes
  lo = h2_min(lo, kCap);
  hi = h2_min(hi, kCap);
  return __byte_perm(lo, hi, 0x6420);
}

constexpr int PB_TX = 128, PB_TY = 16;  // in-plane tile: 128 x positions, 16 rows
constexpr int PB_HALO = 12;             // staged bytes left of the tile (>= R, multiple of 4)
constexpr uint8_t kNone8 = 0xFF;

template <int R>
struct PlaneSmem {
  uint32_t occ[PB_TY + 2 * R][(PB_TX + 2 * PB_HALO) / 4];  // byte j of a row <-> x0 - PB_HALO + j
  uint32_t g1[PB_TY + 2 * R][PB_TX / 4];
};

// In-plane pass on one tile of one z-plane (256 threads):
//   g1 = min_{|dx|<=R, occ} dx^2 along x (a 28-bit occupancy mask per 4
//        positions, nearest set bit on either side),
//   g2 = min_{|dy|<=R} dy^2 + g1 along y (four bytes at a time).
template <int R>
__device__ __forceinline__ void plane_tile(const uint8_t* __restrict__ occ, int dx, int dy, uint8_t* __restrict__ g2,
                                           int x0, int y0, int z, PlaneSmem<R>& sm) {
  static_assert(R >= 1 && R <= PB_HALO - 2, "radius must leave the 28-bit window inside the staged halo");
  constexpr int ROWS = PB_TY + 2 * R, WPR = (PB_TX + 2 * PB_HALO) / 4, GPR = PB_TX / 4;
  const int64_t X = occ_pitch(dx);
  const int64_t zbase = (int64_t)z * dy * X;
  const int ngr = (min(PB_TX, dx - x0) + 3) / 4;
  uint32_t any = 0;
  for (int i = threadIdx.x; i < ROWS * WPR; i += blockDim.x) {
    const int ly = i / WPR, w = i - ly * WPR;
    const int gy = y0 - R + ly, gx = x0 - PB_HALO + 4 * w;
    uint32_t v = 0;
    if (gy >= 0 && gy < dy && gx >= 0 && gx < X)
      v = *reinterpret_cast<const uint32_t*>(occ + zbase + (int64_t)gy * X + gx);
    sm.occ[ly][w] = v;
    any |= v;
  }
  if (!__syncthreads_or(any != 0)) {
    // nothing occupied within R of the tile (most tiles of a grid): every
    // in-plane distance is "none", the value the passes below would produce
    for (int i = threadIdx.x; i < PB_TY * GPR; i += blockDim.x) {
      const int ly = i / GPR, g = i - ly * GPR;
      if (y0 + ly >= dy || g >= ngr) continue;
      *reinterpret_cast<uint32_t*>(g2 + zbase + (int64_t)(y0 + ly) * X + x0 + 4 * g) = 0xFFFFFFFFu;
    }
    return;
  }
  for (int i = threadIdx.x; i < ROWS * GPR; i += blockDim.x) {
    const int ly = i / GPR, g = i - ly * GPR;
    if (g >= ngr) continue;
    uint32_t any = 0;  // most of a grid is far from the surface: no occupied byte in the window
#pragma unroll
    for (int k = 0; k < 7; ++k) any |= sm.occ[ly][g + k];
    if (any == 0) {
      sm.g1[ly][g] = 0xFFFFFFFFu;  // every position: none within R
      continue;
    }
    uint32_t mask = 0;  // bit k <-> staged byte 4g + k
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      const uint32_t w = sm.occ[ly][g + k] & 0x01010101u;
      mask |= ((w | (w >> 7) | (w >> 14) | (w >> 21)) & 0xFu) << (4 * k);
    }
    uint32_t out = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = PB_HALO + q;  // bit of position x0 + 4g + q
      int best = kNone8;
      const uint32_t rw = (mask >> c) & ((1u << (R + 1)) - 1);  // offsets 0..R
      if (rw) {
        const int d = __ffs(rw) - 1;
        best = d * d;
      }
      const uint32_t lw = (mask >> (c - R)) & ((1u << R) - 1);  // offsets -R..-1
      if (lw) {
        const int d = R - (31 - __clz(lw));
        best = min(best, d * d);
      }
      out |= (uint32_t)best << (8 * q);
    }
    sm.g1[ly][g] = out;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < PB_TY * GPR; i += blockDim.x) {
    const int ly = i / GPR, g = i - ly * GPR;
    if (y0 + ly >= dy || g >= ngr) continue;
    uint32_t all = 0xFFFFFFFFu;  // every byte "none" in the window: the min-plus gives 0xFF
#pragma unroll
    for (int d = -R; d <= R; ++d) all &= sm.g1[ly + R + d][g];
    uint32_t best = 0xFFFFFFFFu;
    if (all != 0xFFFFFFFFu) {
      uint32_t bl, bh;
      bytes_to_h2(sm.g1[ly][g], bl, bh);
      bl = h2_add(bl, h2_sq(R));
      bh = h2_add(bh, h2_sq(R));
#pragma unroll
      for (int d = -R + 1; d <= R; ++d) {
        uint32_t l, h;
        bytes_to_h2(sm.g1[ly + R + d][g], l, h);
        bl = h2_min(bl, h2_add(l, h2_sq(d)));
        bh = h2_min(bh, h2_add(h, h2_sq(d)));
      }
      best = h2_to_bytes(bl, bh);
    }
    *reinterpret_cast<uint32_t*>(g2 + zbase + (int64_t)(y0 + ly) * X + x0 + 4 * g) = best;
  }
}

// TDF value of a saturated squared distance: max(0, 1 - sqrtf(g)/R), the
// reference's expression (core/demo.cu:44-56) in IEEE operations; g >= R^2
// gives 0, so the 0xFF saturation is exact.  Filled by the calling block.
template <int R>
__device__ __forceinline__ void tdf_lut(float* lut) {
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    const float v = __fsub_rn(1.0f, __fdiv_rn(__fsqrt_rn((float)i), (float)R));
    lut[i] = v > 0.0f ? v : 0.0f;
  }
}

// Pass along z by one warp over a column segment: lane l owns the 4 voxels
// x = xseg + 4l .. +3 of row y and walks z = z0 .. z1-1 with the 2R+1 words
// of g2 around z in a register ring (one new aligned load per step).  Values
// go through the warp's 128-float staging area so each store instruction
// writes 32 consecutive floats.  Must be called by all 32 lanes.
constexpr int kZChunk = 32;  // z steps per warp work item
template <int R>
__device__ __forceinline__ void z_column(const uint8_t* __restrict__ g2, int dx, int dy, int dz, int y, int xseg,
                                         int z0, int z1, const float* lut, float* s_w, float* __restrict__ tdf) {
  const int lane = threadIdx.x & 31;
  const int64_t X = occ_pitch(dx), pz = (int64_t)dy * X;
  const int x4 = xseg + 4 * lane;
  const bool live = x4 < dx;
  const uint8_t* col = g2 + (int64_t)y * X + x4;
  auto word = [&](int zz) -> uint32_t {
    return (live && zz >= 0 && zz < dz) ? __ldg(reinterpret_cast<const uint32_t*>(col + zz * pz)) : 0xFFFFFFFFu;
  };
  // the window's words as half2 pairs of 1024 + byte (see bytes_to_h2)
  uint32_t rlo[2 * R + 1], rhi[2 * R + 1];
#pragma unroll
  for (int k = 0; k < 2 * R + 1; ++k) bytes_to_h2(word(z0 - R + k), rlo[k], rhi[k]);
  const int n = min(128, dx - xseg);
  for (int z = z0; z < z1; ++z) {
    // when every byte of the window is "none" (0xFF, most of a grid) the
    // min-plus gives 0xFF anyway: (1024 + 255) in every lane
    uint32_t all = rlo[0] & rhi[0];
#pragma unroll
    for (int k = 1; k < 2 * R + 1; ++k) all &= rlo[k] & rhi[k];
    uint32_t best = 0xFFFFFFFFu;
    if (all != 0x64FF64FFu) {
      uint32_t bl = h2_add(rlo[0], h2_sq(R)), bh = h2_add(rhi[0], h2_sq(R));
#pragma unroll
      for (int k = 1; k < 2 * R + 1; ++k) {
        bl = h2_min(bl, h2_add(rlo[k], h2_sq(k - R)));
        bh = h2_min(bh, h2_add(rhi[k], h2_sq(k - R)));
      }
      best = h2_to_bytes(bl, bh);
    }
    float* out = tdf + ((int64_t)z * dy + y) * dx + xseg;
    if (__all_sync(0xffffffffu, best == 0xFFFFFFFFu)) {
      // the whole 128-voxel segment is farther than R from the surface (most
      // of a grid): TDF 0 (lut[255]), stored without the lookup and staging
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (lane + 32 * i < n) out[lane + 32 * i] = 0.0f;
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q) s_w[4 * lane + q] = lut[(best >> (8 * q)) & 0xFFu];
      __syncwarp();
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (lane + 32 * i < n) out[lane + 32 * i] = s_w[lane + 32 * i];
      __syncwarp();
    }
#pragma unroll
    for (int k = 0; k < 2 * R; ++k) {
      rlo[k] = rlo[k + 1];
      rhi[k] = rhi[k + 1];
    }
    bytes_to_h2(word(z + R + 1), rlo[2 * R], rhi[2 * R]);
  }
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
