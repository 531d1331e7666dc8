// Hashed uniform grid of points on the device, shared by the surface overlap
// and ICP: packed cell keys in an open-addressing table of next_pow2(2n)
// slots (at least half stay free), the points of each cell made contiguous by
// a count / exclusive scan / scatter.  Cell placement in the table depends on
// insertion order; nothing computed from the grid does.
#pragma once

#include <algorithm>

#include "common.cuh"

namespace tdm {
namespace {

constexpr uint64_t kEmpty = ~0ull;
constexpr float kCellScale = 1.05f;   // cell edge / radius
// |coordinate| < kMaxCells cells keeps the cell index of x/cell within one
// ulp of 0.008 of a cell, so two points closer than the radius (0.95 cell)
// always lie in adjacent cells
constexpr float kMaxCells = 65536.0f;
constexpr int kScanBlock = 1024;

__host__ __device__ inline int64_t table_slots(int n) {
  int64_t h = 1024;
  while (h < 2 * (int64_t)n) h <<= 1;
  return h;
}

__device__ __forceinline__ uint64_t cell_key(int cx, int cy, int cz) {
  return ((uint64_t)(uint32_t)(cx + (1 << 20)) << 42) | ((uint64_t)(uint32_t)(cy + (1 << 20)) << 21) |
         (uint64_t)(uint32_t)(cz + (1 << 20));
}

__device__ __forceinline__ uint32_t slot_of(uint64_t key, int64_t H) {
  uint64_t z = key * 0x9E3779B97F4A7C15ull;
  z ^= z >> 29;
  z *= 0xBF58476D1CE4E5B9ull;
  z ^= z >> 32;
  return (uint32_t)(z & (uint64_t)(H - 1));
}

__device__ __forceinline__ void cell_of(float x, float y, float z, float cell, int* c) {
  c[0] = (int)floorf(__fdiv_rn(x, cell));
  c[1] = (int)floorf(__fdiv_rn(y, cell));
  c[2] = (int)floorf(__fdiv_rn(z, cell));
}

struct Table {
  uint64_t* keys;
  int32_t* count;
  int32_t* start;
  int32_t* cursor;
  int32_t* pslot;
  float* pts;  // grouped by cell
  int64_t H;
};

__global__ void transform_kernel(const float* __restrict__ b, int n, float r00, float r01, float r02, float r10,
                                 float r11, float r12, float r20, float r21, float r22, float t0, float t1, float t2,
                                 float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float x = b[3 * (int64_t)i], y = b[3 * (int64_t)i + 1], z = b[3 * (int64_t)i + 2];
  out[3 * (int64_t)i] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(r00, x), __fmul_rn(r01, y)), __fmul_rn(r02, z)), t0);
  out[3 * (int64_t)i + 1] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(r10, x), __fmul_rn(r11, y)), __fmul_rn(r12, z)), t1);
  out[3 * (int64_t)i + 2] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(r20, x), __fmul_rn(r21, y)), __fmul_rn(r22, z)), t2);
}

__global__ void clear_kernel(Table T) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < T.H; i += (int64_t)gridDim.x * blockDim.x) {
    T.keys[i] = kEmpty;
    T.count[i] = 0;
    T.cursor[i] = 0;
  }
}

// Claims (or finds) the slot of each point's cell and counts the cell.
__global__ void insert_kernel(const float* __restrict__ p, int n, float cell, float lim, Table T, int* __restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float x = p[3 * (int64_t)i], y = p[3 * (int64_t)i + 1], z = p[3 * (int64_t)i + 2];
  if (!(fabsf(x) < lim && fabsf(y) < lim && fabsf(z) < lim)) {
    atomicExch(err, 1);
    T.pslot[i] = -1;
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
      T.pslot[i] = (int32_t)s;
      return;
    }
    s = (uint32_t)((s + 1) & (T.H - 1));
  }
  atomicExch(err, 2);  // table full (cannot happen: at least half the slots stay free)
  T.pslot[i] = -1;
}

// Exclusive scan of the slot counts: per-block scan, block totals, add.
// `out` may be `in` (each thread reads its element once, before writing it).
__global__ void scan_block_kernel(const int32_t* in, int64_t n, int32_t* out, int32_t* __restrict__ sums) {
  __shared__ int32_t s[kScanBlock];
  const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
  const int32_t mine = i < n ? in[i] : 0;
  s[threadIdx.x] = mine;
  __syncthreads();
  for (int o = 1; o < kScanBlock; o <<= 1) {
    const int32_t v = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += v;
    __syncthreads();
  }
  if (i < n) out[i] = s[threadIdx.x] - mine;
  if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = s[threadIdx.x];
}

__global__ void scan_sums_kernel(int32_t* __restrict__ sums, int nb) {
  __shared__ int32_t s[kScanBlock];
  s[threadIdx.x] = threadIdx.x < nb ? sums[threadIdx.x] : 0;
  __syncthreads();
  for (int o = 1; o < kScanBlock; o <<= 1) {
    const int32_t v = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += v;
    __syncthreads();
  }
  if (threadIdx.x < nb) sums[threadIdx.x] = s[threadIdx.x] - (threadIdx.x < nb ? sums[threadIdx.x] : 0);
}

__global__ void scan_add_kernel(int32_t* __restrict__ out, int64_t n, const int32_t* __restrict__ sums) {
  const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n) out[i] += sums[blockIdx.x];
}

__global__ void scatter_kernel(const float* __restrict__ p, int n, Table T) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t s = T.pslot[i];
  if (s < 0) return;
  const int32_t at = T.start[s] + atomicAdd(T.cursor + s, 1);
  T.pts[3 * (int64_t)at] = p[3 * (int64_t)i];
  T.pts[3 * (int64_t)at + 1] = p[3 * (int64_t)i + 1];
  T.pts[3 * (int64_t)at + 2] = p[3 * (int64_t)i + 2];
}

tdm_status build_table(const float* p, int n, float cell, float lim, Table T, int32_t* sums, int* err,
                       cudaStream_t s) {
  clear_kernel<<<(unsigned)std::min<int64_t>((T.H + 255) / 256, 4096), 256, 0, s>>>(T);
  insert_kernel<<<(n + 255) / 256, 256, 0, s>>>(p, n, cell, lim, T, err);
  const int nblk = (int)((T.H + kScanBlock - 1) / kScanBlock);
  scan_block_kernel<<<nblk, kScanBlock, 0, s>>>(T.count, T.H, T.start, sums);
  scan_sums_kernel<<<1, kScanBlock, 0, s>>>(sums, nblk);
  scan_add_kernel<<<nblk, kScanBlock, 0, s>>>(T.start, T.H, sums);
  scatter_kernel<<<(n + 255) / 256, 256, 0, s>>>(p, n, T);
  note_launches(5);
  TDM_CHECK_LAUNCH("overlap table");
  return TDM_OK;
}


}  // namespace
}  // namespace tdm
