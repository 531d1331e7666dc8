// Surface overlap of a registered pair (core/demo.m:66-72,
// evaluation/geometric-registration/register2Fragments.m:90-97): fragment B is
// moved by Rt, and for each direction the points that have a point of the
// other cloud within the radius (0.05 m) are counted; the reference divides
// the counts by the cloud sizes (ratioAligned) and keeps pairs above 0.30 for
// its logs (writeLog.m).
//
// GPU form: each cloud goes into a hashed uniform grid (cell = 1.05 radius,
// keys are packed cell coordinates, open addressing in a table of
// next_pow2(2n) slots, points grouped per cell by a count / scan / scatter),
// and every query point probes the 27 cells around it and stops at the first
// point within the radius.  The workspace depends on the point counts only.
//
// Arithmetic (compiled with -fmad=false; the oracle restates it):
//   b' = ((R0 x + R1 y) + R2 z) + t   in float, R and t rounded from double,
//   d2 = (dx dx + dy dy) + dz dz      in float, counted when d2 < r r.
#include <algorithm>
#include <cfloat>

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
__global__ void scan_block_kernel(const int32_t* __restrict__ in, int64_t n, int32_t* __restrict__ out,
                                  int32_t* __restrict__ sums) {
  __shared__ int32_t s[kScanBlock];
  const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
  s[threadIdx.x] = i < n ? in[i] : 0;
  __syncthreads();
  for (int o = 1; o < kScanBlock; o <<= 1) {
    const int32_t v = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += v;
    __syncthreads();
  }
  if (i < n) out[i] = s[threadIdx.x] - (i < n ? in[i] : 0);
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

// Counts the query points with a table point closer than the radius.
__global__ void query_kernel(const float* __restrict__ q, int n, float cell, float lim, float r2, Table T,
                             int32_t* __restrict__ found) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool hit = false;
  if (i < n) {
    const float x = q[3 * (int64_t)i], y = q[3 * (int64_t)i + 1], z = q[3 * (int64_t)i + 2];
    if (fabsf(x) < lim && fabsf(y) < lim && fabsf(z) < lim) {
      int c[3];
      cell_of(x, y, z, cell, c);
      for (int d = 0; d < 27 && !hit; ++d) {
        const uint64_t key = cell_key(c[0] + d / 9 - 1, c[1] + (d / 3) % 3 - 1, c[2] + d % 3 - 1);
        uint32_t s = slot_of(key, T.H);
        for (int64_t probe = 0; probe < T.H; ++probe) {
          const uint64_t k = T.keys[s];
          if (k == kEmpty) break;
          if (k == key) {
            const int32_t a = T.start[s], e = a + T.count[s];
            for (int32_t j = a; j < e; ++j) {
              const float dx = __fsub_rn(x, T.pts[3 * (int64_t)j]);
              const float dy = __fsub_rn(y, T.pts[3 * (int64_t)j + 1]);
              const float dz = __fsub_rn(z, T.pts[3 * (int64_t)j + 2]);
              const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
              if (d2 < r2) { hit = true; break; }
            }
            break;
          }
          s = (uint32_t)((s + 1) & (T.H - 1));
        }
      }
    }
  }
  const unsigned b = __ballot_sync(0xffffffffu, hit);
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(found, __popc(b));
}

struct Layout {
  size_t bt, tab[2][6], sums, flag, total;
  int64_t H[2];
};

Layout layout(int na, int nb) {
  Layout L{};
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~(size_t)255; return o; };
  L.bt = take((size_t)nb * 12);
  const int n[2] = {na, nb};
  for (int t = 0; t < 2; ++t) {
    L.H[t] = table_slots(n[t]);
    L.tab[t][0] = take((size_t)L.H[t] * 8);
    L.tab[t][1] = take((size_t)L.H[t] * 4);
    L.tab[t][2] = take((size_t)L.H[t] * 4);
    L.tab[t][3] = take((size_t)L.H[t] * 4);
    L.tab[t][4] = take((size_t)n[t] * 4);
    L.tab[t][5] = take((size_t)n[t] * 12);
  }
  L.sums = take(kScanBlock * 4);
  L.flag = take(16);
  L.total = off;
  return L;
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

using namespace tdm;

extern "C" size_t tdm_overlap_workspace_bytes(int32_t na, int32_t nb) {
  if (na <= 0 || nb <= 0 || na > (1 << 19) || nb > (1 << 19)) return 0;
  return layout(na, nb).total;
}

extern "C" tdm_status tdm_overlap(const float* a, int32_t na, const float* b, int32_t nb, const double rt[12],
                                  float radius, int32_t* counts, void* ws, size_t ws_bytes, tdm_stream s) {
  TDM_REQUIRE(a && b && rt && counts && ws, "tdm_overlap: null pointer");
  TDM_REQUIRE(na > 0 && nb > 0 && na <= (1 << 19) && nb <= (1 << 19), "tdm_overlap: 1 .. 524288 points per cloud");
  TDM_REQUIRE(radius > 0.0f && radius < 1.0e3f, "tdm_overlap: radius must be in (0, 1000)");
  const Layout L = layout(na, nb);
  TDM_REQUIRE(ws_bytes >= L.total, "tdm_overlap: workspace too small");
  uint8_t* w = static_cast<uint8_t*>(ws);
  float* bt = reinterpret_cast<float*>(w + L.bt);
  int32_t* sums = reinterpret_cast<int32_t*>(w + L.sums);
  int* err = reinterpret_cast<int*>(w + L.flag);
  Table T[2];
  for (int t = 0; t < 2; ++t) {
    T[t].keys = reinterpret_cast<uint64_t*>(w + L.tab[t][0]);
    T[t].count = reinterpret_cast<int32_t*>(w + L.tab[t][1]);
    T[t].start = reinterpret_cast<int32_t*>(w + L.tab[t][2]);
    T[t].cursor = reinterpret_cast<int32_t*>(w + L.tab[t][3]);
    T[t].pslot = reinterpret_cast<int32_t*>(w + L.tab[t][4]);
    T[t].pts = reinterpret_cast<float*>(w + L.tab[t][5]);
    T[t].H = L.H[t];
  }
  TDM_CHECK_CUDA(cudaMemsetAsync(err, 0, 16, s));
  TDM_CHECK_CUDA(cudaMemsetAsync(counts, 0, 8, s));
  transform_kernel<<<(nb + 255) / 256, 256, 0, s>>>(
      b, nb, (float)rt[0], (float)rt[1], (float)rt[2], (float)rt[4], (float)rt[5], (float)rt[6], (float)rt[8],
      (float)rt[9], (float)rt[10], (float)rt[3], (float)rt[7], (float)rt[11], bt);
  TDM_CHECK_LAUNCH("transform_kernel");
  const float cell = radius * kCellScale;  // only sizes the grid: results do not depend on it
  const float r2 = radius * radius, lim = cell * kMaxCells;
  tdm_status st = build_table(a, na, cell, lim, T[0], sums, err, s);
  if (!st) st = build_table(bt, nb, cell, lim, T[1], sums, err, s);
  if (st) return st;
  query_kernel<<<(na + 255) / 256, 256, 0, s>>>(a, na, cell, lim, r2, T[1], counts);
  query_kernel<<<(nb + 255) / 256, 256, 0, s>>>(bt, nb, cell, lim, r2, T[0], counts + 1);
  note_launches(1);
  TDM_CHECK_LAUNCH("query_kernel");
  int h = 0;
  TDM_CHECK_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  TDM_CHECK_CUDA(cudaStreamSynchronize(s));
  TDM_REQUIRE(h == 0, "tdm_overlap: a coordinate is non-finite or beyond 65536 grid cells (1.05 radius each)");
  return TDM_OK;
}
