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
#include "hashgrid.cuh"

namespace tdm {
namespace {

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
