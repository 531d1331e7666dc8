// Batched description of many fragments: core/demo.cu's main (grid,
// occupancy, TDF, keypoints, patches, net; core/demo.cu:97-231) over a set of
// fragments of uneven point and keypoint counts and voxel sizes.
//
// One persistent launch per stage.  The host uploads a fragment table (point
// and keypoint offsets, voxel size, seed); a plan kernel turns each
// fragment's bounds into its grid (grid_axis, the single-fragment
// arithmetic) and lays the grids out back to back in one voxel arena; the
// occupancy, TDF, keypoint and gather kernels then walk the table with a
// binary search per work item, so their launch shapes do not depend on the
// data and the whole sequence can be captured once as a CUDA graph and
// replayed for other fragments of the same total keypoint count.
//
// Compiled with -fmad=false: the plan kernel's float arithmetic must give the
// host's bits.
#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "tdf_core.cuh"

namespace tdm {
namespace {

constexpr int kMaxFragments = 1024;

struct FragIn {  // host-written each call
  int64_t pt_off;
  int64_t n_pts;
  int64_t kp_off;
  int32_t k;
  float vs;
  uint64_t seed;
};

struct FragGeo {  // plan-kernel output
  float origin[3];
  int32_t dim[3];
  int64_t vox_off;  // first voxel of the fragment's grid in the arenas
};

struct Totals {
  int64_t voxels;  // arena voxels in use (pitched grids rounded up to 256)
  int64_t tiles;   // in-plane pass tiles
  int64_t rows;    // z-pass warp work items
  int64_t points;
  int32_t status;  // 0, kCapacity or kGeometry
  int32_t bad_fragment;
};
constexpr int32_t kCapacity = 1, kGeometry = 2;

// largest f in [0, F) with b[f] <= i (b ascending, b[0] = 0)
__device__ __forceinline__ int find_frag(const int64_t* b, int F, int64_t i) {
  int lo = 0, hi = F - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (b[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void reset_kernel(int F, int* __restrict__ mm, Totals* __restrict__ tot) {
  for (int i = threadIdx.x; i < 6 * F; i += blockDim.x) mm[i] = (i % 6) < 3 ? INT_MAX : INT_MIN;
  if (threadIdx.x == 0) *tot = Totals{};
}

// Per-fragment bounds.  Each block walks a contiguous range of points, so a
// thread's fragment changes rarely; partial bounds are flushed with atomics
// on the order-preserving integer image of the floats.
__global__ __launch_bounds__(256) void minmax_kernel(const float* __restrict__ pts, int F,
                                                     const int64_t* __restrict__ pt_bound, int* __restrict__ mm) {
  __shared__ int64_t sb[kMaxFragments + 1];
  for (int i = threadIdx.x; i <= F; i += blockDim.x) sb[i] = pt_bound[i];
  __syncthreads();
  const int64_t total = sb[F];
  const int64_t chunk = (total + gridDim.x - 1) / gridDim.x;
  const int64_t start = (int64_t)blockIdx.x * chunk, end = min(total, start + chunk);
  int cur = -1;
  float mn[3], mx[3];
  auto flush = [&](int f) {
    if (f < 0) return;
    for (int a = 0; a < 3; ++a) {
      atomicMin(mm + 6 * f + a, float_to_ordered(mn[a]));
      atomicMax(mm + 6 * f + 3 + a, float_to_ordered(mx[a]));
    }
  };
  for (int64_t i = start + threadIdx.x; i < end; i += blockDim.x) {
    const int f = find_frag(sb, F, i);
    if (f != cur) {
      flush(cur);
      cur = f;
      for (int a = 0; a < 3; ++a) { mn[a] = INFINITY; mx[a] = -INFINITY; }
    }
    for (int a = 0; a < 3; ++a) {
      const float v = pts[3 * i + a];
      mn[a] = fminf(mn[a], v);
      mx[a] = fmaxf(mx[a], v);
    }
  }
  // whole warp on one fragment: reduce first, one lane flushes
  const int f0 = __shfl_sync(0xffffffffu, cur, 0);
  if (__all_sync(0xffffffffu, cur == f0)) {
    if (f0 < 0) return;
    for (int a = 0; a < 3; ++a)
      for (int o = 16; o > 0; o >>= 1) {
        mn[a] = fminf(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
        mx[a] = fmaxf(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
      }
    if ((threadIdx.x & 31) == 0) flush(f0);
  } else {
    flush(cur);
  }
}

// Grid of every fragment (grid_axis, as tdm_grid_from_points), arena offsets
// and plane-tile offsets, capacity check.  One block.
__global__ void plan_kernel(int F, const FragIn* __restrict__ in, const int* __restrict__ mm, int32_t pad,
                            int64_t cap_voxels, FragGeo* __restrict__ geo, int64_t* __restrict__ vox_bound,
                            int64_t* __restrict__ tile_bound, int64_t* __restrict__ row_bound,
                            const int64_t* __restrict__ pt_bound, Totals* __restrict__ tot) {
  __shared__ int64_t sV[kMaxFragments], sT[kMaxFragments], sR[kMaxFragments];
  __shared__ int s_bad;
  if (threadIdx.x == 0) s_bad = INT_MAX;
  __syncthreads();
  for (int f = threadIdx.x; f < F; f += blockDim.x) {
    FragGeo g{};
    int err = in[f].n_pts <= 0;
    int64_t V = 1;
    for (int a = 0; a < 3 && !err; ++a) {
      err |= grid_axis(ordered_to_float(mm[6 * f + a]), ordered_to_float(mm[6 * f + 3 + a]), in[f].vs, pad,
                       &g.dim[a], &g.origin[a]);
      V *= g.dim[a];
    }
    if (!err && V >= ((int64_t)1 << 31)) err = 1;
    if (err) {
      atomicMin(&s_bad, f);
      V = 0;
      g.dim[0] = g.dim[1] = g.dim[2] = 0;
    }
    geo[f] = g;
    const int64_t PV = err ? 0 : occ_pitch(g.dim[0]) * g.dim[1] * g.dim[2];
    sV[f] = (PV + 255) / 256 * 256;
    sT[f] = err ? 0 : (int64_t)((g.dim[0] + PB_TX - 1) / PB_TX) * ((g.dim[1] + PB_TY - 1) / PB_TY) * g.dim[2];
    sR[f] = err ? 0 : (int64_t)g.dim[1] * ((g.dim[0] + 127) / 128) * ((g.dim[2] + kZChunk - 1) / kZChunk);
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  int64_t v = 0, t = 0, rw = 0;
  for (int f = 0; f < F; ++f) {
    vox_bound[f] = v;
    tile_bound[f] = t;
    row_bound[f] = rw;
    geo[f].vox_off = v;
    v += sV[f];
    t += sT[f];
    rw += sR[f];
  }
  vox_bound[F] = v;
  tile_bound[F] = t;
  row_bound[F] = rw;
  Totals r{};
  r.bad_fragment = -1;
  if (s_bad != INT_MAX) {
    r.status = kGeometry;
    r.bad_fragment = s_bad;
  } else if (v > cap_voxels) {
    r.status = kCapacity;
  } else {
    r.voxels = v;
    r.tiles = t;
    r.rows = rw;
    r.points = pt_bound[F];
  }
  *tot = r;
}

__global__ __launch_bounds__(256) void zero_kernel(uint8_t* __restrict__ occ, const Totals* __restrict__ tot) {
  const int64_t n16 = tot->voxels / 16;
  uint4* p = reinterpret_cast<uint4*>(occ);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = make_uint4(0, 0, 0, 0);
}

// occ[vox_off + (z*dy + y)*X + x] = 1 for every point (core/demo.cu:127-135; X = occ_pitch(dx))
__global__ __launch_bounds__(256) void occupancy_kernel(const float* __restrict__ pts, int F,
                                                        const int64_t* __restrict__ pt_bound,
                                                        const FragIn* __restrict__ in, const FragGeo* __restrict__ geo,
                                                        const Totals* __restrict__ tot, uint8_t* __restrict__ occ) {
  __shared__ int64_t sb[kMaxFragments + 1];
  for (int i = threadIdx.x; i <= F; i += blockDim.x) sb[i] = pt_bound[i];
  __syncthreads();
  const int64_t n = tot->points;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int f = find_frag(sb, F, i);
    const FragGeo g = geo[f];
    const float vs = in[f].vs;
    const float px = pts[3 * i], py = pts[3 * i + 1], pz = pts[3 * i + 2];
    if (!(isfinite(px) && isfinite(py) && isfinite(pz))) continue;  // skipped, as by the grid bounds
    const int gx = voxel_coord(px, g.origin[0], vs);
    const int gy = voxel_coord(py, g.origin[1], vs);
    const int gz = voxel_coord(pz, g.origin[2], vs);
    if (gx < 0 || gy < 0 || gz < 0 || gx >= g.dim[0] || gy >= g.dim[1] || gz >= g.dim[2]) continue;
    occ[g.vox_off + ((int64_t)gz * g.dim[1] + gy) * occ_pitch(g.dim[0]) + gx] = 1;
  }
}

// In-plane TDF pass over every fragment's tiles (plane_tile).
template <int R>
__global__ __launch_bounds__(256) void plane_kernel(const uint8_t* __restrict__ occ, uint8_t* __restrict__ g2, int F,
                                                    const int64_t* __restrict__ tile_bound,
                                                    const FragGeo* __restrict__ geo, const Totals* __restrict__ tot) {
  __shared__ PlaneSmem<R> sm;
  __shared__ int64_t sb[kMaxFragments + 1];
  for (int i = threadIdx.x; i <= F; i += blockDim.x) sb[i] = tile_bound[i];
  __syncthreads();
  const int64_t n = tot->tiles;
  for (int64_t t = blockIdx.x; t < n; t += gridDim.x) {
    const int f = find_frag(sb, F, t);
    const FragGeo g = geo[f];
    const int ntx = (g.dim[0] + PB_TX - 1) / PB_TX, nty = (g.dim[1] + PB_TY - 1) / PB_TY;
    const int64_t local = t - sb[f];
    const int z = (int)(local / ((int64_t)ntx * nty));
    const int rem = (int)(local - (int64_t)z * ntx * nty);
    plane_tile<R>(occ + g.vox_off, g.dim[0], g.dim[1], g2 + g.vox_off, (rem % ntx) * PB_TX, (rem / ntx) * PB_TY, z,
                  sm);
    __syncthreads();
  }
}

// Pass along z of every grid (z_column): warp work items (y, 128-voxel x
// segment, 32-step z chunk) numbered fragment after fragment.
constexpr int kZThreads = 128;
template <int R>
__global__ __launch_bounds__(kZThreads) void z_kernel(const uint8_t* __restrict__ g2, float* __restrict__ tdf, int F,
                                                      const int64_t* __restrict__ item_bound,
                                                      const FragGeo* __restrict__ geo, const Totals* __restrict__ tot) {
  __shared__ int64_t sb[kMaxFragments + 1];
  __shared__ float lut[256];
  __shared__ float s_w[kZThreads / 32][128];
  for (int i = threadIdx.x; i <= F; i += blockDim.x) sb[i] = item_bound[i];
  tdf_lut<R>(lut);
  __syncthreads();
  const int64_t n = tot->rows;
  const int w = threadIdx.x >> 5;
  for (int64_t it = (int64_t)blockIdx.x * (kZThreads / 32) + w; it < n; it += (int64_t)gridDim.x * (kZThreads / 32)) {
    const int f = find_frag(sb, F, it);
    const FragGeo g = geo[f];
    const int nseg = (g.dim[0] + 127) / 128, nzc = (g.dim[2] + kZChunk - 1) / kZChunk;
    const int64_t local = it - sb[f];
    const int zc = (int)(local % nzc);
    const int64_t r = local / nzc;
    const int seg = (int)(r % nseg), y = (int)(r / nseg);
    z_column<R>(g2 + g.vox_off, g.dim[0], g.dim[1], g.dim[2], y, seg * 128, zc * kZChunk,
                min(g.dim[2], (zc + 1) * kZChunk), lut, s_w[w], tdf + g.vox_off);
  }
}

// Keypoint i of the batch: fragment f's index stream, coordinates and grid
// cell (core/demo.cu:164-177).
__global__ void keypoint_kernel(const float* __restrict__ pts, int F, const int64_t* __restrict__ kp_bound,
                                const FragIn* __restrict__ in, const FragGeo* __restrict__ geo,
                                const Totals* __restrict__ tot, int64_t total_k, float* __restrict__ keypts,
                                int32_t* __restrict__ kp_grid) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total_k) return;
  if (tot->status != 0) {
    for (int a = 0; a < 3; ++a) { keypts[3 * i + a] = 0.0f; kp_grid[3 * i + a] = 0; }
    return;
  }
  const int f = find_frag(kp_bound, F, i);
  const FragIn fi = in[f];
  const FragGeo g = geo[f];
  const int32_t j = keypoint_index(fi.seed, (uint32_t)fi.n_pts, (int)(i - kp_bound[f]));
  const float* p = pts + 3 * (fi.pt_off + j);
  for (int a = 0; a < 3; ++a) {
    keypts[3 * i + a] = p[a];
    kp_grid[3 * i + a] = voxel_coord(p[a], g.origin[a], fi.vs);
  }
}

// Patches k0 .. k0 + gridDim.x - 1 of the batch (gather_patch).
__global__ __launch_bounds__(256) void gather_kernel(const float* __restrict__ tdf, int F,
                                                     const int64_t* __restrict__ kp_bound,
                                                     const FragGeo* __restrict__ geo, const Totals* __restrict__ tot,
                                                     const int32_t* __restrict__ kp_grid, int64_t k0,
                                                     float* __restrict__ patches) {
  const int64_t i = k0 + blockIdx.x;
  float* out = patches + (int64_t)blockIdx.x * 27000;
  if (tot->status != 0) {
    for (int e = threadIdx.x; e < 27000; e += 256) out[e] = 0.0f;
    return;
  }
  const FragGeo g = geo[find_frag(kp_bound, F, i)];
  gather_patch(tdf + g.vox_off, g.dim[0], g.dim[1], g.dim[2], kp_grid[3 * i] - 15, kp_grid[3 * i + 1] - 15,
               kp_grid[3 * i + 2] - 15, out);
}

template <int R>
void launch_tdf_passes(const uint8_t* occ, uint8_t* g2, float* tdf, int F, const int64_t* tile_bound,
                       const int64_t* row_bound, const FragGeo* geo, const Totals* tot, int sms, cudaStream_t s) {
  plane_kernel<R><<<sms * 8, 256, 0, s>>>(occ, g2, F, tile_bound, geo, tot);
  z_kernel<R><<<sms * 16, kZThreads, 0, s>>>(g2, tdf, F, row_bound, geo, tot);
}

}  // namespace
}  // namespace tdm

using namespace tdm;

struct tdm_batch {
  tdm_batch_config cfg;
  tdm_net* net = nullptr;
  int sms = 148;
  int R = 5;
  int chunk = 2048;
  // device
  uint8_t* table = nullptr;  // upload region | geo | vox/tile bounds | mm | totals
  uint8_t* occ = nullptr;    // occupancy, then in-plane distances (2 x max_voxels)
  float* tdf = nullptr;
  int32_t* kp_grid = nullptr;
  float* patches = nullptr;
  size_t device_bytes = 0;
  // pinned host staging
  uint8_t* up = nullptr;
  uint8_t* down = nullptr;
  // table layout (bytes), fixed by max_fragments
  size_t o_in, o_ptb, o_kpb, up_bytes, o_geo, o_voxb, o_tileb, o_rowb, o_mm, o_tot, down_bytes, table_bytes;
  // captured graph; capture runs on a private stream (the legacy default
  // stream cannot be captured), replays on the caller's
  cudaStream_t cap = nullptr;
  cudaGraphExec_t exec = nullptr;
  const void* key_ptr[3] = {};
  int32_t key_f = -1;
  uint64_t key_gen = 0;
  int64_t key_k = -1;
  int64_t launches_per_call = 0;
  int32_t replayed = 0;

  ~tdm_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (cap) cudaStreamDestroy(cap);
    for (void* p : {(void*)table, (void*)occ, (void*)tdf, (void*)kp_grid, (void*)patches})
      if (p) cudaFree(p);
    if (up) cudaFreeHost(up);
  }
  FragIn* d_in() const { return reinterpret_cast<FragIn*>(table + o_in); }
  int64_t* d_ptb() const { return reinterpret_cast<int64_t*>(table + o_ptb); }
  int64_t* d_kpb() const { return reinterpret_cast<int64_t*>(table + o_kpb); }
  FragGeo* d_geo() const { return reinterpret_cast<FragGeo*>(table + o_geo); }
  int64_t* d_voxb() const { return reinterpret_cast<int64_t*>(table + o_voxb); }
  int64_t* d_tileb() const { return reinterpret_cast<int64_t*>(table + o_tileb); }
  int64_t* d_rowb() const { return reinterpret_cast<int64_t*>(table + o_rowb); }
  int* d_mm() const { return reinterpret_cast<int*>(table + o_mm); }
  Totals* d_tot() const { return reinterpret_cast<Totals*>(table + o_tot); }
};

namespace {

tdm_status batch_alloc(void** p, size_t bytes, size_t* total) {
  cudaError_t e = cudaMalloc(p, bytes < 256 ? 256 : bytes);
  if (e != cudaSuccess) return cuda_status(e, "batch buffer");
  *total += bytes;
  return TDM_OK;
}

// The stage sequence of one call (captured as a graph, or run directly).
tdm_status run_sequence(tdm_batch* b, const float* pts, int F, int64_t total_k, float* keypts, float* desc,
                        cudaStream_t s) {
  TDM_CHECK_CUDA(cudaMemcpyAsync(b->table, b->up, b->up_bytes, cudaMemcpyHostToDevice, s));
  const int g = b->sms * 4;
  reset_kernel<<<1, 256, 0, s>>>(F, b->d_mm(), b->d_tot());
  minmax_kernel<<<g, 256, 0, s>>>(pts, F, b->d_ptb(), b->d_mm());
  plan_kernel<<<1, 1024, 0, s>>>(F, b->d_in(), b->d_mm(), b->cfg.pad, b->cfg.max_voxels, b->d_geo(), b->d_voxb(),
                                 b->d_tileb(), b->d_rowb(), b->d_ptb(), b->d_tot());
  zero_kernel<<<g, 256, 0, s>>>(b->occ, b->d_tot());
  occupancy_kernel<<<g, 256, 0, s>>>(pts, F, b->d_ptb(), b->d_in(), b->d_geo(), b->d_tot(), b->occ);
  note_launches(4);
  TDM_CHECK_LAUNCH("batch plan / occupancy kernels");
  uint8_t* g2 = b->occ + b->cfg.max_voxels;
  switch (b->R) {
#define TDM_R_CASE(R_) \
  case R_: launch_tdf_passes<R_>(b->occ, g2, b->tdf, F, b->d_tileb(), b->d_rowb(), b->d_geo(), b->d_tot(), b->sms, s); break;
    TDM_R_CASE(1) TDM_R_CASE(2) TDM_R_CASE(3) TDM_R_CASE(4) TDM_R_CASE(5)
    TDM_R_CASE(6) TDM_R_CASE(7) TDM_R_CASE(8) TDM_R_CASE(9) TDM_R_CASE(10)
#undef TDM_R_CASE
    default: return fail(TDM_ERR_INVALID_ARG, "tdm_describe_batch: truncation radius must be 1..10 voxels");
  }
  note_launches(1);
  TDM_CHECK_LAUNCH("batch TDF passes");
  if (total_k > 0) {
    keypoint_kernel<<<(unsigned)((total_k + 127) / 128), 128, 0, s>>>(pts, F, b->d_kpb(), b->d_in(), b->d_geo(),
                                                                      b->d_tot(), total_k, keypts, b->kp_grid);
    TDM_CHECK_LAUNCH("batch keypoint_kernel");
  }
  for (int64_t k0 = 0; k0 < total_k; k0 += b->chunk) {
    const int n = (int)std::min<int64_t>(b->chunk, total_k - k0);
    gather_kernel<<<n, 256, 0, s>>>(b->tdf, F, b->d_kpb(), b->d_geo(), b->d_tot(), b->kp_grid, k0, b->patches);
    TDM_CHECK_LAUNCH("batch gather_kernel");
    tdm_status st = tdm_net_forward(b->net, b->patches, n, desc + k0 * 512, s);
    if (st) return st;
  }
  TDM_CHECK_CUDA(cudaMemcpyAsync(b->down, b->table + b->o_geo, b->down_bytes, cudaMemcpyDeviceToHost, s));
  return TDM_OK;
}

}  // namespace

extern "C" tdm_status tdm_batch_create(const tdm_batch_config* cfg, tdm_net* net, tdm_batch** out) {
  TDM_REQUIRE(cfg && net && out, "tdm_batch_create: null pointer");
  TDM_REQUIRE(cfg->max_fragments >= 1 && cfg->max_fragments <= kMaxFragments,
              "tdm_batch_create: max_fragments must be 1..1024");
  TDM_REQUIRE(cfg->max_points > 0 && cfg->max_keypoints >= 0 && cfg->max_voxels > 0 && cfg->pad >= 0 &&
                  cfg->trunc_voxels > 0,
              "tdm_batch_create: bad limits");
  tdm_batch* b = new tdm_batch();
  b->cfg = *cfg;
  b->cfg.max_voxels = (cfg->max_voxels + 255) / 256 * 256;
  b->net = net;
  b->chunk = net_max_batch(net);
  int dev = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || b->sms <= 0) b->sms = 148;
  const size_t F = (size_t)cfg->max_fragments;
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  b->o_in = 0;
  b->o_ptb = al(b->o_in + F * sizeof(FragIn));
  b->o_kpb = al(b->o_ptb + (F + 1) * 8);
  b->up_bytes = al(b->o_kpb + (F + 1) * 8);
  b->o_geo = b->up_bytes;
  b->o_tot = al(b->o_geo + F * sizeof(FragGeo));
  b->down_bytes = b->o_tot + sizeof(Totals) - b->o_geo;
  b->o_voxb = al(b->o_tot + sizeof(Totals));
  b->o_tileb = al(b->o_voxb + (F + 1) * 8);
  b->o_rowb = al(b->o_tileb + (F + 1) * 8);
  b->o_mm = al(b->o_rowb + (F + 1) * 8);
  b->table_bytes = al(b->o_mm + 6 * F * 4);
  tdm_status st = batch_alloc((void**)&b->table, b->table_bytes, &b->device_bytes);
  if (!st) st = batch_alloc((void**)&b->occ, 2 * (size_t)b->cfg.max_voxels, &b->device_bytes);
  if (!st) st = batch_alloc((void**)&b->tdf, 4 * (size_t)b->cfg.max_voxels, &b->device_bytes);
  if (!st) st = batch_alloc((void**)&b->kp_grid, 12 * (size_t)std::max<int64_t>(cfg->max_keypoints, 1), &b->device_bytes);
  if (!st) st = batch_alloc((void**)&b->patches, (size_t)b->chunk * 27000 * 4, &b->device_bytes);
  if (!st && cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking) != cudaSuccess)
    st = fail(TDM_ERR_DEVICE, "tdm_batch_create: capture stream");
  if (!st) {
    cudaError_t e = cudaMallocHost((void**)&b->up, b->up_bytes + al(b->down_bytes));
    if (e != cudaSuccess) st = cuda_status(e, "batch staging");
    else b->down = b->up + b->up_bytes;
  }
  if (st) {
    delete b;
    return st;
  }
  *out = b;
  return TDM_OK;
}

extern "C" tdm_status tdm_batch_destroy(tdm_batch* b) {
  if (b) cudaDeviceSynchronize();
  delete b;
  return TDM_OK;
}

extern "C" size_t tdm_batch_device_bytes(const tdm_batch* b) { return b ? b->device_bytes : 0; }

extern "C" tdm_status tdm_batch_stats(const tdm_batch* b, int64_t* launches_per_call, int32_t* replayed) {
  TDM_REQUIRE(b, "tdm_batch_stats: null batch");
  if (launches_per_call) *launches_per_call = b->launches_per_call;
  if (replayed) *replayed = b->replayed;
  return TDM_OK;
}

extern "C" tdm_status tdm_describe_batch(tdm_batch* b, const float* pts, int32_t F, const int64_t* off,
                                         const float* vs, const int32_t* kps, const uint64_t* seeds, float* keypts,
                                         float* desc, tdm_grid* grids, tdm_stream s) {
  TDM_REQUIRE(b && pts && off && vs && kps && seeds && desc && keypts, "tdm_describe_batch: null pointer");
  TDM_REQUIRE(F >= 1 && F <= b->cfg.max_fragments, "tdm_describe_batch: fragment count outside 1..max_fragments");
  TDM_REQUIRE(off[0] == 0, "tdm_describe_batch: point_offsets[0] must be 0");
  // host table, checked
  FragIn* in = reinterpret_cast<FragIn*>(b->up + b->o_in);
  int64_t* ptb = reinterpret_cast<int64_t*>(b->up + b->o_ptb);
  int64_t* kpb = reinterpret_cast<int64_t*>(b->up + b->o_kpb);
  int64_t k_total = 0;
  int R = -1;
  for (int f = 0; f < F; ++f) {
    const int64_t n = off[f + 1] - off[f];
    TDM_REQUIRE(n > 0 && n < ((int64_t)1 << 31), "tdm_describe_batch: every fragment needs 1 .. 2^31-1 points");
    TDM_REQUIRE(vs[f] > 0.0f && kps[f] >= 0, "tdm_describe_batch: voxel sizes must be > 0 and keypoints >= 0");
    const float trunc = vs[f] * b->cfg.trunc_voxels;
    const int r = (int)roundf(trunc / vs[f]);  // the single-fragment search radius
    TDM_REQUIRE(R < 0 || r == R, "tdm_describe_batch: fragments must share one truncation radius in voxels");
    R = r;
    in[f] = FragIn{off[f], n, k_total, kps[f], vs[f], seeds[f]};
    ptb[f] = off[f];
    kpb[f] = k_total;
    k_total += kps[f];
  }
  ptb[F] = off[F];
  kpb[F] = k_total;
  TDM_REQUIRE(off[F] <= b->cfg.max_points, "tdm_describe_batch: points exceed the batch's max_points");
  TDM_REQUIRE(k_total <= b->cfg.max_keypoints, "tdm_describe_batch: keypoints exceed the batch's max_keypoints");
  TDM_REQUIRE(R >= 1 && R <= 10, "tdm_describe_batch: truncation must round to 1..10 voxels");
  b->R = R;
  const void* key[3] = {pts, keypts, desc};
  const bool same = b->exec && F == b->key_f && k_total == b->key_k && std::equal(key, key + 3, b->key_ptr) &&
                    net_generation(b->net) == b->key_gen;
  if (b->cfg.use_graph && same) {
    TDM_CHECK_CUDA(cudaGraphLaunch(b->exec, s));
    note_launches((int)b->launches_per_call);
    b->replayed = 1;
  } else {
    const int64_t before = tdm_launch_count();
    tdm_status st = run_sequence(b, pts, F, k_total, keypts, desc, s);
    if (st) return st;
    b->launches_per_call = tdm_launch_count() - before;
    b->replayed = 0;
    if (b->cfg.use_graph) {
      if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
      }
      cudaGraph_t graph = nullptr;
      TDM_CHECK_CUDA(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
      st = run_sequence(b, pts, F, k_total, keypts, desc, b->cap);
      cudaError_t e = cudaStreamEndCapture(b->cap, &graph);
      note_launches(-(int)b->launches_per_call);  // captured, not launched
      if (st) {
        if (graph) cudaGraphDestroy(graph);
        return st;
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, graph, 0);
      if (graph) cudaGraphDestroy(graph);
      if (e != cudaSuccess) return cuda_status(e, "tdm_describe_batch: graph capture");
      std::copy(key, key + 3, b->key_ptr);
      b->key_gen = net_generation(b->net);
      b->key_f = F;
      b->key_k = k_total;
    }
  }
  TDM_CHECK_CUDA(cudaStreamSynchronize(s));
  const FragGeo* geo = reinterpret_cast<const FragGeo*>(b->down);
  const Totals* tot = reinterpret_cast<const Totals*>(b->down + (b->o_tot - b->o_geo));
  if (tot->status == kGeometry)
    return fail(TDM_ERR_INVALID_ARG, "tdm_describe_batch: fragment " + std::to_string(tot->bad_fragment) +
                                         " has non-finite points, a too large extent or 2^31 voxels or more");
  if (tot->status == kCapacity) return fail(TDM_ERR_OOM, "tdm_describe_batch: grids exceed the batch's max_voxels");
  if (grids)
    for (int f = 0; f < F; ++f) {
      for (int a = 0; a < 3; ++a) {
        grids[f].dim[a] = geo[f].dim[a];
        grids[f].origin[a] = geo[f].origin[a];
      }
      grids[f].voxel_size = vs[f];
      grids[f].trunc_margin = vs[f] * b->cfg.trunc_voxels;
    }
  return TDM_OK;
}
