// TDF voxelisation, keypoint selection and 30^3 patch gather.
//
// Replaces core/demo.cu:97-218.  The reference's ComputeTDF (core/demo.cu:22-57)
// scans an 11^3 cube per empty voxel (1,331 occupancy reads).  Here the same
// value comes from an exact separable windowed squared distance (an in-plane
// pass per z-plane in shared memory, then a pass along z):
//   g1 = min_{|dx|<=r, occ} dx^2,  g2 = min_{|dy|<=r} dy^2 + g1,  g3 = min_{|dz|<=r} dz^2 + g2
// which is the minimum of dx^2+dy^2+dz^2 over the occupied voxels of the cube.
// Because sqrtf, /r and 1-x are monotone, 1 - sqrtf(g3)/r equals the
// reference's running max of 1 - sqrtf(d^2)/r bit for bit (integer d^2 is
// exact in float; sqrtf and the division are IEEE round-to-nearest).
#include <algorithm>
#include <climits>

#include "common.cuh"
#include "tdf_core.cuh"

namespace tdm {
tdm_status grid_from_minmax(const float mn[3], const float mx[3], float vs, float trunc, int32_t pad, tdm_grid* g);
}
using namespace tdm;

namespace {


__global__ void minmax_init_kernel(int* ws) {
  if (threadIdx.x < 3) ws[threadIdx.x] = INT_MAX;
  else if (threadIdx.x < 6) ws[threadIdx.x] = INT_MIN;
}

__global__ __launch_bounds__(256) void minmax_kernel(const float* __restrict__ pts, int n, int* ws) {
  float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      float v = pts[3 * (int64_t)i + a];
      mn[a] = fminf(mn[a], v);
      mx[a] = fmaxf(mx[a], v);
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mn[a] = fminf(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
      mx[a] = fmaxf(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
    }
  }
  // block reduction first: one set of six atomics per block, not per warp
  __shared__ float s_mn[8][3], s_mx[8][3];
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0)
    for (int a = 0; a < 3; ++a) { s_mn[w][a] = mn[a]; s_mx[w][a] = mx[a]; }
  __syncthreads();
  if (threadIdx.x < 3) {
    const int a = threadIdx.x;
    float lo = s_mn[0][a], hi = s_mx[0][a];
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) { lo = fminf(lo, s_mn[k][a]); hi = fmaxf(hi, s_mx[k][a]); }
    atomicMin(ws + a, float_to_ordered(lo));
    atomicMax(ws + 3 + a, float_to_ordered(hi));
  }
}

// occ[(z*dy + y)*X + x] = 1, x = round((p - o)/vs)   (core/demo.cu:127-135; X = occ_pitch(dx))
__global__ __launch_bounds__(256) void occupancy_kernel(const float* __restrict__ pts, int n, int dx, int dy, int dz,
                                                        float ox, float oy, float oz, float vs,
                                                        uint8_t* __restrict__ occ) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float px = pts[3 * (int64_t)i], py = pts[3 * (int64_t)i + 1], pz = pts[3 * (int64_t)i + 2];
  if (!(isfinite(px) && isfinite(py) && isfinite(pz))) return;  // skipped, as by the grid bounds
  int gx = voxel_coord(px, ox, vs), gy = voxel_coord(py, oy, vs), gz = voxel_coord(pz, oz, vs);
  if (gx < 0 || gy < 0 || gz < 0 || gx >= dx || gy >= dy || gz >= dz) return;
  occ[((int64_t)gz * dy + gy) * occ_pitch(dx) + gx] = 1;
}

// Pass A (plane_tile), one tile of one z-plane per block.
template <int R>
__global__ __launch_bounds__(256) void tdf_plane_kernel(const uint8_t* __restrict__ occ, int dx, int dy,
                                                        uint8_t* __restrict__ g2) {
  __shared__ PlaneSmem<R> sm;
  plane_tile<R>(occ, dx, dy, g2, blockIdx.x * PB_TX, blockIdx.y * PB_TY, blockIdx.z, sm);
}

// Pass B (z_column): a warp work item is (y, 128-voxel x segment, 32-step z
// chunk); blocks of 4 warps walk the items.
constexpr int kZThreads = 128;
template <int R>
__global__ __launch_bounds__(kZThreads) void tdf_z_kernel(const uint8_t* __restrict__ g2, int dx, int dy, int dz,
                                                          float* __restrict__ tdf) {
  __shared__ float lut[256];
  __shared__ float s_w[kZThreads / 32][128];
  tdf_lut<R>(lut);
  __syncthreads();
  const int nseg = (dx + 127) / 128, nzc = (dz + kZChunk - 1) / kZChunk;
  const int64_t items = (int64_t)dy * nseg * nzc;
  const int w = threadIdx.x >> 5;
  for (int64_t it = (int64_t)blockIdx.x * (kZThreads / 32) + w; it < items; it += (int64_t)gridDim.x * (kZThreads / 32)) {
    const int zc = (int)(it % nzc);
    const int64_t r = it / nzc;
    const int seg = (int)(r % nseg), y = (int)(r / nseg);
    z_column<R>(g2, dx, dy, dz, y, seg * 128, zc * kZChunk, min(dz, (zc + 1) * kZChunk), lut, s_w[w], tdf);
  }
}

int z_blocks() { return tdm::device_sm_count() * 16; }

// The reference decodes voxel_idx through float32 (core/demo.cu:32-34); above
// 2^24 that lands on a different (x,y,z).  mode 1 evaluates its expressions
// without contraction, mode 2 with nvcc's default a - b*c -> fma(-b, c, a).
__device__ __forceinline__ void refcompat_decode(int64_t idx, int dx, int dy, int mode, int& x, int& y, int& z) {
  float fi = (float)idx, fx = (float)dx, fy = (float)dy;
  z = (int)floorf(__fdiv_rn(fi, __fmul_rn(fx, fy)));
  float zp = __fmul_rn((float)z, fx);
  float u = mode == 1 ? __fsub_rn(fi, __fmul_rn(zp, fy)) : __fmaf_rn(-zp, fy, fi);
  y = (int)floorf(__fdiv_rn(u, fx));
  float xr = mode == 1 ? __fsub_rn(u, __fmul_rn((float)y, fx)) : __fmaf_rn(-(float)y, fx, u);
  x = (int)xr;
}

// Re-evaluates, for voxels >= 2^24 whose float decode differs from the exact
// one, the reference loop around the mis-decoded centre (clipped window, max of
// 1 - sqrtf(d^2)/r over occupied voxels, initial 0).
__global__ __launch_bounds__(256) void tdf_refcompat_kernel(const uint8_t* __restrict__ occ, int dx, int dy, int dz,
                                                            int r, int mode, int64_t v0, int64_t V,
                                                            float* __restrict__ tdf) {
  int64_t idx = v0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= V) return;
  int64_t plane = (int64_t)dx * dy;
  int ez = (int)(idx / plane);
  int ey = (int)((idx - (int64_t)ez * plane) / dx);
  int ex = (int)(idx - (int64_t)ez * plane - (int64_t)ey * dx);
  int x, y, z;
  refcompat_decode(idx, dx, dy, mode, x, y, z);
  const int64_t X = occ_pitch(dx);
  if ((x == ex && y == ey && z == ez) || occ[((int64_t)ez * dy + ey) * X + ex]) return;
  float best = 0.0f;
  int xa = max(0, x - r), xb = min(dx, x + r + 1);
  int ya = max(0, y - r), yb = min(dy, y + r + 1);
  int za = max(0, z - r), zb = min(dz, z + r + 1);
  for (int iz = za; iz < zb; ++iz)
    for (int iy = ya; iy < yb; ++iy)
      for (int ix = xa; ix < xb; ++ix)
        if (occ[((int64_t)iz * dy + iy) * X + ix]) {
          int d2 = (x - ix) * (x - ix) + (y - iy) * (y - iy) + (z - iz) * (z - iz);
          float v = __fsub_rn(1.0f, __fdiv_rn(__fsqrt_rn((float)d2), (float)r));
          if (v > best) best = v;
        }
  tdf[idx] = best;
}

__global__ void keypoint_index_kernel(uint64_t seed, uint32_t n_pts, int k, int32_t* idx) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k) return;
  idx[i] = keypoint_index(seed, n_pts, i);
}

// keypts = pts[idx]; grid = round((p - o)/vs)   (core/demo.cu:168-176)
__global__ void keypoint_kernel(const float* __restrict__ pts, int n_pts, const int32_t* __restrict__ idx, int k,
                                float ox, float oy, float oz, float vs, float* __restrict__ keypts,
                                int32_t* __restrict__ kp_grid, int* err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k) return;
  int j = idx[i];
  if (j < 0 || j >= n_pts) {
    atomicExch(err, DEV_BAD_INDEX);
    j = 0;
  }
  float o[3] = {ox, oy, oz};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float p = pts[3 * (int64_t)j + a];
    keypts[3 * i + a] = p;
    kp_grid[3 * i + a] = voxel_coord(p, o[a], vs);
  }
}

// patches[k][z][y][x] = tdf[kz-15+z][ky-15+y][kx-15+x]   (core/demo.cu:206-217)
__global__ __launch_bounds__(256) void gather_kernel(const float* __restrict__ tdf, int dx, int dy, int dz,
                                                     const int32_t* __restrict__ kp_grid,
                                                     float* __restrict__ patches) {
  const int k = blockIdx.x;
  gather_patch(tdf, dx, dy, dz, kp_grid[3 * k] - 15, kp_grid[3 * k + 1] - 15, kp_grid[3 * k + 2] - 15,
               patches + (int64_t)k * 27000);
}

// Exact TDF (evaluation/model-fitting-apc/pointCloud2TDF.m,
// deprecated/pointCloud2AccTDF.m): 1 - min(d / trunc, 1) with d the distance
// from the voxel centre o + i vs to the nearest point.  Each point lowers the
// squared distance of every voxel centre within trunc (atomicMin on the bits
// of a non-negative float orders like the float); untouched voxels keep +inf
// and become 0.
__global__ void exact_fill_kernel(uint32_t* __restrict__ d2, int64_t V) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < V; i += (int64_t)gridDim.x * blockDim.x)
    d2[i] = 0x7F800000u;
}

__global__ void exact_scatter_kernel(const float* __restrict__ pts, int n, int dx, int dy, int dz, float ox, float oy,
                                     float oz, float vs, float trunc, uint32_t* __restrict__ d2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float p[3] = {pts[3 * (int64_t)i], pts[3 * (int64_t)i + 1], pts[3 * (int64_t)i + 2]};
  const float o[3] = {ox, oy, oz};
  const int dim[3] = {dx, dy, dz};
  int lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    const float u = (p[a] - o[a]) / vs, w = trunc / vs;
    if (!(u - w < 2.0e9f && u + w > -2.0e9f)) return;  // non-finite or absurd coordinates touch no voxel
    lo[a] = max(0, (int)ceilf(u - w) - 1);
    hi[a] = min(dim[a] - 1, (int)floorf(u + w) + 1);
    if (lo[a] > hi[a]) return;
  }
  // centre - point in double: a float centre o + i vs carries ~1e-7 of the
  // coordinate's magnitude, which is more than the 1e-6 TDF budget allows
  const double t2 = (double)trunc * trunc, vsd = vs;
  for (int z = lo[2]; z <= hi[2]; ++z) {
    const double ez = ((double)o[2] + z * vsd) - p[2];
    for (int y = lo[1]; y <= hi[1]; ++y) {
      const double ey = ((double)o[1] + y * vsd) - p[1];
      const double eyz = ey * ey + ez * ez;
      if (eyz >= t2) continue;
      for (int x = lo[0]; x <= hi[0]; ++x) {
        const double ex = ((double)o[0] + x * vsd) - p[0];
        const double e2 = ex * ex + eyz;
        if (e2 < t2) atomicMin(d2 + ((int64_t)z * dy + y) * dx + x, __float_as_uint((float)e2));
      }
    }
  }
}

__global__ void exact_value_kernel(float* __restrict__ tdf, int64_t V, float trunc) {
  uint32_t* d2 = reinterpret_cast<uint32_t*>(tdf);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < V; i += (int64_t)gridDim.x * blockDim.x) {
    const float e2 = __uint_as_float(d2[i]);
    tdf[i] = 1.0f - fminf(sqrtf(e2) / trunc, 1.0f);
  }
}

template <int R>
void launch_tdf(const uint8_t* occ, uint8_t* g2, const tdm_grid* g, float* tdf, cudaStream_t s) {
  dim3 ga((g->dim[0] + PB_TX - 1) / PB_TX, (g->dim[1] + PB_TY - 1) / PB_TY, g->dim[2]);
  tdf_plane_kernel<R><<<ga, 256, 0, s>>>(occ, g->dim[0], g->dim[1], g2);
  const int64_t items = (int64_t)g->dim[1] * ((g->dim[0] + 127) / 128) * ((g->dim[2] + kZChunk - 1) / kZChunk);
  const int64_t blocks = std::min<int64_t>((items + kZThreads / 32 - 1) / (kZThreads / 32), z_blocks());
  tdf_z_kernel<R><<<(unsigned)blocks, kZThreads, 0, s>>>(g2, g->dim[0], g->dim[1], g->dim[2], tdf);
}

// bytes of the pitched occupancy (and of the pitched in-plane array)
size_t pitched_voxels(const tdm_grid* g) { return (size_t)occ_pitch(g->dim[0]) * g->dim[1] * g->dim[2]; }

int search_radius(const tdm_grid* g) { return (int)roundf(g->trunc_margin / g->voxel_size); }

}  // namespace

extern "C" size_t tdm_grid_workspace_bytes(void) { return 64; }

extern "C" tdm_status tdm_grid_from_points(const float* pts, int32_t n, float vs, float trunc, int32_t pad,
                                           tdm_grid* g, void* ws, tdm_stream s) {
  TDM_REQUIRE(pts && g && ws && n > 0, "tdm_grid_from_points: null pointer or n <= 0");
  int* w = static_cast<int*>(ws);
  minmax_init_kernel<<<1, 32, 0, s>>>(w);
  int blocks = (n + 255) / 256;
  blocks = blocks > 304 ? 304 : blocks;  // two blocks per SM, grid-stride over the points
  minmax_kernel<<<blocks, 256, 0, s>>>(pts, n, w);
  note_launches(1);  // minmax_init_kernel
  TDM_CHECK_LAUNCH("minmax_kernel");
  int h[6];
  TDM_CHECK_CUDA(cudaMemcpyAsync(h, w, sizeof(h), cudaMemcpyDeviceToHost, s));
  TDM_CHECK_CUDA(cudaStreamSynchronize(s));
  float mn[3], mx[3];
  for (int a = 0; a < 3; ++a) {
    mn[a] = ordered_to_float(h[a]);
    mx[a] = ordered_to_float(h[3 + a]);
  }
  return grid_from_minmax(mn, mx, vs, trunc, pad, g);
}

extern "C" size_t tdm_tdf_workspace_bytes(const tdm_grid* g) {
  if (!g) return 0;
  // occupancy + in-plane squared distances, bytes, x rows padded to 4
  return 2 * pitched_voxels(g);
}

extern "C" tdm_status tdm_tdf(const float* pts, int32_t n, const tdm_grid* g, int32_t mode, float* tdf, void* ws,
                              size_t ws_bytes, tdm_stream s) {
  TDM_REQUIRE(pts && g && tdf && ws && n > 0, "tdm_tdf: null pointer or n <= 0");
  TDM_REQUIRE(mode >= 0 && mode <= 2, "tdm_tdf: decode_mode must be 0, 1 or 2");
  const size_t V = (size_t)g->dim[0] * g->dim[1] * g->dim[2];
  TDM_REQUIRE(V > 0 && ws_bytes >= tdm_tdf_workspace_bytes(g), "tdm_tdf: workspace too small");
  int r = search_radius(g);
  TDM_REQUIRE(r >= 1 && r <= 10, "tdm_tdf: trunc_margin/voxel_size must round to 1..10 voxels");
  const size_t PV = pitched_voxels(g);
  uint8_t* occ = static_cast<uint8_t*>(ws);
  uint8_t* g2 = occ + PV;
  TDM_CHECK_CUDA(cudaMemsetAsync(occ, 0, PV, s));
  occupancy_kernel<<<(n + 255) / 256, 256, 0, s>>>(pts, n, g->dim[0], g->dim[1], g->dim[2], g->origin[0],
                                                   g->origin[1], g->origin[2], g->voxel_size, occ);
  TDM_CHECK_LAUNCH("occupancy_kernel");
  switch (r) {
    case 1: launch_tdf<1>(occ, g2, g, tdf, s); break;
    case 2: launch_tdf<2>(occ, g2, g, tdf, s); break;
    case 3: launch_tdf<3>(occ, g2, g, tdf, s); break;
    case 4: launch_tdf<4>(occ, g2, g, tdf, s); break;
    case 5: launch_tdf<5>(occ, g2, g, tdf, s); break;
    case 6: launch_tdf<6>(occ, g2, g, tdf, s); break;
    case 7: launch_tdf<7>(occ, g2, g, tdf, s); break;
    case 8: launch_tdf<8>(occ, g2, g, tdf, s); break;
    case 9: launch_tdf<9>(occ, g2, g, tdf, s); break;
    default: launch_tdf<10>(occ, g2, g, tdf, s); break;
  }
  note_launches(1);
  TDM_CHECK_LAUNCH("tdf_plane_kernel / tdf_z_kernel");
  const int64_t first_bad = (int64_t)1 << 24;
  if (mode != TDM_TDF_EXACT && (int64_t)V > first_bad) {
    int64_t cnt = (int64_t)V - first_bad;
    tdf_refcompat_kernel<<<(unsigned)((cnt + 255) / 256), 256, 0, s>>>(occ, g->dim[0], g->dim[1], g->dim[2], r,
                                                                        mode, first_bad, (int64_t)V, tdf);
    TDM_CHECK_LAUNCH("tdf_refcompat_kernel");
  }
  return TDM_OK;
}

extern "C" tdm_status tdm_tdf_exact(const float* pts, int32_t n, const tdm_grid* g, float* tdf, tdm_stream s) {
  TDM_REQUIRE(pts && g && tdf && n > 0, "tdm_tdf_exact: null pointer or n <= 0");
  TDM_REQUIRE(g->voxel_size > 0.0f && g->trunc_margin > 0.0f, "tdm_tdf_exact: voxel size and truncation must be > 0");
  TDM_REQUIRE(g->trunc_margin <= 32.0f * g->voxel_size, "tdm_tdf_exact: truncation above 32 voxels");
  const int64_t V = (int64_t)g->dim[0] * g->dim[1] * g->dim[2];
  TDM_REQUIRE(V > 0, "tdm_tdf_exact: empty grid");
  uint32_t* d2 = reinterpret_cast<uint32_t*>(tdf);
  exact_fill_kernel<<<(unsigned)std::min<int64_t>((V + 255) / 256, 8192), 256, 0, s>>>(d2, V);
  exact_scatter_kernel<<<(n + 127) / 128, 128, 0, s>>>(pts, n, g->dim[0], g->dim[1], g->dim[2], g->origin[0],
                                                       g->origin[1], g->origin[2], g->voxel_size, g->trunc_margin, d2);
  exact_value_kernel<<<(unsigned)std::min<int64_t>((V + 255) / 256, 8192), 256, 0, s>>>(tdf, V, g->trunc_margin);
  note_launches(2);
  TDM_CHECK_LAUNCH("tdm_tdf_exact");
  return TDM_OK;
}

extern "C" tdm_status tdm_keypoint_indices(uint64_t seed, int32_t n_pts, int32_t k, int32_t* idx, tdm_stream s) {
  TDM_REQUIRE(idx && n_pts > 0 && k >= 0, "tdm_keypoint_indices: bad arguments");
  if (k == 0) return TDM_OK;
  keypoint_index_kernel<<<(k + 255) / 256, 256, 0, s>>>(seed, (uint32_t)n_pts, k, idx);
  TDM_CHECK_LAUNCH("keypoint_index_kernel");
  return TDM_OK;
}

extern "C" tdm_status tdm_keypoints(const float* pts, int32_t n_pts, const int32_t* idx, int32_t k, const tdm_grid* g,
                                    float* keypts, int32_t* kp_grid, tdm_stream s) {
  TDM_REQUIRE(pts && idx && g && keypts && kp_grid && n_pts > 0 && k >= 0, "tdm_keypoints: bad arguments");
  if (k == 0) return TDM_OK;
  int* err = device_error_word();
  if (!err) return fail(TDM_ERR_DEVICE, "device error word unavailable");
  keypoint_kernel<<<(k + 127) / 128, 128, 0, s>>>(pts, n_pts, idx, k, g->origin[0], g->origin[1], g->origin[2],
                                                  g->voxel_size, keypts, kp_grid, err);
  TDM_CHECK_LAUNCH("keypoint_kernel");
  return TDM_OK;
}

extern "C" tdm_status tdm_gather(const float* tdf, const tdm_grid* g, const int32_t* kp_grid, int32_t k, float* patches,
                                 tdm_stream s) {
  TDM_REQUIRE(tdf && g && kp_grid && patches && k >= 0, "tdm_gather: bad arguments");
  if (k == 0) return TDM_OK;
  gather_kernel<<<k, 256, 0, s>>>(tdf, g->dim[0], g->dim[1], g->dim[2], kp_grid, patches);
  TDM_CHECK_LAUNCH("gather_kernel");
  return TDM_OK;
}
