// TSDF fusion and surface extraction.
//
// Replaces Integrate (depth-fusion/demo.cu:18-68), launched there as
// <<<dim_z, dim_y>>> with an x loop inside each thread (every warp touches 32
// different rows: uncoalesced), and SaveVoxelGrid2SurfacePointCloud
// (core/utils.hpp:23-65, a host double pass over the grid).
//
// Here one thread owns one voxel, x fastest (coalesced), and integrates up to
// kMaxFrames frames per launch in order while the voxel's TSDF value and
// weight stay in registers: each launch reads and writes the two grids once.
// The per-frame arithmetic is the reference's, operation for operation; the
// file is compiled with -fmad=false so values match the CPU restatement bit
// for bit.
#include "common.cuh"

namespace tdm {
namespace {

constexpr int kMaxFrames = 32;

struct FrameBatch {
  float K[9];
  float c2b[kMaxFrames][16];
  int n;
};

__global__ void tsdf_init_kernel(float* __restrict__ tsdf, float* __restrict__ w, int64_t V) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < V) {
    tsdf[i] = 1.0f;
    w[i] = 0.0f;
  }
}

__global__ void depth_mm_kernel(const uint16_t* __restrict__ mm, int64_t n, float* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float d = (float)mm[i] / 1000.0f;
  out[i] = d > 6.0f ? 0.0f : d;
}

__global__ __launch_bounds__(256) void integrate_kernel(float* __restrict__ tsdf, float* __restrict__ weight, int dx,
                                                        int dy, int dz, float ox, float oy, float oz, float vs,
                                                        float trunc, const float* __restrict__ depth, int H, int W,
                                                        const FrameBatch fb) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t V = (int64_t)dx * dy * dz;
  if (v >= V) return;
  const int x = (int)(v % dx);
  const int y = (int)((v / dx) % dy);
  const int z = (int)(v / ((int64_t)dx * dy));
  const float bx = ox + (float)x * vs, by = oy + (float)y * vs, bz = oz + (float)z * vs;
  float ts = tsdf[v], wt = weight[v];
  bool touched = false;
  for (int f = 0; f < fb.n; ++f) {
    const float* c = fb.c2b[f];
    float t0 = bx - c[3], t1 = by - c[7], t2 = bz - c[11];
    float cx = c[0] * t0 + c[4] * t1 + c[8] * t2;
    float cy = c[1] * t0 + c[5] * t1 + c[9] * t2;
    float cz = c[2] * t0 + c[6] * t1 + c[10] * t2;
    if (cz <= 0) continue;
    int px = (int)roundf(fb.K[0] * (cx / cz) + fb.K[2]);
    int py = (int)roundf(fb.K[4] * (cy / cz) + fb.K[5]);
    if (px < 0 || px >= W || py < 0 || py >= H) continue;
    float d = __ldg(depth + (int64_t)f * H * W + (int64_t)py * W + px);
    if (d <= 0 || d > 6) continue;
    float qx = cx / cz, qy = cy / cz;
    float diff = (d - cz) * sqrtf(1 + qx * qx + qy * qy);
    if (diff <= -trunc) continue;
    float dist = fminf(1.0f, diff / trunc);
    float wn = wt + 1.0f;
    ts = (ts * wt + dist) / wn;
    wt = wn;
    touched = true;
  }
  if (touched) {
    tsdf[v] = ts;
    weight[v] = wt;
  }
}

constexpr int kExtractPerBlock = 4096;  // voxels per block (256 threads x 16)

__device__ __forceinline__ bool is_surface(const float* tsdf, const float* w, int64_t i, float thr, float wthr) {
  return fabsf(tsdf[i]) < thr && w[i] > wthr;
}

__global__ __launch_bounds__(256) void extract_count_kernel(const float* __restrict__ tsdf, const float* __restrict__ w,
                                                            int64_t V, float thr, float wthr, int* __restrict__ cnt) {
  int64_t base = (int64_t)blockIdx.x * kExtractPerBlock;
  int c = 0;
  for (int k = threadIdx.x; k < kExtractPerBlock; k += 256) {
    int64_t i = base + k;
    if (i < V && is_surface(tsdf, w, i, thr, wthr)) ++c;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  __shared__ int s[8];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int q = 0; q < 8; ++q) t += s[q];
    cnt[blockIdx.x] = t;
  }
}

// Exclusive scan of the block counts (one block) and the grand total.
__global__ __launch_bounds__(1024) void extract_scan_kernel(int* __restrict__ cnt, int nblk, int64_t* __restrict__ offs,
                                                            int64_t* __restrict__ total) {
  __shared__ int64_t s_carry;
  __shared__ int64_t s_w[32];
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int b0 = 0; b0 < nblk; b0 += 1024) {
    int b = b0 + threadIdx.x;
    int64_t v = b < nblk ? cnt[b] : 0;
    int64_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_w[w] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
      int64_t acc = 0;
      for (int q = 0; q < 32; ++q) { int64_t t = s_w[q]; s_w[q] = acc; acc += t; }
    }
    __syncthreads();
    if (b < nblk) offs[b] = s_carry + s_w[w] + x - v;
    __syncthreads();
    if (threadIdx.x == 1023) s_carry += s_w[31] + x;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = s_carry;
}

__global__ __launch_bounds__(256) void extract_write_kernel(const float* __restrict__ tsdf, const float* __restrict__ w,
                                                            int dx, int dy, int64_t V, float ox, float oy, float oz,
                                                            float vs, float thr, float wthr,
                                                            const int64_t* __restrict__ offs, int64_t max_pts,
                                                            float* __restrict__ pts) {
  __shared__ int s_warp[8];
  __shared__ int64_t s_base;
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_base = offs[blockIdx.x];
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kExtractPerBlock;
  for (int k0 = 0; k0 < kExtractPerBlock; k0 += 256) {
    int64_t i = base + k0 + threadIdx.x;
    int f = (i < V && is_surface(tsdf, w, i, thr, wthr)) ? 1 : 0;
    unsigned bal = __ballot_sync(0xffffffffu, f);
    int pre = __popc(bal & ((1u << lane) - 1));
    if (lane == 31) s_warp[wp] = pre + f;
    __syncthreads();
    if (threadIdx.x == 0) {
      int acc = 0;
      for (int q = 0; q < 8; ++q) { int t = s_warp[q]; s_warp[q] = acc; acc += t; }
    }
    __syncthreads();
    if (f) {
      int64_t pos = s_base + s_warp[wp] + pre;
      if (pos < max_pts) {
        int64_t z = i / ((int64_t)dx * dy);
        int64_t y = (i - z * dx * dy) / dx;
        int64_t x = i - z * dx * dy - y * dx;
        pts[3 * pos + 0] = ox + (float)x * vs;
        pts[3 * pos + 1] = oy + (float)y * vs;
        pts[3 * pos + 2] = oz + (float)z * vs;
      }
    }
    // advance by this round's count (the barrier also retires s_warp)
    int cnt_round = __syncthreads_count(f);
    if (threadIdx.x == 0) s_base += cnt_round;
    __syncthreads();
  }
}

}  // namespace
}  // namespace tdm

using namespace tdm;

extern "C" tdm_status tdm_tsdf_init(float* tsdf, float* w, const int32_t dim[3], tdm_stream s) {
  TDM_REQUIRE(tsdf && w && dim && dim[0] > 0 && dim[1] > 0 && dim[2] > 0, "tdm_tsdf_init: bad arguments");
  int64_t V = (int64_t)dim[0] * dim[1] * dim[2];
  tsdf_init_kernel<<<(unsigned)((V + 255) / 256), 256, 0, s>>>(tsdf, w, V);
  TDM_CHECK_LAUNCH("tsdf_init_kernel");
  return TDM_OK;
}

extern "C" tdm_status tdm_depth_from_mm(const uint16_t* mm, int64_t n, float* out, tdm_stream s) {
  TDM_REQUIRE(mm && out && n >= 0, "tdm_depth_from_mm: bad arguments");
  if (n == 0) return TDM_OK;
  depth_mm_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(mm, n, out);
  TDM_CHECK_LAUNCH("depth_mm_kernel");
  return TDM_OK;
}

extern "C" tdm_status tdm_tsdf_integrate(float* tsdf, float* w, const int32_t dim[3], const float origin[3], float vs,
                                         float trunc, const float* depth, int32_t n_frames, int32_t H, int32_t W,
                                         const float K[9], const float* c2b_host, tdm_stream s) {
  TDM_REQUIRE(tsdf && w && dim && origin && depth && K && c2b_host, "tdm_tsdf_integrate: null pointer");
  TDM_REQUIRE(n_frames >= 0 && H > 0 && W > 0 && vs > 0 && trunc > 0, "tdm_tsdf_integrate: bad arguments");
  int64_t V = (int64_t)dim[0] * dim[1] * dim[2];
  TDM_REQUIRE(V > 0, "tdm_tsdf_integrate: empty grid");
  for (int f0 = 0; f0 < n_frames; f0 += kMaxFrames) {
    FrameBatch fb;
    for (int i = 0; i < 9; ++i) fb.K[i] = K[i];
    fb.n = n_frames - f0 < kMaxFrames ? n_frames - f0 : kMaxFrames;
    for (int f = 0; f < fb.n; ++f)
      for (int i = 0; i < 16; ++i) fb.c2b[f][i] = c2b_host[(size_t)(f0 + f) * 16 + i];
    integrate_kernel<<<(unsigned)((V + 255) / 256), 256, 0, s>>>(tsdf, w, dim[0], dim[1], dim[2], origin[0],
                                                                 origin[1], origin[2], vs, trunc,
                                                                 depth + (size_t)f0 * H * W, H, W, fb);
    TDM_CHECK_LAUNCH("integrate_kernel");
  }
  return TDM_OK;
}

extern "C" size_t tdm_extract_workspace_bytes(const int32_t dim[3]) {
  if (!dim) return 0;
  int64_t V = (int64_t)dim[0] * dim[1] * dim[2];
  int64_t nblk = (V + kExtractPerBlock - 1) / kExtractPerBlock;
  return (size_t)nblk * 4 + (size_t)nblk * 8 + 64;
}

extern "C" tdm_status tdm_tsdf_extract(const float* tsdf, const float* w, const int32_t dim[3], const float origin[3],
                                       float vs, float thr, float wthr, float* pts, int64_t max_pts, int64_t* n_pts,
                                       void* ws, size_t ws_bytes, tdm_stream s) {
  TDM_REQUIRE(tsdf && w && dim && origin && pts && n_pts && ws && max_pts >= 0, "tdm_tsdf_extract: bad arguments");
  TDM_REQUIRE(ws_bytes >= tdm_extract_workspace_bytes(dim), "tdm_tsdf_extract: workspace too small");
  int64_t V = (int64_t)dim[0] * dim[1] * dim[2];
  int nblk = (int)((V + kExtractPerBlock - 1) / kExtractPerBlock);
  uint8_t* b = static_cast<uint8_t*>(ws);
  int64_t* offs = reinterpret_cast<int64_t*>(b);
  int* cnt = reinterpret_cast<int*>(b + (size_t)nblk * 8);
  extract_count_kernel<<<nblk, 256, 0, s>>>(tsdf, w, V, thr, wthr, cnt);
  extract_scan_kernel<<<1, 1024, 0, s>>>(cnt, nblk, offs, n_pts);
  extract_write_kernel<<<nblk, 256, 0, s>>>(tsdf, w, dim[0], dim[1], V, origin[0], origin[1], origin[2], vs, thr,
                                            wthr, offs, max_pts, pts);
  note_launches(2);
  TDM_CHECK_LAUNCH("tsdf extract");
  return TDM_OK;
}
