// Library-level entry points: version, error reporting, device error word,
// and the voxel-grid geometry of core/demo.cu:97-124.
#include <atomic>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "tdf_core.cuh"

namespace tdm {

static thread_local std::string g_last_error;
static std::atomic<int64_t> g_launches{0};

void set_error(const std::string& msg) { g_last_error = msg; }

void note_launches(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

tdm_status fail(tdm_status st, const std::string& msg) {
  set_error(msg);
  return st;
}

tdm_status cuda_status(cudaError_t e, const char* what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? TDM_ERR_OOM : TDM_ERR_DEVICE;
}

int* device_error_word() {
  static std::mutex mu;
  static std::vector<int*> words;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if ((int)words.size() <= dev) words.resize(dev + 1, nullptr);
  if (!words[dev]) {
    int* p = nullptr;
    if (cudaMalloc(&p, sizeof(int)) != cudaSuccess) return nullptr;
    // cudaMemset is queued on the legacy stream, which kernels on
    // non-blocking streams do not wait for: finish it before publishing
    if (cudaMemset(p, 0, sizeof(int)) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return nullptr;
    words[dev] = p;
  }
  return words[dev];
}

}  // namespace tdm

using namespace tdm;

extern "C" const char* tdm_version(void) { return "tdm-gb300 0.1 (sm_103a)"; }

extern "C" const char* tdm_last_error(void) { return g_last_error.c_str(); }

extern "C" int64_t tdm_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

extern "C" tdm_status tdm_device_status(tdm_stream s) {
  int* w = device_error_word();
  if (!w) return fail(TDM_ERR_DEVICE, "device error word unavailable");
  int h = 0;
  TDM_CHECK_CUDA(cudaMemcpyAsync(&h, w, sizeof(int), cudaMemcpyDeviceToHost, s));
  TDM_CHECK_CUDA(cudaStreamSynchronize(s));
  if (h == DEV_OK) return TDM_OK;
  TDM_CHECK_CUDA(cudaMemsetAsync(w, 0, sizeof(int), s));
  TDM_CHECK_CUDA(cudaStreamSynchronize(s));
  const char* what = h == DEV_BAD_INDEX ? "index check failed in a kernel" : "a bounded device wait ran out";
  return fail(h == DEV_BAD_INDEX ? TDM_ERR_DEVICE : TDM_ERR_TIMEOUT, std::string("device error: ") + what);
}

// ---------------------------------------------------------------------------
// Grid geometry, core/demo.cu:97-124.  Host float arithmetic exactly as the
// reference writes it (the library is compiled with -ffp-contract=off).
// ---------------------------------------------------------------------------
namespace tdm {
tdm_status grid_from_minmax(const float mn[3], const float mx[3], float vs, float trunc, int32_t pad, tdm_grid* g) {
  if (!(vs > 0.0f) || pad < 0) return fail(TDM_ERR_INVALID_ARG, "voxel_size must be > 0 and pad >= 0");
  int64_t V = 1;
  for (int a = 0; a < 3; ++a) {
    if (grid_axis(mn[a], mx[a], vs, pad, &g->dim[a], &g->origin[a]))
      return fail(TDM_ERR_INVALID_ARG, "non-finite point coordinates or grid extent too large");
    V *= g->dim[a];
  }
  if (V >= ((int64_t)1 << 31)) return fail(TDM_ERR_INVALID_ARG, "grid has 2^31 voxels or more");
  g->voxel_size = vs;
  g->trunc_margin = trunc;
  return TDM_OK;
}
}  // namespace tdm

extern "C" tdm_status tdm_grid_from_points_host(const float* pts, int32_t n, float vs, float trunc, int32_t pad,
                                                tdm_grid* g) {
  TDM_REQUIRE(pts && g && n > 0, "tdm_grid_from_points_host: null pointer or n <= 0");
  float mn[3] = {pts[0], pts[1], pts[2]}, mx[3] = {pts[0], pts[1], pts[2]};
  for (int32_t i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) {
      float v = pts[3 * (int64_t)i + a];
      mn[a] = v < mn[a] ? v : mn[a];
      mx[a] = v > mx[a] ? v : mx[a];
    }
  return grid_from_minmax(mn, mx, vs, trunc, pad, g);
}
