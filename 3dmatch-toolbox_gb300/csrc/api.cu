// Library-level entry points: version, error reporting, device error word,
// and the voxel-grid geometry of core/demo.cu:97-124.
#include <atomic>
#include <cmath>
#include <map>
#include <utility>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "internal.h"
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

int device_sm_count() {
  static std::mutex mu;
  static std::vector<int> counts;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 148;
  std::lock_guard<std::mutex> lk(mu);
  if ((int)counts.size() <= dev) counts.resize(dev + 1, 0);
  if (counts[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return 148;
    counts[dev] = n;
  }
  return counts[dev];
}

// The dynamic shared-memory cap is an attribute of a kernel on one device:
// each (kernel, device) pair gets it once, from whichever host thread comes
// first; later calls return the recorded outcome.
cudaError_t raise_smem_cap(const void* func, int bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, cudaError_t> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_pair(func, dev);
  auto it = done.find(key);
  if (it != done.end()) return it->second;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  done[key] = e;
  return e;
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

extern "C" tdm_status tdm_selftest_wait_timeout(uint32_t budget_us, int32_t* out_dev, tdm_stream s) {
  TDM_REQUIRE(out_dev, "tdm_selftest_wait_timeout: null pointer");
  TDM_REQUIRE(budget_us >= 1 && budget_us <= 1000000, "tdm_selftest_wait_timeout: budget must be 1 us .. 1 s");
  return launch_wait_selftest((uint64_t)budget_us * 1000ull, out_dev, s);
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
  // Bounds as the device form takes them (fminf/fmaxf from +/-inf): a NaN
  // coordinate is skipped, so both forms give the same grid for any input.
  // For finite clouds this is the reference's running min/max from pts[0].
  float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int32_t i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) {
      float v = pts[3 * (int64_t)i + a];
      mn[a] = std::fmin(mn[a], v);
      mx[a] = std::fmax(mx[a], v);
    }
  return grid_from_minmax(mn, mx, vs, trunc, pad, g);
}
