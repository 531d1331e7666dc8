// Device-resident fragment store: the keypoints and descriptors of described
// fragments, kept on the GPU across calls so that a fragment is described once
// and registered against many others.
//
// The reference describes every fragment of a scene once (`demo` per fragment,
// evaluation/geometric-registration/getKeyptsAndDesc.m:34-43, keypts.bin and
// desc.3dmatch.bin on disk) and then registers every pair from those files
// (runFragmentRegistration.m:27-53 -> register2Fragments.m:18-59).  Here the
// files are entries of one device arena of a fixed byte budget:
//   entry = keypoints (k x 3 float) | descriptors (k x 512 float), both
//           256-byte aligned, keyed by a caller-chosen 64-bit fragment key.
// Free space is a coalesced first-fit list; when a new entry does not fit, the
// least recently used entries that no call is reading are evicted.  Writes are
// stream ordered: an entry's `ready` event follows the copy or the forward that
// filled it, readers on other streams wait for it, and eviction waits for it.
#include <cuda_runtime.h>

#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "internal.h"
#include "tdm.h"

namespace tdm {
tdm_status fail(tdm_status st, const std::string& msg);
tdm_status cuda_status(cudaError_t e, const char* what);
}  // namespace tdm

// Status plumbing of the CUDA translation units (common.cuh is device code).
#define TDM_CHECK_CUDA(expr)                                     \
  do {                                                           \
    cudaError_t _e = (expr);                                     \
    if (_e != cudaSuccess) return ::tdm::cuda_status(_e, #expr); \
  } while (0)
#define TDM_REQUIRE(cond, msg)                                   \
  do {                                                           \
    if (!(cond)) return ::tdm::fail(TDM_ERR_INVALID_ARG, msg);   \
  } while (0)

namespace {

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct Entry {
  uint64_t seed = 0;
  int32_t k = 0;
  tdm_grid grid{};
  size_t off = 0, bytes = 0;
  uint64_t stamp = 0;
  int pins = 0;
  bool writing = false;  // reserved, not yet committed: `ready` is not recorded
  cudaEvent_t ready = nullptr;
};

}  // namespace

struct tdm_store {
  std::mutex mu;
  int device = 0;
  uint8_t* arena = nullptr;
  size_t cap = 0, used = 0;
  std::map<uint64_t, Entry> entries;
  std::map<size_t, size_t> free_;  // offset -> bytes, coalesced
  uint64_t clock = 0;
  int64_t hits = 0, misses = 0, evictions = 0;

  ~tdm_store() {
    for (auto& e : entries)
      if (e.second.ready) cudaEventDestroy(e.second.ready);
    if (arena) cudaFree(arena);
  }

  static size_t entry_bytes(int32_t k) { return align256((size_t)k * 12) + align256((size_t)k * 2048); }

  void release(size_t off, size_t bytes) {
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
    used -= bytes;
  }

  bool take(size_t bytes, size_t* off) {
    for (auto it = free_.begin(); it != free_.end(); ++it)
      if (it->second >= bytes) {
        *off = it->first;
        const size_t rest = it->second - bytes, roff = it->first + bytes;
        free_.erase(it);
        if (rest) free_.emplace(roff, rest);
        used += bytes;
        return true;
      }
    return false;
  }

  // Drops an entry (the caller holds mu; the entry is not pinned).
  void drop(std::map<uint64_t, Entry>::iterator it) {
    if (it->second.ready) {
      cudaEventSynchronize(it->second.ready);  // its writer has finished
      cudaEventDestroy(it->second.ready);
    }
    release(it->second.off, it->second.bytes);
    entries.erase(it);
  }

  // Space for `bytes`, evicting least recently used unpinned entries.
  tdm_status make_room(size_t bytes, size_t* off) {
    if (bytes > cap) return tdm::fail(TDM_ERR_OOM, "fragment store: entry larger than the store's budget");
    while (!take(bytes, off)) {
      auto victim = entries.end();
      for (auto it = entries.begin(); it != entries.end(); ++it)
        if (it->second.pins == 0 && (victim == entries.end() || it->second.stamp < victim->second.stamp)) victim = it;
      if (victim == entries.end())
        return tdm::fail(TDM_ERR_OOM, "fragment store: every entry is in use and the budget is full");
      drop(victim);
      ++evictions;
    }
    return TDM_OK;
  }
};

namespace tdm {

// Reserves (or replaces) the entry `key` for k keypoints, pinned for writing.
tdm_status store_reserve(tdm_store* st, uint64_t key, uint64_t seed, int32_t k, const tdm_grid* grid,
                         float** keypts, float** desc) {
  std::lock_guard<std::mutex> lk(st->mu);
  auto it = st->entries.find(key);
  if (it != st->entries.end()) {
    if (it->second.pins) return fail(TDM_ERR_INVALID_ARG, "fragment store: entry is being read or written");
    st->drop(it);
  }
  Entry e;
  e.seed = seed;
  e.k = k;
  if (grid) e.grid = *grid;
  e.bytes = tdm_store::entry_bytes(k);
  tdm_status s = st->make_room(e.bytes, &e.off);
  if (s) return s;
  if (cudaEventCreateWithFlags(&e.ready, cudaEventDisableTiming) != cudaSuccess) {
    st->release(e.off, e.bytes);
    return fail(TDM_ERR_DEVICE, "fragment store: event");
  }
  e.stamp = ++st->clock;
  e.pins = 1;
  e.writing = true;
  *keypts = reinterpret_cast<float*>(st->arena + e.off);
  *desc = reinterpret_cast<float*>(st->arena + e.off + align256((size_t)k * 12));
  st->entries.emplace(key, e);
  return TDM_OK;
}

// Ends a write: records `ready` on the writing stream and unpins.  On failure
// the entry is removed.
tdm_status store_commit(tdm_store* st, uint64_t key, const tdm_grid* grid, bool ok, cudaStream_t s) {
  std::lock_guard<std::mutex> lk(st->mu);
  auto it = st->entries.find(key);
  if (it == st->entries.end()) return fail(TDM_ERR_INVALID_ARG, "fragment store: no such entry");
  it->second.pins -= 1;
  it->second.writing = false;
  if (!ok) {
    cudaStreamSynchronize(s);
    st->drop(it);
    return TDM_OK;
  }
  if (grid) it->second.grid = *grid;
  TDM_CHECK_CUDA(cudaEventRecord(it->second.ready, s));
  return TDM_OK;
}

// Pins an entry for reading on stream s (which then waits for its writer).
tdm_status store_acquire(tdm_store* st, uint64_t key, StoreView* v, cudaStream_t s) {
  std::lock_guard<std::mutex> lk(st->mu);
  auto it = st->entries.find(key);
  if (it == st->entries.end())
    return fail(TDM_ERR_INVALID_ARG, "fragment store: no fragment with key " + std::to_string(key));
  Entry& e = it->second;
  if (e.writing) return fail(TDM_ERR_INVALID_ARG, "fragment store: entry is still being written");
  TDM_CHECK_CUDA(cudaStreamWaitEvent(s, e.ready, 0));
  e.pins += 1;
  e.stamp = ++st->clock;
  v->keypts = reinterpret_cast<const float*>(st->arena + e.off);
  v->desc = reinterpret_cast<const float*>(st->arena + e.off + align256((size_t)e.k * 12));
  v->k = e.k;
  v->grid = e.grid;
  return TDM_OK;
}

bool store_pin(tdm_store* st, uint64_t key) {
  std::lock_guard<std::mutex> lk(st->mu);
  auto it = st->entries.find(key);
  if (it == st->entries.end()) return false;
  it->second.pins += 1;
  return true;
}

void store_release(tdm_store* st, uint64_t key) {
  std::lock_guard<std::mutex> lk(st->mu);
  auto it = st->entries.find(key);
  if (it != st->entries.end() && it->second.pins > 0) it->second.pins -= 1;
}

// Whether `key` is stored with this keypoint stream and count (a hit).
bool store_has(tdm_store* st, uint64_t key, uint64_t seed, int32_t k, bool count) {
  std::lock_guard<std::mutex> lk(st->mu);
  auto it = st->entries.find(key);
  const bool hit = it != st->entries.end() && !it->second.writing && it->second.seed == seed && it->second.k == k;
  if (count) {
    if (hit) {
      ++st->hits;
      it->second.stamp = ++st->clock;
    } else {
      ++st->misses;
    }
  }
  return hit;
}

size_t store_entry_bytes(int32_t k) { return tdm_store::entry_bytes(k); }

}  // namespace tdm

using namespace tdm;

extern "C" tdm_status tdm_store_create(int64_t budget_bytes, tdm_store** out) {
  TDM_REQUIRE(out && budget_bytes >= 4096, "tdm_store_create: budget must be at least 4096 bytes");
  tdm_store* st = new tdm_store();
  cudaGetDevice(&st->device);
  st->cap = (size_t)budget_bytes & ~(size_t)255;
  cudaError_t e = cudaMalloc(&st->arena, st->cap);
  if (e != cudaSuccess) {
    delete st;
    return cuda_status(e, "tdm_store_create: arena");
  }
  st->free_.emplace(0, st->cap);
  *out = st;
  return TDM_OK;
}

extern "C" tdm_status tdm_store_destroy(tdm_store* st) {
  if (st) {
    cudaSetDevice(st->device);
    cudaDeviceSynchronize();
  }
  delete st;
  return TDM_OK;
}

extern "C" tdm_status tdm_store_describe(tdm_store* st, tdm_pipeline* p, uint64_t key, const float* pts_dev, int32_t n,
                                         uint64_t kp_seed, int32_t k, int32_t* hit, tdm_stream s) {
  TDM_REQUIRE(st && p && pts_dev && n > 0 && k > 0, "tdm_store_describe: bad arguments");
  if (store_has(st, key, kp_seed, k, true)) {
    if (hit) *hit = 1;
    return TDM_OK;
  }
  if (hit) *hit = 0;
  float *kp = nullptr, *desc = nullptr;
  tdm_status r = store_reserve(st, key, kp_seed, k, nullptr, &kp, &desc);
  if (r) return r;
  tdm_grid g{};
  r = tdm_describe_fragment(p, pts_dev, n, kp_seed, k, kp, desc, &g, s);
  tdm_status c = store_commit(st, key, &g, r == TDM_OK, s);
  return r ? r : c;
}

extern "C" tdm_status tdm_store_put(tdm_store* st, uint64_t key, uint64_t kp_seed, const float* keypts_dev,
                                    const float* desc_dev, int32_t k, const tdm_grid* grid, tdm_stream s) {
  TDM_REQUIRE(st && keypts_dev && desc_dev && k > 0, "tdm_store_put: bad arguments");
  float *kp = nullptr, *desc = nullptr;
  tdm_status r = store_reserve(st, key, kp_seed, k, grid, &kp, &desc);
  if (r) return r;
  cudaError_t e = cudaMemcpyAsync(kp, keypts_dev, (size_t)k * 12, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(desc, desc_dev, (size_t)k * 2048, cudaMemcpyDeviceToDevice, s);
  store_commit(st, key, grid, e == cudaSuccess, s);
  return e == cudaSuccess ? TDM_OK : cuda_status(e, "tdm_store_put: copy");
}

extern "C" tdm_status tdm_store_get(tdm_store* st, uint64_t key, const float** keypts_dev, const float** desc_dev,
                                    int32_t* k, tdm_grid* grid) {
  TDM_REQUIRE(st, "tdm_store_get: null store");
  std::lock_guard<std::mutex> lk(st->mu);
  auto it = st->entries.find(key);
  if (it == st->entries.end() || it->second.writing)
    return fail(TDM_ERR_INVALID_ARG, "tdm_store_get: no fragment with that key");
  const Entry& e = it->second;
  if (keypts_dev) *keypts_dev = reinterpret_cast<const float*>(st->arena + e.off);
  if (desc_dev) *desc_dev = reinterpret_cast<const float*>(st->arena + e.off + align256((size_t)e.k * 12));
  if (k) *k = e.k;
  if (grid) *grid = e.grid;
  return TDM_OK;
}

extern "C" tdm_status tdm_store_remove(tdm_store* st, uint64_t key) {
  TDM_REQUIRE(st, "tdm_store_remove: null store");
  std::lock_guard<std::mutex> lk(st->mu);
  auto it = st->entries.find(key);
  if (it == st->entries.end()) return TDM_OK;
  if (it->second.pins) return fail(TDM_ERR_INVALID_ARG, "tdm_store_remove: entry is in use");
  st->drop(it);
  return TDM_OK;
}

extern "C" tdm_status tdm_store_get_stats(tdm_store* st, tdm_store_stats* out) {
  TDM_REQUIRE(st && out, "tdm_store_get_stats: null pointer");
  std::lock_guard<std::mutex> lk(st->mu);
  out->entries = (int64_t)st->entries.size();
  out->bytes_used = (int64_t)st->used;
  out->capacity = (int64_t)st->cap;
  out->hits = st->hits;
  out->misses = st->misses;
  out->evictions = st->evictions;
  return TDM_OK;
}
