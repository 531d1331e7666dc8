// Serving loop for fragment-pair registration requests, with continuous
// batching over the batched description kernels and a device-resident
// fragment store.
//
// The reference registers pairs one at a time through files and MATLAB
// (evaluation/geometric-registration/register2Fragments.m), describing each
// fragment once beforehand (getKeyptsAndDesc.m:34-43).  Here requests arrive
// at any time and go to a FIFO queue.  Two threads work on the GPU:
//
//   describer  takes the queued requests that fit the server's device budget
//              (a wave), describes every fragment of the wave that is not in
//              the store with ONE tdm_describe_batch call -- persistent TDF,
//              keypoint and gather kernels over all of the wave's fragments,
//              the net over all of their patches, so patches of different
//              requests share net launches -- and puts keypoints and
//              descriptors into the store;
//   matcher    registers each request of a finished wave from the store
//              (mutual NN, RANSAC, refit) on its own stream.
//
// While the matcher works on wave i the describer already runs wave i + 1, so
// the two requests' kernels overlap on the device (measured: the server
// reports the time both stages were busy at once).  Admission is by each
// request's own footprint: its points, its grids' voxels (from its bounding
// box, computed at submit) and its keypoints count against the wave's device
// capacity, which the HBM budget fixes; a request that cannot fit alone is
// refused at submit, one that does not fit the current wave waits for the
// next.  Fragments submitted with a key stay in the store (least recently used
// eviction), so later requests naming them skip description; anonymous
// fragments are dropped after their pair is registered.  Results do not
// depend on what else is in the wave: the batched kernels give every fragment
// the bits tdm_describe_fragment gives it alone, and matching is per pair.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "internal.h"
#include "tdm.h"

namespace tdm {
tdm_status fail(tdm_status st, const std::string& msg);
tdm_status cuda_status(cudaError_t e, const char* what);
}  // namespace tdm

using namespace tdm;

namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// Store keys of anonymous fragments: top bit set, never a caller key (callers
// use keys below 2^63).
constexpr uint64_t kAnonBit = 1ull << 63;

struct Frag {
  uint64_t key = 0;  // store key (caller's, or an anonymous one)
  bool anon = false;
  std::vector<float> pts;
  uint64_t seed = 0;
  int32_t k = 0;
  int64_t voxels = 0;  // arena voxels its grid takes in the batch
};

struct Request {
  int64_t ticket = 0;
  Frag f[2];
  double t_submit = 0;
  bool cancelled = false;
};

struct Done {
  tdm_status st = TDM_OK;
  tdm_pair_result res{};
  double latency_ms = 0;
  std::string err;
};

// Voxels the batched form's arena gives a grid (x rows padded to 4, then a
// multiple of 256), from host points with the grid arithmetic of the device.
int64_t arena_voxels(const float* pts, int32_t n, const tdm_pipeline_config& c) {
  tdm_grid g;
  if (tdm_grid_from_points_host(pts, n, c.voxel_size, c.voxel_size * c.trunc_voxels, c.pad, &g) != TDM_OK) return -1;
  const int64_t pv = (((int64_t)g.dim[0] + 3) & ~(int64_t)3) * g.dim[1] * g.dim[2];  // x rows padded to 4
  return (pv + 255) / 256 * 256;
}

}  // namespace

struct tdm_server {
  tdm_server_config cfg;
  int device = 0;
  // wave capacity (device buffers of the batch are sized for it)
  int32_t cap_fragments = 0;
  int64_t cap_points = 0, cap_keypoints = 0, cap_voxels = 0;
  size_t device_bytes = 0;
  // GPU objects
  tdm_net* net = nullptr;
  tdm_batch* batch = nullptr;
  tdm_store* store = nullptr;
  tdm_pipeline* match = nullptr;
  cudaStream_t sd = nullptr, sm = nullptr;
  float* d_pts = nullptr;
  float* d_kp = nullptr;
  float* d_desc = nullptr;
  float* h_pts = nullptr;  // pinned staging of a wave's points
  // queues
  std::mutex mu;
  std::condition_variable cv_req, cv_wave, cv_done;
  std::deque<Request> queue;
  std::deque<std::vector<Request>> waves;
  std::map<int64_t, Done> done;
  std::set<int64_t> in_flight;        // taken into a wave, not finished
  std::set<int64_t> cancel_in_flight;  // cancelled while in flight
  int64_t next_ticket = 1;
  uint64_t next_anon = 1;
  bool stop = false;
  std::thread describer, matcher;
  // statistics
  tdm_server_stats stats{};
  int busy[2] = {0, 0};
  double t_last = 0;

  // Busy-time accounting (under mu): stage 0 = describe, 1 = match.
  void account(int stage, int on) {
    const double t = now_ms();
    if (t_last > 0) {
      const double dt = t - t_last;
      if (busy[0]) stats.describe_ms += dt;
      if (busy[1]) stats.match_ms += dt;
      if (busy[0] && busy[1]) stats.overlap_ms += dt;
    }
    t_last = t;
    busy[stage] = on;
  }

  void finish(Request& r, const Done& d) {
    std::lock_guard<std::mutex> lk(mu);
    in_flight.erase(r.ticket);
    if (cancel_in_flight.erase(r.ticket)) {
      Done c;
      c.st = TDM_ERR_CANCELLED;
      c.err = "tdm_server_wait: request was cancelled";
      c.latency_ms = d.latency_ms;
      done[r.ticket] = c;
      ++stats.requests_cancelled;
    } else {
      done[r.ticket] = d;
      ++stats.requests_done;
    }
    cv_done.notify_all();
  }

  void run_describer();
  void run_matcher();
};

void tdm_server::run_describer() {
  cudaSetDevice(device);
  while (true) {
    std::vector<Request> wave;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_req.wait(lk, [&] { return stop || !queue.empty(); });
      if (queue.empty()) break;  // stopping with nothing queued
      // admission by footprint: FIFO until the next request does not fit
      int32_t nf = 0;
      int64_t np = 0, nk = 0, nv = 0;
      std::set<uint64_t> planned;
      while (!queue.empty() && (int32_t)wave.size() < cfg.slots) {
        Request& r = queue.front();
        bool missing = false;  // named by key without points, and no longer stored
        for (const Frag& fr : r.f)
          missing |= fr.pts.empty() && !planned.count(fr.key) && !store_has(store, fr.key, fr.seed, fr.k, false);
        if (missing) {
          Done d;
          d.st = TDM_ERR_INVALID_ARG;
          d.err = "tdm_server_wait: a fragment named without points left the store before the request started";
          d.latency_ms = now_ms() - r.t_submit;
          done[r.ticket] = d;
          ++stats.requests_done;
          queue.pop_front();
          cv_done.notify_all();
          continue;
        }
        int32_t f2 = 0;
        int64_t p2 = 0, k2 = 0, v2 = 0;
        for (const Frag& fr : r.f) {
          if (planned.count(fr.key) || (!fr.anon && store_has(store, fr.key, fr.seed, fr.k, false))) continue;
          f2 += 1;
          p2 += (int64_t)fr.pts.size() / 3;
          k2 += fr.k;
          v2 += fr.voxels;
        }
        if (!wave.empty() && (nf + f2 > cap_fragments || np + p2 > cap_points || nk + k2 > cap_keypoints ||
                              nv + v2 > cap_voxels))
          break;
        for (const Frag& fr : r.f) planned.insert(fr.key);
        nf += f2;
        np += p2;
        nk += k2;
        nv += v2;
        in_flight.insert(r.ticket);
        wave.push_back(std::move(r));
        queue.pop_front();
      }
      account(0, 1);
    }
    // fragments to describe: not stored (or stored with other keypoints).
    // Every fragment the wave names is pinned, once per occurrence, until the
    // matcher has registered its pair: stored ones now (before this wave's
    // own entries can evict them), described ones after they are stored.
    std::vector<Frag*> todo;
    std::map<uint64_t, int> uses;
    for (Request& r : wave)
      for (Frag& fr : r.f) uses[fr.key] += 1;
    std::map<uint64_t, Frag*> with_points;  // per key, an occurrence that carries the points
    for (Request& r : wave)
      for (Frag& fr : r.f)
        if (!fr.pts.empty() && !with_points.count(fr.key)) with_points[fr.key] = &fr;
    std::set<uint64_t> seen;
    for (Request& r : wave)
      for (Frag& fr : r.f) {
        if (seen.count(fr.key)) continue;
        seen.insert(fr.key);
        if (!fr.anon && store_has(store, fr.key, fr.seed, fr.k, true)) {
          for (int u = 0; u < uses[fr.key]; ++u) store_pin(store, fr.key);
          continue;
        }
        todo.push_back(with_points.count(fr.key) ? with_points[fr.key] : &fr);
      }
    tdm_status st = TDM_OK;
    std::string err;
    if (!todo.empty()) {
      const int F = (int)todo.size();
      std::vector<int64_t> off(F + 1, 0);
      std::vector<float> vs(F, cfg.pipeline.voxel_size);
      std::vector<int32_t> ks(F);
      std::vector<uint64_t> seeds(F);
      for (int f = 0; f < F; ++f) {
        const Frag& fr = *todo[f];
        std::memcpy(h_pts + off[f] * 3, fr.pts.data(), fr.pts.size() * sizeof(float));
        off[f + 1] = off[f] + (int64_t)fr.pts.size() / 3;
        ks[f] = fr.k;
        seeds[f] = fr.seed;
      }
      std::vector<tdm_grid> grids(F);
      cudaError_t e = cudaMemcpyAsync(d_pts, h_pts, (size_t)off[F] * 12, cudaMemcpyHostToDevice, sd);
      if (e != cudaSuccess) st = cuda_status(e, "server: points upload");
      if (!st)
        st = tdm_describe_batch(batch, d_pts, F, off.data(), vs.data(), ks.data(), seeds.data(), d_kp, d_desc,
                                grids.data(), sd);
      int64_t k0 = 0;
      for (int f = 0; f < F && !st; ++f) {
        st = tdm_store_put(store, todo[f]->key, todo[f]->seed, d_kp + k0 * 3, d_desc + k0 * 512, todo[f]->k,
                           &grids[f], sd);
        if (!st)
          for (int u = 0; u < uses[todo[f]->key]; ++u) store_pin(store, todo[f]->key);
        k0 += todo[f]->k;
      }
      if (st) err = tdm_last_error();
      std::lock_guard<std::mutex> lk(mu);
      stats.fragments_described += F;
    }
    for (Request& r : wave) r.f[0].pts.clear(), r.f[1].pts.clear();
    {
      std::lock_guard<std::mutex> lk(mu);
      account(0, 0);
      ++stats.waves;
      stats.max_wave_requests = std::max<int64_t>(stats.max_wave_requests, (int64_t)wave.size());
    }
    if (st) {  // the whole wave fails with the description's status
      for (Request& r : wave) {
        Done d;
        d.st = st;
        d.err = err;
        d.latency_ms = now_ms() - r.t_submit;
        for (Frag& fr : r.f) {
          store_release(store, fr.key);
          if (fr.anon) tdm_store_remove(store, fr.key);
        }
        finish(r, d);
      }
      continue;
    }
    {
      std::lock_guard<std::mutex> lk(mu);
      waves.push_back(std::move(wave));
    }
    cv_wave.notify_one();
  }
  std::lock_guard<std::mutex> lk(mu);
  waves.push_back({});  // end marker for the matcher
  cv_wave.notify_one();
}

void tdm_server::run_matcher() {
  cudaSetDevice(device);
  while (true) {
    std::vector<Request> wave;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_wave.wait(lk, [&] { return !waves.empty(); });
      wave = std::move(waves.front());
      waves.pop_front();
      if (wave.empty()) return;
      account(1, 1);
    }
    for (Request& r : wave) {
      Done d;
      bool skip;
      {
        std::lock_guard<std::mutex> lk(mu);
        skip = cancel_in_flight.count(r.ticket) > 0;
      }
      if (!skip) {
        d.st = tdm_register_stored(match, store, r.f[0].key, r.f[1].key, &d.res, sm);
        if (d.st != TDM_OK) d.err = tdm_last_error();
      }
      for (Frag& fr : r.f) {
        store_release(store, fr.key);  // the wave's pin
        if (fr.anon) tdm_store_remove(store, fr.key);
      }
      d.latency_ms = now_ms() - r.t_submit;
      finish(r, d);
    }
    std::lock_guard<std::mutex> lk(mu);
    account(1, 0);
  }
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" tdm_status tdm_server_create(const tdm_server_config* cfg, const tdm_net* net, tdm_server** out) {
  if (!cfg || !net || !out || cfg->slots <= 0 || cfg->hbm_budget_bytes <= 0 || cfg->pipeline.max_points <= 0 ||
      cfg->pipeline.max_keypoints <= 0 || cfg->pipeline.max_voxels <= 0)
    return fail(TDM_ERR_INVALID_ARG, "tdm_server_create: bad arguments");
  tdm_server* s = new tdm_server();
  s->cfg = *cfg;
  cudaGetDevice(&s->device);
  const tdm_pipeline_config& pc = cfg->pipeline;
  // Wave capacity: `slots` requests of the largest admitted size, shrunk to
  // the budget left after the net's activations, the store and matching.
  const int64_t per_req_pts = 2 * (int64_t)pc.max_points, per_req_kp = 2 * (int64_t)pc.max_keypoints;
  const int64_t per_req_vox = 2 * (((int64_t)pc.max_voxels * 34 / 31 + 255) / 256 * 256);  // pitch slack
  // the store holds at least one wave's entries (every fragment of a wave is
  // pinned until its pair is registered)
  const int64_t per_req_store = 2 * (int64_t)store_entry_bytes(pc.max_keypoints);
  int64_t store_bytes = cfg->store_bytes > 0 ? cfg->store_bytes
                                             : std::max<int64_t>(cfg->hbm_budget_bytes / 10, 4 * per_req_store);
  if (store_bytes < per_req_store) {
    delete s;
    return fail(TDM_ERR_INVALID_ARG, "tdm_server_create: store_bytes cannot hold one request's two fragments");
  }
  const size_t fixed = tdm_net_workspace_bytes(net, 2048) + (size_t)store_bytes + pipeline_match_bytes(&pc) +
                       ((size_t)64 << 20);
  if ((int64_t)fixed >= cfg->hbm_budget_bytes) {
    delete s;
    return fail(TDM_ERR_OOM, "tdm_server_create: HBM budget is smaller than the net, store and matching buffers");
  }
  const int64_t left = cfg->hbm_budget_bytes - (int64_t)fixed;
  // per wave slot: points (12 B in, 12 B staging on device), voxels (6 B:
  // TDF + occupancy/in-plane), keypoints (12 B grid + 12 B keypts + 2 KB desc)
  const int64_t per_req = per_req_pts * 24 + per_req_vox * 6 + per_req_kp * (24 + 2048);
  int32_t n = (int32_t)std::min<int64_t>(cfg->slots, left / std::max<int64_t>(per_req, 1));
  n = (int32_t)std::min<int64_t>(n, store_bytes / per_req_store);
  if (n < 1) {
    delete s;
    return fail(TDM_ERR_OOM, "tdm_server_create: HBM budget is smaller than one request of the configured size");
  }
  n = std::min(n, 512);  // two fragments per request, 1024 per batch
  s->cfg.slots = n;
  s->cap_fragments = 2 * n;
  s->cap_points = per_req_pts * n;
  s->cap_keypoints = per_req_kp * n;
  s->cap_voxels = per_req_vox * n;
  tdm_status st = tdm_net_clone(net, &s->net);
  if (!st) {
    tdm_batch_config bc{};
    bc.max_fragments = s->cap_fragments;
    bc.max_points = s->cap_points;
    bc.max_keypoints = s->cap_keypoints;
    bc.max_voxels = s->cap_voxels;
    bc.trunc_voxels = pc.trunc_voxels;
    bc.pad = pc.pad;
    bc.use_graph = 0;  // wave shapes change from call to call
    st = tdm_batch_create(&bc, s->net, &s->batch);
  }
  if (!st) st = tdm_store_create(store_bytes, &s->store);
  if (!st) st = pipeline_create_match_only(&pc, &s->match);
  if (!st && (cudaStreamCreateWithFlags(&s->sd, cudaStreamNonBlocking) != cudaSuccess ||
              cudaStreamCreateWithFlags(&s->sm, cudaStreamNonBlocking) != cudaSuccess))
    st = fail(TDM_ERR_DEVICE, "tdm_server_create: streams");
  if (!st) {
    cudaError_t e = cudaMalloc(&s->d_pts, (size_t)s->cap_points * 12);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_kp, (size_t)s->cap_keypoints * 12);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_desc, (size_t)s->cap_keypoints * 2048);
    if (e == cudaSuccess) e = cudaMallocHost(&s->h_pts, (size_t)s->cap_points * 12);
    if (e != cudaSuccess) st = cuda_status(e, "tdm_server_create: buffers");
  }
  if (st) {
    tdm_server_destroy(s);
    return st;
  }
  s->device_bytes = tdm_batch_device_bytes(s->batch) + tdm_net_workspace_bytes(s->net, 2048) + (size_t)store_bytes +
                    pipeline_match_bytes(&pc) + (size_t)s->cap_points * 12 + (size_t)s->cap_keypoints * 2060;
  s->stats.device_bytes = (int64_t)s->device_bytes;
  s->describer = std::thread([s] { s->run_describer(); });
  s->matcher = std::thread([s] { s->run_matcher(); });
  *out = s;
  return TDM_OK;
}

extern "C" int32_t tdm_server_slots(const tdm_server* s) { return s ? s->cfg.slots : 0; }

extern "C" tdm_status tdm_server_submit_pair(tdm_server* s, const tdm_fragment* a, const tdm_fragment* b,
                                             int64_t* ticket) {
  if (!s || !a || !b || !ticket) return fail(TDM_ERR_INVALID_ARG, "tdm_server_submit_pair: null pointer");
  Request r;
  const tdm_fragment* in[2] = {a, b};
  int64_t p2 = 0, k2 = 0, v2 = 0;
  for (int f = 0; f < 2; ++f) {
    const tdm_fragment& x = *in[f];
    Frag& fr = r.f[f];
    if (x.key & kAnonBit) return fail(TDM_ERR_INVALID_ARG, "tdm_server_submit_pair: keys must be below 2^63");
    if (x.k <= 0 || x.k > s->cfg.pipeline.max_keypoints)
      return fail(TDM_ERR_INVALID_ARG, "tdm_server_submit_pair: keypoints outside 1..max_keypoints");
    fr.k = x.k;
    fr.seed = x.seed;
    const bool stored = x.key != 0 && store_has(s->store, x.key, x.seed, x.k, false);
    if (!x.pts || x.n <= 0) {
      if (!stored)
        return fail(TDM_ERR_INVALID_ARG, "tdm_server_submit_pair: fragment has no points and is not in the store");
    } else {
      if (x.n > s->cfg.pipeline.max_points)
        return fail(TDM_ERR_INVALID_ARG, "tdm_server_submit_pair: fragment has more points than max_points");
      fr.voxels = arena_voxels(x.pts, x.n, s->cfg.pipeline);
      if (fr.voxels < 0 || fr.voxels > s->cap_voxels)
        return fail(TDM_ERR_INVALID_ARG, "tdm_server_submit_pair: fragment grid is invalid or exceeds the capacity");
      fr.pts.assign(x.pts, x.pts + (size_t)x.n * 3);
      p2 += x.n;
      k2 += x.k;
      v2 += fr.voxels;
    }
    fr.key = x.key;
  }
  if (p2 > s->cap_points || k2 > s->cap_keypoints || v2 > s->cap_voxels)
    return fail(TDM_ERR_INVALID_ARG, "tdm_server_submit_pair: request exceeds the server's device capacity");
  r.t_submit = now_ms();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return fail(TDM_ERR_CANCELLED, "tdm_server_submit_pair: server is stopping");
    for (Frag& fr : r.f)
      if (fr.key == 0) {
        fr.key = kAnonBit | s->next_anon++;
        fr.anon = true;
      }
    r.ticket = s->next_ticket++;
    *ticket = r.ticket;
    s->queue.push_back(std::move(r));
  }
  s->cv_req.notify_one();
  return TDM_OK;
}

extern "C" tdm_status tdm_server_submit(tdm_server* s, const float* a, int32_t na, const float* b, int32_t nb,
                                        uint64_t seed, int32_t k, int64_t* ticket) {
  if (!s || !a || !b || !ticket || na <= 0 || nb <= 0 || k <= 0)
    return fail(TDM_ERR_INVALID_ARG, "tdm_server_submit: bad arguments");
  // tdm_register_pair's streams: fragment A from `seed`, B from `seed + 1`
  tdm_fragment fa{0, a, na, seed, k}, fb{0, b, nb, seed + 1, k};
  return tdm_server_submit_pair(s, &fa, &fb, ticket);
}

extern "C" tdm_status tdm_server_cancel(tdm_server* s, int64_t ticket) {
  if (!s) return fail(TDM_ERR_INVALID_ARG, "tdm_server_cancel: null server");
  std::lock_guard<std::mutex> lk(s->mu);
  if (ticket <= 0 || ticket >= s->next_ticket) return fail(TDM_ERR_INVALID_ARG, "tdm_server_cancel: unknown ticket");
  for (auto it = s->queue.begin(); it != s->queue.end(); ++it)
    if (it->ticket == ticket) {
      Done d;
      d.st = TDM_ERR_CANCELLED;
      d.err = "tdm_server_wait: request was cancelled before it started";
      d.latency_ms = now_ms() - it->t_submit;
      s->done[ticket] = d;
      ++s->stats.requests_cancelled;
      s->queue.erase(it);
      s->cv_done.notify_all();
      return TDM_OK;
    }
  if (s->in_flight.count(ticket)) {
    s->cancel_in_flight.insert(ticket);  // its GPU work finishes; the result is dropped
    return TDM_OK;
  }
  return fail(TDM_ERR_INVALID_ARG, "tdm_server_cancel: request already finished");
}

extern "C" tdm_status tdm_server_wait(tdm_server* s, int64_t ticket, int64_t timeout_ms, tdm_pair_result* res,
                                      double* latency_ms) {
  if (!s || !res) return fail(TDM_ERR_INVALID_ARG, "tdm_server_wait: bad arguments");
  std::unique_lock<std::mutex> lk(s->mu);
  if (ticket <= 0 || ticket >= s->next_ticket) return fail(TDM_ERR_INVALID_ARG, "tdm_server_wait: unknown ticket");
  auto ready = [&] { return s->done.count(ticket) > 0; };
  if (timeout_ms < 0) {
    s->cv_done.wait(lk, ready);
  } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
    return fail(TDM_ERR_TIMEOUT, "tdm_server_wait: result not ready within the timeout (the ticket stays valid)");
  }
  Done d = s->done[ticket];
  s->done.erase(ticket);
  *res = d.res;
  if (latency_ms) *latency_ms = d.latency_ms;
  if (d.st != TDM_OK) fail(d.st, d.err);
  return d.st;
}

extern "C" tdm_status tdm_server_get_stats(tdm_server* s, tdm_server_stats* out) {
  if (!s || !out) return fail(TDM_ERR_INVALID_ARG, "tdm_server_get_stats: null pointer");
  std::lock_guard<std::mutex> lk(s->mu);
  s->account(0, s->busy[0]);  // bring the busy times up to now
  *out = s->stats;
  tdm_store_stats ss{};
  if (tdm_store_get_stats(s->store, &ss) == TDM_OK) {
    out->store_hits = ss.hits;
    out->store_entries = ss.entries;
  }
  return TDM_OK;
}

extern "C" tdm_status tdm_server_destroy(tdm_server* s) {
  if (!s) return TDM_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_req.notify_all();
  if (s->describer.joinable()) s->describer.join();
  if (s->matcher.joinable()) s->matcher.join();
  cudaSetDevice(s->device);
  if (s->sd) cudaStreamSynchronize(s->sd);
  if (s->sm) cudaStreamSynchronize(s->sm);
  if (s->match) tdm_pipeline_destroy(s->match);
  if (s->batch) tdm_batch_destroy(s->batch);
  if (s->store) tdm_store_destroy(s->store);
  if (s->net) tdm_net_destroy(s->net);
  if (s->sd) cudaStreamDestroy(s->sd);
  if (s->sm) cudaStreamDestroy(s->sm);
  cudaFree(s->d_pts);
  cudaFree(s->d_kp);
  cudaFree(s->d_desc);
  if (s->h_pts) cudaFreeHost(s->h_pts);
  delete s;
  return TDM_OK;
}
