// Serving loop for fragment-pair registration requests.
//
// The reference registers pairs one at a time through files and MATLAB
// (evaluation/geometric-registration/register2Fragments.m).  Here a server
// owns `slots` independent execution slots, each with its own CUDA stream,
// pipeline buffers (sized for the largest admitted request) and a clone of
// the net.  The number of slots is bounded by the HBM budget: a slot is only
// created while the running total of slot footprints stays within it.
// Requests go to a FIFO queue; every slot's worker thread takes the next
// request as soon as it is free, so requests that arrive while others run are
// admitted as slots free up and their kernels overlap on the device.  Results
// do not depend on which slot or what else is running: each slot has its own
// buffers and every kernel is deterministic.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "internal.h"
#include "tdm.h"

namespace tdm {
tdm_status fail(tdm_status st, const std::string& msg);
}

namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
  int64_t ticket;
  std::vector<float> a, b;
  uint64_t seed;
  int32_t k;
  double t_submit;
};

struct Done {
  tdm_status st;
  tdm_pair_result res;
  double latency_ms;
  std::string err;
};

struct Slot {
  tdm_net* net = nullptr;
  tdm_pipeline* pipe = nullptr;
  cudaStream_t stream = nullptr;
  std::thread worker;
};

}  // namespace

struct tdm_server {
  tdm_server_config cfg;
  int device = 0;
  std::mutex mu;
  std::condition_variable cv_req, cv_done;
  std::deque<Request> queue;
  std::map<int64_t, Done> done;
  int64_t next_ticket = 1;
  int64_t in_flight = 0;
  bool stop = false;
  std::vector<Slot> slots;
  size_t slot_bytes = 0;

  void work(Slot* slot) {
    cudaSetDevice(device);
    while (true) {
      Request r;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_req.wait(lk, [&] { return stop || !queue.empty(); });
        if (stop && queue.empty()) return;
        r = std::move(queue.front());
        queue.pop_front();
      }
      Done d{};
      d.st = tdm_register_pair_host(slot->pipe, r.a.data(), (int32_t)(r.a.size() / 3), r.b.data(),
                                    (int32_t)(r.b.size() / 3), r.seed, r.k, &d.res, slot->stream);
      if (d.st != TDM_OK) d.err = tdm_last_error();
      d.latency_ms = now_ms() - r.t_submit;
      {
        std::lock_guard<std::mutex> lk(mu);
        done[r.ticket] = d;
        --in_flight;
      }
      cv_done.notify_all();
    }
  }
};

// Device bytes one slot holds: pipeline buffers for the largest request plus
// the net's activation workspace for two fragments' patches.
static size_t slot_footprint(const tdm_server_config& c, const tdm_net* net) {
  const size_t K = (size_t)c.pipeline.max_keypoints, N = (size_t)c.pipeline.max_points,
               V = (size_t)c.pipeline.max_voxels;
  size_t bytes = 2 * (N * 12 + K * 28 + V * 4) + tdm::tdf_workspace_cap((int64_t)V) + 2 * K * 27000 * 4 +
                 2 * K * 512 * 4;
  bytes += tdm_mnn_workspace_bytes((int)K, (int)K, 512) + K * 40;
  bytes += tdm_ransac_workspace_bytes((int)K, c.pipeline.ransac.iterations);
  bytes += tdm_net_workspace_bytes(net, (int32_t)(2 * K));
  bytes += (size_t)64 << 20;  // weights and small buffers
  return bytes;
}

extern "C" tdm_status tdm_server_create(const tdm_server_config* cfg, const tdm_net* net, tdm_server** out) {
  if (!cfg || !net || !out || cfg->slots <= 0 || cfg->hbm_budget_bytes <= 0)
    return tdm::fail(TDM_ERR_INVALID_ARG, "tdm_server_create: bad arguments");
  tdm_server* s = new tdm_server();
  s->cfg = *cfg;
  cudaGetDevice(&s->device);
  s->slot_bytes = slot_footprint(*cfg, net);
  int n = cfg->slots;
  if ((int64_t)(s->slot_bytes * (size_t)n) > cfg->hbm_budget_bytes) n = (int)(cfg->hbm_budget_bytes / s->slot_bytes);
  if (n < 1) {
    delete s;
    return tdm::fail(TDM_ERR_OOM, "tdm_server_create: HBM budget is smaller than one slot");
  }
  s->slots.resize(n);
  tdm_status st = TDM_OK;
  for (int i = 0; i < n && st == TDM_OK; ++i) {
    Slot& sl = s->slots[i];
    st = tdm_net_clone(net, &sl.net);
    if (st == TDM_OK) st = tdm_pipeline_create(&cfg->pipeline, sl.net, &sl.pipe);
    if (st == TDM_OK && cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess)
      st = TDM_ERR_DEVICE;
  }
  if (st != TDM_OK) {
    for (auto& sl : s->slots) {
      if (sl.pipe) tdm_pipeline_destroy(sl.pipe);
      if (sl.net) tdm_net_destroy(sl.net);
      if (sl.stream) cudaStreamDestroy(sl.stream);
    }
    delete s;
    return st;
  }
  for (auto& sl : s->slots) sl.worker = std::thread([s, &sl] { s->work(&sl); });
  *out = s;
  return TDM_OK;
}

extern "C" int32_t tdm_server_slots(const tdm_server* s) { return s ? (int32_t)s->slots.size() : 0; }

extern "C" tdm_status tdm_server_submit(tdm_server* s, const float* a, int32_t na, const float* b, int32_t nb,
                                        uint64_t seed, int32_t k, int64_t* ticket) {
  if (!s || !a || !b || !ticket || na <= 0 || nb <= 0 || k <= 0)
    return tdm::fail(TDM_ERR_INVALID_ARG, "tdm_server_submit: bad arguments");
  if (na > s->cfg.pipeline.max_points || nb > s->cfg.pipeline.max_points || k > s->cfg.pipeline.max_keypoints)
    return tdm::fail(TDM_ERR_INVALID_ARG, "tdm_server_submit: request exceeds the slot limits");
  Request r;
  r.a.assign(a, a + (size_t)na * 3);
  r.b.assign(b, b + (size_t)nb * 3);
  r.seed = seed;
  r.k = k;
  r.t_submit = now_ms();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return tdm::fail(TDM_ERR_CANCELLED, "tdm_server_submit: server is stopping");
    r.ticket = s->next_ticket++;
    *ticket = r.ticket;
    ++s->in_flight;
    s->queue.push_back(std::move(r));
  }
  s->cv_req.notify_one();
  return TDM_OK;
}

extern "C" tdm_status tdm_server_wait(tdm_server* s, int64_t ticket, tdm_pair_result* res, double* latency_ms) {
  if (!s || !res) return tdm::fail(TDM_ERR_INVALID_ARG, "tdm_server_wait: bad arguments");
  std::unique_lock<std::mutex> lk(s->mu);
  if (ticket <= 0 || ticket >= s->next_ticket) return tdm::fail(TDM_ERR_INVALID_ARG, "tdm_server_wait: unknown ticket");
  s->cv_done.wait(lk, [&] { return s->done.count(ticket) > 0; });
  Done d = s->done[ticket];
  s->done.erase(ticket);
  *res = d.res;
  if (latency_ms) *latency_ms = d.latency_ms;
  if (d.st != TDM_OK) tdm::fail(d.st, d.err);
  return d.st;
}

extern "C" tdm_status tdm_server_destroy(tdm_server* s) {
  if (!s) return TDM_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_req.notify_all();
  for (auto& sl : s->slots)
    if (sl.worker.joinable()) sl.worker.join();
  for (auto& sl : s->slots) {
    tdm_pipeline_destroy(sl.pipe);
    tdm_net_destroy(sl.net);
    cudaStreamDestroy(sl.stream);
  }
  delete s;
  return TDM_OK;
}
