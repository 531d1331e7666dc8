// Whole registration path for a fragment pair, device resident:
//   points -> grid + TDF -> keypoints -> 30^3 patches -> net -> descriptors
//   -> mutual NN -> RANSAC + Kabsch refit -> 4x4 Rt
// This is core/demo.cu's main (per fragment) followed by core/demo.m:49-64
// (matching and ransacfitRt), without the file round trip between them.
// Both fragments' patches go through the net as one batch.
#include <vector>

#include "common.cuh"
#include "internal.h"

struct tdm_pipeline {
  tdm_pipeline_config cfg;
  tdm_net* net = nullptr;
  float* pts[2] = {};
  int32_t* idx[2] = {};
  float* kp[2] = {};
  int32_t* kpg[2] = {};
  float* tdf[2] = {};
  uint8_t* occ = nullptr;
  void* grid_ws = nullptr;
  float* patches = nullptr;
  float* desc = nullptr;
  void* mnn_ws = nullptr;
  size_t mnn_bytes = 0;
  int32_t *nn_ab = nullptr, *nn_ba = nullptr, *pairs = nullptr, *npairs = nullptr;
  float *x = nullptr, *y = nullptr;
  void* rws = nullptr;
  size_t rws_bytes = 0;
  double* rt = nullptr;
  int32_t* inliers = nullptr;
  int32_t* info = nullptr;
  void* host_stage = nullptr;  // pinned: rt (12 doubles), info (4), npairs (1)
  std::vector<void*> allocs;

  ~tdm_pipeline() {
    for (void* p : allocs) cudaFree(p);
    if (host_stage) cudaFreeHost(host_stage);
  }
  template <typename T>
  tdm_status alloc(T** p, size_t bytes) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, bytes < 16 ? 16 : bytes);
    if (e != cudaSuccess) return tdm::cuda_status(e, "pipeline buffer");
    allocs.push_back(q);
    *p = static_cast<T*>(q);
    return TDM_OK;
  }
};

using namespace tdm;

namespace {

// Matching and RANSAC buffers for fragments of up to K keypoints.
tdm_status alloc_match(tdm_pipeline* p, size_t K) {
  tdm_status st = TDM_OK;
  p->mnn_bytes = tdm_mnn_workspace_bytes((int)K, (int)K, 512);
  if (!st) st = p->alloc(&p->mnn_ws, p->mnn_bytes);
  if (!st) st = p->alloc(&p->nn_ab, K * 4);
  if (!st) st = p->alloc(&p->nn_ba, K * 4);
  if (!st) st = p->alloc(&p->pairs, K * 8);
  if (!st) st = p->alloc(&p->npairs, 4);
  if (!st) st = p->alloc(&p->x, K * 12);
  if (!st) st = p->alloc(&p->y, K * 12);
  p->rws_bytes = tdm_ransac_workspace_bytes((int)K, p->cfg.ransac.iterations);
  if (!st) st = p->alloc(&p->rws, p->rws_bytes);
  if (!st) st = p->alloc(&p->rt, 12 * 8);
  if (!st) st = p->alloc(&p->inliers, K * 4);
  if (!st) st = p->alloc(&p->info, 16);
  if (!st) {
    cudaError_t e = cudaMallocHost(&p->host_stage, 256);
    if (e != cudaSuccess) st = cuda_status(e, "pinned staging");
  }
  return st;
}

tdm_status check_config(const tdm_pipeline_config* cfg) {
  TDM_REQUIRE(cfg->voxel_size > 0 && cfg->trunc_voxels > 0 && cfg->pad >= 0, "tdm_pipeline_create: bad grid");
  TDM_REQUIRE(cfg->max_points > 0 && cfg->max_keypoints > 0 && cfg->max_voxels > 0, "tdm_pipeline_create: bad sizes");
  TDM_REQUIRE(cfg->ransac.iterations >= 0 && cfg->ransac.threshold > 0, "tdm_pipeline_create: bad RANSAC params");
  return TDM_OK;
}

}  // namespace

namespace tdm {

size_t pipeline_match_bytes(const tdm_pipeline_config* cfg) {
  const size_t K = (size_t)cfg->max_keypoints;
  return tdm_mnn_workspace_bytes((int)K, (int)K, 512) + K * 52 + 256 +
         tdm_ransac_workspace_bytes((int)K, cfg->ransac.iterations);
}

tdm_status pipeline_create_match_only(const tdm_pipeline_config* cfg, tdm_pipeline** out) {
  TDM_REQUIRE(cfg && out, "pipeline: null pointer");
  tdm_status st = check_config(cfg);
  if (st) return st;
  tdm_pipeline* p = new tdm_pipeline();
  p->cfg = *cfg;
  st = alloc_match(p, (size_t)cfg->max_keypoints);
  if (st) {
    delete p;
    return st;
  }
  *out = p;
  return TDM_OK;
}

}  // namespace tdm

extern "C" tdm_status tdm_pipeline_create(const tdm_pipeline_config* cfg, tdm_net* net, tdm_pipeline** out) {
  TDM_REQUIRE(cfg && net && out, "tdm_pipeline_create: null pointer");
  tdm_status st = check_config(cfg);
  if (st) return st;
  tdm_pipeline* p = new tdm_pipeline();
  p->cfg = *cfg;
  p->net = net;
  const size_t K = (size_t)cfg->max_keypoints, N = (size_t)cfg->max_points, V = (size_t)cfg->max_voxels;
  for (int f = 0; f < 2 && st == TDM_OK; ++f) {
    st = p->alloc(&p->pts[f], N * 12);
    if (!st) st = p->alloc(&p->idx[f], K * 4);
    if (!st) st = p->alloc(&p->kp[f], K * 12);
    if (!st) st = p->alloc(&p->kpg[f], K * 12);
    if (!st) st = p->alloc(&p->tdf[f], V * 4);
  }
  if (!st) st = p->alloc(&p->occ, tdf_workspace_cap(V));  // occupancy + in-plane distances
  if (!st) st = p->alloc(&p->grid_ws, tdm_grid_workspace_bytes());
  if (!st) st = p->alloc(&p->patches, 2 * K * 27000 * 4);
  if (!st) st = p->alloc(&p->desc, 2 * K * 512 * 4);
  if (!st) st = alloc_match(p, K);
  if (st) {
    delete p;
    return st;
  }
  *out = p;
  return TDM_OK;
}

extern "C" tdm_status tdm_pipeline_destroy(tdm_pipeline* p) {
  delete p;
  return TDM_OK;
}

namespace {

// Grid, TDF, keypoints and patches of one fragment into slot f.
tdm_status fragment_front(tdm_pipeline* p, int f, const float* pts, int32_t n, const tdm_grid& g, uint64_t seed,
                          int32_t k, float* keypts, float* patches, cudaStream_t s) {
  TDM_REQUIRE((int64_t)g.dim[0] * g.dim[1] * g.dim[2] <= p->cfg.max_voxels,
              "fragment grid exceeds the pipeline's max_voxels");
  tdm_status st = tdm_tdf(pts, n, &g, TDM_TDF_EXACT, p->tdf[f], p->occ, tdf_workspace_cap(p->cfg.max_voxels), s);
  if (st) return st;
  st = tdm_keypoint_indices(seed, n, k, p->idx[f], s);
  if (st) return st;
  st = tdm_keypoints(pts, n, p->idx[f], k, &g, keypts, p->kpg[f], s);
  if (st) return st;
  return tdm_gather(p->tdf[f], &g, p->kpg[f], k, patches, s);
}

// core/demo.m:49-64 on two described fragments: mutual NN of the
// descriptors, the matched keypoints, RANSAC + refit; result copied to host.
tdm_status match_back(tdm_pipeline* p, const float* desc_a, const float* kp_a, int32_t ka, const float* desc_b,
                      const float* kp_b, int32_t kb, const tdm_grid g[2], tdm_pair_result* r, cudaStream_t s) {
  const int32_t m_max = ka < kb ? ka : kb;
  tdm_status st = tdm_match_mnn(desc_a, ka, desc_b, kb, 512, p->cfg.match_precision, p->nn_ab, p->nn_ba, p->pairs,
                                p->npairs, p->mnn_ws, p->mnn_bytes, s);
  if (st) return st;
  st = tdm_pairs_to_points(kp_a, kp_b, p->pairs, p->npairs, m_max, p->x, p->y, s);
  if (st) return st;
  st = tdm_ransac(p->x, p->y, p->npairs, m_max, &p->cfg.ransac, p->rt, p->inliers, p->info, p->rws, p->rws_bytes, s);
  if (st) return st;
  double* h_rt = static_cast<double*>(p->host_stage);
  int32_t* h_info = reinterpret_cast<int32_t*>(h_rt + 12);
  TDM_CHECK_CUDA(cudaMemcpyAsync(h_rt, p->rt, 12 * 8, cudaMemcpyDeviceToHost, s));
  TDM_CHECK_CUDA(cudaMemcpyAsync(h_info, p->info, 16, cudaMemcpyDeviceToHost, s));
  TDM_CHECK_CUDA(cudaMemcpyAsync(h_info + 4, p->npairs, 4, cudaMemcpyDeviceToHost, s));
  TDM_CHECK_CUDA(cudaStreamSynchronize(s));
  for (int i = 0; i < 12; ++i) r->rt[i] = h_rt[i];
  r->rt[12] = r->rt[13] = r->rt[14] = 0.0;
  r->rt[15] = 1.0;
  r->n_inliers = h_info[0];
  r->best_trial = h_info[1];
  r->n_matches = h_info[4];
  r->keypoints[0] = ka;
  r->keypoints[1] = kb;
  for (int f = 0; f < 2; ++f)
    for (int a = 0; a < 3; ++a) r->grid_dim[f][a] = g[f].dim[a];
  return TDM_OK;
}

tdm_status pair_back(tdm_pipeline* p, int32_t k, const tdm_grid g[2], tdm_pair_result* r, cudaStream_t s) {
  tdm_status st = tdm_net_forward(p->net, p->patches, 2 * k, p->desc, s);
  if (st) return st;
  return match_back(p, p->desc, p->kp[0], k, p->desc + (size_t)k * 512, p->kp[1], k, g, r, s);
}

}  // namespace

extern "C" tdm_status tdm_describe_fragment(tdm_pipeline* p, const float* pts, int32_t n, uint64_t seed, int32_t k,
                                            float* keypts, float* desc, tdm_grid* grid_out, tdm_stream s) {
  TDM_REQUIRE(p && pts && keypts && desc && n > 0 && k > 0 && p->net, "tdm_describe_fragment: bad arguments");
  TDM_REQUIRE(n <= p->cfg.max_points && k <= p->cfg.max_keypoints, "tdm_describe_fragment: exceeds pipeline limits");
  tdm_grid g;
  const float trunc = p->cfg.voxel_size * p->cfg.trunc_voxels;
  tdm_status st = tdm_grid_from_points(pts, n, p->cfg.voxel_size, trunc, p->cfg.pad, &g, p->grid_ws, s);
  if (st) return st;
  st = fragment_front(p, 0, pts, n, g, seed, k, keypts, p->patches, s);
  if (st) return st;
  st = tdm_net_forward(p->net, p->patches, k, desc, s);
  if (st) return st;
  if (grid_out) *grid_out = g;
  return TDM_OK;
}

extern "C" tdm_status tdm_register_pair(tdm_pipeline* p, const float* a, int32_t na, const float* b, int32_t nb,
                                        uint64_t seed, int32_t k, tdm_pair_result* r, tdm_stream s) {
  TDM_REQUIRE(p && a && b && r && na > 0 && nb > 0 && k > 0 && p->net, "tdm_register_pair: bad arguments");
  TDM_REQUIRE(na <= p->cfg.max_points && nb <= p->cfg.max_points && k <= p->cfg.max_keypoints,
              "tdm_register_pair: exceeds pipeline limits");
  const float trunc = p->cfg.voxel_size * p->cfg.trunc_voxels;
  tdm_grid g[2];
  const float* src[2] = {a, b};
  const int32_t n[2] = {na, nb};
  for (int f = 0; f < 2; ++f) {
    tdm_status st = tdm_grid_from_points(src[f], n[f], p->cfg.voxel_size, trunc, p->cfg.pad, &g[f], p->grid_ws, s);
    if (st) return st;
    // fragment B draws its keypoints from the next seed
    st = fragment_front(p, f, src[f], n[f], g[f], seed + (uint64_t)f, k, p->kp[f],
                        p->patches + (size_t)f * k * 27000, s);
    if (st) return st;
  }
  return pair_back(p, k, g, r, s);
}

extern "C" tdm_status tdm_register_pair_host(tdm_pipeline* p, const float* a, int32_t na, const float* b, int32_t nb,
                                             uint64_t seed, int32_t k, tdm_pair_result* r, tdm_stream s) {
  TDM_REQUIRE(p && a && b && r && na > 0 && nb > 0 && k > 0 && p->net, "tdm_register_pair_host: bad arguments");
  TDM_REQUIRE(na <= p->cfg.max_points && nb <= p->cfg.max_points && k <= p->cfg.max_keypoints,
              "tdm_register_pair_host: exceeds pipeline limits");
  const float trunc = p->cfg.voxel_size * p->cfg.trunc_voxels;
  tdm_grid g[2];
  const float* src[2] = {a, b};
  const int32_t n[2] = {na, nb};
  for (int f = 0; f < 2; ++f) {
    TDM_CHECK_CUDA(cudaMemcpyAsync(p->pts[f], src[f], (size_t)n[f] * 12, cudaMemcpyHostToDevice, s));
    // the grid from the copied points on the device (the same bits as the host
    // form): a host pass over 150k points costs ~0.3 ms while the GPU has
    // nothing queued, the device bounding box ~4 us plus one small readback
    tdm_status st = tdm_grid_from_points(p->pts[f], n[f], p->cfg.voxel_size, trunc, p->cfg.pad, &g[f], p->grid_ws, s);
    if (st) return st;
    st = fragment_front(p, f, p->pts[f], n[f], g[f], seed + (uint64_t)f, k, p->kp[f],
                        p->patches + (size_t)f * k * 27000, s);
    if (st) return st;
  }
  return pair_back(p, k, g, r, s);
}

extern "C" tdm_status tdm_register_stored(tdm_pipeline* p, tdm_store* store, uint64_t key_a, uint64_t key_b,
                                          tdm_pair_result* r, tdm_stream s) {
  TDM_REQUIRE(p && store && r, "tdm_register_stored: null pointer");
  StoreView va{}, vb{};
  tdm_status st = store_acquire(store, key_a, &va, s);
  if (st) return st;
  st = store_acquire(store, key_b, &vb, s);
  if (st) {
    store_release(store, key_a);
    return st;
  }
  if (va.k > p->cfg.max_keypoints || vb.k > p->cfg.max_keypoints)
    st = fail(TDM_ERR_INVALID_ARG, "tdm_register_stored: fragment has more keypoints than the pipeline's max_keypoints");
  const tdm_grid g[2] = {va.grid, vb.grid};
  // match_back synchronizes the stream, so the entries are no longer read
  // when they are released
  if (!st) st = match_back(p, va.desc, va.keypts, va.k, vb.desc, vb.keypts, vb.k, g, r, s);
  store_release(store, key_a);
  store_release(store, key_b);
  return st;
}
