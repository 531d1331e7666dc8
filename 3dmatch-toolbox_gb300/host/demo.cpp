// Drop-in for core/demo.cu:  demo <cloud.ply> <out_prefix> [options]
//
// Same inputs and outputs as the reference:
//   reads a binary little-endian PLY (7 header lines, vertex count as the
//   third token of line 3, then N x 3 float32; core/demo.cu:69-93),
//   writes <prefix>.keypts.bin  (float K, then K x 3 float; :236-244)
//   and    <prefix>.desc.3dmatch.bin (float K, float 512, then K x 512 float; :246-255),
//   reads the net weights from 3dmatch-weights-snapshot-137000.marvin in the
//   working directory (:180-182).
// Exit codes follow the reference: -1 when the cloud is missing, 0 when the
// vertex count is missing.  Options (all default to the reference's values):
//   --weights PATH         weight file
//   --seeded-weights SEED  write and use seeded He-normal weights instead
//   --keypoints K          number of keypoints (500)
//   --seed S               keypoint stream seed (default: random, like the reference)
//   --precision fp32|bf16  net precision (fp32 = the reference's arithmetic)
//   --tdf-out              also write tdf.bin (the commented writer at :257-274)
//   --ref-compat float|fma reproduce the reference's float32 voxel-index decode
//   --info                 stop after reading the cloud and setting up the grid
//                          (prints the count, first/last point and grid; no GPU)
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "tdm.h"

namespace {

bool ok(tdm_status st, const char* what) {
  if (st == TDM_OK) return true;
  std::cerr << what << " failed: " << tdm_last_error() << std::endl;
  return false;
}

template <typename T>
struct DevBuf {
  T* p = nullptr;
  explicit DevBuf(size_t n) {
    if (cudaMalloc(&p, n * sizeof(T) + 16) != cudaSuccess) p = nullptr;
  }
  ~DevBuf() { cudaFree(p); }
};

bool write_floats(std::ofstream& f, const float* v, size_t n) {
  f.write(reinterpret_cast<const char*>(v), n * sizeof(float));
  return static_cast<bool>(f);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::cerr << "usage: demo <cloud.ply> <out_prefix> [--weights PATH] [--seeded-weights SEED] [--keypoints K]"
                 " [--seed S] [--precision fp32|bf16] [--tdf-out] [--ref-compat float|fma] [--info]"
              << std::endl;
    return 2;
  }
  std::string cloud = argv[1], prefix = argv[2];
  std::string weights = "3dmatch-weights-snapshot-137000.marvin";
  bool seeded = false, tdf_out = false, info = false;
  uint64_t wseed = 0, seed = std::random_device{}();
  int k = 50 * 10;
  tdm_precision prec = TDM_FP32;
  int mode = TDM_TDF_EXACT;
  for (int i = 3; i < argc; ++i) {
    std::string a = argv[i];
    auto next = [&]() -> std::string { return i + 1 < argc ? std::string(argv[++i]) : std::string(); };
    if (a == "--weights") weights = next();
    else if (a == "--seeded-weights") { seeded = true; wseed = std::strtoull(next().c_str(), nullptr, 10); }
    else if (a == "--keypoints") k = std::atoi(next().c_str());
    else if (a == "--seed") seed = std::strtoull(next().c_str(), nullptr, 10);
    else if (a == "--precision") { std::string p = next(); prec = p == "bf16" ? TDM_BF16 : TDM_FP32; }
    else if (a == "--tdf-out") tdf_out = true;
    else if (a == "--info") info = true;
    else if (a == "--ref-compat") { std::string m = next(); mode = m == "fma" ? TDM_TDF_REFCOMPAT_FMA : TDM_TDF_REFCOMPAT_FLOAT; }
    else { std::cerr << "unknown option " << a << std::endl; return 2; }
  }
  if (k <= 0) { std::cerr << "--keypoints must be > 0" << std::endl; return 2; }

  std::ifstream f(cloud.c_str(), std::ios::binary);
  if (!f) {
    std::cerr << "Point cloud file not found." << std::endl;
    return -1;
  }
  int num_pts = 0;
  for (int line = 0; line < 7; ++line) {
    std::string s;
    std::getline(f, s);
    if (line == 2) {
      std::istringstream t(s);
      std::string w;
      t >> w >> w >> num_pts;
    }
  }
  if (num_pts <= 0) {
    std::cerr << "Third line of .ply file does not tell me number of points." << std::endl;
    return 0;
  }
  std::vector<float> pts((size_t)num_pts * 3);
  f.read(reinterpret_cast<char*>(pts.data()), (std::streamsize)(pts.size() * sizeof(float)));
  if ((size_t)f.gcount() != pts.size() * sizeof(float)) {
    std::cerr << "Point cloud file is truncated." << std::endl;
    return 1;
  }
  std::cout << "Loaded point cloud with " << num_pts << " points!" << std::endl;

  const float voxel_size = 0.01f, trunc_margin = voxel_size * 5;
  tdm_grid g;
  if (!ok(tdm_grid_from_points_host(pts.data(), num_pts, voxel_size, trunc_margin, 15, &g), "grid")) return 1;
  std::cout << "Size of TDF voxel grid: " << g.dim[0] << " x " << g.dim[1] << " x " << g.dim[2] << std::endl;
  if (info) {
    const size_t last = (size_t)(num_pts - 1) * 3;
    std::printf("points %d first %.9g %.9g %.9g last %.9g %.9g %.9g\n", num_pts, pts[0], pts[1], pts[2], pts[last],
                pts[last + 1], pts[last + 2]);
    std::printf("grid %d %d %d origin %.9g %.9g %.9g\n", g.dim[0], g.dim[1], g.dim[2], g.origin[0], g.origin[1],
                g.origin[2]);
    return 0;
  }
  std::cout << "Computing TDF voxel grid..." << std::endl;
  const size_t V = (size_t)g.dim[0] * g.dim[1] * g.dim[2];
  DevBuf<float> d_pts(pts.size()), d_tdf(V), d_kp((size_t)k * 3), d_patch((size_t)k * 27000), d_desc((size_t)k * 512);
  DevBuf<uint8_t> d_occ(tdm_tdf_workspace_bytes(&g));
  DevBuf<int32_t> d_idx(k), d_kpg((size_t)k * 3);
  if (!d_pts.p || !d_tdf.p || !d_kp.p || !d_patch.p || !d_desc.p || !d_occ.p || !d_idx.p || !d_kpg.p) {
    std::cerr << "out of device memory" << std::endl;
    return 1;
  }
  cudaMemcpy(d_pts.p, pts.data(), pts.size() * sizeof(float), cudaMemcpyHostToDevice);
  tdm_stream s = nullptr;
  if (!ok(tdm_tdf(d_pts.p, num_pts, &g, mode, d_tdf.p, d_occ.p, tdm_tdf_workspace_bytes(&g), s), "TDF")) return 1;

  std::cout << "Finding random surface keypoints (seed " << seed << ")..." << std::endl;
  if (!ok(tdm_keypoint_indices(seed, num_pts, k, d_idx.p, s), "keypoint indices")) return 1;
  if (!ok(tdm_keypoints(d_pts.p, num_pts, d_idx.p, k, &g, d_kp.p, d_kpg.p, s), "keypoints")) return 1;
  if (!ok(tdm_gather(d_tdf.p, &g, d_kpg.p, k, d_patch.p, s), "gather")) return 1;

  if (seeded) {
    weights = prefix + ".seeded-weights.marvin";
    if (!ok(tdm_write_seeded_weights(weights.c_str(), wseed), "seeded weights")) return 1;
  }
  tdm_net* net = nullptr;
  if (!ok(tdm_net_create(weights.c_str(), prec, 1, &net), "net")) return 1;
  std::cout << "3DMatch network architecture successfully loaded!" << std::endl;
  std::cout << "Computing 3DMatch descriptors for " << k << " keypoints..." << std::endl;
  if (!ok(tdm_net_forward(net, d_patch.p, k, d_desc.p, s), "forward")) return 1;
  std::vector<float> kp((size_t)k * 3), desc((size_t)k * 512);
  cudaMemcpy(kp.data(), d_kp.p, kp.size() * sizeof(float), cudaMemcpyDeviceToHost);
  cudaMemcpy(desc.data(), d_desc.p, desc.size() * sizeof(float), cudaMemcpyDeviceToHost);
  if (!ok(tdm_device_status(s), "device")) return 1;
  tdm_net_destroy(net);

  std::cout << "Saving keypoints to disk (keypts.bin)..." << std::endl;
  std::ofstream kf(prefix + ".keypts.bin", std::ios::binary);
  float kf_n = (float)k, dsz = 512.0f;
  if (!write_floats(kf, &kf_n, 1) || !write_floats(kf, kp.data(), kp.size())) { std::cerr << "write failed" << std::endl; return 1; }
  std::cout << "Saving 3DMatch descriptors to disk (desc.3dmatch.bin)..." << std::endl;
  std::ofstream df(prefix + ".desc.3dmatch.bin", std::ios::binary);
  if (!write_floats(df, &kf_n, 1) || !write_floats(df, &dsz, 1) || !write_floats(df, desc.data(), desc.size())) {
    std::cerr << "write failed" << std::endl;
    return 1;
  }
  if (tdf_out) {
    std::vector<float> tdf(V);
    cudaMemcpy(tdf.data(), d_tdf.p, V * sizeof(float), cudaMemcpyDeviceToHost);
    std::ofstream tf("tdf.bin", std::ios::binary);
    float hdr[8] = {(float)g.dim[0], (float)g.dim[1], (float)g.dim[2], g.origin[0], g.origin[1], g.origin[2],
                    g.voxel_size, g.trunc_margin};
    if (!write_floats(tf, hdr, 8) || !write_floats(tf, tdf.data(), V)) { std::cerr << "write failed" << std::endl; return 1; }
  }
  return 0;
}
