// Drop-in for the reference's two other descriptor callers:
//
//   descriptors <volumes.bin> [options]
//     evaluation/keypoint-matching/get3DMatchDescriptors.cu: reads
//     float N, sx, sy, sz then N volumes of sx*sy*sz float (30^3 TDF patches,
//     z, y, x), writes feat.bin = float N, then the feat response dims
//     (512, 1, 1, 1), then one 512-float descriptor per volume.
//
//   descriptors <grid.TDF.bin> <name.keypoints.bin> [options]
//     evaluation/mesh-correspondence-shape2pose/get3DMatchDescriptors.cu:
//     reads float sx, sy, sz then the sx*sy*sz TDF grid (x fastest), and
//     float K then K x 3 float keypoint grid coordinates (rounded with C
//     round()); writes <name.keypoints>.3dmatch.descriptors.bin = float K,
//     float 512, then one descriptor per keypoint.
//
// Like the reference, both process whole batches of 50 only (the last N % 50
// volumes / keypoints get no descriptor) unless --all is given.  Patch voxels
// outside the grid read 0 here; the reference reads past its array.
// Options:
//   --weights PATH         (default 3dmatch-weights-snapshot-137000.marvin,
//                           -131000 for the grid form, as the reference)
//   --seeded-weights SEED  write and use seeded He-normal weights instead
//   --precision fp32|bf16  (fp32)
//   --out PATH             output file name
//   --all                  describe every volume / keypoint
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "tdm.h"

namespace {

bool ok(tdm_status st, const char* what) {
  if (st == TDM_OK) return true;
  std::cerr << what << " failed: " << tdm_last_error() << std::endl;
  return false;
}

bool read_floats(std::ifstream& f, float* v, size_t n) {
  f.read(reinterpret_cast<char*>(v), (std::streamsize)(n * sizeof(float)));
  return (size_t)f.gcount() == n * sizeof(float);
}

bool write_floats(std::ofstream& f, const float* v, size_t n) {
  f.write(reinterpret_cast<const char*>(v), (std::streamsize)(n * sizeof(float)));
  return static_cast<bool>(f);
}

struct Dev {
  void* p = nullptr;
  explicit Dev(size_t bytes) {
    if (cudaMalloc(&p, bytes + 16) != cudaSuccess) p = nullptr;
  }
  ~Dev() { cudaFree(p); }
};

constexpr int kBatch = 50;  // the reference's net batch

}  // namespace

int main(int argc, char** argv) {
  std::vector<std::string> pos;
  std::string weights, out;
  bool seeded = false, all = false;
  uint64_t wseed = 0;
  tdm_precision prec = TDM_FP32;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    auto next = [&]() -> std::string { return i + 1 < argc ? std::string(argv[++i]) : std::string(); };
    if (a == "--weights") weights = next();
    else if (a == "--seeded-weights") { seeded = true; wseed = std::strtoull(next().c_str(), nullptr, 10); }
    else if (a == "--precision") prec = next() == "bf16" ? TDM_BF16 : TDM_FP32;
    else if (a == "--out") out = next();
    else if (a == "--all") all = true;
    else if (a.size() > 1 && a[0] == '-' && a[1] == '-') { std::cerr << "unknown option " << a << std::endl; return 2; }
    else pos.push_back(a);
  }
  if (pos.empty() || pos.size() > 2) {
    std::cerr << "usage: descriptors <volumes.bin> | <grid.TDF.bin> <name.keypoints.bin> [--weights PATH]"
                 " [--seeded-weights SEED] [--precision fp32|bf16] [--out PATH] [--all]"
              << std::endl;
    return 2;
  }
  const bool grid_form = pos.size() == 2;
  if (weights.empty())
    weights = grid_form ? "3dmatch-weights-snapshot-131000.marvin" : "3dmatch-weights-snapshot-137000.marvin";

  std::ifstream f(pos[0].c_str(), std::ios::binary);
  if (!f) {
    std::cerr << "cannot open " << pos[0] << std::endl;
    return 1;
  }
  std::vector<float> patches;  // n x 27000
  int n = 0, described = 0;
  if (!grid_form) {
    float hdr[4];
    if (!read_floats(f, hdr, 4)) { std::cerr << "truncated header" << std::endl; return 1; }
    n = (int)hdr[0];
    const int gx = (int)hdr[1], gy = (int)hdr[2], gz = (int)hdr[3];
    if (n < 0 || gx != 30 || gy != 30 || gz != 30) {
      std::cerr << "expected 30 x 30 x 30 volumes" << std::endl;
      return 1;
    }
    patches.resize((size_t)n * 27000);
    if (!read_floats(f, patches.data(), patches.size())) { std::cerr << "truncated volumes" << std::endl; return 1; }
    std::cout << n << std::endl;
  }
  if (seeded) {
    weights = (grid_form ? pos[1] : pos[0]) + ".seeded-weights.marvin";
    if (!ok(tdm_write_seeded_weights(weights.c_str(), wseed), "seeded weights")) return 1;
  }
  tdm_net* net = nullptr;
  if (!ok(tdm_net_create(weights.c_str(), prec, 1, &net), "net")) return 1;

  tdm_stream s = nullptr;
  std::vector<float> desc;
  if (grid_form) {
    float dims[3];
    if (!read_floats(f, dims, 3)) { std::cerr << "truncated grid header" << std::endl; return 1; }
    tdm_grid g{};
    for (int a = 0; a < 3; ++a) g.dim[a] = (int32_t)dims[a];
    g.voxel_size = 1.0f;
    const size_t V = (size_t)g.dim[0] * g.dim[1] * g.dim[2];
    std::vector<float> tdf(V);
    if (!read_floats(f, tdf.data(), V)) { std::cerr << "truncated grid" << std::endl; return 1; }
    std::ifstream kf(pos[1].c_str(), std::ios::binary);
    float kn = 0;
    if (!kf || !read_floats(kf, &kn, 1)) { std::cerr << "cannot read " << pos[1] << std::endl; return 1; }
    n = (int)kn;
    std::vector<float> kp((size_t)n * 3);
    if (!read_floats(kf, kp.data(), kp.size())) { std::cerr << "truncated keypoints" << std::endl; return 1; }
    std::vector<int32_t> kg(kp.size());
    for (size_t i = 0; i < kp.size(); ++i) kg[i] = (int32_t)std::round(kp[i]);
    described = all ? n : n / kBatch * kBatch;
    Dev d_tdf(V * 4), d_kg(kg.size() * 4), d_p((size_t)std::max(described, 1) * 27000 * 4),
        d_desc((size_t)std::max(described, 1) * 512 * 4);
    if (!d_tdf.p || !d_kg.p || !d_p.p || !d_desc.p) { std::cerr << "out of device memory" << std::endl; return 1; }
    cudaMemcpy(d_tdf.p, tdf.data(), V * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(d_kg.p, kg.data(), kg.size() * 4, cudaMemcpyHostToDevice);
    if (described > 0) {
      if (!ok(tdm_gather(static_cast<float*>(d_tdf.p), &g, static_cast<int32_t*>(d_kg.p), described,
                         static_cast<float*>(d_p.p), s), "gather")) return 1;
      if (!ok(tdm_net_forward(net, static_cast<float*>(d_p.p), described, static_cast<float*>(d_desc.p), s),
              "forward")) return 1;
    }
    desc.resize((size_t)described * 512);
    cudaMemcpy(desc.data(), d_desc.p, desc.size() * 4, cudaMemcpyDeviceToHost);
    if (out.empty()) out = pos[1].substr(0, pos[1].size() >= 4 ? pos[1].size() - 4 : 0) + ".3dmatch.descriptors.bin";
  } else {
    described = all ? n : n / kBatch * kBatch;
    Dev d_p((size_t)std::max(described, 1) * 27000 * 4), d_desc((size_t)std::max(described, 1) * 512 * 4);
    if (!d_p.p || !d_desc.p) { std::cerr << "out of device memory" << std::endl; return 1; }
    cudaMemcpy(d_p.p, patches.data(), (size_t)described * 27000 * 4, cudaMemcpyHostToDevice);
    if (described > 0 &&
        !ok(tdm_net_forward(net, static_cast<float*>(d_p.p), described, static_cast<float*>(d_desc.p), s), "forward"))
      return 1;
    desc.resize((size_t)described * 512);
    cudaMemcpy(desc.data(), d_desc.p, desc.size() * 4, cudaMemcpyDeviceToHost);
    if (out.empty()) out = "feat.bin";
  }
  if (!ok(tdm_device_status(s), "device")) return 1;
  tdm_net_destroy(net);

  std::ofstream of(out.c_str(), std::ios::binary);
  const float nf = (float)n;
  bool w = write_floats(of, &nf, 1);
  if (grid_form) {
    const float dsz = 512.0f;
    w = w && write_floats(of, &dsz, 1);
  } else {
    const float dims[4] = {512.0f, 1.0f, 1.0f, 1.0f};  // the feat response's dims 1..4
    w = w && write_floats(of, dims, 4);
  }
  w = w && write_floats(of, desc.data(), desc.size());
  if (!w) {
    std::cerr << "write failed" << std::endl;
    return 1;
  }
  return 0;
}
