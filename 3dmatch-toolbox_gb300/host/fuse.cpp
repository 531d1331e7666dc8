// Drop-in for depth-fusion/demo.cu:
//   fuse [K_file data_dir base_idx first_idx num_frames ox oy oz voxel_size trunc] [options]
//
// Same inputs and output as the reference (depth-fusion/demo.cu:72-192):
//   K_file       3 x 3 camera intrinsics, text
//   data_dir     frame-XXXXXX.depth.png (16-bit grey, millimetres) and
//                frame-XXXXXX.pose.txt (4 x 4 camera-to-world, text)
//   frames first_idx .. first_idx + num_frames - 1 are fused into a
//   500^3 TSDF (origin and voxel size as given, weights averaged), in the
//   coordinates of frame base_idx, and the surface (|tsdf| < 0.2, weight > 1)
//   is written to tsdf.ply (binary little-endian x, y, z float).
// Without arguments the reference's defaults are used.  Options:
//   --dims X Y Z   grid size (500 500 500)
//   --out PATH     output file (tsdf.ply)
#include <cuda_runtime.h>
#include <zlib.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
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

bool load_matrix(const std::string& path, int n, float* out) {
  FILE* fp = std::fopen(path.c_str(), "r");
  if (!fp) return false;
  bool good = true;
  for (int i = 0; i < n && good; ++i) good = std::fscanf(fp, "%f", &out[i]) == 1;
  std::fclose(fp);
  return good;
}

uint32_t be32(const uint8_t* p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

int paeth(int a, int b, int c) {
  const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
  if (pa <= pb && pa <= pc) return a;
  return pb <= pc ? b : c;
}

// A 16-bit greyscale, non-interlaced PNG into row-major uint16 (what the
// reference reads with cv::imread(..., IMREAD_UNCHANGED)).
bool read_png16(const std::string& path, std::vector<uint16_t>* out, int* w, int* h, std::string* err) {
  std::ifstream f(path.c_str(), std::ios::binary);
  if (!f) { *err = "cannot open " + path; return false; }
  std::vector<uint8_t> b((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
  if (b.size() < 8 || std::memcmp(b.data(), sig, 8) != 0) { *err = path + " is not a PNG"; return false; }
  std::vector<uint8_t> idat;
  *w = *h = 0;
  size_t p = 8;
  while (p + 12 <= b.size()) {
    const uint32_t len = be32(&b[p]);
    if (p + 12 + (size_t)len > b.size()) { *err = path + ": truncated chunk"; return false; }
    const std::string type(reinterpret_cast<const char*>(&b[p + 4]), 4);
    const uint8_t* d = &b[p + 8];
    if (type == "IHDR") {
      if (len < 13) { *err = path + ": bad IHDR"; return false; }
      *w = (int)be32(d);
      *h = (int)be32(d + 4);
      if (d[8] != 16 || d[9] != 0 || d[12] != 0) { *err = path + ": need a 16-bit grey non-interlaced PNG"; return false; }
    } else if (type == "IDAT") {
      idat.insert(idat.end(), d, d + len);
    } else if (type == "IEND") {
      break;
    }
    p += 12 + (size_t)len;
  }
  if (*w <= 0 || *h <= 0) { *err = path + ": no image header"; return false; }
  const size_t stride = (size_t)*w * 2;
  std::vector<uint8_t> raw((stride + 1) * (size_t)*h);
  uLongf n = (uLongf)raw.size();
  if (uncompress(raw.data(), &n, idat.data(), (uLong)idat.size()) != Z_OK || n != raw.size()) {
    *err = path + ": corrupt image data";
    return false;
  }
  std::vector<uint8_t> prev(stride, 0), cur(stride);
  out->resize((size_t)*w * *h);
  for (int r = 0; r < *h; ++r) {
    const uint8_t ft = raw[r * (stride + 1)];
    const uint8_t* in = &raw[r * (stride + 1) + 1];
    for (size_t i = 0; i < stride; ++i) {
      const int a = i >= 2 ? cur[i - 2] : 0, up = prev[i], c = i >= 2 ? prev[i - 2] : 0;
      int pred = 0;
      switch (ft) {
        case 0: pred = 0; break;
        case 1: pred = a; break;
        case 2: pred = up; break;
        case 3: pred = (a + up) >> 1; break;
        case 4: pred = paeth(a, up, c); break;
        default: *err = path + ": bad row filter"; return false;
      }
      cur[i] = (uint8_t)(in[i] + pred);
    }
    for (int x = 0; x < *w; ++x) (*out)[(size_t)r * *w + x] = (uint16_t)((cur[2 * x] << 8) | cur[2 * x + 1]);
    prev.swap(cur);
  }
  return true;
}

// Inverse of a row-major 4x4 by cofactors (adjugate / determinant).
bool invert4(const float m[16], float inv[16]) {
  auto at = [&](int r, int c) { return m[r * 4 + c]; };
  float cof[16];
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      float s[9];
      int k = 0;
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
          if (i != r && j != c) s[k++] = at(i, j);
      const float det3 = s[0] * (s[4] * s[8] - s[5] * s[7]) - s[1] * (s[3] * s[8] - s[5] * s[6]) +
                         s[2] * (s[3] * s[7] - s[4] * s[6]);
      cof[r * 4 + c] = ((r + c) & 1) ? -det3 : det3;
    }
  const float det = at(0, 0) * cof[0] + at(0, 1) * cof[1] + at(0, 2) * cof[2] + at(0, 3) * cof[3];
  if (det == 0.0f) return false;
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) inv[r * 4 + c] = cof[c * 4 + r] / det;
  return true;
}

void mul4(const float a[16], const float b[16], float out[16]) {
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j)
      out[i * 4 + j] = a[i * 4 + 0] * b[0 * 4 + j] + a[i * 4 + 1] * b[1 * 4 + j] + a[i * 4 + 2] * b[2 * 4 + j] +
                       a[i * 4 + 3] * b[3 * 4 + j];
}

std::string frame_name(const std::string& dir, int idx, const char* suffix) {
  std::ostringstream s;
  s << dir << "/frame-" << std::setw(6) << std::setfill('0') << idx << suffix;
  return s.str();
}

}  // namespace

int main(int argc, char** argv) {
  std::string k_file = "../data/sample/depth-fusion-demo/camera-intrinsics.txt";
  std::string dir = "../data/sample/depth-fusion-demo/rgbd-frames";
  int base_idx = 8, first_idx = 8;
  float n_frames_f = 50;
  float origin[3] = {-1.5f, -1.5f, 0.5f};
  float vs = 0.006f, trunc = vs * 5;
  int32_t dim[3] = {500, 500, 500};
  std::string out = "tsdf.ply";
  std::vector<std::string> pos;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    if (a == "--dims" && i + 3 < argc) {
      for (int q = 0; q < 3; ++q) dim[q] = std::atoi(argv[++i]);
    } else if (a == "--out" && i + 1 < argc) {
      out = argv[++i];
    } else if (a.rfind("--", 0) == 0) {
      std::cerr << "unknown option " << a << std::endl;
      return 2;
    } else {
      pos.push_back(a);
    }
  }
  if (!pos.empty()) {
    if (pos.size() < 10) {
      std::cerr << "usage: fuse [K_file data_dir base_idx first_idx num_frames ox oy oz voxel_size trunc]"
                   " [--dims X Y Z] [--out PATH]" << std::endl;
      return 2;
    }
    k_file = pos[0];
    dir = pos[1];
    base_idx = std::atoi(pos[2].c_str());
    first_idx = std::atoi(pos[3].c_str());
    n_frames_f = (float)std::atof(pos[4].c_str());
    for (int q = 0; q < 3; ++q) origin[q] = (float)std::atof(pos[5 + q].c_str());
    vs = (float)std::atof(pos[8].c_str());
    trunc = (float)std::atof(pos[9].c_str());
  }
  const int n_frames = (int)n_frames_f;
  if (n_frames <= 0 || dim[0] <= 0 || dim[1] <= 0 || dim[2] <= 0) {
    std::cerr << "nothing to fuse" << std::endl;
    return 2;
  }
  float K[9], base2world[16], world2base[16];
  if (!load_matrix(k_file, 9, K)) { std::cerr << "cannot read " << k_file << std::endl; return 1; }
  if (!load_matrix(frame_name(dir, base_idx, ".pose.txt"), 16, base2world) || !invert4(base2world, world2base)) {
    std::cerr << "cannot read or invert the base frame pose" << std::endl;
    return 1;
  }
  std::vector<uint16_t> mm;
  std::vector<float> cam2base((size_t)n_frames * 16);
  int W = 0, H = 0;
  for (int f = 0; f < n_frames; ++f) {
    const int idx = first_idx + f;
    std::vector<uint16_t> img;
    int w = 0, h = 0;
    std::string err;
    if (!read_png16(frame_name(dir, idx, ".depth.png"), &img, &w, &h, &err)) { std::cerr << err << std::endl; return 1; }
    if (f == 0) { W = w; H = h; mm.reserve((size_t)n_frames * W * H); }
    if (w != W || h != H) { std::cerr << "depth frames differ in size" << std::endl; return 1; }
    mm.insert(mm.end(), img.begin(), img.end());
    float cam2world[16];
    if (!load_matrix(frame_name(dir, idx, ".pose.txt"), 16, cam2world)) {
      std::cerr << "cannot read the pose of frame " << idx << std::endl;
      return 1;
    }
    mul4(world2base, cam2world, &cam2base[(size_t)f * 16]);
    std::cout << "Fusing: " << frame_name(dir, idx, ".depth.png") << std::endl;
  }
  const size_t V = (size_t)dim[0] * dim[1] * dim[2], npx = (size_t)n_frames * W * H;
  float *d_tsdf = nullptr, *d_w = nullptr, *d_depth = nullptr, *d_pts = nullptr;
  uint16_t* d_mm = nullptr;
  int64_t* d_n = nullptr;
  void* d_ws = nullptr;
  const size_t ws_bytes = tdm_extract_workspace_bytes(dim);
  if (cudaMalloc(&d_tsdf, V * 4) || cudaMalloc(&d_w, V * 4) || cudaMalloc(&d_depth, npx * 4) ||
      cudaMalloc(&d_mm, npx * 2) || cudaMalloc(&d_n, 8) || cudaMalloc(&d_ws, ws_bytes + 16) ||
      cudaMalloc(&d_pts, V * 12)) {
    std::cerr << "out of device memory" << std::endl;
    return 1;
  }
  tdm_stream s = nullptr;
  cudaMemcpy(d_mm, mm.data(), npx * 2, cudaMemcpyHostToDevice);
  if (!ok(tdm_depth_from_mm(d_mm, (int64_t)npx, d_depth, s), "depth")) return 1;
  if (!ok(tdm_tsdf_init(d_tsdf, d_w, dim, s), "init")) return 1;
  if (!ok(tdm_tsdf_integrate(d_tsdf, d_w, dim, origin, vs, trunc, d_depth, n_frames, H, W, K, cam2base.data(), s),
          "integrate"))
    return 1;
  if (!ok(tdm_tsdf_extract(d_tsdf, d_w, dim, origin, vs, 0.2f, 1.0f, d_pts, (int64_t)V, d_n, d_ws, ws_bytes, s),
          "extract"))
    return 1;
  int64_t n = 0;
  cudaMemcpy(&n, d_n, 8, cudaMemcpyDeviceToHost);
  std::vector<float> pts((size_t)n * 3);
  cudaMemcpy(pts.data(), d_pts, pts.size() * 4, cudaMemcpyDeviceToHost);
  if (!ok(tdm_device_status(s), "device")) return 1;
  std::cout << "Saving surface point cloud (" << out << ")..." << std::endl;
  std::ofstream pf(out.c_str(), std::ios::binary);
  pf << "ply\nformat binary_little_endian 1.0\nelement vertex " << n
     << "\nproperty float x\nproperty float y\nproperty float z\nend_header\n";
  pf.write(reinterpret_cast<const char*>(pts.data()), (std::streamsize)(pts.size() * 4));
  if (!pf) {
    std::cerr << "write failed" << std::endl;
    return 1;
  }
  cudaFree(d_tsdf);
  cudaFree(d_w);
  cudaFree(d_depth);
  cudaFree(d_mm);
  cudaFree(d_n);
  cudaFree(d_ws);
  cudaFree(d_pts);
  return 0;
}
