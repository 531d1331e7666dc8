// .marvin tensor files (Marvin's weight format, core/marvin.hpp:2515-2530 type
// ids, 2581-2612 read, 2764-2790 write): repeated records
//   u8 typeid; u32 sizeof; i32 nameLen; char name[nameLen]; i32 nDims;
//   i32 dims[nDims]; T data[prod(dims)]
// Type ids 0 half, 1 float, 2 double are accepted and converted to float, as
// Marvin converts on load (core/marvin.hpp:2634-2705).  Unlike Marvin, a
// missing file is an error, not a retry loop.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "marvin_io.h"

namespace tdm {

static float half_to_float(uint16_t h) {
  uint32_t sign = (uint32_t)(h >> 15) << 31, exp = (h >> 10) & 0x1F, man = h & 0x3FF;
  uint32_t bits;
  if (exp == 0) {
    if (man == 0) {
      bits = sign;
    } else {  // subnormal: renormalise
      int e = -1;
      do { man <<= 1; ++e; } while (!(man & 0x400));
      bits = sign | (uint32_t)(127 - 15 - e) << 23 | (man & 0x3FF) << 13;
    }
  } else if (exp == 31) {
    bits = sign | 0x7F800000u | man << 13;
  } else {
    bits = sign | (exp + 112) << 23 | man << 13;
  }
  float f;
  std::memcpy(&f, &bits, 4);
  return f;
}

tdm_status read_marvin(const char* path, std::map<std::string, MarvinTensor>* out, std::string* err) {
  FILE* fp = std::fopen(path, "rb");
  if (!fp) {
    *err = std::string("cannot open weight file ") + path;
    return TDM_ERR_IO;
  }
  tdm_status st = TDM_OK;
  while (true) {
    int c = std::fgetc(fp);
    if (c == EOF) break;
    uint8_t tid = (uint8_t)c;
    uint32_t tsz = 0;
    int32_t ln = 0, nd = 0;
    if (std::fread(&tsz, 4, 1, fp) != 1 || std::fread(&ln, 4, 1, fp) != 1 || ln < 0 || ln > 4096) {
      *err = "truncated or corrupt tensor header";
      st = TDM_ERR_FORMAT;
      break;
    }
    size_t want = tid == 0 ? 2 : tid == 1 ? 4 : tid == 2 ? 8 : 0;
    if (want == 0 || tsz != want) {
      *err = "unsupported tensor type id " + std::to_string(tid) + " with sizeof " + std::to_string(tsz);
      st = TDM_ERR_FORMAT;
      break;
    }
    std::string name(ln, '\0');
    if (ln > 0 && std::fread(&name[0], 1, ln, fp) != (size_t)ln) {
      *err = "truncated tensor name";
      st = TDM_ERR_FORMAT;
      break;
    }
    if (std::fread(&nd, 4, 1, fp) != 1 || nd < 0 || nd > 16) {
      *err = "bad dimension count for " + name;
      st = TDM_ERR_FORMAT;
      break;
    }
    MarvinTensor t;
    t.dims.resize(nd);
    size_t count = 1;
    if (nd > 0 && std::fread(t.dims.data(), 4, nd, fp) != (size_t)nd) {
      *err = "truncated dims for " + name;
      st = TDM_ERR_FORMAT;
      break;
    }
    for (int d : t.dims) {
      if (d < 0) { st = TDM_ERR_FORMAT; break; }
      count *= (size_t)d;
    }
    if (st != TDM_OK || count > ((size_t)1 << 32)) {
      *err = "bad dims for " + name;
      st = TDM_ERR_FORMAT;
      break;
    }
    std::vector<uint8_t> raw(count * tsz);
    if (count && std::fread(raw.data(), 1, raw.size(), fp) != raw.size()) {
      *err = "truncated data for " + name;
      st = TDM_ERR_FORMAT;
      break;
    }
    t.data.resize(count);
    for (size_t i = 0; i < count; ++i) {
      if (tid == 0) {
        uint16_t h;
        std::memcpy(&h, &raw[2 * i], 2);
        t.data[i] = half_to_float(h);
      } else if (tid == 1) {
        std::memcpy(&t.data[i], &raw[4 * i], 4);
      } else {
        double d;
        std::memcpy(&d, &raw[8 * i], 8);
        t.data[i] = (float)d;
      }
    }
    (*out)[name] = std::move(t);
  }
  std::fclose(fp);
  return st;
}

tdm_status write_marvin_f32(const char* path, const std::vector<std::pair<std::string, MarvinTensor>>& tensors,
                            std::string* err) {
  FILE* fp = std::fopen(path, "wb");
  if (!fp) {
    *err = std::string("cannot create ") + path;
    return TDM_ERR_IO;
  }
  bool ok = true;
  for (const auto& kv : tensors) {
    uint8_t tid = 1;
    uint32_t tsz = 4;
    int32_t ln = (int32_t)kv.first.size(), nd = (int32_t)kv.second.dims.size();
    ok = ok && std::fwrite(&tid, 1, 1, fp) == 1 && std::fwrite(&tsz, 4, 1, fp) == 1 &&
         std::fwrite(&ln, 4, 1, fp) == 1 && std::fwrite(kv.first.data(), 1, ln, fp) == (size_t)ln &&
         std::fwrite(&nd, 4, 1, fp) == 1 && std::fwrite(kv.second.dims.data(), 4, nd, fp) == (size_t)nd &&
         std::fwrite(kv.second.data.data(), 4, kv.second.data.size(), fp) == kv.second.data.size();
  }
  if (std::fclose(fp) != 0) ok = false;
  if (!ok) {
    *err = std::string("write failed: ") + path;
    return TDM_ERR_IO;
  }
  return TDM_OK;
}

// splitmix64 stream -> Box-Muller normals; deterministic for a given seed.
static uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

std::vector<std::pair<std::string, MarvinTensor>> seeded_weights(uint64_t seed) {
  static const int cout[9] = {64, 64, 128, 128, 256, 256, 512, 512, 512};
  static const int cin[9] = {1, 64, 64, 128, 128, 256, 256, 512, 512};
  static const int ks[9] = {3, 3, 3, 3, 3, 3, 3, 3, 1};
  static const char* names[9] = {"conv1", "conv2", "conv3", "conv4", "conv5", "conv6", "conv7", "conv8", "feat"};
  std::vector<std::pair<std::string, MarvinTensor>> out;
  uint64_t ctr = 0;
  auto uniform = [&]() {  // (0, 1]
    uint64_t r = mix64(seed + (++ctr) * 0x9E3779B97F4A7C15ULL);
    return ((double)(r >> 11) + 1.0) * (1.0 / 9007199254740992.0);
  };
  for (int l = 0; l < 9; ++l) {
    MarvinTensor w, b;
    w.dims = {cout[l], cin[l], ks[l], ks[l], ks[l]};
    b.dims = {1, cout[l], 1, 1, 1};
    size_t n = (size_t)cout[l] * cin[l] * ks[l] * ks[l] * ks[l];
    double sd = std::sqrt(2.0 / (double)(cin[l] * ks[l] * ks[l] * ks[l]));
    w.data.resize(n);
    for (size_t i = 0; i < n; i += 2) {
      double u1 = uniform(), u2 = uniform();
      double r = std::sqrt(-2.0 * std::log(u1)), th = 6.283185307179586 * u2;
      w.data[i] = (float)(sd * r * std::cos(th));
      if (i + 1 < n) w.data[i + 1] = (float)(sd * r * std::sin(th));
    }
    b.data.resize(cout[l]);
    for (int k = 0; k < cout[l]; ++k) b.data[k] = (float)(0.1 * uniform() - 0.05);
    out.emplace_back(std::string(names[l]) + ".weight", std::move(w));
    out.emplace_back(std::string(names[l]) + ".bias", std::move(b));
  }
  return out;
}

}  // namespace tdm
