// .marvin weight-file reader/writer and the seeded He-normal initialiser.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "tdm.h"

namespace tdm {

struct MarvinTensor {
  std::vector<int32_t> dims;
  std::vector<float> data;
};

tdm_status read_marvin(const char* path, std::map<std::string, MarvinTensor>* out, std::string* err);
tdm_status write_marvin_f32(const char* path, const std::vector<std::pair<std::string, MarvinTensor>>& tensors,
                            std::string* err);
std::vector<std::pair<std::string, MarvinTensor>> seeded_weights(uint64_t seed);

}  // namespace tdm
