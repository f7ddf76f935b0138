// jpeg.h -- sequential JPEG decoding for the image reader (see jpeg.cpp).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace Pupil::util {

// Baseline / extended sequential Huffman JPEG, 8-bit, grey or YCbCr: 8-bit
// samples, `comp` (1 or 3) per pixel, rows top first.
bool DecodeJpeg(const std::vector<uint8_t> &data, std::vector<uint8_t> &img, uint32_t &width, uint32_t &height,
                int &comp, std::string &error);

}  // namespace Pupil::util
