// inflate.h -- zlib (RFC 1950) / DEFLATE (RFC 1951) decompression for the
// image readers: PNG image data and ZIP-compressed OpenEXR blocks.  The
// reference reads those formats through stb_image and tinyexr, which carry
// their own decompressors; neither library is part of this project.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace Pupil::util {

// Decompresses the zlib stream src[0, n): header check, stored / fixed /
// dynamic Huffman blocks, Adler-32 check.  Appends to `out`.  `limit` bounds
// the output size (a corrupt or hostile stream cannot make it grow beyond).
bool ZlibInflate(const uint8_t *src, size_t n, std::vector<uint8_t> &out, size_t limit, std::string &error);

}  // namespace Pupil::util
