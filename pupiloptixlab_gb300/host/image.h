// image.h -- image readers for bitmap textures and environment maps.
//
// The reference loads images through stb_image (PNG/JPEG/... and Radiance
// .hdr) and tinyexr (framework/util/texture.cpp:87-151); neither library is
// part of this project.  This reader covers the floating-point formats:
//   .hdr  Radiance RGBE (flat or run-length encoded scanlines): value =
//         mantissa * 2^(exponent - 136), 0 when the exponent byte is 0;
//   .pfm  portable float map (PF colour / Pf grey, either byte order, rows
//         stored bottom-up in the file);
//   .png  PNG of every colour type and bit depth, interlaced or not (8-bit
//         samples as an 8-bit load gives them, converted as the reference
//         converts them: (v / 255)^2.2 for colour, v / 255 for alpha);
//   .exr  OpenEXR scanline images, uncompressed or RLE / ZIPS / ZIP
//         compressed (HALF or FLOAT R, G, B and optional A channels; PIZ,
//         PXR24, B44 and DWA are reported as unsupported);
//   .jpg  sequential Huffman-coded JPEG (baseline or extended, grey or YCbCr,
//         any sampling factors, restart intervals), converted like .png;
//         progressive and arithmetic-coded files are reported as unsupported;
// all returned as RGBA floats, alpha 1, first row = top of the image, as
// util::BitmapTexture holds them.  Other formats are reported as unsupported.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace Pupil::util {

bool LoadImageRGBA(const std::string &path, std::vector<float> &rgba, uint32_t &width, uint32_t &height,
                   std::string &error);

// OpenEXR, scanline, uncompressed, channels A B G R as 32-bit floats, one
// scanline per block (the headless counterpart of the GUI's image save,
// framework/util/texture.cpp SaveExr).  rgba: width*height*4, first row = top.
bool SaveExrRGBA(const std::string &path, const float *rgba, uint32_t width, uint32_t height, std::string &error);

}  // namespace Pupil::util
