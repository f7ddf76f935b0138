// hair.cpp -- Cem Yuksel's HAIR files and the curve segments built from them.
//
// File layout (the published HAIR format, read as
// framework/resource/hair/cemyuksel_hair.cpp does): a 128-byte header
//   0 "HAIR"  4 strands (u32)  8 points (u32)  12 flags (u32)
//   16 default segments (u32)  20 default thickness (f32)
//   24 default transparency (f32)  28 default colour (3 f32)  40 info (88 chars)
// then, present by flag bit, the arrays: 0 segments per strand (u16),
// 1 points (3 f32 each), 2 thickness per point (f32), 3 transparency,
// 4 colour.  A strand of s segments holds s + 1 points.
//
// Radii and segments follow ShapeManager::LoadHair
// (framework/resource/shape.cpp:369-420): the file thickness is the radius
// unless the scene gives one; tapered strands fall linearly from the radius
// to zero at the tip; every strand contributes the segments starting at its
// points up to its point count minus the curve degree.  Multi-byte values are
// little-endian, as the format stores them.
#include <cstring>
#include <fstream>

#include "scene.h"

namespace Pupil::resource {

namespace {
uint32_t le32(const unsigned char *p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
float lef32(const unsigned char *p) {
    uint32_t u = le32(p);
    float f;
    memcpy(&f, &u, 4);
    return f;
}
bool read_floats(std::ifstream &in, std::vector<float> &out, size_t n) {
    std::vector<unsigned char> raw(4 * n);
    if (n && !in.read(reinterpret_cast<char *>(raw.data()), (std::streamsize)raw.size())) return false;
    out.resize(n);
    for (size_t i = 0; i < n; i++) out[i] = lef32(raw.data() + 4 * i);
    return true;
}
}  // namespace

bool LoadCyHair(const std::string &path, float radius, bool tapered, uint32_t mode, Curves &out, std::string &error) {
    std::ifstream in(path, std::ios::binary);
    if (!in) {
        error = "cannot open hair file " + path;
        return false;
    }
    unsigned char h[128];
    if (!in.read(reinterpret_cast<char *>(h), 128)) {
        error = path + ": truncated HAIR header";
        return false;
    }
    if (memcmp(h, "HAIR", 4) != 0) {
        error = path + ": not a HAIR file";
        return false;
    }
    const uint32_t strands = le32(h + 4), points = le32(h + 8), flags = le32(h + 12), def_segments = le32(h + 16);
    const float def_thickness = lef32(h + 20);
    if (mode > PT_CURVE_CATMULL_ROM) {
        error = "unknown spline mode";
        return false;
    }
    // every array the flags announce must fit in the file before anything is
    // allocated for it, so that a corrupt count cannot ask for gigabytes
    in.seekg(0, std::ios::end);
    const uint64_t file_bytes = static_cast<uint64_t>(in.tellg());
    in.seekg(128, std::ios::beg);
    const uint64_t body = file_bytes > 128 ? file_bytes - 128 : 0;
    const uint64_t seg_bytes = (flags & 1u) ? 2ull * strands : 0;
    if (seg_bytes > body) {
        error = path + ": truncated segment array";
        return false;
    }
    if (!(flags & 2u)) {
        error = path + ": HAIR file has no points";
        return false;
    }
    if (12ull * points > body - seg_bytes) {
        error = path + ": truncated point array";
        return false;
    }
    if ((flags & 4u) && 4ull * points > body - seg_bytes - 12ull * points) {
        error = path + ": truncated thickness array";
        return false;
    }
    if (strands > points) {  // every strand holds at least one point
        error = path + ": strands need more points than the file holds";
        return false;
    }
    std::vector<uint32_t> segs(strands, def_segments);
    if (flags & 1u) {
        std::vector<unsigned char> raw(2ull * strands);
        if (strands && !in.read(reinterpret_cast<char *>(raw.data()), (std::streamsize)raw.size())) {
            error = path + ": truncated segment array";
            return false;
        }
        for (uint32_t i = 0; i < strands; i++) segs[i] = (uint32_t)raw[2 * i] | ((uint32_t)raw[2 * i + 1] << 8);
    }
    // strand i holds points [first[i], first[i + 1])
    std::vector<uint64_t> first(strands + 1, 0);
    for (uint32_t i = 0; i < strands; i++) first[i + 1] = first[i] + 1 + segs[i];
    if (first[strands] > points) {
        error = path + ": strands need more points than the file holds";
        return false;
    }
    if (!read_floats(in, out.positions, 3ull * points)) {
        error = path + ": truncated point array";
        return false;
    }
    if (flags & 4u) {
        if (!read_floats(in, out.radii, points)) {
            error = path + ": truncated thickness array";
            return false;
        }
    } else {
        out.radii.assign(points, def_thickness);
    }
    if (tapered) {
        const float w = radius == 0.f && points ? out.radii[0] : radius;
        for (uint32_t i = 0; i < strands; i++) {
            const uint32_t start = (uint32_t)first[i], num = (uint32_t)(first[i + 1] - first[i]);
            for (uint32_t k = 0; k < num; k++)
                out.radii[start + k] = num > 1 ? w * (float)(num - 1 - k) / static_cast<float>(num - 1) : w;
        }
    } else if (radius != 0.f) {
        for (float &r : out.radii) r = radius;
    }
    const int64_t degree = mode > 2 ? 3 : mode + 1;
    out.segments.clear();
    for (uint32_t i = 0; i < strands; i++) {
        const int64_t start = (int64_t)first[i], end = (int64_t)first[i + 1] - degree;
        for (int64_t s = start; s < end; s++) out.segments.push_back((uint32_t)s);
    }
    out.type = mode;
    return true;
}

}  // namespace Pupil::resource
