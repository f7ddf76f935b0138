// image.cpp -- Radiance RGBE, PFM and uncompressed OpenEXR readers, OpenEXR
// writer (see image.h).
#include "image.h"

#include <algorithm>
#include <cstdint>
#include <cctype>
#include <cmath>
#include <cstring>
#include <fstream>
#include <sstream>

namespace Pupil::util {

namespace {

std::string lower_ext(const std::string &path) {
    auto dot = path.find_last_of('.');
    std::string e = dot == std::string::npos ? "" : path.substr(dot + 1);
    for (auto &c : e) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
    return e;
}

bool read_all(const std::string &path, std::vector<uint8_t> &data, std::string &error) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        error = "cannot open image '" + path + "'";
        return false;
    }
    data.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    return true;
}

// RGBE pixel -> float RGB
void rgbe(const uint8_t *p, float *out) {
    if (p[3] == 0) {
        out[0] = out[1] = out[2] = 0.f;
        return;
    }
    const float f = std::ldexp(1.0f, static_cast<int>(p[3]) - 136);
    out[0] = p[0] * f;
    out[1] = p[1] * f;
    out[2] = p[2] * f;
}

bool load_hdr(const std::vector<uint8_t> &d, std::vector<float> &rgba, uint32_t &w, uint32_t &h, std::string &error) {
    size_t pos = 0;
    auto line = [&](std::string &s) {
        s.clear();
        while (pos < d.size() && d[pos] != '\n') s.push_back(static_cast<char>(d[pos++]));
        if (pos < d.size()) pos++;
        return pos <= d.size();
    };
    std::string s;
    line(s);
    if (s.rfind("#?", 0) != 0) {
        error = "not a Radiance HDR file";
        return false;
    }
    bool rgbe_format = false;
    while (line(s) && !s.empty())
        if (s == "FORMAT=32-bit_rle_rgbe") rgbe_format = true;
    if (!rgbe_format) {
        error = "HDR file is not in the 32-bit RLE RGBE format";
        return false;
    }
    line(s);
    char ya[3] = {0}, xa[3] = {0};
    int hh = 0, ww = 0;
    if (std::sscanf(s.c_str(), "%2s %d %2s %d", ya, &hh, xa, &ww) != 4 || std::strcmp(ya, "-Y") != 0 ||
        std::strcmp(xa, "+X") != 0 || hh <= 0 || ww <= 0) {
        error = "HDR file: only the '-Y h +X w' orientation is supported";
        return false;
    }
    w = static_cast<uint32_t>(ww);
    h = static_cast<uint32_t>(hh);
    rgba.assign(4ull * w * h, 1.f);
    std::vector<uint8_t> scan(4ull * w);
    for (uint32_t y = 0; y < h; y++) {
        if (pos + 4 > d.size()) {
            error = "HDR file truncated";
            return false;
        }
        const bool rle = w >= 8 && w < 32768 && d[pos] == 2 && d[pos + 1] == 2 && ((d[pos + 2] << 8) | d[pos + 3]) == (int)w;
        if (rle) {
            pos += 4;
            for (int c = 0; c < 4; c++) {
                uint32_t x = 0;
                while (x < w) {
                    if (pos >= d.size()) {
                        error = "HDR file truncated";
                        return false;
                    }
                    uint32_t n = d[pos++];
                    if (n > 128) {  // run
                        n -= 128;
                        if (n > w - x || pos >= d.size()) {
                            error = "HDR file: bad run length";
                            return false;
                        }
                        const uint8_t v = d[pos++];
                        for (uint32_t k = 0; k < n; k++) scan[4 * (x++) + c] = v;
                    } else {  // literal
                        if (n == 0 || n > w - x || pos + n > d.size()) {
                            error = "HDR file: bad literal length";
                            return false;
                        }
                        for (uint32_t k = 0; k < n; k++) scan[4 * (x++) + c] = d[pos++];
                    }
                }
            }
        } else {  // flat scanline
            if (pos + 4ull * w > d.size()) {
                error = "HDR file truncated";
                return false;
            }
            std::memcpy(scan.data(), d.data() + pos, 4ull * w);
            pos += 4ull * w;
        }
        for (uint32_t x = 0; x < w; x++) rgbe(&scan[4 * x], &rgba[4 * ((size_t)y * w + x)]);
    }
    return true;
}

bool load_pfm(const std::vector<uint8_t> &d, std::vector<float> &rgba, uint32_t &w, uint32_t &h, std::string &error) {
    size_t pos = 0;
    auto token = [&]() {
        std::string t;
        while (pos < d.size() && std::isspace(d[pos])) pos++;
        while (pos < d.size() && !std::isspace(d[pos])) t.push_back(static_cast<char>(d[pos++]));
        return t;
    };
    const std::string magic = token();
    const int channels = magic == "PF" ? 3 : magic == "Pf" ? 1 : 0;
    if (!channels) {
        error = "not a PFM file";
        return false;
    }
    const long ww = std::atol(token().c_str()), hh = std::atol(token().c_str());
    const double scale = std::atof(token().c_str());
    pos++;  // the single whitespace byte before the raster
    if (ww <= 0 || hh <= 0 || scale == 0.0) {
        error = "PFM header invalid";
        return false;
    }
    w = static_cast<uint32_t>(ww);
    h = static_cast<uint32_t>(hh);
    const size_t n = (size_t)w * h * channels;
    if (pos + 4 * n > d.size()) {
        error = "PFM file truncated";
        return false;
    }
    const bool little = scale < 0;
    const uint16_t probe = 1;
    const bool host_little = *reinterpret_cast<const uint8_t *>(&probe) == 1;
    rgba.assign(4ull * w * h, 1.f);
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++)
            for (int c = 0; c < channels; c++) {
                uint8_t b[4];
                std::memcpy(b, d.data() + pos + 4 * (((size_t)y * w + x) * channels + c), 4);
                if (little != host_little) std::swap(b[0], b[3]), std::swap(b[1], b[2]);
                float v;
                std::memcpy(&v, b, 4);
                const uint32_t row = h - 1 - y;  // file rows run bottom-up
                float *o = &rgba[4 * ((size_t)row * w + x)];
                if (channels == 1) o[0] = o[1] = o[2] = v;
                else o[c] = v;
            }
    return true;
}

// ---- OpenEXR (scanline, NO_COMPRESSION) ----------------------------------
// Layout per the OpenEXR file format description: magic 20000630, version 2,
// header = attributes (name\0 type\0 int32 size, value) ending with \0, a
// table of uint64 offsets (one per scanline block), then blocks of
// (int32 y, int32 byte count, channel data in the header's channel order).

void put_u32(std::vector<uint8_t> &b, uint32_t v) {
    for (int i = 0; i < 4; i++) b.push_back(static_cast<uint8_t>(v >> (8 * i)));
}
void put_u64(std::vector<uint8_t> &b, uint64_t v) {
    for (int i = 0; i < 8; i++) b.push_back(static_cast<uint8_t>(v >> (8 * i)));
}
void put_f32(std::vector<uint8_t> &b, float f) {
    uint32_t v;
    std::memcpy(&v, &f, 4);
    put_u32(b, v);
}
void put_str(std::vector<uint8_t> &b, const char *s) {
    while (*s) b.push_back(static_cast<uint8_t>(*s++));
    b.push_back(0);
}
void attr(std::vector<uint8_t> &b, const char *name, const char *type, const std::vector<uint8_t> &value) {
    put_str(b, name);
    put_str(b, type);
    put_u32(b, static_cast<uint32_t>(value.size()));
    b.insert(b.end(), value.begin(), value.end());
}

uint32_t get_u32(const std::vector<uint8_t> &d, size_t p) {
    return d[p] | (d[p + 1] << 8) | (d[p + 2] << 16) | (static_cast<uint32_t>(d[p + 3]) << 24);
}
uint64_t get_u64(const std::vector<uint8_t> &d, size_t p) { return get_u32(d, p) | (uint64_t)get_u32(d, p + 4) << 32; }

float half_to_float(uint16_t h) {  // IEEE 754 binary16
    const uint32_t sign = (h >> 15) & 1, e = (h >> 10) & 31, m = h & 1023;
    float v;
    if (e == 0) v = std::ldexp(static_cast<float>(m), -24);
    else if (e == 31) v = m ? NAN : INFINITY;
    else v = std::ldexp(static_cast<float>(m | 1024), static_cast<int>(e) - 25);
    return sign ? -v : v;
}

bool load_exr(const std::vector<uint8_t> &d, std::vector<float> &rgba, uint32_t &w, uint32_t &h, std::string &error) {
    if (d.size() < 8 || get_u32(d, 0) != 20000630u) {
        error = "not an OpenEXR file";
        return false;
    }
    if ((get_u32(d, 4) & 0xff) != 2 || (get_u32(d, 4) & 0x200)) {
        error = "only single-part scanline OpenEXR files are supported";
        return false;
    }
    struct Chan {
        std::string name;
        uint32_t type;
    };
    std::vector<Chan> chans;
    int32_t xmin = 0, ymin = 0, xmax = -1, ymax = -1;
    int compression = -1;
    size_t p = 8;
    auto cstr = [&](std::string &out) {
        out.clear();
        while (p < d.size() && d[p]) out.push_back(static_cast<char>(d[p++]));
        p++;
        return p <= d.size();
    };
    for (;;) {
        std::string name, type;
        if (p >= d.size()) {
            error = "OpenEXR header truncated";
            return false;
        }
        if (d[p] == 0) {
            p++;
            break;
        }
        cstr(name);
        cstr(type);
        if (p + 4 > d.size()) {
            error = "OpenEXR header truncated";
            return false;
        }
        const uint32_t size = get_u32(d, p);
        p += 4;
        if (p + size > d.size()) {
            error = "OpenEXR header truncated";
            return false;
        }
        const size_t end = p + size;
        if (name == "channels") {
            while (p < end && d[p]) {
                Chan c;
                cstr(c.name);
                c.type = get_u32(d, p);
                p += 16;  // type, pLinear + 3 reserved, xSampling, ySampling
                chans.push_back(c);
            }
        } else if (name == "compression") {
            compression = d[p];
        } else if (name == "dataWindow") {
            xmin = static_cast<int32_t>(get_u32(d, p));
            ymin = static_cast<int32_t>(get_u32(d, p + 4));
            xmax = static_cast<int32_t>(get_u32(d, p + 8));
            ymax = static_cast<int32_t>(get_u32(d, p + 12));
        }
        p = end;
    }
    if (compression != 0) {
        error = "compressed OpenEXR files are not supported (only NO_COMPRESSION)";
        return false;
    }
    if (xmax < xmin || ymax < ymin) {
        error = "OpenEXR data window empty";
        return false;
    }
    w = static_cast<uint32_t>(xmax - xmin + 1);
    h = static_cast<uint32_t>(ymax - ymin + 1);
    size_t line_bytes = 0;
    for (auto &c : chans) {
        if (c.type != 1 && c.type != 2) {
            error = "OpenEXR channel '" + c.name + "' is neither HALF nor FLOAT";
            return false;
        }
        line_bytes += (c.type == 1 ? 2 : 4) * (size_t)w;
    }
    rgba.assign(4ull * w * h, 0.f);
    for (size_t i = 0; i < (size_t)w * h; i++) rgba[4 * i + 3] = 1.f;
    const size_t table = p;
    if (table + 8ull * h > d.size()) {
        error = "OpenEXR offset table truncated";
        return false;
    }
    for (uint32_t line = 0; line < h; line++) {
        const uint64_t off = get_u64(d, table + 8ull * line);
        if (off + 8 + line_bytes > d.size()) {
            error = "OpenEXR scanline out of range";
            return false;
        }
        const int32_t y = static_cast<int32_t>(get_u32(d, off)) - ymin;
        if (y < 0 || y >= static_cast<int32_t>(h) || get_u32(d, off + 4) != line_bytes) {
            error = "OpenEXR scanline block malformed";
            return false;
        }
        size_t q = off + 8;
        for (auto &c : chans) {
            const int ch = c.name == "R" ? 0 : c.name == "G" ? 1 : c.name == "B" ? 2 : c.name == "A" ? 3 : -1;
            for (uint32_t x = 0; x < w; x++) {
                float v;
                if (c.type == 1) {
                    v = half_to_float(static_cast<uint16_t>(d[q] | (d[q + 1] << 8)));
                    q += 2;
                } else {
                    const uint32_t u = get_u32(d, q);
                    std::memcpy(&v, &u, 4);
                    q += 4;
                }
                if (ch >= 0) rgba[4 * ((size_t)y * w + x) + ch] = v;
            }
        }
    }
    return true;
}

}  // namespace

bool SaveExrRGBA(const std::string &path, const float *rgba, uint32_t width, uint32_t height, std::string &error) {
    std::vector<uint8_t> b, v;
    put_u32(b, 20000630u);
    put_u32(b, 2u);
    for (const char *c : {"A", "B", "G", "R"}) {  // channel list, sorted by name
        put_str(v, c);
        put_u32(v, 2u);          // FLOAT
        put_u32(v, 0u);          // pLinear + reserved
        put_u32(v, 1u);          // xSampling
        put_u32(v, 1u);          // ySampling
    }
    v.push_back(0);
    attr(b, "channels", "chlist", v);
    attr(b, "compression", "compression", {0});
    v.clear();
    put_u32(v, 0);
    put_u32(v, 0);
    put_u32(v, width - 1);
    put_u32(v, height - 1);
    attr(b, "dataWindow", "box2i", v);
    attr(b, "displayWindow", "box2i", v);
    attr(b, "lineOrder", "lineOrder", {0});
    v.clear();
    put_f32(v, 1.f);
    attr(b, "pixelAspectRatio", "float", v);
    v.clear();
    put_f32(v, 0.f);
    put_f32(v, 0.f);
    attr(b, "screenWindowCenter", "v2f", v);
    v.clear();
    put_f32(v, 1.f);
    attr(b, "screenWindowWidth", "float", v);
    b.push_back(0);  // end of header
    const uint64_t line_bytes = 4ull * 4 * width;
    const uint64_t first = b.size() + 8ull * height;
    for (uint32_t y = 0; y < height; y++) put_u64(b, first + y * (8 + line_bytes));
    for (uint32_t y = 0; y < height; y++) {
        put_u32(b, y);
        put_u32(b, static_cast<uint32_t>(line_bytes));
        for (int ch : {3, 2, 1, 0})  // A, B, G, R
            for (uint32_t x = 0; x < width; x++) put_f32(b, rgba[4 * ((size_t)y * width + x) + ch]);
    }
    std::ofstream f(path, std::ios::binary);
    if (!f) {
        error = "cannot write '" + path + "'";
        return false;
    }
    f.write(reinterpret_cast<const char *>(b.data()), static_cast<std::streamsize>(b.size()));
    return static_cast<bool>(f);
}

bool LoadImageRGBA(const std::string &path, std::vector<float> &rgba, uint32_t &width, uint32_t &height,
                   std::string &error) {
    const std::string ext = lower_ext(path);
    if (ext != "hdr" && ext != "pfm" && ext != "exr") {
        error = "image '" + path + "': only .hdr (RGBE), .pfm and uncompressed .exr images can be read";
        return false;
    }
    std::vector<uint8_t> data;
    if (!read_all(path, data, error)) return false;
    const bool ok = ext == "hdr"   ? load_hdr(data, rgba, width, height, error)
                    : ext == "exr" ? load_exr(data, rgba, width, height, error)
                                   : load_pfm(data, rgba, width, height, error);
    if (!ok) error = "image '" + path + "': " + error;
    return ok;
}

}  // namespace Pupil::util
