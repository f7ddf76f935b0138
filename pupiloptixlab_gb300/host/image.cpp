// image.cpp -- Radiance RGBE and PFM readers (see image.h).
#include "image.h"

#include <algorithm>
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

}  // namespace

bool LoadImageRGBA(const std::string &path, std::vector<float> &rgba, uint32_t &width, uint32_t &height,
                   std::string &error) {
    const std::string ext = lower_ext(path);
    if (ext != "hdr" && ext != "pfm") {
        error = "image '" + path + "': only .hdr (RGBE) and .pfm images can be read";
        return false;
    }
    std::vector<uint8_t> data;
    if (!read_all(path, data, error)) return false;
    const bool ok = ext == "hdr" ? load_hdr(data, rgba, width, height, error) : load_pfm(data, rgba, width, height, error);
    if (!ok) error = "image '" + path + "': " + error;
    return ok;
}

}  // namespace Pupil::util
