// image.cpp -- Radiance RGBE, PFM, PNG and OpenEXR (uncompressed, RLE, ZIP)
// readers, OpenEXR writer (see image.h).
#include "image.h"
#include "inflate.h"
#include "jpeg.h"

#include <algorithm>
#include <cstdint>
#include <cctype>
#include <cmath>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>

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

// Image sizes a reader accepts before it allocates: at most 65,536 pixels on
// a side and 2^28 pixels (4 GiB of RGBA floats), so that a corrupt or hostile
// header cannot ask for more.
bool size_ok(uint64_t w, uint64_t h, std::string &error) {
    if (w == 0 || h == 0 || w > 65536 || h > 65536 || w * h > (1ull << 28)) {
        error = "image size " + std::to_string(w) + " x " + std::to_string(h) + " out of range";
        return false;
    }
    return true;
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
    if (!size_ok((uint64_t)ww, (uint64_t)hh, error)) return false;
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
    if (!size_ok((uint64_t)ww, (uint64_t)hh, error)) return false;
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

// ---- PNG -------------------------------------------------------------------
// Per the PNG specification (ISO/IEC 15948): 8-byte signature, chunks of
// (big-endian length, type, data, CRC-32); IHDR, PLTE, tRNS, IDAT (one zlib
// stream over all IDAT chunks), IEND.  Scanlines carry a filter byte (None,
// Sub, Up, Average, Paeth); interlaced images come as the seven Adam7 passes.

uint32_t be32(const uint8_t *p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }

uint32_t crc32(const uint8_t *p, size_t n) {  // the CRC of the PNG specification (polynomial 0xEDB88320)
    static uint32_t table[256];
    static bool init = false;
    if (!init) {
        for (uint32_t i = 0; i < 256; i++) {
            uint32_t c = i;
            for (int k = 0; k < 8; k++) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            table[i] = c;
        }
        init = true;
    }
    uint32_t c = 0xffffffffu;
    for (size_t i = 0; i < n; i++) c = table[(c ^ p[i]) & 0xff] ^ (c >> 8);
    return c ^ 0xffffffffu;
}

uint8_t paeth(uint8_t a, uint8_t b, uint8_t c) {
    const int p = (int)a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    return (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
}

// Reverses the filters of `rows` scanlines of `line` bytes (each preceded by
// its filter type byte) in place; bpp = bytes per complete pixel (>= 1).
bool unfilter(uint8_t *data, size_t rows, size_t line, size_t bpp, std::string &error) {
    std::vector<uint8_t> prev(line, 0);
    for (size_t r = 0; r < rows; r++) {
        uint8_t *row = data + r * (line + 1);
        const uint8_t f = row[0];
        uint8_t *x = row + 1;
        for (size_t i = 0; i < line; i++) {
            const uint8_t a = i >= bpp ? x[i - bpp] : 0, b = prev[i], c = i >= bpp ? prev[i - bpp] : 0;
            switch (f) {
                case 0: break;
                case 1: x[i] = static_cast<uint8_t>(x[i] + a); break;
                case 2: x[i] = static_cast<uint8_t>(x[i] + b); break;
                case 3: x[i] = static_cast<uint8_t>(x[i] + ((a + b) >> 1)); break;
                case 4: x[i] = static_cast<uint8_t>(x[i] + paeth(a, b, c)); break;
                default: error = "PNG: unknown filter type"; return false;
            }
        }
        std::copy(x, x + line, prev.begin());
    }
    return true;
}

// PNG -> 8-bit samples with `comp` channels per pixel, as an 8-bit image load
// delivers them: grey 1, grey + alpha 2, RGB 3, RGBA 4, palette 3 (4 with a
// tRNS chunk); 16-bit samples keep their high byte, grey samples of 1, 2 or 4
// bits are scaled to 0..255.
bool decode_png(const std::vector<uint8_t> &d, std::vector<uint8_t> &img, uint32_t &w, uint32_t &h, int &comp,
                std::string &error) {
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (d.size() < 8 || std::memcmp(d.data(), sig, 8) != 0) {
        error = "not a PNG file";
        return false;
    }
    uint32_t depth = 0, ctype = 0, interlace = 0;
    std::vector<uint8_t> idat, plte, trns;
    bool have_ihdr = false, have_iend = false;
    size_t p = 8;
    while (p + 12 <= d.size() && !have_iend) {
        const uint32_t len = be32(&d[p]);
        if (len > d.size() - p - 12) {
            error = "PNG: chunk runs past the end of the file";
            return false;
        }
        const uint8_t *type = &d[p + 4], *body = &d[p + 8];
        if (crc32(type, 4 + (size_t)len) != be32(body + len)) {
            error = "PNG: chunk CRC mismatch";
            return false;
        }
        const std::string t(reinterpret_cast<const char *>(type), 4);
        if (t == "IHDR") {
            if (len != 13) {
                error = "PNG: bad IHDR";
                return false;
            }
            w = be32(body);
            h = be32(body + 4);
            depth = body[8];
            ctype = body[9];
            interlace = body[12];
            if (body[10] != 0 || body[11] != 0 || interlace > 1) {
                error = "PNG: unknown compression, filter or interlace method";
                return false;
            }
            have_ihdr = true;
        } else if (t == "PLTE") {
            plte.assign(body, body + len);
        } else if (t == "tRNS") {
            trns.assign(body, body + len);
        } else if (t == "IDAT") {
            idat.insert(idat.end(), body, body + len);
        } else if (t == "IEND") {
            have_iend = true;
        } else if (!(type[0] & 0x20)) {
            error = "PNG: unknown critical chunk " + t;
            return false;
        }
        p += 12 + (size_t)len;
    }
    if (!have_ihdr || idat.empty()) {
        error = "PNG: IHDR or image data missing";
        return false;
    }
    const int chans = ctype == 0 ? 1 : ctype == 2 ? 3 : ctype == 3 ? 1 : ctype == 4 ? 2 : ctype == 6 ? 4 : 0;
    const bool depth_ok = ctype == 0   ? (depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16)
                          : ctype == 3 ? (depth == 1 || depth == 2 || depth == 4 || depth == 8)
                                       : (depth == 8 || depth == 16);
    if (!chans || !depth_ok) {
        error = "PNG: unsupported colour type or bit depth";
        return false;
    }
    if (!size_ok(w, h, error)) return false;
    if (ctype == 3 && (plte.empty() || plte.size() % 3)) {
        error = "PNG: palette missing";
        return false;
    }
    comp = ctype == 3 ? (trns.empty() ? 3 : 4) : chans;
    const size_t bits_px = (size_t)chans * depth, bpp = std::max<size_t>(1, bits_px / 8);
    struct Pass { uint32_t x0, y0, dx, dy; };
    const Pass adam7[7] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4}, {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
    const Pass whole = {0, 0, 1, 1};
    const int npass = interlace ? 7 : 1;
    size_t total = 0;
    for (int k = 0; k < npass; k++) {
        const Pass &ps = interlace ? adam7[k] : whole;
        const size_t pw = w > ps.x0 ? (w - ps.x0 + ps.dx - 1) / ps.dx : 0, ph = h > ps.y0 ? (h - ps.y0 + ps.dy - 1) / ps.dy : 0;
        if (pw && ph) total += ph * ((pw * bits_px + 7) / 8 + 1);
    }
    std::vector<uint8_t> raw;
    if (!ZlibInflate(idat.data(), idat.size(), raw, total, error)) {
        error = "PNG: " + error;
        return false;
    }
    if (raw.size() != total) {
        error = "PNG: image data of the wrong size";
        return false;
    }
    img.assign((size_t)w * h * comp, 0);
    size_t off = 0;
    for (int k = 0; k < npass; k++) {
        const Pass &ps = interlace ? adam7[k] : whole;
        const size_t pw = w > ps.x0 ? (w - ps.x0 + ps.dx - 1) / ps.dx : 0, ph = h > ps.y0 ? (h - ps.y0 + ps.dy - 1) / ps.dy : 0;
        if (!pw || !ph) continue;
        const size_t line = (pw * bits_px + 7) / 8;
        if (!unfilter(raw.data() + off, ph, line, bpp, error)) return false;
        for (size_t y = 0; y < ph; y++) {
            const uint8_t *row = raw.data() + off + y * (line + 1) + 1;
            for (size_t x = 0; x < pw; x++) {
                uint8_t *dst = img.data() + ((size_t)(ps.y0 + y * ps.dy) * w + ps.x0 + x * ps.dx) * comp;
                if (depth < 8) {  // one sample per pixel (grey or palette index), packed high bits first
                    const size_t bit = x * depth;
                    const uint32_t v = (row[bit / 8] >> (8 - depth - bit % 8)) & ((1u << depth) - 1);
                    if (ctype == 3) {
                        if (3 * v + 2 >= plte.size()) { error = "PNG: palette index out of range"; return false; }
                        for (int c = 0; c < 3; c++) dst[c] = plte[3 * v + c];
                        if (comp == 4) dst[3] = v < trns.size() ? trns[v] : 255;
                    } else {
                        dst[0] = static_cast<uint8_t>(v * (255u / ((1u << depth) - 1)));
                    }
                } else if (ctype == 3) {
                    const uint32_t v = row[x];
                    if (3 * v + 2 >= plte.size()) { error = "PNG: palette index out of range"; return false; }
                    for (int c = 0; c < 3; c++) dst[c] = plte[3 * v + c];
                    if (comp == 4) dst[3] = v < trns.size() ? trns[v] : 255;
                } else {
                    const size_t step = depth / 8;  // 16-bit samples: the high (first) byte
                    for (int c = 0; c < chans; c++) dst[c] = row[(x * chans + c) * step];
                }
            }
        }
        off += ph * (line + 1);
    }
    return true;
}

// util::BitmapTexture from an 8-bit image as the reference fills it
// (framework/util/texture.cpp:106-118): for every `c` samples, R, G, B =
// (sample / 255)^2.2 of the first three bytes from there and A = the fourth
// byte / 255 for 4-channel images, else 1.  With fewer than 3 channels the
// reference reads the bytes that follow (the next samples; past the last one
// its buffer ends, read here as 0).
void rgba_from_8bit(const std::vector<uint8_t> &img, int c, uint32_t w, uint32_t h, std::vector<float> &rgba) {
    const size_t size = img.size();
    auto at = [&](size_t i) -> float { return i < size ? static_cast<float>(img[i]) : 0.f; };
    rgba.assign(4ull * w * h, 0.f);
    size_t j = 0;
    for (size_t i = 0; i < size; i += (size_t)c) {
        rgba[j++] = std::pow(at(i) * 1.f / 255.f, 2.2f);
        rgba[j++] = std::pow(at(i + 1) * 1.f / 255.f, 2.2f);
        rgba[j++] = std::pow(at(i + 2) * 1.f / 255.f, 2.2f);
        rgba[j++] = c == 4 ? at(i + 3) * 1.f / 255.f : 1.f;
    }
}

bool load_png(const std::vector<uint8_t> &d, std::vector<float> &rgba, uint32_t &w, uint32_t &h, std::string &error) {
    std::vector<uint8_t> img;
    int c = 0;
    if (!decode_png(d, img, w, h, c, error)) return false;
    rgba_from_8bit(img, c, w, h, rgba);
    return true;
}

bool load_jpeg(const std::vector<uint8_t> &d, std::vector<float> &rgba, uint32_t &w, uint32_t &h, std::string &error) {
    std::vector<uint8_t> img;
    int c = 0;
    if (!DecodeJpeg(d, img, w, h, c, error)) return false;
    rgba_from_8bit(img, c, w, h, rgba);
    return true;
}

// ---- OpenEXR (scanline; NO, RLE, ZIPS, ZIP compression) --------------------
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
                if (p + 16 > end) {
                    error = "OpenEXR channel list truncated";
                    return false;
                }
                c.type = get_u32(d, p);
                p += 16;  // type, pLinear + 3 reserved, xSampling, ySampling
                chans.push_back(c);
            }
        } else if (name == "compression" && size >= 1) {
            compression = d[p];
        } else if (name == "dataWindow" && size >= 16) {
            xmin = static_cast<int32_t>(get_u32(d, p));
            ymin = static_cast<int32_t>(get_u32(d, p + 4));
            xmax = static_cast<int32_t>(get_u32(d, p + 8));
            ymax = static_cast<int32_t>(get_u32(d, p + 12));
        }
        p = end;
    }
    // 0 NO_COMPRESSION, 1 RLE, 2 ZIPS (one scanline per block), 3 ZIP (16)
    if (compression < 0 || compression > 3) {
        error = "OpenEXR compression " + std::to_string(compression) +
                " is not supported (PIZ, PXR24, B44 and DWA are not; NO, RLE, ZIPS and ZIP are)";
        return false;
    }
    if (xmax < xmin || ymax < ymin) {
        error = "OpenEXR data window empty";
        return false;
    }
    if (!size_ok((uint64_t)((int64_t)xmax - xmin + 1), (uint64_t)((int64_t)ymax - ymin + 1), error)) return false;
    w = static_cast<uint32_t>((int64_t)xmax - xmin + 1);
    h = static_cast<uint32_t>((int64_t)ymax - ymin + 1);
    size_t line_bytes = 0;
    for (auto &c : chans) {
        if (c.type != 1 && c.type != 2) {
            error = "OpenEXR channel '" + c.name + "' is neither HALF nor FLOAT";
            return false;
        }
        line_bytes += (c.type == 1 ? 2 : 4) * (size_t)w;
    }
    const size_t table = p;
    const uint32_t lines_per_block = compression == 3 ? 16u : 1u;
    const size_t nblocks = (h + lines_per_block - 1) / lines_per_block;
    if (table + 8ull * nblocks > d.size()) {
        error = "OpenEXR offset table truncated";
        return false;
    }
    rgba.assign(4ull * w * h, 0.f);
    for (size_t i = 0; i < (size_t)w * h; i++) rgba[4 * i + 3] = 1.f;
    std::vector<uint8_t> tmp, unpacked;
    for (size_t blk = 0; blk < nblocks; blk++) {
        const uint64_t off = get_u64(d, table + 8ull * blk);
        if (off + 8 > d.size()) {
            error = "OpenEXR block out of range";
            return false;
        }
        const int64_t y0 = (int64_t)static_cast<int32_t>(get_u32(d, off)) - ymin;
        const uint32_t packed = get_u32(d, off + 4);
        if (y0 < 0 || y0 >= (int64_t)h || y0 % (int64_t)lines_per_block || off + 8 + packed > d.size()) {
            error = "OpenEXR block malformed";
            return false;
        }
        const uint32_t nlines = std::min<uint32_t>(lines_per_block, h - (uint32_t)y0);
        const size_t expect = (size_t)nlines * line_bytes;
        const uint8_t *src = &d[off + 8];
        if (packed != expect) {  // compressed block (a block that would not shrink is stored as is)
            if (compression == 0 || packed > expect) {
                error = "OpenEXR block of the wrong size";
                return false;
            }
            tmp.clear();
            if (compression == 1) {  // run-length: count < 0 -> -count literal bytes, else count + 1 copies
                size_t q = 0;
                while (q < packed && tmp.size() < expect) {
                    const int cnt = static_cast<int8_t>(src[q++]);
                    if (cnt < 0) {
                        if (q + (size_t)(-cnt) > packed) break;
                        tmp.insert(tmp.end(), src + q, src + q + (-cnt));
                        q += (size_t)(-cnt);
                    } else {
                        if (q >= packed) break;
                        tmp.insert(tmp.end(), (size_t)cnt + 1, src[q++]);
                    }
                }
            } else if (!ZlibInflate(src, packed, tmp, expect, error)) {
                error = "OpenEXR: " + error;
                return false;
            }
            if (tmp.size() != expect) {
                error = "OpenEXR: a compressed block unpacks to the wrong size";
                return false;
            }
            // undo the byte predictor, then the split into even / odd bytes
            for (size_t i = 1; i < tmp.size(); i++) tmp[i] = static_cast<uint8_t>(tmp[i - 1] + tmp[i] - 128);
            unpacked.resize(expect);
            const size_t half = (expect + 1) / 2;
            for (size_t i = 0; i < expect; i++) unpacked[i] = (i & 1) ? tmp[half + i / 2] : tmp[i / 2];
            src = unpacked.data();
        }
        for (uint32_t l = 0; l < nlines; l++) {
            const uint32_t y = (uint32_t)y0 + l;
            const uint8_t *q = src + (size_t)l * line_bytes;
            for (auto &c : chans) {
                const int ch = c.name == "R" ? 0 : c.name == "G" ? 1 : c.name == "B" ? 2 : c.name == "A" ? 3 : -1;
                for (uint32_t x = 0; x < w; x++) {
                    float v;
                    if (c.type == 1) {
                        v = half_to_float(static_cast<uint16_t>(q[0] | (q[1] << 8)));
                        q += 2;
                    } else {
                        uint32_t u = (uint32_t)q[0] | (uint32_t)q[1] << 8 | (uint32_t)q[2] << 16 | (uint32_t)q[3] << 24;
                        std::memcpy(&v, &u, 4);
                        q += 4;
                    }
                    if (ch >= 0) rgba[4 * ((size_t)y * w + x) + ch] = v;
                }
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
    const bool jpeg = ext == "jpg" || ext == "jpeg";
    if (ext != "hdr" && ext != "pfm" && ext != "exr" && ext != "png" && !jpeg) {
        error = "image '" + path + "': only .hdr (RGBE), .pfm, .png, sequential .jpg and .exr (uncompressed, RLE, "
                "ZIP) images can be read";
        return false;
    }
    bool ok = false;
    try {  // a reader that cannot allocate reports it instead of throwing through the C interface
        std::vector<uint8_t> data;
        if (!read_all(path, data, error)) return false;
        ok = ext == "hdr"   ? load_hdr(data, rgba, width, height, error)
             : ext == "exr" ? load_exr(data, rgba, width, height, error)
             : ext == "png" ? load_png(data, rgba, width, height, error)
             : jpeg         ? load_jpeg(data, rgba, width, height, error)
                            : load_pfm(data, rgba, width, height, error);
    } catch (const std::exception &e) {
        error = std::string("out of memory (") + e.what() + ")";
        ok = false;
    }
    if (!ok) {
        rgba.clear();
        error = "image '" + path + "': " + error;
    }
    return ok;
}

}  // namespace Pupil::util
