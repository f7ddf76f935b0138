// jpeg.cpp -- sequential (baseline and extended, Huffman-coded, 8-bit) JPEG
// decoding for the image reader, written from ITU-T T.81 / ISO/IEC 10918-1:
// markers (SOI, APPn, COM, DQT, SOF0/SOF1, DHT, DRI, SOS, RSTn, EOI), Huffman
// decoding of DC differences and AC run/size pairs with byte stuffing,
// dequantisation in zig-zag order, the 8x8 inverse DCT of the standard's
// defining formula (A.3.3) in double precision, level shift and clamping,
// chroma up-sampling by pixel replication, and the JFIF YCbCr -> RGB
// conversion.  Progressive and arithmetic-coded files are reported as
// unsupported.
#include "jpeg.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace Pupil::util {

namespace {

// zig-zag scan position -> natural (row-major) position in the 8x8 block
constexpr uint8_t kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                                 12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                                 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                                 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

struct HuffTable {
    bool defined = false;
    uint8_t counts[17] = {0};  // codes of each length 1..16
    uint8_t symbols[256] = {0};
    int mincode[17], maxcode[18], valptr[17];  // T.81 F.2.2.3 decoding procedure
    void build() {
        int code = 0, k = 0;
        for (int l = 1; l <= 16; l++) {
            valptr[l] = k;
            mincode[l] = code;
            code += counts[l];
            k += counts[l];
            maxcode[l] = counts[l] ? code - 1 : -1;
            code <<= 1;
        }
        maxcode[17] = 0x7fffffff;
        defined = true;
    }
};

struct Component {
    int id = 0, h = 1, v = 1, tq = 0, td = 0, ta = 0;
    int bw = 0, bh = 0;  // blocks across / down (padded to whole MCUs)
    std::vector<uint8_t> pix;  // bw*8 x bh*8 samples
    int pred = 0;
};

struct Reader {
    const uint8_t *d;
    size_t n, pos = 0;
    uint32_t bitbuf = 0;
    int bitcnt = 0;
    bool marker_hit = false;  // a marker ended the entropy-coded data
    int bit() {
        if (bitcnt == 0) {
            uint8_t b = 0;
            if (!marker_hit && pos < n) {
                b = d[pos];
                if (b == 0xFF) {
                    if (pos + 1 < n && d[pos + 1] == 0x00) {
                        pos += 2;  // stuffed byte
                    } else {
                        marker_hit = true;  // a marker: feed zeros from here
                        b = 0;
                    }
                } else {
                    pos++;
                }
            }
            bitbuf = b;
            bitcnt = 8;
        }
        bitcnt--;
        return (bitbuf >> bitcnt) & 1;
    }
    int receive(int s) {
        int v = 0;
        for (int i = 0; i < s; i++) v = (v << 1) | bit();
        return v;
    }
    void reset_bits() { bitcnt = 0; }
};

int extend(int v, int s) { return s == 0 ? 0 : (v < (1 << (s - 1)) ? v - (1 << s) + 1 : v); }

int decode_symbol(Reader &r, const HuffTable &t) {
    int code = r.bit();
    for (int l = 1; l <= 16; l++) {
        if (code <= t.maxcode[l] && t.maxcode[l] >= 0) return t.symbols[t.valptr[l] + code - t.mincode[l]];
        code = (code << 1) | r.bit();
    }
    return -1;
}

// 8x8 inverse DCT from the defining formula, separable, in double precision
void idct8x8(const int *coef, uint8_t *out, int stride) {
    static double cosv[8][8];
    static bool init = false;
    if (!init) {
        for (int x = 0; x < 8; x++)
            for (int u = 0; u < 8; u++) {
                const double cu = u == 0 ? std::sqrt(0.5) : 1.0;
                cosv[x][u] = cu * std::cos((2 * x + 1) * u * M_PI / 16.0);
            }
        init = true;
    }
    double tmp[64];
    for (int y = 0; y < 8; y++)  // rows: sum over v
        for (int u = 0; u < 8; u++) {
            double s = 0.0;
            for (int v = 0; v < 8; v++) s += cosv[y][v] * coef[v * 8 + u];
            tmp[y * 8 + u] = s;
        }
    for (int y = 0; y < 8; y++)
        for (int x = 0; x < 8; x++) {
            double s = 0.0;
            for (int u = 0; u < 8; u++) s += cosv[x][u] * tmp[y * 8 + u];
            const long v = std::lround(s / 4.0 + 128.0);
            out[y * stride + x] = static_cast<uint8_t>(v < 0 ? 0 : v > 255 ? 255 : v);
        }
}

uint16_t be16(const uint8_t *p) { return static_cast<uint16_t>((p[0] << 8) | p[1]); }

}  // namespace

bool DecodeJpeg(const std::vector<uint8_t> &d, std::vector<uint8_t> &img, uint32_t &w, uint32_t &h, int &comp,
                std::string &error) {
    if (d.size() < 4 || d[0] != 0xFF || d[1] != 0xD8) {
        error = "not a JPEG file";
        return false;
    }
    uint16_t qt[4][64] = {};
    bool qt_defined[4] = {false, false, false, false};
    HuffTable dc[4], ac[4];
    std::vector<Component> comps;
    int restart = 0;
    bool have_frame = false, done = false;
    size_t p = 2;
    while (p + 4 <= d.size() && !done) {
        if (d[p] != 0xFF) {
            error = "JPEG: marker expected";
            return false;
        }
        const uint8_t m = d[p + 1];
        if (m == 0xFF) {  // fill byte
            p++;
            continue;
        }
        if (m == 0xD9) break;  // EOI
        if (m == 0x01 || (m >= 0xD0 && m <= 0xD7)) {
            p += 2;
            continue;
        }
        const size_t len = be16(&d[p + 2]);
        if (len < 2 || p + 2 + len > d.size()) {
            error = "JPEG: segment runs past the end of the file";
            return false;
        }
        const uint8_t *s = &d[p + 4];
        const size_t sl = len - 2;
        if (m == 0xC2 || m == 0xC6 || m == 0xCA || m == 0xCE) {
            error = "progressive JPEG is not supported (only sequential Huffman-coded JPEG)";
            return false;
        }
        if ((m >= 0xC3 && m <= 0xCF && m != 0xC4 && m != 0xC8 && m != 0xCC) || m == 0xC9 || m == 0xCA || m == 0xCB) {
            error = "lossless, hierarchical or arithmetic-coded JPEG is not supported";
            return false;
        }
        if (m == 0xDB) {  // DQT
            size_t q = 0;
            while (q < sl) {
                const int pq = s[q] >> 4, tq = s[q] & 15;
                q++;
                if (tq > 3 || q + (pq ? 128u : 64u) > sl) {
                    error = "JPEG: bad quantisation table";
                    return false;
                }
                for (int i = 0; i < 64; i++) qt[tq][i] = pq ? be16(&s[q + 2 * i]) : s[q + i];
                q += pq ? 128 : 64;
                qt_defined[tq] = true;
            }
        } else if (m == 0xC4) {  // DHT
            size_t q = 0;
            while (q < sl) {
                if (q + 17 > sl) {
                    error = "JPEG: bad Huffman table";
                    return false;
                }
                const int tc = s[q] >> 4, th = s[q] & 15;
                if (tc > 1 || th > 3) {
                    error = "JPEG: bad Huffman table class or id";
                    return false;
                }
                HuffTable &t = tc ? ac[th] : dc[th];
                int total = 0;
                for (int l = 1; l <= 16; l++) total += (t.counts[l] = s[q + l]);
                q += 17;
                if (total > 256 || q + total > sl) {
                    error = "JPEG: bad Huffman table";
                    return false;
                }
                std::memcpy(t.symbols, &s[q], total);
                q += total;
                t.build();
            }
        } else if (m == 0xDD) {  // DRI
            if (sl < 2) {
                error = "JPEG: bad restart interval";
                return false;
            }
            restart = be16(s);
        } else if (m == 0xC0 || m == 0xC1) {  // SOF0 / SOF1
            if (sl < 6 || s[0] != 8) {
                error = "JPEG: only 8-bit samples are supported";
                return false;
            }
            h = be16(&s[1]);
            w = be16(&s[3]);
            const int nc = s[5];
            if (w == 0 || h == 0 || (nc != 1 && nc != 3) || sl < 6u + 3u * nc) {
                error = "JPEG: only grey or three-component images with a known size are supported";
                return false;
            }
            comps.resize(nc);
            for (int c = 0; c < nc; c++) {
                comps[c].id = s[6 + 3 * c];
                comps[c].h = s[7 + 3 * c] >> 4;
                comps[c].v = s[7 + 3 * c] & 15;
                comps[c].tq = s[8 + 3 * c];
                if (comps[c].h < 1 || comps[c].h > 4 || comps[c].v < 1 || comps[c].v > 4 || comps[c].tq > 3) {
                    error = "JPEG: bad sampling factors";
                    return false;
                }
            }
            have_frame = true;
        } else if (m == 0xDA) {  // SOS: the whole image in one interleaved scan
            if (!have_frame) {
                error = "JPEG: scan before the frame header";
                return false;
            }
            const int ns = s[0];
            if (ns != (int)comps.size() || sl < 4u + 2u * ns) {
                error = "JPEG: only single-scan (interleaved) images are supported";
                return false;
            }
            for (int i = 0; i < ns; i++) {
                bool found = false;
                for (auto &c : comps)
                    if (c.id == s[1 + 2 * i]) {
                        c.td = s[2 + 2 * i] >> 4;
                        c.ta = s[2 + 2 * i] & 15;
                        found = c.td < 4 && c.ta < 4;
                    }
                if (!found) {
                    error = "JPEG: scan names an unknown component";
                    return false;
                }
            }
            int hmax = 1, vmax = 1;
            for (auto &c : comps) {
                hmax = std::max(hmax, c.h);
                vmax = std::max(vmax, c.v);
                if (!qt_defined[c.tq] || !dc[c.td].defined || !ac[c.ta].defined) {
                    error = "JPEG: a table the scan needs is missing";
                    return false;
                }
            }
            if (comps.size() == 1) hmax = vmax = 1;  // a single-component scan: one block per MCU
            const int mcux = (int)((w + 8 * hmax - 1) / (8 * hmax)), mcuy = (int)((h + 8 * vmax - 1) / (8 * vmax));
            if ((uint64_t)mcux * mcuy * 64 * hmax * vmax > (1ull << 28)) {
                error = "JPEG: image too large";
                return false;
            }
            for (auto &c : comps) {
                const int ch = comps.size() == 1 ? 1 : c.h, cv = comps.size() == 1 ? 1 : c.v;
                c.bw = mcux * ch;
                c.bh = mcuy * cv;
                c.pix.assign((size_t)c.bw * 8 * c.bh * 8, 0);
            }
            Reader r{d.data(), d.size(), p + 2 + len};
            int coef[64];
            const int nmcu = mcux * mcuy;
            for (int mcu = 0; mcu < nmcu; mcu++) {
                if (restart && mcu > 0 && mcu % restart == 0) {  // RSTn: byte-aligned, predictors reset
                    r.reset_bits();
                    while (r.pos + 1 < r.n && !(r.d[r.pos] == 0xFF && r.d[r.pos + 1] >= 0xD0 && r.d[r.pos + 1] <= 0xD7))
                        r.pos++;
                    r.pos += 2;
                    r.marker_hit = false;
                    for (auto &c : comps) c.pred = 0;
                }
                const int mx = mcu % mcux, my = mcu / mcux;
                for (auto &c : comps) {
                    const int ch = comps.size() == 1 ? 1 : c.h, cv = comps.size() == 1 ? 1 : c.v;
                    for (int by = 0; by < cv; by++)
                        for (int bx = 0; bx < ch; bx++) {
                            std::memset(coef, 0, sizeof(coef));
                            const int t = decode_symbol(r, dc[c.td]);
                            if (t < 0 || t > 11) {
                                error = "JPEG: bad DC code";
                                return false;
                            }
                            c.pred += extend(r.receive(t), t);
                            coef[0] = c.pred * qt[c.tq][0];
                            for (int k = 1; k < 64;) {
                                const int rs = decode_symbol(r, ac[c.ta]);
                                if (rs < 0) {
                                    error = "JPEG: bad AC code";
                                    return false;
                                }
                                const int run = rs >> 4, sz = rs & 15;
                                if (sz == 0) {
                                    if (run != 15) break;  // EOB
                                    k += 16;           // ZRL
                                    continue;
                                }
                                k += run;
                                if (k > 63) {
                                    error = "JPEG: AC coefficients past the block";
                                    return false;
                                }
                                coef[kZigzag[k]] = extend(r.receive(sz), sz) * qt[c.tq][k];
                                k++;
                            }
                            const int x0 = (mx * ch + bx) * 8, y0 = (my * cv + by) * 8;
                            idct8x8(coef, c.pix.data() + (size_t)y0 * c.bw * 8 + x0, c.bw * 8);
                        }
                }
            }
            done = true;
        }
        p += 2 + len;
    }
    if (!done) {
        error = "JPEG: no image data";
        return false;
    }
    // up-sample by replication and convert to RGB (JFIF)
    comp = comps.size() == 1 ? 1 : 3;
    img.assign((size_t)w * h * comp, 0);
    int hmax = 1, vmax = 1;
    for (auto &c : comps) hmax = std::max(hmax, c.h), vmax = std::max(vmax, c.v);
    auto sample = [&](const Component &c, uint32_t x, uint32_t y) -> double {
        if (comps.size() == 1) return c.pix[(size_t)y * c.bw * 8 + x];
        const uint32_t sx = x * c.h / hmax, sy = y * c.v / vmax;
        return c.pix[(size_t)sy * c.bw * 8 + sx];
    };
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++) {
            uint8_t *o = img.data() + ((size_t)y * w + x) * comp;
            if (comp == 1) {
                o[0] = static_cast<uint8_t>(sample(comps[0], x, y));
                continue;
            }
            const double Y = sample(comps[0], x, y), cb = sample(comps[1], x, y) - 128.0,
                         cr = sample(comps[2], x, y) - 128.0;
            const double rgb[3] = {Y + 1.402 * cr, Y - 0.344136 * cb - 0.714136 * cr, Y + 1.772 * cb};
            for (int k = 0; k < 3; k++) {
                const long v = std::lround(rgb[k]);
                o[k] = static_cast<uint8_t>(v < 0 ? 0 : v > 255 ? 255 : v);
            }
        }
    return true;
}

}  // namespace Pupil::util
