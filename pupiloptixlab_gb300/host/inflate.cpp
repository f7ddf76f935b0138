// inflate.cpp -- zlib / DEFLATE decompression (see inflate.h), written from
// RFC 1950 and RFC 1951: bits are read least significant first, Huffman
// codes most significant bit first, and canonical codes are decoded length by
// length from the number of codes of each length.
#include "inflate.h"

#include <algorithm>
#include <array>

namespace Pupil::util {

namespace {

struct BitReader {
    const uint8_t *p;
    size_t n, pos = 0;  // byte position
    uint32_t bitbuf = 0;
    int bitcnt = 0;
    bool overrun = false;

    int bit() {
        if (bitcnt == 0) {
            if (pos >= n) {
                overrun = true;
                return 0;
            }
            bitbuf = p[pos++];
            bitcnt = 8;
        }
        const int b = static_cast<int>(bitbuf & 1u);
        bitbuf >>= 1;
        bitcnt--;
        return b;
    }
    uint32_t bits(int k) {  // k bits, least significant first
        uint32_t v = 0;
        for (int i = 0; i < k; i++) v |= static_cast<uint32_t>(bit()) << i;
        return v;
    }
    void align() { bitcnt = 0; }
};

// A canonical Huffman code: count[len] codes of each length 1..15 and the
// symbols ordered by (length, symbol value).
struct Huffman {
    std::array<uint16_t, 16> count{};
    std::vector<uint16_t> symbol;

    // false for an over-subscribed set of lengths
    bool build(const uint8_t *lengths, int n) {
        count.fill(0);
        for (int i = 0; i < n; i++) count[lengths[i]]++;
        count[0] = 0;
        int left = 1;
        for (int len = 1; len < 16; len++) {
            left <<= 1;
            left -= count[len];
            if (left < 0) return false;
        }
        std::array<uint16_t, 16> offs{};
        for (int len = 1; len < 15; len++) offs[len + 1] = static_cast<uint16_t>(offs[len] + count[len]);
        symbol.assign(static_cast<size_t>(n), 0);
        for (int i = 0; i < n; i++)
            if (lengths[i]) symbol[offs[lengths[i]]++] = static_cast<uint16_t>(i);
        return true;
    }
    // -1 for a code that is not in the table
    int decode(BitReader &br) const {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; len++) {
            code |= br.bit();
            const int c = count[len];
            if (code - first < c) return symbol[static_cast<size_t>(index + code - first)];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        return -1;
    }
};

// RFC 1951 3.2.5: base lengths and extra bits of length codes 257..285,
// base distances and extra bits of distance codes 0..29
constexpr uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                                   35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
constexpr uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
constexpr uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193,
                                    257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
constexpr uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6,
                                    7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
// RFC 1951 3.2.7: order of the code-length code lengths
constexpr uint8_t kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

bool codes(BitReader &br, const Huffman &lit, const Huffman &dist, std::vector<uint8_t> &out, size_t start,
           size_t limit, std::string &error) {
    for (;;) {
        const int sym = lit.decode(br);
        if (sym < 0 || br.overrun) {
            error = "deflate: bad literal/length code";
            return false;
        }
        if (sym < 256) {
            if (out.size() >= limit) {
                error = "deflate: output larger than expected";
                return false;
            }
            out.push_back(static_cast<uint8_t>(sym));
        } else if (sym == 256) {
            return true;
        } else {
            const int li = sym - 257;
            if (li >= 29) {
                error = "deflate: bad length code";
                return false;
            }
            const size_t len = kLenBase[li] + br.bits(kLenExtra[li]);
            const int ds = dist.decode(br);
            if (ds < 0 || ds >= 30 || br.overrun) {
                error = "deflate: bad distance code";
                return false;
            }
            const size_t d = kDistBase[ds] + br.bits(kDistExtra[ds]);
            if (d > out.size() - start) {
                error = "deflate: distance before the start of the data";
                return false;
            }
            if (out.size() + len > limit) {
                error = "deflate: output larger than expected";
                return false;
            }
            const size_t from = out.size() - d;
            for (size_t i = 0; i < len; i++) out.push_back(out[from + i]);  // may overlap: byte by byte
        }
    }
}

}  // namespace

bool ZlibInflate(const uint8_t *src, size_t n, std::vector<uint8_t> &out, size_t limit, std::string &error) {
    if (n < 6) {
        error = "zlib stream truncated";
        return false;
    }
    const uint8_t cmf = src[0], flg = src[1];
    if ((cmf & 0x0f) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20)) {
        error = "not a zlib deflate stream (or it needs a preset dictionary)";
        return false;
    }
    const size_t start = out.size();
    limit += start;
    BitReader br{src + 2, n - 2};
    Huffman fixed_lit, fixed_dist;
    {
        uint8_t l[288];
        for (int i = 0; i < 144; i++) l[i] = 8;
        for (int i = 144; i < 256; i++) l[i] = 9;
        for (int i = 256; i < 280; i++) l[i] = 7;
        for (int i = 280; i < 288; i++) l[i] = 8;
        fixed_lit.build(l, 288);
        uint8_t dl[30];
        std::fill(dl, dl + 30, 5);
        fixed_dist.build(dl, 30);
    }
    int last = 0;
    do {
        last = br.bit();
        const uint32_t type = br.bits(2);
        if (br.overrun) {
            error = "deflate: stream truncated";
            return false;
        }
        if (type == 0) {  // stored
            br.align();
            if (br.pos + 4 > br.n) {
                error = "deflate: stored block truncated";
                return false;
            }
            const uint32_t len = br.p[br.pos] | (br.p[br.pos + 1] << 8);
            const uint32_t nlen = br.p[br.pos + 2] | (br.p[br.pos + 3] << 8);
            br.pos += 4;
            if ((len ^ 0xffffu) != nlen || br.pos + len > br.n || out.size() + len > limit) {
                error = "deflate: stored block malformed";
                return false;
            }
            out.insert(out.end(), br.p + br.pos, br.p + br.pos + len);
            br.pos += len;
        } else if (type == 1) {
            if (!codes(br, fixed_lit, fixed_dist, out, start, limit, error)) return false;
        } else if (type == 2) {  // dynamic Huffman codes
            const int nlen = static_cast<int>(br.bits(5)) + 257, ndist = static_cast<int>(br.bits(5)) + 1,
                      ncode = static_cast<int>(br.bits(4)) + 4;
            if (nlen > 286 || ndist > 30) {
                error = "deflate: bad code counts";
                return false;
            }
            uint8_t cl[19] = {0};
            for (int i = 0; i < ncode; i++) cl[kClOrder[i]] = static_cast<uint8_t>(br.bits(3));
            Huffman clh;
            if (!clh.build(cl, 19)) {
                error = "deflate: bad code-length code";
                return false;
            }
            uint8_t lengths[286 + 30] = {0};
            int i = 0;
            while (i < nlen + ndist) {
                const int sym = clh.decode(br);
                if (sym < 0 || br.overrun) {
                    error = "deflate: bad code length";
                    return false;
                }
                if (sym < 16) {
                    lengths[i++] = static_cast<uint8_t>(sym);
                } else {
                    uint8_t v = 0;
                    int rep;
                    if (sym == 16) {
                        if (i == 0) {
                            error = "deflate: repeat with no previous length";
                            return false;
                        }
                        v = lengths[i - 1];
                        rep = 3 + static_cast<int>(br.bits(2));
                    } else if (sym == 17) {
                        rep = 3 + static_cast<int>(br.bits(3));
                    } else {
                        rep = 11 + static_cast<int>(br.bits(7));
                    }
                    if (i + rep > nlen + ndist) {
                        error = "deflate: code lengths overrun";
                        return false;
                    }
                    while (rep--) lengths[i++] = v;
                }
            }
            if (lengths[256] == 0) {
                error = "deflate: no end-of-block code";
                return false;
            }
            Huffman lit, dist;
            if (!lit.build(lengths, nlen) || !dist.build(lengths + nlen, ndist)) {
                error = "deflate: over-subscribed code";
                return false;
            }
            if (!codes(br, lit, dist, out, start, limit, error)) return false;
        } else {
            error = "deflate: reserved block type";
            return false;
        }
    } while (!last);
    // Adler-32 of the output, big-endian after the (byte-aligned) stream
    br.align();
    if (br.pos + 4 > br.n) {
        error = "zlib: Adler-32 missing";
        return false;
    }
    uint32_t a = 1, b = 0;
    for (size_t k = start; k < out.size(); k++) {
        a = (a + out[k]) % 65521u;
        b = (b + a) % 65521u;
    }
    const uint32_t want = (static_cast<uint32_t>(br.p[br.pos]) << 24) | (br.p[br.pos + 1] << 16) |
                          (br.p[br.pos + 2] << 8) | br.p[br.pos + 3];
    if (((b << 16) | a) != want) {
        error = "zlib: Adler-32 mismatch";
        return false;
    }
    return true;
}

}  // namespace Pupil::util
