// readers_fuzz.cpp -- mutation test of the host layer's file readers (images,
// OBJ, HAIR, mitsuba XML): every seed file is mutated N times (bit flips,
// byte stores, truncation, insertion, deletion; PNG chunk CRCs repaired for
// half the cases so that the decoder itself runs) and read back.  A reader
// may accept or refuse a mutated file; built with AddressSanitizer and
// UndefinedBehaviorSanitizer, any out-of-bounds access, overflow or uncaught
// exception ends the process with a non-zero status.
//
// usage: readers_fuzz <iterations> <seed files...>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "image.h"
#include "pt_api.h"
#include "scene.h"

// The XML loader's camera comes from the CUDA library; the readers do not need it.
extern "C" int pt_camera_make(float, float, float, float, const float *, pt_camera_desc *out) {
    *out = pt_camera_desc{};
    return 0;
}

namespace {

std::string ext_of(const std::string &p) {
    const size_t d = p.rfind('.');
    return d == std::string::npos ? "" : p.substr(d);
}

void fix_png_crcs(std::vector<char> &d) {
    size_t q = 8;
    while (q + 12 <= d.size()) {
        const uint32_t len = ((uint32_t)(uint8_t)d[q] << 24) | ((uint32_t)(uint8_t)d[q + 1] << 16) |
                             ((uint32_t)(uint8_t)d[q + 2] << 8) | (uint8_t)d[q + 3];
        if (len > d.size() - q - 12) break;
        uint32_t c = 0xffffffffu;
        for (size_t i = q + 4; i < q + 8 + len; i++) {
            c ^= (uint8_t)d[i];
            for (int k = 0; k < 8; k++) c = (c >> 1) ^ (0xedb88320u & (0u - (c & 1u)));
        }
        c ^= 0xffffffffu;
        for (int k = 0; k < 4; k++) d[q + 8 + len + k] = (char)(c >> (24 - 8 * k));
        q += 12 + len;
    }
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s <iterations> <seed files...>\n", argv[0]);
        return 2;
    }
    const int iters = atoi(argv[1]);
    std::mt19937 rng(20261204u);
    for (int a = 2; a < argc; a++) {
        const std::string path = argv[a], ext = ext_of(path);
        std::ifstream f(path, std::ios::binary);
        const std::vector<char> seed((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
        const std::string tmp = path + ".mut" + ext;
        const bool text = ext == ".obj" || ext == ".xml";
        const char *alpha = text ? "<>/=\"' abcdefghijklmnopqrstuvwxyz0123456789.-e,\nfv" : nullptr;
        int accepted = 0;
        for (int it = 0; it < iters; it++) {
            std::vector<char> d = seed;
            const int nm = 1 + (int)(rng() % 6);
            for (int m = 0; m < nm && !d.empty(); m++) {
                const size_t pos = rng() % d.size();
                const char byte = text ? alpha[rng() % 50] : (char)(rng() % 256);
                switch (rng() % 6) {
                    case 0: d[pos] = (char)(d[pos] ^ (1 << (rng() % 8))); break;
                    case 1: d[pos] = byte; break;
                    case 2: d[pos] = (rng() & 1) ? (char)0xff : (char)0; break;
                    case 3: d.resize(pos); break;
                    case 4: d.insert(d.begin() + (long)pos, 1 + rng() % 16, byte); break;
                    default: {
                        const size_t len = 1 + rng() % 32;
                        if (pos + len <= d.size()) d.erase(d.begin() + (long)pos, d.begin() + (long)(pos + len));
                    }
                }
            }
            if (ext == ".png" && (it & 1)) fix_png_crcs(d);
            bool ok = false;
            std::string error;
            if (ext == ".xml") {
                Pupil::resource::Scene s;
                ok = s.LoadFromString(std::string(d.begin(), d.end()), ".");
                if (ok) (void)s.Desc();
            } else {
                {
                    std::ofstream o(tmp, std::ios::binary);
                    o.write(d.data(), (std::streamsize)d.size());
                }
                if (ext == ".obj") {
                    Pupil::resource::Mesh m;
                    ok = Pupil::resource::LoadObj(tmp, m, error);
                } else if (ext == ".hair") {
                    Pupil::resource::Curves c;
                    ok = Pupil::resource::LoadCyHair(tmp, 0.f, (it & 1) != 0, 0, c, error);
                } else {
                    std::vector<float> rgba;
                    uint32_t w = 0, h = 0;
                    ok = Pupil::util::LoadImageRGBA(tmp, rgba, w, h, error);
                    if (ok && rgba.size() != 4ull * w * h) {
                        fprintf(stderr, "%s: %zu values for %u x %u pixels\n", path.c_str(), rgba.size(), w, h);
                        return 1;
                    }
                }
            }
            accepted += ok;
        }
        std::remove(tmp.c_str());
        printf("%s: %d of %d mutations accepted\n", path.c_str(), accepted, iters);
    }
    return 0;
}
