// pt_denoise.cu -- the learned denoiser: a 5-level U-Net over NHWC BF16
// tensors whose 14 convolutions run on the tcgen05 kernels of pt_conv.cu,
// trained with Adam on the L1 loss of log(1 + x), and applied to rendered
// frames with a per-tile fallback to the raw colour.  It replaces the OptiX
// denoiser behind the reference's DenoisePass
// (framework/system/denoise_pass.cpp:50-75, framework/optix/denoiser.cpp:171-267),
// which takes the same three layers: colour, albedo and normal.
//
// Network (level = resolution / 2^level; "cat" = channel concatenation, the
// skip half written in place by the encoder convolution):
//   L0  e0a 16->32, e0b 32->32 (-> cat0[48:80]),  pool
//   L1  e1a 32->48, e1b 48->48 (-> cat1[64:112]), pool
//   L2  e2a 48->64, e2b 64->64 (-> cat2[128:192]), pool
//   L3  e3a 64->128, e3b 128->128 (-> cat3[256:384]), pool
//   L4  b 128->256, nearest 2x up -> cat3[0:256]
//   L3  d3 384->128, up -> cat2[0:128]
//   L2  d2 192->64, up -> cat1[0:64]
//   L1  d1 112->48, up -> cat0[0:48]
//   L0  d0 80->32, out 32->3 (16 computed, FP32, no ReLU)
// All hidden convolutions are followed by ReLU; pooling is the 2x2 mean.
// Input channels: log(1 + max(rgb, 0)), albedo, normal, 7 zero channels.
// Output: a log-domain correction; the denoised colour is
// expm1(output + log(1 + max(rgb, 0))).
#include "pt_nvtx.h"
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "pt_conv.h"
#include "pt_internal.h"

using ptconv::Act;

namespace {

struct LayerSpec {
    int cin, cout, relu;
};
constexpr int kLayers = 14;
constexpr LayerSpec kSpec[kLayers] = {
    {16, 32, 1},   {32, 32, 1},   {32, 48, 1},  {48, 48, 1},   {48, 64, 1}, {64, 64, 1}, {64, 128, 1},
    {128, 128, 1}, {128, 256, 1}, {384, 128, 1}, {192, 64, 1}, {112, 48, 1}, {80, 32, 1}, {32, 16, 0},
};
enum { E0A, E0B, E1A, E1B, E2A, E2B, E3A, E3B, BOT, D3, D2, D1, D0, OUT };
constexpr int kOutChannels = 3;

__device__ __forceinline__ float bf2f(uint16_t h) { return __uint_as_float(static_cast<uint32_t>(h) << 16); }

// 16 BF16 channels = 32 bytes = one sector, moved with one 256-bit access
// (sm_100 and later; every tensor here has channel counts and offsets that
// are multiples of 16 on 256-byte-aligned buffers).
struct C16 {
    uint32_t w[8];
    __device__ __forceinline__ uint16_t operator[](int k) const { return (w[k >> 1] >> (16 * (k & 1))) & 0xffffu; }
    __device__ __forceinline__ void set(int k, uint16_t h) {
        w[k >> 1] = (w[k >> 1] & (0xffff0000u >> (16 * (k & 1)))) | (static_cast<uint32_t>(h) << (16 * (k & 1)));
    }
};
__device__ __forceinline__ C16 ld_c16(const uint16_t *p) {
    C16 v;
    asm volatile("ld.global.v8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(v.w[0]), "=r"(v.w[1]), "=r"(v.w[2]), "=r"(v.w[3]), "=r"(v.w[4]), "=r"(v.w[5]), "=r"(v.w[6]),
                   "=r"(v.w[7])
                 : "l"(p));
    return v;
}
__device__ __forceinline__ void st_c16(uint16_t *p, const C16 &v) {
    asm volatile("st.global.v8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "r"(v.w[0]), "r"(v.w[1]),
                 "r"(v.w[2]), "r"(v.w[3]), "r"(v.w[4]), "r"(v.w[5]), "r"(v.w[6]), "r"(v.w[7])
                 : "memory");
}
__device__ __forceinline__ uint16_t f2bf(float f) {
    __nv_bfloat16 h = __float2bfloat16_rn(f);
    return *reinterpret_cast<uint16_t *>(&h);
}
__device__ __forceinline__ bool pos(uint16_t h) { return h != 0 && (h & 0x8000u) == 0; }

// ---------------------------------------------------------------------------
// elementwise kernels (8 channels = 16 bytes per thread where the layout allows)
// ---------------------------------------------------------------------------
// training layout (FP16 9 channels) -> network input (BF16 16 channels)
__global__ void k_pack_input(const __half *in, long long npix, uint16_t *x0) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix; p += (long long)gridDim.x * blockDim.x) {
        const __half *s = in + p * 9;
        uint16_t o[16];
#pragma unroll
        for (int c = 0; c < 9; c++) {
            float f = __half2float(s[c]);
            if (c < 3) f = log1pf(fmaxf(f, 0.f));
            o[c] = f2bf(f);
        }
#pragma unroll
        for (int c = 9; c < 16; c++) o[c] = 0;
        uint4 *d = reinterpret_cast<uint4 *>(x0 + p * 16);
        d[0] = *reinterpret_cast<uint4 *>(o);
        d[1] = *reinterpret_cast<uint4 *>(o + 8);
    }
}

// rendered frame -> network input, rows [h, hp) and columns [w, wp) zero
__global__ void k_pack_frame(const float4 *color, const float *albedo, const float *normal, int w, int h, int wp,
                             int hp, uint16_t *x0) {
    const long long n = (long long)wp * hp;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        const int x = static_cast<int>(p % wp), y = static_cast<int>(p / wp);
        uint16_t o[16];
#pragma unroll
        for (int c = 0; c < 16; c++) o[c] = 0;
        if (x < w && y < h) {
            const long long q = (long long)y * w + x;
            float4 c4 = color[q];
            o[0] = f2bf(log1pf(fmaxf(c4.x, 0.f)));
            o[1] = f2bf(log1pf(fmaxf(c4.y, 0.f)));
            o[2] = f2bf(log1pf(fmaxf(c4.z, 0.f)));
            for (int c = 0; c < 3; c++) {
                o[3 + c] = f2bf(albedo[q * 3 + c]);
                o[6 + c] = f2bf(normal[q * 3 + c]);
            }
        }
        uint4 *d = reinterpret_cast<uint4 *>(x0 + p * 16);
        d[0] = *reinterpret_cast<uint4 *>(o);
        d[1] = *reinterpret_cast<uint4 *>(o + 8);
    }
}

__global__ void k_pack_f16(const float4 *color, const float *albedo, const float *normal, long long npix, __half *out) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix; p += (long long)gridDim.x * blockDim.x) {
        float4 c4 = color[p];
        __half *o = out + p * 9;
        o[0] = __float2half_rn(c4.x);
        o[1] = __float2half_rn(c4.y);
        o[2] = __float2half_rn(c4.z);
        for (int c = 0; c < 3; c++) {
            o[3 + c] = __float2half_rn(albedo[p * 3 + c]);
            o[6 + c] = __float2half_rn(normal[p * 3 + c]);
        }
    }
}

// dst[n, y, x, 0:c] = mean of src[n, 2y+i, 2x+j, 0:c]   (c % 8 == 0)
__global__ void k_pool(const uint16_t *src, int sctot, int scoff, int c, int n, int h2, int w2, uint16_t *dst) {
    const int groups = c / 8;
    const long long total = (long long)n * h2 * w2 * groups;
    const int w = 2 * w2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int gq = static_cast<int>(i % groups);
        long long p = i / groups;
        const int x = static_cast<int>(p % w2);
        const int y = static_cast<int>((p / w2) % h2);
        const int b = static_cast<int>(p / ((long long)w2 * h2));
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int dy = 0; dy < 2; dy++)
            for (int dx = 0; dx < 2; dx++) {
                const long long q = ((long long)b * 2 * h2 + 2 * y + dy) * w + 2 * x + dx;
                uint4 v = *reinterpret_cast<const uint4 *>(src + q * sctot + scoff + gq * 8);
                const uint16_t *hv = reinterpret_cast<const uint16_t *>(&v);
#pragma unroll
                for (int k = 0; k < 8; k++) acc[k] += bf2f(hv[k]);
            }
        uint16_t o[8];
#pragma unroll
        for (int k = 0; k < 8; k++) o[k] = f2bf(0.25f * acc[k]);
        *reinterpret_cast<uint4 *>(dst + p * c + gq * 8) = *reinterpret_cast<uint4 *>(o);
    }
}

// cat[n, y, x, 0:c] = lo[n, y/2, x/2, 0:c] (when the producing convolution's
// epilogue does not write the up-sampled copy itself)
__global__ void k_upcat(const uint16_t *lo, int c, int n, int h, int w, uint16_t *cat, int cat_ctot) {
    const int groups = c / 8;
    const long long total = (long long)n * h * w * groups;
    const int h2 = h / 2, w2 = w / 2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int gq = static_cast<int>(i % groups);
        long long p = i / groups;
        const int x = static_cast<int>(p % w);
        const int y = static_cast<int>((p / w) % h);
        const int b = static_cast<int>(p / ((long long)w * h));
        const long long q = ((long long)b * h2 + y / 2) * w2 + x / 2;
        *reinterpret_cast<uint4 *>(cat + p * cat_ctot + gq * 8) = *reinterpret_cast<const uint4 *>(lo + q * c + gq * 8);
    }
}

// g_lo[n, y, x, c] = (lo > 0) * sum over the 2x2 children of g_cat[.., 0:c]
__global__ void k_up_back(const uint16_t *gcat, int cat_ctot, const uint16_t *lo, int c, int n, int h2, int w2,
                          uint16_t *glo) {
    const int groups = c / 16;
    const long long total = (long long)n * h2 * w2 * groups;
    const int w = 2 * w2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int gq = static_cast<int>(i % groups);
        long long p = i / groups;
        const int x = static_cast<int>(p % w2);
        const int y = static_cast<int>((p / w2) % h2);
        const int b = static_cast<int>(p / ((long long)w2 * h2));
        float acc[16];
#pragma unroll
        for (int k = 0; k < 16; k++) acc[k] = 0.f;
        for (int dy = 0; dy < 2; dy++)
            for (int dx = 0; dx < 2; dx++) {
                const long long q = ((long long)b * 2 * h2 + 2 * y + dy) * w + 2 * x + dx;
                const C16 v = ld_c16(gcat + q * cat_ctot + gq * 16);
#pragma unroll
                for (int k = 0; k < 16; k++) acc[k] += bf2f(v[k]);
            }
        const C16 m = ld_c16(lo + p * c + gq * 16);
        C16 o{};
#pragma unroll
        for (int k = 0; k < 16; k++) o.set(k, pos(m[k]) ? f2bf(acc[k]) : 0);
        st_c16(glo + p * c + gq * 16, o);
    }
}

// Gradient at an encoder output y (stored as cat[.., coff:coff+c]) that feeds
// both the skip concatenation and the 2x2 mean pool:
//   g[n, y, x, k] = (y > 0) * (g_cat[.., coff + k] + 0.25 * g_pool[n, y/2, x/2, k])
__global__ void k_skip_back(const uint16_t *cat, const uint16_t *gcat, int cat_ctot, int coff, const uint16_t *gpool,
                            int c, int n, int h, int w, uint16_t *g) {
    const int groups = c / 16;
    const long long total = (long long)n * h * w * groups;
    const int h2 = h / 2, w2 = w / 2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int gq = static_cast<int>(i % groups);
        long long p = i / groups;
        const int x = static_cast<int>(p % w);
        const int y = static_cast<int>((p / w) % h);
        const int b = static_cast<int>(p / ((long long)w * h));
        const long long q = ((long long)b * h2 + y / 2) * w2 + x / 2;
        const C16 yv = ld_c16(cat + p * cat_ctot + coff + gq * 16);
        const C16 gv = ld_c16(gcat + p * cat_ctot + coff + gq * 16);
        const C16 pv = ld_c16(gpool + q * c + gq * 16);
        C16 o{};
#pragma unroll
        for (int k = 0; k < 16; k++) o.set(k, pos(yv[k]) ? f2bf(__fmaf_rn(0.25f, bf2f(pv[k]), bf2f(gv[k]))) : 0);
        st_c16(g + p * c + gq * 16, o);
    }
}

// L1 loss on log(1 + x).  The prediction is the network's output plus the
// input's log colour (x0 channels 0-2): the network learns a correction.
// g_out (16 channels) = sign(prediction - log1p(target)) / count; loss_sum += sum |.|.
__global__ void k_loss(const float *out, const uint16_t *x0, const float *target, long long npix, float inv_count,
                       uint16_t *gout, float *loss_sum) {
    float acc = 0.f;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix; p += (long long)gridDim.x * blockDim.x) {
        uint16_t o[16];
#pragma unroll
        for (int c = 0; c < 16; c++) o[c] = 0;
        for (int c = 0; c < kOutChannels; c++) {
            const float d = out[p * 3 + c] + bf2f(x0[p * 16 + c]) - log1pf(fmaxf(target[p * 3 + c], 0.f));
            acc += fabsf(d);
            o[c] = f2bf(d > 0.f ? inv_count : d < 0.f ? -inv_count : 0.f);
        }
        uint4 *dst = reinterpret_cast<uint4 *>(gout + p * 16);
        dst[0] = *reinterpret_cast<uint4 *>(o);
        dst[1] = *reinterpret_cast<uint4 *>(o + 8);
    }
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss_sum, acc);
}

// Adam bias corrections for the step about to run: state = {step, 1/(1-b1^t),
// 1/(1-b2^t), step size}; the step size lives on the device so that the
// captured training graph follows pt_denoiser_set_lr.
__global__ void k_adam_begin(float *state, float beta1, float beta2) {
    const float t = state[0] + 1.f;
    state[0] = t;
    state[1] = 1.f / (1.f - powf(beta1, t));
    state[2] = 1.f / (1.f - powf(beta2, t));
}

// Adam over every layer in one launch.  Layer l's parameters are its weights
// [cout][9][cin] at w_off[l] followed by its bias[cout]; the kernel also
// writes the BF16 weights and their flipped transpose [cin][9][cout] (for the
// data gradient) at wbf_off[l].
struct AdamLayers {
    long long w_off[kLayers], nw[kLayers], wbf_off[kLayers];
    int cin[kLayers], cout[kLayers];
};

__global__ void k_adam(float *p, float *m, float *v, const float *g, const AdamLayers L, const float *state,
                       float beta1, float beta2, float eps, uint16_t *wbf, uint16_t *wtbf) {
    const float c1 = state[1], c2 = state[2], lr = state[3];
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (int l = 0; l < kLayers; l++) {
        const long long nw = L.nw[l], n = nw + L.cout[l], o = L.w_off[l];
        const int cin = L.cin[l], cout = L.cout[l];
        uint16_t *wb = wbf + L.wbf_off[l], *wt = wtbf + L.wbf_off[l];
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
            const float gi = g[o + i];
            const float mi = beta1 * m[o + i] + (1.f - beta1) * gi;
            const float vi = beta2 * v[o + i] + (1.f - beta2) * gi * gi;
            m[o + i] = mi;
            v[o + i] = vi;
            const float pi = p[o + i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
            p[o + i] = pi;
            if (i < nw) {
                const uint16_t b = f2bf(pi);
                wb[i] = b;
                const int ci = static_cast<int>(i % cin);
                const int tap = static_cast<int>((i / cin) % 9);
                const int co = static_cast<int>(i / (9ll * cin));
                wt[(static_cast<long long>(ci) * 9 + (8 - tap)) * cout + co] = b;
            }
        }
    }
}

__global__ void k_weights_to_bf16(const float *p, long long nw, int cout, int cin, uint16_t *wbf, uint16_t *wtbf) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nw; i += (long long)gridDim.x * blockDim.x) {
        const uint16_t b = f2bf(p[i]);
        wbf[i] = b;
        const int ci = static_cast<int>(i % cin);
        const int tap = static_cast<int>((i / cin) % 9);
        const int co = static_cast<int>(i / (9ll * cin));
        wtbf[(static_cast<long long>(ci) * 9 + (8 - tap)) * cout + co] = b;
    }
}

// network output + input log colour -> linear colour, [n][h][w][3]
__global__ void k_expm1(const float *o, const uint16_t *x0, long long npix, float *out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npix * 3;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = fmaxf(expm1f(o[i] + bf2f(x0[(i / 3) * 16 + i % 3])), 0.f);
}

__device__ __forceinline__ float lum(float r, float g, float b) { return 0.2126f * r + 0.7152f * g + 0.0722f * b; }

// linear colour of padded-frame pixel q: expm1(network output + input log colour)
__device__ __forceinline__ float3 denoised(const float *o, const uint16_t *x0, long long q) {
    return make_float3(fmaxf(expm1f(o[q * 3] + bf2f(x0[q * 16])), 0.f),
                       fmaxf(expm1f(o[q * 3 + 1] + bf2f(x0[q * 16 + 1])), 0.f),
                       fmaxf(expm1f(o[q * 3 + 2] + bf2f(x0[q * 16 + 2])), 0.f));
}

// Left-right mirror of every row of the 16-channel network input, in place
// (pixel x <-> wp - 1 - x, 32 bytes each).
__global__ void k_mirror_x0(uint16_t *x0, int wp, int hp) {
    const long long half = (long long)(wp / 2) * hp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < half; i += (long long)gridDim.x * blockDim.x) {
        const long long y = i / (wp / 2), x = i - y * (wp / 2);
        uint4 *a = reinterpret_cast<uint4 *>(x0 + (y * wp + x) * 16);
        uint4 *b = reinterpret_cast<uint4 *>(x0 + (y * wp + (wp - 1 - x)) * 16);
        const uint4 a0 = a[0], a1 = a[1], b0 = b[0], b1 = b[1];
        a[0] = b0;
        a[1] = b1;
        b[0] = a0;
        b[1] = a1;
    }
}

// acc = (acc + mirror(o)) / 2 for the 3-channel network output.
__global__ void k_mirror_average(float *acc, const float *o, int wp, long long npix) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < npix; q += (long long)gridDim.x * blockDim.x) {
        const long long y = q / wp, x = q - y * wp;
        const long long m = y * wp + (wp - 1 - x);
#pragma unroll
        for (int c = 0; c < 3; c++) acc[q * 3 + c] = 0.5f * (acc[q * 3 + c] + o[m * 3 + c]);
    }
}

// One block per tile: mean luminance of the raw and the denoised colour and
// the raw colour's standard error; write the tile's pixels, falling back to
// the raw colour where the denoised mean moved by more than the threshold.
__global__ void k_denoise_out(const float4 *color, const float *o, const uint16_t *xin, int w, int h, int wp, int tile,
                              float rel, float sig, float4 *out, uint8_t *tile_flag, unsigned *fallback_count) {
    const int tiles_x = (w + tile - 1) / tile;
    const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    const int tx0 = tx * tile, ty0 = ty * tile;
    const int tw = min(tile, w - tx0), th = min(tile, h - ty0);
    float s_raw = 0.f, s_raw2 = 0.f, s_den = 0.f;
    for (int i = threadIdx.x; i < tw * th; i += blockDim.x) {
        const int x = tx0 + i % tw, y = ty0 + i / tw;
        const float4 c = color[(long long)y * w + x];
        const float3 dc = denoised(o, xin, (long long)y * wp + x);
        const float lr = lum(c.x, c.y, c.z);
        s_raw += lr;
        s_raw2 += lr * lr;
        s_den += lum(dc.x, dc.y, dc.z);
    }
    __shared__ float red[3][32];
    for (int off = 16; off > 0; off >>= 1) {
        s_raw += __shfl_down_sync(0xffffffffu, s_raw, off);
        s_raw2 += __shfl_down_sync(0xffffffffu, s_raw2, off);
        s_den += __shfl_down_sync(0xffffffffu, s_den, off);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = s_raw;
        red[1][threadIdx.x >> 5] = s_raw2;
        red[2][threadIdx.x >> 5] = s_den;
    }
    __syncthreads();
    __shared__ int fallback;
    if (threadIdx.x == 0) {
        float a = 0.f, a2 = 0.f, dd = 0.f;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
            a += red[0][i];
            a2 += red[1][i];
            dd += red[2][i];
        }
        const float cnt = static_cast<float>(tw * th);
        const float mean = a / cnt, mden = dd / cnt;
        const float var = fmaxf(a2 / cnt - mean * mean, 0.f);
        const float se = sqrtf(var / cnt);
        fallback = (sig > 0.f && fabsf(mden - mean) > fmaxf(rel * mean, sig * se)) ? 1 : 0;
        if (tile_flag) tile_flag[blockIdx.x] = static_cast<uint8_t>(fallback);
        if (fallback) atomicAdd(fallback_count, 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < tw * th; i += blockDim.x) {
        const int x = tx0 + i % tw, y = ty0 + i / tw;
        const long long q = (long long)y * w + x;
        if (fallback) {
            const float4 c = color[q];
            out[q] = make_float4(c.x, c.y, c.z, 1.f);
        } else {
            const float3 dc = denoised(o, xin, (long long)y * wp + x);
            out[q] = make_float4(dc.x, dc.y, dc.z, 1.f);
        }
    }
}

int grid_for(long long n, int threads = 256) {
    return static_cast<int>(std::max<long long>(1, std::min<long long>((n + threads - 1) / threads, 148ll * 16)));
}

// Buffers and prepared convolution launches for one input shape.
struct Plan {
    int n = 0, h = 0, w = 0;
    bool train = false;
    // forward
    DevBuf x0, a0, cat0, p0, a1, cat1, p1, a2, cat2, p2, a3, cat3, p3, b4, d3, d2, d1, d0, out;
    // backward
    DevBuf g_out, g_d0, g_cat0, g_d1, g_cat1, g_d2, g_cat2, g_d3, g_cat3, g_b4, g_p3, g_e3b, g_a3, g_p2, g_e2b, g_a2,
        g_p1, g_e1b, g_a1, g_p0, g_e0b, g_a0;
    DevBuf in_stage, tgt_stage;
    DevBuf out_acc;  // inference: network output averaged over the frame and its mirror image
    ptconv::FwdOp fwd[kLayers], bwd[kLayers];
    ptconv::WgradOp wg[kLayers];
    Act x_of[kLayers], g_of[kLayers];
    cudaGraphExec_t graph = nullptr;
    bool fused_up = true;  // the decoder convolutions write the up-sampled copies themselves

    void release() {
        DevBuf *all[] = {&x0,    &a0,    &cat0,   &p0,    &a1,    &cat1,   &p1,    &a2,    &cat2,  &p2,
                         &a3,    &cat3,  &p3,     &b4,    &d3,    &d2,     &d1,    &d0,    &out,   &g_out,
                         &g_d0,  &g_cat0, &g_d1,  &g_cat1, &g_d2, &g_cat2, &g_d3,  &g_cat3, &g_b4, &g_p3,
                         &g_e3b, &g_a3,  &g_p2,   &g_e2b, &g_a2,  &g_p1,   &g_e1b, &g_a1,  &g_p0,  &g_e0b,
                         &g_a0,  &in_stage, &tgt_stage, &out_acc};
        for (DevBuf *b : all) b->release();
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
        n = h = w = 0;
    }
};

}  // namespace

struct pt_denoiser {
    int device = 0, num_sms = 0;
    pt_denoiser_opts opts{};
    uint64_t w_off[kLayers], b_off[kLayers], wbf_off[kLayers];
    uint64_t nparams = 0, nweights = 0;
    DevBuf params, adam_m, adam_v, grads, wbf, wtbf, adam_state, err, loss, fallback;
    uint32_t loss_steps = 0;
    Plan train_plan, infer_plan;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr, t0 = nullptr, t1 = nullptr;
    // weight gradients on side streams, taken in turn (forked per layer once
    // its output gradient exists, joined before Adam), beside the
    // data-gradient chain
    cudaStream_t side[2] = {};
    cudaEvent_t ev_fork[kLayers] = {}, ev_join[2] = {};
    pt_denoise_stats stats{};
};

namespace {

Act act(const DevBuf &b, int n, int h, int w, int ctot, int coff, int c) {
    Act a;
    a.ptr = b.ptr;
    a.n = n;
    a.h = h;
    a.w = w;
    a.ctot = ctot;
    a.coff = coff;
    a.c = c;
    return a;
}

int alloc_bf16(DevBuf &b, long long elems) { return b.ensure(static_cast<size_t>(std::max<long long>(elems, 8)) * 2); }

const float *bias_ptr(const pt_denoiser *dn, int l) { return dn->params.as<float>() + dn->b_off[l]; }
const uint16_t *wbf_ptr(const pt_denoiser *dn, int l) { return dn->wbf.as<uint16_t>() + dn->wbf_off[l]; }
const uint16_t *wtbf_ptr(const pt_denoiser *dn, int l) { return dn->wtbf.as<uint16_t>() + dn->wbf_off[l]; }

int plan_prepare(pt_denoiser *dn, Plan &P, int n, int h, int w, bool train) {
    if (P.n == n && P.h == h && P.w == w && P.train == train) return PT_OK;
    P.release();
    if (h % 16 || w % 16 || h <= 0 || w <= 0 || n <= 0) {
        pt_set_error("denoiser: height and width must be positive multiples of 16 (got %dx%d)", w, h);
        return PT_ERR_INVALID;
    }
    const long long px[5] = {(long long)n * h * w, (long long)n * h * w / 4, (long long)n * h * w / 16,
                             (long long)n * h * w / 64, (long long)n * h * w / 256};
    int st;
#define PT_A(buf, lvl, c) \
    if ((st = alloc_bf16(P.buf, px[lvl] * (c))) != PT_OK) return st;
    PT_A(x0, 0, 16) PT_A(a0, 0, 32) PT_A(cat0, 0, 80) PT_A(p0, 1, 32) PT_A(a1, 1, 48) PT_A(cat1, 1, 112)
    PT_A(p1, 2, 48) PT_A(a2, 2, 64) PT_A(cat2, 2, 192) PT_A(p2, 3, 64) PT_A(a3, 3, 128) PT_A(cat3, 3, 384)
    PT_A(p3, 4, 128) PT_A(b4, 4, 256) PT_A(d3, 3, 128) PT_A(d2, 2, 64) PT_A(d1, 1, 48) PT_A(d0, 0, 32)
    if ((st = P.out.ensure(px[0] * 3 * sizeof(float))) != PT_OK) return st;
    if (train) {
        PT_A(g_out, 0, 16) PT_A(g_d0, 0, 32) PT_A(g_cat0, 0, 80) PT_A(g_d1, 1, 48) PT_A(g_cat1, 1, 112)
        PT_A(g_d2, 2, 64) PT_A(g_cat2, 2, 192) PT_A(g_d3, 3, 128) PT_A(g_cat3, 3, 384) PT_A(g_b4, 4, 256)
        PT_A(g_p3, 4, 128) PT_A(g_e3b, 3, 128) PT_A(g_a3, 3, 128) PT_A(g_p2, 3, 64) PT_A(g_e2b, 2, 64)
        PT_A(g_a2, 2, 64) PT_A(g_p1, 2, 48) PT_A(g_e1b, 1, 48) PT_A(g_a1, 1, 48) PT_A(g_p0, 1, 32)
        PT_A(g_e0b, 0, 32) PT_A(g_a0, 0, 32)
        if ((st = P.in_stage.ensure(px[0] * 9 * 2)) != PT_OK) return st;
        if ((st = P.tgt_stage.ensure(px[0] * 3 * sizeof(float))) != PT_OK) return st;
    }
#undef PT_A
    const int H[5] = {h, h / 2, h / 4, h / 8, h / 16}, W[5] = {w, w / 2, w / 4, w / 8, w / 16};
    auto A = [&](const DevBuf &b, int lvl, int ctot, int coff, int c) { return act(b, n, H[lvl], W[lvl], ctot, coff, c); };
    // forward: input, output (ctot, coff) per layer
    struct Io {
        Act in;
        const DevBuf *out;
        int lvl, octot, ocoff;
        DevBuf *up = nullptr;  // decoder: the 2x up-sampled copy goes to channels [0, cout) of this concatenation
        int up_ctot = 0;
        DevBuf *pool = nullptr;  // encoder: the 2x2 average (the next level's input), when the kernel can fuse it
    };
    const Io io[kLayers] = {
        {A(P.x0, 0, 16, 0, 16), &P.a0, 0, 32, 0},
        {A(P.a0, 0, 32, 0, 32), &P.cat0, 0, 80, 48, nullptr, 0, &P.p0},
        {A(P.p0, 1, 32, 0, 32), &P.a1, 1, 48, 0},
        {A(P.a1, 1, 48, 0, 48), &P.cat1, 1, 112, 64, nullptr, 0, &P.p1},
        {A(P.p1, 2, 48, 0, 48), &P.a2, 2, 64, 0},         {A(P.a2, 2, 64, 0, 64), &P.cat2, 2, 192, 128},
        {A(P.p2, 3, 64, 0, 64), &P.a3, 3, 128, 0},        {A(P.a3, 3, 128, 0, 128), &P.cat3, 3, 384, 256},
        {A(P.p3, 4, 128, 0, 128), &P.b4, 4, 256, 0, &P.cat3, 384},
        {A(P.cat3, 3, 384, 0, 384), &P.d3, 3, 128, 0, &P.cat2, 192},
        {A(P.cat2, 2, 192, 0, 192), &P.d2, 2, 64, 0, &P.cat1, 112},
        {A(P.cat1, 1, 112, 0, 112), &P.d1, 1, 48, 0, &P.cat0, 80},
        {A(P.cat0, 0, 80, 0, 80), &P.d0, 0, 32, 0},       {A(P.d0, 0, 32, 0, 32), &P.out, 0, 3, 0},
    };
    unsigned *err = dn->err.as<unsigned>();
    const bool separate_up = getenv("PT_DENOISER_SEPARATE_UPSAMPLE") != nullptr;
    P.fused_up = !separate_up;
    for (int l = 0; l < kLayers; l++) {
        const LayerSpec &L = kSpec[l];
        const bool last = l == OUT;
        if ((st = ptconv::fwd_prepare(&P.fwd[l], io[l].in, wbf_ptr(dn, l), L.cout, last ? kOutChannels : L.cout,
                                      bias_ptr(dn, l), last ? ptconv::EPI_F32 : ptconv::EPI_BF16, L.relu,
                                      io[l].out->ptr, io[l].octot, io[l].ocoff, nullptr, err,
                                      io[l].up && !separate_up ? io[l].up->ptr : nullptr, io[l].up_ctot,
                                      io[l].pool ? io[l].pool->ptr : nullptr, L.cout, 0)) != PT_OK)
            return st;
        P.x_of[l] = io[l].in;
    }
    if (train) {
        // gradient w.r.t. each layer's pre-activation, and where each data
        // gradient goes (mask = the ReLU output it passes back through)
        const Act g[kLayers] = {
            A(P.g_a0, 0, 32, 0, 32),   A(P.g_e0b, 0, 32, 0, 32), A(P.g_a1, 1, 48, 0, 48),  A(P.g_e1b, 1, 48, 0, 48),
            A(P.g_a2, 2, 64, 0, 64),   A(P.g_e2b, 2, 64, 0, 64), A(P.g_a3, 3, 128, 0, 128), A(P.g_e3b, 3, 128, 0, 128),
            A(P.g_b4, 4, 256, 0, 256), A(P.g_d3, 3, 128, 0, 128), A(P.g_d2, 2, 64, 0, 64), A(P.g_d1, 1, 48, 0, 48),
            A(P.g_d0, 0, 32, 0, 32),   A(P.g_out, 0, 16, 0, 16),
        };
        struct Back {
            const DevBuf *dst;
            int dctot;
            const DevBuf *mask;  // null: plain
        };
        const Back back[kLayers] = {
            {nullptr, 0, nullptr},  // e0a: no data gradient
            {&P.g_a0, 32, &P.a0},  {&P.g_p0, 32, nullptr}, {&P.g_a1, 48, &P.a1},  {&P.g_p1, 48, nullptr},
            {&P.g_a2, 64, &P.a2},  {&P.g_p2, 64, nullptr}, {&P.g_a3, 128, &P.a3}, {&P.g_p3, 128, nullptr},
            {&P.g_cat3, 384, nullptr}, {&P.g_cat2, 192, nullptr}, {&P.g_cat1, 112, nullptr},
            {&P.g_cat0, 80, nullptr},  {&P.g_d0, 32, &P.d0},
        };
        for (int l = 0; l < kLayers; l++) {
            const LayerSpec &L = kSpec[l];
            P.g_of[l] = g[l];
            if ((st = ptconv::wgrad_prepare(&P.wg[l], P.x_of[l], g[l], dn->grads.as<float>() + dn->w_off[l],
                                            dn->grads.as<float>() + dn->b_off[l], dn->num_sms, err)) != PT_OK)
                return st;
            if (!back[l].dst) continue;
            const int lvl = io[l].lvl;
            Act mask;
            if (back[l].mask) mask = A(*back[l].mask, lvl, L.cin, 0, L.cin);
            if ((st = ptconv::fwd_prepare(&P.bwd[l], g[l], wtbf_ptr(dn, l), L.cin, L.cin, nullptr,
                                          back[l].mask ? ptconv::EPI_BF16_MASK : ptconv::EPI_BF16, 0,
                                          back[l].dst->ptr, back[l].dctot, 0, back[l].mask ? &mask : nullptr,
                                          err)) != PT_OK)
                return st;
        }
    }
    P.n = n;
    P.h = h;
    P.w = w;
    P.train = train;
    return PT_OK;
}

#define PT_TRY(x)                          \
    do {                                   \
        int st_ = (x);                     \
        if (st_ != PT_OK) return st_;      \
    } while (0)

int run_forward(pt_denoiser *dn, Plan &P, cudaStream_t s) {
    const int n = P.n, h = P.h, w = P.w;
    auto pool = [&](const DevBuf &src, int sctot, int scoff, int c, int lvl, DevBuf &dst) {
        const int h2 = h >> (lvl + 1), w2 = w >> (lvl + 1);
        const long long tot = (long long)n * h2 * w2 * (c / 8);
        k_pool<<<grid_for(tot), 256, 0, s>>>(src.as<uint16_t>(), sctot, scoff, c, n, h2, w2, dst.as<uint16_t>());
    };
    PT_TRY(ptconv::fwd_launch(P.fwd[E0A], s));
    PT_TRY(ptconv::fwd_launch(P.fwd[E0B], s));
    if (!ptconv::fwd_pooled(P.fwd[E0B])) pool(P.cat0, 80, 48, 32, 0, P.p0);
    PT_TRY(ptconv::fwd_launch(P.fwd[E1A], s));
    PT_TRY(ptconv::fwd_launch(P.fwd[E1B], s));
    if (!ptconv::fwd_pooled(P.fwd[E1B])) pool(P.cat1, 112, 64, 48, 1, P.p1);
    PT_TRY(ptconv::fwd_launch(P.fwd[E2A], s));
    PT_TRY(ptconv::fwd_launch(P.fwd[E2B], s));
    pool(P.cat2, 192, 128, 64, 2, P.p2);
    PT_TRY(ptconv::fwd_launch(P.fwd[E3A], s));
    PT_TRY(ptconv::fwd_launch(P.fwd[E3B], s));
    pool(P.cat3, 384, 256, 128, 3, P.p3);
    auto up = [&](const DevBuf &lo, int c, int lvl, DevBuf &cat, int cat_ctot) {
        if (P.fused_up) return;
        const int hh = h >> lvl, ww = w >> lvl;
        const long long tot = (long long)n * hh * ww * (c / 8);
        k_upcat<<<grid_for(tot), 256, 0, s>>>(lo.as<uint16_t>(), c, n, hh, ww, cat.as<uint16_t>(), cat_ctot);
    };
    PT_TRY(ptconv::fwd_launch(P.fwd[BOT], s));
    up(P.b4, 256, 3, P.cat3, 384);
    PT_TRY(ptconv::fwd_launch(P.fwd[D3], s));
    up(P.d3, 128, 2, P.cat2, 192);
    PT_TRY(ptconv::fwd_launch(P.fwd[D2], s));
    up(P.d2, 64, 1, P.cat1, 112);
    PT_TRY(ptconv::fwd_launch(P.fwd[D1], s));
    up(P.d1, 48, 0, P.cat0, 80);
    PT_TRY(ptconv::fwd_launch(P.fwd[D0], s));
    PT_TRY(ptconv::fwd_launch(P.fwd[OUT], s));
    PT_CUDA_TRY(cudaGetLastError());
    return PT_OK;
}

// loss + backward; gradients accumulate into dn->grads (zeroed here)
int run_backward(pt_denoiser *dn, Plan &P, const float *target, cudaStream_t s) {
    const int n = P.n, h = P.h, w = P.w;
    const long long npix = (long long)n * h * w;
    PT_CUDA_TRY(cudaMemsetAsync(dn->grads.ptr, 0, dn->nparams * sizeof(float), s));
    k_loss<<<grid_for(npix), 256, 0, s>>>(P.out.as<float>(), P.x0.as<uint16_t>(), target, npix, 1.f / (3.f * npix),
                                          P.g_out.as<uint16_t>(), dn->loss.as<float>());
    // layer l: its weight (and bias) gradient and its data gradient both read
    // only the layer's output gradient, so the weight gradient runs on the
    // side stream while the data gradients continue on s
    const int nside = dn->side[1] ? 2 : dn->side[0] ? 1 : 0;
    int turn = 0;
    auto layer = [&](int l) -> int {
        cudaStream_t ws = nside ? dn->side[turn++ % nside] : s;
        if (nside) {
            PT_CUDA_TRY(cudaEventRecord(dn->ev_fork[l], s));
            PT_CUDA_TRY(cudaStreamWaitEvent(ws, dn->ev_fork[l], 0));
        }
        PT_TRY(ptconv::wgrad_launch(P.wg[l], ws));
        if (!P.wg[l].bias_fused) PT_TRY(ptconv::bias_grad_launch(P.g_of[l], dn->grads.as<float>() + dn->b_off[l], ws));
        if (l != E0A) PT_TRY(ptconv::fwd_launch(P.bwd[l], s));
        return PT_OK;
    };
    auto up_back = [&](const DevBuf &gcat, int cat_ctot, const DevBuf &lo, int c, int lvl, DevBuf &glo) {
        const int h2 = h >> (lvl + 1), w2 = w >> (lvl + 1);
        const long long tot = (long long)n * h2 * w2 * (c / 16);
        k_up_back<<<grid_for(tot), 256, 0, s>>>(gcat.as<uint16_t>(), cat_ctot, lo.as<uint16_t>(), c, n, h2, w2,
                                                 glo.as<uint16_t>());
    };
    auto skip_back = [&](const DevBuf &cat, const DevBuf &gcat, int cat_ctot, int coff, const DevBuf &gpool, int c,
                         int lvl, DevBuf &g) {
        const int hh = h >> lvl, ww = w >> lvl;
        const long long tot = (long long)n * hh * ww * (c / 16);
        k_skip_back<<<grid_for(tot), 256, 0, s>>>(cat.as<uint16_t>(), gcat.as<uint16_t>(), cat_ctot, coff,
                                                   gpool.as<uint16_t>(), c, n, hh, ww, g.as<uint16_t>());
    };
    PT_TRY(layer(OUT));
    PT_TRY(layer(D0));
    up_back(P.g_cat0, 80, P.d1, 48, 0, P.g_d1);
    PT_TRY(layer(D1));
    up_back(P.g_cat1, 112, P.d2, 64, 1, P.g_d2);
    PT_TRY(layer(D2));
    up_back(P.g_cat2, 192, P.d3, 128, 2, P.g_d3);
    PT_TRY(layer(D3));
    up_back(P.g_cat3, 384, P.b4, 256, 3, P.g_b4);
    PT_TRY(layer(BOT));
    skip_back(P.cat3, P.g_cat3, 384, 256, P.g_p3, 128, 3, P.g_e3b);
    PT_TRY(layer(E3B));
    PT_TRY(layer(E3A));
    skip_back(P.cat2, P.g_cat2, 192, 128, P.g_p2, 64, 2, P.g_e2b);
    PT_TRY(layer(E2B));
    PT_TRY(layer(E2A));
    skip_back(P.cat1, P.g_cat1, 112, 64, P.g_p1, 48, 1, P.g_e1b);
    PT_TRY(layer(E1B));
    PT_TRY(layer(E1A));
    skip_back(P.cat0, P.g_cat0, 80, 48, P.g_p0, 32, 0, P.g_e0b);
    PT_TRY(layer(E0B));
    PT_TRY(layer(E0A));
    for (int i = 0; i < nside; i++) {
        PT_CUDA_TRY(cudaEventRecord(dn->ev_join[i], dn->side[i]));
        PT_CUDA_TRY(cudaStreamWaitEvent(s, dn->ev_join[i], 0));
    }
    PT_CUDA_TRY(cudaGetLastError());
    return PT_OK;
}

int run_adam(pt_denoiser *dn, cudaStream_t s) {
    const pt_denoiser_opts &o = dn->opts;
    k_adam_begin<<<1, 1, 0, s>>>(dn->adam_state.as<float>(), o.beta1, o.beta2);
    AdamLayers L;
    long long largest = 0;
    for (int l = 0; l < kLayers; l++) {
        L.w_off[l] = static_cast<long long>(dn->w_off[l]);
        L.nw[l] = 9ll * kSpec[l].cin * kSpec[l].cout;
        L.wbf_off[l] = static_cast<long long>(dn->wbf_off[l]);
        L.cin[l] = kSpec[l].cin;
        L.cout[l] = kSpec[l].cout;
        largest = std::max(largest, L.nw[l] + L.cout[l]);
    }
    k_adam<<<grid_for(largest), 256, 0, s>>>(dn->params.as<float>(), dn->adam_m.as<float>(), dn->adam_v.as<float>(),
                                             dn->grads.as<float>(), L, dn->adam_state.as<float>(), o.beta1, o.beta2,
                                             o.eps, dn->wbf.as<uint16_t>(), dn->wtbf.as<uint16_t>());
    PT_CUDA_TRY(cudaGetLastError());
    return PT_OK;
}

int sync_weights(pt_denoiser *dn, cudaStream_t s) {
    for (int l = 0; l < kLayers; l++) {
        const LayerSpec &L = kSpec[l];
        const long long nw = 9ll * L.cin * L.cout;
        k_weights_to_bf16<<<grid_for(nw), 256, 0, s>>>(dn->params.as<float>() + dn->w_off[l], nw, L.cout, L.cin,
                                                       dn->wbf.as<uint16_t>() + dn->wbf_off[l],
                                                       dn->wtbf.as<uint16_t>() + dn->wbf_off[l]);
    }
    PT_CUDA_TRY(cudaGetLastError());
    return PT_OK;
}

int check_err(pt_denoiser *dn) {
    unsigned e = 0;
    PT_CUDA_TRY(cudaMemcpy(&e, dn->err.ptr, sizeof(e), cudaMemcpyDeviceToHost));
    if (e) {
        pt_set_error("denoiser: a convolution kernel's bounded wait ran out (code %u)", e);
        return PT_ERR_TIMEOUT;
    }
    return PT_OK;
}

// Orders the internal stream after the caller's stream.
int enter(pt_denoiser *dn, cudaStream_t caller) {
    PT_CUDA_TRY(cudaSetDevice(dn->device));
    PT_CUDA_TRY(cudaEventRecord(dn->ev_in, caller));
    PT_CUDA_TRY(cudaStreamWaitEvent(dn->stream, dn->ev_in, 0));
    return PT_OK;
}
int leave(pt_denoiser *dn, cudaStream_t caller) {
    PT_CUDA_TRY(cudaEventRecord(dn->ev_out, dn->stream));
    PT_CUDA_TRY(cudaStreamWaitEvent(caller, dn->ev_out, 0));
    return PT_OK;
}

void init_params(pt_denoiser *dn, std::vector<float> &p) {
    p.assign(dn->nparams, 0.f);
    uint64_t x = dn->opts.seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E5ull;
    auto next = [&x]() {  // splitmix64
        x += 0x9E3779B97F4A7C15ull;
        uint64_t z = x;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return static_cast<double>(z >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < kLayers; l++) {
        const LayerSpec &L = kSpec[l];
        const int cin_used = l == E0A ? 9 : L.cin;
        const int cout_used = l == OUT ? kOutChannels : L.cout;
        // He-uniform; the output layer starts at zero so that the network
        // starts as the identity on the noisy colour (residual output)
        const double bound = l == OUT ? 0.0 : std::sqrt(6.0 / (9.0 * cin_used));
        for (int co = 0; co < L.cout; co++)
            for (int t = 0; t < 9; t++)
                for (int ci = 0; ci < L.cin; ci++) {
                    const float v = static_cast<float>((2.0 * next() - 1.0) * bound);
                    if (co < cout_used && ci < cin_used) p[dn->w_off[l] + (static_cast<uint64_t>(co) * 9 + t) * L.cin + ci] = v;
                }
    }
}

int upload_params(pt_denoiser *dn, const float *host) {
    PT_CUDA_TRY(cudaSetDevice(dn->device));
    PT_CUDA_TRY(cudaMemcpy(dn->params.ptr, host, dn->nparams * sizeof(float), cudaMemcpyHostToDevice));
    PT_CUDA_TRY(cudaMemset(dn->adam_m.ptr, 0, dn->nparams * sizeof(float)));
    PT_CUDA_TRY(cudaMemset(dn->adam_v.ptr, 0, dn->nparams * sizeof(float)));
    const float state[4] = {0.f, 0.f, 0.f, dn->opts.lr};
    PT_CUDA_TRY(cudaMemcpy(dn->adam_state.ptr, state, sizeof(state), cudaMemcpyHostToDevice));
    PT_TRY(sync_weights(dn, 0));
    PT_CUDA_TRY(cudaDeviceSynchronize());
    return PT_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// C-ABI
// ---------------------------------------------------------------------------
extern "C" {

int pt_denoiser_create(pt_context *ctx, const pt_denoiser_opts *opts, pt_denoiser **out) {
    (void)cudaGetLastError();
    if (!ctx || !out) {
        pt_set_error("pt_denoiser_create: NULL argument");
        return PT_ERR_INVALID;
    }
    *out = nullptr;
    auto *dn = new pt_denoiser();
    dn->device = ctx->device;
    dn->num_sms = ctx->num_sms;
    dn->opts = opts ? *opts : pt_denoiser_opts{1e-3f, 0.9f, 0.999f, 1e-8f, 1};
    uint64_t off = 0, woff = 0;
    for (int l = 0; l < kLayers; l++) {
        dn->w_off[l] = off;
        off += 9ull * kSpec[l].cin * kSpec[l].cout;
        dn->b_off[l] = off;
        off += kSpec[l].cout;
        dn->wbf_off[l] = woff;
        woff += 9ull * kSpec[l].cin * kSpec[l].cout;
    }
    dn->nparams = off;
    dn->nweights = woff;
    auto fail = [&](int st) {
        pt_denoiser_destroy(dn);
        return st;
    };
    if (cudaSetDevice(dn->device) != cudaSuccess) {
        pt_set_error("pt_denoiser_create: cudaSetDevice failed");
        return fail(PT_ERR_CUDA);
    }
    int st;
    if ((st = dn->params.ensure(off * 4)) != PT_OK || (st = dn->adam_m.ensure(off * 4)) != PT_OK ||
        (st = dn->adam_v.ensure(off * 4)) != PT_OK || (st = dn->grads.ensure(off * 4)) != PT_OK ||
        (st = dn->wbf.ensure(woff * 2)) != PT_OK || (st = dn->wtbf.ensure(woff * 2)) != PT_OK ||
        (st = dn->adam_state.ensure(16)) != PT_OK || (st = dn->err.ensure(16)) != PT_OK ||
        (st = dn->loss.ensure(16)) != PT_OK || (st = dn->fallback.ensure(16)) != PT_OK)
        return fail(st);
    if (cudaMemset(dn->err.ptr, 0, 16) != cudaSuccess || cudaMemset(dn->loss.ptr, 0, 16) != cudaSuccess ||
        cudaStreamCreateWithFlags(&dn->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&dn->ev_in, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&dn->ev_out, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&dn->t0) != cudaSuccess || cudaEventCreate(&dn->t1) != cudaSuccess) {
        pt_set_error("pt_denoiser_create: CUDA set-up failed");
        return fail(PT_ERR_CUDA);
    }
    if (!getenv("PT_DENOISER_ONE_STREAM")) {  // the side stream for weight gradients
        const int nside = 1;  // a second side stream measured no faster (2.333 vs 2.332 ms per step)
        bool ok = true;
        for (int i = 0; ok && i < nside; i++)
            ok = cudaStreamCreateWithFlags(&dn->side[i], cudaStreamNonBlocking) == cudaSuccess &&
                 cudaEventCreateWithFlags(&dn->ev_join[i], cudaEventDisableTiming) == cudaSuccess;
        for (int l = 0; ok && l < kLayers; l++)
            ok = cudaEventCreateWithFlags(&dn->ev_fork[l], cudaEventDisableTiming) == cudaSuccess;
        if (!ok) {
            pt_set_error("pt_denoiser_create: CUDA set-up failed");
            return fail(PT_ERR_CUDA);
        }
    }
    std::vector<float> p;
    init_params(dn, p);
    if ((st = upload_params(dn, p.data())) != PT_OK) return fail(st);
    *out = dn;
    return PT_OK;
}

void pt_denoiser_destroy(pt_denoiser *dn) {
    if (!dn) return;
    cudaSetDevice(dn->device);
    if (dn->stream) cudaStreamSynchronize(dn->stream);
    dn->train_plan.release();
    dn->infer_plan.release();
    DevBuf *bufs[] = {&dn->params, &dn->adam_m, &dn->adam_v, &dn->grads, &dn->wbf,
                      &dn->wtbf,   &dn->adam_state, &dn->err, &dn->loss, &dn->fallback};
    for (DevBuf *b : bufs) b->release();
    if (dn->ev_in) cudaEventDestroy(dn->ev_in);
    if (dn->ev_out) cudaEventDestroy(dn->ev_out);
    if (dn->t0) cudaEventDestroy(dn->t0);
    if (dn->t1) cudaEventDestroy(dn->t1);
    for (cudaEvent_t e : dn->ev_fork)
        if (e) cudaEventDestroy(e);
    for (int i = 0; i < 2; i++) {
        if (dn->ev_join[i]) cudaEventDestroy(dn->ev_join[i]);
        if (dn->side[i]) {
            cudaStreamSynchronize(dn->side[i]);
            cudaStreamDestroy(dn->side[i]);
        }
    }
    if (dn->stream) cudaStreamDestroy(dn->stream);
    delete dn;
}

int pt_denoiser_num_params(const pt_denoiser *dn, uint64_t *count) {
    if (!dn || !count) {
        pt_set_error("pt_denoiser_num_params: NULL argument");
        return PT_ERR_INVALID;
    }
    *count = dn->nparams;
    return PT_OK;
}

int pt_denoiser_layer(const pt_denoiser *dn, uint32_t index, uint32_t *cin, uint32_t *cout, uint64_t *offset) {
    if (!dn || index >= static_cast<uint32_t>(kLayers)) {
        pt_set_error("pt_denoiser_layer: bad denoiser or index %u", index);
        return PT_ERR_INVALID;
    }
    if (cin) *cin = kSpec[index].cin;
    if (cout) *cout = kSpec[index].cout;
    if (offset) *offset = dn->w_off[index];
    return PT_OK;
}

int pt_denoiser_get_params(const pt_denoiser *dn, float *params) {
    (void)cudaGetLastError();
    if (!dn || !params) {
        pt_set_error("pt_denoiser_get_params: NULL argument");
        return PT_ERR_INVALID;
    }
    PT_CUDA_TRY(cudaSetDevice(dn->device));
    PT_CUDA_TRY(cudaStreamSynchronize(dn->stream));
    PT_CUDA_TRY(cudaMemcpy(params, dn->params.ptr, dn->nparams * sizeof(float), cudaMemcpyDeviceToHost));
    return PT_OK;
}

int pt_denoiser_set_params(pt_denoiser *dn, const float *params) {
    (void)cudaGetLastError();
    if (!dn || !params) {
        pt_set_error("pt_denoiser_set_params: NULL argument");
        return PT_ERR_INVALID;
    }
    PT_CUDA_TRY(cudaSetDevice(dn->device));
    PT_CUDA_TRY(cudaStreamSynchronize(dn->stream));
    return upload_params(dn, params);
}

int pt_denoiser_get_state(const pt_denoiser *dn, float *state) {
    (void)cudaGetLastError();
    if (!dn || !state) {
        pt_set_error("pt_denoiser_get_state: NULL argument");
        return PT_ERR_INVALID;
    }
    PT_CUDA_TRY(cudaSetDevice(dn->device));
    PT_CUDA_TRY(cudaStreamSynchronize(dn->stream));
    const size_t n = dn->nparams;
    PT_CUDA_TRY(cudaMemcpy(state, dn->adam_m.ptr, n * sizeof(float), cudaMemcpyDeviceToHost));
    PT_CUDA_TRY(cudaMemcpy(state + n, dn->adam_v.ptr, n * sizeof(float), cudaMemcpyDeviceToHost));
    PT_CUDA_TRY(cudaMemcpy(state + 2 * n, dn->adam_state.ptr, 4 * sizeof(float), cudaMemcpyDeviceToHost));
    return PT_OK;
}

int pt_denoiser_set_state(pt_denoiser *dn, const float *state) {
    (void)cudaGetLastError();
    if (!dn || !state) {
        pt_set_error("pt_denoiser_set_state: NULL argument");
        return PT_ERR_INVALID;
    }
    const size_t n = dn->nparams;
    if (!(state[2 * n] >= 0.f) || !(state[2 * n + 3] >= 0.f)) {
        pt_set_error("pt_denoiser_set_state: bad step count or step size");
        return PT_ERR_INVALID;
    }
    PT_CUDA_TRY(cudaSetDevice(dn->device));
    PT_CUDA_TRY(cudaStreamSynchronize(dn->stream));
    PT_CUDA_TRY(cudaMemcpy(dn->adam_m.ptr, state, n * sizeof(float), cudaMemcpyHostToDevice));
    PT_CUDA_TRY(cudaMemcpy(dn->adam_v.ptr, state + n, n * sizeof(float), cudaMemcpyHostToDevice));
    PT_CUDA_TRY(cudaMemcpy(dn->adam_state.ptr, state + 2 * n, 4 * sizeof(float), cudaMemcpyHostToDevice));
    return PT_OK;
}

int pt_denoiser_set_lr(pt_denoiser *dn, float lr) {
    (void)cudaGetLastError();
    if (!dn || !(lr >= 0.f)) {
        pt_set_error("pt_denoiser_set_lr: bad denoiser or step size");
        return PT_ERR_INVALID;
    }
    PT_CUDA_TRY(cudaSetDevice(dn->device));
    PT_CUDA_TRY(cudaMemcpyAsync(dn->adam_state.as<float>() + 3, &lr, sizeof(float), cudaMemcpyHostToDevice, dn->stream));
    PT_CUDA_TRY(cudaStreamSynchronize(dn->stream));
    dn->opts.lr = lr;
    return PT_OK;
}

int pt_denoiser_get_grads(const pt_denoiser *dn, float *grads) {
    (void)cudaGetLastError();
    if (!dn || !grads) {
        pt_set_error("pt_denoiser_get_grads: NULL argument");
        return PT_ERR_INVALID;
    }
    PT_CUDA_TRY(cudaSetDevice(dn->device));
    PT_CUDA_TRY(cudaStreamSynchronize(dn->stream));
    PT_CUDA_TRY(cudaMemcpy(grads, dn->grads.ptr, dn->nparams * sizeof(float), cudaMemcpyDeviceToHost));
    return PT_OK;
}

int pt_denoiser_compute_grads(pt_denoiser *dn, const void *input_f16, const float *target, uint32_t n, uint32_t height,
                              uint32_t width, float *loss, void *stream) {
    (void)cudaGetLastError();
    if (!dn || !input_f16 || !target) {
        pt_set_error("pt_denoiser_compute_grads: NULL argument");
        return PT_ERR_INVALID;
    }
    cudaStream_t caller = static_cast<cudaStream_t>(stream);
    PT_TRY(enter(dn, caller));
    Plan &P = dn->train_plan;
    PT_TRY(plan_prepare(dn, P, n, height, width, true));
    cudaStream_t s = dn->stream;
    const long long npix = (long long)n * height * width;
    PT_CUDA_TRY(cudaMemsetAsync(dn->loss.ptr, 0, 16, s));
    k_pack_input<<<grid_for(npix), 256, 0, s>>>(static_cast<const __half *>(input_f16), npix, P.x0.as<uint16_t>());
    PT_TRY(run_forward(dn, P, s));
    PT_TRY(run_backward(dn, P, target, s));
    float sum = 0.f;
    PT_CUDA_TRY(cudaMemcpyAsync(&sum, dn->loss.ptr, sizeof(float), cudaMemcpyDeviceToHost, s));
    PT_CUDA_TRY(cudaStreamSynchronize(s));
    PT_CUDA_TRY(cudaMemset(dn->loss.ptr, 0, 16));
    dn->loss_steps = 0;
    PT_TRY(check_err(dn));
    if (loss) *loss = sum / (3.f * npix);
    return leave(dn, caller);
}

int pt_denoiser_train_step(pt_denoiser *dn, const void *input_f16, const float *target, uint32_t n, uint32_t crop,
                           void *stream) {
    pt_nvtx::Range nv("pt_denoiser_train_step");
    (void)cudaGetLastError();
    if (!dn || !input_f16 || !target) {
        pt_set_error("pt_denoiser_train_step: NULL argument");
        return PT_ERR_INVALID;
    }
    cudaStream_t caller = static_cast<cudaStream_t>(stream);
    PT_TRY(enter(dn, caller));
    Plan &P = dn->train_plan;
    PT_TRY(plan_prepare(dn, P, n, crop, crop, true));
    cudaStream_t s = dn->stream;
    const long long npix = (long long)n * crop * crop;
    PT_CUDA_TRY(cudaMemcpyAsync(P.in_stage.ptr, input_f16, npix * 9 * 2, cudaMemcpyDeviceToDevice, s));
    PT_CUDA_TRY(cudaMemcpyAsync(P.tgt_stage.ptr, target, npix * 3 * sizeof(float), cudaMemcpyDeviceToDevice, s));
    if (!P.graph) {
        cudaGraph_t g = nullptr;
        PT_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        k_pack_input<<<grid_for(npix), 256, 0, s>>>(P.in_stage.as<__half>(), npix, P.x0.as<uint16_t>());
        int st = run_forward(dn, P, s);
        if (st == PT_OK) st = run_backward(dn, P, P.tgt_stage.as<float>(), s);
        if (st == PT_OK) st = run_adam(dn, s);
        cudaError_t ce = cudaStreamEndCapture(s, &g);
        if (st != PT_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (ce != cudaSuccess) {
            pt_set_error("denoiser: graph capture failed: %s", cudaGetErrorString(ce));
            return PT_ERR_CUDA;
        }
        ce = cudaGraphInstantiate(&P.graph, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            P.graph = nullptr;
            pt_set_error("denoiser: graph instantiation failed: %s", cudaGetErrorString(ce));
            return PT_ERR_CUDA;
        }
    }
    PT_CUDA_TRY(cudaGraphLaunch(P.graph, s));
    dn->loss_steps++;
    return leave(dn, caller);
}

int pt_denoiser_read_loss(pt_denoiser *dn, float *mean_loss) {
    (void)cudaGetLastError();
    if (!dn || !mean_loss) {
        pt_set_error("pt_denoiser_read_loss: NULL argument");
        return PT_ERR_INVALID;
    }
    PT_CUDA_TRY(cudaSetDevice(dn->device));
    PT_CUDA_TRY(cudaStreamSynchronize(dn->stream));
    float sum = 0.f;
    PT_CUDA_TRY(cudaMemcpy(&sum, dn->loss.ptr, sizeof(float), cudaMemcpyDeviceToHost));
    PT_CUDA_TRY(cudaMemset(dn->loss.ptr, 0, 16));
    const Plan &P = dn->train_plan;
    const double count = 3.0 * P.n * P.h * P.w * std::max<uint32_t>(dn->loss_steps, 1);
    *mean_loss = static_cast<float>(sum / count);
    dn->loss_steps = 0;
    return check_err(dn);
}

int pt_denoiser_forward(pt_denoiser *dn, const void *input_f16, uint32_t n, uint32_t height, uint32_t width, float *out,
                        void *stream) {
    (void)cudaGetLastError();
    if (!dn || !input_f16 || !out) {
        pt_set_error("pt_denoiser_forward: NULL argument");
        return PT_ERR_INVALID;
    }
    cudaStream_t caller = static_cast<cudaStream_t>(stream);
    PT_TRY(enter(dn, caller));
    Plan &P = dn->infer_plan;
    PT_TRY(plan_prepare(dn, P, n, height, width, false));
    cudaStream_t s = dn->stream;
    const long long npix = (long long)n * height * width;
    k_pack_input<<<grid_for(npix), 256, 0, s>>>(static_cast<const __half *>(input_f16), npix, P.x0.as<uint16_t>());
    PT_TRY(run_forward(dn, P, s));
    k_expm1<<<grid_for(npix * 3), 256, 0, s>>>(P.out.as<float>(), P.x0.as<uint16_t>(), npix, out);
    PT_CUDA_TRY(cudaGetLastError());
    PT_CUDA_TRY(cudaStreamSynchronize(s));
    PT_TRY(check_err(dn));
    return leave(dn, caller);
}

int pt_denoise(pt_denoiser *dn, const pt_denoise_io *io, void *stream) {
    pt_nvtx::Range nv("pt_denoise");
    (void)cudaGetLastError();
    if (!dn || !io || !io->color || !io->albedo || !io->normal || !io->output || !io->width || !io->height) {
        pt_set_error("pt_denoise: NULL argument or empty frame");
        return PT_ERR_INVALID;
    }
    if (io->flags & ~(uint32_t)PT_DENOISE_FLIP_ENSEMBLE) {
        pt_set_error("pt_denoise: unknown flags 0x%x", io->flags);
        return PT_ERR_INVALID;
    }
    cudaStream_t caller = static_cast<cudaStream_t>(stream);
    PT_TRY(enter(dn, caller));
    const int w = io->width, h = io->height;
    const int wp = (w + 15) / 16 * 16, hp = (h + 15) / 16 * 16;
    Plan &P = dn->infer_plan;
    PT_TRY(plan_prepare(dn, P, 1, hp, wp, false));
    cudaStream_t s = dn->stream;
    const int tile = io->tile ? static_cast<int>(io->tile) : 16;
    const int tiles = ((w + tile - 1) / tile) * ((h + tile - 1) / tile);
    PT_CUDA_TRY(cudaMemsetAsync(dn->fallback.ptr, 0, 4, s));
    PT_CUDA_TRY(cudaEventRecord(dn->t0, s));
    const bool ensemble = (io->flags & PT_DENOISE_FLIP_ENSEMBLE) != 0;
    const long long npix = (long long)wp * hp;
    if (ensemble) PT_TRY(P.out_acc.ensure(npix * 3 * sizeof(float)));
    k_pack_frame<<<grid_for((long long)wp * hp), 256, 0, s>>>(reinterpret_cast<const float4 *>(io->color), io->albedo,
                                                               io->normal, w, h, wp, hp, P.x0.as<uint16_t>());
    PT_TRY(run_forward(dn, P, s));
    const float *o = P.out.as<float>();
    if (ensemble) {  // second pass on the mirror image, averaged in the network's output (log residual) space
        PT_CUDA_TRY(cudaMemcpyAsync(P.out_acc.ptr, P.out.ptr, npix * 3 * sizeof(float), cudaMemcpyDeviceToDevice, s));
        k_mirror_x0<<<grid_for(npix / 2), 256, 0, s>>>(P.x0.as<uint16_t>(), wp, hp);
        PT_TRY(run_forward(dn, P, s));
        k_mirror_average<<<grid_for(npix), 256, 0, s>>>(P.out_acc.as<float>(), P.out.as<float>(), wp, npix);
        k_mirror_x0<<<grid_for(npix / 2), 256, 0, s>>>(P.x0.as<uint16_t>(), wp, hp);
        o = P.out_acc.as<float>();
    }
    k_denoise_out<<<tiles, 256, 0, s>>>(reinterpret_cast<const float4 *>(io->color), o,
                                        P.x0.as<uint16_t>(), w, h, wp, tile,
                                        io->fallback_rel, io->fallback_sigma, reinterpret_cast<float4 *>(io->output),
                                        io->tile_fallback, dn->fallback.as<unsigned>());
    PT_CUDA_TRY(cudaGetLastError());
    PT_CUDA_TRY(cudaEventRecord(dn->t1, s));
    PT_CUDA_TRY(cudaEventSynchronize(dn->t1));
    unsigned fb = 0;
    PT_CUDA_TRY(cudaMemcpy(&fb, dn->fallback.ptr, 4, cudaMemcpyDeviceToHost));
    float ms = 0.f;
    PT_CUDA_TRY(cudaEventElapsedTime(&ms, dn->t0, dn->t1));
    dn->stats.tiles = static_cast<uint32_t>(tiles);
    dn->stats.fallback_tiles = fb;
    dn->stats.last_ms = ms;
    PT_TRY(check_err(dn));
    return leave(dn, caller);
}

int pt_denoise_get_stats(const pt_denoiser *dn, pt_denoise_stats *out) {
    if (!dn || !out) {
        pt_set_error("pt_denoise_get_stats: NULL argument");
        return PT_ERR_INVALID;
    }
    *out = dn->stats;
    return PT_OK;
}

int pt_denoise_pack(const float *color, const float *albedo, const float *normal, uint32_t width, uint32_t height,
                    void *out_f16, void *stream) {
    (void)cudaGetLastError();
    if (!color || !albedo || !normal || !out_f16) {
        pt_set_error("pt_denoise_pack: NULL argument");
        return PT_ERR_INVALID;
    }
    const long long npix = (long long)width * height;
    k_pack_f16<<<grid_for(npix), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<const float4 *>(color), albedo, normal, npix, static_cast<__half *>(out_f16));
    PT_CUDA_TRY(cudaGetLastError());
    return PT_OK;
}

// ---- convolution test entry points -------------------------------------
static int conv_err_buf(DevBuf &e) {
    int st = e.ensure(16);
    if (st != PT_OK) return st;
    PT_CUDA_TRY(cudaMemset(e.ptr, 0, 16));
    return PT_OK;
}
static int conv_check(DevBuf &e, cudaStream_t s) {
    PT_CUDA_TRY(cudaStreamSynchronize(s));
    unsigned v = 0;
    PT_CUDA_TRY(cudaMemcpy(&v, e.ptr, 4, cudaMemcpyDeviceToHost));
    if (v) {
        pt_set_error("convolution: a bounded wait ran out (code %u)", v);
        return PT_ERR_TIMEOUT;
    }
    return PT_OK;
}

int pt_conv_set_wait_limit(uint64_t wait_ns, uint32_t stall_next) {
    ptconv::set_wait_limit(wait_ns, stall_next != 0);
    return PT_OK;
}

int pt_conv3x3_forward(const void *x, uint32_t n, uint32_t h, uint32_t w, uint32_t cin, const void *weight,
                       const float *bias, uint32_t cout, int relu, int out_f32, void *y, void *stream) {
    (void)cudaGetLastError();
    if (!x || !weight || !y || cin % 16 || !cout) {
        pt_set_error("pt_conv3x3_forward: NULL pointer or cin not a multiple of 16");
        return PT_ERR_INVALID;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    DevBuf e;
    int st = conv_err_buf(e);
    ptconv::FwdOp op;
    Act in;
    in.ptr = const_cast<void *>(x);
    in.n = n;
    in.h = h;
    in.w = w;
    in.ctot = cin;
    in.c = cin;
    const int cout_pad = (cout + 15) / 16 * 16;
    if (st == PT_OK)
        st = ptconv::fwd_prepare(&op, in, weight, cout_pad, cout, bias, out_f32 ? ptconv::EPI_F32 : ptconv::EPI_BF16,
                                 relu, y, cout, 0, nullptr, e.as<unsigned>());
    if (st == PT_OK) st = ptconv::fwd_launch(op, s);
    if (st == PT_OK) st = conv_check(e, s);
    e.release();
    return st;
}

int pt_conv3x3_backward_data(const void *dy, uint32_t n, uint32_t h, uint32_t w, uint32_t cout, const void *weight,
                             uint32_t cin, const void *mask, void *dx, void *stream) {
    (void)cudaGetLastError();
    if (!dy || !weight || !dx || cin % 16 || !cout) {
        pt_set_error("pt_conv3x3_backward_data: NULL pointer or cin not a multiple of 16");
        return PT_ERR_INVALID;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int cout_pad = (cout + 15) / 16 * 16;
    DevBuf e, wt;
    int st = conv_err_buf(e);
    if (st == PT_OK) st = wt.ensure(9ull * cin * cout_pad * 2);
    if (st == PT_OK)
        st = ptconv::flip_transpose_launch(static_cast<const uint16_t *>(weight), cout_pad, cin, wt.as<uint16_t>(), s);
    Act g;
    g.ptr = const_cast<void *>(dy);
    g.n = n;
    g.h = h;
    g.w = w;
    g.ctot = cout_pad;
    g.c = cout_pad;
    Act m = g;
    m.ptr = const_cast<void *>(mask);
    m.ctot = cin;
    m.c = cin;
    ptconv::FwdOp op;
    if (st == PT_OK)
        st = ptconv::fwd_prepare(&op, g, wt.ptr, cin, cin, nullptr, mask ? ptconv::EPI_BF16_MASK : ptconv::EPI_BF16, 0,
                                 dx, cin, 0, mask ? &m : nullptr, e.as<unsigned>());
    if (st == PT_OK) st = ptconv::fwd_launch(op, s);
    if (st == PT_OK) st = conv_check(e, s);
    e.release();
    wt.release();
    return st;
}

int pt_conv3x3_backward_weights(const void *x, uint32_t n, uint32_t h, uint32_t w, uint32_t cin, const void *dy,
                                uint32_t cout, float *dweight, float *dbias, void *stream) {
    (void)cudaGetLastError();
    if (!x || !dy || !dweight || cin % 16 || cout % 16 || !cout) {
        pt_set_error("pt_conv3x3_backward_weights: NULL pointer or channels not multiples of 16");
        return PT_ERR_INVALID;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int dev = 0, sms = 0;
    PT_CUDA_TRY(cudaGetDevice(&dev));
    PT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    DevBuf e;
    int st = conv_err_buf(e);
    Act xa;
    xa.ptr = const_cast<void *>(x);
    xa.n = n;
    xa.h = h;
    xa.w = w;
    xa.ctot = cin;
    xa.c = cin;
    Act ga = xa;
    ga.ptr = const_cast<void *>(dy);
    ga.ctot = cout;
    ga.c = cout;
    ptconv::WgradOp op;
    if (st == PT_OK) st = ptconv::wgrad_prepare(&op, xa, ga, dweight, dbias, sms, e.as<unsigned>());
    if (st == PT_OK) st = ptconv::wgrad_launch(op, s);
    if (st == PT_OK && dbias && !op.bias_fused) st = ptconv::bias_grad_launch(ga, dbias, s);
    if (st == PT_OK) st = conv_check(e, s);
    e.release();
    return st;
}

}  // extern "C"
