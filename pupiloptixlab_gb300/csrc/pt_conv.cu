// pt_conv.cu -- BF16 3x3 convolutions as implicit GEMMs on tcgen05 tensor
// cores, operands brought into shared memory by TMA (no multicast), FP32
// accumulators in tensor memory.  Interface and GEMM shapes: pt_conv.h.
//
// Tiling.  Accumulator tiles have 128 rows:
//   forward / data gradient: 128 pixels (one 128-wide row segment, or
//     128 / W whole rows of a narrow image) x n_tile output channels.  Persistent
//     CTAs of 6 warps walk the tiles: warp 0 streams operands into a ring of
//     `stages` buffers, warp 1 issues the MMAs into one of two accumulators,
//     warps 2-5 run the epilogue of the other (k_conv_fwd_persistent);
//   weight gradient: 128 (tap, input channel) rows x n_tile output channels,
//     accumulated over a range of pixel tiles and added to the FP32 result,
//     one CTA of 4 warps per (row tile, channel tile, pixel range): thread 0
//     loads, thread 32 issues the MMAs, all four warps read the accumulator
//     (warp w owns TMEM lanes 32w..32w+31).
//
// Shared-memory operand layouts are the canonical swizzled ones for a row of
// R = 2 * KC bytes (R = 32, 64, 128 B, TMA swizzle of the same width):
//   K-major (forward A = pixels x channels, B = out channels x channels):
//     rows R bytes apart, 8-row groups SBO = 8R apart; a 16-element K slice
//     starts 32 B further along the row.
//   MN-major (weight gradient, A = channels x pixels, B = channels x pixels):
//     each TMA box holds 128 pixels (K) x KC channels (MN) as 128 rows of R
//     bytes; 8-pixel groups are SBO = 8R apart, consecutive KC-channel blocks
//     LBO = 128R apart; a 16-pixel K slice starts 16R further on.
// The zero padding of the convolution comes from TMA's out-of-bounds fill:
// the box for tap (dy, dx) starts at (x0 + dx - 1, y0 + dy - 1).
//
// Every wait is bounded (%globaltimer, 2 s): on expiry the kernel records a
// code in *err, stops issuing work, lets issued copies and MMAs drain (again
// with a bound), frees its tensor memory and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>

#include "pt_conv.h"
#include "pt_internal.h"

namespace ptconv {

constexpr int kMaxStages = 8;
constexpr uint64_t kWaitNs = 2000000000ull;

// ---------------------------------------------------------------------------
// device primitives (inline PTX)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ uint64_t gtimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for the phase with the given parity to complete: false after
// limit_ns of %globaltimer, or as soon as *abort is set (another warp of the
// CTA gave up), so that a failing CTA leaves within one limit.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, bool backoff = false,
                                          uint64_t limit_ns = kWaitNs, const volatile int *abort = nullptr) {
    if (mbar_try(bar, parity)) return true;
    const uint64_t t0 = gtimer();
    while (!mbar_try(bar, parity)) {
        if (backoff) __nanosleep(128);
        if (gtimer() - t0 > limit_ns) return false;
        if (abort && *abort) return false;
    }
    return true;
}
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap *map, uint32_t bar, int c0, int c1, int c2,
                                            int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, uint32_t bar, int c0, int c1) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(cols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void umma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
// 32 lanes x 16 consecutive 32-bit columns: thread t of the warp gets lane
// (warp base + t), columns col..col+15.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor (tcgen05): start, leading and stride byte
// offsets in 16-byte units, descriptor version 1 at bit 46, swizzle mode in
// bits 61-63 (2 = 128 B, 4 = 64 B, 6 = 32 B).
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo, uint32_t swz) {
    return static_cast<uint64_t>((addr >> 4) & 0x3FFFu) | (static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16) |
           (static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46) | (static_cast<uint64_t>(swz) << 61);
}
// Instruction descriptor, kind::f16: FP32 D, BF16 A and B, K-major (0) or
// MN-major (1) operands, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n, bool a_mn, bool b_mn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16) |
           (static_cast<uint32_t>(n >> 3) << 17) | (static_cast<uint32_t>(m >> 4) << 24);
}
template <int KC>
__host__ __device__ constexpr uint32_t swz_mode() {
    return KC == 64 ? 2u : KC == 32 ? 4u : 6u;
}

__device__ __forceinline__ void record_error(unsigned *err, unsigned code) {
    if (err) atomicOr(err, code);
}

__device__ __forceinline__ uint16_t f2bf(float f) {
    __nv_bfloat16 h = __float2bfloat16_rn(f);
    return *reinterpret_cast<uint16_t *>(&h);
}

// 32-byte global accesses (256-bit loads and stores, sm_100 and later): the
// 16 BF16 channels a thread handles per step are one full sector.
__device__ __forceinline__ void ld_global_v8(const uint16_t *p, uint4 &a, uint4 &b) {
    asm volatile("ld.global.v8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(a.x), "=r"(a.y), "=r"(a.z), "=r"(a.w), "=r"(b.x), "=r"(b.y), "=r"(b.z), "=r"(b.w)
                 : "l"(p));
}
__device__ __forceinline__ void st_global_v8(uint16_t *p, uint4 a, uint4 b) {
    asm volatile("st.global.v8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "r"(a.x), "r"(a.y), "r"(a.z),
                 "r"(a.w), "r"(b.x), "r"(b.y), "r"(b.z), "r"(b.w)
                 : "memory");
}

// Forward epilogue: accumulator row `tid` = pixel (x0 + tid % tile_w,
// y0 + tid / tile_w); warp w reads TMEM lanes 32w..32w+31, 16 columns at a time.
__device__ __forceinline__ void fwd_epilogue(const FwdArgs &a, uint32_t tmem, int tid, int warp, int img, int x0, int y0,
                                             int n0, bool ok) {
    const int px = tid % a.tile_w, py = tid / a.tile_w;
    const int x = x0 + px, y = y0 + py;
    const bool valid = ok && py < a.tile_rows && x < a.W && y < a.H;
    const size_t pix = ((size_t)img * a.H + (valid ? y : 0)) * a.W + (valid ? x : 0);
    const uint32_t trow = tmem + (static_cast<uint32_t>(warp * 32) << 16);
    for (int c = 0; c < a.n_tile; c += 16) {
        float v[16];
        tmem_ld16(trow + c, v);
        const int ch0 = n0 + c;
        if (!valid || ch0 >= a.cout) continue;
        const int nvalid = min(16, a.cout - ch0);
        if (a.epi == EPI_F32) {
            float *o = static_cast<float *>(a.out) + pix * a.out_ctot + a.out_coff + ch0;
            for (int i = 0; i < nvalid; i++) o[i] = v[i] + (a.bias ? a.bias[ch0 + i] : 0.f);
            continue;
        }
        if (a.epi == EPI_BF16) {
            float b[16];
            if (a.bias && nvalid == 16 && a.bias16) {  // 16 biases in four 16-byte loads
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const float4 q = __ldg(reinterpret_cast<const float4 *>(a.bias + ch0) + i);
                    b[4 * i] = q.x;
                    b[4 * i + 1] = q.y;
                    b[4 * i + 2] = q.z;
                    b[4 * i + 3] = q.w;
                }
            } else {
#pragma unroll
                for (int i = 0; i < 16; i++) b[i] = (a.bias && i < nvalid) ? a.bias[ch0 + i] : 0.f;
            }
#pragma unroll
            for (int i = 0; i < 16; i++) {
                const float f = v[i] + b[i];
                v[i] = a.relu ? fmaxf(f, 0.f) : f;
            }
        } else {
            const uint16_t *m = a.mask + pix * a.mask_ctot + a.mask_coff + ch0;
            if (nvalid == 16) {
                uint4 q0, q1;
                if (a.wide_io) {
                    ld_global_v8(m, q0, q1);
                } else {
                    q0 = *reinterpret_cast<const uint4 *>(m);
                    q1 = *reinterpret_cast<const uint4 *>(m + 8);
                }
                const uint16_t *h0 = reinterpret_cast<const uint16_t *>(&q0), *h1 = reinterpret_cast<const uint16_t *>(&q1);
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    if (!(h0[i] != 0 && (h0[i] & 0x8000u) == 0)) v[i] = 0.f;
                    if (!(h1[i] != 0 && (h1[i] & 0x8000u) == 0)) v[i + 8] = 0.f;
                }
            } else {
                for (int i = 0; i < nvalid; i++)
                    if (!(m[i] != 0 && (m[i] & 0x8000u) == 0)) v[i] = 0.f;
            }
        }
        uint16_t *o = static_cast<uint16_t *>(a.out) + pix * a.out_ctot + a.out_coff + ch0;
        // the four up-sampled copies (pixel (2y + i, 2x + j) of the 2H x 2W tensor)
        uint16_t *u = a.up ? a.up + (((size_t)img * 2 * a.H + 2 * y) * 2 * a.W + 2 * x) * a.up_ctot + ch0 : nullptr;
        const size_t urow = static_cast<size_t>(2 * a.W) * a.up_ctot;
        if (nvalid == 16) {
            uint4 q0, q1;
            uint32_t *w0 = reinterpret_cast<uint32_t *>(&q0), *w1 = reinterpret_cast<uint32_t *>(&q1);
#pragma unroll
            for (int i = 0; i < 4; i++) {
                w0[i] = f2bf(v[2 * i]) | (static_cast<uint32_t>(f2bf(v[2 * i + 1])) << 16);
                w1[i] = f2bf(v[8 + 2 * i]) | (static_cast<uint32_t>(f2bf(v[8 + 2 * i + 1])) << 16);
            }
            if (a.wide_io) {
                st_global_v8(o, q0, q1);
                if (u) {
                    st_global_v8(u, q0, q1);
                    st_global_v8(u + a.up_ctot, q0, q1);
                    st_global_v8(u + urow, q0, q1);
                    st_global_v8(u + urow + a.up_ctot, q0, q1);
                }
            } else {
                reinterpret_cast<uint4 *>(o)[0] = q0;
                reinterpret_cast<uint4 *>(o)[1] = q1;
                for (int k = 0; u && k < 4; k++) {
                    uint16_t *uk = u + (k >> 1) * urow + (k & 1) * a.up_ctot;
                    reinterpret_cast<uint4 *>(uk)[0] = q0;
                    reinterpret_cast<uint4 *>(uk)[1] = q1;
                }
            }
        } else {
            for (int i = 0; i < nvalid; i++) {
                const uint16_t b = f2bf(v[i]);
                o[i] = b;
                for (int k = 0; u && k < 4; k++) u[(k >> 1) * urow + (k & 1) * a.up_ctot + i] = b;
            }
        }
    }

}

// Two-row halo tile with the pooled output (EPI_BF16, cout a multiple of 16,
// 32-byte aligned rows): thread `tid` holds pixel x = x0 + tid of rows y0 and
// y0 + 1 (accumulators tmem and tmem + n_tile), its neighbour lane x ^ 1.
// Each row is written as fwd_epilogue writes it; the even lane of each pair
// writes the average of the four BF16 outputs, summed in the order
// (y0, x), (y0, x + 1), (y0 + 1, x), (y0 + 1, x + 1).
__device__ __forceinline__ void fwd_epilogue_pool2(const FwdArgs &a, uint32_t tmem, int tid, int warp, int img, int x0,
                                                   int y0, int n0) {
    const int x = x0 + tid;
    const bool valid = x < a.W && y0 < a.H;
    const size_t pix0 = ((size_t)img * a.H + (valid ? y0 : 0)) * a.W + (valid ? x : 0);
    const size_t ppix = ((size_t)img * (a.H / 2) + (valid ? y0 / 2 : 0)) * (a.W / 2) + (valid ? x / 2 : 0);
    const uint32_t trow = tmem + (static_cast<uint32_t>(warp * 32) << 16);
    for (int c = 0; c < a.n_tile; c += 16) {
        float v[2][16];
        tmem_ld16(trow + c, v[0]);
        tmem_ld16(trow + a.n_tile + c, v[1]);
        const int ch0 = n0 + c;
        if (ch0 >= a.cout) continue;  // uniform across the warp
        float b[16];
        if (a.bias && a.bias16) {
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const float4 q = __ldg(reinterpret_cast<const float4 *>(a.bias + ch0) + i);
                b[4 * i] = q.x;
                b[4 * i + 1] = q.y;
                b[4 * i + 2] = q.z;
                b[4 * i + 3] = q.w;
            }
        } else {
#pragma unroll
            for (int i = 0; i < 16; i++) b[i] = a.bias ? a.bias[ch0 + i] : 0.f;
        }
        uint32_t w[2][8];
#pragma unroll
        for (int r = 0; r < 2; r++)
#pragma unroll
            for (int i = 0; i < 8; i++) {
                float f0 = v[r][2 * i] + b[2 * i], f1 = v[r][2 * i + 1] + b[2 * i + 1];
                if (a.relu) {
                    f0 = fmaxf(f0, 0.f);
                    f1 = fmaxf(f1, 0.f);
                }
                w[r][i] = f2bf(f0) | (static_cast<uint32_t>(f2bf(f1)) << 16);
            }
        uint32_t pw[8];
#pragma unroll
        for (int i = 0; i < 8; i++) {
            float acc[2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const float own0 = __uint_as_float((w[0][i] >> (16 * h)) << 16);
                const float own1 = __uint_as_float((w[1][i] >> (16 * h)) << 16);
                const float nb0 = __shfl_xor_sync(0xffffffffu, own0, 1);
                const float nb1 = __shfl_xor_sync(0xffffffffu, own1, 1);
                acc[h] = 0.25f * ((((0.f + own0) + nb0) + own1) + nb1);  // k_pool's order, from 0
            }
            pw[i] = f2bf(acc[0]) | (static_cast<uint32_t>(f2bf(acc[1])) << 16);
        }
        if (!valid) continue;
#pragma unroll
        for (int r = 0; r < 2; r++) {
            uint16_t *o = static_cast<uint16_t *>(a.out) + (pix0 + (size_t)r * a.W) * a.out_ctot + a.out_coff + ch0;
            st_global_v8(o, make_uint4(w[r][0], w[r][1], w[r][2], w[r][3]), make_uint4(w[r][4], w[r][5], w[r][6], w[r][7]));
        }
        if ((tid & 1) == 0) {
            uint16_t *o = a.pool + ppix * a.pool_ctot + a.pool_coff + ch0;
            st_global_v8(o, make_uint4(pw[0], pw[1], pw[2], pw[3]), make_uint4(pw[4], pw[5], pw[6], pw[7]));
        }
    }
}

// ---------------------------------------------------------------------------
// halo operand layout (forward / data gradient, images at least 128 pixels wide)
// ---------------------------------------------------------------------------
// The pixel tile is a 128-pixel row segment.  Per 16-channel chunk one TMA box
// brings its 3 x 130-pixel neighbourhood (the segment and a one-pixel border,
// zero outside the image) as 32-byte pixel rows in the 32-byte-swizzled
// K-major layout, pixels in row-major order.  The A operand of tap (dy, dx) is
// the same box read from pixel row dy * 130 + dx on (stride byte offset =
// 256 B between 8-row groups): the tensor cores apply the swizzle to the
// absolute shared-memory address, as the TMA wrote it, so a start at any
// 32-byte row reads the right data.  The input is thus read from L2 once per
// chunk instead of once per tap.  (PT_CONV_HALO_PLANES=1 selects the earlier
// layout: two TMA boxes per chunk into non-swizzled planes of 8 channels,
// 16 bytes per pixel, leading byte offset = plane size.)  B holds the chunk's weights for all nine
// taps (32-byte swizzle, one TMA box per tap).  When one channel tile covers
// every output channel and all (chunk, tap) weight boxes fit in
// kMaxResidentWeights bytes, they are loaded once per CTA ahead of the ring
// (on their own barrier) and the stages carry only the A box.
// A tile may cover two output rows (halo_rows = 2: a 4-row box, two M = 128
// accumulators sharing each B operand), so that every input row crosses L2
// twice per pass instead of three times; the second row's A operand is the
// same box read one box row (130 pixels) further on.
constexpr int kHaloW = 130;
__host__ __device__ constexpr int halo_box_bytes(int rows) { return kHaloW * (rows + 2) * 16; }
__host__ __device__ constexpr int halo_plane_bytes(int rows) { return (halo_box_bytes(rows) + 1023) / 1024 * 1024; }
__host__ __device__ constexpr int halo_b_tap_bytes(int n_tile) { return (n_tile * 32 + 1023) / 1024 * 1024; }
constexpr int kMaxResidentWeights = 64 * 1024;

// ---------------------------------------------------------------------------
// persistent forward / data-gradient kernel
// ---------------------------------------------------------------------------
// One CTA per SM slot walks the output tiles (pixel tile x output-channel
// tile) with a stride of gridDim.x.  Warp 0 streams operands into a ring of
// `stages` buffers across tile boundaries, warp 1 issues the MMAs into one of
// two accumulators in tensor memory (2 x n_tile columns), and warps 2-5 run
// the epilogue of tile i from one accumulator while the MMAs of tile i + 1
// fill the other.  Warp w of the epilogue reads TMEM lanes 32 * (w % 4) + 0..31.
// HALO: the A operand comes from one 3 x 130-pixel halo box per 16-channel
// chunk (width >= 128, see above); otherwise one box per (tap, chunk).
template <int KC, bool HALO>
__global__ void __launch_bounds__(192, 1)
    k_conv_fwd_persistent(const __grid_constant__ CUtensorMap act, const __grid_constant__ CUtensorMap wgt,
                          const FwdArgs a) {
    constexpr int R = KC * 2;
    constexpr uint32_t SWZ = swz_mode<KC>();
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t bars[2 * kMaxStages + 7];
    __shared__ uint32_t tmem_slot;
    __shared__ int s_fail;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const bool wres = HALO && a.wres_bytes > 0;  // weights resident ahead of the ring
    const uint32_t wbase = (smem_u32(smem_raw) + 1023u) & ~1023u;
    const uint32_t base = wbase + (wres ? static_cast<uint32_t>(a.wres_bytes) : 0u);
    const int S = a.stages;
    const int tiles_img = a.tiles_x * a.tiles_y;
    const int n_n = a.n_tiles_n;
    const int total = a.n_img * tiles_img * n_n;
    const int nk = HALO ? a.nchunks : 9 * a.nchunks;  // stages per tile
    const int a_bytes = HALO ? a.halo_a_bytes : 128 * R;
    const int b_tap = HALO ? halo_b_tap_bytes(a.n_tile) : 0;
    const int hrows = HALO ? a.halo_rows : 1;  // output rows (accumulators) per tile
    const uint32_t tx_bytes = HALO ? static_cast<uint32_t>(a.halo_a_tx + (wres ? 0 : 9 * a.n_tile * R))
                                   : static_cast<uint32_t>(a.tile_w * a.tile_rows * R + a.n_tile * R);
    const uint32_t bar0 = smem_u32(bars);
    auto full = [&](int s) { return bar0 + 8u * s; };
    auto empty = [&](int s) { return bar0 + 8u * (kMaxStages + s); };
    auto acc_full = [&](int b) { return bar0 + 8u * (2 * kMaxStages + b); };
    auto acc_empty = [&](int b) { return bar0 + 8u * (2 * kMaxStages + 2 + b); };
    const uint32_t wbar = bar0 + 8u * (2 * kMaxStages + 4);  // resident weights landed
    const uint32_t sbar = bar0 + 8u * (2 * kMaxStages + 5);  // never arrived at: the stall test waits on it
    const uint32_t mdone = bar0 + 8u * (2 * kMaxStages + 6);  // MMAs of a failing CTA completed
    const uint64_t lim = a.wait_ns;
    auto tile_of = [&](int t, int &img, int &x0, int &y0, int &n0) {
        const int pt = t / n_n;
        n0 = (t - pt * n_n) * a.n_tile;
        img = pt / tiles_img;
        const int r = pt - img * tiles_img;
        x0 = (r % a.tiles_x) * a.tile_w;
        y0 = (r / a.tiles_x) * a.tile_rows;
    };

    if (warp == 0) tmem_alloc(smem_u32(&tmem_slot), a.tmem_cols);
    if (tid == 32) {
        for (int s = 0; s < S; s++) {
            mbar_init(full(s), 1);
            mbar_init(empty(s), 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(acc_full(b), 1);
            mbar_init(acc_empty(b), 128);
        }
        mbar_init(wbar, 1);
        mbar_init(sbar, 1);
        mbar_init(mdone, 1);
        mbar_fence_init();
        s_fail = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    volatile int *fail = &s_fail;

    if (warp == 0) {
        if (lane == 0) {  // producer
            if (wres) {  // every (chunk, tap) weight box once: b_tap apart, chunk-major
                mbar_expect_tx(wbar, static_cast<uint32_t>(a.nchunks * 9 * a.n_tile * R));
                for (int k = 0; k < a.nchunks; k++)
                    for (int tap = 0; tap < 9; tap++)
                        tma_load_2d(wbase + static_cast<uint32_t>((k * 9 + tap) * b_tap), &wgt, wbar,
                                    tap * a.cin + k * 16, 0);
            }
            int kg = 0;  // stages issued so far (ring position and phase)
            for (int t = blockIdx.x; t < total && !*fail; t += gridDim.x) {
                int img, x0, y0, n0;
                tile_of(t, img, x0, y0, n0);
                for (int k = 0; k < nk; k++, kg++) {
                    const int s = kg % S;
                    if (kg >= S && !mbar_wait(empty(s), ((kg / S) - 1) & 1, false, lim, fail)) {
                        record_error(a.err, 1u);
                        *fail = 1;
                        break;
                    }
                    const uint32_t sa = base + s * a.stage_bytes, sb = sa + a_bytes;
                    if ((sa | sb) & 1023u) {  // never with a layout fwd_prepare accepted: give up, bounded
                        record_error(a.err, 8u);
                        *fail = 1;
                        break;
                    }
                    mbar_expect_tx(full(s), tx_bytes);
                    if (HALO) {
                        if (a.halo_sw32) {
                            tma_load_4d(sa, &act, full(s), k * 16, x0 - 1, y0 - 1, img);
                        } else {
                            tma_load_4d(sa, &act, full(s), k * 16, x0 - 1, y0 - 1, img);
                            tma_load_4d(sa + a.halo_plane_bytes, &act, full(s), k * 16 + 8, x0 - 1, y0 - 1, img);
                        }
                        if (!wres)
                            for (int tap = 0; tap < 9; tap++)
                                tma_load_2d(sb + tap * b_tap, &wgt, full(s), tap * a.cin + k * 16, n0);
                    } else {
                        const int tap = k / a.nchunks, ch = k - tap * a.nchunks;
                        const int dy = tap / 3, dx = tap - dy * 3;
                        tma_load_4d(sa, &act, full(s), ch * KC, x0 + dx - 1, y0 + dy - 1, img);
                        tma_load_2d(sb, &wgt, full(s), tap * a.cin + ch * KC, n0);
                    }
                }
            }
            // drain: every copy this thread issued has landed before the CTA
            // leaves (the last issue on each ring slot, and the resident
            // weights), also when another warp gave up; within the normal limit
            for (int k = kg - S; k < kg; k++)
                if (k >= 0) (void)mbar_wait(full(k % S), (k / S) & 1, true);
            if (wres) (void)mbar_wait(wbar, 0, true);
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer
            const uint32_t idesc = idesc_bf16(128, a.n_tile, false, false);
            if (a.stall && !mbar_wait(sbar, 0, true, lim)) {  // the stall test: this wait always runs out
                record_error(a.err, 2u);
                *fail = 1;
            }
            if (wres && !*fail && !mbar_wait(wbar, 0, false, lim, fail)) {
                record_error(a.err, 2u);
                *fail = 1;
            }
            int kg = 0, j = 0;
            for (int t = blockIdx.x; t < total && !*fail; t += gridDim.x, j++) {
                const int buf = j & 1;
                if (!mbar_wait(acc_empty(buf), ((j >> 1) & 1) ^ 1, false, lim, fail)) {  // epilogue of tile j - 2 done
                    record_error(a.err, 2u);
                    *fail = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t d = tmem + static_cast<uint32_t>(buf * hrows * a.n_tile);
                for (int k = 0; k < nk; k++, kg++) {
                    const int s = kg % S;
                    if (!mbar_wait(full(s), (kg / S) & 1, false, lim, fail)) {
                        record_error(a.err, 2u);
                        *fail = 1;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t sa = base + s * a.stage_bytes;
                    const uint32_t sb = wres ? wbase + static_cast<uint32_t>(k * 9 * b_tap) : sa + a_bytes;
                    if (HALO) {
#pragma unroll
                        for (int tap = 0; tap < 9; tap++) {
                            const int dy = tap / 3, dx = tap - 3 * (tap / 3);
                            const uint64_t db = sdesc(sb + tap * b_tap, 16u, 8u * R, SWZ);
                            for (int r = 0; r < hrows; r++) {
                                uint64_t da;
                                if (a.halo_sw32) {  // 32-byte rows, 32-byte swizzle, 8-row groups 256 B apart
                                    da = sdesc(sa + 32u * ((dy + r) * kHaloW + dx), 16u, 256u, 6u);
                                } else {
                                    da = sdesc(sa + 16u * ((dy + r) * kHaloW + dx),
                                               static_cast<uint32_t>(a.halo_plane_bytes), 128u, 0u);
                                }
                                umma_bf16(d + static_cast<uint32_t>(r * a.n_tile), da, db, idesc,
                                          (k | tap) != 0 ? 1u : 0u);
                            }
                        }
                    } else {
#pragma unroll
                        for (int q = 0; q < KC / 16; q++) {
                            const uint64_t da = sdesc(sa + 32u * q, 16u, 8u * R, SWZ);
                            const uint64_t db = sdesc(sb + 32u * q, 16u, 8u * R, SWZ);
                            umma_bf16(d, da, db, idesc, (k | q) != 0 ? 1u : 0u);
                        }
                    }
                    umma_commit(empty(s));
                }
                if (*fail) break;
                umma_commit(acc_full(buf));
            }
            if (*fail && kg > 0) {  // let the MMAs already issued finish before tensor memory is freed
                umma_commit(mdone);
                (void)mbar_wait(mdone, 0, true);
            }
        }
    } else {  // epilogue warps 2-5
        const int quad = warp & 3;
        const int row = quad * 32 + lane;
        int j = 0;
        for (int t = blockIdx.x; t < total; t += gridDim.x, j++) {
            const int buf = j & 1;
            const bool ok = mbar_wait(acc_full(buf), (j >> 1) & 1, true, lim, fail);
            if (!ok) {
                if (row == 0) record_error(a.err, 4u);
                break;
            }
            tc_fence_after();
            int img, x0, y0, n0;
            tile_of(t, img, x0, y0, n0);
            if (HALO && a.pool)
                fwd_epilogue_pool2(a, tmem + static_cast<uint32_t>(buf * 2 * a.n_tile), row, quad, img, x0, y0, n0);
            else
                for (int r = 0; r < hrows; r++)
                    fwd_epilogue(a, tmem + static_cast<uint32_t>((buf * hrows + r) * a.n_tile), row, quad, img, x0,
                                 y0 + r, n0, true);
            tc_fence_before();
            mbar_arrive(acc_empty(buf));
        }
    }
    __syncwarp();
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, a.tmem_cols);
}

// ---------------------------------------------------------------------------
// weight-gradient kernel
// ---------------------------------------------------------------------------
template <int KCA, int KCB>
__global__ void __launch_bounds__(128, 1)
    k_conv_wgrad(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap gmap, const WgradArgs a) {
    constexpr int RA = KCA * 2, RB = KCB * 2;
    constexpr uint32_t SWZA = swz_mode<KCA>(), SWZB = swz_mode<KCB>();
    constexpr int A_BLOCKS = 128 / KCA;
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t bars[2 * kMaxStages + 1];
    __shared__ uint32_t tmem_slot;
    __shared__ int s_issued, s_consumed, s_fail;

    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
    const int S = a.stages;
    const int blk0 = blockIdx.x * A_BLOCKS;
    const int nblk = min(A_BLOCKS, 9 * a.nchunks_a - blk0);
    const int n0 = blockIdx.y * a.n_tile;
    const int nbb = a.n_tile / KCB;
    const int t_begin = blockIdx.z * a.tiles_per_split;
    const int nk = max(0, min(a.total_tiles, t_begin + a.tiles_per_split) - t_begin);
    const int a_bytes = 128 * 128 * 2;
    const int tile_px = a.tile_w * a.tile_rows;  // pixels one box delivers
    const uint32_t tx_bytes = static_cast<uint32_t>(nblk * tile_px * RA + nbb * tile_px * RB);
    const int tiles_img = a.tiles_x * a.tiles_y;
    const uint32_t bar0 = smem_u32(bars);
    auto full = [&](int s) { return bar0 + 8u * s; };
    auto empty = [&](int s) { return bar0 + 8u * (kMaxStages + s); };
    const uint32_t done = bar0 + 8u * (2 * kMaxStages);

    // The last M tile's spare A chunk holds BF16 ones in every stage (no box
    // writes it), so its D rows are the sums of gy over the pixels: the bias
    // gradient from the same MMAs.
    const bool ones = a.db != nullptr && a.ones_row >= 0 && blockIdx.x == gridDim.x - 1;
    if (a.zero_fill || ones) {  // zero fill: rows that no box covers must read as zero pixels
        const int ob = ones ? (a.ones_row / KCA) * 128 * RA : a.stage_bytes;  // ones chunk offset in a stage
        uint8_t *p = smem_raw + (base - smem_u32(smem_raw));
        for (int i = tid; i < S * a.stage_bytes / 16; i += blockDim.x) {
            const int off = (i * 16) % a.stage_bytes;
            if (off >= ob && off < ob + 128 * RA)
                reinterpret_cast<uint4 *>(p)[i] = make_uint4(0x3f803f80u, 0x3f803f80u, 0x3f803f80u, 0x3f803f80u);
            else if (a.zero_fill)
                reinterpret_cast<uint4 *>(p)[i] = make_uint4(0, 0, 0, 0);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(smem_u32(&tmem_slot), a.tmem_cols);
    if (tid == 32) {
        for (int s = 0; s < S; s++) {
            mbar_init(full(s), 1);
            mbar_init(empty(s), 1);
        }
        mbar_init(done, 1);
        mbar_fence_init();
        s_issued = 0;
        s_consumed = 0;
        s_fail = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    if (tid == 0) {
        int k = 0;
        for (; k < nk; k++) {
            const int s = k % S;
            if (k >= S && !mbar_wait(empty(s), ((k / S) - 1) & 1, false, a.wait_ns)) {
                record_error(a.err, 1u);
                s_fail = 1;
                break;
            }
            if (*reinterpret_cast<volatile int *>(&s_fail)) break;
            const int tile = t_begin + k;
            const int img = tile / tiles_img, t = tile - img * tiles_img;
            const int x0 = (t % a.tiles_x) * a.tile_w, y0 = (t / a.tiles_x) * a.tile_rows;
            const uint32_t sa = base + s * a.stage_bytes, sb = sa + a_bytes;
            mbar_expect_tx(full(s), tx_bytes);
            for (int q = 0; q < nblk; q++) {
                const int b = blk0 + q;
                const int tap = b / a.nchunks_a, ch = b - tap * a.nchunks_a;
                const int dy = tap / 3, dx = tap - dy * 3;
                tma_load_4d(sa + q * 128 * RA, &xmap, full(s), ch * KCA, x0 + dx - 1, y0 + dy - 1, img);
            }
            for (int q = 0; q < nbb; q++) tma_load_4d(sb + q * 128 * RB, &gmap, full(s), n0 + q * KCB, x0, y0, img);
        }
        s_issued = k;
    } else if (tid == 32) {
        const uint32_t idesc = idesc_bf16(128, a.n_tile, true, true);
        int k = 0;
        for (; k < nk; k++) {
            const int s = k % S;
            if (!mbar_wait(full(s), (k / S) & 1, false, a.wait_ns)) {
                record_error(a.err, 2u);
                s_fail = 1;
                break;
            }
            tc_fence_after();
            const uint32_t sa = base + s * a.stage_bytes, sb = sa + a_bytes;
#pragma unroll
            for (int j = 0; j < 8; j++) {  // 16 pixels per MMA
                const uint64_t da = sdesc(sa + 16u * RA * j, 128u * RA, 8u * RA, SWZA);
                const uint64_t db = sdesc(sb + 16u * RB * j, 128u * RB, 8u * RB, SWZB);
                umma_bf16(tmem, da, db, idesc, (k | j) != 0 ? 1u : 0u);
            }
            umma_commit(empty(s));
        }
        s_consumed = k;
        umma_commit(done);
    }
    __syncwarp();
    const bool ok = nk > 0 && mbar_wait(done, 0, true, a.wait_ns);
    if (!ok && nk > 0 && tid == 0) record_error(a.err, 4u);
    tc_fence_after();

    // epilogue: row tid = A row (tap, ci) index g; dw[co][g] += D[tid][co - n0]
    const int g = blk0 * KCA + tid;
    const bool valid = ok && tid < nblk * KCA;
    const bool bias_row = ok && ones && tid == a.ones_row;  // db[co] += D[ones_row][co - n0]
    const uint32_t trow = tmem + (static_cast<uint32_t>(warp * 32) << 16);
    const size_t kdim = 9 * static_cast<size_t>(a.cin);
    for (int c = 0; c < a.n_tile; c += 16) {
        float v[16];
        tmem_ld16(trow + c, v);
        if (!valid && !bias_row) continue;
        float *dst = valid ? a.dw + g : a.db;
        const size_t stride = valid ? kdim : 1;
        for (int i = 0; i < 16; i++) {
            const int co = n0 + c + i;
            if (co < a.cout) atomicAdd(dst + co * stride, v[i]);
        }
    }

    tc_fence_before();
    __syncthreads();
    if (tid == 0 && s_fail) {
        for (int k = s_consumed; k < s_issued; k++) (void)mbar_wait(full(k % S), (k / S) & 1);
    }
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, a.tmem_cols);
}

// ---------------------------------------------------------------------------
// small kernels
// ---------------------------------------------------------------------------
__global__ void k_bias_grad(const uint16_t *g, int ctot, int coff, int c, long long npix, float *db) {
    extern __shared__ float sacc[];
    const int per = blockDim.x / c;  // pixels per pass
    const int lane_c = threadIdx.x % c, lane_p = threadIdx.x / c;
    float acc = 0.f;
    if (lane_p < per) {
        for (long long p = (long long)blockIdx.x * per + lane_p; p < npix; p += (long long)gridDim.x * per) {
            uint32_t bits = static_cast<uint32_t>(g[p * ctot + coff + lane_c]) << 16;
            acc += __uint_as_float(bits);
        }
    }
    sacc[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x < c) {
        float s = 0.f;
        for (int i = 0; i < per; i++) s += sacc[i * c + threadIdx.x];
        atomicAdd(db + threadIdx.x, s);
    }
}

__global__ void k_flip_transpose(const uint16_t *w, int cout, int cin, uint16_t *wt) {
    const long long n = 9ll * cout * cin;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int ci = static_cast<int>(i % cin);
        const int tap = static_cast<int>((i / cin) % 9);
        const int co = static_cast<int>(i / (9ll * cin));
        wt[(static_cast<long long>(ci) * 9 + (8 - tap)) * cout + co] = w[i];
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

CUtensorMapSwizzle swizzle_for(int kc) {
    return kc == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : kc == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B;
}

struct Tiling {
    int tile_w, tile_rows, tiles_x, tiles_y;
};
Tiling tiling_for(int h, int w) {
    Tiling t;
    if (w >= 128) {
        t.tile_w = 128;
        t.tile_rows = 1;
    } else {
        t.tile_w = w;
        t.tile_rows = std::min(128 / w, h);
    }
    t.tiles_x = (w + t.tile_w - 1) / t.tile_w;
    t.tiles_y = (h + t.tile_rows - 1) / t.tile_rows;
    return t;
}

int act_map_box(CUtensorMap *m, const Act &a, int box_c, int box_w, int box_h, CUtensorMapSwizzle swz, int kc) {
    auto fn = encode_fn();
    if (!fn) {
        pt_set_error("cuTensorMapEncodeTiled is not available from the driver");
        return PT_ERR_CUDA;
    }
    char *p = static_cast<char *>(a.ptr) + 2ull * a.coff;
    if ((reinterpret_cast<uintptr_t>(p) & 15) || (a.ctot % 8) || (a.c % kc)) {
        pt_set_error("activation tensor: base, channel stride or channel count misaligned (ctot %d coff %d c %d)", a.ctot,
                     a.coff, a.c);
        return PT_ERR_INVALID;
    }
    cuuint64_t dims[4] = {(cuuint64_t)a.c, (cuuint64_t)a.w, (cuuint64_t)a.h, (cuuint64_t)a.n};
    cuuint64_t strides[3] = {2ull * a.ctot, 2ull * a.ctot * a.w, 2ull * a.ctot * a.w * a.h};
    cuuint32_t box[4] = {(cuuint32_t)box_c, (cuuint32_t)box_w, (cuuint32_t)box_h, 1};
    cuuint32_t es[4] = {1, 1, 1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, p, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    swz, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        pt_set_error("cuTensorMapEncodeTiled (activation %dx%dx%dx%d, box %dx%dx%d) failed: %d", a.n, a.h, a.w, a.c,
                     box_c, box_w, box_h, static_cast<int>(r));
        return PT_ERR_CUDA;
    }
    return PT_OK;
}

// Tile boxes: kc channels x the pixel tile, swizzled to the row width.
int act_map(CUtensorMap *m, const Act &a, int kc, const Tiling &t) {
    return act_map_box(m, a, kc, t.tile_w, t.tile_rows, swizzle_for(kc), kc);
}

int wgt_map(CUtensorMap *m, const void *w, int kdim, int rows, int kc, int n_tile) {
    auto fn = encode_fn();
    if (!fn) {
        pt_set_error("cuTensorMapEncodeTiled is not available from the driver");
        return PT_ERR_CUDA;
    }
    if ((reinterpret_cast<uintptr_t>(w) & 15) || (kdim % 8)) {
        pt_set_error("weight tensor misaligned");
        return PT_ERR_INVALID;
    }
    cuuint64_t dims[2] = {(cuuint64_t)kdim, (cuuint64_t)rows};
    cuuint64_t strides[1] = {2ull * kdim};
    cuuint32_t box[2] = {(cuuint32_t)kc, (cuuint32_t)n_tile};
    cuuint32_t es[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(w), dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(kc), CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        pt_set_error("cuTensorMapEncodeTiled (weights %dx%d, box %dx%d) failed: %d", rows, kdim, kc, n_tile,
                     static_cast<int>(r));
        return PT_ERR_CUDA;
    }
    return PT_OK;
}

int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
            n = 1;
    }
    return n;
}

bool getenv_flag(const char *name) {
    const char *v = getenv(name);
    return v && *v && *v != '0';
}

int pow2_cols(int n) {
    int c = 32;
    while (c < n) c <<= 1;
    return c;
}

// Dynamic shared memory for `stages` buffers, raised where needed so that no
// more CTAs share an SM than its 512 tensor-memory columns can hold.
int smem_request(int stages, int stage_bytes, int tmem_cols) {
    const int by_stages = stages * stage_bytes + 1024;
    const int max_ctas = 512 / tmem_cols;
    const int floor_bytes = (228 * 1024) / (max_ctas + 1) + 1024;
    return std::max(by_stages, max_ctas >= 32 ? 0 : floor_bytes);
}

// Raises a kernel instantiation's dynamic shared-memory limit to `bytes`
// when a launch needs more than it was given so far (per process).
template <class K>
int set_smem_attr(K kernel, int bytes) {
    static std::mutex mu;
    static std::map<const void *, int> raised;  // kernel -> limit set so far
    std::lock_guard<std::mutex> lock(mu);
    const void *key = reinterpret_cast<const void *>(kernel);
    auto it = raised.find(key);
    const int have = it == raised.end() ? 48 * 1024 : it->second;
    if (bytes <= have) return PT_OK;
    PT_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    raised[key] = bytes;
    return PT_OK;
}

}  // namespace

int pick_kc(int c) {
    if (c % 64 == 0) return 64;
    if (c % 32 == 0) return 32;
    return 16;
}

// Limit of the kernels' bounded waits (pt_conv_set_wait_limit; 0 = kWaitNs)
// and the one-shot request to stall the next forward convolution.
static std::atomic<unsigned long long> g_wait_ns{0};
static std::atomic<int> g_stall_next{0};
unsigned long long wait_limit_ns() {
    const unsigned long long v = g_wait_ns.load();
    return v ? v : kWaitNs;
}
bool take_stall_request() { return g_stall_next.exchange(0) != 0; }
void set_wait_limit(unsigned long long ns, bool stall_next) {
    g_wait_ns.store(ns);
    g_stall_next.store(stall_next ? 1 : 0);
}

int fwd_prepare(FwdOp *op, const Act &in, const void *w, int w_rows, int cout, const float *bias, int epi, int relu,
                void *out, int out_ctot, int out_coff, const Act *mask, unsigned *err, void *up, int up_ctot,
                void *pool, int pool_ctot, int pool_coff) {
    if (in.c <= 0 || in.c % 16 || cout <= 0 || in.n <= 0 || in.h <= 0 || in.w <= 0) {
        pt_set_error("conv forward: channel counts must be positive multiples of 16 (cin %d, cout %d)", in.c, cout);
        return PT_ERR_INVALID;
    }
    if (epi == EPI_BF16_MASK && (!mask || mask->n != in.n || mask->h != in.h || mask->w != in.w)) {
        pt_set_error("conv forward: mask tensor missing or of the wrong shape");
        return PT_ERR_INVALID;
    }
    if (epi != EPI_F32 && ((out_ctot % 8) || (out_coff % 8))) {
        pt_set_error("conv forward: bf16 output channel stride/offset must be multiples of 8");
        return PT_ERR_INVALID;
    }
    const bool halo = in.w >= 128 && !getenv_flag("PT_CONV_NO_HALO");
    const int kc = halo ? 16 : pick_kc(in.c);
    const Tiling t = tiling_for(in.h, in.w);
    const int cout_pad = (cout + 15) / 16 * 16;
    int ntiles = (cout_pad + 255) / 256;
    int n_tile = ((cout_pad / ntiles) + 15) / 16 * 16;
    ntiles = (cout_pad + n_tile - 1) / n_tile;
    // two output rows per halo tile whenever both rows' double-buffered
    // accumulators fit the 512 tensor-memory columns, even at one CTA per SM
    // (training step 2.174 vs 2.243 ms against two rows only up to 256
    // columns); PT_CONV_HALO_ROWS=1..4 overrides
    int halo_rows = pow2_cols(4 * n_tile) <= 512 ? 2 : 1;
    if (const char *e = getenv("PT_CONV_HALO_ROWS")) halo_rows = std::min(std::max(atoi(e), 1), 4);
    while (halo_rows > 1 && pow2_cols(2 * halo_rows * n_tile) > 512) halo_rows--;
    int st;
    if (halo) {
        if (!getenv_flag("PT_CONV_HALO_PLANES")) {
            if ((st = act_map_box(&op->act, in, 16, kHaloW, halo_rows + 2, CU_TENSOR_MAP_SWIZZLE_32B, 16)) != PT_OK)
                return st;
        } else if ((st = act_map_box(&op->act, in, 8, kHaloW, halo_rows + 2, CU_TENSOR_MAP_SWIZZLE_NONE, 8)) != PT_OK) {
            return st;
        }
    } else if ((st = act_map(&op->act, in, kc, t)) != PT_OK) {
        return st;
    }
    if ((st = wgt_map(&op->wgt, w, 9 * in.c, w_rows, kc, n_tile)) != PT_OK) return st;
    FwdArgs &a = op->args;
    memset(&a, 0, sizeof(a));
    a.n_img = in.n;
    a.H = in.h;
    a.W = in.w;
    a.tile_w = t.tile_w;
    a.tile_rows = t.tile_rows;
    a.tiles_x = t.tiles_x;
    a.tiles_y = t.tiles_y;
    a.cin = in.c;
    a.nchunks = in.c / kc;
    a.n_tile = n_tile;
    a.cout = cout;
    a.n_tiles_n = ntiles;
    a.tmem_cols = pow2_cols(2 * (halo ? halo_rows : 1) * n_tile);  // double-buffered accumulators
    a.halo_rows = halo_rows;
    a.halo_box_bytes = halo_box_bytes(halo_rows);
    a.halo_plane_bytes = halo_plane_bytes(halo_rows);
    a.halo_sw32 = halo && !getenv_flag("PT_CONV_HALO_PLANES");
    a.halo_a_tx = a.halo_sw32 ? 2 * halo_box_bytes(halo_rows) : 2 * a.halo_box_bytes;
    a.halo_a_bytes = a.halo_sw32 ? (a.halo_a_tx + 1023) / 1024 * 1024 : 2 * a.halo_plane_bytes;
    const int wres_bytes = a.nchunks * 9 * halo_b_tap_bytes(n_tile);
    a.wres_bytes = (halo && ntiles == 1 && wres_bytes <= kMaxResidentWeights && !getenv_flag("PT_CONV_NO_RESIDENT"))
                       ? wres_bytes : 0;
    a.stage_bytes = halo ? a.halo_a_bytes + (a.wres_bytes ? 0 : 9 * halo_b_tap_bytes(n_tile))
                         : (128 * 2 * kc + n_tile * 2 * kc + 1023) / 1024 * 1024;
    // CTAs per SM the ring is sized for (PT_CONV_FWD_CTAS=1..4 overrides):
    // training step at batch 16 x 256^2 2.308 / 2.251 / 2.298 ms for 2 / 3 / 4
    int max_ctas = 3;
    if (const char *e = getenv("PT_CONV_FWD_CTAS")) max_ctas = std::min(std::max(atoi(e), 1), 4);
    const int target_ctas = std::min(512 / a.tmem_cols, max_ctas);
    const int budget = (225 * 1024) / target_ctas - 2048 - a.wres_bytes;
    a.stages = std::max(2, std::min(kMaxStages, budget / a.stage_bytes));
    // every TMA destination (stage, A box or plane, weight tap region) on a
    // 1 KiB boundary of the 1 KiB-aligned ring; the producer checks it again
    if (a.stage_bytes % 1024 || a.wres_bytes % 1024 ||
        (halo && (a.halo_a_bytes % 1024 || a.halo_plane_bytes % 1024 || halo_b_tap_bytes(n_tile) % 1024))) {
        pt_set_error("conv forward: shared-memory layout off 1 KiB boundaries");
        return PT_ERR_INVALID;
    }
    if (halo) {
        a.tile_w = 128;
        a.tile_rows = halo_rows;
        a.tiles_x = (in.w + 127) / 128;
        a.tiles_y = (in.h + halo_rows - 1) / halo_rows;
    }
    a.epi = epi;
    a.relu = relu;
    a.bias = bias;
    a.out = out;
    a.out_ctot = out_ctot;
    a.out_coff = out_coff;
    if (mask) {
        a.mask = static_cast<const uint16_t *>(mask->ptr);
        a.mask_ctot = mask->ctot;
        a.mask_coff = mask->coff;
    }
    // 32-byte accesses when every 16-channel group of the output (and mask)
    // starts on a 32-byte boundary
    auto al32 = [](const void *ptr, int ctot, int coff) {
        return (reinterpret_cast<uintptr_t>(ptr) % 32) == 0 && ctot % 16 == 0 && coff % 16 == 0;
    };
    a.bias16 = bias && (reinterpret_cast<uintptr_t>(bias) % 16) == 0 ? 1 : 0;
    if (up && epi == EPI_BF16) {
        if (up_ctot < cout || up_ctot % 8) {
            pt_set_error("conv forward: up-sampled output needs at least cout channels, a multiple of 8");
            return PT_ERR_INVALID;
        }
        a.up = static_cast<uint16_t *>(up);
        a.up_ctot = up_ctot;
    }
    // the 2x2 average pooling of the output, in the epilogue of two-row halo
    // tiles (both rows of a pixel pair are in one thread, the pair in
    // neighbouring lanes); otherwise the caller pools
    if (pool && halo && halo_rows == 2 && epi == EPI_BF16 && cout % 16 == 0 && in.w % 128 == 0 && in.h % 2 == 0 &&
        ntiles == 1 && al32(pool, pool_ctot, pool_coff) && al32(out, out_ctot, out_coff) &&
        !getenv_flag("PT_CONV_NO_FUSED_POOL")) {  // (the pooled epilogue writes both outputs with 32-byte stores)
        a.pool = static_cast<uint16_t *>(pool);
        a.pool_ctot = pool_ctot;
        a.pool_coff = pool_coff;
    }
    a.wide_io = epi != EPI_F32 && al32(out, out_ctot, out_coff) &&
                (!mask || al32(mask->ptr, mask->ctot, mask->coff)) && (!a.up || al32(a.up, a.up_ctot, 0)) &&
                !getenv_flag("PT_CONV_NO_WIDE_IO");
    a.err = err;
    a.wait_ns = wait_limit_ns();
    a.stall = take_stall_request() ? 1 : 0;
    op->kc = kc;
    op->halo = halo;
    while (a.stages > 2 && smem_request(a.stages, a.stage_bytes, a.tmem_cols) + a.wres_bytes > 220 * 1024) a.stages--;
    op->smem = smem_request(a.stages, a.stage_bytes, a.tmem_cols) + a.wres_bytes;
    const long long total = (long long)in.n * a.tiles_x * a.tiles_y * ntiles;
    const int per_sm = std::max(1, std::min((228 * 1024) / (op->smem + 1024), 512 / a.tmem_cols));
    op->grid = dim3(static_cast<unsigned>(std::min<long long>(total, (long long)per_sm * sm_count())), 1, 1);
    if (op->smem > 220 * 1024) {
        pt_set_error("conv forward: shared memory request %d too large", op->smem);
        return PT_ERR_INVALID;
    }
    return PT_OK;
}

template <int KC, bool HALO>
static int fwd_persistent_go(const FwdOp &op, cudaStream_t stream) {
    int st = set_smem_attr(k_conv_fwd_persistent<KC, HALO>, op.smem);
    if (st != PT_OK) return st;
    k_conv_fwd_persistent<KC, HALO><<<op.grid, 192, op.smem, stream>>>(op.act, op.wgt, op.args);
    PT_CUDA_TRY(cudaGetLastError());
    return PT_OK;
}

int fwd_launch(const FwdOp &op, cudaStream_t stream) {
    if (op.halo) return fwd_persistent_go<16, true>(op, stream);
    if (op.kc == 64) return fwd_persistent_go<64, false>(op, stream);
    if (op.kc == 32) return fwd_persistent_go<32, false>(op, stream);
    return fwd_persistent_go<16, false>(op, stream);
}

int wgrad_prepare(WgradOp *op, const Act &x, const Act &gy, float *dw, float *db, int num_sms, unsigned *err) {
    if (x.n != gy.n || x.h != gy.h || x.w != gy.w || x.c % 16 || gy.c % 16 || x.c <= 0 || gy.c <= 0) {
        pt_set_error("conv weight gradient: shapes differ or channels not multiples of 16");
        return PT_ERR_INVALID;
    }
    const int kca = pick_kc(x.c);
    const Tiling t = tiling_for(x.h, x.w);
    // output channels per CTA: a multiple of the dy chunk, at most 256
    int kcb = pick_kc(gy.c);
    int ntiles = (gy.c + 255) / 256;
    while (gy.c % (ntiles * kcb) != 0 && kcb > 16) kcb /= 2;
    while (gy.c % (ntiles * kcb) != 0) ntiles++;
    const int n_tile = gy.c / ntiles;
    int st;
    if ((st = act_map(&op->act, x, kca, t)) != PT_OK) return st;
    if ((st = act_map(&op->grad, gy, kcb, t)) != PT_OK) return st;
    WgradArgs &a = op->args;
    memset(&a, 0, sizeof(a));
    a.n_img = x.n;
    a.H = x.h;
    a.W = x.w;
    a.tile_w = t.tile_w;
    a.tile_rows = t.tile_rows;
    a.tiles_x = t.tiles_x;
    a.tiles_y = t.tiles_y;
    a.cin = x.c;
    a.nchunks_a = x.c / kca;
    a.cout = gy.c;
    a.n_tile = n_tile;
    a.tmem_cols = pow2_cols(n_tile);
    a.stage_bytes = 128 * 128 * 2 + 256 * n_tile;
    // two stages per CTA, so that two CTAs (two producer / MMA thread pairs)
    // share an SM: 2.66 ms per training step at batch 16 x 256^2 instead of
    // 3.21 ms with up to four stages and one CTA per SM
    a.stages = 2;
    a.total_tiles = x.n * t.tiles_x * t.tiles_y;
    a.zero_fill = t.tile_w * t.tile_rows < 128 ? 1 : 0;
    const int m_tiles = (9 * a.nchunks_a * kca + 127) / 128;
    const int base_ctas = m_tiles * ntiles;
    const int last_blocks = 9 * a.nchunks_a - (m_tiles - 1) * (128 / kca);  // chunks in the last M tile
    a.ones_row = last_blocks < 128 / kca ? last_blocks * kca : -1;
    a.db = a.ones_row >= 0 && !getenv_flag("PT_CONV_NO_FUSED_BIAS") ? db : nullptr;
    op->bias_fused = a.db != nullptr;
    op->smem = smem_request(a.stages, a.stage_bytes, a.tmem_cols);
    // split the pixel tiles so that the grid is one full wave of resident CTAs
    const int per_sm = std::max(1, std::min((228 * 1024) / (op->smem + 1024), 512 / a.tmem_cols));
    int splits = std::max(1, (per_sm * std::max(num_sms, 1)) / base_ctas);
    splits = std::min(splits, std::max(1, a.total_tiles / 4));
    a.tiles_per_split = (a.total_tiles + splits - 1) / splits;
    splits = (a.total_tiles + a.tiles_per_split - 1) / a.tiles_per_split;
    a.dw = dw;
    a.err = err;
    a.wait_ns = wait_limit_ns();
    op->kca = kca;
    op->kcb = kcb;
    op->grid = dim3(static_cast<unsigned>(m_tiles), static_cast<unsigned>(ntiles), static_cast<unsigned>(splits));
    if (op->smem > 220 * 1024) {
        pt_set_error("conv weight gradient: shared memory request %d too large", op->smem);
        return PT_ERR_INVALID;
    }
    return PT_OK;
}

template <int KCA, int KCB>
static int wgrad_go(const WgradOp &op, cudaStream_t stream) {
    int st = set_smem_attr(k_conv_wgrad<KCA, KCB>, op.smem);
    if (st != PT_OK) return st;
    k_conv_wgrad<KCA, KCB><<<op.grid, 128, op.smem, stream>>>(op.act, op.grad, op.args);
    PT_CUDA_TRY(cudaGetLastError());
    return PT_OK;
}

int wgrad_launch(const WgradOp &op, cudaStream_t stream) {
#define PT_WG(A, B) \
    if (op.kca == A && op.kcb == B) return wgrad_go<A, B>(op, stream);
    PT_WG(64, 64) PT_WG(64, 32) PT_WG(64, 16) PT_WG(32, 64) PT_WG(32, 32) PT_WG(32, 16) PT_WG(16, 64) PT_WG(16, 32)
    PT_WG(16, 16)
#undef PT_WG
    pt_set_error("conv weight gradient: unsupported chunk pair %d/%d", op.kca, op.kcb);
    return PT_ERR_INVALID;
}

int bias_grad_launch(const Act &g, float *db, cudaStream_t stream) {
    if (g.c <= 0 || g.c > 512) {
        pt_set_error("bias gradient: %d channels", g.c);
        return PT_ERR_INVALID;
    }
    const int threads = std::max(g.c, (256 / g.c) * g.c);
    const long long npix = (long long)g.n * g.h * g.w;
    const int blocks = static_cast<int>(std::min<long long>(1024, (npix + 63) / 64));
    k_bias_grad<<<blocks, threads, threads * sizeof(float), stream>>>(static_cast<const uint16_t *>(g.ptr), g.ctot,
                                                                       g.coff, g.c, npix, db);
    PT_CUDA_TRY(cudaGetLastError());
    return PT_OK;
}

int flip_transpose_launch(const uint16_t *w, int cout, int cin, uint16_t *wt, cudaStream_t stream) {
    const long long n = 9ll * cout * cin;
    const int blocks = static_cast<int>(std::min<long long>(4096, (n + 255) / 256));
    k_flip_transpose<<<blocks, 256, 0, stream>>>(w, cout, cin, wt);
    PT_CUDA_TRY(cudaGetLastError());
    return PT_OK;
}

}  // namespace ptconv
