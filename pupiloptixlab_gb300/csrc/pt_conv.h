// pt_conv.h -- 3x3 / stride 1 / padding 1 BF16 convolutions of NHWC tensors
// as implicit GEMMs on the fifth-generation tensor cores (tcgen05.mma with
// the FP32 accumulator in tensor memory, operands staged by TMA).  Host-side
// interface used by the denoiser (pt_denoise.cu) and by the C-ABI test entry
// points (pt_conv3x3_*).
//
// Forward:          y[p, co] = epi( sum_{tap, ci} x[p + off(tap), ci] * w[co][tap][ci] + b[co] )
//                   GEMM M = 128 pixels, N = output channels, K = 9 * cin.
// Data gradient:    the forward kernel over dy with the flipped, transposed
//                   weights w'[ci][8 - tap][co] = w[co][tap][ci].
// Weight gradient:  dw[co][tap][ci] += sum_p x[p + off(tap), ci] * dy[p, co]
//                   GEMM M = 128 (tap, ci) rows, N = output channels, K = pixels,
//                   both operands MN-major, split over pixel ranges (FP32 atomics).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace ptconv {

// Channels [coff, coff + c) of an NHWC bf16 tensor with ctot channels.
struct Act {
    void *ptr = nullptr;
    int n = 0, h = 0, w = 0;
    int ctot = 0, coff = 0, c = 0;
};

enum Epilogue : int {
    EPI_BF16 = 0,       // bf16 out = x + bias, optional ReLU
    EPI_F32 = 1,        // f32 out = x + bias
    EPI_BF16_MASK = 2,  // bf16 out = x * (mask > 0)   (data gradient through a ReLU)
};

struct FwdArgs {
    int n_img, H, W;
    int tile_w, tile_rows, tiles_x, tiles_y;
    int cin, nchunks;     // K = 9 * cin, in chunks of KC channels per tap
    int n_tile, cout;     // N per CTA; valid output channels
    int tmem_cols, stages, stage_bytes;
    int halo_a_bytes;     // halo kernel: bytes of the A planes at the start of a stage
    int wres_bytes;       // halo kernel: > 0 = all weights resident in shared memory (loaded once per CTA)
    int n_tiles_n;        // output-channel tiles (persistent kernel: tile = pixel tile x channel tile)
    int epi, relu;
    const float *bias;
    void *out;
    int out_ctot, out_coff;
    const uint16_t *mask;
    int mask_ctot, mask_coff;
    unsigned *err;
    unsigned long long wait_ns;  // limit of every bounded wait (kWaitNs unless pt_conv_set_wait_limit changed it)
    int stall;                   // test of the timeout path: the MMA warp first waits on a barrier nothing arrives at
    int halo_rows;               // halo kernel: output rows per tile (1-4); the box holds halo_rows + 2 rows
    int halo_box_bytes;          // halo kernel: bytes of one 8-channel plane as TMA writes it
    int halo_plane_bytes;        // halo kernel: plane stride (1 KiB-aligned TMA destinations)
    int wide_io;                 // BF16 output / mask rows 32-byte aligned: 256-bit accesses in the epilogue
    int halo_sw32;               // halo kernel: one 16-channel box per chunk, 32-byte swizzle (else two planes)
    int halo_a_tx;               // halo kernel: bytes of A the TMA delivers per stage
    int bias16;                  // bias 16-byte aligned: the epilogue reads it in 16-byte loads
    uint16_t *up;                // EPI_BF16: also written, 2x nearest up-sampled, to channels [0, cout) of
    int up_ctot;                 // this (n, 2H, 2W, up_ctot) tensor (the decoder's concatenation)
    uint16_t *pool;              // halo kernel, two-row tiles, EPI_BF16: the 2x2 average of the BF16 outputs
    int pool_ctot, pool_coff;    // also goes to this (n, H/2, W/2, pool_ctot) tensor at channel pool_coff
};

struct WgradArgs {
    int n_img, H, W;
    int tile_w, tile_rows, tiles_x, tiles_y;
    int cin, nchunks_a;   // A rows: (tap, chunk) blocks of KCA channels, 9 * nchunks_a blocks
    int cout, n_tile;     // N per CTA (a multiple of KCB)
    int tmem_cols, stages, stage_bytes;
    int total_tiles, tiles_per_split;
    int zero_fill;        // pixel tiles smaller than 128: clear the stages once
    float *dw;            // [cout][9][cin] FP32, accumulated
    float *db;            // [cout] FP32, accumulated through the ones row (null: not fused)
    int ones_row;         // row of the last M tile whose A block holds ones (its D row = sum of gy)
    unsigned *err;
    unsigned long long wait_ns;
};

struct FwdOp {
    CUtensorMap act, wgt;
    FwdArgs args;
    dim3 grid;
    int smem = 0, kc = 0;
    bool halo = false;  // halo loads (width >= 128)
};

struct WgradOp {
    CUtensorMap act, grad;
    WgradArgs args;
    dim3 grid;
    int smem = 0, kca = 0, kcb = 0;
    bool bias_fused = false;  // the kernel also accumulates db (else bias_grad_launch does)
};

// Largest chunk in {64, 32, 16} channels dividing c (c a multiple of 16).
int pick_kc(int c);

// Limit of every bounded wait of the convolution kernels prepared from now on
// (0 = the default of 2 s), and a one-shot request that the next prepared
// forward convolution first waits on a barrier nothing arrives at, so that the
// wait runs out and the kernel takes its error path (test of that path).
void set_wait_limit(unsigned long long ns, bool stall_next);
unsigned long long wait_limit_ns();
bool take_stall_request();

// Forward (or data-gradient) launch over `in`.  Images at least 128 pixels
// wide use the halo kernel (one input load per 16-channel chunk for all nine
// taps, two output rows per tile); the environment variable PT_CONV_NO_HALO=1
// selects the per-tap kernel for every width, for comparison runs.  `w` holds
// rows [w_rows][9][in.c] in bf16 (rows beyond w_rows read as zero); `cout`
// output channels are written to channels [out_coff, out_coff + cout) of `out`
// (out_ctot channels, same n/h/w as `in`).  `mask` (EPI_BF16_MASK) is a tensor
// of the output's shape.
int fwd_prepare(FwdOp *op, const Act &in, const void *w, int w_rows, int cout, const float *bias, int epi,
                int relu, void *out, int out_ctot, int out_coff, const Act *mask, unsigned *err, void *up = nullptr,
                int up_ctot = 0, void *pool = nullptr, int pool_ctot = 0, int pool_coff = 0);
// Whether the forward launch prepared in op also wrote the 2x2-pooled output.
inline bool fwd_pooled(const FwdOp &op) { return op.args.pool != nullptr; }
int fwd_launch(const FwdOp &op, cudaStream_t stream);

// dw[co][tap][ci] += sum over pixels of x[p + off(tap), ci] * gy[p, co].
// When db is given and the last 128-row block of (tap, channel) rows has a
// spare chunk, that chunk of A is filled with ones and the same MMAs also give
// db[co] += sum over pixels of gy[p, co] (op->bias_fused); otherwise the
// caller runs bias_grad_launch.
int wgrad_prepare(WgradOp *op, const Act &x, const Act &gy, float *dw, float *db, int num_sms, unsigned *err);
int wgrad_launch(const WgradOp &op, cudaStream_t stream);

// db[c] += sum over pixels of g[p, c].
int bias_grad_launch(const Act &g, float *db, cudaStream_t stream);

// w'[ci][tap][co] = w[8 - tap ... ] flipped and transposed, bf16, rows padded
// with zeros: w is [cout][9][cin], w' is [cin][9][cout].
int flip_transpose_launch(const uint16_t *w, int cout, int cin, uint16_t *wt, cudaStream_t stream);

}  // namespace ptconv
