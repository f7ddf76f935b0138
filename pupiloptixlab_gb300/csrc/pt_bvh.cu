// pt_bvh.cu -- GPU acceleration-structure build and refit.
//
// Replaces the closed OptiX builds GAS::Create / IAS::Create / IAS::Update
// (framework/world/gas_manager.cpp:69-245, framework/world/ias_manager.cpp:
// 29-151).  Pipeline (all on the device, one GPU):
//   1. primitive boxes and centroid bounds (block reduction + ordered atomics)
//   2. 63-bit Morton codes (21 bits per axis)
//   3. stable LSD radix sort of (code, primitive) pairs, 8 passes of 8 bits:
//      tile histogram -> one-block exclusive scan -> warp-multisplit scatter
//      (__match_any_sync ranks, per-warp digit counts in shared memory)
//   4. binary tree: PLOC clustering (default) or the Karras (HPG 2012)
//      binary radix tree, equal codes split by index
//   5. bottom-up boxes with an SAH cost per node (leaf vs split decision,
//      leaves of at most max_leaf_size primitives)
//   6. SAH-optimal assignment of the binary subtrees to the slots of 2/4/8-wide
//      nodes (dynamic programming, bottom up), then a top-down,
//      level-synchronous collapse that follows it; nodes come out in
//      breadth-first order.
//   7. primitive records gathered into leaf order
// Child boxes are padded outward (relative to the box and scene magnitude) so
// that the conservative slab test never rejects a primitive the exact test
// would hit.

#include "pt_nvtx.h"
#include "pt_internal.h"
#include "pt_traverse.cuh"

#include <algorithm>
#include <cfloat>

namespace {

using ptd::f3;

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr float kCostNode = 1.2f;
constexpr float kCostPrim = 1.0f;
constexpr float kCostCurvePiece = 3.0f;  // a round-cone test costs about three triangle tests

// SAH intersection cost of one primitive record (triangle and sphere 1).
__device__ __forceinline__ float prim_cost(const float4 *prims, uint32_t p) {
    const float4 a = prims[3 * (size_t)p], b = prims[3 * (size_t)p + 1];
    return (__float_as_int(a.w) < 0 && __float_as_int(b.w) != 0) ? kCostCurvePiece : kCostPrim;
}

__device__ __forceinline__ uint32_t f2ord(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__device__ __forceinline__ void prim_box(const float4 *prims, uint32_t p, float3 &lo, float3 &hi) {
    float4 a = prims[3 * (size_t)p], b = prims[3 * (size_t)p + 1];
    if (__float_as_int(a.w) >= 0) {
        float4 c = prims[3 * (size_t)p + 2];
        lo = f3(fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z)));
        hi = f3(fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z)));
    } else if (__float_as_int(b.w) == 0) {  // sphere
        float r = b.x;
        lo = f3(a.x - r, a.y - r, a.z - r);
        hi = f3(a.x + r, a.y + r, a.z + r);
    } else {  // round-cone curve piece: the boxes of its two end spheres
        float4 c = prims[3 * (size_t)p + 2];
        float r0 = b.x, r1 = b.y;
        lo = f3(fminf(a.x - r0, c.x - r1), fminf(a.y - r0, c.y - r1), fminf(a.z - r0, c.z - r1));
        hi = f3(fmaxf(a.x + r0, c.x + r1), fmaxf(a.y + r0, c.y + r1), fmaxf(a.z + r0, c.z + r1));
    }
}

// 1. per-primitive boxes (SoA float4) + centroid bounds into 6 ordered uints.
__global__ void k_prim_bounds(const float4 *prims, uint32_t n, float4 *plo, float4 *phi, uint32_t *cb) {
    __shared__ float red[6][32];
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float v[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
    if (i < n) {
        float3 lo, hi;
        prim_box(prims, i, lo, hi);
        plo[i] = make_float4(lo.x, lo.y, lo.z, 0.f);
        phi[i] = make_float4(hi.x, hi.y, hi.z, 0.f);
        float cx = 0.5f * (lo.x + hi.x), cy = 0.5f * (lo.y + hi.y), cz = 0.5f * (lo.z + hi.z);
        v[0] = cx; v[1] = cy; v[2] = cz; v[3] = cx; v[4] = cy; v[5] = cz;
    }
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        float x = v[k];
        for (int o = 16; o > 0; o >>= 1) {
            float y = __shfl_xor_sync(0xffffffffu, x, o);
            x = k < 3 ? fminf(x, y) : fmaxf(x, y);
        }
        if (lane == 0) red[k][warp] = x;
    }
    __syncthreads();
    if (warp == 0) {
        int nw = blockDim.x >> 5;
#pragma unroll
        for (int k = 0; k < 6; k++) {
            float x = lane < nw ? red[k][lane] : (k < 3 ? FLT_MAX : -FLT_MAX);
            for (int o = 16; o > 0; o >>= 1) {
                float y = __shfl_xor_sync(0xffffffffu, x, o);
                x = k < 3 ? fminf(x, y) : fmaxf(x, y);
            }
            if (lane == 0) {
                if (k < 3) atomicMin(&cb[k], f2ord(x));
                else atomicMax(&cb[k], f2ord(x));
            }
        }
    }
}

__device__ __forceinline__ uint64_t split3(uint32_t a) {
    uint64_t x = a & 0x1fffffu;
    x = (x | x << 32) & 0x1f00000000ffffULL;
    x = (x | x << 16) & 0x1f0000ff0000ffULL;
    x = (x | x << 8) & 0x100f00f00f00f00fULL;
    x = (x | x << 4) & 0x10c30c30c30c30c3ULL;
    x = (x | x << 2) & 0x1249249249249249ULL;
    return x;
}

// 2. Morton codes of the box centroids.
__global__ void k_morton(const float4 *plo, const float4 *phi, uint32_t n, const uint32_t *cb, uint64_t *keys, uint32_t *vals) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float mn[3] = {ord2f(cb[0]), ord2f(cb[1]), ord2f(cb[2])};
    float mx[3] = {ord2f(cb[3]), ord2f(cb[4]), ord2f(cb[5])};
    float4 lo = plo[i], hi = phi[i];
    float c[3] = {0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z)};
    uint32_t q[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        float ext = mx[k] - mn[k];
        float t = ext > 0.f ? (c[k] - mn[k]) / ext : 0.f;
        float s = t * 2097152.0f;
        q[k] = (uint32_t)fminf(fmaxf(s, 0.f), 2097151.f);
    }
    keys[i] = (split3(q[0]) << 2) | (split3(q[1]) << 1) | split3(q[2]);
    vals[i] = i;
}

// 3a. per-tile digit histogram, stored digit-major: hist[d * tiles + tile].
__global__ void k_radix_hist(const uint64_t *keys, uint32_t n, int shift, uint32_t *hist, uint32_t tiles) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    size_t base = (size_t)blockIdx.x * kSortTile;
#pragma unroll 4
    for (int k = 0; k < kSortItems; k++) {
        size_t idx = base + (size_t)k * kSortThreads + threadIdx.x;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// 3b. in-place exclusive scan of m values with one block of 1024 threads.
__global__ void k_scan_excl(uint32_t *data, uint32_t m) {
    __shared__ uint32_t part[1024];
    uint32_t per = (m + 1023) / 1024;
    uint32_t b = threadIdx.x * per, e = min(m, b + per);
    uint32_t sum = 0;
    for (uint32_t i = b; i < e; i++) sum += data[i];
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        uint32_t v = threadIdx.x >= (uint32_t)o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - sum;
    for (uint32_t i = b; i < e; i++) {
        uint32_t v = data[i];
        data[i] = run;
        run += v;
    }
}

// 3c. stable scatter: ranks within a tile come from warp multisplit.
__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const uint64_t *kin, const uint32_t *vin, uint64_t *kout,
                                                                uint32_t *vout, uint32_t n, int shift,
                                                                const uint32_t *hist, uint32_t tiles) {
    __shared__ uint32_t base_off[256];
    __shared__ uint32_t wcnt[kSortThreads / 32][256];
    __shared__ uint32_t tot[256];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    base_off[tid] = hist[(size_t)tid * tiles + blockIdx.x];
    const uint32_t lt = (1u << lane) - 1u;
    size_t base = (size_t)blockIdx.x * kSortTile;
    for (int k = 0; k < kSortItems; k++) {
#pragma unroll
        for (int w = 0; w < kSortThreads / 32; w++) wcnt[w][tid] = 0;
        __syncthreads();
        size_t idx = base + (size_t)k * kSortThreads + tid;
        bool valid = idx < n;
        uint64_t key = valid ? kin[idx] : 0;
        uint32_t val = valid ? vin[idx] : 0;
        uint32_t digit = valid ? (uint32_t)((key >> shift) & 255u) : 256u;
        uint32_t peers = __match_any_sync(0xffffffffu, digit);
        uint32_t lrank = __popc(peers & lt);
        if (valid && lrank == 0) wcnt[warp][digit] = __popc(peers);
        __syncthreads();
        {
            uint32_t run = 0;
#pragma unroll
            for (int w = 0; w < kSortThreads / 32; w++) {
                uint32_t c = wcnt[w][tid];
                wcnt[w][tid] = run;
                run += c;
            }
            tot[tid] = run;
        }
        __syncthreads();
        if (valid) {
            uint32_t pos = base_off[digit] + wcnt[warp][digit] + lrank;
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
        base_off[tid] += tot[tid];
    }
}

__device__ __forceinline__ int delta(const uint64_t *keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    uint64_t a = keys[i], b = keys[j];
    if (a == b) return 64 + __clz((uint32_t)(i ^ j));
    return __clzll(a ^ b);
}

// 4. Karras binary radix tree.  Internal nodes 0..n-2, leaf k is node n-1+k.
__global__ void k_karras(const uint64_t *keys, int n, int *left, int *right, int *parent, int *rfirst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = delta(keys, n, i, j);
    int s = 0;
    int div = 2, t;
    do {
        t = (l + div - 1) / div;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
        div <<= 1;
    } while (t > 1);
    int gamma = i + s * d + min(d, 0);
    int first = min(i, j), last = max(i, j);
    int lc = (first == gamma) ? (n - 1 + gamma) : gamma;
    int rc = (last == gamma + 1) ? (n - 1 + gamma + 1) : gamma + 1;
    left[i] = lc;
    right[i] = rc;
    parent[lc] = i;
    parent[rc] = i;
    rfirst[i] = first;
}

__device__ __forceinline__ float half_area(float4 lo, float4 hi) {
    float ex = hi.x - lo.x, ey = hi.y - lo.y, ez = hi.z - lo.z;
    return ex * ey + ey * ez + ez * ex;
}

// 5. bottom-up boxes, counts and SAH costs (second arrival processes a node).
__global__ void k_bottom_up(int n, const int *left, const int *right, const int *parent, const uint32_t *order,
                            const float4 *prims, const float4 *plo, const float4 *phi, float4 *nlo, float4 *nhi,
                            int *ncount, float *ncost, float *nwt, int *nleaf, int *flags, int max_leaf) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int leaf = n - 1 + k;
    uint32_t p = order[k];
    float4 lo = plo[p], hi = phi[p];
    const float w = prim_cost(prims, p);
    nlo[leaf] = lo;
    nhi[leaf] = hi;
    ncount[leaf] = 1;
    ncost[leaf] = w * half_area(lo, hi);
    nwt[leaf] = w;
    nleaf[leaf] = 1;
    int cur = parent[leaf];
    while (cur >= 0) {
        __threadfence();
        if (atomicAdd(&flags[cur], 1) == 0) return;
        __threadfence();
        int l = left[cur], r = right[cur];
        float4 llo = __ldcg(&nlo[l]), lhi = __ldcg(&nhi[l]), rlo = __ldcg(&nlo[r]), rhi = __ldcg(&nhi[r]);
        float4 blo = make_float4(fminf(llo.x, rlo.x), fminf(llo.y, rlo.y), fminf(llo.z, rlo.z), 0.f);
        float4 bhi = make_float4(fmaxf(lhi.x, rhi.x), fmaxf(lhi.y, rhi.y), fmaxf(lhi.z, rhi.z), 0.f);
        int cnt = __ldcg(&ncount[l]) + __ldcg(&ncount[r]);
        float wsum = __ldcg(&nwt[l]) + __ldcg(&nwt[r]);
        float a = half_area(blo, bhi);
        float c_split = kCostNode * a + __ldcg(&ncost[l]) + __ldcg(&ncost[r]);
        float c_leaf = cnt <= max_leaf ? a * wsum : FLT_MAX;
        bool mk_leaf = c_leaf <= c_split;
        nlo[cur] = blo;
        nhi[cur] = bhi;
        ncount[cur] = cnt;
        nwt[cur] = wsum;
        ncost[cur] = mk_leaf ? c_leaf : c_split;
        nleaf[cur] = mk_leaf ? 1 : 0;
        cur = parent[cur];
    }
}

// 4'/5'. PLOC: parallel locally-ordered clustering (Meister and Bittner,
// IEEE TVCG 2018), the default build.  The Morton-sorted primitives start as
// clusters (leaf k = node n-1+k); each pass every cluster finds the cluster
// within kPlocRadius positions whose union has the smallest surface area,
// mutual nearest neighbours merge into a new internal node (id from a
// counter, 0..n-2) that takes the lower position, and the array is compacted.
// Boxes, counts and the SAH leaf-or-split decision of a node are made when it
// forms (its children are complete by then).  Subtrees are then laid out
// depth first so that every subtree covers a contiguous range of the
// primitive order, as the wide collapse expects.
constexpr int kPlocRadius = 16;
constexpr int kPlocBlock = 256;
constexpr int kPlocMaxDepth = 256;  // a deeper binary tree makes the build fall back to the radix tree

__global__ void k_ploc_init(int n, const uint32_t *order, const float4 *prims, const float4 *plo, const float4 *phi,
                            float4 *nlo, float4 *nhi, int *ncount, float *ncost, float *nwt, int *nleaf, int *cl) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int leaf = n - 1 + k;
    uint32_t p = order[k];
    float4 lo = plo[p], hi = phi[p];
    const float w = prim_cost(prims, p);
    nlo[leaf] = lo;
    nhi[leaf] = hi;
    ncount[leaf] = 1;
    ncost[leaf] = w * half_area(lo, hi);
    nwt[leaf] = w;
    nleaf[leaf] = 1;
    cl[k] = leaf;
}

// Nearest neighbour of every cluster: smallest union area, ties to the lower
// position (so the closest pair overall is always mutual).
__global__ void __launch_bounds__(kPlocBlock) k_ploc_nn(int m, const int *cl, const float4 *nlo, const float4 *nhi,
                                                        int *nn) {
    __shared__ float4 slo[kPlocBlock + 2 * kPlocRadius], shi[kPlocBlock + 2 * kPlocRadius];
    const int b0 = blockIdx.x * kPlocBlock;
    for (int t = threadIdx.x; t < kPlocBlock + 2 * kPlocRadius; t += blockDim.x) {
        const int g = b0 - kPlocRadius + t;
        if (g >= 0 && g < m) {
            const int id = cl[g];
            slo[t] = nlo[id];
            shi[t] = nhi[id];
        }
    }
    __syncthreads();
    const int i = b0 + threadIdx.x;
    if (i >= m) return;
    const float4 lo = slo[threadIdx.x + kPlocRadius], hi = shi[threadIdx.x + kPlocRadius];
    float best = FLT_MAX;
    int bj = -1;
    for (int o = -kPlocRadius; o <= kPlocRadius; o++) {
        const int j = i + o;
        if (o == 0 || j < 0 || j >= m) continue;
        const float4 l2 = slo[threadIdx.x + kPlocRadius + o], h2 = shi[threadIdx.x + kPlocRadius + o];
        const float4 ulo = make_float4(fminf(lo.x, l2.x), fminf(lo.y, l2.y), fminf(lo.z, l2.z), 0.f);
        const float4 uhi = make_float4(fmaxf(hi.x, h2.x), fmaxf(hi.y, h2.y), fmaxf(hi.z, h2.z), 0.f);
        const float a = half_area(ulo, uhi);
        if (a < best) {  // positions are visited in increasing order: ties keep the lower one
            best = a;
            bj = j;
        }
    }
    nn[i] = bj;
}

// Merge mutual pairs: keep[i] = 1 where position i survives, out_id[i] its node.
__global__ void k_ploc_merge(int m, const int *cl, const int *nn, uint32_t *keep, int *out_id, uint32_t *node_ctr,
                             int *left, int *right, int *parent, float4 *nlo, float4 *nhi, int *ncount, float *ncost,
                             float *nwt, int *nleaf, int max_leaf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int j = nn[i];
    const bool mutual = j >= 0 && nn[j] == i;
    if (!mutual) {
        keep[i] = 1;
        out_id[i] = cl[i];
        return;
    }
    if (i > j) {
        keep[i] = 0;
        return;
    }
    const int a = cl[i], b = cl[j];
    const int id = (int)atomicAdd(node_ctr, 1u);
    const float4 la = nlo[a], ha = nhi[a], lb = nlo[b], hb = nhi[b];
    const float4 blo = make_float4(fminf(la.x, lb.x), fminf(la.y, lb.y), fminf(la.z, lb.z), 0.f);
    const float4 bhi = make_float4(fmaxf(ha.x, hb.x), fmaxf(ha.y, hb.y), fmaxf(ha.z, hb.z), 0.f);
    const int cnt = ncount[a] + ncount[b];
    const float wsum = nwt[a] + nwt[b];
    const float area = half_area(blo, bhi);
    const float c_split = kCostNode * area + ncost[a] + ncost[b];
    const float c_leaf = cnt <= max_leaf ? area * wsum : FLT_MAX;
    const bool mk_leaf = c_leaf <= c_split;
    left[id] = a;
    right[id] = b;
    parent[a] = id;
    parent[b] = id;
    nlo[id] = blo;
    nhi[id] = bhi;
    ncount[id] = cnt;
    nwt[id] = wsum;
    ncost[id] = mk_leaf ? c_leaf : c_split;
    nleaf[id] = mk_leaf ? 1 : 0;
    keep[i] = 1;
    out_id[i] = id;
}

// Order-preserving compaction of the surviving positions in blocks of
// kCompactBlock: survivors per block (warp ballots), an exclusive scan of the
// block counts, then each survivor's rank = block offset + warp offset + its
// rank among the warp's survivors.
constexpr int kCompactBlock = 1024;

__global__ void __launch_bounds__(kCompactBlock) k_ploc_block_counts(int m, const uint32_t *keep, uint32_t *bsum) {
    __shared__ uint32_t wc[kCompactBlock / 32];
    const int i = blockIdx.x * kCompactBlock + threadIdx.x;
    const unsigned b = __ballot_sync(0xffffffffu, i < m && keep[i] != 0);
    if ((threadIdx.x & 31) == 0) wc[threadIdx.x >> 5] = __popc(b);
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t v = wc[threadIdx.x];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) bsum[blockIdx.x] = v;
    }
}

__global__ void __launch_bounds__(kCompactBlock) k_ploc_compact(int m, const uint32_t *keep, const uint32_t *boff,
                                                                const int *out_id, int *cl_next) {
    __shared__ uint32_t woff[kCompactBlock / 32];
    const int i = blockIdx.x * kCompactBlock + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool k = i < m && keep[i] != 0;
    const unsigned b = __ballot_sync(0xffffffffu, k);
    if (lane == 0) woff[warp] = __popc(b);
    __syncthreads();
    if (warp == 0) {  // exclusive scan of the per-warp counts
        const uint32_t v = woff[lane];
        uint32_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        woff[lane] = x - v;
    }
    __syncthreads();
    if (k) cl_next[boff[blockIdx.x] + woff[warp] + __popc(b & ((1u << lane) - 1u))] = out_id[i];
}

// Depth-first position of every node (leftmost leaf of its subtree): the sum
// of the left siblings' primitive counts along the path to the root.  A path
// longer than kPlocMaxDepth raises the failure flag.
__global__ void k_ploc_offsets(int n, const int *left, const int *right, const int *parent, const int *ncount,
                               int *offs, uint32_t *fail) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= 2 * n - 1) return;
    int cur = x, off = 0, steps = 0;
    for (int p = parent[cur]; p >= 0; p = parent[cur]) {
        if (right[p] == cur) off += ncount[left[p]];
        cur = p;
        if (++steps > kPlocMaxDepth) {
            atomicOr(fail, 1u);
            break;
        }
    }
    offs[x] = off;
}

// Renumber leaves to their depth-first positions (leaf at position q is node
// n-1+q), record every internal node's first position, permute the order.
__global__ void k_ploc_finish(int n, const int *offs, const uint32_t *order, const float4 *nlo, const float4 *nhi,
                              const int *parent, int *left, int *right, int *rfirst, uint32_t *order_out,
                              float4 *leaf_lo, float4 *leaf_hi, int *parent_out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= 2 * n - 1) return;
    if (x >= n - 1) {
        const int q = offs[x];
        order_out[q] = order[x - (n - 1)];
        leaf_lo[q] = nlo[x];
        leaf_hi[q] = nhi[x];
        parent_out[n - 1 + q] = parent[x];
    } else {
        parent_out[x] = parent[x];
        rfirst[x] = offs[x];
        const int l = left[x], r = right[x];
        left[x] = l >= n - 1 ? n - 1 + offs[l] : l;
        right[x] = r >= n - 1 ? n - 1 + offs[r] : r;
    }
}

__device__ __forceinline__ void padded(float4 lo, float4 hi, float scene_mag, float3 &plo, float3 &phi) {
    float mag = fmaxf(fmaxf(fmaxf(fabsf(lo.x), fabsf(lo.y)), fmaxf(fabsf(lo.z), fabsf(hi.x))), fmaxf(fabsf(hi.y), fabsf(hi.z)));
    float ext = fmaxf(fmaxf(hi.x - lo.x, hi.y - lo.y), hi.z - lo.z);
    float pad = 4e-7f * (mag + scene_mag) + 1e-6f * ext;
    plo = f3(lo.x - pad, lo.y - pad, lo.z - pad);
    phi = f3(hi.x + pad, hi.y + pad, hi.z + pad);
}

template <int K>
__device__ __forceinline__ void write_slot(float *node, int c, float3 lo, float3 hi, int child, int count) {
    node[c] = lo.x;
    node[K + c] = hi.x;
    node[2 * K + c] = lo.y;
    node[3 * K + c] = hi.y;
    node[4 * K + c] = lo.z;
    node[5 * K + c] = hi.z;
    node[6 * K + c] = __int_as_float(child);
    node[7 * K + c] = __int_as_float(count);
}
template <int K>
__device__ __forceinline__ void write_empty(float *node, int c) {
    write_slot<K>(node, c, f3(1e30f, 1e30f, 1e30f), f3(1e30f, 1e30f, 1e30f), -1, 0);
}

// 6. SAH-optimal wide collapse (Ylitie, Karras and Laine, HPG 2017): for
// every binary node x and i = 1..K, S(x, i) is the cheapest way to represent
// its subtree with at most i slots of a wide parent:
//   S(x, 1) = min(leaf: area * primitive weight (if count <= max_leaf),
//                 wide node: 1.2 * area + min_j S(l, j) + S(r, K - j))
//   S(x, i) = min(S(x, i - 1), min_j S(l, j) + S(r, i - j))
// computed bottom up (second arrival processes a node).  dsel[8x] keeps the
// wide node's split j, dsel[8x + i - 1] the split for i = 2..K slots (0: use
// i - 1 slots), and nleaf[x] the leaf-or-wide choice; the collapse below
// follows them.
template <int K>
__global__ void k_wide_dp(int n, const int *left, const int *right, const int *parent, const float4 *nlo,
                          const float4 *nhi, const int *ncount, const float *nwt, float *dval, uint8_t *dsel,
                          int *nleaf, int *flags, int max_leaf) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int leaf = n - 1 + k;
    const float v = half_area(nlo[leaf], nhi[leaf]) * nwt[leaf];
#pragma unroll
    for (int i = 0; i < K; i++) dval[(size_t)leaf * 8 + i] = v;
    int cur = parent[leaf];
    while (cur >= 0) {
        __threadfence();
        if (atomicAdd(&flags[cur], 1) == 0) return;
        __threadfence();
        const int l = left[cur], r = right[cur];
        float sl[K + 1], sr[K + 1], sx[K + 1];
#pragma unroll
        for (int i = 1; i <= K; i++) {
            sl[i] = __ldcg(&dval[(size_t)l * 8 + i - 1]);
            sr[i] = __ldcg(&dval[(size_t)r * 8 + i - 1]);
        }
        const float area = half_area(nlo[cur], nhi[cur]);
        float best = FLT_MAX;
        int jw = 1;
#pragma unroll
        for (int j = 1; j < K; j++) {
            const float c = sl[j] + sr[K - j];
            if (c < best) {
                best = c;
                jw = j;
            }
        }
        const float c_wide = kCostNode * area + best;
        const float c_leaf = ncount[cur] <= max_leaf ? area * nwt[cur] : FLT_MAX;
        const bool mk_leaf = c_leaf <= c_wide;
        sx[1] = mk_leaf ? c_leaf : c_wide;
        dsel[(size_t)cur * 8] = (uint8_t)jw;
#pragma unroll
        for (int i = 2; i <= K; i++) {
            float vi = sx[i - 1];
            int sel = 0;
#pragma unroll
            for (int j = 1; j < i; j++) {
                const float c = sl[j] + sr[i - j];
                if (c < vi) {
                    vi = c;
                    sel = j;
                }
            }
            sx[i] = vi;
            dsel[(size_t)cur * 8 + i - 1] = (uint8_t)sel;
        }
#pragma unroll
        for (int i = 1; i <= K; i++) dval[(size_t)cur * 8 + i - 1] = sx[i];
        nleaf[cur] = mk_leaf ? 1 : 0;
        cur = parent[cur];
    }
}

// 6'. one level of the collapse, following the choices of k_wide_dp: the
// wide node of binary node b gets the slots of left(b) (dsel[8b] of them) and
// right(b) (the rest), each expanded while its choice splits it further.
template <int K>
__global__ void k_collapse_dp(int n, const int2 *items_in, const uint32_t *n_in_ptr, int2 *items_out, uint32_t *n_out,
                              uint32_t *n_wide, float *nodes, const int *left, const int *right, const int *rfirst,
                              const float4 *nlo, const float4 *nhi, const int *ncount, const int *nleaf,
                              const uint8_t *dsel, float scene_mag) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= *n_in_ptr) return;
    const int2 it = items_in[t];
    const int b = it.y;
    int slot[K];
    int ns = 0;
    int stn[K], sti[K];  // pending (node, slots); their slots sum to at most K
    int sp = 0;
    const int jw = dsel[(size_t)b * 8];
    stn[sp] = right[b];
    sti[sp++] = K - jw;
    stn[sp] = left[b];
    sti[sp++] = jw;
    while (sp > 0) {
        --sp;
        const int x = stn[sp];
        int si = sti[sp];
        if (x < n - 1) {
            while (si > 1 && dsel[(size_t)x * 8 + si - 1] == 0) si--;
        }
        if (x >= n - 1 || si <= 1) {
            if (ns < K) slot[ns++] = x;
            continue;
        }
        const int sel = dsel[(size_t)x * 8 + si - 1];
        if (sp + 2 > K) {  // cannot happen (slots on the stack sum to at most K)
            if (ns < K) slot[ns++] = x;
            continue;
        }
        stn[sp] = right[x];
        sti[sp++] = si - sel;
        stn[sp] = left[x];
        sti[sp++] = sel;
    }
    float *node = nodes + (size_t)it.x * 8 * K;
    for (int c = 0; c < K; c++) {
        if (c >= ns) {
            write_empty<K>(node, c);
            continue;
        }
        const int x = slot[c];
        float3 lo, hi;
        padded(nlo[x], nhi[x], scene_mag, lo, hi);
        if (x >= n - 1) {
            write_slot<K>(node, c, lo, hi, x - (n - 1), 1);
        } else if (nleaf[x]) {
            write_slot<K>(node, c, lo, hi, rfirst[x], ncount[x]);
        } else {
            const uint32_t w = atomicAdd(n_wide, 1u);
            const uint32_t q = atomicAdd(n_out, 1u);
            items_out[q] = make_int2((int)w, x);
            write_slot<K>(node, c, lo, hi, (int)w, 0);
        }
    }
}

// Root that is a single leaf (tiny scenes): one wide node, slot 0 = all primitives.
template <int K>
__global__ void k_leaf_root(float *nodes, int n, const float4 *nlo, const float4 *nhi, int root, float scene_mag) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int c = 0; c < K; c++) write_empty<K>(nodes, c);
    if (n > 0) {
        float3 lo, hi;
        padded(nlo[root], nhi[root], scene_mag, lo, hi);
        write_slot<K>(nodes, 0, lo, hi, 0, n);
    }
}

// 7. primitive records into leaf order.
__global__ void k_gather_prims(const float4 *src, const uint32_t *order, uint32_t n, float4 *dst) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t p = order[i];
    dst[3 * (size_t)i] = src[3 * (size_t)p];
    dst[3 * (size_t)i + 1] = src[3 * (size_t)p + 1];
    dst[3 * (size_t)i + 2] = src[3 * (size_t)p + 2];
}

// SAH cost of the wide tree: sum over slots of area * (node or primitive cost).
template <int K>
__global__ void k_sah(const float *nodes, uint32_t num_nodes, double *acc) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < num_nodes) {
        const float *nd = nodes + (size_t)i * 8 * K;
        for (int c = 0; c < K; c++) {
            int ch = __float_as_int(nd[6 * K + c]);
            if (ch < 0) continue;
            float ex = nd[K + c] - nd[c], ey = nd[3 * K + c] - nd[2 * K + c], ez = nd[5 * K + c] - nd[4 * K + c];
            float a = ex * ey + ey * ez + ez * ex;
            int cnt = __float_as_int(nd[7 * K + c]);
            v += (double)a * (cnt > 0 ? (double)kCostPrim * cnt : (double)kCostNode);
        }
    }
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(acc, v);
}

// Refit of one level: leaf slots from the primitives, inner slots from the
// union of the child node's slots (deeper levels are refit first).
template <int K>
__global__ void k_refit_level(float *nodes, uint32_t first, uint32_t last, const float4 *prims_bvh, float scene_mag) {
    uint32_t i = first + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= last) return;
    float *nd = nodes + (size_t)i * 8 * K;
    for (int c = 0; c < K; c++) {
        int ch = __float_as_int(nd[6 * K + c]);
        if (ch < 0) continue;
        int cnt = __float_as_int(nd[7 * K + c]);
        float4 lo = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.f), hi = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f);
        if (cnt > 0) {
            for (int j = 0; j < cnt; j++) {
                float3 a, b;
                prim_box(prims_bvh, (uint32_t)(ch + j), a, b);
                lo = make_float4(fminf(lo.x, a.x), fminf(lo.y, a.y), fminf(lo.z, a.z), 0.f);
                hi = make_float4(fmaxf(hi.x, b.x), fmaxf(hi.y, b.y), fmaxf(hi.z, b.z), 0.f);
            }
        } else {
            const float *cn = nodes + (size_t)ch * 8 * K;
            for (int g = 0; g < K; g++) {
                if (__float_as_int(cn[6 * K + g]) < 0) continue;
                lo = make_float4(fminf(lo.x, cn[g]), fminf(lo.y, cn[2 * K + g]), fminf(lo.z, cn[4 * K + g]), 0.f);
                hi = make_float4(fmaxf(hi.x, cn[K + g]), fmaxf(hi.y, cn[3 * K + g]), fmaxf(hi.z, cn[5 * K + g]), 0.f);
            }
        }
        float3 plo, phi;
        padded(lo, hi, scene_mag, plo, phi);
        write_slot<K>(nd, c, plo, phi, ch, cnt);
    }
}

// World-space re-transform of one mesh instance's vertices (same arithmetic
// order as the host flattening: x' = m0*x + m1*y + m2*z + m3, unfused).
__global__ void k_transform_vertices(const float *obj, uint32_t nv, float4 m0, float4 m1, float4 m2, float4 *vpos) {
    uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    float x = obj[3 * v], y = obj[3 * v + 1], z = obj[3 * v + 2];
    float wx = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m0.x, x), __fmul_rn(m0.y, y)), __fmul_rn(m0.z, z)), m0.w);
    float wy = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m1.x, x), __fmul_rn(m1.y, y)), __fmul_rn(m1.z, z)), m1.w);
    float wz = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m2.x, x), __fmul_rn(m2.y, y)), __fmul_rn(m2.z, z)), m2.w);
    vpos[v] = make_float4(wx, wy, wz, 0.f);
}
__global__ void k_rebuild_tri_records(const uint32_t *tri_vidx, const float4 *vpos, uint32_t first, uint32_t count,
                                      float4 *prims) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    uint32_t p = first + t;
    float4 a = vpos[tri_vidx[3 * p]], b = vpos[tri_vidx[3 * p + 1]], c = vpos[tri_vidx[3 * p + 2]];
    float4 *r = prims + 3 * (size_t)p;
    float w = r[0].w;  // keep the id
    r[0] = make_float4(a.x, a.y, a.z, w);
    r[1] = make_float4(b.x, b.y, b.z, 0.f);
    r[2] = make_float4(c.x, c.y, c.z, 0.f);
}

// All mesh instances at once: world vertex v belongs to the instance whose
// range [vstart, vstart + count) holds it (binary search over vstart).
struct XformRec {
    uint32_t vstart, count, src;  // world vertex range, first object vertex of its mesh
    uint32_t pad;
    float4 m0, m1, m2;
};
__global__ void k_transform_all(const float *obj, const XformRec *recs, uint32_t nrec, uint32_t total, float4 *vpos) {
    uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= total) return;
    uint32_t lo = 0, hi = nrec - 1;
    while (lo < hi) {
        uint32_t mid = (lo + hi + 1) >> 1;
        if (recs[mid].vstart <= v) lo = mid;
        else hi = mid - 1;
    }
    const XformRec r = recs[lo];
    uint32_t k = r.src + (v - r.vstart);
    float x = obj[3 * (size_t)k], y = obj[3 * (size_t)k + 1], z = obj[3 * (size_t)k + 2];
    float wx = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(r.m0.x, x), __fmul_rn(r.m0.y, y)), __fmul_rn(r.m0.z, z)), r.m0.w);
    float wy = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(r.m1.x, x), __fmul_rn(r.m1.y, y)), __fmul_rn(r.m1.z, z)), r.m1.w);
    float wz = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(r.m2.x, x), __fmul_rn(r.m2.y, y)), __fmul_rn(r.m2.z, z)), r.m2.w);
    vpos[v] = make_float4(wx, wy, wz, 0.f);
}

// Root box area for the SAH normalisation: union of the root node's slots.
template <int K>
__global__ void k_root_area(const float *nodes, double *out) {
    if (threadIdx.x || blockIdx.x) return;
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int c = 0; c < K; c++) {
        if (__float_as_int(nodes[6 * K + c]) < 0) continue;
        for (int a = 0; a < 3; a++) {
            lo[a] = fminf(lo[a], nodes[2 * a * K + c]);
            hi[a] = fmaxf(hi[a], nodes[(2 * a + 1) * K + c]);
        }
    }
    double ex = hi[0] - lo[0], ey = hi[1] - lo[1], ez = hi[2] - lo[2];
    *out = lo[0] <= hi[0] ? ex * ey + ey * ez + ez * ex : 0.0;
}

inline uint32_t blocks(size_t n, int b) { return (uint32_t)((n + b - 1) / b); }

// Compressed copies of 8-wide float nodes (layout in pt_traverse.cuh, same
// node indices).  The grid origin is the low corner of the union of the
// children's boxes; each axis's cell size is the smallest power of two for
// which 255 cells span the union; each child's cells are rounded outwards and
// then checked with the same fused multiply-add the traversal evaluates, so
// the decoded box always encloses the child's padded float box.  Children go
// to slots by a greedy matching on dot(child centroid - node centroid,
// direction of the slot's octant), smallest first (Ylitie, Karras and Laine,
// HPG 2017): slot s holds the child met first by rays of octant s.
__global__ void k_compress8(const float *nodes, uint32_t n, float4 *out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float *f = nodes + (size_t)i * 64;
        float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        uint32_t occupied = 0;
        for (int c = 0; c < 8; c++) {
            if (__float_as_int(f[48 + c]) < 0) continue;
            occupied |= 1u << c;
            for (int a = 0; a < 3; a++) {
                lo[a] = fminf(lo[a], f[16 * a + c]);
                hi[a] = fmaxf(hi[a], f[16 * a + 8 + c]);
            }
        }
        float4 *q = out + (size_t)i * ptd::kCwFloat4;
        if (!occupied) {
            q[0] = make_float4(0.f, 0.f, 0.f, __uint_as_float(127u | 127u << 8 | 127u << 16));
            q[1] = q[2] = q[3] = make_float4(0.f, 0.f, 0.f, 0.f);
            q[4] = q[5] = make_float4(__int_as_float(ptd::kNoItem), __int_as_float(ptd::kNoItem),
                                      __int_as_float(ptd::kNoItem), __int_as_float(ptd::kNoItem));
            continue;
        }
        uint32_t eb[3];
        float cell[3];
        for (int a = 0; a < 3; a++) {
            const float r = __fdiv_ru(__fsub_ru(hi[a], lo[a]), 255.f);
            uint32_t e = 1;
            if (r > 0.f) {
                const uint32_t bits = __float_as_uint(r);
                e = (bits >> 23) + ((bits & 0x7fffffu) ? 1u : 0u);
                e = e < 1u ? 1u : e;
            }
            while (e < 254u && __fmaf_rn(255.f, __uint_as_float(e << 23), lo[a]) < hi[a]) e++;
            eb[a] = e;
            cell[a] = __uint_as_float(e << 23);
        }
        // slot assignment
        float cen[8][3];
        for (int c = 0; c < 8; c++)
            for (int a = 0; a < 3; a++)
                cen[c][a] = (occupied >> c) & 1u ? 0.5f * (f[16 * a + c] + f[16 * a + 8 + c]) - 0.5f * (lo[a] + hi[a])
                                                 : 0.f;
        int slot_of[8];
        for (int c = 0; c < 8; c++) slot_of[c] = -1;
        uint32_t used = 0, todo = occupied;
        while (todo) {
            float best = FLT_MAX;
            int bc = -1, bs = -1;
            for (int c = 0; c < 8; c++) {
                if (!((todo >> c) & 1u)) continue;
                for (int sl = 0; sl < 8; sl++) {
                    if ((used >> sl) & 1u) continue;
                    const float cost = (sl & 1 ? -cen[c][0] : cen[c][0]) + (sl & 2 ? -cen[c][1] : cen[c][1]) +
                                       (sl & 4 ? -cen[c][2] : cen[c][2]);
                    if (bc < 0 || cost < best) {
                        best = cost;
                        bc = c;
                        bs = sl;
                    }
                }
            }
            slot_of[bc] = bs;
            used |= 1u << bs;
            todo &= ~(1u << bc);
        }
        uint32_t cl[3][2] = {{0, 0}, {0, 0}, {0, 0}}, ch[3][2] = {{0, 0}, {0, 0}, {0, 0}};
        int items[8];
        for (int sl = 0; sl < 8; sl++) items[sl] = ptd::kNoItem;
        for (int c = 0; c < 8; c++) {
            const int sl = slot_of[c];
            if (sl < 0) continue;
            for (int a = 0; a < 3; a++) {
                const float clo = f[16 * a + c], chi = f[16 * a + 8 + c];
                const float inv_cell = __frcp_rn(cell[a]);
                int ql = (int)floorf(__fmul_rd(__fsub_rd(clo, lo[a]), inv_cell));
                ql = min(max(ql, 0), 255);
                while (ql > 0 && __fmaf_rn((float)ql, cell[a], lo[a]) > clo) ql--;
                int qh = (int)ceilf(__fmul_ru(__fsub_ru(chi, lo[a]), inv_cell));
                qh = min(max(qh, 0), 255);
                while (qh < 255 && __fmaf_rn((float)qh, cell[a], lo[a]) < chi) qh++;
                cl[a][sl >> 2] |= (uint32_t)ql << (8 * (sl & 3));
                ch[a][sl >> 2] |= (uint32_t)qh << (8 * (sl & 3));
            }
            const int child = __float_as_int(f[48 + c]), count = __float_as_int(f[56 + c]);
            items[sl] = count > 0 ? ptd::make_leaf(child, count) : child;
        }
        q[0] = make_float4(lo[0], lo[1], lo[2], __uint_as_float(eb[0] | eb[1] << 8 | eb[2] << 16 | used << 24));
        for (int a = 0; a < 3; a++)
            q[1 + a] = make_float4(__uint_as_float(cl[a][0]), __uint_as_float(cl[a][1]), __uint_as_float(ch[a][0]),
                                   __uint_as_float(ch[a][1]));
        q[4] = make_float4(__int_as_float(items[0]), __int_as_float(items[1]), __int_as_float(items[2]),
                           __int_as_float(items[3]));
        q[5] = make_float4(__int_as_float(items[4]), __int_as_float(items[5]), __int_as_float(items[6]),
                           __int_as_float(items[7]));
    }
}

struct Scratch {
    uint64_t *keys[2];
    uint32_t *vals[2];
    uint32_t *hist;
    float4 *plo, *phi;
    int *left, *right, *parent, *rfirst, *ncount, *nleaf, *flags;
    float4 *nlo, *nhi;
    float *ncost, *nwt;  // SAH cost and summed primitive cost weight of each binary node
    int2 *items[2];
    uint32_t *counters;  // [0..5] centroid bounds, [6] n_wide, [7] n_out0, [8] n_out1, [9] PLOC nodes, [10] PLOC failure
    double *sah;
    int *cl[2], *nn, *out_id, *offs;  // PLOC clusters, neighbours, merge results, depth-first positions
    uint32_t *keep, *order2, *bsum;  // survival flags, permuted order, per-block survivor counts
    int *par2;                       // parents renumbered with the leaves
    float *dval;                     // wide-collapse costs S(x, 1..8)
    uint8_t *dsel;                   // wide-collapse choices
    float4 *leaf_lo, *leaf_hi;
};

template <class T>
T *carve(char *&p, size_t count) {
    T *r = reinterpret_cast<T *>(p);
    size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
    p += bytes;
    return r;
}
size_t carve_size(size_t n, uint32_t tiles) {
    size_t t = 0;
    auto add = [&](size_t bytes) { t += (bytes + 255) & ~size_t(255); };
    add(8 * n); add(8 * n); add(4 * n); add(4 * n);
    add(4 * (size_t)256 * tiles);
    add(16 * n); add(16 * n);
    add(4 * n); add(4 * n); add(4 * 2 * n); add(4 * n); add(4 * 2 * n); add(4 * 2 * n); add(4 * n);
    add(16 * 2 * n); add(16 * 2 * n);
    add(4 * 2 * n);
    add(8 * n); add(8 * n);
    add(64); add(64);
    add(4 * n); add(4 * n); add(4 * n); add(4 * n); add(4 * 2 * n);
    add(4 * (n + 1)); add(4 * n);
    add(16 * n); add(16 * n);
    add(4 * 2 * n);
    add(4 * (n / 1024 + 2));
    add(4 * 2 * n); add(4 * 8 * 2 * n); add(8 * 2 * n);
    return t;
}

template <int K>
int build_wide(pt_scene *s, const Scratch &sc, uint32_t n, int root, int max_leaf, cudaStream_t st) {
    s->level_start.clear();
    size_t node_bytes = (size_t)std::max<uint32_t>(1, n > 1 ? n - 1 : 1) * 32 * K;
    int e = s->nodes.ensure(node_bytes);
    if (e != PT_OK) return e;
    float *nodes = s->nodes.as<float>();
    const int tb = 256;
    if (n > 1) {  // SAH-optimal slot assignment for this width (also the final leaf decisions)
        PT_CUDA_TRY(cudaMemsetAsync(sc.flags, 0, 4 * (size_t)n, st));
        k_wide_dp<K><<<blocks(n, tb), tb, 0, st>>>((int)n, sc.left, sc.right, sc.parent, sc.nlo, sc.nhi, sc.ncount,
                                                   sc.nwt, sc.dval, sc.dsel, sc.nleaf, sc.flags, max_leaf);
        PT_CUDA_TRY(cudaGetLastError());
    }
    // root: binary node `root` (internal), or the single leaf (node 0 when n == 1)
    int root_leaf = 0;
    if (n > 1) PT_CUDA_TRY(cudaMemcpyAsync(&root_leaf, sc.nleaf + root, sizeof(int), cudaMemcpyDeviceToHost, st));
    PT_CUDA_TRY(cudaStreamSynchronize(st));
    if (n <= 1 || root_leaf) {
        k_leaf_root<K><<<1, 32, 0, st>>>(nodes, (int)n, sc.nlo, sc.nhi, n > 1 ? root : 0, s->scene_mag);
        s->level_start = {0, 1};
        return PT_OK;
    }
    uint32_t h_init[3] = {1, 1, 0};  // n_wide = 1 (root), n_out0 = 1 (root item), n_out1 = 0
    PT_CUDA_TRY(cudaMemcpyAsync(sc.counters + 6, h_init, sizeof(h_init), cudaMemcpyHostToDevice, st));
    int2 root_item = make_int2(0, root);
    PT_CUDA_TRY(cudaMemcpyAsync(sc.items[0], &root_item, sizeof(int2), cudaMemcpyHostToDevice, st));
    uint32_t level_count = 1, start = 0;
    int cur = 0;
    while (level_count > 0) {
        s->level_start.push_back(start);
        uint32_t *n_in = sc.counters + 7 + cur, *n_out = sc.counters + 7 + (cur ^ 1);
        PT_CUDA_TRY(cudaMemsetAsync(n_out, 0, sizeof(uint32_t), st));
        k_collapse_dp<K><<<blocks(level_count, tb), tb, 0, st>>>((int)n, sc.items[cur], n_in, sc.items[cur ^ 1], n_out,
                                                                sc.counters + 6, nodes, sc.left, sc.right, sc.rfirst,
                                                                sc.nlo, sc.nhi, sc.ncount, sc.nleaf, sc.dsel,
                                                                s->scene_mag);
        PT_CUDA_TRY(cudaGetLastError());
        uint32_t nxt = 0;
        PT_CUDA_TRY(cudaMemcpyAsync(&nxt, n_out, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        PT_CUDA_TRY(cudaStreamSynchronize(st));
        start += level_count;
        level_count = nxt;
        cur ^= 1;
    }
    s->level_start.push_back(start);
    return PT_OK;
}

template <int K>
void refit_levels(pt_scene *s, cudaStream_t st) {
    float *nodes = s->nodes.as<float>();
    for (int L = (int)s->level_start.size() - 2; L >= 0; L--) {
        uint32_t a = s->level_start[L], b = s->level_start[L + 1];
        if (b > a) k_refit_level<K><<<blocks(b - a, 128), 128, 0, st>>>(nodes, a, b, s->prims_bvh.as<float4>(), s->scene_mag);
    }
}

template <int K>
void sah_launch(pt_scene *s, double *acc, cudaStream_t st) {
    uint32_t nn = s->level_start.back();
    k_sah<K><<<blocks(nn, 256), 256, 0, st>>>(s->nodes.as<float>(), nn, acc);
    k_root_area<K><<<1, 1, 0, st>>>(s->nodes.as<float>(), acc + 1);
}

// SAH cost of the current wide tree (node cost 1.2, primitive cost 1),
// normalised by the root box area.
int compute_sah(pt_scene *s, double *scratch2, cudaStream_t st, float &out) {
    PT_CUDA_TRY(cudaMemsetAsync(scratch2, 0, 2 * sizeof(double), st));
    switch (s->bvh_opts.width) {
        case 2: sah_launch<2>(s, scratch2, st); break;
        case 4: sah_launch<4>(s, scratch2, st); break;
        default: sah_launch<8>(s, scratch2, st); break;
    }
    double h[2] = {0.0, 0.0};
    PT_CUDA_TRY(cudaMemcpyAsync(h, scratch2, sizeof(h), cudaMemcpyDeviceToHost, st));
    PT_CUDA_TRY(cudaStreamSynchronize(st));
    out = h[1] > 0 ? (float)((kCostNode * h[1] + h[0]) / h[1]) : 0.f;
    return PT_OK;
}

// PLOC over the sorted order in s->bvh_order (n >= 2).  Returns PT_OK with
// the binary root in *root, or PT_OK with *root = -1 when clustering stalls
// (ties in degenerate scenes) or the tree is deeper than the traversal can
// handle; the caller then builds the radix tree instead.
int ploc_build(pt_scene *s, const Scratch &sc, uint32_t n, int max_leaf, cudaStream_t st, int *root) {
    *root = -1;
    const int tb = 256;
    uint32_t *order = s->bvh_order.as<uint32_t>();
    PT_CUDA_TRY(cudaMemsetAsync(sc.parent, 0xff, 4 * (2 * (size_t)n - 1), st));
    PT_CUDA_TRY(cudaMemsetAsync(sc.counters + 9, 0, 2 * sizeof(uint32_t), st));
    k_ploc_init<<<blocks(n, tb), tb, 0, st>>>((int)n, order, s->prims_world.as<float4>(), sc.plo, sc.phi, sc.nlo,
                                              sc.nhi, sc.ncount, sc.ncost, sc.nwt, sc.nleaf, sc.cl[0]);
    PT_CUDA_TRY(cudaGetLastError());
    uint32_t m = n;
    int cur = 0;
    int log2n = 0;
    while ((1u << log2n) < n) log2n++;
    const int max_passes = 64 + 8 * log2n;
    for (int pass = 0; m > 1; pass++) {
        if (pass >= max_passes) return PT_OK;  // too slow to converge: radix tree
        k_ploc_nn<<<blocks(m, kPlocBlock), kPlocBlock, 0, st>>>((int)m, sc.cl[cur], sc.nlo, sc.nhi, sc.nn);
        k_ploc_merge<<<blocks(m, tb), tb, 0, st>>>((int)m, sc.cl[cur], sc.nn, sc.keep, sc.out_id, sc.counters + 9,
                                                   sc.left, sc.right, sc.parent, sc.nlo, sc.nhi, sc.ncount, sc.ncost,
                                                   sc.nwt, sc.nleaf, max_leaf);
        const uint32_t nb = (m + kCompactBlock - 1) / kCompactBlock;
        k_ploc_block_counts<<<nb, kCompactBlock, 0, st>>>((int)m, sc.keep, sc.bsum);
        PT_CUDA_TRY(cudaMemsetAsync(sc.bsum + nb, 0, sizeof(uint32_t), st));
        k_scan_excl<<<1, 1024, 0, st>>>(sc.bsum, nb + 1);
        k_ploc_compact<<<nb, kCompactBlock, 0, st>>>((int)m, sc.keep, sc.bsum, sc.out_id, sc.cl[cur ^ 1]);
        PT_CUDA_TRY(cudaGetLastError());
        uint32_t next = 0;
        PT_CUDA_TRY(cudaMemcpyAsync(&next, sc.bsum + nb, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        PT_CUDA_TRY(cudaStreamSynchronize(st));
        if (next == 0 || next >= m) return PT_OK;  // cannot happen (the closest pair always merges)
        m = next;
        cur ^= 1;
    }
    const uint32_t nodes2 = 2 * n - 1;
    k_ploc_offsets<<<blocks(nodes2, tb), tb, 0, st>>>((int)n, sc.left, sc.right, sc.parent, sc.ncount, sc.offs,
                                                     sc.counters + 10);
    k_ploc_finish<<<blocks(nodes2, tb), tb, 0, st>>>((int)n, sc.offs, order, sc.nlo, sc.nhi, sc.parent, sc.left,
                                                    sc.right, sc.rfirst, sc.order2, sc.leaf_lo, sc.leaf_hi, sc.par2);
    PT_CUDA_TRY(cudaGetLastError());
    PT_CUDA_TRY(cudaMemcpyAsync(sc.parent, sc.par2, 4 * (size_t)nodes2, cudaMemcpyDeviceToDevice, st));
    PT_CUDA_TRY(cudaMemcpyAsync(order, sc.order2, 4 * (size_t)n, cudaMemcpyDeviceToDevice, st));
    PT_CUDA_TRY(cudaMemcpyAsync(sc.nlo + (n - 1), sc.leaf_lo, 16 * (size_t)n, cudaMemcpyDeviceToDevice, st));
    PT_CUDA_TRY(cudaMemcpyAsync(sc.nhi + (n - 1), sc.leaf_hi, 16 * (size_t)n, cudaMemcpyDeviceToDevice, st));
    uint32_t h[2] = {0, 0};
    int r = -1;
    PT_CUDA_TRY(cudaMemcpyAsync(h, sc.counters + 9, sizeof(h), cudaMemcpyDeviceToHost, st));
    PT_CUDA_TRY(cudaMemcpyAsync(&r, sc.cl[cur], sizeof(int), cudaMemcpyDeviceToHost, st));
    PT_CUDA_TRY(cudaStreamSynchronize(st));
    if (h[1] != 0 || h[0] != n - 1) return PT_OK;  // too deep (or incomplete): radix tree
    *root = r;
    return PT_OK;
}

}  // namespace

int pt_bvh_build_impl(pt_scene *s, const pt_bvh_opts *o, cudaStream_t st) {
    pt_nvtx::Range nv("pt_bvh_build");
    const uint32_t n = s->num_prims;
    const uint32_t tiles = std::max<uint32_t>(1, (n + kSortTile - 1) / kSortTile);
    const int K = (int)o->width;
    PT_CUDA_TRY(cudaEventRecord(s->ev0, st));
    int e = s->bvh_scratch.ensure(carve_size(std::max<uint32_t>(n, 2), tiles));
    if (e != PT_OK) return e;
    Scratch sc;
    char *p = static_cast<char *>(s->bvh_scratch.ptr);
    size_t nn = std::max<uint32_t>(n, 2);
    sc.keys[0] = carve<uint64_t>(p, nn);
    sc.keys[1] = carve<uint64_t>(p, nn);
    sc.vals[0] = carve<uint32_t>(p, nn);
    sc.vals[1] = carve<uint32_t>(p, nn);
    sc.hist = carve<uint32_t>(p, (size_t)256 * tiles);
    sc.plo = carve<float4>(p, nn);
    sc.phi = carve<float4>(p, nn);
    sc.left = carve<int>(p, nn);
    sc.right = carve<int>(p, nn);
    sc.parent = carve<int>(p, 2 * nn);
    sc.rfirst = carve<int>(p, nn);
    sc.ncount = carve<int>(p, 2 * nn);
    sc.nleaf = carve<int>(p, 2 * nn);
    sc.flags = carve<int>(p, nn);
    sc.nlo = carve<float4>(p, 2 * nn);
    sc.nhi = carve<float4>(p, 2 * nn);
    sc.ncost = carve<float>(p, 2 * nn);
    sc.items[0] = carve<int2>(p, nn);
    sc.items[1] = carve<int2>(p, nn);
    sc.counters = carve<uint32_t>(p, 16);
    sc.sah = carve<double>(p, 8);
    sc.cl[0] = carve<int>(p, nn);
    sc.cl[1] = carve<int>(p, nn);
    sc.nn = carve<int>(p, nn);
    sc.out_id = carve<int>(p, nn);
    sc.offs = carve<int>(p, 2 * nn);
    sc.keep = carve<uint32_t>(p, nn + 1);
    sc.order2 = carve<uint32_t>(p, nn);
    sc.leaf_lo = carve<float4>(p, nn);
    sc.leaf_hi = carve<float4>(p, nn);
    sc.nwt = carve<float>(p, 2 * nn);
    sc.bsum = carve<uint32_t>(p, nn / 1024 + 2);
    sc.par2 = carve<int>(p, 2 * nn);
    sc.dval = carve<float>(p, 8 * 2 * nn);
    sc.dsel = carve<uint8_t>(p, 8 * 2 * nn);
    if ((e = s->bvh_order.ensure(std::max<size_t>(4 * (size_t)n, 16))) != PT_OK) return e;
    if ((e = s->prims_bvh.ensure(std::max<size_t>(48 * (size_t)n, 48))) != PT_OK) return e;

    const int tb = 256;
    uint32_t cb_init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
    PT_CUDA_TRY(cudaMemcpyAsync(sc.counters, cb_init, sizeof(cb_init), cudaMemcpyHostToDevice, st));
    int cur = 0;  // sort buffer holding the sorted (code, primitive) pairs
    if (n > 0) {
        const float4 *prims = s->prims_world.as<float4>();
        k_prim_bounds<<<blocks(n, tb), tb, 0, st>>>(prims, n, sc.plo, sc.phi, sc.counters);
        k_morton<<<blocks(n, tb), tb, 0, st>>>(sc.plo, sc.phi, n, sc.counters, sc.keys[0], sc.vals[0]);
        for (int pass = 0; pass < 8; pass++) {
            int shift = pass * 8;
            k_radix_hist<<<tiles, kSortThreads, 0, st>>>(sc.keys[cur], n, shift, sc.hist, tiles);
            k_scan_excl<<<1, 1024, 0, st>>>(sc.hist, 256 * tiles);
            k_radix_scatter<<<tiles, kSortThreads, 0, st>>>(sc.keys[cur], sc.vals[cur], sc.keys[cur ^ 1], sc.vals[cur ^ 1],
                                                             n, shift, sc.hist, tiles);
            cur ^= 1;
        }
        PT_CUDA_TRY(cudaGetLastError());
        // after 8 passes the sorted pairs are back in buffer 0
        PT_CUDA_TRY(cudaMemcpyAsync(s->bvh_order.ptr, sc.vals[cur], 4 * (size_t)n, cudaMemcpyDeviceToDevice, st));
    }
    // binary tree: PLOC by default, the radix tree for PT_BVH_FAST_BUILD, for
    // a PLOC build that did not converge, or one whose wide tree is deeper
    // than the traversal stack covers (kShortStack + kSpillStack entries)
    const auto radix_tree = [&]() -> int {
        if (n == 0) return PT_OK;  // no primitives: nothing to sort or link (2n - 1 would wrap)
        PT_CUDA_TRY(cudaMemcpyAsync(s->bvh_order.ptr, sc.vals[cur], 4 * (size_t)n, cudaMemcpyDeviceToDevice, st));
        PT_CUDA_TRY(cudaMemsetAsync(sc.parent, 0xff, 4 * (2 * (size_t)n - 1), st));
        PT_CUDA_TRY(cudaMemsetAsync(sc.flags, 0, 4 * (size_t)n, st));
        if (n > 1) k_karras<<<blocks(n - 1, tb), tb, 0, st>>>(sc.keys[cur], (int)n, sc.left, sc.right, sc.parent, sc.rfirst);
        k_bottom_up<<<blocks(n, tb), tb, 0, st>>>((int)n, sc.left, sc.right, sc.parent, s->bvh_order.as<uint32_t>(),
                                                  s->prims_world.as<float4>(), sc.plo, sc.phi, sc.nlo, sc.nhi, sc.ncount,
                                                  sc.ncost, sc.nwt, sc.nleaf, sc.flags, (int)o->max_leaf_size);
        PT_CUDA_TRY(cudaGetLastError());
        return PT_OK;
    };
    const auto wide = [&](int root) -> int {
        if (n > 0) {
            k_gather_prims<<<blocks(n, tb), tb, 0, st>>>(s->prims_world.as<float4>(), s->bvh_order.as<uint32_t>(), n,
                                                         s->prims_bvh.as<float4>());
            PT_CUDA_TRY(cudaGetLastError());
        }
        switch (K) {
            case 2: return build_wide<2>(s, sc, n, root, (int)o->max_leaf_size, st);
            case 4: return build_wide<4>(s, sc, n, root, (int)o->max_leaf_size, st);
            default: return build_wide<8>(s, sc, n, root, (int)o->max_leaf_size, st);
        }
    };
    // curve pieces (long, thin, often diagonal) trace faster under the radix
    // tree although PLOC gives them a lower SAH cost (50 k-strand hair at
    // 1080p: 341 vs 320 Msamples/s), so curve-dominated scenes use it
    const bool curve_heavy = 2ull * s->num_curve_pieces > n;
    int root = -1;
    if (n > 1 && !(o->flags & PT_BVH_FAST_BUILD) && !curve_heavy)
        if ((e = ploc_build(s, sc, n, (int)o->max_leaf_size, st, &root)) != PT_OK) return e;
    bool clustered = root >= 0;
    if (!clustered) {
        if ((e = radix_tree()) != PT_OK) return e;
        root = 0;
    }
    if ((e = wide(root)) != PT_OK) return e;
    const uint32_t stack_levels = (uint32_t)ptd::kTraversalStackEntries / (uint32_t)(K - 1);
    if (clustered && s->level_start.size() - 1 > stack_levels) {
        clustered = false;
        if ((e = radix_tree()) != PT_OK) return e;
        if ((e = wide(0)) != PT_OK) return e;
    }
    if (o->width == 8) {  // the traversal reads compressed copies of the 8-wide nodes
        const uint32_t nn = s->level_start.back();
        if ((e = s->cnodes.ensure((size_t)std::max<uint32_t>(nn, 1) * 16 * ptd::kCwFloat4)) != PT_OK) return e;
        if ((e = pt_compress_wide8(s->nodes.as<float>(), nn, s->cnodes.as<float4>(), st)) != PT_OK) return e;
    }
    PT_CUDA_TRY(cudaEventRecord(s->ev1, st));
    PT_CUDA_TRY(cudaEventSynchronize(s->ev1));
    float ms = 0.f;
    PT_CUDA_TRY(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    s->bvh_opts = *o;
    float sah = 0.f;
    if ((e = s->sah_scratch.ensure(64)) != PT_OK) return e;
    if ((e = compute_sah(s, s->sah_scratch.as<double>(), st, sah)) != PT_OK) return e;

    pt_bvh_stats &bs = s->bvh_stats;
    bs.width = o->width;
    bs.num_nodes = s->level_start.back();
    bs.num_prims = n;
    bs.max_depth = (uint32_t)s->level_start.size() - 1;
    bs.sah_cost = sah;
    bs.build_ms = ms;
    bs.node_bytes = (uint64_t)bs.num_nodes * (K == 8 ? 16 * ptd::kCwFloat4 : 32 * K);  // the bytes the traversal reads
    bs.builder = clustered ? PT_BVH_BUILDER_PLOC : PT_BVH_BUILDER_RADIX;
    bs.prim_bytes = (uint64_t)n * 48;
    bs.num_leaves = 0;

    ptd::DevScene &d = s->dev;
    d.nodes = s->nodes.as<float4>();
    d.cnodes = o->width == 8 ? s->cnodes.as<float4>() : nullptr;
    d.prims = s->prims_bvh.as<float4>();
    d.width = o->width;
    d.num_nodes = bs.num_nodes;
    uint32_t max_smem = (uint32_t)std::max(0, s->max_smem_per_block - 64 * 1024) / (32 * K);
    d.smem_nodes = o->width == 8 ? 0 : std::min<uint32_t>(std::min(o->smem_nodes, bs.num_nodes), max_smem);
    d.pad_mag = s->scene_mag;
    s->bvh_built = true;
    return PT_OK;
}

int pt_compress_wide8(const float *nodes, uint32_t n, float4 *out, cudaStream_t st) {
    if (n) k_compress8<<<blocks(n, 128), 128, 0, st>>>(nodes, n, out);
    PT_CUDA_TRY(cudaGetLastError());
    return PT_OK;
}

int pt_bvh_refit_impl(pt_scene *s, cudaStream_t st) {
    pt_nvtx::Range nv("pt_bvh_refit");
    const uint32_t n = s->num_prims;
    PT_CUDA_TRY(cudaEventRecord(s->ev0, st));
    if (n > 0)
        k_gather_prims<<<blocks(n, 256), 256, 0, st>>>(s->prims_world.as<float4>(), s->bvh_order.as<uint32_t>(), n,
                                                        s->prims_bvh.as<float4>());
    switch (s->bvh_opts.width) {
        case 2: refit_levels<2>(s, st); break;
        case 4: refit_levels<4>(s, st); break;
        default: refit_levels<8>(s, st); break;
    }
    PT_CUDA_TRY(cudaGetLastError());
    if (s->bvh_opts.width == 8) {
        const int e = pt_compress_wide8(s->nodes.as<float>(), s->bvh_stats.num_nodes, s->cnodes.as<float4>(), st);
        if (e != PT_OK) return e;
    }
    PT_CUDA_TRY(cudaEventRecord(s->ev1, st));
    PT_CUDA_TRY(cudaEventSynchronize(s->ev1));
    float ms = 0.f;
    PT_CUDA_TRY(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    s->bvh_stats.build_ms = ms;
    int e = s->sah_scratch.ensure(64);
    if (e != PT_OK) return e;
    return compute_sah(s, s->sah_scratch.as<double>(), st, s->bvh_stats.sah_cost);
}

int pt_update_all_world_vertices(pt_scene *s, const float *d_obj_pos, cudaStream_t st) {
    const uint32_t nrec = (uint32_t)s->mesh_instances.size();
    if (nrec == 0) return PT_OK;
    if (!s->xform_table.ptr) {
        std::vector<uint64_t> mesh_start(s->mesh_num_vertices.size() + 1, 0);
        for (size_t m = 0; m < s->mesh_num_vertices.size(); m++) mesh_start[m + 1] = mesh_start[m] + s->mesh_num_vertices[m];
        std::vector<XformRec> recs(nrec);
        for (uint32_t i = 0; i < nrec; i++) {
            const MeshInstanceRef &r = s->mesh_instances[i];
            const float *m = r.to_world;
            recs[i].vstart = r.vertex_offset;
            recs[i].count = s->mesh_num_vertices[r.mesh];
            recs[i].src = (uint32_t)mesh_start[r.mesh];
            recs[i].pad = 0;
            recs[i].m0 = make_float4(m[0], m[1], m[2], m[3]);
            recs[i].m1 = make_float4(m[4], m[5], m[6], m[7]);
            recs[i].m2 = make_float4(m[8], m[9], m[10], m[11]);
        }
        int e = s->xform_table.ensure(sizeof(XformRec) * nrec);
        if (e != PT_OK) return e;
        PT_CUDA_TRY(cudaMemcpy(s->xform_table.ptr, recs.data(), sizeof(XformRec) * nrec, cudaMemcpyHostToDevice));
    }
    const uint32_t total = s->num_vertices;
    if (total) k_transform_all<<<blocks(total, 256), 256, 0, st>>>(d_obj_pos, s->xform_table.as<XformRec>(), nrec, total,
                                                                   s->vpos.as<float4>());
    if (s->num_tris)
        k_rebuild_tri_records<<<blocks(s->num_tris, 256), 256, 0, st>>>(s->tri_vidx.as<uint32_t>(), s->vpos.as<float4>(), 0,
                                                                        s->num_tris, s->prims_world.as<float4>());
    PT_CUDA_TRY(cudaGetLastError());
    PT_CUDA_TRY(cudaStreamSynchronize(st));
    return PT_OK;
}

int pt_update_world_vertices(pt_scene *s, uint32_t mesh, const float *d_obj_pos, uint32_t nv, cudaStream_t st) {
    for (const MeshInstanceRef &r : s->mesh_instances) {
        if (r.mesh != mesh) continue;
        const float *m = r.to_world;
        float4 m0 = make_float4(m[0], m[1], m[2], m[3]), m1 = make_float4(m[4], m[5], m[6], m[7]),
               m2 = make_float4(m[8], m[9], m[10], m[11]);
        if (nv) k_transform_vertices<<<blocks(nv, 256), 256, 0, st>>>(d_obj_pos, nv, m0, m1, m2, s->vpos.as<float4>() + r.vertex_offset);
        uint32_t first = r.prim_offset;
        uint32_t count = 0;
        // triangles of this instance: up to the next mesh instance's first primitive
        uint32_t next = s->num_tris;
        for (const MeshInstanceRef &q : s->mesh_instances)
            if (q.prim_offset > first && q.prim_offset < next) next = q.prim_offset;
        count = next - first;
        if (count) k_rebuild_tri_records<<<blocks(count, 256), 256, 0, st>>>(s->tri_vidx.as<uint32_t>(), s->vpos.as<float4>(),
                                                                             first, count, s->prims_world.as<float4>());
    }
    PT_CUDA_TRY(cudaGetLastError());
    PT_CUDA_TRY(cudaStreamSynchronize(st));
    return PT_OK;
}
