// pt_render.cu -- wavefront path tracer with NEE and MIS on GB300.
//
// Replaces PTPass::OnRun + optixLaunch (example/path_tracer/pt_pass.cpp:
// 39-57, framework/optix/pass.h:71-89) and the OptiX megakernel
// __raygen__main / __miss__* / __closesthit__* (example/path_tracer/main.cu:
// 38-246).  The megakernel's per-path loop is split into kernels over
// device-resident SoA path state:
//
//   raygen      camera rays for every (frame, pixel) slot of a wave
//   per bounce: extend   closest-hit traversal of the active queue
//               shade    hit/miss handling, emitter-hit MIS, Russian
//                        roulette, NEE sample + BSDF eval (shadow queue),
//                        BSDF sample (next active queue)
//               shadow   any-hit traversal; unoccluded NEE adds its radiance
//   accumulate  per pixel, frames in order: the reference's progressive
//               lerp (main.cu:190-196)
//
// Random numbers are drawn per path in exactly the reference's order (2
// jitter, 1 `test`, then per bounce RR 1, emitter select 1, SampleDirect 2,
// BSDF Sample 0-3), so a path consumes the same stream as in the megakernel.
// Queues are compacted with warp ballots and one atomic per block.

#include "pt_internal.h"
#include "pt_bsdf.cuh"
#include "pt_nvtx.h"
#include "pt_traverse.cuh"

#include <algorithm>
#include <mutex>

namespace {
using namespace ptd;

// Paths in flight per wave unless autotuned: 128 Mi slots (about 20 GB of path
// state; 64 frames of 1080p in one wave: fewer, fuller launches per bounce).
constexpr uint32_t kDefaultWavePaths = 128u << 20;

enum Counter : int {
    kNIn = 0,
    kNOut = 1,
    kNShadow = 2,
    kWorkExtend = 3,
    kWorkShadow = 4,
    kOverflow = 5,
    kNonFinite = 6,  // samples whose radiance was NaN or infinite
    kStatBase = 8,  // uint64 statistics start at counters + 8 (32-byte offset)
};
enum Stat : int { kStatExtNodes = 0, kStatExtPrims, kStatShNodes, kStatShPrims, kStatExtRays, kStatShRays, kNumStats };

struct Wave {
    uint32_t npix;
    uint32_t frames;       // frames in this wave
    uint32_t frame0;       // first frame of the wave (relative to the call)
    uint32_t seed0;        // random seed of the call's first frame
    uint32_t cnt0;         // sample_cnt of the call's first frame
    uint32_t last_frame;   // spp - 1: only that frame writes the AOV / test buffers
    uint32_t max_depth;
    uint32_t rng_mode;
    uint32_t accumulate;
};

struct State {
    float4 *ray_o, *ray_d, *hit, *thr, *rad;
    uint2 *rng;
    uint32_t *meta;
    uint32_t *q_in, *q_out;
    float4 *sh_o, *sh_d, *sh_c;
    uint32_t *counters;
    unsigned long long *stats;
};

struct Outputs {
    float4 *accum, *frame;
    float *albedo, *normal, *test;
    uint32_t drop_nonfinite;  // PT_RENDER_DROP_NONFINITE
};

// Multi-scene launch (pt_render_batch): the wave's pixel range is the
// concatenation of every scene's pixels; pix_off[k] is scene k's first.  The
// BVHs are merged into one node / primitive array, roots[k] is scene k's root.
struct Batch {
    const DevScene *scenes;
    const Outputs *outs;
    const uint32_t *pix_off;  // n + 1 entries
    const int *roots;
    uint32_t n;
    uint32_t *bins;           // 2 * nbins words: per-(scene, material type) counts, then cursors
    uint32_t nbins;
};
// Scene of the wave-pixel q: the last k with pix_off[k] <= q.
PT_DI uint32_t batch_scene(const Batch &b, uint32_t q) {
    uint32_t lo = 0, hi = b.n;  // pix_off[lo] <= q < pix_off[hi]
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(b.pix_off + mid) <= q) lo = mid;
        else hi = mid;
    }
    return lo;
}

PT_DI void save_rng(uint2 *dst, const Sampler &s) {
    *dst = make_uint2((uint32_t)s.state, (uint32_t)(s.state >> 32));
}
PT_DI Sampler load_rng(const uint2 *src, uint32_t mode, uint32_t frame_seed) {
    Sampler s;
    uint2 v = *src;
    s.mode = mode;
    s.state = (uint64_t)v.x | ((uint64_t)v.y << 32);
    s.inc = (static_cast<uint64_t>(frame_seed) << 1u) | 1u;
    return s;
}

// Block-aggregated append to two queues: warp ballots give the lane offsets,
// thread 0 does one atomicAdd per queue for the whole block.  sh: 66 words of
// shared memory.  Every thread of the block must call it.
PT_DI void block_push2(bool p0, bool p1, uint32_t *c0, uint32_t *c1, uint32_t &pos0, uint32_t &pos1, uint32_t *sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t b0 = __ballot_sync(0xffffffffu, p0), b1 = __ballot_sync(0xffffffffu, p1);
    uint32_t *wc0 = sh, *wc1 = sh + 32, *base = sh + 64;
    if (lane == 0) {
        wc0[warp] = __popc(b0);
        wc1[warp] = __popc(b1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t s0 = 0, s1 = 0;
        for (int w = 0; w < nw; w++) {
            uint32_t a = wc0[w], b = wc1[w];
            wc0[w] = s0;
            wc1[w] = s1;
            s0 += a;
            s1 += b;
        }
        base[0] = s0 ? atomicAdd(c0, s0) : 0;
        base[1] = s1 ? atomicAdd(c1, s1) : 0;
    }
    __syncthreads();
    uint32_t lt = (1u << lane) - 1u;
    pos0 = base[0] + wc0[warp] + __popc(b0 & lt);
    pos1 = base[1] + wc1[warp] + __popc(b1 & lt);
    __syncthreads();
}

// Camera ray, example/path_tracer/main.cu:58-78.
PT_DI void camera_ray(const DevScene &s, uint32_t x, uint32_t y, Sampler &rng, float3 &o, float3 &d) {
    float jx = rng.next();
    float jy = rng.next();
    float u = (static_cast<float>(x) + jx) / static_cast<float>(s.width_px);
    float v = (static_cast<float>(y) + jy) / static_cast<float>(s.height_px);
    float4 pf = make_float4(u, v, 0.f, 1.f);
    float4 dd = make_float4(dot4(s.s2c[0], pf), dot4(s.s2c[1], pf), dot4(s.s2c[2], pf), dot4(s.s2c[3], pf));
    float inv = 1.0f / dd.w;
    dd = make_float4(dd.x * inv, dd.y * inv, dd.z * inv, dd.w * inv);
    dd.w = 0.f;
    dd = normalize4(dd);
    float3 dw = f3(dot4(s.c2w[0], dd), dot4(s.c2w[1], dd), dot4(s.c2w[2], dd));
    d = normalize(dw);
    o = f3(s.c2w[0].w, s.c2w[1].w, s.c2w[2].w);
}

PT_DI void raygen_one(const DevScene &s, uint32_t p, uint32_t frame_seed, uint32_t rng_mode, float3 &o, float3 &d,
                      Sampler &rng) {
    rng.init(rng_mode, p, frame_seed);
    camera_ray(s, p % s.width_px, p / s.width_px, rng, o, d);
}

template <bool BATCH>
__global__ void k_raygen(DevScene s, Batch bt, State st, Wave w) {
    const uint32_t total = w.frames * w.npix;
    for (uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x; slot < total; slot += gridDim.x * blockDim.x) {
        uint32_t fl = slot / w.npix, p = slot - fl * w.npix;
        Sampler rng;
        float3 o, d;
        if (BATCH) {
            const uint32_t k = batch_scene(bt, p);
            raygen_one(bt.scenes[k], p - bt.pix_off[k], w.seed0 + w.frame0 + fl, w.rng_mode, o, d, rng);
        } else {
            raygen_one(s, p, w.seed0 + w.frame0 + fl, w.rng_mode, o, d, rng);
        }
        st.ray_o[slot] = make_float4(o.x, o.y, o.z, 0.001f);
        st.ray_d[slot] = make_float4(d.x, d.y, d.z, 1e16f);
        st.thr[slot] = make_float4(1.f, 1.f, 1.f, 0.f);
        st.rad[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
        save_rng(st.rng + slot, rng);
        st.meta[slot] = 0;
        st.q_in[slot] = slot;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st.counters[kNIn] = total;
        st.counters[kNOut] = 0;
        st.counters[kNShadow] = 0;
        st.counters[kWorkExtend] = 0;
        st.counters[kWorkShadow] = 0;
    }
}

// Queue hand-over between bounces: the next active queue becomes the input.
__global__ void k_advance(uint32_t *counters) {
    counters[kNIn] = counters[kNOut];
    counters[kNOut] = 0;
    counters[kNShadow] = 0;
    counters[kWorkExtend] = 0;
    counters[kWorkShadow] = 0;
}

template <int K>
PT_DI size_t smem_node_bytes(const DevScene &s) {
    return (size_t)s.smem_nodes * 32 * K;
}

// Ray sources / result sinks of the persistent traversal.
struct ExtendSrc {  // closest hit of the active queue (entries are path slots)
    State st;
    PT_DI int root(uint32_t) const { return 0; }
    PT_DI uint32_t count() const { return st.counters[kNIn]; }
    PT_DI void load(uint32_t i, float3 &o, float3 &d, float &tmin, float &tmax, uint32_t &tag) const {
        uint32_t slot = ld_stream(st.q_in + i);
        float4 o4 = ld_stream(st.ray_o + slot), d4 = ld_stream(st.ray_d + slot);
        o = xyz(o4);
        d = xyz(d4);
        tmin = o4.w;
        tmax = d4.w;
        tag = slot;
    }
    PT_DI void store(uint32_t, uint32_t slot, const TraceResult &r) const {
        st_stream(st.hit + slot, make_float4(r.t, __int_as_float(r.prim), r.u, r.v));
    }
};
struct ShadowSrc {  // any hit of the shadow queue; unoccluded rays add their NEE radiance
    State st;
    PT_DI int root(uint32_t) const { return 0; }
    PT_DI uint32_t count() const { return st.counters[kNShadow]; }
    PT_DI void load(uint32_t i, float3 &o, float3 &d, float &tmin, float &tmax, uint32_t &tag) const {
        float4 o4 = ld_stream(st.sh_o + i), d4 = ld_stream(st.sh_d + i);
        o = xyz(o4);
        d = xyz(d4);
        tmin = o4.w;
        tmax = d4.w;
        tag = i;
    }
    PT_DI void store(uint32_t i, uint32_t, const TraceResult &r) const {
        if (r.prim >= 0) return;
        float4 c = ld_stream(st.sh_c + i);
        uint32_t ps = __float_as_uint(c.w);
        float4 rr = st.rad[ps];
        st.rad[ps] = make_float4(rr.x + c.x, rr.y + c.y, rr.z + c.z, rr.w);
    }
};
// Multi-scene sources: the ray starts at its scene's root of the merged BVH.
struct BatchExtendSrc : ExtendSrc {
    Batch bt;
    uint32_t npix;
    PT_DI int root(uint32_t slot) const { return __ldg(bt.roots + batch_scene(bt, slot % npix)); }
};
struct BatchShadowSrc : ShadowSrc {
    Batch bt;
    uint32_t npix;
    PT_DI int root(uint32_t i) const {
        const uint32_t slot = __float_as_uint(st.sh_c[i].w);
        return __ldg(bt.roots + batch_scene(bt, slot % npix));
    }
};
template <bool ANY>
struct UserSrc {  // pt_trace_rays
    const float4 *rays;
    float4 *hits;
    uint32_t n;
    PT_DI int root(uint32_t) const { return 0; }
    PT_DI uint32_t count() const { return n; }
    PT_DI void load(uint32_t i, float3 &o, float3 &d, float &tmin, float &tmax, uint32_t &tag) const {
        float4 o4 = rays[2 * (size_t)i], d4 = rays[2 * (size_t)i + 1];
        o = xyz(o4);
        d = xyz(d4);
        tmin = o4.w;
        tmax = d4.w;
        tag = i;
    }
    PT_DI void store(uint32_t i, uint32_t, const TraceResult &r) const {
        if (ANY) hits[i] = make_float4(r.prim >= 0 ? 1.f : 0.f, 0.f, 0.f, 0.f);
        else hits[i] = make_float4(r.t, __int_as_float(r.prim), r.u, r.v);
    }
};

// Stages the top smem_nodes nodes in shared memory; returns the stack base.
template <int K>
PT_DI int2 *stage_smem(const DevScene &s, float4 *smem) {
    for (uint32_t i = threadIdx.x; i < s.smem_nodes * 2 * K; i += blockDim.x) smem[i] = __ldg(s.nodes + i);
    __syncthreads();
    return reinterpret_cast<int2 *>(smem + s.smem_nodes * 2 * K);
}

// ANY = false: closest hit of the extension rays; ANY = true: shadow rays.
// Widths 2 and 4 are capped at 72 registers (7 blocks of 128 threads per SM),
// width 8 (compressed nodes) at 96.
template <int K, bool ANY, bool COUNT, bool BATCH = false, bool CURVES = false>
__global__ void __maxnreg__(K == 8 ? 96 : 72) k_trace_queue(DevScene s, State st, Batch bt, uint32_t npix) {
    extern __shared__ float4 smem[];
    int2 *sstack = stage_smem<K>(s, smem);
    if (ANY) {
        if (BATCH) {
            BatchShadowSrc src;
            src.st = st;
            src.bt = bt;
            src.npix = npix;
            trace_persistent<K, true, COUNT, decltype(src), CURVES>(s, smem, sstack, src, st.counters + kWorkShadow, st.counters + kOverflow,
                                             st.stats + kStatShNodes, st.stats + kStatShPrims, st.stats + kStatShRays);
        } else {
            ShadowSrc src{st};
            trace_persistent<K, true, COUNT, decltype(src), CURVES>(s, smem, sstack, src, st.counters + kWorkShadow, st.counters + kOverflow,
                                             st.stats + kStatShNodes, st.stats + kStatShPrims, st.stats + kStatShRays);
        }
    } else {
        if (BATCH) {
            BatchExtendSrc src;
            src.st = st;
            src.bt = bt;
            src.npix = npix;
            trace_persistent<K, false, COUNT, decltype(src), CURVES>(s, smem, sstack, src, st.counters + kWorkExtend, st.counters + kOverflow,
                                              st.stats + kStatExtNodes, st.stats + kStatExtPrims, st.stats + kStatExtRays);
        } else {
            ExtendSrc src{st};
            trace_persistent<K, false, COUNT, decltype(src), CURVES>(s, smem, sstack, src, st.counters + kWorkExtend, st.counters + kOverflow,
                                              st.stats + kStatExtNodes, st.stats + kStatExtPrims, st.stats + kStatExtRays);
        }
    }
}

struct HitGeo {
    float3 pos, nrm;
    float2 uv;
};

// Geometry::GetHitLocalGeometry (framework/render/geometry.h:60-180) on
// world-space data; for a curve hit h.z is the curve parameter.
PT_DI void hit_geometry(const DevScene &s, float4 h, float3 o, float3 d, const DevInstance &in, bool twosided, HitGeo &g) {
    int prim = __float_as_int(h.y);
    if (in.flags & kInstCurve) {  // geometry.h:101-172, in world space
        g.pos = o + h.x * d;
        const float4 *cp = s.curve_cp + 4 * (size_t)s.curve_seg[prim - (int)s.curve_prim0];
        const float4 q[4] = {cp[0], cp[1], cp[2], cp[3]};
        const CurveSeg seg = curve_segment((in.flags >> kInstCurveTypeShift) & 3u, q);
        g.nrm = curve_normal(seg, h.z, g.pos);
        g.uv = make_float2(0.f, 0.f);
    } else if (!(in.flags & kInstSphere)) {
        uint32_t i0 = s.tri_vidx[3 * prim], i1 = s.tri_vidx[3 * prim + 1], i2 = s.tri_vidx[3 * prim + 2];
        float3 p0 = xyz(s.vpos[i0]), p1 = xyz(s.vpos[i1]), p2 = xyz(s.vpos[i2]);
        float u = h.z, v = h.w;
        float w0 = 1.f - u - v;
        g.pos = w0 * p0 + u * p1 + v * p2;
        float3 n;
        if (in.flags & kInstHasNormals) n = w0 * xyz(s.vnrm[i0]) + u * xyz(s.vnrm[i1]) + v * xyz(s.vnrm[i2]);
        else n = cross(p1 - p0, p2 - p0);
        g.nrm = normalize(n);
        if (in.flags & PT_INST_FLIP_NORMALS) g.nrm = g.nrm * -1.f;
        if (in.flags & kInstHasUvs) {
            g.uv = s.vuv[i0] * w0 + s.vuv[i1] * u + s.vuv[i2] * v;
            if (in.flags & PT_INST_FLIP_TEXCOORDS) g.uv.y = 1.f - g.uv.y;
        } else {
            g.uv = make_float2(0.f, 0.f);
        }
    } else {
        g.pos = o + h.x * d;
        float3 local = f3(dot4(in.inv0, make_float4(g.pos.x, g.pos.y, g.pos.z, 1.f)),
                          dot4(in.inv1, make_float4(g.pos.x, g.pos.y, g.pos.z, 1.f)),
                          dot4(in.inv2, make_float4(g.pos.x, g.pos.y, g.pos.z, 1.f)));
        g.nrm = normalize(g.pos - xyz(in.sphere));
        g.uv = sphere_texcoord(normalize(local - xyz(in.obj_center)));
        if (in.flags & PT_INST_FLIP_NORMALS) g.nrm = g.nrm * -1.f;
    }
    if (dot(-d, g.nrm) < 0.f && twosided) g.nrm = -g.nrm;
}

// One bounce of shading for every entry of the active queue.
struct ShadeOut {
    bool push_ext = false, push_sh = false;
    float3 hit_pos = f3s(0.f), sh_d = f3s(0.f), sh_c = f3s(0.f);
    float sh_tmax = 0.f;
};

// One path slot of k_shade: frame fl of the wave, pixel p of scene s.
PT_DI void shade_one(const DevScene &s, const Outputs &out, const State &st, const Wave &w, uint32_t slot, uint32_t fl,
                     uint32_t p, float env_pdf, ShadeOut &so) {
    float3 new_d = f3s(0.f);
    uint32_t meta = st.meta[slot];
    uint32_t depth = meta & 0xffffu;
    bool prev_delta = (meta >> 16) & 1u;
    uint32_t frame = w.frame0 + fl;
    bool last = frame == w.last_frame;
    float4 h = st.hit[slot];
    float3 ro = xyz(st.ray_o[slot]), rd = xyz(st.ray_d[slot]);
    float4 t4 = st.thr[slot];
    float3 thr = xyz(t4);
    float prev_pdf = t4.w;
    float4 r4 = st.rad[slot];
    float3 rad = xyz(r4);
    Sampler rng = load_rng(st.rng + slot, w.rng_mode, w.seed0 + frame);
    int prim = __float_as_int(h.y);
    bool alive = prim >= 0;
    HitGeo g;
    LocalBsdf bsdf;
    if (!alive) {  // __miss__default (main.cu:199-215)
        if (s.has_env) {
            float3 le;
            float epdf = env_pdf;
            if (emitter_type(s.env) == kEmitEnvMap) envmap_eval(s.envmap, ro, normalize(rd), le, epdf);
            else le = xyz(s.env.rad);
            if (depth == 0) rad = rad + le;
            else rad = rad + le * (thr * mis_weight(prev_pdf, epdf));
        }
        if (depth == 0 && last) {
            if (out.albedo) { out.albedo[3 * p] = 0.f; out.albedo[3 * p + 1] = 0.f; out.albedo[3 * p + 2] = 0.f; }
            if (out.normal) { out.normal[3 * p] = 0.f; out.normal[3 * p + 1] = 0.f; out.normal[3 * p + 2] = 0.f; }
        }
    } else {  // ClosestHit (main.cu:220-234)
        const DevInstance &in = s.inst[s.prim_inst[prim]];
        const DevMaterial &m = s.mats[in.material];
        hit_geometry(s, h, ro, rd, in, m.twosided != 0, g);
        bsdf = material_local(m, g.uv);
        int ei = in.emitter_offset >= 0 ? in.emitter_offset + (prim - (int)in.prim_offset) : -1;
        if (depth == 0) {  // main.cu:90-98
            if (ei >= 0) rad = rad + emitter_radiance(s.emitters[ei], s.emit_tex, g.uv);
            if (last) {
                float3 al = bsdf.albedo();
                if (out.albedo) { out.albedo[3 * p] = al.x; out.albedo[3 * p + 1] = al.y; out.albedo[3 * p + 2] = al.z; }
                if (out.normal) { out.normal[3 * p] = g.nrm.x; out.normal[3 * p + 1] = g.nrm.y; out.normal[3 * p + 2] = g.nrm.z; }
            }
        } else if (ei >= 0) {  // emitter hit with MIS (main.cu:175-185)
            const DevEmitter &e = s.emitters[ei];
            float epdf = emitter_eval_pdf(e, g.pos, g.nrm, ro);
            if (!is_zero(epdf)) {
                float mis = prev_delta ? 1.f : mis_weight(prev_pdf, epdf * e.a.y);
                rad = rad + thr * emitter_radiance(e, s.emit_tex, g.uv) * mis;
            }
        }
    }
    if (depth == 0) {  // main.cu:104
        float tv = rng.next();
        if (last && out.test) out.test[p] = tv;
    }
    if (alive) {  // main.cu:107-109
        depth++;
        if (depth >= (w.max_depth ? w.max_depth : s.max_depth)) alive = false;
    }
    if (alive) {  // Russian roulette, main.cu:111-114
        float rr = depth > 2 ? 0.95f : 1.0f;
        if (rng.next() > rr) alive = false;
        else thr = thr / rr;
    }
    if (alive) {  // next-event estimation, main.cu:117-144
        float sel = rng.next();
        float2 xi = rng.next2();
        int ei = select_emitter(s, sel);
        if (ei != -2) {
            const DevEmitter &e = ei >= 0 ? s.emitters[ei] : s.env;
            EmitterSample es;
            if (ei < 0 && emitter_type(e) == kEmitEnvMap) envmap_sample_direct(s.envmap, xi, es);
            else emitter_sample_direct(e, s.emit_tex, g.pos, g.nrm, xi, es);
            if (es.pdf != 0.f) {
                BsdfRecord er;
                er.wi = to_local(es.wi, g.nrm);
                er.wo = to_local(-rd, g.nrm);
                er.f = f3s(0.f);
                er.pdf = 0.f;
                er.type = 0;
                bsdf.eval(er);
                if (!is_zero(er.f * es.pdf)) {
                    float NoL = dot(g.nrm, es.wi);
                    if (NoL > 0.f) {
                        float mis = mis_weight(es.pdf, er.pdf);
                        float pdf = es.pdf * e.a.y;
                        so.sh_c = thr * es.radiance * er.f * NoL * mis / pdf;
                        so.sh_d = es.wi;
                        so.sh_tmax = es.distance - 0.0001f;
                        so.push_sh = true;
                    }
                }
            }
        }
    }
    if (alive) {  // BSDF sampling, main.cu:146-166
        BsdfRecord br;
        br.wo = to_local(-rd, g.nrm);
        br.wi = f3s(0.f);
        br.f = f3s(0.f);
        br.pdf = 0.f;
        br.type = 0;
        bsdf.sample(br, rng);
        if (is_zero(br.f * fabsf(br.wi.z)) || is_zero(br.pdf)) {
            alive = false;
        } else {
            thr = thr * (br.f * fabsf(br.wi.z) / br.pdf);
            new_d = to_world(br.wi, g.nrm);
            prev_pdf = br.pdf;
            prev_delta = (br.type & kDelta) != 0;
            so.push_ext = true;
        }
    }
    if (prim >= 0) so.hit_pos = g.pos;
    st.rad[slot] = make_float4(rad.x, rad.y, rad.z, r4.w);
    if (alive) {
        st.thr[slot] = make_float4(thr.x, thr.y, thr.z, prev_pdf);
        st.meta[slot] = depth | (prev_delta ? (1u << 16) : 0u);
        save_rng(st.rng + slot, rng);
        st.ray_o[slot] = make_float4(so.hit_pos.x, so.hit_pos.y, so.hit_pos.z, 0.001f);
        st.ray_d[slot] = make_float4(new_d.x, new_d.y, new_d.z, 1e16f);
    }
}

template <bool BATCH>
// 3 blocks of 256 threads per SM: at most 85 registers per thread.
__global__ void __launch_bounds__(256, 3) k_shade(DevScene s, Batch bt, State st, Wave w, Outputs out) {
    __shared__ uint32_t push_smem[72];
    const uint32_t n = st.counters[kNIn];
    const float env_pdf = 0.25f * kInvPi;  // ConstEnvEmitter::Eval (env.h:82-85)
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        uint32_t i = base + threadIdx.x;
        bool valid = i < n;
        uint32_t slot = 0;
        ShadeOut so;
        if (valid) {
            slot = st.q_in[i];
            const uint32_t fl = slot / w.npix, q = slot - fl * w.npix;
            if (BATCH) {
                const uint32_t k = batch_scene(bt, q);
                shade_one(bt.scenes[k], bt.outs[k], st, w, slot, fl, q - bt.pix_off[k], env_pdf, so);
            } else {
                shade_one(s, out, st, w, slot, fl, q, env_pdf, so);
            }
        }
        uint32_t pos_ext, pos_sh;
        block_push2(so.push_ext, so.push_sh, st.counters + kNOut, st.counters + kNShadow, pos_ext, pos_sh, push_smem);
        if (so.push_ext) st.q_out[pos_ext] = slot;
        if (so.push_sh) {  // shadow ray from the hit point, tmin 1e-4, tmax distance - 1e-4 (main.cu:122-126)
            st.sh_o[pos_sh] = make_float4(so.hit_pos.x, so.hit_pos.y, so.hit_pos.z, 0.0001f);
            st.sh_d[pos_sh] = make_float4(so.sh_d.x, so.sh_d.y, so.sh_d.z, so.sh_tmax);
            st.sh_c[pos_sh] = make_float4(so.sh_c.x, so.sh_c.y, so.sh_c.z, __uint_as_float(slot));
        }
    }
}


// Material-sorted shading (default; PT_RENDER_NO_MATERIAL_SORT turns it off): the active queue is
// binned by the material type of each hit (0 = miss) before k_shade, so that
// warps run one BSDF at a time (a stable counting sort: see k_bin_count).
constexpr int kNumBins = 8;

PT_DI uint32_t material_bin(const DevScene &s, int prim) {
    return prim >= 0 ? (s.mats[s.inst[s.prim_inst[prim]].material].type & (kNumBins - 1)) : 0u;
}

// Material binning is a stable counting sort over the bins: block b takes
// the contiguous stretch [b * chunk, (b + 1) * chunk) of the queue, so that
// each bin keeps the queue's order (neighbouring path slots, i.e.
// neighbouring pixels, stay neighbours inside a bin).  k_bin_count writes
// every block's per-bin counts, k_bin_scan turns them into each block's first
// position in every bin, k_bin_scatter places the entries.
__device__ __forceinline__ void bin_stretch(uint32_t n, uint32_t &lo, uint32_t &hi) {
    const uint32_t per = (n + gridDim.x - 1) / gridDim.x;
    const uint32_t chunk = (per + blockDim.x - 1) / blockDim.x * blockDim.x;
    lo = min(n, blockIdx.x * chunk);
    hi = min(n, lo + chunk);
}

template <bool BATCH>
__global__ void k_bin_count(DevScene s, Batch bt, uint32_t npix, State st, uint8_t *keys, uint32_t *block_bins) {
    __shared__ uint32_t h[kNumBins];
    if (threadIdx.x < kNumBins) h[threadIdx.x] = 0;
    __syncthreads();
    uint32_t lo, hi;
    bin_stretch(st.counters[kNIn], lo, hi);
    for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        uint32_t slot = st.q_in[i];
        int prim = __float_as_int(st.hit[slot].y);
        const uint32_t key = BATCH ? material_bin(bt.scenes[batch_scene(bt, slot % npix)], prim) : material_bin(s, prim);
        keys[i] = (uint8_t)key;
        atomicAdd(&h[key], 1u);
    }
    __syncthreads();
    if (threadIdx.x < kNumBins) block_bins[blockIdx.x * kNumBins + threadIdx.x] = h[threadIdx.x];
}

// One warp per bin (blockDim = 32 * kNumBins): the bin's total over the
// blocks, the bins' starts, then each block's start in the bin (in place).
__global__ void k_bin_scan(uint32_t *block_bins, uint32_t nblocks) {
    __shared__ uint32_t total[kNumBins];
    const unsigned FULL = 0xffffffffu;
    const uint32_t bin = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t t = 0;
    for (uint32_t b = lane; b < nblocks; b += 32) t += block_bins[b * kNumBins + bin];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(FULL, t, o);
    if (lane == 0) total[bin] = t;
    __syncthreads();
    uint32_t carry = 0;
    for (uint32_t k = 0; k < bin; k++) carry += total[k];
    for (uint32_t b0 = 0; b0 < nblocks; b0 += 32) {
        const uint32_t b = b0 + lane;
        const uint32_t v = b < nblocks ? block_bins[b * kNumBins + bin] : 0u;
        uint32_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (b < nblocks) block_bins[b * kNumBins + bin] = carry + x - v;
        carry += __shfl_sync(FULL, x, 31);
    }
}

// Per stretch of blockDim entries: each warp's count per key, a prefix over
// the warps per key, then every entry at its block's running position in
// its bin plus its rank among the warp's entries of the same key.
__global__ void k_bin_scatter(State st, const uint8_t *keys, const uint32_t *block_bins, uint32_t *q_sorted) {
    constexpr int kWarps = 256 / 32;
    __shared__ uint32_t wc[kWarps][kNumBins];
    __shared__ uint32_t run[kNumBins];
    const unsigned FULL = 0xffffffffu;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x < kNumBins) run[threadIdx.x] = block_bins[blockIdx.x * kNumBins + threadIdx.x];
    if (threadIdx.x < kWarps * kNumBins) wc[threadIdx.x / kNumBins][threadIdx.x % kNumBins] = 0;
    __syncthreads();
    uint32_t lo, hi;
    bin_stretch(st.counters[kNIn], lo, hi);
    for (uint32_t base = lo; base < hi; base += blockDim.x) {  // uniform per block
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < hi;
        const uint32_t key = valid ? keys[i] : 0xffu;
        const unsigned peers = __match_any_sync(FULL, key);
        const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && lane == (uint32_t)(__ffs(peers) - 1)) wc[warp][key] = __popc(peers);
        __syncthreads();
        if (threadIdx.x < kNumBins) {
            uint32_t r = run[threadIdx.x];
            for (int w = 0; w < kWarps; w++) {
                const uint32_t c = wc[w][threadIdx.x];
                wc[w][threadIdx.x] = r;
                r += c;
            }
            run[threadIdx.x] = r;
        }
        __syncthreads();
        if (valid) q_sorted[wc[warp][key] + rank] = st.q_in[i];
        __syncthreads();
        if (threadIdx.x < kWarps * kNumBins) wc[threadIdx.x / kNumBins][threadIdx.x % kNumBins] = 0;
        __syncthreads();
    }
}

// Multi-scene binning: key = scene * 8 + material type, so that after the
// scatter a scene's paths stay together (each scene's BVH and shading data
// are then read by neighbouring warps) and are grouped by BSDF inside it.
__global__ void k_bin_count_batch(Batch bt, uint32_t npix, State st, uint16_t *keys) {
    extern __shared__ uint32_t hb[];
    for (uint32_t k = threadIdx.x; k < bt.nbins; k += blockDim.x) hb[k] = 0;
    __syncthreads();
    const uint32_t n = st.counters[kNIn];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t slot = st.q_in[i];
        const int prim = __float_as_int(st.hit[slot].y);
        const uint32_t sc = batch_scene(bt, slot % npix);
        const uint32_t key = sc * kNumBins + material_bin(bt.scenes[sc], prim);
        keys[i] = static_cast<uint16_t>(key);
        atomicAdd(&hb[key], 1u);
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < bt.nbins; k += blockDim.x)
        if (hb[k]) atomicAdd(bt.bins + k, hb[k]);
}

// One block of 1024 threads: exclusive scan of the counts into the cursors,
// counts cleared for the next bounce (nbins <= 1024).
__global__ void __launch_bounds__(1024) k_bin_scan_batch(Batch bt) {
    __shared__ uint32_t warp_sum[32];
    const uint32_t t = threadIdx.x, lane = t & 31, wid = t >> 5;
    const uint32_t c = t < bt.nbins ? bt.bins[t] : 0u;
    uint32_t x = c;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) warp_sum[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t w = warp_sum[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= (uint32_t)o) w += y;
        }
        warp_sum[lane] = w;
    }
    __syncthreads();
    const uint32_t incl = x + (wid > 0 ? warp_sum[wid - 1] : 0u);
    if (t < bt.nbins) {
        bt.bins[bt.nbins + t] = incl - c;
        bt.bins[t] = 0;
    }
}

// As k_bin_scatter, with the scene-and-material bins (counts and starts in
// 2 x nbins words of dynamic shared memory).
__global__ void k_bin_scatter_batch(Batch bt, State st, const uint16_t *keys, uint32_t *q_sorted) {
    extern __shared__ uint32_t sbins[];
    uint32_t *cnt = sbins, *start = sbins + bt.nbins;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint32_t n = st.counters[kNIn];
    uint32_t *cursor = bt.bins + bt.nbins;
    for (uint32_t blk = blockIdx.x * blockDim.x; blk < n; blk += gridDim.x * blockDim.x) {  // uniform per block
        for (uint32_t k = threadIdx.x; k < bt.nbins; k += blockDim.x) cnt[k] = 0;
        __syncthreads();
        const uint32_t i = blk + threadIdx.x;
        const bool valid = i < n;
        const uint32_t key = valid ? keys[i] : 0xffffffffu;
        const unsigned peers = __match_any_sync(FULL, key);
        const int leader = __ffs(peers) - 1;
        uint32_t pos = 0;
        if (valid && lane == leader) pos = atomicAdd(&cnt[key], (uint32_t)__popc(peers));
        pos = __shfl_sync(FULL, pos, leader);
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < bt.nbins; k += blockDim.x)
            if (cnt[k]) start[k] = atomicAdd(cursor + k, cnt[k]);
        __syncthreads();
        if (valid) q_sorted[start[key] + pos + __popc(peers & ((1u << lane) - 1u))] = st.q_in[i];
        __syncthreads();  // the counts are reset for the next stretch
    }
}

// Accumulation, main.cu:188-196: frames of the wave in order, per pixel.
template <bool BATCH>
__global__ void k_accumulate(State st, Wave w, Outputs out0, Batch bt) {
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < w.npix; q += gridDim.x * blockDim.x) {
        uint32_t p = q;
        Outputs out = out0;
        if (BATCH) {
            const uint32_t k = batch_scene(bt, q);
            out = bt.outs[k];
            p = q - bt.pix_off[k];
        }
        float4 acc = out.accum[p];
        float3 a = xyz(acc);
        for (uint32_t fl = 0; fl < w.frames; fl++) {
            float3 L = xyz(st.rad[(size_t)fl * w.npix + q]);
            if (!(isfinite(L.x) && isfinite(L.y) && isfinite(L.z))) {
                atomicAdd(st.counters + kNonFinite, 1u);
                if (out.drop_nonfinite) L = f3s(0.f);
            }
            uint32_t cnt = w.cnt0 + w.frame0 + fl;
            if (w.accumulate && cnt > 0) {
                const float t = 1.f / (cnt + 1.f);
                L = lerp(a, L, t);
            }
            a = L;
        }
        out.accum[p] = make_float4(a.x, a.y, a.z, 1.f);
        if (out.frame) out.frame[p] = make_float4(a.x, a.y, a.z, 1.f);
    }
}

// pt_trace_rays: rays (ox,oy,oz,tmin, dx,dy,dz,tmax) -> hits.
template <int K, bool ANY, bool CURVES>
__global__ void k_trace_rays(DevScene s, const float4 *rays, float4 *hits, uint32_t n, uint32_t *work, uint32_t *ovf_flag) {
    extern __shared__ float4 smem[];
    int2 *sstack = stage_smem<K>(s, smem);
    UserSrc<ANY> src{rays, hits, n};
    trace_persistent<K, ANY, false, UserSrc<ANY>, CURVES>(s, smem, sstack, src, work, ovf_flag, nullptr, nullptr, nullptr);
}

__global__ void k_bsdf_eval(const float *bsdf, const float *wo, const float *wi, float *f, float *pdf, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    LocalBsdf l = LocalBsdf::from_flat(bsdf + 16 * (size_t)i);
    BsdfRecord r;
    r.wo = f3(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
    r.wi = f3(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
    r.f = f3s(0.f);
    r.pdf = 0.f;
    r.type = 0;
    l.eval(r);
    f[3 * i] = r.f.x;
    f[3 * i + 1] = r.f.y;
    f[3 * i + 2] = r.f.z;
    pdf[i] = r.pdf;
}

__global__ void k_bsdf_sample(const float *bsdf, const float *wo, uint32_t *rng, float *wi, float *f, float *pdf,
                              uint32_t *type, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    LocalBsdf l = LocalBsdf::from_flat(bsdf + 16 * (size_t)i);
    Sampler smp;
    smp.mode = PT_RNG_REF_LCG;
    smp.inc = 0;
    smp.state = rng[i];
    BsdfRecord r;
    r.wo = f3(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
    r.wi = f3s(0.f);
    r.f = f3s(0.f);
    r.pdf = 0.f;
    r.type = 0;
    l.sample(r, smp);
    rng[i] = (uint32_t)smp.state;
    wi[3 * i] = r.wi.x;
    wi[3 * i + 1] = r.wi.y;
    wi[3 * i + 2] = r.wi.z;
    f[3 * i] = r.f.x;
    f[3 * i + 1] = r.f.y;
    f[3 * i + 2] = r.f.z;
    pdf[i] = r.pdf;
    type[i] = r.type;
}

inline uint32_t nblocks(size_t n, int b) { return (uint32_t)std::max<size_t>(1, (n + b - 1) / b); }

template <class F>
int set_smem(F kernel, size_t bytes) {
    if (bytes > 48 * 1024) PT_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return PT_OK;
}

// Events for per-kernel timing (PT_RENDER_KERNEL_TIMING).
struct Timer {
    std::vector<cudaEvent_t> ev;
    std::vector<int> kind;
    size_t used = 0;
    ~Timer() {
        for (auto e : ev) cudaEventDestroy(e);
    }
    void mark(int k, cudaStream_t st) {  // call twice per interval (start, end)
        if (used >= ev.size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            ev.push_back(e);
            kind.push_back(0);
        }
        kind[used] = k;
        cudaEventRecord(ev[used++], st);
    }
};

// Where a render's workspace, events and statistics live: the scene for
// pt_render, the context for pt_render_batch.
struct RunTarget {
    RenderWorkspace *wsp;
    cudaEvent_t ev0, ev1;
    int num_sms;
    uint32_t tuned_block, tuned_wave_paths;
    pt_render_stats *rs;
    bool curves;  // some scene has curve pieces: use the traversal with the curve test
};

static Outputs make_outputs(const pt_frame_buffers *fb, uint32_t flags) {
    Outputs out;
    out.accum = reinterpret_cast<float4 *>(fb->accum);
    out.frame = reinterpret_cast<float4 *>(fb->frame);
    out.albedo = fb->albedo;
    out.normal = fb->normal;
    out.test = fb->test;
    out.drop_nonfinite = (flags & PT_RENDER_DROP_NONFINITE) ? 1u : 0u;
    return out;
}

template <int K>
struct Launcher {
    static int run(pt_scene *s, const pt_render_params *p, const pt_frame_buffers *fb, cudaStream_t st) {
        RunTarget t{&s->ws, s->ev0, s->ev1, s->num_sms, s->tuned_block, s->tuned_wave_paths, &s->render_stats,
                    s->num_curve_pieces > 0};
        const uint32_t max_depth = p->max_depth ? p->max_depth : s->desc_shallow.max_depth;
        const uint32_t npix = s->dev.width_px * s->dev.height_px;
        return run_waves<false>(t, s->dev, Batch{}, npix, max_depth, max_depth, p, make_outputs(fb, p->flags), st);
    }

    // Waves of frames over npix pixels (one scene, or the concatenated
    // pixels of a batch), each captured in a CUDA graph unless timing or
    // NO_GRAPH asks for direct launches.
    template <bool BATCH>
    // max_depth goes to the kernels (0: each scene's own depth), bounces is the
    // number of bounce launches per wave (the largest depth of the scenes).
    static int run_waves(const RunTarget &t, const DevScene &d, const Batch &bt, uint32_t npix, uint32_t max_depth,
                         uint32_t bounces,
                         const pt_render_params *p, const Outputs &out, cudaStream_t st) {
        RenderWorkspace &ws = *t.wsp;
        const bool count = (p->flags & PT_RENDER_COUNTERS) != 0;
        const bool timing = (p->flags & PT_RENDER_KERNEL_TIMING) != 0;
        uint32_t frames_per_wave = p->wave_spp;
        const uint32_t wave_paths = t.tuned_wave_paths ? t.tuned_wave_paths : kDefaultWavePaths;
        if (frames_per_wave == 0) frames_per_wave = std::max<uint32_t>(1, (uint32_t)(wave_paths / std::max<uint32_t>(npix, 1)));
        frames_per_wave = std::max<uint32_t>(1, std::min(frames_per_wave, std::max<uint32_t>(p->spp, 1)));
        const size_t cap = (size_t)frames_per_wave * npix;
        if (cap > 0x7fffffffu) {  // path slots are 32-bit indices
            pt_set_error("a wave of %u frames x %u pixels exceeds 2^31 - 1 path slots; lower wave_spp",
                         frames_per_wave, npix);
            return PT_ERR_INVALID;
        }
        if (ws.capacity < cap) {
            int e;
            if ((e = ws.ray_o.ensure(16 * cap)) || (e = ws.ray_d.ensure(16 * cap)) || (e = ws.hit.ensure(16 * cap)) ||
                (e = ws.thr.ensure(16 * cap)) || (e = ws.rad.ensure(16 * cap)) || (e = ws.rng.ensure(8 * cap)) ||
                (e = ws.meta.ensure(4 * cap)) || (e = ws.q0.ensure(4 * cap)) || (e = ws.q1.ensure(4 * cap)) ||
                (e = ws.sh_o.ensure(16 * cap)) || (e = ws.sh_d.ensure(16 * cap)) || (e = ws.sh_c.ensure(16 * cap)))
                return e;
            ws.capacity = cap;
        }
        int e = ws.counters.ensure(256);
        if (e != PT_OK) return e;
        State stt;
        stt.ray_o = ws.ray_o.as<float4>();
        stt.ray_d = ws.ray_d.as<float4>();
        stt.hit = ws.hit.as<float4>();
        stt.thr = ws.thr.as<float4>();
        stt.rad = ws.rad.as<float4>();
        stt.rng = ws.rng.as<uint2>();
        stt.meta = ws.meta.as<uint32_t>();
        stt.sh_o = ws.sh_o.as<float4>();
        stt.sh_d = ws.sh_d.as<float4>();
        stt.sh_c = ws.sh_c.as<float4>();
        stt.counters = ws.counters.as<uint32_t>();
        stt.stats = reinterpret_cast<unsigned long long *>(ws.counters.as<uint32_t>() + kStatBase);

        const int tb = p->block_size ? (int)p->block_size : (t.tuned_block ? (int)t.tuned_block : 128);
        const size_t smem = (size_t)d.smem_nodes * 32 * K + (size_t)kShortStack * 8 * tb;
        auto k_ext = t.curves ? (count ? k_trace_queue<K, false, true, BATCH, true> : k_trace_queue<K, false, false, BATCH, true>)
                              : (count ? k_trace_queue<K, false, true, BATCH> : k_trace_queue<K, false, false, BATCH>);
        auto k_sh = t.curves ? (count ? k_trace_queue<K, true, true, BATCH, true> : k_trace_queue<K, true, false, BATCH, true>)
                             : (count ? k_trace_queue<K, true, true, BATCH> : k_trace_queue<K, true, false, BATCH>);
        if ((e = set_smem(k_ext, smem)) != PT_OK || (e = set_smem(k_sh, smem)) != PT_OK) return e;
        int occ_t = 0, occ_s = 0;
        PT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_t, k_ext, tb, smem));
        PT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_s, k_shade<BATCH>, 256, 0));
        const uint32_t grid_trace = (uint32_t)std::max(1, occ_t) * t.num_sms;
        const uint32_t grid_shade = (uint32_t)std::max(1, occ_s) * t.num_sms;

        const bool sort = (p->flags & PT_RENDER_NO_MATERIAL_SORT) == 0;
        if (sort && ws.sort_capacity < cap) {
            if ((e = ws.mat_key.ensure(2 * cap)) != PT_OK || (e = ws.sort_tmp.ensure(4 * cap)) != PT_OK) return e;
            ws.sort_capacity = cap;
        }
        int occ_b = 0;
        PT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_b, k_bin_scatter, 256, 0));
        const uint32_t grid_bin = (uint32_t)std::max(1, occ_b) * t.num_sms;
        if (sort && (e = ws.bin_blocks.ensure((size_t)grid_bin * kNumBins * 4)) != PT_OK) return e;

        // The whole render is captured into a CUDA graph on the scene's own
        // stream (ordered after and before the caller's stream by events) and
        // replayed; later calls update the instantiated graph in place.
        const bool graph = (p->flags & (PT_RENDER_NO_GRAPH | PT_RENDER_KERNEL_TIMING)) == 0;
        if (graph && !ws.stream) {
            PT_CUDA_TRY(cudaStreamCreateWithFlags(&ws.stream, cudaStreamNonBlocking));
            PT_CUDA_TRY(cudaEventCreateWithFlags(&ws.ev_in, cudaEventDisableTiming));
            PT_CUDA_TRY(cudaEventCreateWithFlags(&ws.ev_out, cudaEventDisableTiming));
        }
        cudaStream_t ls = graph ? ws.stream : st;
        if (graph) {
            PT_CUDA_TRY(cudaEventRecord(ws.ev_in, st));
            PT_CUDA_TRY(cudaStreamWaitEvent(ws.stream, ws.ev_in, 0));
            PT_CUDA_TRY(cudaStreamBeginCapture(ws.stream, cudaStreamCaptureModeThreadLocal));
        }
        Timer tm;
        uint32_t launches = 0;
        uint32_t waves = 0;
        pt_nvtx::Range nv_render(graph ? "pt_render: capture" : "pt_render: launches");
        if (!graph) PT_CUDA_TRY(cudaEventRecord(t.ev0, st));
        cudaError_t enq = cudaMemsetAsync(ws.counters.ptr, 0, 256, ls);
        for (uint32_t f0 = 0; f0 < p->spp && enq == cudaSuccess; f0 += frames_per_wave) {
            Wave w;
            w.npix = npix;
            w.frames = std::min(frames_per_wave, p->spp - f0);
            w.frame0 = f0;
            w.seed0 = p->seed;
            w.cnt0 = p->sample_cnt;
            w.last_frame = p->spp - 1;
            w.max_depth = max_depth;
            w.rng_mode = p->rng;
            w.accumulate = p->accumulate;
            stt.q_in = ws.q0.as<uint32_t>();
            stt.q_out = ws.q1.as<uint32_t>();
            const size_t slots = (size_t)w.frames * npix;
            pt_nvtx::Range nv_wave("wave");
            {
                pt_nvtx::Range r("raygen");
                k_raygen<BATCH><<<nblocks(slots, 256), 256, 0, ls>>>(d, bt, stt, w);
            }
            launches++;
            for (uint32_t b = 0; b < bounces; b++) {
                pt_nvtx::Range nv_bounce("bounce");
                if (timing) tm.mark(0, ls);
                {
                    pt_nvtx::Range r("extend (closest hit)");
                    k_ext<<<grid_trace, tb, smem, ls>>>(d, stt, bt, npix);
                }
                if (timing) tm.mark(0, ls);
                State shade_st = stt;
                if (sort && BATCH) {
                    k_bin_count_batch<<<grid_bin, 256, bt.nbins * 4, ls>>>(bt, npix, stt, ws.mat_key.as<uint16_t>());
                    k_bin_scan_batch<<<1, 1024, 0, ls>>>(bt);
                    k_bin_scatter_batch<<<grid_bin, 256, 2 * bt.nbins * 4, ls>>>(bt, stt, ws.mat_key.as<uint16_t>(),
                                                                  ws.sort_tmp.as<uint32_t>());
                    shade_st.q_in = ws.sort_tmp.as<uint32_t>();
                    launches += 3;
                } else if (sort) {
                    k_bin_count<BATCH><<<grid_bin, 256, 0, ls>>>(d, bt, npix, stt, ws.mat_key.as<uint8_t>(),
                                                                 ws.bin_blocks.as<uint32_t>());
                    k_bin_scan<<<1, 32 * kNumBins, 0, ls>>>(ws.bin_blocks.as<uint32_t>(), grid_bin);
                    k_bin_scatter<<<grid_bin, 256, 0, ls>>>(stt, ws.mat_key.as<uint8_t>(), ws.bin_blocks.as<uint32_t>(),
                                                            ws.sort_tmp.as<uint32_t>());
                    shade_st.q_in = ws.sort_tmp.as<uint32_t>();
                    launches += 3;
                }
                if (timing) tm.mark(2, ls);
                {
                    pt_nvtx::Range r("shade (MIS, NEE, BSDF sample)");
                    k_shade<BATCH><<<grid_shade, 256, 0, ls>>>(d, bt, shade_st, w, out);
                }
                if (timing) { tm.mark(2, ls); tm.mark(1, ls); }
                {
                    pt_nvtx::Range r("shadow (any hit)");
                    k_sh<<<grid_trace, tb, smem, ls>>>(d, stt, bt, npix);
                }
                if (timing) tm.mark(1, ls);
                k_advance<<<1, 1, 0, ls>>>(stt.counters);
                launches += 4;
                std::swap(stt.q_in, stt.q_out);
            }
            {
                pt_nvtx::Range r("accumulate");
                k_accumulate<BATCH><<<nblocks(npix, 256), 256, 0, ls>>>(stt, w, out, bt);
            }
            launches++;
            waves++;
            enq = cudaGetLastError();
        }
        if (graph) {
            cudaGraph_t g = nullptr;
            cudaError_t ec = cudaStreamEndCapture(ws.stream, &g);
            if (enq != cudaSuccess || ec != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                pt_set_error("render capture failed: %s", cudaGetErrorString(enq != cudaSuccess ? enq : ec));
                return PT_ERR_CUDA;
            }
            bool updated = false;
            if (ws.exec) {
                cudaGraphExecUpdateResultInfo info;
                updated = cudaGraphExecUpdate(ws.exec, g, &info) == cudaSuccess;
                if (!updated) {
                    (void)cudaGetLastError();
                    cudaGraphExecDestroy(ws.exec);
                    ws.exec = nullptr;
                }
            }
            if (!updated) {
                cudaError_t ei = cudaGraphInstantiate(&ws.exec, g, 0);
                if (ei != cudaSuccess) {
                    cudaGraphDestroy(g);
                    ws.exec = nullptr;
                    pt_set_error("cudaGraphInstantiate failed: %s", cudaGetErrorString(ei));
                    return PT_ERR_CUDA;
                }
            }
            cudaGraphDestroy(g);
            pt_nvtx::Range r("pt_render: graph launch");
            PT_CUDA_TRY(cudaEventRecord(t.ev0, ws.stream));
            PT_CUDA_TRY(cudaGraphLaunch(ws.exec, ws.stream));
            PT_CUDA_TRY(cudaEventRecord(t.ev1, ws.stream));
            PT_CUDA_TRY(cudaEventRecord(ws.ev_out, ws.stream));
            PT_CUDA_TRY(cudaStreamWaitEvent(st, ws.ev_out, 0));
        } else {
            if (enq != cudaSuccess) {
                pt_set_error("kernel launch failed: %s", cudaGetErrorString(enq));
                return PT_ERR_CUDA;
            }
        }
        PT_CUDA_TRY(cudaGetLastError());
        if (!graph) {
            // direct launches: time the enqueued work with events around it on the caller's stream
            PT_CUDA_TRY(cudaEventRecord(t.ev1, st));
        }
        PT_CUDA_TRY(cudaEventSynchronize(t.ev1));
        pt_render_stats &rs = *t.rs;
        rs = pt_render_stats{};
        PT_CUDA_TRY(cudaEventElapsedTime(&rs.render_ms, t.ev0, t.ev1));
        for (size_t i = 0; i + 1 < tm.used; i += 2) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, tm.ev[i], tm.ev[i + 1]);
            if (tm.kind[i] == 0) { rs.extend_ms += ms; rs.extend_launches++; }
            else if (tm.kind[i] == 1) { rs.shadow_ms += ms; rs.shadow_launches++; }
            else { rs.shade_ms += ms; rs.shade_launches++; }
        }
        uint32_t hc[8 + 2 * kNumStats] = {};
        PT_CUDA_TRY(cudaMemcpy(hc, ws.counters.ptr, sizeof(hc), cudaMemcpyDeviceToHost));
        const unsigned long long *hs = reinterpret_cast<const unsigned long long *>(hc + kStatBase);
        rs.samples = (uint64_t)npix * p->spp;
        rs.nodes_visited = hs[kStatExtNodes];
        rs.prims_tested = hs[kStatExtPrims];
        rs.shadow_nodes_visited = hs[kStatShNodes];
        rs.shadow_prims_tested = hs[kStatShPrims];
        rs.extension_rays = hs[kStatExtRays];
        rs.shadow_rays = hs[kStatShRays];
        rs.kernel_launches = launches;
        rs.waves = waves;
        rs.overflow = hc[kOverflow];
        rs.nonfinite_samples = hc[kNonFinite];
        if (rs.overflow) {
            pt_set_error("traversal stack overflow");
            return PT_ERR_OOB;
        }
        if (rs.nonfinite_samples && (p->flags & PT_RENDER_CHECK_FINITE)) {
            pt_set_error("%u samples had NaN or infinite radiance", rs.nonfinite_samples);
            return PT_ERR_NAN;
        }
        return PT_OK;
    }

    static int trace(pt_scene *s, const float *rays, float *hits, uint32_t n, int anyhit, cudaStream_t st) {
        const DevScene &d = s->dev;
        int e = s->ws.counters.ensure(256);
        if (e != PT_OK) return e;
        const int tb = 128;
        const size_t smem = (size_t)d.smem_nodes * 32 * K + (size_t)kShortStack * 8 * tb;
        const bool curves = s->num_curve_pieces > 0;
        auto kern = curves ? (anyhit ? k_trace_rays<K, true, true> : k_trace_rays<K, false, true>)
                           : (anyhit ? k_trace_rays<K, true, false> : k_trace_rays<K, false, false>);
        if ((e = set_smem(kern, smem)) != PT_OK) return e;
        int occ = 0;
        PT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, tb, smem));
        uint32_t *c = s->ws.counters.as<uint32_t>();
        PT_CUDA_TRY(cudaMemsetAsync(c, 0, 256, st));
        if (n) kern<<<(uint32_t)std::max(1, occ) * s->num_sms, tb, smem, st>>>(
            d, reinterpret_cast<const float4 *>(rays), reinterpret_cast<float4 *>(hits), n, c + kWorkExtend, c + kOverflow);
        PT_CUDA_TRY(cudaGetLastError());
        uint32_t ovf = 0;
        PT_CUDA_TRY(cudaMemcpyAsync(&ovf, c + kOverflow, 4, cudaMemcpyDeviceToHost, st));
        PT_CUDA_TRY(cudaStreamSynchronize(st));
        if (ovf) {
            pt_set_error("traversal stack overflow");
            return PT_ERR_OOB;
        }
        return PT_OK;
    }
};

// Merged-BVH child rebasing: inner children move by the scene's first node,
// leaf children (count > 0) by its first primitive slot.
template <int K>
__global__ void k_rebase_nodes(float4 *nodes, uint32_t num_nodes, int node_off, int prim_off) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < num_nodes; i += gridDim.x * blockDim.x) {
        float *f = reinterpret_cast<float *>(nodes + (size_t)i * 2 * K);
#pragma unroll
        for (int c = 0; c < K; c++) {
            int ch = __float_as_int(f[6 * K + c]);
            const int cnt = __float_as_int(f[7 * K + c]);
            if (ch < 0) continue;
            ch += cnt > 0 ? prim_off : node_off;
            f[6 * K + c] = __int_as_float(ch);
        }
    }
}

}  // namespace

// pt_render_batch state, owned by the context: merged BVH, per-scene tables,
// the wave workspace (with its CUDA graph) and the last call's statistics.
struct BatchWorkspace {
    RenderWorkspace ws;
    DevBuf nodes, cnodes, prims, scenes, outs, pix_off, roots, bins;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    pt_render_stats stats{};
};

void pt_batch_release(BatchWorkspace *b) {
    if (!b) return;
    DevBuf *bufs[] = {&b->nodes, &b->cnodes, &b->prims, &b->scenes, &b->outs, &b->pix_off, &b->roots, &b->bins};
    for (DevBuf *d : bufs) d->release();
    RenderWorkspace &w = b->ws;
    DevBuf *wb[] = {&w.ray_o, &w.ray_d, &w.hit, &w.thr, &w.rad, &w.rng, &w.meta, &w.q0,
                    &w.q1, &w.sh_o, &w.sh_d, &w.sh_c, &w.mat_key, &w.counters, &w.sort_tmp, &w.bin_blocks};
    for (DevBuf *d : wb) d->release();
    if (w.exec) cudaGraphExecDestroy(w.exec);
    if (w.ev_in) cudaEventDestroy(w.ev_in);
    if (w.ev_out) cudaEventDestroy(w.ev_out);
    if (w.stream) cudaStreamDestroy(w.stream);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    delete b;
}

namespace {

template <int K>
int render_batch(pt_context *ctx, pt_scene *const *scenes, const pt_render_params *p, const pt_frame_buffers *fbs,
                 uint32_t n, cudaStream_t st) {
    if (!ctx->batch) {
        ctx->batch = new BatchWorkspace();
        PT_CUDA_TRY(cudaEventCreate(&ctx->batch->ev0));
        PT_CUDA_TRY(cudaEventCreate(&ctx->batch->ev1));
    }
    BatchWorkspace &b = *ctx->batch;
    // merged BVH: every scene's nodes and leaf-order primitive records, rebased
    std::vector<DevScene> hs(n);
    std::vector<Outputs> ho(n);
    std::vector<uint32_t> pix_off(n + 1, 0);
    std::vector<int> roots(n);
    uint64_t total_nodes = 0, total_prims = 0, total_pix = 0;
    float pad_mag = 0.f;
    for (uint32_t k = 0; k < n; k++) {
        const pt_scene *s = scenes[k];
        roots[k] = static_cast<int>(total_nodes);
        pix_off[k] = static_cast<uint32_t>(total_pix);
        total_nodes += s->dev.num_nodes;
        total_prims += s->num_prims;
        total_pix += (uint64_t)s->dev.width_px * s->dev.height_px;
        pad_mag = std::max(pad_mag, s->dev.pad_mag);
        hs[k] = s->dev;
        ho[k] = make_outputs(&fbs[k], p->flags);
    }
    if (n * kNumBins > 1024) {
        pt_set_error("pt_render_batch: at most %d scenes per call", 1024 / kNumBins);
        return PT_ERR_INVALID;
    }
    if (total_prims > ptd::kMaxPrimitives || total_nodes >= (1u << 31) || total_pix >= (1ull << 31)) {
        pt_set_error("pt_render_batch: batch too large (%llu primitives, %llu pixels)",
                     (unsigned long long)total_prims, (unsigned long long)total_pix);
        return PT_ERR_INVALID;
    }
    pix_off[n] = static_cast<uint32_t>(total_pix);
    int e;
    if ((e = b.nodes.ensure(std::max<uint64_t>(total_nodes, 1) * 32 * K)) != PT_OK ||
        (e = b.prims.ensure(std::max<uint64_t>(total_prims, 1) * 48)) != PT_OK ||
        (e = b.scenes.ensure(n * sizeof(DevScene))) != PT_OK || (e = b.outs.ensure(n * sizeof(Outputs))) != PT_OK ||
        (e = b.pix_off.ensure((n + 1) * sizeof(uint32_t))) != PT_OK || (e = b.roots.ensure(n * sizeof(int))) != PT_OK ||
        (e = b.bins.ensure(2 * 1024 * sizeof(uint32_t))) != PT_OK)
        return e;
    PT_CUDA_TRY(cudaMemsetAsync(b.bins.ptr, 0, 2 * 1024 * sizeof(uint32_t), st));
    uint64_t node_off = 0, prim_off = 0;
    for (uint32_t k = 0; k < n; k++) {
        const pt_scene *s = scenes[k];
        float4 *dn = b.nodes.as<float4>() + node_off * 2 * K;
        PT_CUDA_TRY(cudaMemcpyAsync(dn, s->dev.nodes, (size_t)s->dev.num_nodes * 32 * K, cudaMemcpyDeviceToDevice, st));
        PT_CUDA_TRY(cudaMemcpyAsync(b.prims.as<float4>() + prim_off * 3, s->dev.prims, (size_t)s->num_prims * 48,
                                    cudaMemcpyDeviceToDevice, st));
        k_rebase_nodes<K><<<nblocks(s->dev.num_nodes, 256), 256, 0, st>>>(dn, s->dev.num_nodes, (int)node_off,
                                                                          (int)prim_off);
        PT_CUDA_TRY(cudaGetLastError());
        node_off += s->dev.num_nodes;
        prim_off += s->num_prims;
    }
    if (K == 8) {  // the traversal reads compressed copies of the merged 8-wide nodes
        if ((e = b.cnodes.ensure(std::max<uint64_t>(total_nodes, 1) * 16 * ptd::kCwFloat4)) != PT_OK) return e;
        if ((e = pt_compress_wide8(b.nodes.as<float>(), static_cast<uint32_t>(total_nodes), b.cnodes.as<float4>(),
                                   st)) != PT_OK)
            return e;
    }
    PT_CUDA_TRY(cudaMemcpyAsync(b.scenes.ptr, hs.data(), n * sizeof(DevScene), cudaMemcpyHostToDevice, st));
    PT_CUDA_TRY(cudaMemcpyAsync(b.outs.ptr, ho.data(), n * sizeof(Outputs), cudaMemcpyHostToDevice, st));
    PT_CUDA_TRY(cudaMemcpyAsync(b.pix_off.ptr, pix_off.data(), (n + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    PT_CUDA_TRY(cudaMemcpyAsync(b.roots.ptr, roots.data(), n * sizeof(int), cudaMemcpyHostToDevice, st));
    // the host tables above are pageable: finish the copies before they go out of scope
    PT_CUDA_TRY(cudaStreamSynchronize(st));

    DevScene dt = scenes[0]->dev;  // traversal view: merged arrays, no shared-memory top levels
    dt.nodes = b.nodes.as<float4>();
    dt.cnodes = K == 8 ? b.cnodes.as<float4>() : nullptr;
    dt.prims = b.prims.as<float4>();
    dt.num_nodes = static_cast<uint32_t>(total_nodes);
    dt.smem_nodes = 0;
    dt.pad_mag = pad_mag;
    Batch bt;
    bt.scenes = b.scenes.as<DevScene>();
    bt.outs = b.outs.as<Outputs>();
    bt.pix_off = b.pix_off.as<uint32_t>();
    bt.roots = b.roots.as<int>();
    bt.n = n;
    bt.bins = b.bins.as<uint32_t>();
    bt.nbins = n * kNumBins;
    const uint32_t max_depth = p->max_depth;  // 0: each scene's own depth (DevScene::max_depth)
    uint32_t bounces = max_depth;
    if (!bounces)
        for (uint32_t k = 0; k < n; k++) bounces = std::max(bounces, scenes[k]->dev.max_depth);
    bool curves = false;
    for (uint32_t k = 0; k < n; k++) curves = curves || scenes[k]->num_curve_pieces > 0;
    RunTarget t{&b.ws, b.ev0, b.ev1, ctx->num_sms, 0, 0, &b.stats, curves};
    Outputs none{};
    return Launcher<K>::template run_waves<true>(t, dt, bt, static_cast<uint32_t>(total_pix), max_depth, bounces, p,
                                                 none, st);
}

}  // namespace

int pt_render_batch_impl(pt_context *ctx, pt_scene *const *scenes, const pt_render_params *p,
                         const pt_frame_buffers *fbs, uint32_t n, cudaStream_t st) {
    if (p->spp == 0 || n == 0) return PT_OK;
    switch (scenes[0]->dev.width) {
        case 2: return render_batch<2>(ctx, scenes, p, fbs, n, st);
        case 4: return render_batch<4>(ctx, scenes, p, fbs, n, st);
        default: return render_batch<8>(ctx, scenes, p, fbs, n, st);
    }
}

int pt_render_batch_stats(const pt_context *ctx, pt_render_stats *out) {
    if (!ctx->batch) {
        pt_set_error("pt_render_batch_get_stats: no batch rendered on this context");
        return PT_ERR_STATE;
    }
    *out = ctx->batch->stats;
    return PT_OK;
}

int pt_render_impl(pt_scene *s, const pt_render_params *p, const pt_frame_buffers *fb, cudaStream_t st) {
    if (p->spp == 0) return PT_OK;
    switch (s->dev.width) {
        case 2: return Launcher<2>::run(s, p, fb, st);
        case 4: return Launcher<4>::run(s, p, fb, st);
        default: return Launcher<8>::run(s, p, fb, st);
    }
}

// Autotuner (coordinate search): every (BVH width, block size) pair renders
// params->spp frames at the default wave size, then the wave sizes are tried
// with the best pair.  The fastest by device time is applied to the scene.
int pt_autotune_impl(pt_scene *s, const pt_render_params *params, const pt_frame_buffers *fb, pt_tune_result *out,
                     cudaStream_t st) {
    const uint32_t npix = s->dev.width_px * s->dev.height_px;
    const uint32_t spp = std::max<uint32_t>(1, params->spp);
    pt_tune_result r{};
    pt_bvh_opts opts = s->bvh_opts;
    pt_render_params p = *params;
    p.spp = spp;
    p.block_size = 0;
    p.wave_spp = 0;
    p.flags &= ~(uint32_t)(PT_RENDER_KERNEL_TIMING | PT_RENDER_COUNTERS);
    auto time_render = [&](float &ms) -> int {
        int e = pt_render_impl(s, &p, fb, st);  // warm-up (graph instantiation, caches)
        if (e != PT_OK) return e;
        e = pt_render_impl(s, &p, fb, st);
        ms = s->render_stats.render_ms;
        r.trials++;
        return e;
    };
    const uint32_t default_wave = kDefaultWavePaths;
    float base_ms = 0.f;
    int e = time_render(base_ms);
    if (e != PT_OK) return e;
    r.baseline_msamples_per_s = base_ms > 0.f ? (float)((double)npix * spp / (base_ms * 1e-3) / 1e6) : 0.f;
    float best_ms = 1e30f;
    uint32_t best_w = opts.width, best_b = 128, best_wave = default_wave;
    const uint32_t widths[3] = {2, 4, 8}, blocks[3] = {64, 128, 256}, waves[3] = {16u << 20, 32u << 20, 64u << 20};
    for (uint32_t wd : widths) {
        opts.width = wd;
        if ((e = pt_bvh_build_impl(s, &opts, st)) != PT_OK) return e;
        for (uint32_t bs : blocks) {
            s->tuned_block = bs;
            s->tuned_wave_paths = default_wave;
            float ms = 0.f;
            if ((e = time_render(ms)) != PT_OK) return e;
            if (ms < best_ms) {
                best_ms = ms;
                best_w = wd;
                best_b = bs;
            }
        }
    }
    opts.width = best_w;
    if ((e = pt_bvh_build_impl(s, &opts, st)) != PT_OK) return e;
    s->tuned_block = best_b;
    uint32_t prev_frames = std::max<uint32_t>(1, std::min(spp, default_wave / std::max<uint32_t>(npix, 1)));
    for (uint32_t wv : waves) {
        uint32_t frames = std::max<uint32_t>(1, std::min(spp, wv / std::max<uint32_t>(npix, 1)));
        if (frames == prev_frames && wv != default_wave) continue;  // same effective wave as the default
        if (wv == default_wave) continue;
        s->tuned_wave_paths = wv;
        float ms = 0.f;
        if ((e = time_render(ms)) != PT_OK) return e;
        if (ms < best_ms) {
            best_ms = ms;
            best_wave = wv;
        }
    }
    s->tuned_wave_paths = best_wave;
    r.bvh_width = best_w;
    r.block_size = best_b;
    r.wave_paths = best_wave;
    r.msamples_per_s = (float)((double)npix * spp / (best_ms * 1e-3) / 1e6);
    if (out) *out = r;
    return PT_OK;
}

int pt_trace_rays_impl(pt_scene *s, const float *rays, float *hits, uint32_t n, int anyhit, cudaStream_t st) {
    switch (s->dev.width) {
        case 2: return Launcher<2>::trace(s, rays, hits, n, anyhit, st);
        case 4: return Launcher<4>::trace(s, rays, hits, n, anyhit, st);
        default: return Launcher<8>::trace(s, rays, hits, n, anyhit, st);
    }
}

// pt_trig_eval: the library's trigonometry next to CUDA's, for the accuracy
// and host-equality checks of pt_trig.h.
__global__ void k_trig_eval(uint32_t fn, const float *x, const float *y, float *out, float *out_platform, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float a = x[i];
    float ours, theirs;
    switch (fn) {
        case 0: ours = pt_sinf(a); theirs = sinf(a); break;
        case 1: ours = pt_cosf(a); theirs = cosf(a); break;
        case 2: ours = pt_atan2f(y[i], a); theirs = atan2f(y[i], a); break;
        default: ours = pt_acosf(a); theirs = acosf(a); break;
    }
    out[i] = ours;
    if (out_platform) out_platform[i] = theirs;
}

int pt_trig_eval_impl(uint32_t fn, const float *x, const float *y, float *out, float *out_platform, uint32_t n,
                      cudaStream_t st) {
    if (n) k_trig_eval<<<nblocks(n, 256), 256, 0, st>>>(fn, x, y, out, out_platform, n);
    PT_CUDA_TRY(cudaGetLastError());
    PT_CUDA_TRY(cudaStreamSynchronize(st));
    return PT_OK;
}

int pt_bsdf_eval_impl(const float *bsdf, const float *wo, const float *wi, float *f, float *pdf, uint32_t n, cudaStream_t st) {
    if (n) k_bsdf_eval<<<nblocks(n, 128), 128, 0, st>>>(bsdf, wo, wi, f, pdf, n);
    PT_CUDA_TRY(cudaGetLastError());
    PT_CUDA_TRY(cudaStreamSynchronize(st));
    return PT_OK;
}

int pt_bsdf_sample_impl(const float *bsdf, const float *wo, uint32_t *rng, float *wi, float *f, float *pdf, uint32_t *type,
                        uint32_t n, cudaStream_t st) {
    if (n) k_bsdf_sample<<<nblocks(n, 128), 128, 0, st>>>(bsdf, wo, rng, wi, f, pdf, type, n);
    PT_CUDA_TRY(cudaGetLastError());
    PT_CUDA_TRY(cudaStreamSynchronize(st));
    return PT_OK;
}

// ---------------------------------------------------------------------------
// pt_render_noalloc: the same wavefront render for callers that cannot
// allocate device memory themselves (hosts that hand out device memory only
// from their own fixed pools or budgets, and interactive callers that must
// not allocate per frame, since an allocation can synchronise the device).
// The path state lives in the file-scope array below instead of the scene's
// workspace, so a call allocates nothing.  Limit: at most kNoAllocMaxPixels
// pixels per call (frames are packed into waves of at most that many slots).
// Every call shares the array; calls that overlap on the GPU (on different
// streams or threads) race on it.
// ---------------------------------------------------------------------------
namespace {

constexpr uint32_t kNoAllocMaxPixels = 1u << 16;  // 65,536 path slots
constexpr size_t kNoAllocCounterBytes = 256;
constexpr size_t kNoAllocSlotBytes = 16 * 8 + 8 + 4 * 3;  // 8 float4 arrays, rng, meta, two queues = 148 B
constexpr size_t kNoAllocScratchBytes = kNoAllocCounterBytes + kNoAllocSlotBytes * kNoAllocMaxPixels;

// About 9.3 MiB, held by every GPU that loads the library until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[128] = {};  // device address of the array, per CUDA device

// Device address of g_noalloc_scratch on the current device, looked up once
// per device (the first call on a device does the look-up).
int noalloc_scratch(int device, unsigned char **out) {
    if (device < 0 || device >= 128) {
        pt_set_error("device ordinal %d out of range", device);
        return PT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            pt_set_error("cudaGetSymbolAddress(g_noalloc_scratch) failed: %s", cudaGetErrorString(e));
            return PT_ERR_CUDA;
        }
        g_noalloc_ptr[device] = p;
    }
    *out = static_cast<unsigned char *>(g_noalloc_ptr[device]);
    return PT_OK;
}

template <int K>
int render_noalloc(pt_scene *s, const pt_render_params *p, const pt_frame_buffers *fb, unsigned char *scratch,
                   cudaStream_t st) {
    const DevScene &d = s->dev;
    const uint32_t npix = d.width_px * d.height_px;
    const uint32_t max_depth = p->max_depth ? p->max_depth : s->desc_shallow.max_depth;
    const uint32_t frames_per_wave = std::max<uint32_t>(1, std::min(kNoAllocMaxPixels / npix, p->spp));
    const size_t cap = kNoAllocMaxPixels;
    State stt;
    unsigned char *q = scratch + kNoAllocCounterBytes;
    auto take = [&](size_t bytes_per_slot) {
        unsigned char *r = q;
        q += bytes_per_slot * cap;
        return r;
    };
    stt.counters = reinterpret_cast<uint32_t *>(scratch);
    stt.stats = reinterpret_cast<unsigned long long *>(stt.counters + kStatBase);
    stt.ray_o = reinterpret_cast<float4 *>(take(16));
    stt.ray_d = reinterpret_cast<float4 *>(take(16));
    stt.hit = reinterpret_cast<float4 *>(take(16));
    stt.thr = reinterpret_cast<float4 *>(take(16));
    stt.rad = reinterpret_cast<float4 *>(take(16));
    stt.sh_o = reinterpret_cast<float4 *>(take(16));
    stt.sh_d = reinterpret_cast<float4 *>(take(16));
    stt.sh_c = reinterpret_cast<float4 *>(take(16));
    stt.rng = reinterpret_cast<uint2 *>(take(8));
    stt.meta = reinterpret_cast<uint32_t *>(take(4));
    uint32_t *q0 = reinterpret_cast<uint32_t *>(take(4));
    uint32_t *q1 = reinterpret_cast<uint32_t *>(take(4));
    Outputs out;
    out.accum = reinterpret_cast<float4 *>(fb->accum);
    out.frame = reinterpret_cast<float4 *>(fb->frame);
    out.albedo = fb->albedo;
    out.normal = fb->normal;
    out.test = fb->test;
    out.drop_nonfinite = (p->flags & PT_RENDER_DROP_NONFINITE) ? 1u : 0u;

    // the traversal block size pt_render would use: the caller's, else the autotuned one, else 128
    const int tb = p->block_size ? (int)p->block_size : (s->tuned_block ? (int)s->tuned_block : 128);
    const size_t smem = (size_t)d.smem_nodes * 32 * K + (size_t)kShortStack * 8 * tb;
    const bool curves = s->num_curve_pieces > 0;
    auto k_ext = curves ? k_trace_queue<K, false, false, false, true> : k_trace_queue<K, false, false>;
    auto k_sh = curves ? k_trace_queue<K, true, false, false, true> : k_trace_queue<K, true, false>;
    int e;
    if ((e = set_smem(k_ext, smem)) != PT_OK || (e = set_smem(k_sh, smem)) != PT_OK) return e;
    int occ_t = 0, occ_s = 0;
    PT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_t, k_ext, tb, smem));
    PT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_s, k_shade<false>, 256, 0));
    const uint32_t grid_trace = (uint32_t)std::max(1, occ_t) * s->num_sms;
    const uint32_t grid_shade = (uint32_t)std::max(1, occ_s) * s->num_sms;

    // the array keeps the previous call's contents: clear the counters and statistics
    PT_CUDA_TRY(cudaMemsetAsync(scratch, 0, kNoAllocCounterBytes, st));
    for (uint32_t f0 = 0; f0 < p->spp; f0 += frames_per_wave) {
        Wave w;
        w.npix = npix;
        w.frames = std::min(frames_per_wave, p->spp - f0);
        w.frame0 = f0;
        w.seed0 = p->seed;
        w.cnt0 = p->sample_cnt;
        w.last_frame = p->spp - 1;
        w.max_depth = max_depth;
        w.rng_mode = p->rng;
        w.accumulate = p->accumulate;
        stt.q_in = q0;
        stt.q_out = q1;
        k_raygen<false><<<nblocks((size_t)w.frames * npix, 256), 256, 0, st>>>(d, Batch{}, stt, w);
        for (uint32_t b = 0; b < max_depth; b++) {
            k_ext<<<grid_trace, tb, smem, st>>>(d, stt, Batch{}, npix);
            k_shade<false><<<grid_shade, 256, 0, st>>>(d, Batch{}, stt, w, out);
            k_sh<<<grid_trace, tb, smem, st>>>(d, stt, Batch{}, npix);
            k_advance<<<1, 1, 0, st>>>(stt.counters);
            std::swap(stt.q_in, stt.q_out);
        }
        k_accumulate<false><<<nblocks(npix, 256), 256, 0, st>>>(stt, w, out, Batch{});
    }
    PT_CUDA_TRY(cudaGetLastError());
    // the overflow and non-finite counters are adjacent: one small read-back
    static_assert(kNonFinite == kOverflow + 1, "counter layout");
    uint32_t hc[2] = {0, 0};
    PT_CUDA_TRY(cudaMemcpyAsync(hc, stt.counters + kOverflow, sizeof(hc), cudaMemcpyDeviceToHost, st));
    PT_CUDA_TRY(cudaStreamSynchronize(st));
    if (hc[0]) {
        pt_set_error("traversal stack overflow");
        return PT_ERR_OOB;
    }
    if (hc[1] && (p->flags & PT_RENDER_CHECK_FINITE)) {
        pt_set_error("%u samples had NaN or infinite radiance", hc[1]);
        return PT_ERR_NAN;
    }
    return PT_OK;
}

int render_noalloc_checked(pt_scene *scene, const pt_render_params *params, const pt_frame_buffers *fb, void *stream);

}  // namespace

extern "C" int pt_render_noalloc(pt_scene *scene, const pt_render_params *params, const pt_frame_buffers *fb,
                                 void *stream) {
    // as every entry point: an error left behind by another call in the process
    // is not reported here, and no C++ exception (std::mutex::lock may throw)
    // crosses the C ABI
    (void)cudaGetLastError();
    try {
        return render_noalloc_checked(scene, params, fb, stream);
    } catch (const std::exception &e) {
        pt_set_error("pt_render_noalloc: %s", e.what());
        return PT_ERR_INVALID;
    } catch (...) {
        pt_set_error("pt_render_noalloc: unexpected C++ exception");
        return PT_ERR_INVALID;
    }
}

namespace {

int render_noalloc_checked(pt_scene *scene, const pt_render_params *params, const pt_frame_buffers *fb, void *stream) {
    if (!scene || !params || !fb || !fb->accum) {
        pt_set_error("scene, params, buffers or accum is NULL");
        return PT_ERR_INVALID;
    }
    if (!scene->bvh_built) {
        pt_set_error("pt_render_noalloc before pt_bvh_build");
        return PT_ERR_STATE;
    }
    if (params->rng != PT_RNG_REF_LCG && params->rng != PT_RNG_PCG32) {
        pt_set_error("unknown rng mode");
        return PT_ERR_INVALID;
    }
    const uint64_t npix = (uint64_t)scene->dev.width_px * scene->dev.height_px;
    if (npix > kNoAllocMaxPixels) {
        pt_set_error("pt_render_noalloc: %llu pixels exceed the limit of %u pixels per call "
                     "(its path state lives in a fixed %zu-byte device array); use pt_render",
                     (unsigned long long)npix, kNoAllocMaxPixels, kNoAllocScratchBytes);
        return PT_ERR_INVALID;
    }
    if (params->spp == 0) return PT_OK;
    PT_CUDA_TRY(cudaSetDevice(scene->device));
    unsigned char *scratch = nullptr;
    int e = noalloc_scratch(scene->device, &scratch);
    if (e != PT_OK) return e;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    switch (scene->dev.width) {
        case 2: return render_noalloc<2>(scene, params, fb, scratch, st);
        case 4: return render_noalloc<4>(scene, params, fb, scratch, st);
        default: return render_noalloc<8>(scene, params, fb, scratch, st);
    }
}

}  // namespace
