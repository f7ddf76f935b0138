// pt_traverse.cuh -- short-stack closest-hit and any-hit traversal of the
// wide BVH (2, 4 or 8 children per node) on FP32 SIMT cores.
//
// Replaces optixTrace (example/path_tracer/main.cu:80-85,161-166; closest hit,
// tmin 0.001, tmax 1e16) and Emitter::TraceShadowRay (framework/render/
// emitter.h:91-100; terminate on first hit).  Result semantics (shared with
// the CPU oracle): a primitive is hit at tmin < t < tmax; the closest hit is
// the smallest t, ties broken by the smaller primitive id, so the answer does
// not depend on traversal order.  The triangle test is the watertight test of
// Woop, Benthin and Wald (JCGT 2013) evaluated with explicitly rounded
// operations (no FMA contraction), which makes hit ids and distances bit-equal
// to the host restatement.
//
// Memory layout (HBM):
//   node  = 8*K floats: lo_x[K] hi_x[K] lo_y[K] hi_y[K] lo_z[K] hi_z[K]
//           child[K] count[K]; count > 0: leaf over primitive slots
//           [child, child + count); count == 0 and child >= 0: inner node;
//           child < 0: empty slot.  Loaded as 2*K float4 (128-bit) loads.
//   prim  = 3 float4 per slot: triangle (v0, id) (v1, 0) (v2, 0);
//           sphere (centre, id | 1<<31) (radius, 0, 0, 0) (0);
//           curve piece (c0, id | 1<<31) (r0, r1, u0, kind bits) (c1, u1):
//           a round cone from centre c0 / radius r0 to c1 / r1 covering the
//           curve parameters [u0, u1] of its segment (pt_curve.h).
// Nodes are in breadth-first order, so the first smem_nodes nodes are the
// top levels; those are staged in shared memory once per (persistent) block.
// Width 8 traverses compressed copies of the nodes instead (CwNode below).
#pragma once

#include "pt_curve.h"
#include "pt_device.cuh"

namespace ptd {

constexpr int kShortStack = 16;  // shared-memory entries per thread
constexpr int kSpillStack = kTraversalStackEntries - kShortStack;  // local-memory overflow entries per thread
constexpr float kSlabScale = 1.0000004f;  // 1 + 2*gamma(3): robust slab far bound (Ize 2013)

struct TraceResult {
    float t;
    int prim;
    float u, v;
};

struct RayWT {  // per-ray constants of the watertight test
    int kx, ky, kz;
    float sx, sy, sz;
};

PT_DI float sel3(float3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

PT_DI RayWT ray_wt(float3 d) {
    RayWT r;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    r.kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    r.kx = r.kz + 1 == 3 ? 0 : r.kz + 1;
    r.ky = r.kx + 1 == 3 ? 0 : r.kx + 1;
    float dz = sel3(d, r.kz);
    if (dz < 0.f) {
        int t = r.kx;
        r.kx = r.ky;
        r.ky = t;
    }
    r.sx = __fdiv_rn(sel3(d, r.kx), dz);
    r.sy = __fdiv_rn(sel3(d, r.ky), dz);
    r.sz = __frcp_rn(dz);
    return r;
}

// Watertight ray/triangle test with explicitly rounded operations.
PT_DI bool intersect_triangle(float3 o, const RayWT &w, float3 p0, float3 p1, float3 p2, float tmin, float tmax,
                              float &t_out, float &u_out, float &v_out) {
    float3 A = f3(__fsub_rn(p0.x, o.x), __fsub_rn(p0.y, o.y), __fsub_rn(p0.z, o.z));
    float3 B = f3(__fsub_rn(p1.x, o.x), __fsub_rn(p1.y, o.y), __fsub_rn(p1.z, o.z));
    float3 C = f3(__fsub_rn(p2.x, o.x), __fsub_rn(p2.y, o.y), __fsub_rn(p2.z, o.z));
    float Akz = sel3(A, w.kz), Bkz = sel3(B, w.kz), Ckz = sel3(C, w.kz);
    float Ax = __fsub_rn(sel3(A, w.kx), __fmul_rn(w.sx, Akz));
    float Ay = __fsub_rn(sel3(A, w.ky), __fmul_rn(w.sy, Akz));
    float Bx = __fsub_rn(sel3(B, w.kx), __fmul_rn(w.sx, Bkz));
    float By = __fsub_rn(sel3(B, w.ky), __fmul_rn(w.sy, Bkz));
    float Cx = __fsub_rn(sel3(C, w.kx), __fmul_rn(w.sx, Ckz));
    float Cy = __fsub_rn(sel3(C, w.ky), __fmul_rn(w.sy, Ckz));
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.f || V == 0.f || W == 0.f) {  // double-precision fallback on edges
        U = __double2float_rn(__dsub_rn(__dmul_rn((double)Cx, (double)By), __dmul_rn((double)Cy, (double)Bx)));
        V = __double2float_rn(__dsub_rn(__dmul_rn((double)Ax, (double)Cy), __dmul_rn((double)Ay, (double)Cx)));
        W = __double2float_rn(__dsub_rn(__dmul_rn((double)Bx, (double)Ay), __dmul_rn((double)By, (double)Ax)));
    }
    if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
    float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.f) return false;
    float Az = __fmul_rn(w.sz, Akz), Bz = __fmul_rn(w.sz, Bkz), Cz = __fmul_rn(w.sz, Ckz);
    float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
    float rcp = __frcp_rn(det);
    float t = __fmul_rn(T, rcp);
    if (!(t > tmin && t < tmax)) return false;
    t_out = t;
    u_out = __fmul_rn(V, rcp);
    v_out = __fmul_rn(W, rcp);
    return true;
}

// Ray/sphere with the two precision improvements of Haines, Guenther and
// Akenine-Moeller ("Precision Improvements for Ray/Sphere Intersection", Ray
// Tracing Gems, 2019): the discriminant from the distance of the closest
// approach to the centre, r^2 - |f + (b'/a) d|^2, instead of b^2 - ac (which
// cancels for distant or small spheres), and the two roots as c/q and q/a with
// q = b' + sign(b') sqrt(a * disc) (no subtraction of nearly equal values).
// The roots are then accurate to a few ulp of t, so a hit always lies inside
// the sphere's (padded) bounding box and the result cannot depend on which
// BVH nodes the traversal culls.  Every step is rounded separately, as in
// the oracle's host build of the same formula.
PT_DI bool intersect_sphere(float3 o, float3 d, float3 c, float r, float tmin, float tmax, float &t_out) {
    const float3 f = f3(__fsub_rn(o.x, c.x), __fsub_rn(o.y, c.y), __fsub_rn(o.z, c.z));
    const float a = __fadd_rn(__fadd_rn(__fmul_rn(d.x, d.x), __fmul_rn(d.y, d.y)), __fmul_rn(d.z, d.z));
    const float bp = -__fadd_rn(__fadd_rn(__fmul_rn(f.x, d.x), __fmul_rn(f.y, d.y)), __fmul_rn(f.z, d.z));
    const float s = __fdiv_rn(bp, a);
    const float3 l = f3(__fadd_rn(f.x, __fmul_rn(s, d.x)), __fadd_rn(f.y, __fmul_rn(s, d.y)),
                        __fadd_rn(f.z, __fmul_rn(s, d.z)));
    const float rr = __fmul_rn(r, r);
    const float disc = __fsub_rn(rr, __fadd_rn(__fadd_rn(__fmul_rn(l.x, l.x), __fmul_rn(l.y, l.y)), __fmul_rn(l.z, l.z)));
    if (!(disc >= 0.f)) return false;
    const float cc = __fsub_rn(__fadd_rn(__fadd_rn(__fmul_rn(f.x, f.x), __fmul_rn(f.y, f.y)), __fmul_rn(f.z, f.z)), rr);
    const float q = __fadd_rn(bp, copysignf(__fsqrt_rn(__fmul_rn(a, disc)), bp));
    float t0 = __fdiv_rn(cc, q), t1 = __fdiv_rn(q, a);
    if (t0 > t1) {
        const float tt = t0;
        t0 = t1;
        t1 = tt;
    }
    if (t0 > tmin && t0 < tmax) {
        t_out = t0;
        return true;
    }
    if (t1 > tmin && t1 < tmax) {
        t_out = t1;
        return true;
    }
    return false;
}

// ---------------------------------------------------------------- curve pieces
PT_DI float dot_rn(float3 a, float3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
PT_DI float3 sub_rn(float3 a, float3 b) { return f3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)); }
PT_DI float3 madd_rn(float3 a, float s, float3 b) {  // a + s*b, rounded per step
    return f3(__fadd_rn(a.x, __fmul_rn(s, b.x)), __fadd_rn(a.y, __fmul_rn(s, b.y)), __fadd_rn(a.z, __fmul_rn(s, b.z)));
}

// Entry into a sphere, the ray origin first moved to the point of closest
// approach (Haines et al., "Precision Improvements for Ray/Sphere
// Intersection", Ray Tracing Gems 2019), which keeps hair-thin spheres exact
// for distant origins.  Only the entering root counts.
PT_DI bool curve_sphere_entry(float3 o, float3 d, float dd, float3 c, float r, float tmin, float tmax, float &t_out) {
    const float3 f = sub_rn(o, c);
    const float tc = __fdiv_rn(-dot_rn(f, d), dd);
    const float3 l = madd_rn(f, tc, d);
    const float h = __fsub_rn(__fmul_rn(r, r), dot_rn(l, l));
    if (!(h >= 0.f)) return false;
    const float t = __fsub_rn(tc, __fsqrt_rn(__fdiv_rn(h, dd)));
    if (!(t > tmin && t < tmax)) return false;
    t_out = t;
    return true;
}

// Round-cone piece: the lateral surface of the cone frustum between the
// planes through c0 and c1 normal to the axis (radius linear along the
// axis), plus spheres at the ends that the kind bits ask for.  The frustum
// quadratic is formed from the components normal to the axis, origin moved to
// the closest approach to c0; its entering root is (-B - sqrt(B^2 - AC)) / A
// whatever the sign of A.  Returns the smallest entering t in (tmin, tmax)
// and the curve parameter there (projection onto the axis, mapped to [u0, u1]).
PT_DI bool intersect_curve_piece(float3 o, float3 d, float4 a, float4 b, float4 c, float tmin, float tmax, float &t_out,
                                 float &u_out) {
    const int kind = __float_as_int(b.w);
    const float3 c0 = xyz(a), c1 = xyz(c);
    const float r0 = b.x, r1 = b.y, u0 = b.z, u1 = c.w;
    const float dd = dot_rn(d, d);
    bool hit = false;
    float best = tmax, bu = 0.f, t;
    if ((kind & kPieceSphere0) && curve_sphere_entry(o, d, dd, c0, r0, tmin, best, t)) {
        hit = true;
        best = t;
        bu = u0;
    }
    if ((kind & kPieceSphere1) && curve_sphere_entry(o, d, dd, c1, r1, tmin, best, t)) {
        hit = true;
        best = t;
        bu = u1;
    }
    const float3 e = sub_rn(c1, c0);
    const float len = __fsqrt_rn(dot_rn(e, e));
    if (len > 0.f) {
        const float inv_len = __frcp_rn(len);
        const float3 ax = f3(__fmul_rn(e.x, inv_len), __fmul_rn(e.y, inv_len), __fmul_rn(e.z, inv_len));
        const float k = __fmul_rn(__fsub_rn(r1, r0), inv_len);  // dr / dz
        const float3 f = sub_rn(o, c0);
        const float tc = __fdiv_rn(-dot_rn(f, d), dd);
        const float3 w = madd_rn(f, tc, d);
        const float we = dot_rn(w, ax), de = dot_rn(d, ax);
        const float3 wp = madd_rn(w, -we, ax), dp = madd_rn(d, -de, ax);
        const float rz = __fadd_rn(r0, __fmul_rn(k, we));
        const float kde = __fmul_rn(k, de);
        const float A = __fsub_rn(dot_rn(dp, dp), __fmul_rn(kde, kde));
        const float B = __fsub_rn(dot_rn(wp, dp), __fmul_rn(kde, rz));
        const float C = __fsub_rn(dot_rn(wp, wp), __fmul_rn(rz, rz));
        const float disc = __fsub_rn(__fmul_rn(B, B), __fmul_rn(A, C));
        if (disc >= 0.f && A != 0.f) {
            const float tp = __fdiv_rn(__fsub_rn(-B, __fsqrt_rn(disc)), A);
            const float z = __fadd_rn(we, __fmul_rn(tp, de));
            const float tt = __fadd_rn(tc, tp);
            if (z >= 0.f && z <= len && tt > tmin && tt < best) {
                hit = true;
                best = tt;
                bu = __fadd_rn(u0, __fmul_rn(__fmul_rn(z, inv_len), __fsub_rn(u1, u0)));
            }
        }
    }
    if (!hit) return false;
    if (kind & kPieceClampU) bu = fminf(fmaxf(bu, kCurveUMin), kCurveUMax);
    t_out = best;
    u_out = bu;
    return true;
}

PT_DI float3 safe_inv(float3 d) {
    return f3(d.x != 0.f ? __frcp_rn(d.x) : copysignf(1e30f, d.x), d.y != 0.f ? __frcp_rn(d.y) : copysignf(1e30f, d.y),
              d.z != 0.f ? __frcp_rn(d.z) : copysignf(1e30f, d.z));
}

template <int K>
struct WideNode {
    float f[8 * K];
    PT_DI float lox(int c) const { return f[c]; }
    PT_DI float hix(int c) const { return f[K + c]; }
    PT_DI float loy(int c) const { return f[2 * K + c]; }
    PT_DI float hiy(int c) const { return f[3 * K + c]; }
    PT_DI float loz(int c) const { return f[4 * K + c]; }
    PT_DI float hiz(int c) const { return f[5 * K + c]; }
    PT_DI int child(int c) const { return __float_as_int(f[6 * K + c]); }
    PT_DI int count(int c) const { return __float_as_int(f[7 * K + c]); }
};

// BVH nodes and primitive records are read many times per wave while the ray
// state streams through once: node and primitive loads ask L1 to evict them
// last, the ray state's loads and stores ask for evict-first (ld/st .cs).
// Measured on the 1M-triangle scene: closest hit 1.1 % faster than plain
// loads; an additional L2 evict-last access policy on the BVH loads gave
// back half of that.
PT_DI float4 ld_bvh(const float4 *p) {
    float4 v;
    asm("ld.global.nc.L1::evict_last.v4.f32 {%0, %1, %2, %3}, [%4];"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
        : "l"(p));
    return v;
}
// 32 bytes per load (256-bit global loads, sm_100 and later): a node is
// 32 * K bytes at a 32-byte-aligned offset of a cudaMalloc'd array.
PT_DI void ld_bvh8(const float4 *p, float *f) {
    asm("ld.global.nc.L1::evict_last.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(f[0]), "=f"(f[1]), "=f"(f[2]), "=f"(f[3]), "=f"(f[4]), "=f"(f[5]), "=f"(f[6]), "=f"(f[7])
        : "l"(p));
}

template <typename T>
PT_DI T ld_stream(const T *p) {
    return __ldcs(p);
}
template <typename T>
PT_DI void st_stream(T *p, T v) {
    __stcs(p, v);
}

template <int K>
PT_DI void load_node(const float4 *__restrict__ p, WideNode<K> &n) {
#pragma unroll
    for (int i = 0; i < K; i++) ld_bvh8(p + 2 * i, n.f + 8 * i);
}
template <int K>
PT_DI void load_node_smem(const float4 *p, WideNode<K> &n) {
#pragma unroll
    for (int i = 0; i < 2 * K; i++) {
        float4 v = p[i];
        n.f[4 * i + 0] = v.x;
        n.f[4 * i + 1] = v.y;
        n.f[4 * i + 2] = v.z;
        n.f[4 * i + 3] = v.w;
    }
}

// Traversal items: a node index (>= 0), a leaf (bit 31 | first << 4 | count)
// or kNoItem.  Leaves must start below 2^27 - 1 (checked at scene upload).
constexpr int kNoItem = -1;
PT_DI int make_leaf(int first, int count) { return (int)(0x80000000u | ((uint32_t)first << 4) | (uint32_t)count); }
PT_DI bool is_leaf(int item) { return item < 0 && item != kNoItem; }
PT_DI int leaf_first(int item) { return (int)(((uint32_t)item >> 4) & 0x7ffffffu); }
PT_DI int leaf_count(int item) { return item & 15; }

// Compressed 8-wide nodes: 96 bytes (6 float4) per node, after the quantised
// wide nodes of Ylitie, Karras and Laine ("Efficient Incoherent Ray Traversal
// on GPUs Through Compressed Wide BVHs", HPG 2017), with 32-bit child items:
//   q0      xyz: grid origin p; w bits: biased exponents of the per-axis cell
//           sizes 2^e (bytes 0-2), mask of the occupied slots (byte 3)
//   q1..q3  axis x, y, z: low cells of slots 0-7 (8 bytes), high cells (8 bytes)
//   q4, q5  child items of slots 0-7 (inner node index, leaf item or kNoItem)
// Slot c's box is [fma(lo, 2^e, p), fma(hi, 2^e, p)] per axis; the builder
// picks the cells so that these bounds enclose the child's padded float box.
// Slot s holds the child that rays of direction octant s (bit 0: d.x < 0,
// bit 1: d.y < 0, bit 2: d.z < 0) should visit first, and a ray takes the hit
// children in the order slot ^ octant: no sorting of the children.
constexpr int kCwFloat4 = 6;

// Cell `c` (0-7) of the 8 bytes held by the words (w0, w1): the byte is
// placed in the mantissa of 2^23 with one byte permute, and 2^23 is taken
// off again (exact), which avoids the slower integer-to-float conversion.
PT_DI float cw_cell(uint32_t w0, uint32_t w1, int c) {
    const uint32_t v = __byte_perm(c & 4 ? w1 : w0, 0x4b000000u, 0x7650u | static_cast<uint32_t>(c & 3));
    return __fsub_rn(__uint_as_float(v), 8388608.f);
}
PT_DI int cw_pick(int4 i0, int4 i1, int c) {
    const int4 h = c & 4 ? i1 : i0;
    return c & 2 ? (c & 1 ? h.w : h.z) : (c & 1 ? h.y : h.x);
}

// Slab test of the 8 children of compressed node `p`, in visiting order:
// entry k is slot k ^ oct.  ci[k] = child item (kNoItem: missed or empty),
// ct[k] = entry distance.  fast: origin within the magnitude the boxes were
// padded for, so t = fma(cell, 2^e * inv, (p - o) * inv) is conservative
// (its error, at most about 2 ulp of |p - o|, stays inside the padding);
// otherwise each bound is formed as in the build and tested as a float box.
PT_DI void cw_children(const float4 *p, float3 o, float3 inv, bool fast, float tmin, float tlimit, int oct, int *ci,
                       float *ct) {
    float f[24];  // 96 bytes at a 32-byte-aligned offset: three 256-bit loads
    ld_bvh8(p, f);
    ld_bvh8(p + 2, f + 8);
    ld_bvh8(p + 4, f + 16);
    const float4 q0 = make_float4(f[0], f[1], f[2], f[3]), q1 = make_float4(f[4], f[5], f[6], f[7]),
                 q2 = make_float4(f[8], f[9], f[10], f[11]), q3 = make_float4(f[12], f[13], f[14], f[15]);
    const int4 i0 = make_int4(__float_as_int(f[16]), __float_as_int(f[17]), __float_as_int(f[18]), __float_as_int(f[19])),
               i1 = make_int4(__float_as_int(f[20]), __float_as_int(f[21]), __float_as_int(f[22]), __float_as_int(f[23]));
    const uint32_t meta = __float_as_uint(q0.w);
    const float sx = __uint_as_float((meta & 0xffu) << 23), sy = __uint_as_float(((meta >> 8) & 0xffu) << 23),
                sz = __uint_as_float(((meta >> 16) & 0xffu) << 23);
    const uint32_t occupied = meta >> 24;
    const float ax = __fmul_rn(sx, inv.x), ay = __fmul_rn(sy, inv.y), az = __fmul_rn(sz, inv.z);
    const float bx = __fmul_rn(__fsub_rn(q0.x, o.x), inv.x), by = __fmul_rn(__fsub_rn(q0.y, o.y), inv.y),
                bz = __fmul_rn(__fsub_rn(q0.z, o.z), inv.z);
    const uint32_t lx0 = __float_as_uint(q1.x), lx1 = __float_as_uint(q1.y), hx0 = __float_as_uint(q1.z),
                   hx1 = __float_as_uint(q1.w);
    const uint32_t ly0 = __float_as_uint(q2.x), ly1 = __float_as_uint(q2.y), hy0 = __float_as_uint(q2.z),
                   hy1 = __float_as_uint(q2.w);
    const uint32_t lz0 = __float_as_uint(q3.x), lz1 = __float_as_uint(q3.y), hz0 = __float_as_uint(q3.z),
                   hz1 = __float_as_uint(q3.w);
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int c = k ^ oct;
        ci[k] = kNoItem;
        ct[k] = __int_as_float(0x7f800000);
        if (!((occupied >> c) & 1u)) continue;
        const float clx = cw_cell(lx0, lx1, c), chx = cw_cell(hx0, hx1, c);
        const float cly = cw_cell(ly0, ly1, c), chy = cw_cell(hy0, hy1, c);
        const float clz = cw_cell(lz0, lz1, c), chz = cw_cell(hz0, hz1, c);
        float tx0, tx1, ty0, ty1, tz0, tz1;
        if (fast) {
            tx0 = __fmaf_rn(clx, ax, bx);
            tx1 = __fmaf_rn(chx, ax, bx);
            ty0 = __fmaf_rn(cly, ay, by);
            ty1 = __fmaf_rn(chy, ay, by);
            tz0 = __fmaf_rn(clz, az, bz);
            tz1 = __fmaf_rn(chz, az, bz);
        } else {
            tx0 = __fmul_rn(__fsub_rn(__fmaf_rn(clx, sx, q0.x), o.x), inv.x);
            tx1 = __fmul_rn(__fsub_rn(__fmaf_rn(chx, sx, q0.x), o.x), inv.x);
            ty0 = __fmul_rn(__fsub_rn(__fmaf_rn(cly, sy, q0.y), o.y), inv.y);
            ty1 = __fmul_rn(__fsub_rn(__fmaf_rn(chy, sy, q0.y), o.y), inv.y);
            tz0 = __fmul_rn(__fsub_rn(__fmaf_rn(clz, sz, q0.z), o.z), inv.z);
            tz1 = __fmul_rn(__fsub_rn(__fmaf_rn(chz, sz, q0.z), o.z), inv.z);
        }
        const float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tmin));
        float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
        tf = fminf(__fmul_rn(tf, kSlabScale), tlimit);
        if (!(tn <= tf)) continue;
        ci[k] = cw_pick(i0, i1, c);
        ct[k] = tn;
    }
}

// Per-thread traversal stack of (item, entry distance): kShortStack entries
// in shared memory (strided by the block size to avoid bank conflicts), the
// rest in local memory.
struct ShortStack {
    int2 *smem;  // base + threadIdx.x
    int stride;
    int2 spill[kSpillStack];
    int sp;
    PT_DI void push(int item, float t, uint32_t &overflow) {
        int2 e = make_int2(item, __float_as_int(t));
        if (sp < kShortStack) smem[sp * stride] = e;
        else if (sp < kShortStack + kSpillStack) spill[sp - kShortStack] = e;
        else {  // cannot happen for trees of depth <= 32 (width 4), 13 (width 8); reported, entry dropped
            overflow = 1;
            return;
        }
        sp++;
    }
    PT_DI int2 pop() {
        sp--;
        return sp < kShortStack ? smem[sp * stride] : spill[sp - kShortStack];
    }
};


// Lanes refill their ray when at most this many lanes of the warp are busy.
constexpr int kRefillBusyMax = 20;

// Persistent "while-while" traversal (after Aila & Laine, HPG 2009), adapted
// to wide nodes with inline leaves.  Each warp keeps 32 rays in flight:
//   refill   when at most kRefillBusyMax lanes are busy, the idle lanes take
//            new rays with one atomic per warp;
//   nodes    lanes step through inner nodes until every busy lane has found a
//            leaf (it is postponed) or run out of work;
//   leaves   lanes intersect their postponed leaf (and leaves that follow it
//            on the stack);
//   finish   lanes without work store their result and become idle.
// Children are slab-tested (robust far bound), sorted by entry distance; the
// nearest is the next item, the others go on the stack with their distance,
// which is re-checked against the current closest hit when popped.
//
// Src provides: count(), load(i, o, d, tmin, tmax, tag), root(tag) (the node
// the ray starts at), store(i, tag, result).
// CURVES = false compiles the leaf test without the curve-piece branch (a
// record with non-zero kind bits is then treated as a sphere), so that scenes
// without curves run the smaller kernel.
template <int K, bool ANY, bool COUNT, class Src, bool CURVES = false>
PT_DI void trace_persistent(const DevScene &s, const float4 *snodes, int2 *sstack_base, Src &src, uint32_t *work,
                            uint32_t *ovf_flag, unsigned long long *stat_nodes, unsigned long long *stat_prims,
                            unsigned long long *stat_rays) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const uint32_t n = src.count();
    ShortStack st;
    st.smem = sstack_base + threadIdx.x;
    st.stride = blockDim.x;
    st.sp = 0;
    bool active = false, exhausted = false;
    uint32_t idx = 0, tag = 0;
    float3 o = f3s(0.f), d = f3s(0.f), inv = f3s(0.f), oi = f3s(0.f);
    bool fma_slab = false;
    int oct = 0;  // direction octant (compressed 8-wide nodes)
    RayWT w{0, 1, 2, 0.f, 0.f, 1.f};
    float tmin = 0.f, tmax = 0.f;
    TraceResult best{0.f, -1, 0.f, 0.f};
    int item = kNoItem, leaf = kNoItem;
    uint32_t nodes = 0, prims = 0, rays = 0, ovf = 0;

    auto pop_valid = [&]() -> int {
        while (st.sp > 0) {
            int2 e = st.pop();
            if (__int_as_float(e.y) <= best.t * kSlabScale) return e.x;
        }
        return kNoItem;
    };

    for (;;) {
        unsigned busy = __ballot_sync(FULL, active);
        if (!exhausted && __popc(busy) <= kRefillBusyMax) {
            unsigned idle = ~busy;
            uint32_t cnt = __popc(idle);
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(work, cnt);
            base = __shfl_sync(FULL, base, 0);
            if (!active) {
                uint32_t r = base + __popc(idle & lt);
                if (r < n) {
                    idx = r;
                    src.load(r, o, d, tmin, tmax, tag);
                    w = ray_wt(d);
                    inv = safe_inv(d);
                    oi = f3(o.x * inv.x, o.y * inv.y, o.z * inv.z);
                    // the FMA slab form is conservative for origins inside the
                    // magnitude the boxes were padded for
                    fma_slab = fmaxf(fmaxf(fabsf(o.x), fabsf(o.y)), fabsf(o.z)) <= s.pad_mag;
                    oct = (d.x < 0.f ? 1 : 0) | (d.y < 0.f ? 2 : 0) | (d.z < 0.f ? 4 : 0);
                    best.t = tmax;
                    best.prim = -1;
                    best.u = best.v = 0.f;
                    item = src.root(tag);
                    leaf = kNoItem;
                    st.sp = 0;
                    active = true;
                    if (COUNT) rays++;
                }
            }
            if (base + cnt >= n) exhausted = true;
            busy = __ballot_sync(FULL, active);
        }
        if (busy == 0) break;

        // Inner nodes.  A lane keeps stepping while its current item is an
        // inner node, even after it has postponed a leaf (speculative
        // traversal); the phase ends when every busy lane holds a leaf or
        // no lane can step.
        for (;;) {
            bool can_step = active && item >= 0;
            bool satisfied = !active || leaf != kNoItem || item == kNoItem;
            if (__all_sync(FULL, satisfied)) break;
            if (!__any_sync(FULL, can_step)) break;
            if (!can_step) continue;
            if constexpr (K == 8) {  // compressed node: children come in the octant's visiting order
                if (COUNT) nodes++;
                int ci[8];
                float ct[8];
                cw_children(s.cnodes + (size_t)item * kCwFloat4, o, inv, fma_slab, tmin, best.t * kSlabScale, oct, ci,
                            ct);
                // the first hit child is descended, the later ones pushed (popped in visiting order)
                int next = kNoItem;
                float next_t = 0.f;
#pragma unroll
                for (int i = 7; i >= 0; i--) {
                    if (ci[i] == kNoItem) continue;
                    if (next != kNoItem) st.push(next, next_t, ovf);
                    next = ci[i];
                    next_t = ct[i];
                }
                item = next != kNoItem ? next : pop_valid();
            } else {
                WideNode<K> nd;
                if (item < static_cast<int>(s.smem_nodes)) load_node_smem<K>(snodes + (size_t)item * 2 * K, nd);
                else load_node<K>(s.nodes + (size_t)item * 2 * K, nd);
                if (COUNT) nodes++;
                int ci[K];
                float ct[K];
                const float tlimit = best.t * kSlabScale;
#pragma unroll
                for (int c = 0; c < K; c++) {
                    ci[c] = kNoItem;
                    ct[c] = __int_as_float(0x7f800000);
                    int ch = nd.child(c);
                    if (ch < 0) continue;
                    float tx0, tx1, ty0, ty1, tz0, tz1;
                    if (fma_slab) {  // t = lo * inv - o * inv: one rounding, conservative within pad_mag
                        tx0 = __fmaf_rn(nd.lox(c), inv.x, -oi.x);
                        tx1 = __fmaf_rn(nd.hix(c), inv.x, -oi.x);
                        ty0 = __fmaf_rn(nd.loy(c), inv.y, -oi.y);
                        ty1 = __fmaf_rn(nd.hiy(c), inv.y, -oi.y);
                        tz0 = __fmaf_rn(nd.loz(c), inv.z, -oi.z);
                        tz1 = __fmaf_rn(nd.hiz(c), inv.z, -oi.z);
                    } else {
                        tx0 = (nd.lox(c) - o.x) * inv.x;
                        tx1 = (nd.hix(c) - o.x) * inv.x;
                        ty0 = (nd.loy(c) - o.y) * inv.y;
                        ty1 = (nd.hiy(c) - o.y) * inv.y;
                        tz0 = (nd.loz(c) - o.z) * inv.z;
                        tz1 = (nd.hiz(c) - o.z) * inv.z;
                    }
                    float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tmin));
                    float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
                    tf = fminf(tf * kSlabScale, tlimit);
                    if (!(tn <= tf)) continue;
                    int cnt = nd.count(c);
                    ci[c] = cnt > 0 ? make_leaf(ch, cnt) : ch;
                    ct[c] = tn;
                }
                // closest hit: nearest child first (sorting network); any hit: order
                // does not matter, the children are taken as they come
#pragma unroll
                for (int i = 1; i < (ANY ? 1 : K); i++) {
#pragma unroll
                    for (int j = i; j > 0; j--) {
                        if (ct[j] < ct[j - 1]) {
                            float tt = ct[j];
                            ct[j] = ct[j - 1];
                            ct[j - 1] = tt;
                            int ti = ci[j];
                            ci[j] = ci[j - 1];
                            ci[j - 1] = ti;
                        }
                    }
                }
                if (ANY) {  // unsorted: the first hit child is descended, the others pushed
#pragma unroll
                    for (int i = 1; i < K; i++)
                        if (ci[0] == kNoItem && ci[i] != kNoItem) {
                            ci[0] = ci[i];
                            ci[i] = kNoItem;
                        }
                }
#pragma unroll
                for (int i = K - 1; i >= 1; i--)
                    if (ci[i] != kNoItem) st.push(ci[i], ct[i], ovf);
                item = ci[0] != kNoItem ? ci[0] : pop_valid();
            }
            if (is_leaf(item) && leaf == kNoItem) {  // postpone the first leaf
                leaf = item;
                item = pop_valid();
            }
        }

        // leaves
        if (active) {
            while (leaf != kNoItem) {
                const int first = leaf_first(leaf), cnt = leaf_count(leaf);
                for (int j = 0; j < cnt; j++) {
                    const float4 *pr = s.prims + (size_t)(first + j) * 3;
                    float4 a = ld_bvh(pr);
                    float4 b = ld_bvh(pr + 1);
                    if (COUNT) prims++;
                    int pid = __float_as_int(a.w);
                    float t, u = 0.f, v = 0.f;
                    float tlim = best.prim < 0 ? tmax : __int_as_float(__float_as_int(best.t) + 1);
                    bool hit;
                    if (pid >= 0) {
                        float4 cc = ld_bvh(pr + 2);
                        hit = intersect_triangle(o, w, xyz(a), xyz(b), xyz(cc), tmin, tlim, t, u, v);
                    } else if (!CURVES || __float_as_int(b.w) == 0) {
                        pid &= 0x7fffffff;
                        hit = intersect_sphere(o, d, xyz(a), b.x, tmin, tlim, t);
                    } else {
                        pid &= 0x7fffffff;
                        float4 cc = ld_bvh(pr + 2);
                        hit = intersect_curve_piece(o, d, a, b, cc, tmin, tlim, t, u);
                    }
                    if (!hit) continue;
                    if (ANY) {
                        best.t = t;
                        best.prim = pid;
                        break;
                    }
                    if (t < best.t || pid < best.prim) {
                        best.t = t;
                        best.prim = pid;
                        best.u = u;
                        best.v = v;
                    }
                }
                leaf = kNoItem;
                if (ANY && best.prim >= 0) {  // any hit ends the ray
                    item = kNoItem;
                    st.sp = 0;
                    break;
                }
                if (is_leaf(item)) {
                    leaf = item;
                    item = pop_valid();
                }
            }
            if (item == kNoItem && leaf == kNoItem) {
                src.store(idx, tag, best);
                active = false;
            }
        }
    }
    if (ovf) atomicOr(ovf_flag, 1u);
    if (COUNT) {
        for (int off = 16; off > 0; off >>= 1) {
            nodes += __shfl_xor_sync(FULL, nodes, off);
            prims += __shfl_xor_sync(FULL, prims, off);
            rays += __shfl_xor_sync(FULL, rays, off);
        }
        if (lane == 0) {
            atomicAdd(stat_nodes, (unsigned long long)nodes);
            atomicAdd(stat_prims, (unsigned long long)prims);
            atomicAdd(stat_rays, (unsigned long long)rays);
        }
    }
}

}  // namespace ptd
