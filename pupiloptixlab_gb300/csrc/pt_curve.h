// pt_curve.h -- round curve segments (hair strands), host and device.
//
// A segment of degree n (1 linear, 2 quadratic B-spline, 3 cubic B-spline or
// Catmull-Rom) is held in the power basis, xyz = centre line, w = radius:
//   linear     P(u) = c0 + u c1
//   quadratic  P(u) = (c0 u + c1) u + c2
//   cubic      P(u) = ((c0 u + c1) u + c2) u + c3
// converted from the control points with the standard basis matrices and
// evaluated by Horner's rule, in the operation order of the reference's
// interpolators (framework/render/curve.h:35-238) so that results agree bit
// for bit when FMA contraction is off.  curve_normal() is the hit-point
// normal of the reference's SurfaceNormal (curve.h:240-342) as
// Geometry::GetHitLocalGeometry applies it per curve type
// (framework/render/geometry.h:101-172): flat-end-cap normals at u = 0 / 1 for
// the spline types, round caps for linear segments, otherwise the normal of
// the swept circle through the hit point projected onto the plane normal to
// the curve.
//
// Intersection is not the reference's (OptiX's built-in curve intersector is
// closed): each segment is split into round-cone pieces (curve_piece_count)
// that the traversal intersects exactly; see pt_traverse.cuh.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

#include "pt_device.cuh"

namespace ptd {

enum : uint32_t { kCurveLinear = 0, kCurveQuadratic = 1, kCurveCubic = 2, kCurveCatmullRom = 3 };
constexpr uint32_t kCurveMaxPieces = 16;       // round-cone pieces per segment
constexpr float kCurvePieceTol = 0.05f;        // chord deviation bound, fraction of the largest radius
constexpr float kCurveUMin = 9.5367431640625e-07f;  // 2^-20: spline hits never report u = 0 or 1
constexpr float kCurveUMax = 0.99999904632568359375f;  // 1 - 2^-20

// Kind bits of a curve-piece primitive record (a sphere record has kind 0):
// a piece is a round cone; Sphere0 / Sphere1 close it with a sphere at its
// start / end; ClampU keeps the reported parameter inside (0, 1).
enum : int { kPieceCurve = 1, kPieceSphere0 = 2, kPieceSphere1 = 4, kPieceClampU = 8 };

// shape.cpp:383: control points per segment minus one.
PT_HDI uint32_t curve_degree(uint32_t type) { return type > 2 ? 3u : type + 1u; }

PT_HDI float4 c4add(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
PT_HDI float4 c4sub(float4 a, float4 b) { return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
PT_HDI float4 c4mul(float4 a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }
// float4 / s as the reference's vector helpers form it: times 1/s.
PT_HDI float4 c4div(float4 a, float s) { return c4mul(a, 1.0f / s); }

struct CurveSeg {
    float4 c[4];      // power-basis coefficients, highest power first
    uint32_t degree;  // 1, 2 or 3
};

// Control points q[0..degree] (xyz centre, w radius) -> power basis.
PT_HDI CurveSeg curve_segment(uint32_t type, const float4 *q) {
    CurveSeg s;
    s.c[0] = s.c[1] = s.c[2] = s.c[3] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (type == kCurveLinear) {
        s.degree = 1;
        s.c[0] = q[0];
        s.c[1] = c4sub(q[1], q[0]);
    } else if (type == kCurveQuadratic) {
        // B-spline basis [[1,-2,1],[-2,2,0],[1,1,0]] / 2
        s.degree = 2;
        s.c[0] = c4div(c4add(c4sub(q[0], c4mul(q[1], 2.0f)), q[2]), 2.0f);
        s.c[1] = c4div(c4add(c4mul(q[0], -2.0f), c4mul(q[1], 2.0f)), 2.0f);
        s.c[2] = c4div(c4add(q[0], q[1]), 2.0f);
    } else if (type == kCurveCubic) {
        // B-spline basis [[-1,3,-3,1],[3,-6,3,0],[-3,0,3,0],[1,4,1,0]] / 6
        s.degree = 3;
        s.c[0] = c4div(c4add(c4add(c4add(c4mul(q[0], -1.0f), c4mul(q[1], 3.0f)), c4mul(q[2], -3.0f)), q[3]), 6.0f);
        s.c[1] = c4div(c4add(c4add(c4mul(q[0], 3.0f), c4mul(q[1], -6.0f)), c4mul(q[2], 3.0f)), 6.0f);
        s.c[2] = c4div(c4add(c4mul(q[0], -3.0f), c4mul(q[2], 3.0f)), 6.0f);
        s.c[3] = c4div(c4add(c4add(c4mul(q[0], 1.0f), c4mul(q[1], 4.0f)), c4mul(q[2], 1.0f)), 6.0f);
    } else {
        // Catmull-Rom basis [[-1,3,-3,1],[2,-5,4,-1],[-1,0,1,0],[0,2,0,0]] / 2
        s.degree = 3;
        s.c[0] = c4div(c4add(c4add(c4add(c4mul(q[0], -1.0f), c4mul(q[1], 3.0f)), c4mul(q[2], -3.0f)), c4mul(q[3], 1.0f)), 2.0f);
        s.c[1] = c4div(c4add(c4add(c4add(c4mul(q[0], 2.0f), c4mul(q[1], -5.0f)), c4mul(q[2], 4.0f)), c4mul(q[3], -1.0f)), 2.0f);
        s.c[2] = c4div(c4add(c4mul(q[0], -1.0f), c4mul(q[2], 1.0f)), 2.0f);
        s.c[3] = c4div(c4mul(q[1], 2.0f), 2.0f);
    }
    return s;
}

PT_HDI float4 curve_pos(const CurveSeg &s, float u) {
    if (s.degree == 1) return c4add(s.c[0], c4mul(s.c[1], u));
    if (s.degree == 2) return c4add(c4mul(c4add(c4mul(s.c[0], u), s.c[1]), u), s.c[2]);
    return c4add(c4mul(c4add(c4mul(c4add(c4mul(s.c[0], u), s.c[1]), u), s.c[2]), u), s.c[3]);
}

PT_HDI float4 curve_vel(const CurveSeg &s, float u) {
    if (s.degree == 1) return s.c[1];
    if (s.degree == 2) return c4add(c4mul(c4mul(s.c[0], 2.0f), u), s.c[1]);
    // the cubic derivative is taken just inside the ends (triple knots)
    if (u == 0.f) u = 0.000001f;
    if (u == 1.f) u = 0.999999f;
    return c4add(c4mul(c4add(c4mul(c4mul(s.c[0], 3.0f), u), c4mul(s.c[1], 2.0f)), u), s.c[2]);
}

PT_HDI float3 curve_acc(const CurveSeg &s, float u) {
    if (s.degree == 1) return f3s(0.f);
    if (s.degree == 2) return xyz(c4mul(s.c[0], 2.0f));
    return xyz(c4add(c4mul(c4mul(s.c[0], 6.0f), u), c4mul(s.c[1], 2.0f)));
}

// Surface normal at a hit point ps near the tube (world space here; the
// reference works in object space, identical for similarity transforms).
PT_HDI float3 curve_normal(const CurveSeg &s, float u, float3 ps) {
    float3 n;
    if (s.degree == 1) {
        if (u == 0.f) {
            n = ps - xyz(s.c[0]);  // round cap
        } else if (u >= 1.f) {
            n = ps - (xyz(s.c[1]) + xyz(s.c[0]));
        } else {
            const float4 p4 = curve_pos(s, u), d4 = curve_vel(s, u);
            const float3 p = xyz(p4), d = xyz(d4);
            const float r = p4.w, dr = d4.w, dd = dot(d, d);
            float3 o1 = ps - p;
            o1 = o1 - (dot(o1, d) / dd) * d;  // onto the plane through p normal to d
            o1 = o1 * (r / length(o1));       // and out to the radius
            n = dd * o1 - (dr * r) * d;       // tilt of a cone (no curvature term)
        }
    } else {
        if (u == 0.f) {
            n = -xyz(curve_vel(s, 0.f));  // flat cap
        } else if (u == 1.f) {
            n = xyz(curve_vel(s, 1.f));
        } else {
            const float4 p4 = curve_pos(s, u), d4 = curve_vel(s, u);
            const float3 p = xyz(p4), d = xyz(d4);
            const float r = p4.w, dr = d4.w;
            float dd = dot(d, d);
            float3 o1 = ps - p;
            o1 = o1 - (dot(o1, d) / dd) * d;
            o1 = o1 * (r / length(o1));
            dd = dd - dot(curve_acc(s, u), o1);  // curvature of the centre line
            n = dd * o1 - (dr * r) * d;
        }
    }
    return normalize(n);
}

// Number of round-cone pieces for a segment: a polynomial piece of parameter
// length h deviates from its chord by at most h^2/8 * max|P''|, which must stay
// below kCurvePieceTol times the largest control radius.  For the spline
// types |P''| is linear in u, so its maximum is at an end.
PT_HDI uint32_t curve_piece_count(const CurveSeg &s, float max_radius) {
    if (s.degree == 1) return 1u;
    float3 a0, a1;
    if (s.degree == 2) {
        a0 = a1 = xyz(c4mul(s.c[0], 2.0f));
    } else {
        a0 = xyz(c4mul(s.c[1], 2.0f));
        a1 = xyz(c4add(c4mul(s.c[0], 6.0f), c4mul(s.c[1], 2.0f)));
    }
    const float acc = fmaxf(length(a0), length(a1));
    const float tol = kCurvePieceTol * max_radius;
    if (!(tol > 0.f) || !(acc > 0.f)) return 1u;
    const float q = sqrtf(acc / (8.0f * tol));
    if (!(q < (float)kCurveMaxPieces)) return kCurveMaxPieces;
    const uint32_t n = (uint32_t)ceilf(q);
    return n < 1u ? 1u : n;
}

}  // namespace ptd
