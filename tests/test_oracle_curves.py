"""Curve (hair) primitives on the CPU: the oracle's round-cone intersection
scheme checked against geometry computed independently here in numpy
(float64 power-basis evaluation of the four curve types), and the
oracle's BVH against its brute force.  The GPU kernels are pinned to this
oracle bit for bit in tests/test_gpu_curves.py; the interpolators and the
surface normal are pinned to the reference's own curve.h through the golden
vectors (test_oracle_golden.py)."""
import numpy as np
import pytest

import oracle
from pupiloptixlab_gb300 import abi, scenes

# Basis matrices (rows: power u^3.., columns: control points), the standard
# uniform B-spline and Catmull-Rom forms.
_BASIS = {
    abi.CURVE_LINEAR: np.array([[-1, 1], [1, 0]], np.float64),
    abi.CURVE_QUADRATIC_BSPLINE: np.array([[1, -2, 1], [-2, 2, 0], [1, 1, 0]], np.float64) / 2,
    abi.CURVE_CUBIC_BSPLINE: np.array([[-1, 3, -3, 1], [3, -6, 3, 0], [-3, 0, 3, 0], [1, 4, 1, 0]], np.float64) / 6,
    abi.CURVE_CATMULL_ROM: np.array([[-1, 3, -3, 1], [2, -5, 4, -1], [-1, 0, 1, 0], [0, 2, 0, 0]], np.float64) / 2,
}


def curve_eval(ctype, q, u):
    """Centre xyz + radius and the derivative at u for control points q (deg+1, 4)."""
    m = _BASIS[ctype]
    deg = m.shape[0] - 1
    coef = m @ q  # highest power first
    pw = np.array([u ** (deg - i) for i in range(deg + 1)])
    dpw = np.array([(deg - i) * u ** (deg - i - 1) if deg - i > 0 else 0.0 for i in range(deg + 1)])
    return pw @ coef, dpw @ coef


def single_strand_scene(ctype, pts, radius, to_world=None):
    s = scenes.Scene(32, 32, 4, name="strand")
    cv = scenes.Curves.from_strands([pts], [radius], ctype)
    s.add_instance(abi.SHAPE_CURVES, s.add_curves(cv), s.add_material(scenes.diffuse(0.5)), to_world)
    s.camera = scenes.camera(40.0, 1.0, scenes.look_at_to_world((0, 0, 5), (0, 0, 0)))
    return s, cv


def make_rays(o, d, tmin=1e-3, tmax=1e16):
    r = np.zeros((o.shape[0], 8), np.float32)
    r[:, 0:3], r[:, 3], r[:, 4:7], r[:, 7] = o, tmin, d, tmax
    return r


def test_linear_segment_analytic():
    """One straight linear segment of radius 0.1 along x: rays straight down
    hit the cylinder at t = 2 - sqrt(r^2 - z^2) with u = (x + 1) / 2, and the
    round caps beyond the ends report u = 0 and u = 1."""
    pts = np.array([[-1, 0, 0], [1, 0, 0]], np.float32)
    sc, _ = single_strand_scene(abi.CURVE_LINEAR, pts, 0.1)
    o = oracle.OracleScene(sc)
    rng = np.random.default_rng(1)
    n = 2000
    x = rng.uniform(-0.95, 0.95, n)
    z = rng.uniform(-0.099, 0.099, n)
    org = np.stack([x, np.full(n, 2.0), z], 1)
    d = np.tile([0.0, -1.0, 0.0], (n, 1))
    h = o.trace(make_rays(org, d), brute_force=True)
    assert (h[:, 1].view(np.int32) == 0).all()
    assert np.allclose(h[:, 0], 2.0 - np.sqrt(0.01 - z ** 2), atol=2e-6)
    assert np.allclose(h[:, 2], (x + 1) / 2, atol=2e-6)
    # caps: beyond the ends, inside the sphere's silhouette
    xc = np.array([-1.05, 1.05, -1.09, 1.09])
    h = o.trace(make_rays(np.stack([xc, np.full(4, 2.0), np.zeros(4)], 1), np.tile([0.0, -1.0, 0.0], (4, 1))),
                brute_force=True)
    assert (h[:, 1].view(np.int32) == 0).all()
    assert list(h[:, 2]) == [0.0, 1.0, 0.0, 1.0]
    assert np.allclose(h[:, 0], 2.0 - np.sqrt(0.01 - (np.abs(xc) - 1.0) ** 2), atol=2e-6)
    # a ray starting inside the tube reports nothing (entering hits only)
    h = o.trace(make_rays(np.array([[0.0, 0.0, 0.0]]), np.array([[0.0, 1.0, 0.0]])), brute_force=True)
    assert h[0, 1].view(np.int32) == -1


@pytest.mark.parametrize("ctype", [0, 1, 2, 3])
def test_hits_lie_on_the_swept_surface_and_leave_no_cracks(ctype):
    """Rays aimed at the centre line of a bent strand, normal to its tangent,
    from one unit away: every ray hits the strand (no cracks between pieces or
    segments; the spline types' open ends are cut normal to the end piece's
    axis, so the outer 2 % there are left out), the hit point lies at the
    radius from the centre point of the reported u (within the 5 % chord
    tolerance of the piece split), and the distance is 1 - r to the same
    tolerance."""
    rng = np.random.default_rng(ctype)
    t = np.linspace(0, 1, 9)
    pts = np.stack([np.cos(3 * t) * 1.5, np.sin(2 * t) * 0.8, t * 2 - 1], 1).astype(np.float32)
    r = 0.05
    sc, cv = single_strand_scene(ctype, pts, r)
    o = oracle.OracleScene(sc)
    pieces = o.curve_pieces()
    deg = 3 if ctype > 2 else ctype + 1
    q_all = np.concatenate([cv.positions, cv.radii[:, None]], 1).astype(np.float64)
    n = 3000
    seg = rng.integers(0, cv.segments.shape[0], n)
    u = rng.uniform(0.0, 1.0, n)
    if ctype != abi.CURVE_LINEAR:
        # the open strand ends are cut normal to the first / last piece's
        # axis, not to the tangent: keep 2 % away from them
        last = cv.segments.shape[0] - 1
        u = np.where(seg == 0, np.maximum(u, 0.02), u)
        u = np.where(seg == last, np.minimum(u, 0.98), u)
    cen, tan = np.zeros((n, 3)), np.zeros((n, 3))
    for i in range(n):
        q = q_all[cv.segments[seg[i]]:cv.segments[seg[i]] + deg + 1]
        p, dp = curve_eval(ctype, q, u[i])
        cen[i], tan[i] = p[:3], dp[:3]
    side = rng.normal(size=(n, 3))
    side -= (np.sum(side * tan, 1) / np.sum(tan * tan, 1))[:, None] * tan
    side /= np.linalg.norm(side, axis=1, keepdims=True)
    h = o.trace(make_rays(cen + side, -side), brute_force=True)
    pid = h[:, 1].view(np.int32)
    assert (pid >= 0).all(), f"{(pid < 0).sum()} rays slipped through the strand"
    assert np.allclose(h[:, 0], 1.0 - r, atol=0.06 * r)
    # the reported u: hit point at radius r from the centre point at u
    hit_seg = pieces[pid, 11].astype(np.int64)
    x = cen + side * (1.0 - h[:, 0:1])
    for i in range(n):
        q = q_all[cv.segments[hit_seg[i]]:cv.segments[hit_seg[i]] + deg + 1]
        p, _ = curve_eval(ctype, q, float(h[i, 2]))
        assert abs(np.linalg.norm(x[i] - p[:3]) - r) <= 0.06 * r, (i, np.linalg.norm(x[i] - p[:3]))
    if ctype != abi.CURVE_LINEAR:
        assert (h[:, 2] > 0).all() and (h[:, 2] < 1).all()


@pytest.mark.parametrize("ctype", [0, 1, 2, 3])
def test_hair_bvh_equals_brute_force_and_any_hit(ctype):
    sc = scenes.hair_scene(48, 32, curve_type=ctype, num_strands=200, tapered=ctype == 2)
    o = oracle.OracleScene(sc)
    rng = np.random.default_rng(9)
    n = 6000
    org = rng.uniform(-2, 2, (n, 3)) + [0, 1.5, 0]
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([o.camera_rays(abi.RNG_PCG32, 0), make_rays(org, d)])
    a = o.trace(rays, brute_force=True)
    b = o.trace(rays)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    nt, ns = o.num_prims()
    assert (a[:, 1].view(np.int32) >= nt + ns).sum() > 150
    rays[:, 7] = rng.uniform(0.05, 3.0, rays.shape[0])
    anyh = o.trace(rays, anyhit=True, brute_force=True)
    closest = o.trace(rays, brute_force=True)
    assert np.array_equal(anyh[:, 0] > 0, closest[:, 1].view(np.int32) >= 0)  # any hit: column 0 = occluded


def test_pieces_follow_the_segment_rules():
    """Linear segments: one piece, a sphere at every vertex (the strand's last
    vertex too); spline segments: pieces span [0, 1], joint spheres everywhere
    except the strand's open ends, u clamped inside (0, 1)."""
    pts = [np.cumsum(np.random.default_rng(k).normal(size=(7, 3)) * 0.3, 0) for k in range(3)]
    for ctype in range(4):
        s = scenes.Scene(8, 8, 2)
        cv = scenes.Curves.from_strands(pts, [0.02] * 3, ctype)
        s.add_instance(abi.SHAPE_CURVES, s.add_curves(cv), s.add_material(scenes.diffuse(0.5)))
        o = oracle.OracleScene(s)
        p = o.curve_pieces()
        nseg, npc = o.num_curves()
        assert nseg == cv.segments.shape[0] == 3 * (7 - (3 if ctype > 2 else ctype + 1))
        kind = p[:, 10].astype(int)
        segs = p[:, 11].astype(int)
        for k in range(nseg):
            pk = p[segs == k]
            assert pk[0, 8] == 0.0 and pk[-1, 9] == 1.0 and np.all(pk[1:, 8] == pk[:-1, 9])
        if ctype == abi.CURVE_LINEAR:
            assert npc == nseg and np.all(kind & 2)
            assert ((kind & 4) != 0).sum() == 3  # one end sphere per strand
        else:
            assert np.all(kind & 8)
            assert ((kind & 2) == 0).sum() == 3  # the strands' first pieces are open
            assert not np.any(kind & 4)
