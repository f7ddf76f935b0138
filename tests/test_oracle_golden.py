"""The CPU oracle against golden vectors produced by the reference's own
render-layer headers compiled for the host (tests/golden/make_golden.py).
The oracle restates that code with the same operation order and no FMA
contraction, so every value must match bit for bit (NaN == NaN)."""
import ctypes as C

import numpy as np
import pytest

import oracle


def P(a):
    return a.ctypes.data_as(C.c_void_p)


def same_bits(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    if a.dtype.kind == "f":
        return np.array_equal(a, b, equal_nan=True)
    return np.array_equal(a, b)


def test_bsdf_eval_matches_reference(golden):
    f, pdf = oracle.bsdf_eval(golden["eval_bsdf"], golden["eval_wo"], golden["eval_wi"])
    for k in range(1, 8):
        m = golden["eval_bsdf"][:, 0] == k
        assert same_bits(f[m], golden["eval_f"][m]), f"material {k}: f"
        assert same_bits(pdf[m], golden["eval_pdf"][m]), f"material {k}: pdf"


def test_bsdf_sample_matches_reference(golden):
    wi, f, pdf, typ, rng = oracle.bsdf_sample(golden["sample_bsdf"], golden["sample_wo"], golden["sample_seed"])
    for k in range(1, 8):
        m = golden["sample_bsdf"][:, 0] == k
        assert same_bits(wi[m], golden["sample_wi"][m]), f"material {k}: wi"
        assert same_bits(f[m], golden["sample_f"][m]), f"material {k}: f"
        assert same_bits(pdf[m], golden["sample_pdf"][m]), f"material {k}: pdf"
        assert same_bits(typ[m], golden["sample_type"][m]), f"material {k}: lobe"
        assert same_bits(rng[m], golden["sample_seed_out"][m]), f"material {k}: random numbers drawn"


def test_every_material_and_lobe_is_covered(golden):
    types = set(int(t) for t in golden["sample_bsdf"][:, 0])
    assert types == set(range(1, 8))
    lobes = set(int(t) for t in golden["sample_type"])
    # diffuse, glossy reflection/transmission, delta reflection/transmission and the early-return "unknown"
    assert {0, 2, 8, 16, 32, 64} <= lobes


def test_reference_random_stream(golden):
    for i, (p, s) in enumerate(zip(golden["rng_pixel"], golden["rng_seed"])):
        assert same_bits(oracle.rng_stream(0, int(p), int(s), 64), golden["rng_stream"][i])


@pytest.mark.parametrize("name,ins,outs,width", [
    ("oracle_fresnel_dielectric", "fresnel_in", "fresnel_out", 2),
    ("oracle_fresnel_conductor", "conductor_in", "conductor_out", 1),
    ("oracle_fresnel_diffuse", "fdr_in", "fdr_out", 1),
    ("oracle_ggx", "ggx_in", "ggx_out", 7),
    ("oracle_sampling", "sampling_in", "sampling_out", 20),
])
def test_math_kats(golden, name, ins, outs, width):
    lib = oracle.load()
    x = np.ascontiguousarray(golden[ins])
    n = x.shape[0]
    out = np.zeros((n, width), np.float32).squeeze() if width == 1 else np.zeros((n, width), np.float32)
    getattr(lib, name)(P(x), P(out), n)
    assert same_bits(out, golden[outs])


@pytest.mark.parametrize("kind,key", [(1, "emit_tri"), (2, "emit_sphere"), (3, "emit_env")])
def test_emitter_sample_direct(golden, kind, key):
    lib = oracle.load()
    x = np.ascontiguousarray(golden["emit_in"])
    out = np.zeros((x.shape[0], 12), np.float32)
    params = np.ascontiguousarray(golden[key])
    assert lib.oracle_emitter_sample_raw(kind, P(params), P(x), P(out), x.shape[0]) == 0
    ref = golden[key + "_out"]
    valid = ref[:, 11] > 0
    # distance and pdf only exist where the sample is usable; positions and
    # directions are always written
    assert same_bits(out[:, 11], ref[:, 11])
    assert same_bits(out[:, :7], ref[:, :7])
    assert same_bits(out[valid, 7], ref[valid, 7])
    if kind != 3:
        assert same_bits(out[:, 8:11], ref[:, 8:11])


def test_select_emitter(golden):
    lib = oracle.load()
    probs = np.ascontiguousarray(golden["select_probs"])
    p = np.ascontiguousarray(golden["select_p"])
    for has_env, key in ((1, "select_env"), (0, "select_noenv")):
        out = np.zeros(p.shape[0], np.int32)
        lib.oracle_select_emitter(P(probs), probs.shape[0], has_env, P(p), P(out), p.shape[0])
        assert np.array_equal(out, golden[key])


def test_golden_vectors_regenerate_identically(golden):
    """Where the reference tree is available, the committed vectors are what
    the reference's code produces today."""
    ref = oracle.load_ref()
    if ref is None:
        pytest.skip("reference tree not present: committed golden vectors are used as is")
    n = golden["eval_bsdf"].shape[0]
    f = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    ref.ref_bsdf_eval(P(golden["eval_bsdf"]), P(golden["eval_wo"]), P(golden["eval_wi"]), P(f), P(pdf), n)
    assert same_bits(f, golden["eval_f"]) and same_bits(pdf, golden["eval_pdf"])


def test_envmap_matches_reference(golden):
    """EnvMapEmitter::SampleDirect / Eval (render/emitter/env.h) of the
    reference, compiled for the host over the oracle's CDF tables, against the
    oracle's restatement (tables built from the same map).  The search
    indices agree exactly (same direction); radiance, direction and pdf to
    float rounding (the reference calls sin/cos in double)."""
    px = golden["envmap_pixels"]
    tw, tl = golden["envmap_tw"], golden["envmap_tl"]
    s, _ = oracle.envmap(0, px, 1.5, tw, tl, golden["envmap_xi"])
    ref = golden["envmap_sample"]
    assert np.allclose(s[:, 3:6], ref[:, 3:6], rtol=1e-5, atol=1e-6)
    assert np.allclose(s[:, 0:3], ref[:, 0:3], rtol=1e-5, atol=1e-6)
    assert np.allclose(s[:, 6], ref[:, 6], rtol=1e-4, atol=1e-6)
    e, _ = oracle.envmap(1, px, 1.5, tw, tl, golden["envmap_eval_in"])
    assert np.allclose(e, golden["envmap_eval"], rtol=1e-4, atol=1e-6)
    assert (s[:, 6] > 0).mean() > 0.9


@pytest.mark.parametrize("curve_type", [0, 1, 2, 3])
def test_curve_interpolators_and_normal_match_reference(golden, curve_type):
    """Curve interpolators (Position4, Velocity4, Acceleration3) and
    SurfaceNormal of render/curve.h, compiled for the host from the reference
    tree, against the oracle's restatement: bit for bit, including the cap
    normals at u = 0 / 1 and the cubic derivative's triple-knot nudge."""
    k = f"curve{curve_type}"
    got = oracle.curve(curve_type, golden[k + "_ctrl"], golden[k + "_u"], golden[k + "_ps"])
    ref = golden[k + "_out"]
    assert np.isfinite(ref).all()
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
