"""Device BSDF code (pt_bsdf_eval_batch / pt_bsdf_sample_batch) against the
golden vectors of the reference's own material headers compiled for the
host.  Tolerance: 1e-5 absolute + 1e-5 relative.  Evaluation involves no
transcendental function and is compiled without contraction, so it must also
be bit-identical; sampling goes through CUDA's sinf/cosf, which may differ by
an ulp from the host's."""
import numpy as np
import pytest
import torch

from pupiloptixlab_gb300 import api

pytestmark = pytest.mark.gpu

RTOL = ATOL = 1e-5


def close(a, b):
    return np.allclose(a, b, rtol=RTOL, atol=ATOL, equal_nan=True)


def T(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_eval_matches_reference(cuda_ctx, golden):
    f, pdf = api.bsdf_eval(T(golden["eval_bsdf"]), T(golden["eval_wo"]), T(golden["eval_wi"]))
    f, pdf = f.cpu().numpy(), pdf.cpu().numpy()
    for k in range(1, 8):
        m = golden["eval_bsdf"][:, 0] == k
        assert close(f[m], golden["eval_f"][m]), f"material {k}: f"
        assert close(pdf[m], golden["eval_pdf"][m]), f"material {k}: pdf"
    assert np.array_equal(f, golden["eval_f"], equal_nan=True)
    assert np.array_equal(pdf, golden["eval_pdf"], equal_nan=True)


def test_sample_matches_reference(cuda_ctx, golden):
    import oracle
    seeds = golden["sample_seed"].view(np.int32)
    wi, f, pdf, typ, rng = api.bsdf_sample(T(golden["sample_bsdf"]), T(golden["sample_wo"]), T(seeds))
    wi, f, pdf = wi.cpu().numpy(), f.cpu().numpy(), pdf.cpu().numpy()
    typ, rng = typ.cpu().numpy().view(np.uint32), rng.cpu().numpy().view(np.uint32)
    same_path = (typ == golden["sample_type"]) & (rng == golden["sample_seed_out"])
    # a lobe choice can only flip when a random number sits within an ulp of a threshold
    assert same_path.mean() > 0.998
    assert close(wi[same_path], golden["sample_wi"][same_path])
    delta = same_path & ((typ & 0x60) != 0)
    # delta lobes: reflect / refract / Fresnel use no transcendental function -> identical
    assert np.array_equal(f[delta], golden["sample_f"][delta], equal_nan=True)
    assert np.array_equal(pdf[delta], golden["sample_pdf"][delta], equal_nan=True)
    # sampled non-delta lobes: value and pdf are the reference's evaluation at the
    # direction the GPU drew (which may differ from the host's by an ulp of sin/cos)
    smooth = same_path & ((typ & 0x60) == 0) & (typ != 0)
    # early returns after the lobe was chosen (e.g. a refraction that stays on
    # the same side, rough_dielectric.h:149-150) leave f = pdf = 0 on both sides
    rejected = smooth & (golden["sample_pdf"] == 0)
    assert np.all(pdf[rejected] == 0) and np.all(f[rejected] == 0)
    smooth &= golden["sample_pdf"] != 0
    ref_f, ref_pdf = oracle.bsdf_eval(golden["sample_bsdf"][smooth], golden["sample_wo"][smooth], wi[smooth])
    assert close(f[smooth], ref_f)
    assert close(pdf[smooth], ref_pdf)
    for k in range(1, 8):
        m = (golden["sample_bsdf"][:, 0] == k) & same_path & ~delta & ~smooth
        assert close(f[m], golden["sample_f"][m]) and close(pdf[m], golden["sample_pdf"][m]), f"material {k}"
