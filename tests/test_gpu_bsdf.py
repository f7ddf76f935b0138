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
    # the shared trigonometry makes every sample identical to the reference's
    # headers compiled for the host: same lobe, random stream and bits
    assert np.array_equal(typ, golden["sample_type"]) and np.array_equal(rng, golden["sample_seed_out"])
    assert close(wi, golden["sample_wi"])
    assert np.array_equal(wi, golden["sample_wi"], equal_nan=True)
    assert np.array_equal(f, golden["sample_f"], equal_nan=True)
    assert np.array_equal(pdf, golden["sample_pdf"], equal_nan=True)
    # sampled non-delta lobes: value and pdf also equal the reference's
    # evaluation at the drawn direction (within the eval tolerance)
    smooth = ((typ & 0x60) == 0) & (typ != 0) & (golden["sample_pdf"] != 0)
    ref_f, ref_pdf = oracle.bsdf_eval(golden["sample_bsdf"][smooth], golden["sample_wo"][smooth], wi[smooth])
    assert close(f[smooth], ref_f)
    assert close(pdf[smooth], ref_pdf)
