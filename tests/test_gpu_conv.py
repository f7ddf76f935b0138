"""Denoiser convolution kernels (tcgen05 implicit GEMM, TMA-staged operands)
against PyTorch-CPU FP32 convolutions of the same BF16 values.

Tolerances: FP32 outputs differ from the CPU only by accumulation order
(|err| <= 2e-3 * max|ref|, relative L2 <= 1e-4); BF16 outputs additionally by one rounding
(relative L2 <= 4e-3)."""
import pytest
import torch
import torch.nn.functional as F

pytestmark = pytest.mark.gpu


def _bf16(shape, gen, scale=1.0):
    return (torch.randn(*shape, generator=gen) * scale).to(torch.bfloat16)


def _ref_conv(x_nhwc, w_oti, bias):
    """x (n,h,w,cin) bf16, w (cout,9,cin) bf16 -> (n,h,w,cout) f32 on the CPU."""
    cout, _, cin = w_oti.shape
    x = x_nhwc.float().permute(0, 3, 1, 2)
    w = w_oti.float().reshape(cout, 3, 3, cin).permute(0, 3, 1, 2)
    y = F.conv2d(x, w, bias, padding=1)
    return y.permute(0, 2, 3, 1)


def _rel_l2(a, b):
    return float((a - b).norm() / max(float(b.norm()), 1e-30))


SHAPES = [
    # n, h, w, cin, cout
    (2, 16, 16, 16, 32),      # KC 16, narrow image (two rows per tile... 8 rows of 16)
    (1, 24, 200, 32, 48),     # KC 32, width >= 128 not a multiple of 128
    (2, 12, 48, 64, 64),      # KC 64, width < 128 not dividing 128
    (1, 8, 256, 128, 256),    # N = 256
    (1, 8, 64, 384, 128),     # K = 9 * 384
    (1, 16, 32, 80, 384),     # N tiled (2 x 192)
    (3, 4, 4, 48, 16),        # tiny images
    (2, 7, 130, 16, 32),      # two-row halo tiles, odd height (the last tile's second row is outside)
    (1, 6, 128, 32, 112),     # two-row halo tiles with 448 of the 512 TMEM columns (one CTA per SM)
]


@pytest.mark.parametrize("shape", [(2, 7, 130, 16, 32), (1, 9, 256, 32, 64), (2, 6, 128, 48, 48),
                                   (1, 4, 256, 16, 80)])
def test_conv_forward_halo_rows_agree(cuda_ctx, shape, monkeypatch):
    """Halo tiles of one to four output rows issue the same MMAs per output
    row in the same order: the FP32 results are identical."""
    from pupiloptixlab_gb300 import denoiser as dnm
    n, h, w, cin, cout = shape
    g = torch.Generator().manual_seed(5 + h)
    x = _bf16((n, h, w, cin), g).cuda()
    wt = _bf16((cout, 9, cin), g, 0.1).cuda()
    b = torch.randn(cout, generator=g).cuda()
    ys = []
    for rows in ("1", "2", "3", "4"):
        monkeypatch.setenv("PT_CONV_HALO_ROWS", rows)
        ys.append(dnm.conv3x3_forward(x, wt, b, cout, relu=False, out_f32=True).cpu())
    for y in ys[1:]:
        assert torch.equal(ys[0], y)
    assert _rel_l2(ys[0], _ref_conv(x.cpu(), wt.cpu(), b.cpu())) <= 1e-4


@pytest.mark.parametrize("shape", SHAPES)
def test_conv_forward_f32(cuda_ctx, shape):
    from pupiloptixlab_gb300 import denoiser as dnm
    n, h, w, cin, cout = shape
    g = torch.Generator().manual_seed(hash(shape) & 0xFFFF)
    x = _bf16((n, h, w, cin), g)
    wt = _bf16((cout, 9, cin), g, 0.1)
    b = torch.randn(cout, generator=g)
    y = dnm.conv3x3_forward(x.cuda(), wt.cuda(), b.cuda(), cout, relu=False, out_f32=True).cpu()
    ref = _ref_conv(x, wt, b)
    assert torch.isfinite(y).all()
    assert float((y - ref).abs().max()) <= 2e-3 * float(ref.abs().max())
    assert _rel_l2(y, ref) <= 1e-4


@pytest.mark.parametrize("shape", SHAPES[:4])
def test_conv_forward_bf16_relu(cuda_ctx, shape):
    from pupiloptixlab_gb300 import denoiser as dnm
    n, h, w, cin, cout = shape
    g = torch.Generator().manual_seed(7 + cin)
    x = _bf16((n, h, w, cin), g)
    wt = _bf16((cout, 9, cin), g, 0.1)
    b = torch.randn(cout, generator=g) * 0.1
    y = dnm.conv3x3_forward(x.cuda(), wt.cuda(), b.cuda(), cout, relu=True).cpu().float()
    ref = torch.relu(_ref_conv(x, wt, b))
    assert _rel_l2(y, ref) <= 4e-3
    assert float(((y == 0) == (ref <= 0)).float().mean()) > 0.99


@pytest.mark.parametrize("shape", [(2, 16, 16, 32, 16), (1, 24, 200, 48, 32), (1, 8, 64, 384, 128),
                                   (2, 12, 48, 64, 64), (1, 8, 32, 16, 256)])
def test_conv_backward_data(cuda_ctx, shape):
    from pupiloptixlab_gb300 import denoiser as dnm
    n, h, w, cin, cout = shape
    g = torch.Generator().manual_seed(11 + cout)
    dy = _bf16((n, h, w, cout), g)
    wt = _bf16((cout, 9, cin), g, 0.1)
    mask = _bf16((n, h, w, cin), g)
    dx = dnm.conv3x3_backward_data(dy.cuda(), wt.cuda(), cin, mask.cuda()).cpu().float()
    # reference: gradient of conv2d w.r.t. its input, times (mask > 0)
    xr = torch.zeros(n, cin, h, w, requires_grad=True)
    wr = wt.float().reshape(cout, 3, 3, cin).permute(0, 3, 1, 2)
    F.conv2d(xr, wr, padding=1).backward(dy.float().permute(0, 3, 1, 2))
    ref = xr.grad.permute(0, 2, 3, 1) * (mask.float() > 0)
    assert _rel_l2(dx, ref) <= 4e-3
    dx2 = dnm.conv3x3_backward_data(dy.cuda(), wt.cuda(), cin).cpu().float()
    assert _rel_l2(dx2, xr.grad.permute(0, 2, 3, 1)) <= 4e-3


@pytest.mark.parametrize("shape", [(2, 16, 16, 16, 32), (1, 8, 256, 32, 48), (2, 16, 64, 64, 64),
                                   (1, 8, 32, 384, 128), (2, 8, 8, 128, 256), (4, 2, 2, 48, 16),
                                   (1, 4, 200, 80, 32)])
def test_conv_backward_weights(cuda_ctx, shape):
    from pupiloptixlab_gb300 import denoiser as dnm
    n, h, w, cin, cout = shape
    g = torch.Generator().manual_seed(23 + cin)
    x = _bf16((n, h, w, cin), g)
    dy = _bf16((n, h, w, cout), g)
    dw, db = dnm.conv3x3_backward_weights(x.cuda(), dy.cuda())
    dw, db = dw.cpu(), db.cpu()
    wr = torch.zeros(cout, cin, 3, 3, requires_grad=True)
    br = torch.zeros(cout, requires_grad=True)
    F.conv2d(x.float().permute(0, 3, 1, 2), wr, br, padding=1).backward(dy.float().permute(0, 3, 1, 2))
    ref = wr.grad.permute(0, 2, 3, 1).reshape(cout, 9, cin)
    assert _rel_l2(dw, ref) <= 1e-4
    assert _rel_l2(db, br.grad) <= 1e-4


@pytest.mark.parametrize("shape", [(4, 64, 64, 16, 32), (2, 8, 256, 32, 48), (2, 16, 64, 80, 32)])
def test_conv_backward_weights_repeatable(cuda_ctx, shape):
    """Repeated weight gradients (and the bias gradient taken from the same
    MMAs) differ only by the order of the FP32 atomic sums: no stage is read
    before its copies landed or after the next tile's copies overwrote it."""
    from pupiloptixlab_gb300 import denoiser as dnm
    n, h, w, cin, cout = shape
    g = torch.Generator().manual_seed(31 + cin)
    x = _bf16((n, h, w, cin), g).cuda()
    dy = _bf16((n, h, w, cout), g).cuda()
    outs = []
    for _ in range(6):
        dw, db = dnm.conv3x3_backward_weights(x, dy)
        outs.append((dw.cpu(), db.cpu()))
    scale_w = float(outs[0][0].abs().max())
    scale_b = float(outs[0][1].abs().max())
    for dw, db in outs[1:]:
        assert float((dw - outs[0][0]).abs().max()) <= 1e-5 * scale_w
        assert float((db - outs[0][1]).abs().max()) <= 1e-5 * scale_b


@pytest.mark.parametrize("shape", [(2, 16, 16, 16, 32), (1, 8, 256, 128, 256)], ids=["ring", "halo_resident"])
def test_bounded_wait_runs_out_and_the_next_convolution_is_right(cuda_ctx, shape):
    """The timeout path of the forward kernel, without a fault: with a 1 ms
    limit and the stall request, the MMA warp waits on a barrier that nothing
    arrives at; the wait runs out, the CTA records the error, lets the copies
    it issued land (and the other warps stop waiting), frees its tensor memory
    and returns.  The call reports PT_ERR_TIMEOUT well inside the normal 2 s
    limit, and the next convolution, with the default limit, is correct."""
    import time

    from pupiloptixlab_gb300 import abi
    from pupiloptixlab_gb300 import denoiser as dnm
    n, h, w, cin, cout = shape
    g = torch.Generator().manual_seed(7)
    x = _bf16((n, h, w, cin), g).cuda()
    wt = _bf16((cout, 9, cin), g, 0.1).cuda()
    lib = cuda_ctx.lib
    assert lib.pt_conv_set_wait_limit(1_000_000, 1) == 0
    try:
        t0 = time.perf_counter()
        with pytest.raises(abi.PtError) as e:
            dnm.conv3x3_forward(x, wt, None, cout, relu=False, out_f32=True)
        elapsed = time.perf_counter() - t0
    finally:
        assert lib.pt_conv_set_wait_limit(0, 0) == 0
    assert e.value.status == 4 and "bounded wait ran out" in str(e.value)
    assert elapsed < 1.5, elapsed
    # the context is healthy: the same convolution with the default limit
    y = dnm.conv3x3_forward(x, wt, None, cout, relu=False, out_f32=True).cpu()
    ref = _ref_conv(x.cpu(), wt.cpu(), None)
    assert float((y - ref).abs().max()) <= 2e-3 * float(ref.abs().max())
    assert _rel_l2(y, ref) <= 1e-4
