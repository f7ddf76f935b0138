"""CPU reference of the learned denoiser -- TEST INFRASTRUCTURE ONLY.

PyTorch-CPU FP32 restatement of the U-Net that libpt_gb300.so trains and runs
on the GPU (the reference's OptiX denoiser, framework/optix/denoiser.cpp:171-267,
is a closed model, so the network is this project's own and this module is its
specification): 14 3x3 convolutions, 2x2 mean pooling, nearest 2x upsampling,
concatenation [upsampled, skip], ReLU after every hidden convolution, log-domain
input, output = the input's log colour plus the network's correction, L1 loss on
log(1 + x).  With ``bf16=True`` every stored tensor
(network input, weights, activations) is rounded to bfloat16 where the GPU stores
it, and autograd passes gradients straight through the rounding.

Only tests/ may import this module.
"""
from __future__ import annotations

import numpy as np
import torch
import torch.nn.functional as F

# (cin, cout, relu) per layer, in the library's parameter order
LAYERS = [
    (16, 32, 1), (32, 32, 1), (32, 48, 1), (48, 48, 1), (48, 64, 1), (64, 64, 1), (64, 128, 1),
    (128, 128, 1), (128, 256, 1), (384, 128, 1), (192, 64, 1), (112, 48, 1), (80, 32, 1), (32, 16, 0),
]


def split_params(flat: np.ndarray) -> list[tuple[np.ndarray, np.ndarray]]:
    out, off = [], 0
    for cin, cout, _ in LAYERS:
        nw = 9 * cin * cout
        out.append((flat[off:off + nw].reshape(cout, 9, cin), flat[off + nw:off + nw + cout]))
        off += nw + cout
    return out


def _r(t: torch.Tensor, bf16: bool) -> torch.Tensor:
    if not bf16:
        return t
    return t + (t.to(torch.bfloat16).to(torch.float32) - t).detach()


def to_torch_weight(w: np.ndarray) -> torch.Tensor:
    """(cout, 9, cin) -> torch conv weight (cout, cin, 3, 3)."""
    cout, _, cin = w.shape
    return torch.from_numpy(np.ascontiguousarray(w.reshape(cout, 3, 3, cin).transpose(0, 3, 1, 2)))


def from_torch_weight(w: torch.Tensor) -> np.ndarray:
    cout, cin = w.shape[:2]
    return w.detach().numpy().transpose(0, 2, 3, 1).reshape(cout, 9, cin)


def pack_input(inp: torch.Tensor, bf16: bool) -> torch.Tensor:
    """(n, h, w, 9) colour/albedo/normal -> (n, 16, h, w) network input."""
    x = inp.to(torch.float32)
    rgb = torch.log1p(torch.clamp(x[..., :3], min=0.0))
    feat = torch.cat([rgb, x[..., 3:9], torch.zeros(*x.shape[:3], 7)], dim=-1)
    return _r(feat.permute(0, 3, 1, 2).contiguous(), bf16)


def forward(params: list[tuple[torch.Tensor, torch.Tensor]], inp: torch.Tensor, bf16: bool = True) -> torch.Tensor:
    """Returns the log-domain output (n, 3, h, w)."""
    def conv(i, x):
        w, b = params[i]
        y = F.conv2d(x, _r(w, bf16), b, padding=1)
        if LAYERS[i][2]:
            y = torch.relu(y)
        return y

    def rconv(i, x):
        return _r(conv(i, x), bf16)

    def pool(x):
        return _r(F.avg_pool2d(x, 2), bf16)

    def up(x):
        return F.interpolate(x, scale_factor=2, mode="nearest")

    x0 = pack_input(inp, bf16)
    a0 = rconv(0, x0)
    e0 = rconv(1, a0)
    a1 = rconv(2, pool(e0))
    e1 = rconv(3, a1)
    a2 = rconv(4, pool(e1))
    e2 = rconv(5, a2)
    a3 = rconv(6, pool(e2))
    e3 = rconv(7, a3)
    b4 = rconv(8, pool(e3))
    d3 = rconv(9, torch.cat([up(b4), e3], dim=1))
    d2 = rconv(10, torch.cat([up(d3), e2], dim=1))
    d1 = rconv(11, torch.cat([up(d2), e1], dim=1))
    d0 = rconv(12, torch.cat([up(d1), e0], dim=1))
    out = conv(13, d0)
    return out[:, :3] + x0[:, :3]  # residual: the network corrects the input's log colour


def loss_and_grads(flat: np.ndarray, inp: np.ndarray, target: np.ndarray, bf16: bool = True):
    """L1 loss on log(1 + x) and the flat gradient vector (library layout)."""
    params = []
    for w, b in split_params(flat):
        params.append((to_torch_weight(w).requires_grad_(True), torch.from_numpy(b.copy()).requires_grad_(True)))
    inp_t = torch.from_numpy(np.asarray(inp, dtype=np.float32))
    tgt = torch.log1p(torch.clamp(torch.from_numpy(np.asarray(target, dtype=np.float32)), min=0.0)).permute(0, 3, 1, 2)
    out = forward(params, inp_t, bf16)
    loss = (out - tgt).abs().mean()
    loss.backward()
    grads = []
    for w, b in params:
        grads.append(from_torch_weight(w.grad).ravel())
        grads.append(b.grad.numpy().ravel())
    return float(loss), np.concatenate(grads).astype(np.float32)


def denoise(flat: np.ndarray, inp: np.ndarray, bf16: bool = True) -> np.ndarray:
    """Network output as linear RGB, (n, h, w, 3)."""
    params = [(to_torch_weight(w), torch.from_numpy(b.copy())) for w, b in split_params(flat)]
    with torch.no_grad():
        out = forward(params, torch.from_numpy(np.asarray(inp, dtype=np.float32)), bf16)
    return torch.clamp(torch.expm1(out), min=0.0).permute(0, 2, 3, 1).numpy()
