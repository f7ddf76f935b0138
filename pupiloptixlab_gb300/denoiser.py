"""Python wrapper of the learned denoiser's C-ABI (pt_denoiser_* / pt_denoise /
pt_conv3x3_*).  Tensors are torch CUDA tensors used as device buffers; every
computation runs in libpt_gb300.so's kernels.

Layouts: activations NHWC (bf16 for the convolution entry points), training
inputs ``(n, h, w, 9)`` float16 (colour, albedo, normal), targets
``(n, h, w, 3)`` float32 linear RGB, weights ``(cout_pad, 9, cin)`` with the
tap index ``3 * dy + dx``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import abi
from .api import Context, _stream_ptr


def _p(t: torch.Tensor | None) -> C.c_void_p:
    return C.c_void_p(t.data_ptr() if t is not None else 0)


def conv3x3_forward(x: torch.Tensor, w: torch.Tensor, bias: torch.Tensor | None, cout: int, relu: bool = False,
                    out_f32: bool = False) -> torch.Tensor:
    """x (n, h, w, cin) bf16, w (cout_pad, 9, cin) bf16, bias (cout,) f32."""
    lib = abi.load()
    n, h, wd, cin = x.shape
    y = torch.empty(n, h, wd, cout, device=x.device, dtype=torch.float32 if out_f32 else torch.bfloat16)
    abi.check(lib.pt_conv3x3_forward(_p(x.contiguous()), n, h, wd, cin, _p(w.contiguous()),
                                     _p(bias.contiguous() if bias is not None else None), cout, int(relu), int(out_f32),
                                     _p(y), _stream_ptr()), "pt_conv3x3_forward", lib)
    return y


def conv3x3_backward_data(dy: torch.Tensor, w: torch.Tensor, cin: int, mask: torch.Tensor | None = None) -> torch.Tensor:
    """dy (n, h, w, cout_pad) bf16, w (cout_pad, 9, cin) bf16 -> dx (n, h, w, cin) bf16."""
    lib = abi.load()
    n, h, wd, cout = dy.shape
    dx = torch.empty(n, h, wd, cin, device=dy.device, dtype=torch.bfloat16)
    abi.check(lib.pt_conv3x3_backward_data(_p(dy.contiguous()), n, h, wd, cout, _p(w.contiguous()), cin,
                                           _p(mask.contiguous() if mask is not None else None), _p(dx), _stream_ptr()),
              "pt_conv3x3_backward_data", lib)
    return dx


def conv3x3_backward_weights(x: torch.Tensor, dy: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    """x (n, h, w, cin) bf16, dy (n, h, w, cout) bf16 -> (dw (cout, 9, cin) f32, db (cout,) f32)."""
    lib = abi.load()
    n, h, wd, cin = x.shape
    cout = dy.shape[-1]
    dw = torch.zeros(cout, 9, cin, device=x.device, dtype=torch.float32)
    db = torch.zeros(cout, device=x.device, dtype=torch.float32)
    abi.check(lib.pt_conv3x3_backward_weights(_p(x.contiguous()), n, h, wd, cin, _p(dy.contiguous()), cout, _p(dw),
                                              _p(db), _stream_ptr()), "pt_conv3x3_backward_weights", lib)
    return dw, db


def pack_frame(buffers: dict, width: int, height: int) -> torch.Tensor:
    """Render buffers (accum float4, albedo float3, normal float3) -> (h, w, 9) float16."""
    lib = abi.load()
    out = torch.empty(height, width, 9, device=buffers["accum"].device, dtype=torch.float16)
    abi.check(lib.pt_denoise_pack(_p(buffers["accum"]), _p(buffers["albedo"]), _p(buffers["normal"]), width, height,
                                  _p(out), _stream_ptr()), "pt_denoise_pack", lib)
    return out


class Denoiser:
    """The U-Net denoiser (pt_denoiser)."""

    def __init__(self, ctx: Context, lr: float = 1e-3, seed: int = 1, beta1: float = 0.9, beta2: float = 0.999,
                 eps: float = 1e-8):
        self.ctx = ctx
        self.lib = ctx.lib
        opts = abi.DenoiserOpts(lr, beta1, beta2, eps, seed)
        h = C.c_void_p()
        abi.check(self.lib.pt_denoiser_create(ctx.handle, C.byref(opts), C.byref(h)), "pt_denoiser_create", self.lib)
        self.handle = h
        n = C.c_uint64()
        abi.check(self.lib.pt_denoiser_num_params(h, C.byref(n)), "pt_denoiser_num_params", self.lib)
        self.num_params = n.value
        self.layers = []
        i = 0
        while True:
            cin, cout, off = C.c_uint32(), C.c_uint32(), C.c_uint64()
            if self.lib.pt_denoiser_layer(h, i, C.byref(cin), C.byref(cout), C.byref(off)) != 0:
                break
            self.layers.append((cin.value, cout.value, off.value))
            i += 1

    def close(self):
        if getattr(self, "handle", None):
            self.lib.pt_denoiser_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # parameters ------------------------------------------------------------
    def get_params(self) -> np.ndarray:
        p = np.empty(self.num_params, dtype=np.float32)
        abi.check(self.lib.pt_denoiser_get_params(self.handle, p.ctypes.data_as(C.c_void_p)), "get_params", self.lib)
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.num_params
        abi.check(self.lib.pt_denoiser_set_params(self.handle, p.ctypes.data_as(C.c_void_p)), "set_params", self.lib)

    def get_state(self) -> np.ndarray:
        """Adam's moments and counters (2 * num_params + 4 floats)."""
        out = np.empty(2 * self.num_params + 4, np.float32)
        abi.check(self.lib.pt_denoiser_get_state(self.handle, out.ctypes.data_as(C.c_void_p)), "pt_denoiser_get_state",
                  self.lib)
        return out

    def set_state(self, state: np.ndarray) -> None:
        st = np.ascontiguousarray(state, np.float32)
        assert st.shape == (2 * self.num_params + 4,)
        abi.check(self.lib.pt_denoiser_set_state(self.handle, st.ctypes.data_as(C.c_void_p)), "pt_denoiser_set_state",
                  self.lib)

    def save(self, path) -> None:
        """Weights and optimizer state to one .npz file."""
        np.savez(path, params=self.get_params(), state=self.get_state())

    def load(self, path) -> None:
        d = np.load(path)
        self.set_params(d["params"])
        self.set_state(d["state"])

    def get_grads(self) -> np.ndarray:
        g = np.empty(self.num_params, dtype=np.float32)
        abi.check(self.lib.pt_denoiser_get_grads(self.handle, g.ctypes.data_as(C.c_void_p)), "get_grads", self.lib)
        return g

    def split(self, flat: np.ndarray) -> list[tuple[np.ndarray, np.ndarray]]:
        """Flat parameter vector -> [(w (cout, 9, cin), b (cout,))] per layer."""
        out = []
        for cin, cout, off in self.layers:
            nw = 9 * cin * cout
            out.append((flat[off:off + nw].reshape(cout, 9, cin), flat[off + nw:off + nw + cout]))
        return out

    # training / inference --------------------------------------------------
    def compute_grads(self, inputs: torch.Tensor, targets: torch.Tensor) -> float:
        n, h, w, _ = inputs.shape
        loss = C.c_float()
        abi.check(self.lib.pt_denoiser_compute_grads(self.handle, _p(inputs.contiguous()), _p(targets.contiguous()), n,
                                                     h, w, C.byref(loss), _stream_ptr()), "compute_grads", self.lib)
        return loss.value

    def train_step(self, inputs: torch.Tensor, targets: torch.Tensor) -> None:
        n, h, w, _ = inputs.shape
        assert h == w
        abi.check(self.lib.pt_denoiser_train_step(self.handle, _p(inputs), _p(targets), n, h, _stream_ptr()),
                  "pt_denoiser_train_step", self.lib)

    def set_lr(self, lr: float) -> None:
        abi.check(self.lib.pt_denoiser_set_lr(self.handle, lr), "pt_denoiser_set_lr", self.lib)

    def read_loss(self) -> float:
        v = C.c_float()
        abi.check(self.lib.pt_denoiser_read_loss(self.handle, C.byref(v)), "pt_denoiser_read_loss", self.lib)
        return v.value

    def forward(self, inputs: torch.Tensor) -> torch.Tensor:
        n, h, w, _ = inputs.shape
        out = torch.empty(n, h, w, 3, device=inputs.device, dtype=torch.float32)
        abi.check(self.lib.pt_denoiser_forward(self.handle, _p(inputs.contiguous()), n, h, w, _p(out), _stream_ptr()),
                  "pt_denoiser_forward", self.lib)
        return out

    def denoise(self, buffers: dict, width: int, height: int, tile: int = 16, fallback_rel: float = 0.25,
                fallback_sigma: float = 4.0, want_tiles: bool = False, ensemble: bool = False):
        """Denoise a rendered frame; returns (output (h*w, 4) f32, stats, tile flags or None).
        ensemble = True averages the network over the frame and its mirror image."""
        dev = buffers["accum"].device
        out = torch.empty(width * height, 4, device=dev, dtype=torch.float32)
        tiles = ((width + tile - 1) // tile) * ((height + tile - 1) // tile)
        flags = torch.zeros(tiles, dtype=torch.uint8, device=dev) if want_tiles else None
        io = abi.DenoiseIO(width, height, buffers["accum"].data_ptr(), buffers["albedo"].data_ptr(),
                           buffers["normal"].data_ptr(), out.data_ptr(), tile, fallback_rel, fallback_sigma,
                           flags.data_ptr() if flags is not None else None,
                           abi.DENOISE_FLIP_ENSEMBLE if ensemble else 0)
        abi.check(self.lib.pt_denoise(self.handle, C.byref(io), _stream_ptr()), "pt_denoise", self.lib)
        st = abi.DenoiseStats()
        abi.check(self.lib.pt_denoise_get_stats(self.handle, C.byref(st)), "pt_denoise_get_stats", self.lib)
        return out, st, flags
