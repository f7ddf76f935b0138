"""Python host wrapper over the C-ABI.  Device buffers are torch CUDA tensors
(plumbing only: every computation runs in libpt_gb300.so's kernels)."""
from __future__ import annotations

import ctypes as C

import torch

from . import abi
from .scenes import Scene


def _stream_ptr(stream=None) -> C.c_void_p:
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


class Context:
    def __init__(self, device: int = 0):
        self.lib = abi.load()
        opts = abi.DeviceOpts(device, 0)
        h = C.c_void_p()
        abi.check(self.lib.pt_context_create(C.byref(opts), C.byref(h)), "pt_context_create", self.lib)
        self.handle = h
        self.device = device

    def close(self):
        if self.handle:
            self.lib.pt_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuScene:
    """A scene uploaded to the GPU with its acceleration structure."""

    def __init__(self, ctx: Context, scene: Scene, bvh_width: int = 4, max_leaf: int = 4, smem_nodes: int = 0,
                 build: bool = True, bvh_flags: int = 0):
        self.ctx = ctx
        self.lib = ctx.lib
        self.scene = scene
        self.width, self.height = scene.width, scene.height
        desc = scene.desc()
        h = C.c_void_p()
        abi.check(self.lib.pt_scene_upload(ctx.handle, C.byref(desc), C.byref(h)), "pt_scene_upload", self.lib)
        self.handle = h
        if build:
            self.build_bvh(bvh_width, max_leaf, smem_nodes, flags=bvh_flags)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.pt_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def build_bvh(self, width: int | None = None, max_leaf: int | None = None, smem_nodes: int | None = None,
                  stream=None, flags: int | None = None) -> abi.BvhStats:
        """pt_bvh_build; flags = abi.BVH_FAST_BUILD builds the radix tree instead of PLOC.
        An option left out keeps the value of the previous build (at the first
        build: width 4, leaves of up to 4 primitives, no shared-memory nodes, PLOC)."""
        prev = getattr(self, "_bvh_args", (4, 4, 0, 0))
        args = tuple(p if v is None else v for v, p in zip((width, max_leaf, smem_nodes, flags), prev))
        o = abi.BvhOpts(*args)
        abi.check(self.lib.pt_bvh_build(self.handle, C.byref(o), _stream_ptr(stream)), "pt_bvh_build", self.lib)
        self._bvh_args = args
        return self.bvh_stats()

    def refit(self, stream=None) -> abi.BvhStats:
        abi.check(self.lib.pt_bvh_refit(self.handle, _stream_ptr(stream)), "pt_bvh_refit", self.lib)
        return self.bvh_stats()

    def update_vertices(self, mesh: int, positions) -> None:
        import numpy as np
        p = np.ascontiguousarray(positions, np.float32)
        abi.check(self.lib.pt_scene_update_vertices(self.handle, mesh, p.ctypes.data_as(C.c_void_p), p.shape[0]),
                  "pt_scene_update_vertices", self.lib)

    def update_all_vertices(self, positions, stream=None) -> None:
        """positions: all meshes' object-space vertices concatenated in mesh
        order, as a (N, 3) float32 CUDA tensor or host array."""
        if isinstance(positions, torch.Tensor) and positions.is_cuda:
            p = positions.contiguous()
            st = self.lib.pt_scene_update_all_vertices(self.handle, C.c_void_p(p.data_ptr()), 1, _stream_ptr(stream))
        else:
            import numpy as np
            p = np.ascontiguousarray(positions, np.float32)
            st = self.lib.pt_scene_update_all_vertices(self.handle, p.ctypes.data_as(C.c_void_p), 0, _stream_ptr(stream))
        abi.check(st, "pt_scene_update_all_vertices", self.lib)

    def bvh_stats(self) -> abi.BvhStats:
        st = abi.BvhStats()
        abi.check(self.lib.pt_bvh_get_stats(self.handle, C.byref(st)), "pt_bvh_get_stats", self.lib)
        return st

    def render_stats(self) -> abi.RenderStats:
        st = abi.RenderStats()
        abi.check(self.lib.pt_render_get_stats(self.handle, C.byref(st)), "pt_render_get_stats", self.lib)
        return st

    def num_prims(self) -> tuple[int, int]:
        a, b = C.c_uint32(), C.c_uint32()
        abi.check(self.lib.pt_scene_num_prims(self.handle, C.byref(a), C.byref(b)), "pt_scene_num_prims", self.lib)
        return a.value, b.value

    def num_curves(self) -> tuple[int, int]:
        """(curve segments, round-cone pieces) of the scene's curve instances."""
        a, b = C.c_uint32(), C.c_uint32()
        abi.check(self.lib.pt_scene_num_curves(self.handle, C.byref(a), C.byref(b)), "pt_scene_num_curves", self.lib)
        return a.value, b.value

    def set_camera(self, cam: abi.CameraDesc) -> None:
        abi.check(self.lib.pt_scene_set_camera(self.handle, C.byref(cam)), "pt_scene_set_camera", self.lib)

    def alloc_buffers(self, aovs: bool = True) -> dict:
        n = self.width * self.height
        dev = torch.device("cuda", self.ctx.device)
        b = {"accum": torch.zeros(n, 4, device=dev), "frame": torch.zeros(n, 4, device=dev)}
        if aovs:
            b["albedo"] = torch.zeros(n, 3, device=dev)
            b["normal"] = torch.zeros(n, 3, device=dev)
            b["test"] = torch.zeros(n, device=dev)
        return b

    def render(self, spp: int, seed: int = 0, sample_cnt: int = 0, accumulate: bool = True,
               rng: int = abi.RNG_PCG32, max_depth: int = 0, wave_spp: int = 0, block_size: int = 0, flags: int = 0,
               buffers: dict | None = None, stream=None) -> dict:
        b = buffers if buffers is not None else self.alloc_buffers()
        p = abi.RenderParams(spp, max_depth, seed, sample_cnt, 1 if accumulate else 0, rng, wave_spp, block_size, flags)
        fb = abi.FrameBuffers(*[b[k].data_ptr() if k in b else None for k in ("accum", "frame", "albedo", "normal", "test")])
        abi.check(self.lib.pt_render(self.handle, C.byref(p), C.byref(fb), _stream_ptr(stream)), "pt_render", self.lib)
        return b

    def autotune(self, spp: int = 4, rng: int = abi.RNG_PCG32, buffers: dict | None = None, stream=None) -> abi.TuneResult:
        b = buffers if buffers is not None else self.alloc_buffers()
        p = abi.RenderParams(spp, 0, 0, 0, 1, rng, 0, 0, 0)
        fb = abi.FrameBuffers(*[b[k].data_ptr() if k in b else None for k in ("accum", "frame", "albedo", "normal", "test")])
        r = abi.TuneResult()
        abi.check(self.lib.pt_autotune(self.handle, C.byref(p), C.byref(fb), C.byref(r), _stream_ptr(stream)),
                  "pt_autotune", self.lib)
        return r

    def trace(self, rays: torch.Tensor, anyhit: bool = False, stream=None) -> torch.Tensor:
        assert rays.is_cuda and rays.dtype == torch.float32 and rays.shape[-1] == 8
        rays = rays.contiguous()
        hits = torch.empty(rays.shape[0], 4, device=rays.device, dtype=torch.float32)
        abi.check(self.lib.pt_trace_rays(self.handle, C.c_void_p(rays.data_ptr()), C.c_void_p(hits.data_ptr()),
                                         rays.shape[0], 1 if anyhit else 0, _stream_ptr(stream)), "pt_trace_rays", self.lib)
        return hits


def render_batch(ctx: Context, scenes: list, spp: int, seed: int = 0, sample_cnt: int = 0, accumulate: bool = True,
                 rng: int = abi.RNG_PCG32, max_depth: int = 0, wave_spp: int = 0, block_size: int = 0, flags: int = 0,
                 buffers: list | None = None, stream=None) -> list:
    """pt_render_batch: every GpuScene of `scenes` rendered in one launch per
    bounce; returns one buffer dict per scene."""
    lib = ctx.lib
    bufs = buffers if buffers is not None else [g.alloc_buffers() for g in scenes]
    handles = (C.c_void_p * len(scenes))(*[g.handle.value if isinstance(g.handle, C.c_void_p) else g.handle
                                            for g in scenes])
    fbs = (abi.FrameBuffers * len(scenes))(*[
        abi.FrameBuffers(*[b[k].data_ptr() if k in b else None for k in ("accum", "frame", "albedo", "normal", "test")])
        for b in bufs])
    p = abi.RenderParams(spp, max_depth, seed, sample_cnt, 1 if accumulate else 0, rng, wave_spp, block_size, flags)
    abi.check(lib.pt_render_batch(ctx.handle, C.cast(handles, C.c_void_p), C.byref(p), C.cast(fbs, C.c_void_p),
                                  len(scenes), _stream_ptr(stream)), "pt_render_batch", lib)
    return bufs


def render_batch_stats(ctx: Context) -> abi.RenderStats:
    st = abi.RenderStats()
    abi.check(ctx.lib.pt_render_batch_get_stats(ctx.handle, C.byref(st)), "pt_render_batch_get_stats", ctx.lib)
    return st


def bsdf_eval(bsdf: torch.Tensor, wo: torch.Tensor, wi: torch.Tensor):
    lib = abi.load()
    n = bsdf.shape[0]
    f = torch.empty(n, 3, device=bsdf.device)
    pdf = torch.empty(n, device=bsdf.device)
    abi.check(lib.pt_bsdf_eval_batch(*[C.c_void_p(t.data_ptr()) for t in (bsdf.contiguous(), wo.contiguous(),
                                                                          wi.contiguous(), f, pdf)], n, _stream_ptr()),
              "pt_bsdf_eval_batch", lib)
    return f, pdf


def bsdf_sample(bsdf: torch.Tensor, wo: torch.Tensor, rng_state: torch.Tensor):
    lib = abi.load()
    n = bsdf.shape[0]
    dev = bsdf.device
    rng = rng_state.clone().contiguous()
    wi = torch.empty(n, 3, device=dev)
    f = torch.empty(n, 3, device=dev)
    pdf = torch.empty(n, device=dev)
    typ = torch.empty(n, dtype=torch.int32, device=dev)
    abi.check(lib.pt_bsdf_sample_batch(*[C.c_void_p(t.data_ptr()) for t in (bsdf.contiguous(), wo.contiguous(), rng,
                                                                            wi, f, pdf, typ)], n, _stream_ptr()),
              "pt_bsdf_sample_batch", lib)
    return wi, f, pdf, typ, rng
