"""Training pairs for the learned denoiser, rendered by the tracer itself.

Each pair is a ``crop x crop`` view of a seeded icosphere-field scene (the
generator of the 1M-triangle headline scene, with a seeded number of
instances) seen from a seeded random camera: the input is a ``noisy_spp`` render packed
as 9 FP16 channels (colour, albedo, normal; pt_denoise_pack) and the target
is an independent ``target_spp`` render of the same view (FP32 RGB).  Both
renders drop non-finite samples (PT_RENDER_DROP_NONFINITE) so that a single
NaN sample cannot poison a training target.

Everything stays on the device: the returned tensors are CUDA tensors that
pt_denoiser_train_step reads in place.
"""
from __future__ import annotations

import math
import time

import numpy as np
import torch

from . import abi, scenes
from .api import Context, GpuScene
from .denoiser import pack_frame


def random_view(rng: np.random.Generator, aspect: float = 1.0) -> abi.CameraDesc:
    """A camera somewhere around the icosphere field, looking into it."""
    r = rng.uniform(14.0, 40.0)
    phi = rng.uniform(0.0, 2.0 * math.pi)
    eye = (r * math.cos(phi), rng.uniform(2.0, 30.0), r * math.sin(phi))
    target = (rng.uniform(-8.0, 8.0), rng.uniform(2.0, 18.0), rng.uniform(-8.0, 8.0))
    fov = rng.uniform(20.0, 55.0)
    return scenes.camera(fov, aspect, scenes.look_at_to_world(eye, target))


def render_pairs(ctx: Context, count: int, crop: int = 256, noisy_spp=4, target_spp: int = 1024,
                 crops_per_scene: int = 32, instances=(60, 200), first_seed: int = 1, max_depth: int = 8,
                 log=None) -> tuple[torch.Tensor, torch.Tensor, dict]:
    """Render `count` training pairs: (inputs (count, crop, crop, 9) f16,
    targets (count, crop, crop, 3) f32, info).  `noisy_spp` is an int or a
    sequence to draw each pair's input spp from; `instances` an int or a
    (low, high) range drawn per scene."""
    spp_choices = [int(noisy_spp)] if np.isscalar(noisy_spp) else [int(v) for v in noisy_spp]
    inst_range = (int(instances), int(instances)) if np.isscalar(instances) else tuple(int(v) for v in instances)
    dev = torch.device("cuda", ctx.device)
    inputs = torch.empty(count, crop, crop, 9, device=dev, dtype=torch.float16)
    targets = torch.empty(count, crop, crop, 3, device=dev, dtype=torch.float32)
    t0 = time.perf_counter()
    render_s = 0.0
    made = 0
    scene_seed = first_seed
    while made < count:
        rng = np.random.default_rng(10007 * scene_seed + 1)
        n_inst = int(rng.integers(inst_range[0], inst_range[1] + 1))
        sc = scenes.icosphere_field(crop, crop, max_depth=max_depth, num_instances=n_inst, seed=scene_seed)
        g = GpuScene(ctx, sc)
        noisy = g.alloc_buffers()
        ref = g.alloc_buffers(aovs=False)
        for _ in range(min(crops_per_scene, count - made)):
            g.set_camera(random_view(rng))
            torch.cuda.synchronize()
            t = time.perf_counter()
            s = int(rng.integers(0, 1 << 20))
            spp = spp_choices[int(rng.integers(0, len(spp_choices)))]
            g.render(spp=spp, seed=s, flags=abi.RENDER_DROP_NONFINITE, buffers=noisy)
            g.render(spp=target_spp, seed=s + (1 << 21), flags=abi.RENDER_DROP_NONFINITE, buffers=ref)
            inputs[made] = pack_frame(noisy, crop, crop)
            targets[made] = ref["accum"][:, :3].reshape(crop, crop, 3)
            torch.cuda.synchronize()
            render_s += time.perf_counter() - t
            made += 1
        g.close()
        if log:
            log(f"denoiser data: scene {scene_seed}, {made}/{count} pairs")
        scene_seed += 1
    info = {"pairs": count, "crop": crop, "noisy_spp": spp_choices, "target_spp": target_spp,
            "scenes": scene_seed - first_seed, "instances_per_scene": list(inst_range),
            "render_s": render_s, "total_s": time.perf_counter() - t0}
    return inputs, targets, info
