"""Benchmark of the path-tracing-with-MIS hot path on one GB300.

Workload: the 1M-triangle procedural scene -- 200 seeded FBM-displaced
icospheres (5,120 triangles each) in a 20^3 box over a ground plane, each
with one of the 7 materials, constant environment 0.5 plus 4 emissive
spheres -- rendered at 1920x1080, 64 samples per pixel, max depth 8, NEE +
MIS, FP32, PCG32 streams.  One step = one full 64-spp frame (132.7 M samples).

  value      Msamples/s, device-timed with CUDA events around each step's
             pt_render call (scene and BVH resident in HBM; L2 flushed with a
             256 MiB write between steps, outside the timed events)
  e2e        the same metric through the C-ABI with host buffers: per step
             the camera + launch parameters go in from pinned host memory and
             the accumulated frame comes back to pinned host memory
  roofline   closest-hit traversal kernel: algorithmic bytes (wide nodes +
             primitive records fetched + 32 B ray + 16 B hit, from the
             traversal counters of an identical untimed render) / its
             CUDA-event-timed duration, against the measured HBM bandwidth
  cpu_baseline  the CPU oracle (C++ restatement of the reference integrator)
             on all host cores, on a bounded pixel subset of the same frame

The default run also carries the method's other configurations, each
measured on the same GPU after the headline (keys of the same JSON line;
`--headline-only` skips them):
  cornell_256x256_16spp
             Cornell box 256x256, 16 spp, depth 4: Msamples/s and the
             CPU oracle on the same frame
  batch      64 seeded scenes (10k-2M triangles, 256^2-1280x720), 16 spp,
             depth 8: one multi-scene launch per bounce vs 64 serial renders
  dynamic    4.1M triangles jittered per frame, 120 frames: rebuild vs refit
             build ms, traversal Mrays/s, SAH ratio
  denoise    the learned denoiser trained on tracer-rendered pairs (inputs of
             1-128 spp, 4096-spp targets, batch 16; crop and step counts cut
             to fit, as stated in the result), then time-to-RMSE 0.01 at 1080p,
             render + denoise vs plain accumulation, both measured directly

`--impl reference` times the reference's CPU implementation of the path
(the oracle port; the reference's OptiX/DX12 build cannot run here) on the
same workload and metric.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = "{m:.0f}M-triangle displaced-icosphere field ({n} x 5120 tris + 8192 ground tris + 4 sphere lights), " \
           "{w}x{h}, {spp} spp, max depth {d}, NEE+MIS, 7 materials"
METRIC = "Msamples/s at 1080p depth 8 (1 GB300)"
HAIR_WORKLOAD = "{n} strands x 16 points (curve type {t}, radius 0.003) on a head sphere + floor + sphere light, " \
                "{w}x{h}, {spp} spp, max depth {d}, NEE+MIS"
# Options that shape the closest-hit launches: the committed DRAM-traffic
# capture of a workload applies only when these keep their defaults.
CAPTURE_KEYS = ("width", "height", "spp", "depth", "instances", "hair_strands", "hair_type", "bvh_width", "max_leaf",
                "bvh_fast_build", "smem_nodes", "block_size", "wave_spp", "no_material_sort", "autotune")
HAIR_METRIC = "Msamples/s at 1080p depth 8, hair (1 GB300)"


def headline_workload(args) -> str:
    return WORKLOAD.format(m=(args.instances * 5120 + 8192) / 1e6, n=args.instances, w=args.width, h=args.height,
                           spp=args.spp, d=args.depth)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="headline", choices=["headline", "dynamic", "denoise", "batch", "hair"],
                    help="headline: the 1M-triangle 1080p frame; dynamic: 4M jittered triangles, rebuild vs refit; "
                         "hair: cubic B-spline strands on a head, the same 1080p frame measurement")
    ap.add_argument("--hair-strands", type=int, default=50000, help="strands of the hair workload")
    ap.add_argument("--hair-type", type=int, default=2, help="curve type of the hair workload (0..3, PT_CURVE_*)")
    ap.add_argument("--frames", type=int, default=120, help="frames of the dynamic workload")
    ap.add_argument("--batch-scenes", type=int, default=64, help="scenes of the multi-scene workload")
    ap.add_argument("--batch-spp", type=int, default=16)
    ap.add_argument("--dn-pairs", type=int, default=256, help="denoiser training pairs rendered by the tracer "
                    "(the learned-denoiser configuration names 4000; cut to fit the run)")
    ap.add_argument("--dn-target-spp", type=int, default=4096, help="spp of the denoiser training targets")
    ap.add_argument("--dn-noisy-spp", default="1,2,4,8,16,32,64,128",
                    help="spp of the denoiser training inputs: one value or a comma-separated list drawn from per "
                         "pair (inputs of 4 spp alone leave the network at RMSE 0.016 on higher-spp frames: it "
                         "never reaches 0.01)")
    ap.add_argument("--dn-steps", type=int, default=6000, help="denoiser training steps (20k in the stated "
                    "configuration; cut to fit the run)")
    ap.add_argument("--headline-only", action="store_true",
                    help="default workload: skip the Cornell, multi-scene, dynamic and denoiser results")
    ap.add_argument("--dn-batch", type=int, default=16)
    ap.add_argument("--dn-crop", type=int, default=256)
    ap.add_argument("--dn-lr", type=float, default=1e-3)
    ap.add_argument("--dn-ref-spp", type=int, default=4096, help="spp of the 1080p reference image")
    ap.add_argument("--dn-single-pass", action="store_true",
                    help="denoise with one network pass instead of the frame + mirror-image ensemble")
    ap.add_argument("--dn-train-only", action="store_true",
                    help="time denoiser training steps on a seeded random batch (no rendering, no evaluation)")
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--spp", type=int, default=64)
    ap.add_argument("--depth", type=int, default=8)
    ap.add_argument("--instances", type=int, default=200)
    ap.add_argument("--bvh-width", type=int, default=4)
    ap.add_argument("--max-leaf", type=int, default=4)
    ap.add_argument("--bvh-fast-build", action="store_true",
                    help="build the binary tree as a Morton radix tree instead of by PLOC clustering")
    ap.add_argument("--smem-nodes", type=int, default=0)
    ap.add_argument("--block-size", type=int, default=0)
    ap.add_argument("--wave-spp", type=int, default=0)
    ap.add_argument("--no-material-sort", action="store_true", help="shade hits in queue order")
    ap.add_argument("--no-graph", action="store_true", help="launch kernels directly instead of a CUDA graph")
    ap.add_argument("--autotune", action="store_true", help="run pt_autotune at the benchmark's spp before measuring")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    args = ap.parse_args()
    args.at_capture_config = all(getattr(args, k) == ap.get_default(k) for k in CAPTURE_KEYS)
    return args


def replica_throughput(local_ms: float, units_per_rank: float, ws: int, device: str = "cuda"):
    """Whole-job throughput of `ws` independent replicas (one per GPU, each
    processing units_per_rank): all units over the slowest rank's time
    (max over ranks, all-reduced), in millions per second.  Returns
    (value, max_ms)."""
    t_max = float(local_ms)
    if ws > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([t_max], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_max = float(t.item())
    return ws * units_per_rank / (t_max / 1e3) / 1e6, t_max


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic(workload: str = "headline"):
    """DRAM bytes per closest-hit ray, cache hit rates and throughputs of the
    closest-hit kernel from the committed ncu summary of a small case of the
    same workload (profiles/extend_traffic*.json)."""
    p = ROOT / "profiles" / ("extend_traffic.json" if workload == "headline" else f"extend_traffic_{workload}.json")
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            return None
    return None


class ClockSampler:
    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.tmp = None

    def start(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.device), "-lms", "200"], stdout=self.tmp,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.tmp.flush()
        rows = [l.split(",") for l in Path(self.tmp.name).read_text().strip().splitlines() if l.strip()]
        os.unlink(self.tmp.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(scene, spp_seed0: int, seconds: float, depth: int):
    """The oracle on all host cores over growing pixel subsets until about
    `seconds` of work have been timed; Msamples/s."""
    import numpy as np

    import oracle
    from pupiloptixlab_gb300 import abi
    o = oracle.OracleScene(scene, bvh=True)
    npix = scene.width * scene.height
    threads = os.cpu_count() or 1
    p = abi.RenderParams(spp=1, max_depth=depth, seed=spp_seed0, sample_cnt=0, accumulate=1, rng=abi.RNG_PCG32)
    stride = 257
    done, t_total = 0, 0.0
    offset = 0
    while t_total < seconds and offset < stride:
        px = np.arange(offset, npix, stride, dtype=np.uint32)
        t0 = time.perf_counter()
        o.render(p, pixels=px, threads=threads)
        t_total += time.perf_counter() - t0
        done += px.shape[0]
        offset += 1
    return {"value": done / t_total / 1e6, "unit": "Msamples/s", "cores": threads, "kind": "port",
            "sample": f"{done} samples (1 spp on {offset} strided 1/{stride} pixel subsets of the 1920x1080 frame, "
                      f"depth {depth}) in {t_total:.1f} s"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import numpy as np

    import oracle
    from pupiloptixlab_gb300 import abi, scenes
    # the scene's camera from the oracle's own camera arithmetic: this arm never
    # loads the library under test
    with scenes.camera_maker(oracle.camera_make):
        sc = scenes.icosphere_field(args.width, args.height, args.depth, args.instances)
    o = oracle.OracleScene(sc, bvh=True)
    threads = os.cpu_count() or 1
    npix = sc.width * sc.height
    stride = 64
    times, samples = [], []
    for step in range(args.warmup + args.steps):
        px = np.arange(step % stride, npix, stride, dtype=np.uint32)
        p = abi.RenderParams(spp=1, max_depth=args.depth, seed=step, sample_cnt=0, accumulate=1, rng=abi.RNG_PCG32)
        t0 = time.perf_counter()
        o.render(p, pixels=px, threads=threads)
        dt = time.perf_counter() - t0
        if step >= args.warmup:
            times.append(dt)
            samples.append(px.shape[0])
    total_t = sum(times)
    value = sum(samples) / total_t / 1e6
    sample = (f"each step: 1 spp on a strided 1/{stride} pixel subset ({samples[0]} samples) of the "
              f"{args.width}x{args.height} frame, depth {args.depth}")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Msamples/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_t / len(times) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": headline_workload(args), "implementation": "CPU restatement of the reference integrator "
                       "(oracle/pt_oracle.cpp: reference BSDF/emitter/RNG math, host binned-SAH BVH2); the "
                       "reference's OptiX 7.5 / DX12 build is unavailable on this box"},
            "cpu_baseline": {"value": value, "unit": "Msamples/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def dynamic_result(args, ctx) -> dict:
    """Dynamic geometry: 800 displaced icospheres (4.1 M triangles); every
    frame the object-space vertices are the rest positions plus seeded
    N(0, 0.002) noise (seed = frame), then a full rebuild (PLOC clustering, or
    the radix tree with PT_BVH_FAST_BUILD) or a refit of the initial PLOC
    tree, then 4 spp at 1920x1080, depth 6."""
    import numpy as np
    import torch

    from pupiloptixlab_gb300 import abi, scenes
    from pupiloptixlab_gb300.api import GpuScene
    sc = scenes.icosphere_field(args.width, args.height, 6, num_instances=800, seed=1)
    g = GpuScene(ctx, sc, bvh_width=args.bvh_width, max_leaf=args.max_leaf)
    base = torch.from_numpy(np.concatenate([m.positions for m in sc.meshes]).astype(np.float32)).cuda()
    buffers = g.alloc_buffers()
    res = {}
    sah_by_frame = {}
    for mode in ("rebuild", "rebuild_fast", "refit"):
        fl = abi.BVH_FAST_BUILD if mode == "rebuild_fast" else 0
        g.update_all_vertices(base)
        g.build_bvh(args.bvh_width, args.max_leaf, flags=fl)
        build_ms, rays, trace_ms, render_ms, sah = [], 0, 0.0, 0.0, []
        for f in range(args.frames):
            gen = torch.Generator(device="cuda").manual_seed(f)
            jit = base + 0.002 * torch.randn(base.shape, generator=gen, device="cuda")
            g.update_all_vertices(jit)
            st = g.build_bvh(args.bvh_width, args.max_leaf, flags=fl) if mode != "refit" else g.refit()
            build_ms.append(st.build_ms)
            sah.append(st.sah_cost)
            g.render(4, seed=f * 4, rng=abi.RNG_PCG32, max_depth=6, buffers=buffers,
                     flags=abi.RENDER_KERNEL_TIMING | abi.RENDER_COUNTERS)
            rs = g.render_stats()
            rays += rs.extension_rays + rs.shadow_rays
            trace_ms += rs.extend_ms + rs.shadow_ms
            render_ms += rs.render_ms
        res[mode] = {"build_ms_mean": float(np.mean(build_ms)), "build_ms_max": float(np.max(build_ms)),
                     "traversal_mrays_per_s": rays / (trace_ms * 1e-3) / 1e6,
                     "render_ms_per_frame": render_ms / args.frames, "sah_cost_mean": float(np.mean(sah))}
        sah_by_frame[mode] = np.array(sah)
    n_tris = g.num_prims()[0]
    g.close()
    return {"metric": "dynamic geometry: build ms, traversal Mrays/s, SAH refit/rebuild", "unit": "mixed",
            "workload": f"800 displaced icospheres ({n_tris} triangles), per-frame N(0, 0.002) vertex jitter, "
                        f"{args.frames} frames, 4 spp {args.width}x{args.height} depth 6, BVH{args.bvh_width}",
            "frames": args.frames, "rebuild": res["rebuild"], "rebuild_fast": res["rebuild_fast"],
            "refit": res["refit"],
            "sah_ratio_refit_over_rebuild": float(np.mean(sah_by_frame["refit"] / sah_by_frame["rebuild"])),
            "timing": "build: CUDA events inside pt_bvh_build / pt_bvh_refit; traversal: CUDA events around every "
                      "closest-hit and any-hit launch (PT_RENDER_KERNEL_TIMING)",
            "dtype": "f32", "data": "synthetic (seeded procedural scene)"}


def batch_result(args, ctx) -> dict:
    """Multi-scene launches: `--batch-scenes` seeded icosphere fields with
    triangle counts log-uniform in [10k, 2M] and resolutions drawn from
    {256^2, 512^2, 1024^2, 1280x720}, `--batch-spp` spp at depth 8, rendered
    (a) one pt_render call per scene, back to back, and (b) one
    pt_render_batch call; aggregate Msamples/s of both, device-timed."""
    import numpy as np
    import torch

    from pupiloptixlab_gb300 import scenes
    from pupiloptixlab_gb300.api import GpuScene, render_batch, render_batch_stats
    pool = scenes.mesh_pool(32)
    rng = np.random.default_rng(2)
    res = [(256, 256), (512, 512), (1024, 1024), (1280, 720)]
    specs = []
    for k in range(args.batch_scenes):
        tris = float(np.exp(rng.uniform(np.log(1e4), np.log(2e6))))
        inst = max(1, int(round((tris - 8192) / 5120)))
        w, h = res[int(rng.integers(0, len(res)))]
        specs.append((k, inst, w, h))
    gs = [GpuScene(ctx, scenes.pooled_field(1000 + k, inst, w, h, args.depth, pool), bvh_width=args.bvh_width,
                   max_leaf=args.max_leaf) for k, inst, w, h in specs]
    tris = [g.num_prims()[0] for g in gs]
    pixels = sum(g.width * g.height for g in gs)
    samples = pixels * args.batch_spp
    bufs_serial = [g.alloc_buffers() for g in gs]
    bufs_batch = [g.alloc_buffers() for g in gs]
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def serial(seed):
        a, z = ev(), ev()
        a.record()
        for g, b in zip(gs, bufs_serial):
            g.render(spp=args.batch_spp, seed=seed, max_depth=args.depth, buffers=b)
        z.record()
        torch.cuda.synchronize()
        return a.elapsed_time(z)

    def batched(seed):
        a, z = ev(), ev()
        a.record()
        render_batch(ctx, gs, spp=args.batch_spp, seed=seed, max_depth=args.depth, buffers=bufs_batch)
        z.record()
        torch.cuda.synchronize()
        return a.elapsed_time(z)

    for i in range(max(1, args.warmup)):
        serial(i)
        batched(i)
    steps = max(1, min(args.steps, 5))
    t_serial = [serial(100 + i) for i in range(steps)]
    t_batch = [batched(100 + i) for i in range(steps)]
    same = all(torch.equal(a["accum"], b["accum"]) for a, b in zip(bufs_serial, bufs_batch))
    st = render_batch_stats(ctx)
    ms_s, ms_b = statistics.median(t_serial), statistics.median(t_batch)
    for g in gs:
        g.close()
    return {"metric": "multi-scene aggregate Msamples/s (one launch per bounce vs serial renders)",
            "unit": "Msamples/s", "value": samples / (ms_b * 1e-3) / 1e6,
            "serial_value": samples / (ms_s * 1e-3) / 1e6, "speedup_vs_serial": ms_s / ms_b, "ms_batch": ms_b,
            "ms_serial": ms_s, "steps": steps, "images_identical_to_serial": bool(same), "batch_waves": st.waves,
            "batch_kernel_launches": st.kernel_launches, "higher_is_better": True,
            "workload": f"{len(gs)} icosphere fields, {min(tris)}-{max(tris)} triangles (total {sum(tris)}), "
                        f"{pixels} pixels, {args.batch_spp} spp, depth {args.depth}, BVH{args.bvh_width}",
            "dtype": "f32", "data": "synthetic (seeded procedural scenes)"}


def cornell_result(args, ctx) -> dict:
    """The small plain configuration: procedural Cornell box, 256x256, 16 spp,
    max depth 4, PCG32, seed 0 per step; device-timed Msamples/s (CUDA events
    around each pt_render on the launching stream; the whole scene fits in L2,
    which is the configuration as stated), plus the CPU oracle on all host
    cores over the same frame."""
    import torch

    import oracle
    from pupiloptixlab_gb300 import abi, scenes
    from pupiloptixlab_gb300.api import GpuScene
    W = H = 256
    spp, depth = 16, 4
    sc = scenes.cornell_box(W, H, max_depth=depth)
    g = GpuScene(ctx, sc)
    buffers = g.alloc_buffers()
    stream = torch.cuda.current_stream()
    for w in range(max(3, args.warmup)):
        g.render(spp, seed=1000 + w * spp, rng=abi.RNG_PCG32, buffers=buffers)
    torch.cuda.synchronize()
    times = []
    steps = max(5, args.steps)
    for step in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.render(spp, seed=step * spp, rng=abi.RNG_PCG32, buffers=buffers)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    g.close()
    samples = W * H * spp
    out = {"metric": "Msamples/s, Cornell box 256x256 16 spp depth 4", "unit": "Msamples/s",
           "value": samples * steps / (sum(times) * 1e-3) / 1e6, "ms_per_step": sum(times) / steps, "steps": steps,
           "l2": "not flushed: the 34-triangle scene and its 2 MiB of frame buffers stay in L2, as the configuration "
                 "is stated"}
    if not args.no_cpu_baseline:
        o = oracle.OracleScene(sc, bvh=False)
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        o.render(abi.RenderParams(spp=spp, max_depth=depth, seed=0, sample_cnt=0, accumulate=1, rng=abi.RNG_PCG32),
                 threads=threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": samples / dt / 1e6, "unit": "Msamples/s", "cores": threads, "kind": "port",
                               "sample": f"the whole 256x256 16-spp frame ({samples} samples) in {dt:.1f} s"}
    return out


def unet_flops(layers, n: int, h: int, w: int) -> float:
    """Algorithmic FLOPs of one denoiser training step (forward, data and
    weight gradients of the 14 convolutions; 2 FLOPs per multiply-add).
    layers: (cin, cout, offset) per convolution, as pt_denoiser_layer reports."""
    levels = [0, 0, 1, 1, 2, 2, 3, 3, 4, 3, 2, 1, 0, 0]
    tot = 0.0
    for i, ((cin, cout, _), lv) in enumerate(zip(layers, levels)):
        px = n * (h >> lv) * (w >> lv)
        f = 2.0 * 9 * cin * cout * px
        tot += 2 * f if i == 0 else 3 * f  # the first layer needs no data gradient
    return tot


def denoise_result(args, ctx, log) -> dict:
    """Learned denoiser: training pairs rendered by the tracer (seeded
    icosphere-field scenes, random 256^2 views, `--dn-noisy-spp` inputs,
    `--dn-target-spp` targets), Adam training with the library's tcgen05
    kernels (crops flipped / transposed at random each step), then on the
    1080p headline frame the time to reach RMSE 0.01 against a 4,096-spp
    reference, plain accumulation vs render + denoise, each measured
    directly: plain accumulation is rendered at the smallest spp that reaches
    the threshold (found by bisection over renders) and that render is timed;
    render + denoise is timed at each spp of a ladder, with one network pass
    and with the mirror-image ensemble."""
    import numpy as np
    import torch

    from pupiloptixlab_gb300 import abi, scenes
    from pupiloptixlab_gb300.api import GpuScene
    from pupiloptixlab_gb300.denoise_data import render_pairs
    from pupiloptixlab_gb300.denoiser import Denoiser
    noisy = [int(v) for v in str(args.dn_noisy_spp).split(",")]
    inputs, targets, data_info = render_pairs(ctx, args.dn_pairs, crop=args.dn_crop, target_spp=args.dn_target_spp,
                                              noisy_spp=noisy if len(noisy) > 1 else noisy[0], log=log)
    dn = Denoiser(ctx, lr=args.dn_lr, seed=1)
    B, P = args.dn_batch, args.dn_pairs
    inp_buf = torch.empty((B,) + tuple(inputs.shape[1:]), device=inputs.device, dtype=inputs.dtype)
    tgt_buf = torch.empty((B,) + tuple(targets.shape[1:]), device=targets.device, dtype=targets.dtype)
    gen = torch.Generator(device="cpu").manual_seed(5)

    def stage(k):
        """Batch k: B random pairs, each flipped / transposed at random (8 variants)."""
        idx = torch.randint(0, P, (B,), generator=gen)
        mode = int(torch.randint(0, 8, (1,), generator=gen))
        x, y = inputs[idx.to(inputs.device)], targets[idx.to(targets.device)]
        if mode & 1:
            x, y = x.flip(2), y.flip(2)
        if mode & 2:
            x, y = x.flip(1), y.flip(1)
        if mode & 4:
            x, y = x.transpose(1, 2), y.transpose(1, 2)
        inp_buf.copy_(x)
        tgt_buf.copy_(y)

    for i in range(3):  # warm-up (graph capture)
        stage(i)
        dn.train_step(inp_buf, tgt_buf)
    first_loss = dn.read_loss()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    losses, step_ms_sum = [], 0.0
    for k in range(args.dn_steps):
        if k % 250 == 0:  # cosine decay of the Adam step size to 5 % over the run
            dn.set_lr(args.dn_lr * (0.05 + 0.95 * 0.5 * (1.0 + math.cos(math.pi * k / max(args.dn_steps, 1)))))
        stage(k)
        if k % 100 == 0:
            e0.record()
            dn.train_step(inp_buf, tgt_buf)
            e1.record()
            e1.synchronize()
            step_ms_sum += e0.elapsed_time(e1)
        else:
            dn.train_step(inp_buf, tgt_buf)
        if (k + 1) % 500 == 0:
            losses.append((k + 1, dn.read_loss()))
    torch.cuda.synchronize()
    step_ms = step_ms_sum / max(1, (args.dn_steps + 99) // 100)
    flops = unet_flops(dn.layers, B, args.dn_crop, args.dn_crop)
    pk_file = ROOT / "MEASURED_PEAKS.json"
    bf16_peak, bf16_src = (float(json.loads(pk_file.read_text())["bf16_tflops_sustained"]), "measured") \
        if pk_file.exists() else (1700.0, "fallback")
    tf = flops / (step_ms * 1e-3) / 1e12
    log(f"denoiser trained: {args.dn_steps} steps, {step_ms:.3f} ms/step, {tf:.1f} TFLOP/s, losses {losses[-3:]}")
    del inputs, targets

    # evaluation on the 1080p headline frame
    W, H = args.width, args.height
    sc = scenes.icosphere_field(W, H, args.depth)
    g = GpuScene(ctx, sc, bvh_width=args.bvh_width, max_leaf=args.max_leaf)
    flags = abi.RENDER_DROP_NONFINITE
    buf = g.alloc_buffers()

    def timed_render(spp, seed):
        torch.cuda.synchronize()
        a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        g.render(spp=spp, seed=seed, flags=flags, buffers=buf)
        z.record()
        torch.cuda.synchronize()
        return a.elapsed_time(z) * 1e-3

    g.render(spp=8, seed=0, flags=flags, buffers=buf)  # warm-up (graph capture)
    ref_s = timed_render(args.dn_ref_spp, 1 << 22)
    R = buf["accum"][:, :3].clone()
    thr = 0.01

    def rmse(x):
        x = x[:, :3]
        lin = float((x.clamp(0, 1) - R.clamp(0, 1)).pow(2).mean().sqrt())
        lg = float((torch.log1p(x.clamp(min=0)) - torch.log1p(R.clamp(min=0))).pow(2).mean().sqrt())
        return lin, lg

    plain_cache = {}

    def plain(spp):
        if spp not in plain_cache:
            t = timed_render(spp, 0)
            plain_cache[spp] = {"spp": spp, "s": t, "rmse": rmse(buf["accum"])}
        return plain_cache[spp]

    def plain_time_to(k):
        """Smallest spp whose plain render reaches thr in space k, found by
        doubling and then bisection over renders; its measured render time."""
        hi = 1
        while plain(hi)["rmse"][k] > thr:
            if hi >= args.dn_ref_spp // 2:
                return None
            hi *= 2
        lo = hi // 2
        while hi - lo > 1:
            mid = (lo + hi) // 2
            if plain(mid)["rmse"][k] <= thr:
                hi = mid
            else:
                lo = mid
        return plain(hi)

    out = {}
    plain_best = {0: plain_time_to(0), 1: plain_time_to(1)}
    den = []
    ladder = (1, 2, 4, 8, 12, 16, 24, 32, 48, 64, 80, 96, 128, 160, 192, 256)
    for spp in ladder:
        t = timed_render(spp, 0)
        row = {"spp": spp, "render_s": t, "rmse_input": rmse(buf["accum"])}
        for ens, key in ((False, "single"), (True, "ensemble")):
            dn.denoise(buf, W, H, ensemble=ens)  # warm
            o, st, _ = dn.denoise(buf, W, H, ensemble=ens)
            row[key] = {"s": t + st.last_ms * 1e-3, "denoise_ms": st.last_ms, "rmse": rmse(o),
                        "fallback_tiles": st.fallback_tiles, "tiles": st.tiles}
        den.append(row)
        if row["single"]["rmse"][0] <= thr and row["single"]["rmse"][1] <= thr and \
                row["ensemble"]["rmse"][0] <= thr and row["ensemble"]["rmse"][1] <= thr:
            break
    for k, name in ((0, "display_clamped"), (1, "log1p")):
        pb = plain_best[k]
        entry = {"plain_s": pb["s"] if pb else None, "plain_spp": pb["spp"] if pb else None}
        for key in ("single", "ensemble"):
            hits = [(r[key]["s"], r["spp"]) for r in den if r[key]["rmse"][k] <= thr]
            td, sd = min(hits) if hits else (None, None)
            entry[f"{key}_s"] = td
            entry[f"{key}_spp"] = sd
            entry[f"{key}_speedup"] = (pb["s"] / td) if (pb and td) else None
        out[name] = entry
    g.close()
    best = out["display_clamped"]
    return {"metric": "denoiser: time-to-RMSE 0.01 at 1080p, render+denoise vs plain accumulation", "unit": "s",
            "value": best["ensemble_s"], "higher_is_better": False,
            "speedup_single_pass": best["single_speedup"], "speedup_ensemble": best["ensemble_speedup"],
            "time_to_rmse_0.01": out, "rmse_spaces": {"display_clamped": "RGB clamped to [0,1], linear",
                                                      "log1p": "log(1 + RGB)"},
            "reference_image": {"spp": args.dn_ref_spp, "render_s": ref_s},
            "plain_curve": sorted(plain_cache.values(), key=lambda c: c["spp"]), "denoised_curve": den,
            "training": {"data": data_info, "steps": args.dn_steps, "batch": B, "crop": args.dn_crop,
                         "augmentation": "each batch: random pairs, one of 8 flips/transposes",
                         "step_ms": step_ms, "flops_per_step": flops, "tflops": tf,
                         "first_loss": first_loss, "losses": losses,
                         "cut_from_stated": f"{args.dn_pairs} of 4000 crops, {args.dn_steps} of 20000 steps"},
            "roofline": {"bound": "tensor", "achieved": tf, "peak": bf16_peak, "peak_source": bf16_src,
                         "unit": "TFLOP/s", "frac": tf / bf16_peak, "traffic": None,
                         "note": "whole training step (14 convolutions x forward, data and weight gradients, "
                                 "pooling, up-sampling, loss, Adam) over its algorithmic convolution FLOPs; "
                                 "peak = sustained cuBLAS bf16"},
            "workload": f"U-Net 5 levels 32-256 ch, {dn.num_params} params, batch {B} x {args.dn_crop}^2, inputs "
                        f"{args.dn_noisy_spp} spp, targets {args.dn_target_spp} spp; eval on the {W}x{H} icosphere "
                        f"field vs a {args.dn_ref_spp}-spp reference",
            "dtype": "bf16 (fp32 accumulate)", "data": "synthetic (rendered by the tracer from seeded scenes)"}


def run_dynamic(args):
    import torch

    from pupiloptixlab_gb300.api import Context
    torch.cuda.set_device(0)
    print(json.dumps(dynamic_result(args, Context(0))), flush=True)


def run_batch(args):
    import torch

    from pupiloptixlab_gb300.api import Context
    torch.cuda.set_device(0)
    print(json.dumps(batch_result(args, Context(0))), flush=True)


def run_denoise(args):
    import torch

    from pupiloptixlab_gb300.api import Context
    from pupiloptixlab_gb300.denoiser import Denoiser
    torch.cuda.set_device(0)
    ctx = Context(0)
    log = lambda m: print(m, file=sys.stderr, flush=True)  # noqa: E731
    if args.dn_train_only:
        gen = torch.Generator(device="cuda").manual_seed(0)
        shape = (args.dn_batch, args.dn_crop, args.dn_crop)
        inp = torch.rand(*shape, 9, device="cuda", generator=gen).half()
        tgt = torch.rand(*shape, 3, device="cuda", generator=gen)
        dn = Denoiser(ctx, lr=args.dn_lr, seed=1)
        for _ in range(max(args.warmup, 3)):
            dn.train_step(inp, tgt)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.dn_steps):
            dn.train_step(inp, tgt)
        e1.record()
        torch.cuda.synchronize()
        step_ms = e0.elapsed_time(e1) / max(args.dn_steps, 1)
        flops = unet_flops(dn.layers, args.dn_batch, args.dn_crop, args.dn_crop)
        print(json.dumps({"metric": "denoiser training step", "unit": "ms", "value": step_ms,
                          "tflops": flops / (step_ms * 1e-3) / 1e12, "steps": args.dn_steps,
                          "batch": args.dn_batch, "crop": args.dn_crop, "loss": dn.read_loss()}), flush=True)
        return
    print(json.dumps(denoise_result(args, ctx, log)), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "dynamic":
        run_dynamic(args)
        return
    if args.workload == "denoise":
        run_denoise(args)
        return
    if args.workload == "batch":
        run_batch(args)
        return
    ws, rank, local = dist_env()
    import numpy as np
    import torch

    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from pupiloptixlab_gb300 import abi, scenes
    from pupiloptixlab_gb300.api import Context, GpuScene

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    if args.workload == "hair":
        sc = scenes.hair_scene(args.width, args.height, curve_type=args.hair_type, num_strands=args.hair_strands,
                               points=16, radius=0.003, max_depth=args.depth, curl=0.08)
        metric, workload = HAIR_METRIC, HAIR_WORKLOAD.format(n=args.hair_strands, t=args.hair_type, w=args.width,
                                                             h=args.height, spp=args.spp, d=args.depth)
    else:
        sc = scenes.icosphere_field(args.width, args.height, args.depth, args.instances)
        metric, workload = METRIC, headline_workload(args)
    ctx = Context(local)
    g = GpuScene(ctx, sc, bvh_width=args.bvh_width, max_leaf=args.max_leaf, smem_nodes=args.smem_nodes,
                 bvh_flags=abi.BVH_FAST_BUILD if args.bvh_fast_build else 0)
    buffers = g.alloc_buffers()
    tune = None
    if args.autotune:
        t = g.autotune(spp=args.spp, buffers=buffers)
        tune = {"bvh_width": t.bvh_width, "block_size": t.block_size, "wave_paths": t.wave_paths, "trials": t.trials,
                "tuning_msamples_per_s": t.msamples_per_s, "default_msamples_per_s": t.baseline_msamples_per_s}
        args.bvh_width = t.bvh_width
    bst = g.bvh_stats()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    base_flags = (abi.RENDER_NO_MATERIAL_SORT if args.no_material_sort else 0) | (abi.RENDER_NO_GRAPH if args.no_graph else 0)
    kw = dict(rng=abi.RNG_PCG32, block_size=args.block_size, wave_spp=args.wave_spp, buffers=buffers)

    for w in range(args.warmup):
        g.render(args.spp, seed=1000 + w * args.spp, flags=base_flags, **kw)
    torch.cuda.synchronize()
    # identical untimed render with traversal counters (same seeds as step 0)
    g.render(args.spp, seed=0, flags=abi.RENDER_COUNTERS | base_flags, **kw)
    torch.cuda.synchronize()
    cst = g.render_stats()

    clocks = ClockSampler(local)
    stream = torch.cuda.current_stream()
    step_ms, launches = [], 0
    barrier()
    clocks.start()
    for step in range(args.steps):
        flush.fill_(float(step))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.render(args.spp, seed=step * args.spp, flags=base_flags, **kw)
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        launches += g.render_stats().kernel_launches
    barrier()
    clk = clocks.stop()
    # the same steps again with every traversal / shading launch timed by CUDA
    # events on the launching stream (direct launches): durations for the roofline
    ext_ms, ext_launches, sh_ms, shade_ms, timed_ms = 0.0, 0, 0.0, 0.0, []
    for step in range(args.steps):
        flush.fill_(float(step))
        g.render(args.spp, seed=step * args.spp, flags=abi.RENDER_KERNEL_TIMING | base_flags, **kw)
        rs = g.render_stats()
        ext_ms += rs.extend_ms
        ext_launches += rs.extend_launches
        sh_ms += rs.shadow_ms
        shade_ms += rs.shade_ms
        timed_ms.append(rs.render_ms)
    samples_per_step = args.width * args.height * args.spp
    value, t_max = replica_throughput(sum(step_ms), samples_per_step * args.steps, ws, device="cuda")

    e2e = None
    if not args.no_e2e:
        import ctypes as C
        host_frame = torch.empty(args.width * args.height, 4, dtype=torch.float32, pin_memory=True)
        host_cam = torch.empty(32, dtype=torch.float32, pin_memory=True)
        host_cam.numpy()[:] = np.frombuffer(bytes(sc.camera), dtype=np.float32)
        barrier()
        t0 = time.perf_counter()
        for step in range(args.steps):
            cam = abi.CameraDesc.from_buffer_copy(host_cam.numpy().tobytes())  # camera from pinned host memory
            g.set_camera(cam)
            g.render(args.spp, seed=step * args.spp, flags=base_flags, **kw)
            host_frame.copy_(buffers["accum"], non_blocking=True)
            torch.cuda.synchronize()
        barrier()
        t_e2e = time.perf_counter() - t0
        e2e = {"value": ws * samples_per_step * args.steps / t_e2e / 1e6, "unit": "Msamples/s",
               "h2d_bytes_per_step": C.sizeof(abi.CameraDesc) + C.sizeof(abi.RenderParams),
               "d2h_bytes_per_step": host_frame.numel() * 4}

    if rank != 0:
        return
    # algorithmic bytes of the closest-hit kernel (per-ray counters of the identical counting render)
    node_bytes = 96 if args.bvh_width == 8 else 32 * args.bvh_width  # 8-wide nodes are read compressed
    ext_bytes = cst.nodes_visited * node_bytes + cst.prims_tested * 48 + cst.extension_rays * (32 + 16)
    # per launch: one step's algorithmic bytes over that step's closest-hit launches
    launches_per_step = max(1, ext_launches // args.steps)
    per_launch_bytes = ext_bytes / launches_per_step
    avg_launch_s = ext_ms / max(1, ext_launches) * 1e-3
    achieved = per_launch_bytes / avg_launch_s / 1e9 if ext_ms > 0 else None
    peak, peak_kind = measured_peaks()
    traffic = committed_traffic(args.workload) if args.at_capture_config else None
    # DRAM traffic per launch: the small case's DRAM bytes per ray times this
    # workload's closest-hit rays per launch
    traffic_per_launch = (traffic["dram_bytes_per_ray"] * cst.extension_rays / launches_per_step) if traffic else None
    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_baseline(sc, 0, args.cpu_seconds, args.depth)
    line = {
        "metric": metric, "value": value, "unit": "Msamples/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
        "config": {"workload": workload, "width": args.width, "height": args.height, "spp": args.spp,
                   "max_depth": args.depth, "rng": "pcg32", "bvh_width": args.bvh_width, "max_leaf": args.max_leaf,
                   "smem_nodes": args.smem_nodes, "primitives": int(bst.num_prims),
                   "curve_segments_pieces": list(g.num_curves()) if args.workload == "hair" else None,
                   "material_sort": not args.no_material_sort, "autotune": tune, "cuda_graph": not args.no_graph,
                   "l2": "flushed between steps (256 MiB write, outside the timed events)",
                   "parallelism": "replicas only" if ws > 1 else "single GPU"},
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None,
                     "traffic": traffic_per_launch,
                     "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum per closest-hit ray on the "
                                        "2-spp case of this workload (profiles/extend_traffic.json), times this "
                                        "launch's rays") if traffic else None,
                     "kernel": "k_trace_queue closest hit (extend)",
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else
                     "fallback 6.8 TB/s",
                     "algorithmic_bytes_per_ray": ext_bytes / max(1, cst.extension_rays),
                     "dram_bytes_per_ray": traffic["dram_bytes_per_ray"] if traffic else None,
                     "l2_hit_rate_pct": traffic.get("lts_sector_hit_rate_pct") if traffic else None,
                     "l1_hit_rate_pct": traffic.get("l1tex_sector_hit_rate_pct") if traffic else None,
                     "l1_throughput_pct_of_peak": traffic.get("l1tex_throughput_pct_of_peak") if traffic else None,
                     "l2_throughput_pct_of_peak": traffic.get("lts_throughput_pct_of_peak") if traffic else None,
                     "active_lanes_of_32": traffic.get("active_lanes_per_warp_instruction") if traffic else None,
                     "nodes_per_ray": cst.nodes_visited / max(1, cst.extension_rays),
                     "prims_per_ray": cst.prims_tested / max(1, cst.extension_rays),
                     "extend_ms_per_step": ext_ms / args.steps, "shadow_ms_per_step": sh_ms / args.steps,
                     "shade_ms_per_step": shade_ms / args.steps,
                     "timed_launches_ms_per_step": sum(timed_ms) / args.steps},
        "rays_per_step": {"extension": cst.extension_rays, "shadow": cst.shadow_rays,
                          "shadow_nodes_per_ray": cst.shadow_nodes_visited / max(1, cst.shadow_rays),
                          "shadow_prims_per_ray": cst.shadow_prims_tested / max(1, cst.shadow_rays)},
        "bvh": {"nodes": int(bst.num_nodes), "sah_cost": float(bst.sah_cost), "build_ms": float(bst.build_ms),
                "depth": int(bst.max_depth),
                "builder": "ploc" if bst.builder == abi.BVH_BUILDER_PLOC else "radix tree"},
        "cpu_baseline": cpu,
    }
    if ws == 1 and args.workload == "headline" and not args.headline_only:
        # the other configurations of the same method, on the same GPU, after
        # the headline measurement: the small plain case, multi-scene
        # launches, dynamic geometry and the learned denoiser
        g.close()
        del buffers, flush
        torch.cuda.empty_cache()
        log = lambda m: print(m, file=sys.stderr, flush=True)  # noqa: E731
        for key, fn in (("cornell_256x256_16spp", lambda: cornell_result(args, ctx)),
                        ("batch", lambda: batch_result(args, ctx)),
                        ("dynamic", lambda: dynamic_result(args, ctx)),
                        ("denoise", lambda: denoise_result(args, ctx, log))):
            t0 = time.perf_counter()
            try:
                line[key] = fn()
            except Exception as e:  # one failing part must not lose the headline line
                line[key] = {"error": repr(e)}
            line[key]["wall_s"] = time.perf_counter() - t0
            log(f"{key}: done in {line[key]['wall_s']:.1f} s")
            torch.cuda.empty_cache()
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
