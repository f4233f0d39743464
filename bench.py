"""Benchmark of the Lucent GB300 hot path; prints ONE JSON line on rank 0.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Workloads:
  pt       (default) path tracing of the box scene (81,956 triangles) at
           512x512, 16 spp, depth 8: one step = one 16-spp frame; the metric
           is closest-hit rays per second inside the renderer, with spp/s
  closest  random soup, 65,536 triangles, 10^6 rays, seed 0: one step = one
           closest-hit pass over all rays (the reference's intersectBVH)
  adjoint  8 views of workloads.adjoint_scene at 512x512, 32 spp, depth 6:
           one step = forward + path-replay backward of every view; value =
           backward / forward time
  batch    64 scenes of workloads.batch_scene (10^4..2*10^6 triangles,
           256^2..1024^2 pixels), 64 spp, depth 8: one step renders every
           scene as one batch; reports the one-renderer-after-another figure
           beside it and whether both give identical images
  knot     the large-mesh frame: 2,000,000-triangle displaced torus knot at
           1920x1080, depth 12, thin lens, lognormal HDRI with a sun disk:
           one step = --knot-spp samples of the frame (the 256-spp frame's
           rate without rendering all of it); value = spp/s, with closest-hit
           Mrays/s, its roofline and the 5-iteration a-trous time
The default workload's line also carries, in extra.targets, the figures of
the other configurations measured in the same run (large-mesh spp/s, the
adjoint/forward ratio, batched vs per-scene spp/s with identical images);
--no-targets skips them.
Under torchrun (N > 1) every rank runs an independent replica of the same
workload on its own GPU (weak scaling: the work is rays, which need no
exchange); the timed region is bracketed by barriers and the max over ranks
is reported. `--impl reference` times the reference's CPU algorithm (the
oracle's binary64 restatement, all host threads) on the same workload.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MEASURED = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM = 6800.0  # GB/s, used only when MEASURED_PEAKS.json is absent
ALG_BYTES = os.path.join(ROOT, "tests", "golden", "algorithmic_bytes.json")


def peaks():
    if os.path.exists(MEASURED):
        d = json.load(open(MEASURED))
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM, "fallback"


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.p = None
        if self.p is not None:
            # Wait (5 s at most) for nvidia-smi's first sample, taken before the
            # timed region and dropped: its start-up holds the driver for a
            # while and must not fall inside the timed region.
            import threading
            t = threading.Thread(target=self.p.stdout.readline, daemon=True)
            t.start()
            t.join(5.0)
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.p is not None:
            time.sleep(0.25)
            self.p.terminate()
            try:
                out, _ = self.p.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
                out, _ = self.p.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, n in enumerate(names):
                if f[4 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------- closest-hit workload
def setup_closest(args):
    import oracle  # noqa: F401  (not used here; the BVH comes from the GPU builder when available)
    return None


def run_ours_closest(args, rank, world, local):
    import torch
    from lucent_gb300 import DeviceBVH, workloads
    from lucent_gb300 import bvh as B

    torch.cuda.set_device(local)
    pos, rays = workloads.soup_and_rays(seed=0, n_tri=65536, n_rays=1_000_000)
    gb = B.build_bvh(pos)
    dev = DeviceBVH(gb.nodes, gb.tri_indices, pos, gb.node_count)
    n = rays.shape[0]
    rays_d = torch.from_numpy(rays).cuda()
    prim = torch.empty(n, dtype=torch.int32, device="cuda")
    tt, uu, vv = (torch.empty(n, dtype=torch.float32, device="cuda") for _ in range(3))
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step():
        dev.intersect_device(rays_d.data_ptr(), n, prim.data_ptr(), tt.data_ptr(), uu.data_ptr(), vv.data_ptr(),
                             1e-5, math.inf, sp)

    for _ in range(args.warmup):
        step()
    dev.check(sp)
    barrier(world)
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        for k in range(args.steps):
            flush.fill_(float(k))  # evict L2 (256 MB > 129 MB) between timed steps
            evs[k][0].record(stream)
            step()
            evs[k][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    dev.check(sp)
    ms = [a.elapsed_time(b) for a, b in evs]
    dev_s = sum(ms) / 1000.0
    dev_s = max_over_ranks(dev_s, world)
    rays_total = n * args.steps * world
    value = rays_total / dev_s / 1e6

    # End to end through the C ABI with pinned host buffers (copies timed).
    rays_h = torch.from_numpy(rays).pin_memory()
    outs_h = [torch.empty(n, dtype=t).pin_memory() for t in (torch.int32, torch.float32, torch.float32, torch.float32)]
    import ctypes as C
    from lucent_gb300 import _native as N
    L = N.lib()

    def e2e_step():
        N.check(L.lucent_bvh_intersect(dev.handle, C.cast(rays_h.data_ptr(), N.F32P), n, 1e-5, math.inf,
                                       C.cast(outs_h[0].data_ptr(), N.I32P), C.cast(outs_h[1].data_ptr(), N.F32P),
                                       C.cast(outs_h[2].data_ptr(), N.F32P), C.cast(outs_h[3].data_ptr(), N.F32P),
                                       sp))

    for _ in range(max(1, args.warmup)):
        e2e_step()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e = {"value": rays_total / e2e_s / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": int(rays.nbytes),
           "d2h_bytes_per_step": int(n * 16)}

    # Roofline: algorithmic bytes per ray (oracle counts of the reference's GLSL
    # traversal order, committed as a fixture) over the kernel's device time.
    alg = json.load(open(ALG_BYTES))["closest"] if os.path.exists(ALG_BYTES) else None
    peak, which = peaks()
    roof = None
    if alg:
        per_launch = alg["bytes_per_ray"] * n
        achieved = per_launch / (sum(ms) / len(ms) / 1000.0) / 1e9
        roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": NCU_DRAM_BYTES_CLOSEST_LAUNCH,
                "traffic_scope": "DRAM bytes of one launch over the 1e6 rays; ncu capture of this workload "
                                 "summarised in profiles/closest_wide_soup65k_1Mrays.md",
                "peak_source": which, "kernel": "k_closest_wide_t<ApiPolicy> (+ slow path)",
                "bytes_per_ray": alg["bytes_per_ray"]}
    return {
        "metric": "closest-hit Mrays/s (intersectBVH, 65,536-triangle soup, 1e6 rays)",
        "value": round(value, 2), "unit": "Mrays/s", "ms_per_step": round(sum(ms) / len(ms), 4),
        "wall_s": round(wall, 3), "e2e": e2e, "roofline": roof, "clocks": clk.summary(),
        "gpu_launches": 2 * args.steps, "dtype": "f32+f64", "config": CONFIGS["closest"],
    }


def cpu_closest(threads, sample_rays=1_000_000, reps=3):
    import oracle
    from lucent_gb300 import workloads
    pos, rays = workloads.soup_and_rays(seed=0, n_tri=65536, n_rays=sample_rays)
    ob = oracle.build_bvh(pos)
    oracle.intersect_bvh(ob, pos, rays[:10000], threads=threads)
    t0 = time.perf_counter()
    for _ in range(reps):
        oracle.intersect_bvh(ob, pos, rays, threads=threads)
    dt = time.perf_counter() - t0
    return sample_rays * reps / dt / 1e6, "%d rays x %d reps of the same workload" % (sample_rays, reps)


# ----------------------------------------------------------------------------- path-tracing workload
PT_W, PT_H, PT_SPP, PT_DEPTH = 512, 512, 16, 8
CPU_BASELINE_SECONDS = 10.0
# dram__bytes_read.sum + dram__bytes_write.sum of the closest-hit launches,
# from ncu captures of the same workloads (the source is named in each line's
# traffic_scope).
NCU_DRAM_BYTES_PT_FRAME = 553_000_000
NCU_DRAM_BYTES_CLOSEST_LAUNCH = 115_400_000
PT_METRIC = ("closest-hit Mrays/s inside path tracing: box scene (81,956 triangles), 512x512, 16 spp, "
             "max depth 8 (also spp/s)")
CONFIGS = {
    "pt": {"workload": "pt: box scene seed 0 (5 Lambert walls, quad light 15, 2 rotated boxes, "
                       "81,920-triangle icosphere, layered BSDF), 512x512, 16 spp, depth 8, RR from bounce 2",
           "l2": "flushed between timed frames (256 MB write); working set above L2 (0.5 GB of path records per wave)",
           "hit_ids": "bit-exact vs intersectBVH (tMin 1e-6, tMax 1e30)"},
    "closest": {"workload": "closest: random soup 65,536 tris (PCG64 seed 0), 1e6 sphere rays, tMin 1e-5",
                "l2": "flushed between timed steps (256 MB write)", "hit_ids": "bit-exact vs intersectBVH"},
    "knot": {"workload": "knot: torus knot (2,3) 2,000,000 triangles, 3-octave displacement 0.05, 16 materials "
                         "(4 dielectrics, 10% alpha-blended), 1024x512 lognormal HDRI + 0.5 deg sun disk, thin lens "
                         "0.02, 1920x1080, depth 12, a-trous 5 iterations",
             "l2": "working set above L2 (224 MB of triangles and attributes, 1.5 GB of path state)"},
    "build": {"workload": "build: soup_65k (config 1), box_82k (config 2), knot_2m (config 3); maxLeafSize 4, "
                          "12 bins"},
    "adjoint": {"workload": "adjoint: adjoint_scene(0, 6) (81,956 triangles, 33 materials, 256x128 HDRI), "
                            "8 views 512x512 (renderer views sharing one scene), 32 spp forward / 32 replayed, "
                            "depth 6"},
}


def run_ours_pt(args, rank, world, local):
    import ctypes as C

    import torch
    from lucent_gb300 import _native as N
    from lucent_gb300 import workloads as W
    from lucent_gb300 import _native_render as NR
    from lucent_gb300.renderer import Renderer

    torch.cuda.set_device(local)
    r = Renderer(PT_W, PT_H)
    r.settings.max_bounces = PT_DEPTH
    r.load_scene(W.box_scene(0, 6))
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step():
        r.reset()
        r.trace_samples(PT_SPP, sp)

    for k in range(args.warmup):
        flush.fill_(float(k))  # the fill kernel's first launch (module load) stays out of the timed region
        step()
    r.check(sp)
    s0 = r.stats()
    barrier(world)
    torch.cuda.synchronize()
    # One event pair around all K frames: successive frames' waves overlap
    # (pipelined on the renderer's streams), so per-frame intervals would not
    # hold each frame's work; the L2 flushes count inside the timed region.
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        ev0.record(stream)
        for k in range(args.steps):
            flush.fill_(float(k))  # evict L2 (256 MB > 129 MB) between timed frames
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    r.check(sp)
    s1 = r.stats()
    dev_s = max_over_ranks(ev0.elapsed_time(ev1) / 1000.0, world)
    closest = (s1["closest_rays"] - s0["closest_rays"]) * world
    shadow = (s1["shadow_rays"] - s0["shadow_rays"]) * world
    value = closest / dev_s / 1e6
    paths = PT_W * PT_H * PT_SPP * args.steps * world
    spp_per_s = PT_SPP * args.steps / dev_s  # per GPU frame stream; all ranks render the same size
    # Per-phase device time of one frame (events between the renderer's kernels).
    r.set_profiling(True)
    step()
    r.check(sp)
    ph = r.stats()["phase_ms"]
    r.set_profiling(False)

    # End to end through the C ABI with host buffers: camera and settings from
    # host structs, trace, colour target (512 x 512 x RGBA32F) back to pinned
    # host memory, one buffer per frame (the asynchronous readback), every
    # copy finished inside the timed region.
    L = N.lib()
    outs = [torch.empty(PT_W * PT_H * 4, dtype=torch.float32).pin_memory() for _ in range(args.steps)]
    cam = r.camera_state
    settings = NR.SettingsDesc(PT_DEPTH, r.settings.firefly_clamp)

    def e2e_step(out):
        N.check(L.lucent_renderer_upload_camera(r.handle, C.byref(cam)))
        N.check(L.lucent_renderer_apply_settings(r.handle, C.byref(settings)))
        N.check(L.lucent_renderer_trace(r.handle, PT_SPP, sp))
        N.check(L.lucent_renderer_read_color_async(r.handle, C.cast(out.data_ptr(), N.F32P), sp))

    for _ in range(max(1, args.warmup)):
        e2e_step(outs[0])
    N.check(L.lucent_renderer_check(r.handle, sp))
    barrier(world)
    t0 = time.perf_counter()
    for k in range(args.steps):
        e2e_step(outs[k])
    N.check(L.lucent_renderer_check(r.handle, sp))
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    per_frame_closest = closest / (args.steps * world)
    e2e = {"value": round(per_frame_closest * args.steps * world / e2e_s / 1e6, 2), "unit": "Mrays/s",
           "h2d_bytes_per_step": C.sizeof(cam) + C.sizeof(settings), "d2h_bytes_per_step": PT_W * PT_H * 16,
           "spp_per_s": round(PT_SPP * args.steps / e2e_s, 2)}

    alg = json.load(open(ALG_BYTES)).get("pt_box") if os.path.exists(ALG_BYTES) else None
    peak, which = peaks()
    roof = None
    if alg and ph.get("closest"):
        per_frame = alg["bytes_per_closest_ray"] * per_frame_closest
        achieved = per_frame / (ph["closest"] / 1000.0) / 1e9
        roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": NCU_DRAM_BYTES_PT_FRAME,
                "traffic_scope": "DRAM bytes of the frame's 9 closest-hit launches, like achieved; ncu capture of "
                                 "this workload summarised in profiles/closest_pt_box512_16spp.md",
                "peak_source": which, "kernel": "k_closest_wide_t<PathClosestMulti> (+ slow path)",
                "bytes_per_closest_ray": alg["bytes_per_closest_ray"],
                "closest_ms_per_frame": round(ph["closest"], 3)}
    # Kernels launched in the timed frames, as the renderer counts them (reset + trace: camera, 7 per bounce,
    # a counter reset per forked bounce, 3 per ray sort, accumulate, seed advance).
    launches = s1["kernel_launches"] - s0["kernel_launches"]
    r.dispose()
    extra = {"mpaths_per_s": round(paths / dev_s / 1e6, 2), "shadow_mrays_per_s": round(shadow / dev_s / 1e6, 2),
             "closest_rays_per_frame": int(per_frame_closest),
             "phase_ms_per_frame": {k: round(v, 3) for k, v in ph.items()}}
    if args.targets and world == 1:
        extra["targets"] = run_targets(args, local)
    return {
        "metric": PT_METRIC, "value": round(value, 2), "unit": "Mrays/s", "ms_per_step": round(1e3 * dev_s / args.steps, 4),
        "wall_s": round(wall, 3), "e2e": e2e, "roofline": roof, "clocks": clk.summary(),
        "gpu_launches": int(launches), "dtype": "f32 (+f64 exact hit decisions)",
        "spp_per_s": round(spp_per_s, 2), "extra": extra,
        "config": CONFIGS["pt"],
    }


def cpu_pt(threads, reps=1, crop=512):
    """The oracle (C++ restatement of trace.frag with the binary64 intersectBVH
    restatement) on a centred crop of the same frame; closest-hit rays it traced
    per second."""
    from oracle import render as R
    from lucent_gb300 import workloads as W
    prep = R.prepare(W.box_scene(0, 6))
    x0 = (PT_W - crop) // 2
    crop_box = (x0, x0, crop, crop)
    R.render_work(prep, PT_W, PT_H, 0, 1, max_bounces=PT_DEPTH, crop=(x0, x0, 16, 16), threads=threads,
                  detailed=False)
    t0 = time.perf_counter()
    rays = 0
    for _ in range(reps):
        w = R.render_work(prep, PT_W, PT_H, 0, PT_SPP, max_bounces=PT_DEPTH, crop=crop_box, threads=threads,
                          detailed=False)
        rays += w["closest_rays"]
    dt = time.perf_counter() - t0
    return rays / dt / 1e6, "%dx%d centre crop of the 512x512 frame, 16 spp x %d reps" % (crop, crop, reps)


# ----------------------------------------------------------------------------- BVH build workload
def _build_meshes():
    """Positions of the configurations' meshes: config 1's soup (65,536
    triangles), config 2's box scene (81,956) and config 3's displaced knot
    (2,000,000)."""
    from lucent_gb300 import scene as S
    from lucent_gb300 import workloads as W
    soup, _ = W.soup_and_rays(seed=0, n_tri=65536, n_rays=1)
    return {"soup_65k": soup, "box_82k": S.pack_scene(W.box_scene(0, 6)).positions,
            "knot_2m": W.knot_mesh(0).positions}


def run_ours_build(args, rank, world, local):
    """buildBVH on the GPU (lucent_bvh_build_device from device-resident
    positions; the build is synchronous and includes its host steps). One
    step = one build of each mesh; value = triangles per second over the
    three. Also the reference-facing call (lucent_bvh_build: host positions
    in, the reference's node array and triIndices out) per mesh."""
    import torch
    from lucent_gb300 import bvh as B
    torch.cuda.set_device(local)
    meshes = _build_meshes()
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in meshes.items()}
    for k in meshes:  # warm-up
        for _ in range(max(1, args.warmup)):
            B.build_device(dev[k].data_ptr(), meshes[k].size // 9).close()
    torch.cuda.synchronize()
    per = {k: [] for k in meshes}
    with Clocks(local) as clk:
        for _ in range(args.steps):
            for k in meshes:
                t0 = time.perf_counter()
                B.build_device(dev[k].data_ptr(), meshes[k].size // 9).close()
                per[k].append(time.perf_counter() - t0)
    e2e = {}
    for k, v in meshes.items():
        t0 = time.perf_counter()
        b = B.build_bvh(v)
        e2e[k] = time.perf_counter() - t0
        b._device.close()
    tris = sum(v.size // 9 for v in meshes.values())
    total = max_over_ranks(sum(min(x) for x in per.values()), world)
    return {
        "metric": "GPU BVH build Mtris/s (buildBVH, bit-exact nodes): configs 1-3 meshes (65,536 / 81,956 / "
                  "2,000,000 triangles)",
        "value": round(tris * world / total / 1e6, 3), "unit": "Mtris/s", "ms_per_step": round(1e3 * total, 3),
        "higher_is_better": True,
        "e2e": {"value": round(tris / sum(e2e.values()) / 1e6, 3), "unit": "Mtris/s",
                "h2d_bytes_per_step": int(sum(v.nbytes for v in meshes.values())),
                "d2h_bytes_per_step": int(sum((2 * (v.size // 9) - 1) * 32 + (v.size // 9) * 4
                                              for v in meshes.values()))},
        "roofline": None, "clocks": clk.summary(), "gpu_launches": None, "dtype": "f32 data, f64 decisions",
        "config": CONFIGS["build"],
        "extra": {"build_ms": {k: round(1e3 * min(v), 3) for k, v in per.items()},
                  "reference_call_ms": {k: round(1e3 * v, 3) for k, v in e2e.items()}},
    }


def cpu_build(threads, reps=1):
    """The oracle's buildBVH (single-threaded, like the reference) on the same meshes."""
    import oracle
    global _BUILD_MESHES
    if _BUILD_MESHES is None:
        _BUILD_MESHES = _build_meshes()
    t0 = time.perf_counter()
    tris = 0
    for _ in range(reps):
        for v in _BUILD_MESHES.values():
            oracle.build_bvh(v)
            tris += v.size // 9
    dt = time.perf_counter() - t0
    return tris / dt / 1e6, "the three meshes x %d reps, one thread (the reference builds on one worker)" % reps


_BUILD_MESHES = None


def cpu_build_ms():
    """Per-mesh single-thread oracle build time (ms)."""
    import oracle
    global _BUILD_MESHES
    if _BUILD_MESHES is None:
        _BUILD_MESHES = _build_meshes()
    out = {}
    for k, v in _BUILD_MESHES.items():
        t0 = time.perf_counter()
        oracle.build_bvh(v)
        out[k] = round(1e3 * (time.perf_counter() - t0), 2)
    return out


def env_sampler_times(local, reps=5):
    """buildEnvSampler on the large-mesh workload's 1024 x 512 HDRI: the host
    build (lucent_env_sampler, which upload_lighting runs) against the GPU
    build (lucent_env_sampler_device from a device copy of the map)."""
    import ctypes as C

    import torch
    from lucent_gb300 import _native as N
    from lucent_gb300 import workloads as W
    torch.cuda.set_device(local)
    img = W.knot_scene(0, tubular=8, radial=4, env_width=1024).env.map
    rgb = np.ascontiguousarray(img.data, np.float32)
    L = N.lib()
    gw, gh, tot = C.c_uint32(), C.c_uint32(), C.c_double()
    table = np.zeros(1024 * 512 * 4, np.float32)
    d_rgb = torch.from_numpy(rgb).cuda()
    d_tab = torch.zeros(1024 * 512 * 4, dtype=torch.float32, device="cuda")

    def host():
        N.check(L.lucent_env_sampler(N.ptr(rgb, C.c_float), img.width, img.height, 1024, C.byref(gw), C.byref(gh),
                                     N.ptr(table, C.c_float), C.byref(tot)))

    def device():
        N.check(L.lucent_env_sampler_device(d_rgb.data_ptr(), img.width, img.height, 1024, C.byref(gw),
                                            C.byref(gh), d_tab.data_ptr(), C.byref(tot), None))

    out = {}
    for name, fn in (("host_ms", host), ("gpu_ms", device)):
        fn()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        out[name] = round(1e3 * min(ts), 3)
    out["cells"] = int(gw.value * gh.value)
    return out


# ----------------------------------------------------------------------------- large-mesh workload
KNOT_W, KNOT_H, KNOT_DEPTH, KNOT_ATROUS = 1920, 1080, 12, 5


def run_ours_knot(args, rank, world, local):
    """The large-mesh frame (workloads.knot_scene(0): 2,000,000 triangles at
    1920x1080, depth 12). One step = --knot-spp samples of the frame traced
    through the renderer (the full frame has 256); value = samples per second
    of the whole frame. Also: closest-hit Mrays/s, the closest-hit roofline
    (oracle bytes per ray of this scene over the phase's device time), and
    the 5-iteration a-trous denoiser plus display pass at this size."""
    import ctypes as C

    import torch
    from lucent_gb300 import _native as N
    from lucent_gb300 import workloads as W
    from lucent_gb300.renderer import Renderer
    torch.cuda.set_device(local)
    spp = args.knot_spp
    t0 = time.perf_counter()
    sc = W.knot_scene(0)
    t1 = time.perf_counter()
    r = Renderer(KNOT_W, KNOT_H)
    r.settings.max_bounces = KNOT_DEPTH
    r.load_scene(sc)
    torch.cuda.synchronize()
    load_s = time.perf_counter() - t1
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream

    def step():
        r.reset()
        r.trace_samples(spp, sp)

    for _ in range(args.warmup):
        step()
    r.check(sp)
    s0 = r.stats()
    barrier(world)
    torch.cuda.synchronize()
    # one event pair around all steps: the waves of successive steps overlap (pipelined)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        ev0.record(stream)
        for k in range(args.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
    r.check(sp)
    s1 = r.stats()
    dev_s = max_over_ranks(ev0.elapsed_time(ev1) / 1000.0, world)
    closest = (s1["closest_rays"] - s0["closest_rays"]) * world
    value = spp * args.steps * world / dev_s
    r.set_profiling(True)
    step()
    r.check(sp)
    ph = r.stats()["phase_ms"]
    per_frame_closest = (r.stats()["closest_rays"] - s1["closest_rays"])
    r.set_profiling(False)
    # denoiser (variance + 5 a-trous iterations, as the workload fixes) on the accumulated frame
    dn = []
    for _ in range(4):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r.denoise(levels=KNOT_ATROUS, stream=sp)
        e1.record(stream)
        torch.cuda.synchronize()
        dn.append(e0.elapsed_time(e1))
    # end to end: camera and settings from host structs, trace, denoise, display to RGBA8 host memory
    L = N.lib()
    out8 = torch.empty(KNOT_W * KNOT_H * 4, dtype=torch.uint8).pin_memory()
    cam = r.camera_state
    from lucent_gb300 import _native_render as NR
    settings = NR.SettingsDesc(KNOT_DEPTH, r.settings.firefly_clamp)

    def e2e_step():
        N.check(L.lucent_renderer_upload_camera(r.handle, C.byref(cam)))
        N.check(L.lucent_renderer_apply_settings(r.handle, C.byref(settings)))
        N.check(L.lucent_renderer_trace(r.handle, spp, sp))
        N.check(L.lucent_renderer_denoise(r.handle, KNOT_ATROUS, 4.0, 64.0, 1.5, sp))
        N.check(L.lucent_renderer_display(r.handle, 1.0, 0, 1.0, C.cast(out8.data_ptr(), N.U8P), None, sp))

    e2e_step()
    torch.cuda.synchronize()
    t0e = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0e, world)
    alg = json.load(open(ALG_BYTES)).get("pt_knot") if os.path.exists(ALG_BYTES) else None
    peak, which = peaks()
    roof = None
    if alg and ph.get("closest"):
        per_frame = alg["bytes_per_closest_ray"] * per_frame_closest
        achieved = per_frame / (ph["closest"] / 1000.0) / 1e9
        roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": None,
                "traffic_scope": "not captured for this workload",
                "peak_source": which, "kernel": "k_closest_wide_t<PathClosestMulti> (+ slow path)",
                "bytes_per_closest_ray": alg["bytes_per_closest_ray"],
                "closest_ms_per_step": round(ph["closest"], 3)}
    r.dispose()
    return {
        "metric": "large-mesh spp/s: 2,000,000-triangle knot, 1920x1080, depth 12 (closest-hit Mrays/s beside it)",
        "value": round(value, 3), "unit": "spp/s", "ms_per_step": round(1e3 * dev_s / args.steps, 3),
        "e2e": {"value": round(spp * args.steps * world / e2e_s, 3), "unit": "spp/s",
                "h2d_bytes_per_step": C.sizeof(cam) + C.sizeof(settings),
                "d2h_bytes_per_step": KNOT_W * KNOT_H * 4,
                "includes": "trace, 5 a-trous iterations, display, RGBA8 read-back"},
        "roofline": roof, "clocks": clk.summary(),
        "gpu_launches": int(s1["kernel_launches"] - s0["kernel_launches"]), "dtype": "f32 (+f64 exact hit decisions)",
        "config": CONFIGS["knot"],
        "extra": {"closest_mrays_per_s": round(closest / dev_s / 1e6, 2), "spp_per_step": spp,
                  "frame_256spp_s_projected": round(256 / value, 3),
                  "denoise_atrous5_ms": round(float(np.median(dn)), 3),
                  "phase_ms_per_step": {k: round(v, 3) for k, v in ph.items()},
                  "scene_generate_s": round(t1 - t0, 2), "scene_load_s": round(load_s, 2)},
    }


def cpu_knot(threads, reps=1, crop=32):
    """Oracle on a crop x crop window at the frame centre, 1 spp: closest-hit rays per second."""
    from oracle import render as R
    from lucent_gb300 import workloads as W
    global _KNOT_PREP
    if _KNOT_PREP is None:
        _KNOT_PREP = R.prepare(W.knot_scene(0))
    x0, y0 = (KNOT_W - crop) // 2, (KNOT_H - crop) // 2
    t0 = time.perf_counter()
    px = 0
    for _ in range(reps):
        R.render(_KNOT_PREP, KNOT_W, KNOT_H, 0, 1, max_bounces=KNOT_DEPTH, crop=(x0, y0, crop, crop),
                 threads=threads)
        px += crop * crop
    dt = time.perf_counter() - t0
    # pixel-samples per second over the frame's pixels = frame samples per second
    return px / dt / (KNOT_W * KNOT_H), "%dx%d centre crop of the 1920x1080 frame, 1 spp x %d reps" % (
        crop, crop, reps)


_KNOT_PREP = None


def run_targets(args, local):
    """The other configurations, measured after the default workload in the
    same run: each a bounded run of its own workload (one timed step after
    one warm-up, or a few samples of a frame)."""
    import types
    out = {}
    out["env_sampler"] = env_sampler_times(local)
    t0 = time.perf_counter()
    c = run_ours_closest(types.SimpleNamespace(steps=5, warmup=3), 0, 1, local)
    out["bvh_closest"] = {"mrays_per_s": c["value"], "ms_per_1m_rays": c["ms_per_step"],
                          "e2e_mrays_per_s": c["e2e"]["value"],
                          "roofline_frac": c["roofline"]["frac"] if c["roofline"] else None,
                          "config": c["config"]["workload"], "clocks": c["clocks"],
                          "wall_s": round(time.perf_counter() - t0, 1)}
    t0 = time.perf_counter()
    bb = run_ours_build(types.SimpleNamespace(steps=3, warmup=1), 0, 1, local)
    out["bvh_build"] = {"gpu_ms": bb["extra"]["build_ms"], "reference_call_ms": bb["extra"]["reference_call_ms"],
                        "cpu_oracle_single_thread_ms": cpu_build_ms(),
                        "wall_s": round(time.perf_counter() - t0, 1)}
    t0 = time.perf_counter()
    k = run_ours_knot(types.SimpleNamespace(steps=2, warmup=1, knot_spp=args.knot_spp), 0, 1, local)
    out["large_mesh"] = {"spp_per_s": k["value"], "closest_mrays_per_s": k["extra"]["closest_mrays_per_s"],
                         "roofline_frac": k["roofline"]["frac"] if k["roofline"] else None,
                         "roofline_achieved_gbs": k["roofline"]["achieved"] if k["roofline"] else None,
                         "denoise_atrous5_ms": k["extra"]["denoise_atrous5_ms"],
                         "e2e_spp_per_s": k["e2e"]["value"], "spp_per_step": args.knot_spp, "clocks": k["clocks"],
                         "wall_s": round(time.perf_counter() - t0, 1)}
    t0 = time.perf_counter()
    a = run_ours_adjoint(types.SimpleNamespace(steps=1, warmup=1), 0, 1, local)
    bf = a["extra"]["batched_forward"]
    out["adjoint"] = {"backward_over_forward": a["value"], "target": "<= 3",
                      "forward_ms_per_view": a["extra"]["forward_ms_per_view"],
                      "backward_ms_per_view": a["extra"]["backward_ms_per_view"],
                      "batched_over_sequential_32spp": bf["32_spp_per_call"]["batched_over_sequential"],
                      "batched_over_sequential_1spp": bf["1_spp_per_call"]["batched_over_sequential"],
                      "batched_over_pipelined_renderers_32spp":
                          bf["32_spp_per_call"]["batched_over_pipelined_renderers"],
                      "batched_over_pipelined_renderers_1spp": bf["1_spp_per_call"]["batched_over_pipelined_renderers"],
                      "clocks": a["clocks"], "wall_s": round(time.perf_counter() - t0, 1)}
    t0 = time.perf_counter()
    # The autotuner's choice on this workload (waves of 8 consecutive scenes,
    # two parts on two streams, measured with the full autotune of
    # `--workload batch`), so this bounded run skips the tuning itself.
    b = run_ours_batch(types.SimpleNamespace(steps=1, warmup=1, batch_scenes=64,
                                             batch_options={"scenes_per_wave": 8, "streams": 2, "top_levels": False}),
                       0, 1, local)
    out["batch"] = {"batched_mpaths_per_s": b["value"], "sequential_mpaths_per_s": b["extra"]["sequential_mpaths_per_s"],
                    "batched_over_sequential": b["extra"]["batched_over_sequential"], "target": ">= 2",
                    "identical_images": b["extra"]["identical_images"], "tuned_options": b["extra"]["tuned_options"],
                    "scenes": 64, "config": b["config"]["workload"], "clocks": b["clocks"],
                    "setup_s": b["extra"]["setup_s"], "wall_s": round(time.perf_counter() - t0, 1)}
    return out


# ----------------------------------------------------------------------------- batch workload
BATCH_SPP, BATCH_DEPTH = 64, 8


def _batch_setup(n, timing=None):
    """Renderers for batch scenes 0..n-1; `timing` collects seconds spent
    generating the synthetic scenes ("generate") and loading them through
    the C ABI ("load": packing, GPU BVH build, wide view, upload, lighting)."""
    import torch
    from lucent_gb300 import workloads as W
    from lucent_gb300.renderer import Renderer
    timing = {} if timing is None else timing
    timing.setdefault("generate", 0.0)
    timing.setdefault("load", 0.0)
    rs = []
    t0 = time.perf_counter()
    scenes = _generate_batch_scenes(n)
    timing["generate"] += time.perf_counter() - t0
    for seed in range(n):
        sc, res = scenes[seed]
        scenes[seed] = None
        t1 = time.perf_counter()
        r = Renderer(res, res)
        r.settings.max_bounces = BATCH_DEPTH
        r.load_scene(sc)
        torch.cuda.synchronize()
        timing["load"] += time.perf_counter() - t1
        rs.append(r)
    return rs


def _generate_batch_scenes(n):
    """workloads.batch_scene(0 .. n-1), generated by a pool of spawned
    processes (host-only work; spawn, never fork, once CUDA is initialised)."""
    import concurrent.futures as cf
    import multiprocessing as mp
    from lucent_gb300 import workloads as W
    workers = min(n, max(1, (os.cpu_count() or 1)))
    if workers <= 1:
        return [W.batch_scene(seed) for seed in range(n)]
    with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        return list(ex.map(W.batch_scene, range(n)))


def _image_digest(r):
    import hashlib
    col, alb, nrm, hist = r.read()
    h = hashlib.sha1()
    for a in (col, alb, nrm, hist):
        h.update(a.tobytes())
    return h.hexdigest()


def run_ours_batch(args, rank, world, local):
    """Many scenes: `--batch-scenes` seeded scenes of workloads.batch_scene
    (triangles log-uniform in [1e4, 2e6], resolutions from {256..1024}^2,
    512x256 HDRIs), 64 spp each, depth 8. One step renders every scene once
    (a) one renderer after another and (b) as one batch (autotuned wave size,
    captured waves); value = batched Mpaths/s, with the sequential figure
    and a check that both produce the same images bit for bit."""
    import torch
    from lucent_gb300.renderer import Batch
    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    t_setup = time.perf_counter()
    setup_t = {}
    rs = _batch_setup(args.batch_scenes, setup_t)
    setup_s = time.perf_counter() - t_setup
    px = sum(r.width * r.height for r in rs)
    tris = sum(r.stats()["triangles"] for r in rs)
    paths_per_step = px * BATCH_SPP

    def seq_step(digests=None):
        ms = 0.0
        for i, r in enumerate(rs):
            r.reset()
            r.set_seed(1000)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r.trace_samples(BATCH_SPP, sp)
            e1.record(stream)
            r.check(sp)
            ms += e0.elapsed_time(e1)
            if digests is not None:
                digests.append(_image_digest(r))
            r.trim()
        return ms

    b = Batch(rs)
    for r in rs:  # allocate each renderer's buffers once, outside the timed steps
        r.trace_samples(1, sp)
        r.check(sp)
        r.trim()
    if getattr(args, "batch_options", None):
        # fixed options (the autotuner's choice on this workload), for bounded runs
        b.set_options(**args.batch_options)
        tuned, trials = dict(args.batch_options), {}
    else:
        tuned, trials = b.autotune(samples=8)
    barrier(world)
    torch.cuda.synchronize()
    for _ in range(args.warmup):
        seq_step()
    seq_ms, digests = [], []
    for k in range(args.steps):
        seq_ms.append(seq_step(digests if k == 0 else None))

    def batch_step():
        for r in rs:
            r.reset()
            r.set_seed(1000)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.trace_samples(BATCH_SPP, sp)
        e1.record(stream)
        st = b.check(sp)
        return e0.elapsed_time(e1), st

    st0 = b.check(sp)
    for _ in range(args.warmup):
        _, st0 = batch_step()
    with Clocks(local) as clk:
        bat = [batch_step() for _ in range(args.steps)]
    launches = bat[-1][1]["kernel_launches"] - st0["kernel_launches"] if bat else 0
    bat_ms = [m for m, _ in bat]
    same = all(_image_digest(r) == d for r, d in zip(rs, digests))
    # end to end: the batched call plus every image read back to host memory
    t0 = time.perf_counter()
    _, st = batch_step()
    for r in rs:
        r.read()
    e2e_s = time.perf_counter() - t0
    dev_b = max_over_ranks(sum(bat_ms) / 1000.0, world)
    dev_s = max_over_ranks(sum(seq_ms) / 1000.0, world)
    value = paths_per_step * args.steps * world / dev_b / 1e6
    seq_value = paths_per_step * args.steps * world / dev_s / 1e6
    return {
        "metric": "batched path-tracing Mpaths/s: %d scenes (workloads.batch_scene seeds 0..%d), %d spp, depth %d"
                  % (len(rs), len(rs) - 1, BATCH_SPP, BATCH_DEPTH),
        "value": round(value, 2), "unit": "Mpaths/s", "ms_per_step": round(sum(bat_ms) / len(bat_ms), 3),
        "e2e": {"value": round(paths_per_step * world / e2e_s / 1e6, 2), "unit": "Mpaths/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": px * 52},
        "roofline": None, "clocks": clk.summary(), "gpu_launches": int(launches),
        "dtype": "f32 (+f64 exact hit decisions)",
        "config": {"workload": "batch: %d scenes, %d triangles, %d pixels, %d spp, depth %d" % (
            len(rs), tris, px, BATCH_SPP, BATCH_DEPTH), "l2": "working set far above L2 (>10 GB of path state)"},
        "extra": {"sequential_mpaths_per_s": round(seq_value, 2), "batched_over_sequential": round(dev_s / dev_b, 3),
                  "identical_images": bool(same), "tuned_options": tuned,
                  "autotune_trials_s": {str(k): round(v, 4) for k, v in trials.items()},
                  "waves_per_step": st["waves"] // max(1, args.steps + args.warmup + 1), "setup_s": round(setup_s, 1),
                  "generate_s": round(setup_t["generate"], 2), "load_s": round(setup_t["load"], 2),
                  "load_ms_per_scene": round(1e3 * setup_t["load"] / len(rs), 1)},
    }


def cpu_batch(threads, reps=1, crop=16):
    """Oracle on a crop x crop window at the centre of the first 4 batch scenes, 64 spp."""
    from lucent_gb300 import workloads as W
    from oracle import render as R
    paths, dt = 0, 0.0
    for seed in range(4):
        sc, res = W.batch_scene(seed)
        prep = R.prepare(sc)
        x0 = (res - crop) // 2
        t0 = time.perf_counter()
        for _ in range(reps):
            R.render(prep, res, res, 1000, BATCH_SPP, max_bounces=BATCH_DEPTH, crop=(x0, x0, crop, crop),
                     threads=threads)
        dt += time.perf_counter() - t0
        paths += crop * crop * BATCH_SPP * reps
    return paths / dt / 1e6, "%dx%d centre crops of batch scenes 0-3, %d spp" % (crop, crop, BATCH_SPP)


# ----------------------------------------------------------------------------- adjoint workload
ADJ_W, ADJ_SPP, ADJ_DEPTH, ADJ_VIEWS = 512, 32, 6, 8
ADJ_METRIC = "adjoint/forward time ratio: path-replay backward vs forward, 8 views 512x512, 32 spp, depth 6"


def run_ours_adjoint(args, rank, world, local):
    """Inverse rendering: workloads.adjoint_scene (the box scene's geometry,
    32 materials, 256x128 HDRI) seen from 8 views at 512x512, depth 6. One
    step = one optimisation iteration (inverse.InverseRendering): 32-spp
    forward renders of the views and the 32-spp path-replay backward of each
    against the L2 image loss, one all-reduce of the 98,503-value gradient
    vector over the ranks (views are sharded v % world), one Adam step on
    materials and environment. value = backward / forward time ratio. Also
    times this rank's forward views as one batch vs one by one, at 32 spp per
    call and at 1 spp per call (progressive)."""
    import torch
    from lucent_gb300 import adjoint as AD
    from lucent_gb300 import inverse as INV
    from lucent_gb300 import workloads as W
    from lucent_gb300.renderer import Batch, Renderer
    from lucent_gb300 import scene as S
    torch.cuda.set_device(local)
    sc = W.adjoint_scene(0, 6)
    mine = INV.views_of_rank(ADJ_VIEWS, rank, world)
    cams = W.adjoint_views(ADJ_VIEWS)
    views = []
    for v in mine:  # the first renderer loads the scene, the others are views of it (shared device data)
        if not views:
            r = Renderer(ADJ_W, ADJ_W)
            r.load_scene(S.Scene(name=sc.name, camera=cams[v], env=sc.env, meshes=sc.meshes))
        else:
            r = Renderer.view(views[0].renderer, ADJ_W, ADJ_W, camera=cams[v])
        r.settings.max_bounces = ADJ_DEPTH
        r.apply_settings()
        views.append(INV.RendererView(r, AD.forward(r, ADJ_SPP, 0), ADJ_SPP, 1))
    rs = [v.renderer for v in views]
    rng = np.random.default_rng(0)
    gt = AD.get_params(rs[0].packed.materials)
    theta = np.clip(gt + rng.normal(0, 0.1, gt.shape), 0, 1)
    env_gt = sc.env.map.data.reshape(sc.env.map.height, sc.env.map.width, 3).astype(np.float64)
    env = np.maximum(env_gt + rng.normal(0, 0.1, env_gt.shape), 0)
    reduce = INV.TorchAllReduce(device="cuda:%d" % local) if world > 1 else None
    opt = INV.InverseRendering(views, theta, env, reduce=reduce)

    for _ in range(args.warmup):
        opt.step()
    for v in views:
        v.timing = dict.fromkeys(v.timing, 0.0)
    opt.timing = dict.fromkeys(opt.timing, 0.0)
    barrier(world)
    with Clocks(local) as clk:
        for _ in range(args.steps):
            opt.step()
    barrier(world)
    tf = max_over_ranks(sum(v.timing["forward"] for v in views), world)
    tb = max_over_ranks(sum(v.timing["backward"] for v in views), world)
    tu = max_over_ranks(sum(v.timing["upload"] for v in views) + opt.timing["update"], world)
    tr = max_over_ranks(opt.timing["reduce"], world)
    paths = len(views) * ADJ_W * ADJ_W * ADJ_SPP * args.steps

    # forward of the 8 views: one batch vs one renderer after another
    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    b = Batch(rs, use_graph=True)

    def seq(spp, calls):
        for _ in range(calls):
            for r in rs:
                r.trace_samples(spp)
        for r in rs:
            r.check()

    def bat(spp, calls):
        for _ in range(calls):
            b.trace_samples(spp)
        b.check()

    def timed_seq(spp, calls, pipelined):
        for r in rs:
            r.set_pipelining(pipelined)
            r.reset()
        seq(spp, 2)  # warm-up (allocations, graph capture)
        for r in rs:
            r.reset()
        t = timed(lambda: seq(spp, calls))
        for r in rs:
            r.set_pipelining(True)
        return t

    modes = {}
    for spp, calls in ((ADJ_SPP, 1), (1, ADJ_SPP)):
        # Per-scene launches: each renderer's waves on the caller's stream,
        # one renderer's launches after the other's (no pipelining); also with
        # pipelining, where each renderer's waves overlap the previous one's.
        ts = timed_seq(spp, calls, False)
        tp = timed_seq(spp, calls, True)
        px = len(rs) * ADJ_W * ADJ_W * spp * calls
        m = {"sequential_mpaths_per_s": round(px / ts / 1e6, 2),
             "sequential_pipelined_mpaths_per_s": round(px / tp / 1e6, 2)}
        best = best_p = 0.0
        for streams in (1, 2):  # one batch, or its views in two parts on two streams
            b.set_options(streams=streams)
            bat(spp, 2)
            for r in rs:
                r.reset()
            tbt = timed(lambda: bat(spp, calls))
            m["batched_streams%d_mpaths_per_s" % streams] = round(px / tbt / 1e6, 2)
            best, best_p = max(best, ts / tbt), max(best_p, tp / tbt)
        m["batched_over_sequential"] = round(best, 3)  # the better of the two batch settings
        m["batched_over_pipelined_renderers"] = round(best_p, 3)
        modes["%d_spp_per_call" % spp] = m
    ratio = tb / tf
    return {
        "metric": ADJ_METRIC,
        "value": round(ratio, 3), "unit": "x", "ms_per_step": round(1e3 * (tf + tb + tu + tr) / args.steps, 2),
        "higher_is_better": False,
        "e2e": {"value": round(ratio, 3), "unit": "x", "h2d_bytes_per_step": ADJ_VIEWS * ADJ_W * ADJ_W * 16,
                "d2h_bytes_per_step": ADJ_VIEWS * ADJ_W * ADJ_W * 52},
        "roofline": None, "clocks": clk.summary(), "gpu_launches": None, "dtype": "f32 (+f64 exact hit decisions)",
        "config": CONFIGS["adjoint"],
        "extra": {"forward_ms_per_view": round(1e3 * tf / (len(views) * args.steps), 2),
                  "backward_ms_per_view": round(1e3 * tb / (len(views) * args.steps), 2),
                  "upload_and_adam_ms_per_step": round(1e3 * tu / args.steps, 2),
                  "allreduce_ms_per_step": round(1e3 * tr / args.steps, 3),
                  "views_per_rank": len(views), "gradient_values": opt.size,
                  "forward_mpaths_per_s": round(paths / tf / 1e6, 2),
                  "loss": [round(x, 3) for x in opt.history],
                  "batched_forward": modes},
    }


def cpu_adjoint(threads, reps=1):
    """Oracle forward on a 32x32 crop of view 0 at 32 spp (the backward has no CPU counterpart)."""
    from lucent_gb300 import workloads as W
    from oracle import render as R
    sc = W.adjoint_scene(0, 6)
    prep = R.prepare(sc)
    t0 = time.perf_counter()
    for _ in range(reps):
        R.render(prep, ADJ_W, ADJ_W, 1, ADJ_SPP, max_bounces=ADJ_DEPTH, crop=(240, 240, 32, 32), threads=threads)
    dt = time.perf_counter() - t0
    return 32 * 32 * ADJ_SPP * reps / dt / 1e6, "32x32 crop of view 0, 32 spp, forward only (Mpaths/s)"


# ----------------------------------------------------------------------------- plumbing
_pg = None


def init_dist(world, local):
    global _pg
    if world > 1 and _pg is None:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
        _pg = dist


def barrier(world):
    if world > 1:
        _pg.barrier()


def max_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    _pg.all_reduce(t, op=_pg.ReduceOp.MAX)
    return float(t.item())


WORKLOADS = {"closest": (run_ours_closest, cpu_closest, "Mrays/s"), "pt": (run_ours_pt, cpu_pt, "Mrays/s"),
             "batch": (run_ours_batch, cpu_batch, "Mpaths/s"), "adjoint": (run_ours_adjoint, cpu_adjoint, "Mpaths/s"),
             "knot": (run_ours_knot, cpu_knot, "spp/s"), "build": (run_ours_build, cpu_build, "Mtris/s")}
METRICS = {"closest": "closest-hit Mrays/s (intersectBVH, 65,536-triangle soup, 1e6 rays)", "pt": PT_METRIC,
           "knot": "large-mesh spp/s: 2,000,000-triangle knot, 1920x1080, depth 12 (closest-hit Mrays/s beside it)",
           "build": "GPU BVH build Mtris/s (buildBVH, bit-exact nodes): configs 1-3 meshes (65,536 / 81,956 / "
                    "2,000,000 triangles)"}
DEFAULT_WORKLOAD = "pt"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="default 20 (batch: 1)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-scenes", type=int, default=64, help="scenes of the batch workload")
    ap.add_argument("--knot-spp", type=int, default=8, help="samples per step of the large-mesh workload")
    ap.add_argument("--no-targets", dest="targets", action="store_false",
                    help="skip the other configurations' figures in the default line")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = {"batch": 1, "adjoint": 3, "knot": 3}.get(args.workload, 20)
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    rank, world, local = dist_env()
    run, cpu, unit = WORKLOADS[args.workload]
    cores = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return
        if args.workload == "adjoint":
            # Our line's value is a backward/forward time ratio; the reference
            # renders forward only, so it has no such ratio to time.
            print(json.dumps({"impl": "reference", "metric": ADJ_METRIC, "unavailable":
                              "the reference has no backward pass (no differentiable renderer), so no "
                              "backward/forward ratio exists to time"}), flush=True)
            return
        if args.workload == "batch":
            print(json.dumps({"impl": "reference", "metric": None, "unavailable":
                              "the reference renders one scene per WebGL context; its CPU code has no batch path"}),
                  flush=True)
            return
        vals = []
        for _ in range(args.warmup):
            cpu(cores, reps=1)
        sample = ""
        for _ in range(args.steps):
            v, sample = cpu(cores, reps=1)
            vals.append(v)
        v = float(np.mean(vals))
        line = {"impl": "reference", "metric": None, "value": round(v, 3), "unit": unit, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "data": "synthetic",
                "cpu_baseline": {"value": round(v, 3), "unit": unit, "cores": cores, "kind": "port",
                                 "sample": sample + " (oracle: C++ restatement of the reference's TypeScript, "
                                                    "binary64, std::thread on all host cores; not V8)"},
                "e2e": {"value": round(v, 3), "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        line["metric"] = METRICS[args.workload]
        line["config"] = CONFIGS[args.workload]
        print(json.dumps(line), flush=True)
        return

    init_dist(world, local)
    res = run(args, rank, world, local)
    if rank != 0:
        return
    line = {"metric": res["metric"], "value": res["value"], "unit": res["unit"], "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["ms_per_step"],
            "higher_is_better": res.get("higher_is_better", True), "scaling": "weak", "vs_baseline": None,
            "dtype": res["dtype"],
            "data": "synthetic", "config": res["config"], "e2e": res["e2e"], "roofline": res["roofline"],
            "clocks": res["clocks"], "gpu_launches": res["gpu_launches"]}
    for k in ("spp_per_s", "extra"):
        if k in res:
            line[k] = res[k]
    if world == 1 and not args.no_cpu_baseline:
        # a bounded sample of the same workload, repeated to about CPU_BASELINE_SECONDS of CPU work
        t0, vals = time.perf_counter(), []
        while not vals or time.perf_counter() - t0 < CPU_BASELINE_SECONDS:
            v, sample = cpu(cores)
            vals.append(v)
        v = float(np.mean(vals))
        sample += ", %d runs in %.1f s" % (len(vals), time.perf_counter() - t0)
        line["cpu_baseline"] = {"value": round(v, 3), "unit": unit, "cores": cores, "kind": "port",
                                "sample": sample + " (oracle C++ restatement, binary64, not V8)"}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
