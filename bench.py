"""Benchmark of the Lucent GB300 hot path; prints ONE JSON line on rank 0.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Workloads:
  pt       (default) path tracing of the box scene (81,956 triangles) at
           512x512, 16 spp, depth 8: one step = one 16-spp frame; the metric
           is closest-hit rays per second inside the renderer, with spp/s
  closest  random soup, 65,536 triangles, 10^6 rays, seed 0: one step = one
           closest-hit pass over all rays (the reference's intersectBVH)
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
                "peak_source": which, "bytes_per_ray": alg["bytes_per_ray"]}
    return {
        "metric": "closest-hit Mrays/s (intersectBVH, 65,536-triangle soup, 1e6 rays)",
        "value": round(value, 2), "unit": "Mrays/s", "ms_per_step": round(sum(ms) / len(ms), 4),
        "wall_s": round(wall, 3), "e2e": e2e, "roofline": roof, "clocks": clk.summary(),
        "gpu_launches": 2 * args.steps, "dtype": "f32+f64",
        "config": {"workload": "closest: random soup 65,536 tris (PCG64 seed 0), 1e6 sphere rays, tMin 1e-5",
                   "l2": "flushed between timed steps (256 MB write)", "hit_ids": "bit-exact vs intersectBVH"},
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
# dram__bytes_read.sum + dram__bytes_write.sum from ncu captures of the same
# workloads (profiles/closest_pt_box512_16spp.md, closest_fast_soup65k_1Mrays.md).
NCU_DRAM_BYTES_PT_FRAME = 1_042_000_000
NCU_DRAM_BYTES_CLOSEST_LAUNCH = 33_500_000
PT_METRIC = ("closest-hit Mrays/s inside path tracing: box scene (81,956 triangles), 512x512, 16 spp, "
             "max depth 8 (also spp/s)")


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

    for _ in range(args.warmup):
        step()
    r.check(sp)
    s0 = r.stats()
    barrier(world)
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        for k in range(args.steps):
            flush.fill_(float(k))  # evict L2 (256 MB > 129 MB) between timed frames
            evs[k][0].record(stream)
            step()
            evs[k][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    r.check(sp)
    s1 = r.stats()
    ms = [a.elapsed_time(b) for a, b in evs]
    dev_s = max_over_ranks(sum(ms) / 1000.0, world)
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
    # host structs, trace, colour target (512 x 512 x RGBA32F) back to pinned host memory.
    L = N.lib()
    out = torch.empty(PT_W * PT_H * 4, dtype=torch.float32).pin_memory()
    cam = r.camera_state
    settings = NR.SettingsDesc(PT_DEPTH, r.settings.firefly_clamp)

    def e2e_step():
        N.check(L.lucent_renderer_upload_camera(r.handle, C.byref(cam)))
        N.check(L.lucent_renderer_apply_settings(r.handle, C.byref(settings)))
        N.check(L.lucent_renderer_trace(r.handle, PT_SPP, sp))
        N.check(L.lucent_renderer_read(r.handle, C.cast(out.data_ptr(), N.F32P), None, None, None))

    for _ in range(max(1, args.warmup)):
        e2e_step()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
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
                "traffic_scope": "DRAM bytes of the frame's 9 closest-hit launches (ncu), like achieved",
                "peak_source": which, "kernel": "k_closest_fast_t<PathClosest> (+ slow path)",
                "bytes_per_closest_ray": alg["bytes_per_closest_ray"],
                "closest_ms_per_frame": round(ph["closest"], 3)}
    launches_per_frame = 2 + 8 * (PT_DEPTH + 1)
    return {
        "metric": PT_METRIC, "value": round(value, 2), "unit": "Mrays/s", "ms_per_step": round(sum(ms) / len(ms), 4),
        "wall_s": round(wall, 3), "e2e": e2e, "roofline": roof, "clocks": clk.summary(),
        "gpu_launches": launches_per_frame * args.steps, "dtype": "f32 (+f64 exact hit decisions)",
        "spp_per_s": round(spp_per_s, 2),
        "extra": {"mpaths_per_s": round(paths / dev_s / 1e6, 2), "shadow_mrays_per_s": round(shadow / dev_s / 1e6, 2),
                  "closest_rays_per_frame": int(per_frame_closest),
                  "phase_ms_per_frame": {k: round(v, 3) for k, v in ph.items()}},
        "config": {"workload": "pt: box scene seed 0 (5 Lambert walls, quad light 15, 2 rotated boxes, "
                               "81,920-triangle icosphere, layered BSDF), 512x512, 16 spp, depth 8, RR from bounce 2",
                   "l2": "flushed between timed frames (256 MB write)",
                   "hit_ids": "bit-exact vs intersectBVH (tMin 1e-6, tMax 1e30)"},
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


WORKLOADS = {"closest": (run_ours_closest, cpu_closest, "Mrays/s"), "pt": (run_ours_pt, cpu_pt, "Mrays/s")}
DEFAULT_WORKLOAD = "pt"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    rank, world, local = dist_env()
    run, cpu, unit = WORKLOADS[args.workload]
    cores = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
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
        ours_metric = {"closest": "closest-hit Mrays/s (intersectBVH, 65,536-triangle soup, 1e6 rays)", "pt": PT_METRIC}
        line["metric"] = ours_metric.get(args.workload, args.workload)
        line["config"] = {"workload": args.workload}
        print(json.dumps(line), flush=True)
        return

    init_dist(world, local)
    res = run(args, rank, world, local)
    if rank != 0:
        return
    line = {"metric": res["metric"], "value": res["value"], "unit": res["unit"], "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": res["dtype"],
            "data": "synthetic", "config": res["config"], "e2e": res["e2e"], "roofline": res["roofline"],
            "clocks": res["clocks"], "gpu_launches": res["gpu_launches"]}
    for k in ("spp_per_s", "extra"):
        if k in res:
            line[k] = res[k]
    if world == 1 and not args.no_cpu_baseline:
        v, sample = cpu(cores)
        line["cpu_baseline"] = {"value": round(v, 3), "unit": res["unit"], "cores": cores, "kind": "port",
                                "sample": sample + " (oracle C++ restatement, binary64, not V8)"}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
