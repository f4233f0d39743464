"""Renderer mirroring the reference's Renderer class (src/renderer.ts:171-871).

Same calls and meaning: load_scene, upload_lighting, upload_ground,
upload_camera, apply_settings, reset, resize, trace_samples, render,
benchmark, stats, dispose. WebGL state is replaced by device buffers owned by
a lucent_renderer handle; the canvas is replaced by explicit width/height.
"""
import ctypes as C
import math
import time
from dataclasses import dataclass

import numpy as np

from . import _native as N
from . import _native_render as NR
from . import scene as S

ATROUS_STEPS = [1, 2, 4, 8, 16]  # renderer.ts:140
PHASES = ("camera", "closest", "shade", "shadow", "resolve", "accumulate")


def atrous_levels(spp):  # renderer.ts:142
    return 5 if spp <= 4 else 4 if spp <= 16 else 3 if spp <= 64 else 2 if spp <= 256 else 1


def denoise_weight(spp):  # renderer.ts:144
    return min(1.0, max(0.0, (1024 - spp) / (1024 - 128)))


@dataclass
class RenderSettings:
    """RenderSettings / DEFAULT_SETTINGS (renderer.ts:42-84), the fields this build uses."""
    max_bounces: int = 6
    exposure: float = 1.0
    tonemap: str = "aces"
    firefly_clamp: float = 8.0
    denoise: bool = True
    temporal: bool = True
    samples_per_frame: int = 1
    max_samples: int = 0


TONEMAPS = {"aces": 0, "reinhard": 1, "none": 2}  # display.frag uTonemap
SIGMA_L, SIGMA_N, SIGMA_P = 4.0, 64.0, 1.5  # runDenoiser uniforms (renderer.ts:815-817)


def _f(a):
    return N.ptr(a, C.c_float) if a is not None else None


class Renderer:
    def __init__(self, width, height):
        self.settings = RenderSettings()
        h = C.c_void_p()
        N.check(N.lib().lucent_renderer_create(width, height, C.byref(h)))
        self._h = h
        self.width, self.height = width, height
        self.scene = None
        self._keep = []
        self.camera_state = None

    @classmethod
    def view(cls, src, width, height, camera=None):
        """A renderer of `src`'s loaded scene seen from `camera` (default:
        the scene's), sharing the scene's device data instead of copying it
        (lucent_renderer_create_view): geometry, BVH, materials, textures.
        Targets, camera, settings, ground and lighting are the view's own;
        materials set through any of them change for all."""
        from dataclasses import replace
        r = cls.__new__(cls)
        r.settings = RenderSettings()
        h = C.c_void_p()
        N.check(N.lib().lucent_renderer_create_view(src.handle, width, height, C.byref(h)))
        r._h = h
        r.width, r.height = width, height
        r._keep = []
        r.camera_state = None
        r.source = src  # the source must outlive its views
        r.packed = src.packed
        r.scene = replace(src.scene, camera=camera) if camera is not None else src.scene
        r.upload_ground(r.scene.ground)
        r.upload_lighting(r.scene)
        r.upload_camera(r.scene.camera, False)
        r.apply_settings()
        r.reset()
        return r

    @property
    def handle(self):
        return self._h

    def dispose(self):
        if getattr(self, "_h", None):
            N.lib().lucent_renderer_destroy(self._h)
            self._h = None

    __del__ = dispose

    # ------------------------------------------------------------------ scene
    def load_scene(self, scene: S.Scene, bvh=None):
        """loadScene (renderer.ts:279-312); `bvh` is a prebuilt reference-layout BVH."""
        p = S.pack_scene(scene)
        self.packed = p
        d = NR.SceneDesc()
        d.tri_count = p.tri_count
        keep = [p.positions, p.normals, p.tri_material, p.tri_light, p.tri_alpha, p.materials, p.spheres,
                p.sphere_materials, p.sphere_lights, p.lights]
        d.positions, d.normals = _f(p.positions), _f(p.normals)
        d.uvs = _f(p.uvs) if p.uvs is not None else None
        if p.uvs is not None:
            keep.append(p.uvs)
        d.tri_material = N.ptr(p.tri_material, C.c_int32)
        d.tri_light = N.ptr(p.tri_light, C.c_int32)
        d.tri_alpha = N.ptr(p.tri_alpha, C.c_uint8)
        if bvh is not None:
            nodes = np.ascontiguousarray(bvh.nodes, np.float32)
            tri = np.ascontiguousarray(bvh.tri_indices, np.uint32)
            keep += [nodes, tri]
            d.bvh_nodes, d.bvh_node_count, d.bvh_tri_indices = _f(nodes), bvh.node_count, N.ptr(tri, C.c_uint32)
        d.materials, d.material_count = _f(p.materials), p.material_count
        d.spheres, d.sphere_count = _f(p.spheres), len(scene.spheres)
        d.sphere_materials = N.ptr(p.sphere_materials, C.c_int32)
        d.sphere_lights = N.ptr(p.sphere_lights, C.c_int32)
        d.lights, d.light_count = _f(p.lights), p.light_count
        d.ground_material = p.ground_material
        if p.color_layers or p.data_layers:  # texture maps (buildTextureArrays, renderer.ts:314-333)
            imgs = [np.ascontiguousarray(t.image, np.uint8) for t in scene.textures]
            for i, im in enumerate(imgs):
                if im.ndim != 3 or im.shape[2] != 4:
                    raise ValueError("texture %d is not an RGBA8 [h, w, 4] image" % i)
            ptrs = (NR.U8P * len(imgs))(*[N.ptr(im, C.c_uint8) for im in imgs])
            ws = np.array([im.shape[1] for im in imgs], np.uint32)
            hs = np.array([im.shape[0] for im in imgs], np.uint32)
            cl = np.array(p.color_layers, np.int32)
            dl = np.array(p.data_layers, np.int32)
            keep += [imgs, ptrs, ws, hs, cl, dl]
            d.texture_count, d.texture_rgba8 = len(imgs), ptrs
            d.texture_width, d.texture_height = N.ptr(ws, C.c_uint32), N.ptr(hs, C.c_uint32)
            d.color_layers, d.color_layer_count = N.ptr(cl, C.c_int32), len(cl)
            d.data_layers, d.data_layer_count = N.ptr(dl, C.c_int32), len(dl)
        N.check(N.lib().lucent_renderer_load_scene(self._h, C.byref(d)))
        self.scene = scene
        self.upload_ground(scene.ground)
        self.upload_lighting(scene)
        self.upload_camera(scene.camera, False)
        self.apply_settings()
        self.reset()

    def upload_lighting(self, scene: S.Scene):
        """uploadLighting (renderer.ts:355-387)."""
        L = S.lighting(scene)
        env = np.ascontiguousarray(L.env.data, np.float32)
        self._env = env
        d = NR.LightingDesc()
        d.sun_enabled = L.sun_enabled
        d.sun_dir[:] = L.sun_dir
        d.sun_radiance[:] = L.sun_radiance
        d.sun_cos_angle, d.sun_pdf = L.sun_cos_angle, L.sun_pdf
        d.env_width, d.env_height, d.env_rgb = L.env.width, L.env.height, _f(env)
        d.env_rotation_cos, d.env_rotation_sin = L.env_rotation
        d.env_intensity, d.env_background = L.env_intensity, L.env_background
        d.backdrop[:] = L.backdrop
        N.check(N.lib().lucent_renderer_upload_lighting(self._h, C.byref(d)))

    def upload_ground(self, ground: S.Ground):
        N.check(N.lib().lucent_renderer_upload_ground(self._h, 1 if ground.enabled else 0, ground.height))

    def upload_camera(self, cam: S.Camera, moving=True):
        """uploadCamera (renderer.ts:424-439); any camera change restarts the average."""
        f, r, u = S.camera_basis(cam)
        d = NR.CameraDesc()
        d.position[:] = cam.position
        d.right[:], d.up[:], d.forward[:] = r, u, f
        d.tan_half_fov = math.tan(cam.fov * math.pi / 360)
        d.aperture, d.focus_distance = cam.aperture, cam.focus_distance
        self.camera_state = d
        N.check(N.lib().lucent_renderer_upload_camera(self._h, C.byref(d)))

    def apply_settings(self):
        d = NR.SettingsDesc(self.settings.max_bounces, self.settings.firefly_clamp, 1 if self.settings.temporal else 0)
        N.check(N.lib().lucent_renderer_apply_settings(self._h, C.byref(d)))

    def reset(self):
        N.check(N.lib().lucent_renderer_reset(self._h))

    def resize(self, width, height):
        N.check(N.lib().lucent_renderer_resize(self._h, width, height))
        self.width, self.height = width, height

    def set_seed(self, seed):
        N.check(N.lib().lucent_renderer_set_seed(self._h, seed))

    # ------------------------------------------------------------------ work
    def trace_samples(self, count, stream=None):
        """traceSamples (renderer.ts:702-737), asynchronous on `stream`: the
        samples are in the targets for work queued on `stream` afterwards.
        With pipelining (default) the waves run on the renderer's own streams,
        so successive calls overlap one wave's last bounces with the next's
        first; only the accumulation is queued on `stream`."""
        N.check(N.lib().lucent_renderer_trace(self._h, count, stream))

    def check(self, stream=None):
        N.check(N.lib().lucent_renderer_check(self._h, stream))

    def read(self):
        """(color4, albedo4, normal4, history) as numpy arrays [H, W, ...], row 0 = bottom."""
        n = self.width * self.height
        col = np.empty(n * 4, np.float32)
        alb = np.empty(n * 4, np.float32)
        nrm = np.empty(n * 4, np.float32)
        hist = np.empty(n, np.float32)
        N.check(N.lib().lucent_renderer_read(self._h, _f(col), _f(alb), _f(nrm), _f(hist)))
        sh = (self.height, self.width)
        return col.reshape(*sh, 4), alb.reshape(*sh, 4), nrm.reshape(*sh, 4), hist.reshape(sh)

    def stats(self):
        st = NR.RenderStats()
        N.check(N.lib().lucent_renderer_stats(self._h, C.byref(st)))
        out = {k: getattr(st, k) for k, _ in NR.RenderStats._fields_}
        out["phase_ms"] = dict(zip(PHASES, list(st.phase_ms)))
        out["traversal"] = dict(zip(("rays", "slab_f64", "triangle_f64", "closest_f64", "final_f64"),
                                    [int(x) for x in st.traversal]))
        return out

    def set_ray_sort(self, enabled=True):
        """Sort the rays of bounces 1 and 2 by direction and origin (lucent_renderer_set_ray_sort)."""
        N.check(N.lib().lucent_renderer_set_ray_sort(self._h, 1 if enabled else 0))

    def read_texture_arrays(self):
        """(colour layers, data layers) as uint8 [layers, size, size, 4] (lucent_renderer_read_textures)."""
        size = C.c_uint32()
        N.check(N.lib().lucent_renderer_read_textures(self._h, C.byref(size), None, None))
        n = size.value
        p = self.packed
        col = np.zeros((len(p.color_layers), n, n, 4), np.uint8)
        dat = np.zeros((len(p.data_layers), n, n, 4), np.uint8)
        N.check(N.lib().lucent_renderer_read_textures(self._h, C.byref(size), N.ptr(col, C.c_uint8),
                                                      N.ptr(dat, C.c_uint8)))
        return col, dat

    def set_wide_bvh(self, enabled=True):
        """Closest hit over the four-wide BVH view (lucent_renderer_set_wide_bvh)."""
        N.check(N.lib().lucent_renderer_set_wide_bvh(self._h, 1 if enabled else 0))

    def set_pipelining(self, enabled=True):
        """Alternate successive waves between two path buffers traced on the
        renderer's own streams (lucent_renderer_set_pipelining; default on)."""
        N.check(N.lib().lucent_renderer_set_pipelining(self._h, 1 if enabled else 0))

    def read_color_async(self, out, stream=None):
        """Queues a copy of the colour target into `out` (a pinned torch or
        numpy float32 buffer of width*height*4, alive until the stream reaches
        the copy) and returns; check(stream) waits for it."""
        ptr = out.data_ptr() if hasattr(out, "data_ptr") else out.ctypes.data
        N.check(N.lib().lucent_renderer_read_color_async(self._h, C.cast(ptr, N.F32P), stream))

    def set_top_levels(self, enabled=True):
        """Stage the top BVH levels in shared memory (lucent_renderer_set_top_levels)."""
        N.check(N.lib().lucent_renderer_set_top_levels(self._h, 1 if enabled else 0))

    def trim(self):
        """Frees the path-state buffers until the next trace (lucent_renderer_trim)."""
        N.check(N.lib().lucent_renderer_trim(self._h))

    def set_profiling(self, enabled=True, counters=False):
        """Per-phase event timing (lucent_renderer_set_profiling); `counters`
        adds the closest-hit traversal counters, which slow that kernel."""
        N.check(N.lib().lucent_renderer_set_profiling(self._h, (2 if counters else 1) if enabled else 0))

    def set_env_device(self, rgb_ptr, width, height, stream=None):
        """Replaces the environment map with a device RGB map (an int device
        pointer, width * height * 3 floats) and builds its sampler on the GPU
        (lucent_renderer_set_env_device); other lighting stays as uploaded."""
        N.check(N.lib().lucent_renderer_set_env_device(self._h, rgb_ptr, width, height, stream))

    def capture_rays(self, bounces=(), max_rays=1 << 22):
        """Keep the closest-hit and shadow rays of these bounces of the next
        traces' last wave (lucent_renderer_capture_rays); () turns it off."""
        mask = 0
        for b in bounces:
            mask |= 1 << int(b)
        N.check(N.lib().lucent_renderer_capture_rays(self._h, mask, max_rays if mask else 0))
        self._cap_rays = max_rays if mask else 0

    def read_rays(self, bounce, shadow=False):
        """Captured rays of `bounce` as a [n, 16] float32 array (lucent_renderer_read_rays).
        Closest: origin, path id bits, direction, scene bits, t, u, v, slot bits, key bits.
        Shadow: origin, t_max, direction, key bits, occluded, shadow slot bits."""
        count = C.c_uint32(0)
        N.check(N.lib().lucent_renderer_read_rays(self._h, bounce, 1 if shadow else 0, None, 0, C.byref(count)))
        m = min(count.value, getattr(self, "_cap_rays", 0))
        out = np.zeros((m, 16), np.float32)
        if m:
            N.check(N.lib().lucent_renderer_read_rays(self._h, bounce, 1 if shadow else 0, _f(out), m,
                                                      C.byref(count)))
        return out

    # --------------------------------------------------------- denoise/display
    def samples(self):
        """Samples behind the current average (the reference's `frame`)."""
        return self.stats()["samples"]

    def denoise(self, levels=None, sigma_l=SIGMA_L, sigma_n=SIGMA_N, sigma_p=SIGMA_P, stream=None):
        """runDenoiser (renderer.ts:788-830): variance, then atrousLevels(frame) a-trous steps."""
        if levels is None:
            levels = atrous_levels(self.samples())
        N.check(N.lib().lucent_renderer_denoise(self._h, levels, sigma_l, sigma_n, sigma_p, stream))

    def read_denoised(self):
        """Filtered illumination (rgb) and variance (a), [H, W, 4], row 0 = bottom."""
        out = np.empty(self.width * self.height * 4, np.float32)
        N.check(N.lib().lucent_renderer_read_denoised(self._h, _f(out)))
        return out.reshape(self.height, self.width, 4)

    def display(self, denoise_weight=0.0, exposure=None, tonemap=None, want_float=False, stream=None, view=None):
        """The display pass (renderer.ts:573-591): RGBA8 canvas [H, W, 4], row 0 = bottom;
        with want_float also the RGB values before quantization. `view` = (width, height)
        shows the renderer's image in a canvas of that size (Catmull-Rom upsampling of the
        reduced-resolution preview, display.frag:44-60; lucent_renderer_display_view)."""
        exposure = self.settings.exposure if exposure is None else exposure
        tm = TONEMAPS[self.settings.tonemap if tonemap is None else tonemap]
        vw, vh = (self.width, self.height) if view is None else (int(view[0]), int(view[1]))
        n = vw * vh
        rgba = np.empty(n * 4, np.uint8)
        rgb = np.empty(n * 3, np.float32) if want_float else None
        N.check(N.lib().lucent_renderer_display_view(self._h, vw, vh, denoise_weight, tm, exposure,
                                                     N.ptr(rgba, C.c_uint8), _f(rgb), stream))
        img = rgba.reshape(vh, vw, 4)
        return (img, rgb.reshape(vh, vw, 3)) if want_float else img

    def render(self):
        """render() (renderer.ts:553-611) with a fixed samples_per_frame budget:
        trace, filter when the denoiser is on, present. Returns the RGBA8 canvas."""
        st = self.settings
        frame = self.samples()
        remaining = st.max_samples - frame if st.max_samples > 0 else st.samples_per_frame
        n = max(0, min(st.samples_per_frame, remaining))
        if n:
            self.trace_samples(n)
            frame += n
        weight = denoise_weight(frame) if st.denoise and frame > 0 else 0.0
        if weight > 0:
            self.denoise(atrous_levels(frame))
        return self.display(weight)

    def benchmark(self, samples):
        """benchmark(n) (renderer.ts:745-777): one warm-up sample, then `samples` timed."""
        self.reset()
        self.trace_samples(1)
        self.check()
        t0 = time.perf_counter()
        self.trace_samples(samples)
        self.check()
        trace_ms = (time.perf_counter() - t0) * 1e3
        return {"trace_ms": trace_ms, "mpaths_per_sec": samples * self.width * self.height / (trace_ms / 1e3) / 1e6,
                "width": self.width, "height": self.height}


def bsdf_grad_tuples(tuples):
    """f and its derivatives in (albedo r, g, b, roughness, metallic,
    clearcoat) on [n, 32] tuples -> [n, 24] float32 (f 3, then 6 x 3)."""
    t = np.ascontiguousarray(tuples, np.float32).reshape(-1, 32)
    out = np.zeros((t.shape[0], 24), np.float32)
    N.check(N.lib().lucent_bsdf_grad_tuples(_f(t), t.shape[0], _f(out)))
    return out


def bsdf_eval_tuples(tuples):
    """The renderer's BSDF code on [n, 32] float tuples -> [n, 24] float32
    (layout in csrc/bsdf_tuples.cu: evalOpaque f, pdf; sampleOpaque dir,
    weight, pdf; sampleDielectric ok, dir, weight, reflected)."""
    t = np.ascontiguousarray(tuples, np.float32).reshape(-1, 32)
    out = np.zeros((t.shape[0], 24), np.float32)
    N.check(N.lib().lucent_bsdf_eval_tuples(_f(t), t.shape[0], _f(out)))
    return out


class Batch:
    """Several renderers traced as one wavefront (lucent_batch_*): the next
    `samples` samples of every renderer, bit for bit what trace_samples on
    each renderer alone would give. Options (lucent_batch_options):
    samples_per_wave (0 = as many as max_wave_paths allows), max_wave_paths,
    use_graph (replay a captured wave), trace_blocks / shade_blocks (grid
    sizes, 0 = all resident blocks), sort_rays, top_levels, wide_bvh (as
    the renderer's set_ray_sort / set_top_levels / set_wide_bvh),
    scenes_per_wave (waves hold groups of this many consecutive scenes,
    each traced for all samples before the next; 0 = all scenes), streams
    (the renderers in that many parts, traced side by side on their own
    streams)."""

    DEFAULTS = {"samples_per_wave": 0, "max_wave_paths": 1 << 25, "use_graph": True, "trace_blocks": 0,
                "shade_blocks": 0, "sort_rays": True, "top_levels": True, "wide_bvh": True, "scenes_per_wave": 0,
                "streams": 1}

    def __init__(self, renderers, **options):
        self.renderers = list(renderers)
        arr = (C.c_void_p * len(self.renderers))(*[r.handle.value for r in self.renderers])
        h = C.c_void_p()
        N.check(N.lib().lucent_batch_create(arr, len(self.renderers), C.byref(h)))
        self._h = h
        self.options = dict(self.DEFAULTS)
        self.set_options(**options)

    def set_options(self, **options):
        unknown = set(options) - set(self.DEFAULTS)
        if unknown:
            raise KeyError("unknown batch options: %s" % sorted(unknown))
        self.options.update(options)
        o = self.options
        d = NR.BatchOptions(o["samples_per_wave"], o["max_wave_paths"], 1 if o["use_graph"] else 0,
                            o["trace_blocks"], o["shade_blocks"], 1 if o["sort_rays"] else 0,
                            1 if o["top_levels"] else 0, 1 if o["wide_bvh"] else 0, o["scenes_per_wave"],
                            o["streams"])
        N.check(N.lib().lucent_batch_set_options(self._h, C.byref(d)))

    def trace_samples(self, count, stream=None):
        N.check(N.lib().lucent_batch_trace(self._h, count, stream))

    def check(self, stream=None):
        st = NR.BatchStats()
        N.check(N.lib().lucent_batch_check(self._h, stream, C.byref(st)))
        return {k: int(getattr(st, k)) for k, _ in NR.BatchStats._fields_}

    def signature(self):
        """Workload key for the tuning cache: scene count, pixels, triangles, bounces."""
        px = sum(r.width * r.height for r in self.renderers)
        tris = sum(r.stats()["triangles"] for r in self.renderers)
        mb = max(r.settings.max_bounces for r in self.renderers)
        return "n%d_px%d_tri%d_b%d" % (len(self.renderers), px, tris, mb)

    # Second tuning stage: one option at a time from the best wave configuration
    # (ray sorting, the shared-memory top BVH levels, the grid of the shade /
    # resolve / any-hit kernels); none of them changes an image.
    REFINE = ({"sort_rays": False}, {"top_levels": False}, {"shade_blocks": 152 * 3}, {"shade_blocks": 152 * 8},
              {"streams": 2})

    def autotune(self, samples=2, candidates=None, cache=None, refine=True):
        """Times at least `samples` samples (two full waves) under each
        candidate option set (wall clock around trace + synchronise, so launch
        overhead counts) and keeps the fastest per sample; then, if `refine`,
        tries each REFINE change on top of the winner and keeps those that are
        faster (coordinate descent). The samples are real: reset the renderers
        afterwards for a fresh average. With `cache` (a JSON file path) a
        result for the same signature() is reused, and new results are stored
        there. Returns (chosen options, {candidate index: seconds per sample})."""
        import json
        import os
        key = self.signature()
        if cache and os.path.exists(cache):
            with open(cache) as f:
                known = json.load(f)
            if key in known:
                self.set_options(**known[key])
                return dict(self.options), {}
        if candidates is None:  # wave budgets of 2^23 .. 2^25 paths, with and without graph replay
            px = sum(r.width * r.height for r in self.renderers)
            waves = sorted({max(1, (1 << k) // px) for k in (23, 24, 25)})
            candidates = [{"samples_per_wave": s, "use_graph": g, "max_wave_paths": max(s * px, 1),
                           "scenes_per_wave": 0} for s in waves for g in (True, False)]
            # waves of a few consecutive scenes at a time (each group traced for all its samples)
            candidates += [{"samples_per_wave": 0, "use_graph": True, "max_wave_paths": 1 << 25, "scenes_per_wave": k}
                           for k in (1, 2, 4, 8, 16) if k < len(self.renderers)]
        base = dict(self.options)
        times = {}

        def measure(opts):
            self.set_options(**opts)
            n = max(samples, 2 * opts.get("samples_per_wave", 1))  # at least two full waves
            self.trace_samples(n)  # allocation and graph capture happen outside the timed call
            self.check()
            t0 = time.perf_counter()
            self.trace_samples(n)
            self.check()
            return (time.perf_counter() - t0) / n  # seconds per sample

        for i, c in enumerate(candidates):
            times[i] = measure({**base, **c})
        best = min(times, key=times.get)
        chosen, best_t = {**base, **candidates[best]}, times[best]
        tuned = dict(candidates[best])
        if refine:
            for j, change in enumerate(self.REFINE):
                if all(chosen.get(k) == v for k, v in change.items()):
                    continue
                t = measure({**chosen, **change})
                times["refine%d" % j] = t
                if t < best_t:
                    chosen, best_t = {**chosen, **change}, t
                    tuned.update(change)
        self.set_options(**chosen)
        candidates = list(candidates) + [tuned]
        best = len(candidates) - 1
        if cache:
            known = {}
            if os.path.exists(cache):
                with open(cache) as f:
                    known = json.load(f)
            known[key] = {k: self.options[k] for k in candidates[best]}
            os.makedirs(os.path.dirname(os.path.abspath(cache)), exist_ok=True)
            with open(cache, "w") as f:
                json.dump(known, f, indent=1, sort_keys=True)
        return dict(self.options), times

    def dispose(self):
        if getattr(self, "_h", None):
            N.lib().lucent_batch_destroy(self._h)
            self._h = None

    __del__ = dispose
