"""Oracle renderer wrapper (TEST INFRASTRUCTURE ONLY: the checker).

Prepares everything the reference computes on the CPU before drawing, with
the oracle's own code: buildBVH over the merged triangles, packScene's gather
into BVH leaf order (src/scene/scene.ts:215-235), buildEnvSampler
(environment.ts:52-85) and the sheen LUT rounded to half precision
(renderer.ts:241-242), then runs the C++ restatement of trace.frag.
"""
import ctypes as C

import numpy as np

from . import _p, build_bvh, build_env_sampler, lib, sheen_lut

P = C.POINTER
F, D, U32, I32 = C.c_float, C.c_double, C.c_uint32, C.c_int32


class OrcScene(C.Structure):
    _fields_ = [("tri_count", U32), ("positions", P(F)), ("geo", P(F)), ("attr", P(F)), ("nodes", P(F)),
                ("node_count", U32), ("tri_indices", P(U32)), ("materials", P(F)), ("material_count", U32),
                ("spheres", P(F)), ("sphere_materials", P(I32)), ("sphere_lights", P(I32)),
                ("sphere_count", U32), ("lights", P(F)), ("light_count", U32), ("ground_material", I32),
                ("ground_height", F), ("sun_enabled", I32), ("sun_dir", F * 3), ("sun_radiance", F * 3),
                ("sun_cos_angle", F), ("sun_pdf", F), ("env_width", U32), ("env_height", U32),
                ("env_rgb", P(F)), ("env_grid_w", U32), ("env_grid_h", U32), ("env_alias", P(F)),
                ("env_rot_cos", F), ("env_rot_sin", F), ("env_intensity", F), ("env_sampling", I32),
                ("env_background", I32), ("backdrop", F * 3), ("sheen_lut", P(F)), ("color_maps", P(C.c_uint8)),
                ("data_maps", P(C.c_uint8)), ("tex_size", U32)]


class OrcCamera(C.Structure):
    _fields_ = [("pos", F * 3), ("right", F * 3), ("up", F * 3), ("forward", F * 3), ("tan_half_fov", F),
                ("aperture", F), ("focus_dist", F)]


def declare(L):
    L.orc_render.argtypes = [P(OrcScene), P(OrcCamera), U32, F, U32, U32, U32, U32, U32, U32, U32, U32, C.c_int,
                             P(F), P(F), P(F), P(F), C.c_int]
    L.orc_render_work.argtypes = [P(OrcScene), P(OrcCamera), U32, F, U32, U32, U32, U32, U32, U32, U32, U32, P(F),
                                  P(F), P(F), P(F), C.c_int, C.c_int, P(C.c_uint64)]
    L.orc_bsdf_tuples.argtypes = [P(F), C.c_uint64, C.c_int, P(D), C.c_int]
    L.orc_bsdf_set_lut.argtypes = [P(F)]
    L.orc_denoise.argtypes = [P(F), P(F), P(F), P(F), U32, U32, P(OrcCamera), U32, F, F, F, P(F)]
    L.orc_detached_dot.argtypes = [P(OrcScene), P(OrcCamera), U32, F, U32, U32, U32, U32, P(F), P(F), P(F), C.c_int]
    L.orc_detached_dot.restype = C.c_double
    L.orc_display.argtypes = [P(F), P(F), P(F), U32, U32, F, F, C.c_int, P(F)]
    L.orc_display_view.argtypes = [P(F), P(F), P(F), U32, U32, U32, U32, F, F, C.c_int, P(F)]
    L.orc_resample_layer.argtypes = [P(C.c_uint8), U32, U32, U32, C.c_int, P(C.c_uint8)]
    L.orc_texture_size.argtypes = [P(U32), P(U32), U32]
    L.orc_texture_size.restype = U32
    L.orc_closest_slots.argtypes = [P(OrcScene), P(F), P(U32), C.c_uint64, D, D, P(I32), P(D), C.c_int]
    L.orc_any_slots.argtypes = [P(OrcScene), P(F), P(U32), C.c_uint64, D, P(C.c_uint8), C.c_int]


def half_lut():
    """The 16x16 sheen LUT as the reference uploads it: R16F (half) values."""
    return sheen_lut(16, 96).astype(np.float16).astype(np.float32)


class Prepared:
    """A packed scene + lighting ready for orc_render (arrays kept alive here)."""

    def __init__(self, packed, lighting, camera, ground=None, textures=()):
        from lucent_gb300 import scene as S
        self.keep = []
        keep = self.keep.append
        p = packed
        n = p.tri_count
        self.packed = p
        bvh = build_bvh(p.positions)
        self.bvh = bvh
        src = bvh.tri_indices.astype(np.int64)
        pos = p.positions.reshape(-1, 3, 3)[src] if n else np.zeros((0, 3, 3), np.float32)
        nrm = p.normals.reshape(-1, 3, 3)[src] if n else np.zeros((0, 3, 3), np.float32)
        geo = np.zeros((n, 3, 4), np.float32)  # scene.ts:213-235
        geo[:, :, :3] = pos
        geo[:, 0, 3] = p.tri_material[src]
        geo[:, 1, 3] = p.tri_light[src]
        geo[:, 2, 3] = p.tri_alpha[src]
        attr = np.zeros((n, 4, 4), np.float32)
        attr[:, :3, :3] = nrm
        if p.uvs is not None and n:
            uv = p.uvs.reshape(-1, 3, 2)[src]
            attr[:, :3, 3] = uv[:, :, 0]
            attr[:, 3, :3] = uv[:, :, 1]
        s = OrcScene()
        s.tri_count = n
        for name, arr, ct in (("positions", p.positions, F), ("geo", geo, F), ("attr", attr, F),
                              ("nodes", bvh.nodes, F), ("tri_indices", bvh.tri_indices, U32),
                              ("materials", p.materials, F), ("spheres", p.spheres, F),
                              ("sphere_materials", p.sphere_materials, I32), ("sphere_lights", p.sphere_lights, I32),
                              ("lights", p.lights, F)):
            a = np.ascontiguousarray(arr, np.float32 if ct is F else (np.uint32 if ct is U32 else np.int32))
            if a.size == 0:
                a = np.zeros(4, a.dtype)
            keep(a)
            setattr(s, name, _p(a, ct))
        s.node_count = bvh.node_count
        s.material_count = p.material_count
        s.sphere_count = p.sphere_materials.size
        s.light_count = p.light_count
        g = ground if ground is not None else S.Ground()
        s.ground_material = p.ground_material if g.enabled else -1
        s.ground_height = g.height
        L = lighting
        s.sun_enabled = L.sun_enabled
        s.sun_dir[:] = L.sun_dir
        s.sun_radiance[:] = L.sun_radiance
        s.sun_cos_angle, s.sun_pdf = L.sun_cos_angle, L.sun_pdf
        env = np.ascontiguousarray(L.env.data, np.float32)
        keep(env)
        self.env_data = env
        s.env_width, s.env_height, s.env_rgb = L.env.width, L.env.height, _p(env, F)
        gw, gh, table, total = build_env_sampler(env, L.env.width, L.env.height, 1024)
        keep(table)
        s.env_grid_w, s.env_grid_h, s.env_alias = gw, gh, _p(table, F)
        s.env_rot_cos, s.env_rot_sin = L.env_rotation
        s.env_intensity = L.env_intensity
        s.env_sampling = 1 if total > 0 else 0
        s.env_background = L.env_background
        s.backdrop[:] = L.backdrop
        lut = half_lut()
        keep(lut)
        s.sheen_lut = _p(lut, F)
        self.color_maps, self.data_maps, self.tex_size = texture_arrays(textures, p.color_layers, p.data_layers)
        keep(self.color_maps)
        keep(self.data_maps)
        s.color_maps = _p(self.color_maps, C.c_uint8)
        s.data_maps = _p(self.data_maps, C.c_uint8)
        s.tex_size = self.tex_size
        self.scene = s
        f, r, u = S.camera_basis(camera)
        cam = OrcCamera()
        cam.pos[:] = camera.position
        cam.right[:], cam.up[:], cam.forward[:] = r, u, f
        cam.tan_half_fov = float(np.tan(camera.fov * np.pi / 360))
        cam.aperture, cam.focus_dist = camera.aperture, camera.focus_distance
        self.camera = cam


def resample_layer(rgba, size, srgb):
    """orc_resample_layer: one texture-array layer [size, size, 4] uint8 from an RGBA8 image."""
    img = np.ascontiguousarray(rgba, np.uint8)
    out = np.zeros((size, size, 4), np.uint8)
    if lib().orc_resample_layer(_p(img, C.c_uint8), img.shape[1], img.shape[0], size, 1 if srgb else 0,
                                _p(out, C.c_uint8)):
        raise RuntimeError("orc_resample_layer failed")
    return out


def texture_arrays(textures, color_layers, data_layers):
    """(colour array, data array, size) of buildTextureArrays (renderer.ts:314-333)."""
    used = list(color_layers) + list(data_layers)
    if not used:
        return np.zeros(4, np.uint8), np.zeros(4, np.uint8), 0
    w = np.array([textures[t].image.shape[1] for t in used], np.uint32)
    h = np.array([textures[t].image.shape[0] for t in used], np.uint32)
    size = int(lib().orc_texture_size(_p(w, U32), _p(h, U32), len(used)))
    arrays = []
    for layers, srgb in ((color_layers, True), (data_layers, False)):
        arr = np.zeros((max(1, len(layers)), size, size, 4), np.uint8)
        for i, t in enumerate(layers):
            arr[i] = resample_layer(textures[t].image, size, srgb)
        arrays.append(arr)
    return arrays[0], arrays[1], size


def prepare(scene):
    from lucent_gb300 import scene as S
    return Prepared(S.pack_scene(scene), S.lighting(scene), scene.camera, scene.ground, scene.textures)


def render(prep, width, height, seed0, samples, max_bounces=6, clamp=8.0, precision=32, crop=None, threads=0):
    """orc_render over a crop (x0, y0, w, h) of a width x height image.
    Returns (color4, albedo4, normal4, history) shaped [h, w, ...] (row 0 = bottom)."""
    x0, y0, cw, ch = crop if crop is not None else (0, 0, width, height)
    col = np.zeros(cw * ch * 4, np.float32)
    alb = np.zeros(cw * ch * 4, np.float32)
    nrm = np.zeros(cw * ch * 4, np.float32)
    his = np.zeros(cw * ch, np.float32)
    st = lib().orc_render(C.byref(prep.scene), C.byref(prep.camera), max_bounces, clamp, width, height, x0, y0, cw,
                          ch, seed0, samples, precision, _p(col, F), _p(alb, F), _p(nrm, F), _p(his, F), threads)
    if st:
        raise RuntimeError("orc_render failed")
    return col.reshape(ch, cw, 4), alb.reshape(ch, cw, 4), nrm.reshape(ch, cw, 4), his.reshape(ch, cw)


def render_work(prep, width, height, seed0, samples, max_bounces=6, clamp=8.0, crop=None, threads=0, detailed=True):
    """Rays traced by the render and, if `detailed`, their reference GLSL traversal work."""
    x0, y0, cw, ch = crop if crop is not None else (0, 0, width, height)
    bufs = [np.zeros(cw * ch * 4, np.float32) for _ in range(3)] + [np.zeros(cw * ch, np.float32)]
    work = np.zeros(6, np.uint64)
    lib().orc_render_work(C.byref(prep.scene), C.byref(prep.camera), max_bounces, clamp, width, height, x0, y0, cw,
                          ch, seed0, samples, *[_p(b, F) for b in bufs], threads, 1 if detailed else 0,
                          work.ctypes.data_as(P(C.c_uint64)))
    keys = ["closest_rays", "closest_inner", "closest_tris", "shadow_rays", "shadow_nodes", "shadow_tris"]
    return dict(zip(keys, (int(x) for x in work)))


def closest_slots(prep, rays, keys=None, t_min=1e-6, t_max=1e30, threads=0):
    """orc_closest_slots: (slot per ray, -1 on a miss; binary64 t) of the
    renderer's triangle closest hit on binary32 rays [n, 6]."""
    r = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
    n = r.shape[0]
    k = None if keys is None else np.ascontiguousarray(keys, np.uint32)
    slot = np.zeros(n, np.int32)
    t = np.zeros(n, np.float64)
    lib().orc_closest_slots(C.byref(prep.scene), _p(r, F), None if k is None else _p(k, U32), n, t_min, t_max,
                            _p(slot, I32), _p(t, D), threads)
    return slot, t


def any_slots(prep, rays7, keys=None, t_min=1e-6, threads=0):
    """orc_any_slots: occlusion (bool) of shadow rays [n, 7] = origin, direction, t_max."""
    r = np.ascontiguousarray(rays7, np.float32).reshape(-1, 7)
    n = r.shape[0]
    k = None if keys is None else np.ascontiguousarray(keys, np.uint32)
    occ = np.zeros(n, np.uint8)
    lib().orc_any_slots(C.byref(prep.scene), _p(r, F), None if k is None else _p(k, U32), n, t_min,
                        occ.ctypes.data_as(P(C.c_uint8)), threads)
    return occ.astype(bool)


def bsdf_tuples(tuples, precision=64, threads=0):
    t = np.ascontiguousarray(tuples, np.float32).reshape(-1, 32)
    lut = half_lut()
    lib().orc_bsdf_set_lut(_p(lut, F))
    out = np.zeros((t.shape[0], 24), np.float64)
    lib().orc_bsdf_tuples(_p(t, F), t.shape[0], precision, _p(out, D), threads)
    return out


def _c32(a, shape):
    return np.ascontiguousarray(np.asarray(a, np.float32).reshape(shape))


def denoise(color4, albedo4, normal4, history, camera, levels, sigma_l=4.0, sigma_n=64.0, sigma_p=1.5):
    """orc_denoise: variance + `levels` a-trous steps over [H, W, 4] targets
    (albedo/normal as the RGBA16F values). `camera` is an OrcCamera.
    Returns [H, W, 4] float32 (illumination rgb, variance)."""
    h, w = color4.shape[:2]
    c, a, n = (_c32(x, (h, w, 4)) for x in (color4, albedo4, normal4))
    hi = _c32(history, (h, w))
    out = np.zeros((h, w, 4), np.float32)
    lib().orc_denoise(_p(c, F), _p(a, F), _p(n, F), _p(hi, F), w, h, C.byref(camera), levels, sigma_l, sigma_n,
                      sigma_p, _p(out, F))
    return out


def display(color4, albedo4, denoised4, denoise_weight, exposure=1.0, tonemap=0):
    """orc_display: [H, W, 3] float32 values written to the RGBA8 canvas before quantization."""
    h, w = color4.shape[:2]
    c, a = _c32(color4, (h, w, 4)), _c32(albedo4, (h, w, 4))
    d = _c32(denoised4 if denoised4 is not None else np.zeros((h, w, 4)), (h, w, 4))
    out = np.zeros((h, w, 3), np.float32)
    lib().orc_display(_p(c, F), _p(a, F), _p(d, F), w, h, denoise_weight, exposure, tonemap, _p(out, F))
    return out


def display_view(color4, albedo4, denoised4, view_w, view_h, denoise_weight, exposure=1.0, tonemap=0):
    """orc_display_view: the [H, W] targets shown in a view_h x view_w view (Catmull-Rom when the sizes
    differ), [view_h, view_w, 3] float32 values before quantization."""
    h, w = color4.shape[:2]
    c, a = _c32(color4, (h, w, 4)), _c32(albedo4, (h, w, 4))
    d = _c32(denoised4 if denoised4 is not None else np.zeros((h, w, 4)), (h, w, 4))
    out = np.zeros((view_h, view_w, 3), np.float32)
    lib().orc_display_view(_p(c, F), _p(a, F), _p(d, F), w, h, view_w, view_h, denoise_weight, exposure, tonemap,
                           _p(out, F))
    return out


def detached_dot(prep, width, height, seed0, samples, dl4, materials_eval=None, env_eval=None, max_bounces=6,
                 clamp=8.0, threads=0):
    """orc_detached_dot: sum_px dl4[px].rgb . mean radiance, sampling from
    prep's scene, BSDF values / environment radiance from the given
    materials (flat, 40 per material) and env map (flat RGB), binary64."""
    d = np.ascontiguousarray(dl4, np.float32).reshape(-1)
    m = np.ascontiguousarray(materials_eval, np.float32).reshape(-1) if materials_eval is not None else None
    e = np.ascontiguousarray(env_eval, np.float32).reshape(-1) if env_eval is not None else None
    return lib().orc_detached_dot(C.byref(prep.scene), C.byref(prep.camera), max_bounces, clamp, width, height, seed0,
                                  samples, _p(m, F) if m is not None else None, _p(e, F) if e is not None else None,
                                  _p(d, F), threads)


class OrcHistory(C.Structure):
    _fields_ = [("cam", P(OrcCamera)), ("w", U32), ("h", U32), ("color4", P(F)), ("albedo4", P(F)),
                ("normal4", P(F)), ("history", P(F))]


def camera_of(camera):
    """OrcCamera of a scene.Camera (the renderer's uploadCamera basis)."""
    from lucent_gb300 import scene as S
    f, r, u = S.camera_basis(camera)
    c = OrcCamera()
    c.pos[:] = camera.position
    c.right[:], c.up[:], c.forward[:] = r, u, f
    c.tan_half_fov = float(np.tan(camera.fov * np.pi / 360))
    c.aperture, c.focus_dist = camera.aperture, camera.focus_distance
    return c


def render_reproject(prep, camera, width, height, seed0, samples, prev_camera, prev, max_bounces=6, clamp=8.0,
                     precision=32, threads=0):
    """orc_render_reproject of the full width x height image with the view
    `camera` (OrcCamera), the first sample of each pixel starting from the
    previous view's targets `prev` = (color4, albedo4, normal4, history) seen
    from `prev_camera` (OrcCamera). Returns (color4, albedo4, normal4, history)."""
    L = lib()
    L.orc_render_reproject.argtypes = [P(OrcScene), P(OrcCamera), P(OrcHistory), U32, F, U32, U32, U32, U32, U32,
                                       U32, U32, U32, C.c_int, P(F), P(F), P(F), P(F), C.c_int]
    ph, pw = prev[3].shape
    arrs = [np.ascontiguousarray(a, np.float32) for a in prev]
    hist = OrcHistory(C.pointer(prev_camera), pw, ph, *[_p(a, F) for a in arrs])
    out = [np.zeros(width * height * 4, np.float32) for _ in range(3)] + [np.zeros(width * height, np.float32)]
    st = L.orc_render_reproject(C.byref(prep.scene), C.byref(camera), C.byref(hist), max_bounces, clamp, width,
                                height, 0, 0, width, height, seed0, samples, precision, *[_p(b, F) for b in out],
                                threads)
    if st:
        raise RuntimeError("orc_render_reproject failed")
    return (out[0].reshape(height, width, 4), out[1].reshape(height, width, 4), out[2].reshape(height, width, 4),
            out[3].reshape(height, width))
