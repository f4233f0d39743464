"""Scene model mirroring the reference's src/scene/{scene,material,environment}.ts.

`pack_scene` performs packScene's host work (scene.ts:162-305): material
deduplication by identity, the per-triangle material / light / alpha arrays,
emissive quads and spheres turned into explicit lights, the sphere table and
the ground material. The BVH-order gather of triangle data runs on the GPU
(lucent_renderer_load_scene). `lighting` computes uploadLighting's uniforms
(renderer.ts:355-413) and bakes the procedural sky (environment.ts:106-132).
"""
import math
from dataclasses import dataclass, field, replace
from typing import List, Optional, Tuple

import numpy as np

from . import mesh as M

Vec3 = Tuple[float, float, float]

MAX_SPHERES = 64  # scene.ts:79
MAX_LIGHTS = 8  # scene.ts:80
MATERIAL_TEXELS = 10  # material.ts:121
ALPHA_CODE = {"opaque": 0, "mask": 1, "blend": 2}  # material.ts:125


@dataclass(eq=False)
class Material:
    """material.ts:17-57 with DEFAULT_MATERIAL (material.ts:61-86). Compared by identity."""
    albedo: Vec3 = (0.8, 0.8, 0.8)
    metallic: float = 0.0
    roughness: float = 0.5
    transmission: float = 0.0
    ior: float = 1.5
    emission: Vec3 = (0.0, 0.0, 0.0)
    checker_scale: float = 0.0
    albedo2: Vec3 = (0.2, 0.2, 0.2)
    alpha: float = 1.0
    alpha_mode: str = "opaque"
    alpha_cutoff: float = 0.5
    clearcoat: float = 0.0
    clearcoat_roughness: float = 0.0
    sheen_color: Vec3 = (0.0, 0.0, 0.0)
    sheen_roughness: float = 0.0
    thin_walled: bool = False
    attenuation_color: Vec3 = (1.0, 1.0, 1.0)
    attenuation_distance: float = math.inf
    base_color_map: int = -1
    metal_rough_map: int = -1
    normal_map: int = -1
    emissive_map: int = -1
    normal_scale: float = 1.0
    uv_transform: Tuple[float, float, float, float, float, float] = (1, 0, 0, 0, 1, 0)


def material(**kw):
    return Material(**kw)


def matte(albedo, roughness=1.0):  # material.ts:92
    return Material(albedo=tuple(albedo), roughness=roughness)


def metal(albedo, roughness=0.1):  # material.ts:93-94
    return Material(albedo=tuple(albedo), metallic=1.0, roughness=roughness)


def glass(albedo=(1.0, 1.0, 1.0), ior=1.5, roughness=0.0):  # material.ts:95-96
    return Material(albedo=tuple(albedo), transmission=1.0, ior=ior, roughness=roughness)


def light(color, strength):  # material.ts:97-101
    return Material(albedo=(0.0, 0.0, 0.0), emission=tuple(c * strength for c in color))


def is_emissive(m):  # material.ts:105
    return m.emission[0] > 0 or m.emission[1] > 0 or m.emission[2] > 0


def needs_alpha_test(m):  # material.ts:111
    return m.alpha_mode != "opaque" and (m.alpha < 1 or m.base_color_map >= 0)


def pack_materials(mats):
    """packMaterials (material.ts:132-149): 10 RGBA texels (40 floats) per material."""
    out = np.zeros((len(mats), 40), np.float32)
    for i, m in enumerate(mats):
        uv = m.uv_transform
        out[i] = [*m.albedo, m.metallic, m.roughness, m.ior, m.transmission, m.checker_scale, *m.emission, m.alpha,
                  *m.albedo2, ALPHA_CODE[m.alpha_mode], m.base_color_map, m.metal_rough_map, m.normal_map,
                  m.emissive_map, m.normal_scale, m.clearcoat, m.clearcoat_roughness, m.alpha_cutoff,
                  *m.sheen_color, m.sheen_roughness, *m.attenuation_color,
                  m.attenuation_distance if math.isfinite(m.attenuation_distance) else 0.0,
                  uv[0], uv[1], uv[2], 1.0 if m.thin_walled else 0.0, uv[3], uv[4], uv[5], 0.0]
    return out.reshape(-1)


@dataclass
class Camera:
    """scene.ts:10-19."""
    position: Vec3 = (0.0, 0.0, 5.0)
    target: Vec3 = (0.0, 0.0, 0.0)
    fov: float = 45.0
    aperture: float = 0.0
    focus_distance: float = 5.0


@dataclass
class Sun:
    """scene.ts:21-30."""
    elevation: float = 45.0
    azimuth: float = 0.0
    color: Vec3 = (1.0, 1.0, 1.0)
    intensity: float = 0.0
    angular_radius: float = 0.27


@dataclass
class Sky:
    """scene.ts:32-38."""
    enabled: bool = False
    zenith: Vec3 = (0.2, 0.4, 0.9)
    horizon: Vec3 = (0.8, 0.85, 0.95)
    ground: Vec3 = (0.3, 0.25, 0.2)
    intensity: float = 1.0


@dataclass
class HDRImage:
    """environment.ts:5-10: linear RGB, rows top to bottom."""
    width: int
    height: int
    data: np.ndarray


@dataclass
class Environment:
    """environment.ts:12-22."""
    map: Optional[HDRImage] = None
    name: str = "Procedural sky"
    rotation: float = 0.0
    intensity: float = 1.0
    background: bool = True
    backdrop: Vec3 = (0.02, 0.02, 0.025)


@dataclass
class Ground:
    enabled: bool = False
    height: float = 0.0
    material: Material = field(default_factory=lambda: matte((0.5, 0.5, 0.5)))


@dataclass
class Sphere:
    center: Vec3
    radius: float
    material: Material


@dataclass
class MeshInstance:
    mesh: M.Mesh
    material: Material


@dataclass
class Texture:
    """SceneTexture (scene.ts:58-62): a decoded image, 8-bit RGBA [h, w, 4],
    row 0 = top (v = 0), unpremultiplied; resampled on upload to the shared
    texture-array size."""
    image: np.ndarray
    name: str = "texture"


@dataclass
class Scene:
    """scene.ts:64-77."""
    name: str = "scene"
    camera: Camera = field(default_factory=Camera)
    sun: Sun = field(default_factory=Sun)
    sky: Sky = field(default_factory=Sky)
    env: Environment = field(default_factory=Environment)
    ground: Ground = field(default_factory=Ground)
    spheres: List[Sphere] = field(default_factory=list)
    meshes: List[MeshInstance] = field(default_factory=list)
    exposure: float = 1.0
    textures: List[Texture] = field(default_factory=list)


def quad_from_mesh(m):
    """quadFromMesh (scene.ts:312-324): parallelogram of a quad() mesh, else None."""
    if M.triangle_count(m) != 2:
        return None
    v = m.positions.astype(np.float64).reshape(6, 3)
    a, b, c, a2, c2, d = v
    same = lambda p, q: np.linalg.norm(p - q) < 1e-6
    if not same(a, a2) or not same(c, c2):
        return None
    e1, e2 = b - a, d - a
    if not same(a + e1 + e2, c) or np.linalg.norm(np.cross(e1, e2)) < 1e-9:
        return None
    return a, e1, e2


@dataclass
class PackedScene:
    positions: np.ndarray
    normals: np.ndarray
    uvs: Optional[np.ndarray]
    tri_material: np.ndarray
    tri_light: np.ndarray
    tri_alpha: np.ndarray
    materials: np.ndarray
    material_count: int
    spheres: np.ndarray
    sphere_materials: np.ndarray
    sphere_lights: np.ndarray
    lights: np.ndarray
    light_count: int
    ground_material: int
    # scene texture index in each layer of the sRGB (colour) and linear (data) arrays (scene.ts:124-126)
    color_layers: List[int] = field(default_factory=list)
    data_layers: List[int] = field(default_factory=list)

    @property
    def tri_count(self):
        return self.positions.size // 9


def _layer_map():
    """layerMap (scene.ts:136-154): one layer per referenced texture, in first-use order."""
    layers, index = [], {}

    def layer(tex):
        if tex < 0:
            return -1
        if tex not in index:
            index[tex] = len(layers)
            layers.append(tex)
        return index[tex]

    return layers, layer


def pack_scene(scene: Scene) -> PackedScene:
    """packScene (scene.ts:162-305) up to the BVH-order gather."""
    if len(scene.spheres) > MAX_SPHERES:
        raise ValueError("scene has %d spheres; max is %d" % (len(scene.spheres), MAX_SPHERES))
    mats, ids = [], {}

    def mindex(m):
        i = ids.get(id(m))
        if i is None:
            i = len(mats)
            mats.append(m)
            ids[id(m)] = i
        return i

    lights = []

    def add_light(rec):
        if len(lights) >= MAX_LIGHTS:
            return -1
        lights.append(rec)
        return len(lights) - 1

    merged = M.merge_meshes([mi.mesh for mi in scene.meshes]) if scene.meshes else M.Mesh(
        np.zeros(0, np.float32), np.zeros(0, np.float32))
    n = merged.positions.size // 9
    tri_mat = np.zeros(n, np.int32)
    tri_light = np.full(n, -1, np.int32)
    tri_alpha = np.zeros(n, np.uint8)
    cursor = 0
    for inst in scene.meshes:
        k = M.triangle_count(inst.mesh)
        tri_mat[cursor:cursor + k] = mindex(inst.material)
        if needs_alpha_test(inst.material):
            tri_alpha[cursor:cursor + k] = 1
        q = quad_from_mesh(inst.mesh) if is_emissive(inst.material) else None
        if q is not None:
            li = add_light(("quad", q[0], 0.0, q[1], q[2], inst.material.emission))
            tri_light[cursor:cursor + k] = li
        cursor += k
    spheres = np.zeros((MAX_SPHERES, 4), np.float32)
    sph_mat = np.zeros(MAX_SPHERES, np.int32)
    sph_light = np.full(MAX_SPHERES, -1, np.int32)
    for i, s in enumerate(scene.spheres):
        spheres[i] = [*s.center, s.radius]
        sph_mat[i] = mindex(s.material)
        if is_emissive(s.material):
            sph_light[i] = add_light(("sphere", s.center, s.radius, (0, 0, 0), (0, 0, 0), s.material.emission))
    ground_material = mindex(scene.ground.material)  # always packed (scene.ts:259-260)
    # sRGB maps (base colour, emissive) and linear maps (metal-rough, normal) get separate arrays (scene.ts:271-283)
    color_layers, color = _layer_map()
    data_layers, data = _layer_map()
    layered = [replace(m, base_color_map=color(m.base_color_map), emissive_map=color(m.emissive_map),
                       metal_rough_map=data(m.metal_rough_map), normal_map=data(m.normal_map)) for m in mats]
    for t in color_layers + data_layers:
        if t >= len(scene.textures):
            raise ValueError("material references texture %d, scene has %d" % (t, len(scene.textures)))
    lt = np.zeros((MAX_LIGHTS, 16), np.float32)
    for i, (kind, pos, radius, e1, e2, rad) in enumerate(lights):  # scene.ts:262-269
        lt[i] = [*pos, 0.0 if kind == "sphere" else 1.0, *e1, radius, *e2, 0.0, *rad, 0.0]
    return PackedScene(merged.positions, merged.normals, merged.uvs, tri_mat, tri_light, tri_alpha,
                       pack_materials(layered), len(mats), spheres.reshape(-1)[: 4 * len(scene.spheres)].copy(),
                       sph_mat[: len(scene.spheres)].copy(), sph_light[: len(scene.spheres)].copy(),
                       lt.reshape(-1)[: 16 * len(lights)].copy(), len(lights), ground_material,
                       color_layers, data_layers)


def from_spherical(elevation, azimuth):
    """vec3.ts:57-60 (radians, Y up)."""
    c = math.cos(elevation)
    return (c * math.sin(azimuth), math.sin(elevation), c * math.cos(azimuth))


def direction_from_uv(u, v):
    """environment.ts:88-93 (vectorised)."""
    phi = (u - 0.5) * 2 * math.pi
    theta = v * math.pi
    s = np.sin(theta)
    return s * np.cos(phi), np.cos(theta), s * np.sin(phi)


def bake_sky(sky: Sky, sun: Sun, width=1024) -> HDRImage:
    """bakeSky (environment.ts:106-132): gradient sky plus the sun's glow."""
    height = width // 2
    if not sky.enabled or sky.intensity <= 0:
        return HDRImage(width, height, np.zeros(width * height * 3, np.float32))
    sd = from_spherical(sun.elevation * math.pi / 180, sun.azimuth * math.pi / 180)
    sun_on = sun.intensity > 0 and sun.elevation > -sun.angular_radius
    x = (np.arange(width) + 0.5) / width
    y = (np.arange(height) + 0.5) / height
    X, Y = np.meshgrid(x, y)
    dx, dy, dz = direction_from_uv(X, Y)
    t = dy
    out = np.zeros((height, width, 3), np.float32)  # the reference's Float32Array: every store rounds
    for c in range(3):
        up = sky.horizon[c] + (sky.zenith[c] - sky.horizon[c]) * np.power(np.maximum(t, 0), 0.55)
        dn = sky.horizon[c] + (sky.ground[c] - sky.horizon[c]) * np.minimum(1, -t * 4)
        out[..., c] = np.where(t >= 0, up, dn)
    if sun_on:
        s = np.maximum(0, dx * sd[0] + dy * sd[1] + dz * sd[2])
        glow = 0.12 * s ** 24 + 0.5 * s ** 400
        for c in range(3):
            out[..., c] = out[..., c].astype(np.float64) + sun.color[c] * glow
    for c in range(3):
        out[..., c] = out[..., c].astype(np.float64) * sky.intensity
    return HDRImage(width, height, out.reshape(-1))


@dataclass
class Lighting:
    """uploadLighting's uniforms (renderer.ts:355-413)."""
    sun_enabled: int
    sun_dir: Vec3
    sun_radiance: Vec3
    sun_cos_angle: float
    sun_pdf: float
    env: HDRImage
    env_rotation: Tuple[float, float]
    env_intensity: float
    env_background: int
    backdrop: Vec3


def lighting(scene: Scene) -> Lighting:
    sun, sky, env = scene.sun, scene.sky, scene.env
    d = from_spherical(sun.elevation * math.pi / 180, sun.azimuth * math.pi / 180)
    cos_angle = math.cos(sun.angular_radius * math.pi / 180)
    solid = 2 * math.pi * (1 - cos_angle)
    enabled = env.map is None and sun.intensity > 0 and sun.elevation > -sun.angular_radius
    img = env.map if env.map is not None else bake_sky(sky, sun)
    rot = env.rotation * math.pi / 180 if env.map is not None else 0.0
    return Lighting(1 if enabled else 0, d, tuple(c * sun.intensity / solid for c in sun.color), cos_angle,
                    1 / solid if solid > 0 else 0.0, img, (math.cos(rot), math.sin(rot)),
                    env.intensity if env.map is not None else 1.0, 1 if env.background else 0, env.backdrop)


def camera_basis(cam: Camera):
    """cameraBasis (renderer.ts:156-161)."""
    f = np.asarray(cam.target, np.float64) - np.asarray(cam.position, np.float64)
    f = f / np.linalg.norm(f)
    world_up = np.array([0.0, 0.0, 1.0]) if abs(f[1]) > 0.999 else np.array([0.0, 1.0, 0.0])
    r = np.cross(f, world_up)
    r = r / np.linalg.norm(r)
    return f, r, np.cross(r, f)
