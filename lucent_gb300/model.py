"""Models as scenes, mirroring the reference's src/loaders/model.ts.

load_model reads a .glb, or a .gltf with its buffers and images found next
to it (loadModelFiles, model.ts:80-93); decode_images turns the asset's
encoded images into textures, dropping the maps of an image that cannot be
decoded with the reference's warning (decodeImages, model.ts:43-72);
scene_from_model wraps the model in a scene: rescaled to a unit bounding
sphere, standing on an analytic ground plane, framed by the camera, volume
attenuation rescaled with the geometry (sceneFromModel, model.ts:129-166).
"""
import math
import os
import urllib.parse
from dataclasses import dataclass, replace
from typing import List, Optional

import numpy as np

from . import mesh as M
from . import scene as S
from .gltf import GLTFAsset, load_gltf
from .images import ImageDecodeError, decode_image


@dataclass
class LoadedModel:
    """LoadedModel (model.ts:16-21)."""
    name: str
    asset: GLTFAsset
    textures: List[S.Texture]
    warnings: List[str]


def default_sun(**kw):  # presets.ts:16-23
    return S.Sun(**{**dict(elevation=38.0, azimuth=215.0, color=(1.0, 0.93, 0.82), intensity=7.0,
                           angular_radius=1.2), **kw})


def day_sky(intensity=1.0):  # presets.ts:25-31
    return S.Sky(enabled=True, zenith=(0.22, 0.42, 0.85), horizon=(0.78, 0.86, 0.98), ground=(0.28, 0.25, 0.22),
                 intensity=intensity)


def decode_images(asset: GLTFAsset):
    """decodeImages (model.ts:43-72): (textures, warnings). An image that
    fails to decode becomes a 1x1 placeholder and every map using it is
    dropped from the materials."""
    textures, warnings = [], []
    for i, img in enumerate(asset.images):
        try:
            textures.append(S.Texture(decode_image(img.data, img.mime_type), img.name))
        except ImageDecodeError:
            warnings.append('could not decode image "%s"' % img.name)
            for m in asset.materials:
                for f in ("base_color_map", "metal_rough_map", "normal_map", "emissive_map"):
                    if getattr(m, f) == i:
                        setattr(m, f, -1)
            textures.append(S.Texture(np.zeros((1, 1, 4), np.uint8), img.name))
    return textures, warnings


def _normalize_path(uri):
    """normalizePath (model.ts:26-34)."""
    p = uri.split("?")[0].split("#")[0].replace("\\", "/")
    try:
        p = urllib.parse.unquote(p, errors="strict")
    except UnicodeDecodeError:
        pass
    return p[2:] if p.startswith("./") else p


def load_model(path: str, name: Optional[str] = None) -> LoadedModel:
    """A .glb or .gltf file; external buffers and images are looked up
    relative to its folder, then by file name in that folder."""
    folder = os.path.dirname(os.path.abspath(path))
    stem = os.path.splitext(os.path.basename(path))[0]

    def resolve(uri):
        rel = _normalize_path(uri)
        for cand in (os.path.join(folder, rel), os.path.join(folder, os.path.basename(rel))):
            if os.path.isfile(cand):
                with open(cand, "rb") as f:
                    return f.read()
        raise FileNotFoundError('"%s" is missing; keep it together with %s' % (rel, os.path.basename(path)))

    with open(path, "rb") as f:
        asset = load_gltf(f.read(), resolve)
    return model_from_asset(name or stem, asset)


def model_from_asset(name: str, asset: GLTFAsset) -> LoadedModel:
    """finish (model.ts:74-77)."""
    textures, warnings = decode_images(asset)
    return LoadedModel(name, asset, textures, asset.warnings + warnings)


def _place(mesh, offset, s):
    """placeMesh (model.ts:103-111)."""
    p = ((mesh.positions.astype(np.float64).reshape(-1, 3) - np.array(offset)) * s).astype(np.float32).reshape(-1)
    return M.Mesh(p, mesh.normals, mesh.uvs)


def scene_from_model(model: LoadedModel, env: S.Environment, azimuth=30.0, elevation=14.0, distance=1.1,
                     exposure=1.0, ground_color=(0.4, 0.4, 0.42), ground_roughness=0.9) -> S.Scene:
    """sceneFromModel (model.ts:129-166)."""
    lo, hi = model.asset.bounds
    radius = 0.5 * math.sqrt(sum((hi[i] - lo[i]) ** 2 for i in range(3))) or 1.0
    s = 1.0 / radius
    offset = ((lo[0] + hi[0]) / 2, lo[1], (lo[2] + hi[2]) / 2)
    mats = [replace(m, attenuation_distance=m.attenuation_distance * s) if math.isfinite(m.attenuation_distance)
            else m for m in model.asset.materials]
    height = (hi[1] - lo[1]) * s
    half_width = 0.5 * max(hi[0] - lo[0], hi[2] - lo[2]) * s
    fov = 40.0
    tan = math.tan(fov * math.pi / 360)
    target = (0.0, height / 2, 0.0)
    dist = max(height / 2 / tan, half_width / (tan * 1.5)) * distance + half_width
    az, el = azimuth * math.pi / 180, elevation * math.pi / 180
    position = (target[0] + dist * math.sin(az) * math.cos(el), target[1] + dist * math.sin(el),
                target[2] + dist * math.cos(az) * math.cos(el))
    return S.Scene(
        name=model.name,
        camera=S.Camera(position=position, target=target, fov=fov, aperture=0.0, focus_distance=dist),
        sun=default_sun(), sky=day_sky(1.0), env=env,
        # a hair below the model so flat bases do not z-fight with the plane
        ground=S.Ground(enabled=True, height=-1e-3, material=S.matte(ground_color, ground_roughness)),
        spheres=[],
        meshes=[S.MeshInstance(_place(mesh, offset, s), mats[mi]) for mesh, mi in model.asset.meshes],
        exposure=exposure,
        textures=model.textures,
    )
