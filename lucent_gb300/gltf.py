"""glTF 2.0 / GLB ingestion, mirroring the reference's src/loaders/gltf.ts.

load_gltf turns a .glb or .gltf file into world-space meshes (one per
primitive), materials of the layered model and the encoded images that some
material samples, with the reference's rules and error messages:

* GLB container: magic, version 2, JSON chunk, first BIN chunk (gltf.ts:58-82);
* buffers from the GLB chunk, data URIs or a resolver (gltf.ts:208-217);
* accessors of every component type, normalized integers, byte strides and
  sparse overrides, read into float32 (gltf.ts:229-281);
* node hierarchy with matrices or T·R·S, normals by the inverse transpose,
  winding kept under mirroring transforms, flat normals when NORMAL is
  missing, triangle lists, strips and fans (gltf.ts:384-497);
* metal-rough materials with the emissive-strength, transmission, ior,
  volume, clearcoat, sheen and unlit extensions, KHR_texture_transform, and
  glTF's default material (gltf.ts:324-377);
* images fetched only when a material uses them (gltf.ts:283-322).

Geometry is read and transformed with numpy; arithmetic that decides stored
values (the world transform, normal transform) is evaluated in binary64 in
the reference's operation order and rounded once to binary32.
"""
import base64
import json as _json
import math
import struct
import urllib.parse
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Tuple

import numpy as np

from . import mesh as M
from .scene import Material

GLB_MAGIC = 0x46546C67
CHUNK_JSON = 0x4E4F534A
CHUNK_BIN = 0x004E4942

UNSUPPORTED_REQUIRED = {  # gltf.ts:40-46
    "KHR_draco_mesh_compression", "EXT_meshopt_compression", "KHR_texture_basisu", "MSFT_texture_dds",
    "EXT_mesh_gpu_instancing",
}
HANDLED_MATERIAL_EXTENSIONS = {  # gltf.ts:48-56
    "KHR_materials_emissive_strength", "KHR_materials_transmission", "KHR_materials_ior", "KHR_materials_volume",
    "KHR_materials_clearcoat", "KHR_materials_sheen", "KHR_materials_unlit",
}
COMPONENTS = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT2": 4, "MAT3": 9, "MAT4": 16}
# componentType -> (little-endian dtype, normalized divisor, normalized lower clamp)
COMPONENT_TYPES = {
    5120: ("<i1", 127.0, -1.0), 5121: ("<u1", 255.0, None), 5122: ("<i2", 32767.0, -1.0),
    5123: ("<u2", 65535.0, None), 5125: ("<u4", None, None), 5126: ("<f4", None, None),
}
IDENTITY_UV = (1.0, 0.0, 0.0, 0.0, 1.0, 0.0)


class GLTFError(ValueError):
    """A file the loader refuses (the reference throws an Error with the same text)."""


@dataclass
class GLTFImage:
    data: bytes
    mime_type: str
    name: str


@dataclass
class GLTFAsset:
    """GLTFAsset (gltf.ts:17-27): meshes already in world space; `material`
    indexes `materials`; material map fields index `images`."""
    meshes: List[Tuple[M.Mesh, int]]
    materials: List[Material]
    images: List[GLTFImage]
    bounds: Tuple[Tuple[float, float, float], Tuple[float, float, float]]
    triangle_count: int
    warnings: List[str] = field(default_factory=list)


Resolver = Callable[[str], bytes]


def is_glb(buf) -> bool:
    return len(buf) >= 12 and struct.unpack_from("<I", buf, 0)[0] == GLB_MAGIC


def parse_glb(buf):
    """parseGLB (gltf.ts:62-82): (json, bin chunk or None)."""
    buf = bytes(buf)
    if not is_glb(buf):
        raise GLTFError("not a GLB file (bad magic)")
    version, declared = struct.unpack_from("<II", buf, 4)
    if version != 2:
        raise GLTFError("GLB version %d is not supported; only glTF 2.0" % version)
    end = min(declared, len(buf))
    at, doc, bin_chunk = 12, None, None
    while at + 8 <= end:
        length, kind = struct.unpack_from("<II", buf, at)
        start = at + 8
        if start + length > end:
            raise GLTFError("GLB chunk runs past the end of the file")
        if kind == CHUNK_JSON:
            doc = _json.loads(buf[start:start + length].decode("utf-8"))
        elif kind == CHUNK_BIN and bin_chunk is None:
            bin_chunk = buf[start:start + length]
        at = start + length + (-length % 4)
    if doc is None:
        raise GLTFError("GLB has no JSON chunk")
    return doc, bin_chunk


def decode_data_uri(uri: str) -> bytes:
    """decodeDataUri (gltf.ts:84-94)."""
    comma = uri.find(",")
    if comma < 0:
        raise GLTFError("malformed data URI")
    meta, payload = uri[5:comma], uri[comma + 1:]
    if not meta.endswith(";base64"):
        return urllib.parse.unquote(payload).encode("utf-8")
    return base64.b64decode(payload)


def _mime_from_data_uri(uri: str) -> str:
    head = uri[5:]
    end = min([i for i in (head.find(";"), head.find(",")) if i >= 0] or [len(head)])
    return head[:end]


def mime_from_name(name: str) -> str:
    """mimeFromName (gltf.ts:98-105)."""
    base = name.split("?")[0].split("#")[0]
    ext = base.rsplit(".", 1)[-1].lower() if "." in base else ""
    return {"png": "image/png", "jpg": "image/jpeg", "jpeg": "image/jpeg", "webp": "image/webp",
            "ktx2": "image/ktx2"}.get(ext, "application/octet-stream")


def compose_trs(t, q, s):
    """composeTRS (gltf.ts:144-161): column-major T·R·S as 16 binary64 values."""
    x, y, z, w = (float(c) for c in q)
    m = np.zeros(16, np.float64)
    m[0] = (1 - 2 * (y * y + z * z)) * s[0]
    m[1] = 2 * (x * y + z * w) * s[0]
    m[2] = 2 * (x * z - y * w) * s[0]
    m[4] = 2 * (x * y - z * w) * s[1]
    m[5] = (1 - 2 * (x * x + z * z)) * s[1]
    m[6] = 2 * (y * z + x * w) * s[1]
    m[8] = 2 * (x * z + y * w) * s[2]
    m[9] = 2 * (y * z - x * w) * s[2]
    m[10] = (1 - 2 * (x * x + y * y)) * s[2]
    m[12:15] = t[0], t[1], t[2]
    m[15] = 1.0
    return m


def _multiply(a, b):
    """Column-major a·b; each sum in k order like gltf.ts:131-141."""
    out = np.zeros(16, np.float64)
    for c in range(4):
        for r in range(4):
            s = 0.0
            for k in range(4):
                s += a[k * 4 + r] * b[c * 4 + k]
            out[c * 4 + r] = s
    return out


def _normal_matrix(m):
    """normalMatrix (gltf.ts:164-178): row-major inverse transpose of the 3×3 and its determinant."""
    a, b, c = m[0], m[4], m[8]
    d, e, f = m[1], m[5], m[9]
    g, h, i = m[2], m[6], m[10]
    A, B, C = e * i - f * h, -(d * i - f * g), d * h - e * g
    det = a * A + b * B + c * C
    inv = 0.0 if det == 0 else 1.0 / det
    n = [A * inv, B * inv, C * inv,
         -(b * i - c * h) * inv, (a * i - c * g) * inv, -(a * h - b * g) * inv,
         (b * f - c * e) * inv, -(a * f - c * d) * inv, (a * e - b * d) * inv]
    return n, det


def texture_transform(ext):
    """textureTransform (gltf.ts:181-189): KHR_texture_transform as a row-major 2×3 matrix."""
    if not ext:
        return IDENTITY_UV
    ox, oy = ext.get("offset", [0, 0])
    sx, sy = ext.get("scale", [1, 1])
    r = ext.get("rotation", 0)
    c, s = math.cos(r), math.sin(r)
    return (c * sx, -s * sy, float(ox), s * sx, c * sy, float(oy))


def _no_resolver(uri):
    raise GLTFError('"%s" is missing: no resolver for external resources' % uri)


def load_gltf(source, resolve: Optional[Resolver] = None) -> GLTFAsset:
    """loadGLTF (gltf.ts:191-502) on the bytes of a .glb or .gltf file;
    `resolve(uri) -> bytes` fetches external buffers and images."""
    resolve = resolve or _no_resolver
    source = bytes(source)
    glb_bin = None
    if is_glb(source):
        doc, glb_bin = parse_glb(source)
    else:
        doc = _json.loads(source.decode("utf-8"))
    version = str(((doc or {}).get("asset") or {}).get("version", ""))
    if not version.startswith("2"):
        raise GLTFError('glTF version "%s" is not supported; only 2.0' % (version or "unknown"))
    warnings: List[str] = []

    def warn(msg):
        if msg not in warnings:
            warnings.append(msg)

    for ext in doc.get("extensionsRequired", []) or []:
        if ext in UNSUPPORTED_REQUIRED:
            raise GLTFError("this file requires %s, which Lucent does not support" % ext)

    buffers = []
    for i, b in enumerate(doc.get("buffers", []) or []):
        uri = b.get("uri")
        if uri is None:
            if i == 0 and glb_bin is not None:
                buffers.append(glb_bin)
                continue
            raise GLTFError("buffer %d has no uri and there is no GLB binary chunk" % i)
        buffers.append(decode_data_uri(uri) if str(uri).startswith("data:") else bytes(resolve(uri)))

    views = doc.get("bufferViews", []) or []

    def view_bytes(index):
        if index is None or not (0 <= index < len(views)):
            raise GLTFError("missing bufferView %s" % index)
        v = views[index]
        if not (0 <= v.get("buffer", -1) < len(buffers)):
            raise GLTFError("bufferView %d references missing buffer %s" % (index, v.get("buffer")))
        buf = buffers[v["buffer"]]
        start = v.get("byteOffset", 0)
        if start + v["byteLength"] > len(buf):
            raise GLTFError("bufferView %d runs past its buffer" % index)
        return buf[start:start + v["byteLength"]], v.get("byteStride", 0)

    accessors = doc.get("accessors", []) or []
    cache = {}

    def read_elements(data, dtype, offset, step, count, size):
        """count elements of `size` components starting at `offset`, `step` bytes apart."""
        if count == 0:
            return np.zeros((0, size), dtype)
        arr = np.ndarray((count, size), dtype=np.dtype(dtype), buffer=data, offset=offset,
                         strides=(step, np.dtype(dtype).itemsize))
        return np.array(arr)

    def to_float(raw, ctype, normalized):
        _, div, lo = COMPONENT_TYPES[ctype]
        if normalized and div is not None:
            x = raw.astype(np.float64) / div
            if lo is not None:
                x = np.maximum(x, lo)
            return x.astype(np.float32)
        return raw.astype(np.float32)

    def read_accessor(index):
        if index in cache:
            return cache[index]
        if not (isinstance(index, int) and 0 <= index < len(accessors)):
            raise GLTFError("missing accessor %s" % index)
        acc = accessors[index]
        size = COMPONENTS.get(acc.get("type"))
        ctype = acc.get("componentType")
        if not size or ctype not in COMPONENT_TYPES:
            raise GLTFError("accessor %d has unsupported type %s/%s" % (index, acc.get("type"), ctype))
        dtype = COMPONENT_TYPES[ctype][0]
        comp = np.dtype(dtype).itemsize
        count = int(acc["count"])
        normalized = acc.get("normalized") is True
        out = np.zeros((count, size), np.float32)
        if acc.get("bufferView") is not None:
            data, stride = view_bytes(acc["bufferView"])
            elem = size * comp
            step = stride or elem
            base = acc.get("byteOffset", 0)
            if count > 0 and base + step * (count - 1) + elem > len(data):
                raise GLTFError("accessor %d reads past its bufferView" % index)
            out = to_float(read_elements(data, dtype, base, step, count, size), ctype, normalized)
        sparse = acc.get("sparse")
        if sparse:
            n = int(sparse["count"])
            idx_info, val_info = sparse["indices"], sparse["values"]
            idata, _ = view_bytes(idx_info.get("bufferView"))
            vdata, _ = view_bytes(val_info.get("bufferView"))
            itype = idx_info["componentType"]
            idt = COMPONENT_TYPES[itype][0]
            targets = read_elements(idata, idt, idx_info.get("byteOffset", 0), np.dtype(idt).itemsize, n, 1)[:, 0]
            values = to_float(read_elements(vdata, dtype, val_info.get("byteOffset", 0), size * comp, n, size),
                              ctype, normalized)
            for k in range(n):
                t = int(targets[k])
                if t >= count:
                    raise GLTFError("sparse index %d out of range in accessor %d" % (t, index))
                out[t] = values[k]
        cache[index] = out
        return out

    images_doc = doc.get("images", []) or []
    textures_doc = doc.get("textures", []) or []
    image_slot = {}
    images: List[GLTFImage] = []

    def use_image(index):
        if index in image_slot:
            return image_slot[index]
        if not (isinstance(index, int) and 0 <= index < len(images_doc)):
            return -1
        img = images_doc[index]
        name = str(img.get("name", img.get("uri", "image %d" % index)))
        if img.get("bufferView") is not None:
            data, _ = view_bytes(img["bufferView"])
            entry = GLTFImage(bytes(data), img.get("mimeType", "image/png"), name)
        else:
            uri = str(img.get("uri"))
            if uri.startswith("data:"):
                entry = GLTFImage(decode_data_uri(uri), _mime_from_data_uri(uri), name)
            else:
                entry = GLTFImage(bytes(resolve(uri)), img.get("mimeType", mime_from_name(uri)), name)
        image_slot[index] = len(images)
        images.append(entry)
        return image_slot[index]

    def texture_slot(info):
        if not info or info.get("index") is None:
            return -1
        ti = info["index"]
        if not (0 <= ti < len(textures_doc)):
            return -1
        tex = textures_doc[ti]
        if info.get("texCoord", 0) != 0:
            warn("textures on TEXCOORD_1 or higher are sampled with TEXCOORD_0")
        exts = tex.get("extensions", {}) or {}
        src = (exts.get("EXT_texture_webp") or {}).get("source", tex.get("source"))
        if src is None:
            if exts.get("KHR_texture_basisu"):
                warn("KTX2/Basis textures are not supported and were skipped")
            return -1
        img = images_doc[src] if 0 <= src < len(images_doc) else {}
        mime = img.get("mimeType", mime_from_name(str(img.get("uri", ""))))
        if mime == "image/ktx2":
            warn("KTX2/Basis textures are not supported and were skipped")
            return -1
        return use_image(src)

    def convert_material(m):
        pbr = m.get("pbrMetallicRoughness", {}) or {}
        ext = m.get("extensions", {}) or {}
        for name in ext:
            if name not in HANDLED_MATERIAL_EXTENSIONS:
                warn("material extension %s is ignored" % name)
        bc = pbr.get("baseColorFactor", [1, 1, 1, 1])
        strength = (ext.get("KHR_materials_emissive_strength") or {}).get("emissiveStrength", 1)
        ef = m.get("emissiveFactor", [0, 0, 0])
        transform_src = next((t for t in (pbr.get("baseColorTexture"), pbr.get("metallicRoughnessTexture"),
                                          m.get("normalTexture"), m.get("emissiveTexture"))
                              if t and (t.get("extensions") or {}).get("KHR_texture_transform")), None)
        volume = ext.get("KHR_materials_volume")
        mode = {"MASK": "mask", "BLEND": "blend"}.get(m.get("alphaMode"), "opaque")
        coat = ext.get("KHR_materials_clearcoat") or {}
        sheen = ext.get("KHR_materials_sheen") or {}
        out = Material(
            albedo=(float(bc[0]), float(bc[1]), float(bc[2])),
            alpha=float(bc[3]) if len(bc) > 3 else 1.0,
            alpha_mode=mode,
            alpha_cutoff=float(m.get("alphaCutoff", 0.5)),
            metallic=float(pbr.get("metallicFactor", 1)),
            roughness=float(pbr.get("roughnessFactor", 1)),
            base_color_map=texture_slot(pbr.get("baseColorTexture")),
            metal_rough_map=texture_slot(pbr.get("metallicRoughnessTexture")),
            normal_map=texture_slot(m.get("normalTexture")),
            normal_scale=float((m.get("normalTexture") or {}).get("scale", 1)),
            emissive_map=texture_slot(m.get("emissiveTexture")),
            emission=(ef[0] * strength, ef[1] * strength, ef[2] * strength),
            transmission=float((ext.get("KHR_materials_transmission") or {}).get("transmissionFactor", 0)),
            ior=float((ext.get("KHR_materials_ior") or {}).get("ior", 1.5)),
            thin_walled=not volume or (volume.get("thicknessFactor", 0) or 0) == 0,
            attenuation_color=tuple(float(c) for c in (volume or {}).get("attenuationColor", [1, 1, 1])),
            attenuation_distance=float((volume or {}).get("attenuationDistance", math.inf)),
            clearcoat=float(coat.get("clearcoatFactor", 0)),
            clearcoat_roughness=float(coat.get("clearcoatRoughnessFactor", 0)),
            sheen_color=tuple(float(c) for c in sheen.get("sheenColorFactor", [0, 0, 0])),
            sheen_roughness=float(sheen.get("sheenRoughnessFactor", 0)),
            uv_transform=texture_transform(((transform_src or {}).get("extensions") or {}).get("KHR_texture_transform")),
        )
        if "KHR_materials_unlit" in ext:
            out.emission, out.emissive_map = out.albedo, out.base_color_map
            out.albedo, out.metallic = (0.0, 0.0, 0.0), 0.0
        return out

    materials = [convert_material(m) for m in doc.get("materials", []) or []]
    default = [-1]

    def material_for(index):
        if isinstance(index, int) and 0 <= index < len(materials):
            return index
        if default[0] < 0:  # glTF's default material: white, fully metallic, fully rough
            default[0] = len(materials)
            materials.append(Material(albedo=(1.0, 1.0, 1.0), metallic=1.0, roughness=1.0))
        return default[0]

    meshes: List[Tuple[M.Mesh, int]] = []
    lo = np.full(3, np.inf)
    hi = np.full(3, -np.inf)
    count = [0]

    def emit(prim, world):
        mode = prim.get("mode", 4)
        if mode not in (4, 5, 6):
            warn("point and line primitives are skipped")
            return
        if (prim.get("extensions") or {}).get("KHR_draco_mesh_compression"):
            raise GLTFError("Draco-compressed meshes are not supported")
        attrs = prim.get("attributes", {}) or {}
        if attrs.get("POSITION") is None:
            return
        pos = read_accessor(attrs["POSITION"])
        nrm = read_accessor(attrs["NORMAL"]) if attrs.get("NORMAL") is not None else None
        uv = read_accessor(attrs["TEXCOORD_0"]) if attrs.get("TEXCOORD_0") is not None else None
        nvert = pos.shape[0]
        if prim.get("indices") is not None:
            verts = read_accessor(prim["indices"])[:, 0].astype(np.int64)
        else:
            verts = np.arange(nvert, dtype=np.int64)
        n = verts.size
        if mode == 4:
            k = (n // 3) * 3
            tris = verts[:k].reshape(-1, 3)
        elif mode == 5:  # strips: odd triangles swap their last two corners
            k = np.arange(max(n - 2, 0))
            a, b, c = verts[k], verts[k + 1], verts[k + 2]
            odd = (k % 2) == 1
            tris = np.stack([a, np.where(odd, c, b), np.where(odd, b, c)], 1)
        else:  # fans
            k = np.arange(1, max(n - 1, 1))
            tris = np.stack([verts[k], verts[k + 1], np.full(k.size, verts[0] if n else 0)], 1)
        if tris.shape[0] == 0:
            return
        nm, det = _normal_matrix(world)
        if det < 0:  # mirroring reverses winding: swap two corners
            tris = tris[:, [0, 2, 1]]
        flat = tris.reshape(-1)
        if flat.max() >= nvert:
            bad = int(flat[flat >= nvert][0])
            raise GLTFError("index %d out of range (%d vertices)" % (bad, nvert))
        p = pos[flat].astype(np.float64)
        x, y, z = p[:, 0], p[:, 1], p[:, 2]
        W = world
        wp = np.stack([W[0] * x + W[4] * y + W[8] * z + W[12],
                       W[1] * x + W[5] * y + W[9] * z + W[13],
                       W[2] * x + W[6] * y + W[10] * z + W[14]], 1)
        positions = wp.astype(np.float32)
        lo[:] = np.minimum(lo, wp.min(0))
        hi[:] = np.maximum(hi, wp.max(0))
        if nrm is not None:
            q = nrm[flat].astype(np.float64)
            a, b, d = q[:, 0], q[:, 1], q[:, 2]
            nn = np.stack([nm[0] * a + nm[1] * b + nm[2] * d,
                           nm[3] * a + nm[4] * b + nm[5] * d,
                           nm[6] * a + nm[7] * b + nm[8] * d], 1)
            length = np.sqrt((nn * nn).sum(1))
            length[length == 0] = 1.0
            normals = (nn / length[:, None]).astype(np.float32)
        else:  # glTF: missing normals mean flat shading
            tp = positions.astype(np.float64).reshape(-1, 3, 3)
            cr = np.cross(tp[:, 1] - tp[:, 0], tp[:, 2] - tp[:, 0])
            length = np.sqrt((cr * cr).sum(1))
            length[length == 0] = 1.0
            normals = np.repeat((cr / length[:, None]).astype(np.float32), 3, axis=0)
        uvs = uv[flat, :2].astype(np.float32).reshape(-1) if uv is not None else None
        count[0] += tris.shape[0]
        meshes.append((M.Mesh(positions.reshape(-1), normals.reshape(-1), uvs), material_for(prim.get("material"))))

    nodes = doc.get("nodes", []) or []
    meshes_doc = doc.get("meshes", []) or []

    def visit(index, parent, depth):
        if depth > 64:
            raise GLTFError("node hierarchy is deeper than 64 levels (cycle?)")
        if not (isinstance(index, int) and 0 <= index < len(nodes)):
            raise GLTFError("missing node %s" % index)
        node = nodes[index]
        if node.get("matrix") is not None:
            local = np.array(node["matrix"], np.float64)
        else:
            local = compose_trs(node.get("translation", [0, 0, 0]), node.get("rotation", [0, 0, 0, 1]),
                                node.get("scale", [1, 1, 1]))
        world = _multiply(parent, local)
        if node.get("mesh") is not None:
            mi = node["mesh"]
            if not (0 <= mi < len(meshes_doc)):
                raise GLTFError("node %d references missing mesh %s" % (index, mi))
            for prim in meshes_doc[mi].get("primitives", []) or []:
                emit(prim, world)
        for child in node.get("children", []) or []:
            visit(child, world, depth + 1)

    scenes = doc.get("scenes", []) or []
    si = doc.get("scene", 0)
    if isinstance(si, int) and 0 <= si < len(scenes):
        roots = scenes[si].get("nodes", []) or []
    else:
        children = {c for nd in nodes for c in (nd.get("children", []) or [])}
        roots = [i for i in range(len(nodes)) if i not in children]
    identity = np.zeros(16, np.float64)
    identity[[0, 5, 10, 15]] = 1.0
    for r in roots:
        visit(r, identity, 0)
    if count[0] == 0:
        raise GLTFError("the file contains no triangle meshes")
    bounds = (tuple(float(v) for v in lo), tuple(float(v) for v in hi))
    return GLTFAsset(meshes, materials, images, bounds, count[0], warnings)


def write_glb(doc, bin_bytes=None) -> bytes:
    """A GLB container (glTF 2.0 binary): the JSON chunk padded with spaces,
    the BIN chunk padded with zeros (the layout parse_glb reads)."""
    js = _json.dumps(doc, separators=(",", ":")).encode("utf-8")
    js += b" " * (-len(js) % 4)
    body = struct.pack("<II", len(js), CHUNK_JSON) + js
    if bin_bytes is not None:
        b = bytes(bin_bytes) + b"\0" * (-len(bin_bytes) % 4)
        body += struct.pack("<II", len(b), CHUNK_BIN) + b
    return struct.pack("<III", GLB_MAGIC, 2, 12 + len(body)) + body
