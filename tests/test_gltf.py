"""Model ingestion on the CPU: the glTF/GLB parser (lucent_gb300/gltf.py)
against the reference's own parser tests (test/gltf.test.ts) restated on the
same inputs, texture-layer packing (test/scene.test.ts:121-166), the PNG
decoder, and the model-to-scene wrapper (src/loaders/model.ts)."""
import base64
import json
import math
import struct
import zlib

import numpy as np
import pytest

from lucent_gb300 import gltf as G
from lucent_gb300 import images as I
from lucent_gb300 import mesh as M
from lucent_gb300 import model as MD
from lucent_gb300 import scene as S

FLOAT = 5126


def make_glb(doc, bin_bytes=None):
    """A GLB container (JSON chunk padded with spaces, BIN chunk with zeros)."""
    js = json.dumps(doc).encode()
    js += b" " * (-len(js) % 4)
    out = struct.pack("<III", G.GLB_MAGIC, 2, 0) + struct.pack("<II", len(js), G.CHUNK_JSON) + js
    if bin_bytes is not None:
        b = bytes(bin_bytes) + b"\0" * (-len(bin_bytes) % 4)
        out += struct.pack("<II", len(b), G.CHUNK_BIN) + b
    return out[:8] + struct.pack("<I", len(out)) + out[12:]


def pack(*parts):
    """Concatenated, each part 4-byte aligned: (bytes, offsets)."""
    data, offsets = b"", []
    for p in parts:
        offsets.append(len(data))
        raw = np.ascontiguousarray(p).tobytes()
        data += raw + b"\0" * (-len(raw) % 4)
    return data, offsets


def triangle_glb(node=None, extra=None):
    """One triangle in the XY plane facing +Z, with normals, UVs, indices and an embedded image."""
    positions = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32)
    normals = np.array([0, 0, 1, 0, 0, 1, 0, 0, 1], np.float32)
    uvs = np.array([0, 0, 1, 0, 0, 1], np.float32)
    indices = np.array([0, 1, 2], np.uint16)
    png = np.array([0x89, 0x50, 0x4E, 0x47], np.uint8)
    data, off = pack(positions, normals, uvs, indices, png)
    doc = {
        "asset": {"version": "2.0"}, "scene": 0, "scenes": [{"nodes": [0]}],
        "nodes": [{"mesh": 0, **(node or {})}],
        "meshes": [{"primitives": [{"attributes": {"POSITION": 0, "NORMAL": 1, "TEXCOORD_0": 2}, "indices": 3,
                                    "material": 0}]}],
        "materials": [{"pbrMetallicRoughness": {"baseColorTexture": {"index": 0},
                                                "baseColorFactor": [1, 0.5, 0.25, 1]}}],
        "textures": [{"source": 0}],
        "images": [{"bufferView": 4, "mimeType": "image/png"}],
        "accessors": [
            {"bufferView": 0, "componentType": FLOAT, "count": 3, "type": "VEC3"},
            {"bufferView": 1, "componentType": FLOAT, "count": 3, "type": "VEC3"},
            {"bufferView": 2, "componentType": FLOAT, "count": 3, "type": "VEC2"},
            {"bufferView": 3, "componentType": 5123, "count": 3, "type": "SCALAR"},
        ],
        "bufferViews": [
            {"buffer": 0, "byteOffset": off[0], "byteLength": 36},
            {"buffer": 0, "byteOffset": off[1], "byteLength": 36},
            {"buffer": 0, "byteOffset": off[2], "byteLength": 24},
            {"buffer": 0, "byteOffset": off[3], "byteLength": 6},
            {"buffer": 0, "byteOffset": off[4], "byteLength": 4},
        ],
        "buffers": [{"byteLength": len(data)}],
    }
    doc.update(extra or {})
    return make_glb(doc, data)


def vertex(p, i):
    return [round(float(x), 5) + 0.0 for x in p[i * 3:i * 3 + 3]]


def no_fetch(uri):
    raise AssertionError("unexpected fetch of %s" % uri)


# ------------------------------------------------------------------ parseGLB (gltf.test.ts:49-60)
def test_parse_glb_splits_chunks():
    doc, b = G.parse_glb(make_glb({"asset": {"version": "2.0"}}, bytes([1, 2, 3])))
    assert doc["asset"]["version"] == "2.0" and list(b[:3]) == [1, 2, 3]


def test_parse_glb_rejects_other_files():
    with pytest.raises(G.GLTFError, match="magic"):
        G.parse_glb(b'{"asset":{}}')


# ------------------------------------------------------------------ loadGLTF (gltf.test.ts:62-268)
def test_indexed_textured_triangle():
    a = G.load_gltf(triangle_glb(), no_fetch)
    assert a.triangle_count == 1
    mesh, mi = a.meshes[0]
    assert vertex(mesh.positions, 1) == [1, 0, 0]
    assert vertex(mesh.normals, 0) == [0, 0, 1]
    assert list(mesh.uvs) == [0, 0, 1, 0, 0, 1]
    m = a.materials[mi]
    assert m.albedo == (1, 0.5, 0.25) and m.base_color_map == 0
    assert len(a.images) == 1 and a.images[0].mime_type == "image/png"
    assert list(a.images[0].data) == [0x89, 0x50, 0x4E, 0x47]
    assert a.bounds == ((0, 0, 0), (1, 1, 0))


def test_trs_rotates_normals_with_geometry():
    s = math.sqrt(0.5)  # 90 degrees about +Y maps +X to -Z and +Z to +X
    a = G.load_gltf(triangle_glb({"translation": [1, 2, 3], "rotation": [0, s, 0, s], "scale": [2, 2, 2]}), no_fetch)
    p, n = a.meshes[0][0].positions, a.meshes[0][0].normals
    assert vertex(p, 0) == [1, 2, 3] and vertex(p, 1) == [1, 2, 1] and vertex(p, 2) == [1, 4, 3]
    assert vertex(n, 0) == [1, 0, 0]


def test_transforms_accumulate_down_the_hierarchy():
    glb = triangle_glb({}, {"scenes": [{"nodes": [1]}], "nodes": [
        {"mesh": 0, "translation": [0, 0, 5]},
        {"children": [0], "matrix": [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 10, 0, 0, 1]}]})
    assert vertex(G.load_gltf(glb, no_fetch).meshes[0][0].positions, 0) == [10, 0, 5]


def test_mirroring_keeps_winding_and_normals_consistent():
    a = G.load_gltf(triangle_glb({"scale": [-1, 1, 1]}), no_fetch)
    p, n = a.meshes[0][0].positions, a.meshes[0][0].normals
    e1, e2 = p[3:6] - p[0:3], p[6:9] - p[0:3]
    gz = e1[0] * e2[1] - e1[1] * e2[0]
    assert np.sign(gz) == np.sign(n[2]) and n[2] == pytest.approx(1)


def test_flat_normals_and_default_material():
    positions = np.array([0, 0, 0, 0, 0, 1, 1, 0, 0], np.float32)
    data, _ = pack(positions)
    doc = {"asset": {"version": "2.0"}, "nodes": [{"mesh": 0}],
           "meshes": [{"primitives": [{"attributes": {"POSITION": 0}}]}],
           "accessors": [{"bufferView": 0, "componentType": FLOAT, "count": 3, "type": "VEC3"}],
           "bufferViews": [{"buffer": 0, "byteLength": 36}], "buffers": [{"byteLength": len(data)}]}
    a = G.load_gltf(make_glb(doc, data), no_fetch)
    assert vertex(a.meshes[0][0].normals, 2) == [0, 1, 0]
    m = a.materials[a.meshes[0][1]]
    assert (m.albedo, m.metallic, m.roughness) == ((1, 1, 1), 1, 1)


def test_interleaved_normalized_strip_data():
    stride = 16
    buf = bytearray(stride * 4)
    for i, v in enumerate([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]]):
        struct.pack_into("<fff", buf, i * stride, *v)
        struct.pack_into("<HH", buf, i * stride + 12, v[0] * 65535, 32768)
    doc = {"asset": {"version": "2.0"}, "nodes": [{"mesh": 0}],
           "meshes": [{"primitives": [{"mode": 5, "attributes": {"POSITION": 0, "TEXCOORD_0": 1}}]}],
           "accessors": [{"bufferView": 0, "componentType": FLOAT, "count": 4, "type": "VEC3"},
                         {"bufferView": 0, "byteOffset": 12, "componentType": 5123, "normalized": True, "count": 4,
                          "type": "VEC2"}],
           "bufferViews": [{"buffer": 0, "byteLength": len(buf), "byteStride": stride}],
           "buffers": [{"byteLength": len(buf)}]}
    a = G.load_gltf(make_glb(doc, bytes(buf)), no_fetch)
    p, n, uv = a.meshes[0][0].positions, a.meshes[0][0].normals, a.meshes[0][0].uvs
    assert a.triangle_count == 2
    assert n[2] == pytest.approx(1) and n[11] == pytest.approx(1)  # strip triangles (0,1,2), (1,3,2) face +Z
    assert vertex(p, 4) == [1, 1, 0]
    assert uv[2] == pytest.approx(1) and uv[3] == pytest.approx(32768 / 65535)


def test_sparse_accessor_overrides():
    positions = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32)
    data, off = pack(positions, np.array([2], np.uint16), np.array([0, 7, 0], np.float32))
    doc = {"asset": {"version": "2.0"}, "nodes": [{"mesh": 0}],
           "meshes": [{"primitives": [{"attributes": {"POSITION": 0}}]}],
           "accessors": [{"bufferView": 0, "componentType": FLOAT, "count": 3, "type": "VEC3",
                          "sparse": {"count": 1, "indices": {"bufferView": 1, "componentType": 5123},
                                     "values": {"bufferView": 2}}}],
           "bufferViews": [{"buffer": 0, "byteOffset": off[0], "byteLength": 36},
                           {"buffer": 0, "byteOffset": off[1], "byteLength": 2},
                           {"buffer": 0, "byteOffset": off[2], "byteLength": 12}],
           "buffers": [{"byteLength": len(data)}]}
    assert vertex(G.load_gltf(make_glb(doc, data), no_fetch).meshes[0][0].positions, 2) == [0, 7, 0]


def test_gltf_json_with_data_uri_fetches_only_used_images():
    positions = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32)
    uvs = np.array([0, 0, 1, 0, 0, 1], np.float32)
    data, off = pack(positions, uvs)
    doc = {"asset": {"version": "2.0"}, "nodes": [{"mesh": 0}],
           "meshes": [{"primitives": [{"attributes": {"POSITION": 0, "TEXCOORD_0": 1}, "material": 0}]}],
           "materials": [{"normalTexture": {"index": 0, "scale": 0.5}}],
           "textures": [{"source": 1}],
           "images": [{"uri": "unused.png"}, {"uri": "tex%20normal.jpg"}],
           "accessors": [{"bufferView": 0, "componentType": FLOAT, "count": 3, "type": "VEC3"},
                         {"bufferView": 1, "componentType": FLOAT, "count": 3, "type": "VEC2"}],
           "bufferViews": [{"buffer": 0, "byteOffset": off[0], "byteLength": 36},
                           {"buffer": 0, "byteOffset": off[1], "byteLength": 24}],
           "buffers": [{"byteLength": len(data),
                        "uri": "data:application/octet-stream;base64," + base64.b64encode(data).decode()}]}
    fetched = []

    def fetch(uri):
        fetched.append(uri)
        return bytes([9])

    a = G.load_gltf(json.dumps(doc).encode(), fetch)
    assert fetched == ["tex%20normal.jpg"]
    assert a.images[0].mime_type == "image/jpeg"
    m = a.materials[0]
    assert [m.normal_map, m.normal_scale, m.base_color_map] == [0, 0.5, -1]


def test_pbr_extensions_map_onto_the_material_model():
    glb = triangle_glb({}, {"materials": [{
        "alphaMode": "MASK", "alphaCutoff": 0.3, "emissiveFactor": [1, 0.5, 0],
        "pbrMetallicRoughness": {"metallicFactor": 0.25, "roughnessFactor": 0.75},
        "extensions": {
            "KHR_materials_emissive_strength": {"emissiveStrength": 4},
            "KHR_materials_transmission": {"transmissionFactor": 0.9},
            "KHR_materials_ior": {"ior": 1.33},
            "KHR_materials_volume": {"thicknessFactor": 0.1, "attenuationDistance": 2,
                                     "attenuationColor": [1, 0.5, 0.5]},
            "KHR_materials_clearcoat": {"clearcoatFactor": 1, "clearcoatRoughnessFactor": 0.1},
            "KHR_materials_sheen": {"sheenColorFactor": [0.2, 0.3, 0.4], "sheenRoughnessFactor": 0.5},
            "KHR_materials_iridescence": {"iridescenceFactor": 1}}}]})
    a = G.load_gltf(glb, no_fetch)
    m = a.materials[0]
    assert m.alpha_mode == "mask" and m.alpha_cutoff == 0.3
    assert m.emission == (4, 2, 0)
    assert [m.metallic, m.roughness, m.transmission, m.ior] == [0.25, 0.75, 0.9, 1.33]
    assert [m.thin_walled, m.attenuation_distance, m.attenuation_color] == [False, 2, (1, 0.5, 0.5)]
    assert [m.clearcoat, m.clearcoat_roughness, m.sheen_roughness] == [1, 0.1, 0.5]
    assert m.sheen_color == (0.2, 0.3, 0.4)
    assert any("KHR_materials_iridescence" in w for w in a.warnings)
    assert len(a.images) == 0  # no texture referenced: the embedded image is not returned


def test_transmission_without_volume_is_thin_walled():
    a = G.load_gltf(triangle_glb({}, {"materials": [{"extensions": {
        "KHR_materials_transmission": {"transmissionFactor": 1}}}]}), no_fetch)
    assert a.materials[0].thin_walled is True


def test_refuses_required_compression():
    with pytest.raises(G.GLTFError, match="KHR_draco_mesh_compression"):
        G.load_gltf(triangle_glb({}, {"extensionsRequired": ["KHR_draco_mesh_compression"]}), no_fetch)


def test_rejects_gltf_1():
    with pytest.raises(G.GLTFError, match="only 2.0"):
        G.load_gltf(json.dumps({"asset": {"version": "1.0"}}).encode(), no_fetch)


def test_texture_transform():  # gltf.test.ts:270-285
    def apply(m, u, v):
        return [round(m[0] * u + m[1] * v + m[2], 6) + 0.0, round(m[3] * u + m[4] * v + m[5], 6) + 0.0]

    assert apply(G.texture_transform(None), 0.3, 0.7) == [0.3, 0.7]
    m = G.texture_transform({"offset": [0.5, 0.25], "scale": [2, 3], "rotation": math.pi / 2})
    assert apply(m, 1, 0) == [0.5, 2.25]  # scale, rotate 90 degrees, offset
    assert apply(m, 0, 1) == [-2.5, 0.25]


# ------------------------------------------------------------------ beyond the reference's cases
def test_fans_unlit_and_skipped_primitives():
    positions = np.array([0, 0, 0, 1, 0, 0, 1, 1, 0, 0, 1, 0], np.float32)
    data, _ = pack(positions)
    doc = {"asset": {"version": "2.0"}, "nodes": [{"mesh": 0}],
           "meshes": [{"primitives": [{"mode": 6, "attributes": {"POSITION": 0}, "material": 0},
                                      {"mode": 1, "attributes": {"POSITION": 0}}]}],
           "materials": [{"pbrMetallicRoughness": {"baseColorFactor": [0.5, 0.6, 0.7, 1]},
                          "extensions": {"KHR_materials_unlit": {}}}],
           "accessors": [{"bufferView": 0, "componentType": FLOAT, "count": 4, "type": "VEC3"}],
           "bufferViews": [{"buffer": 0, "byteLength": 48}], "buffers": [{"byteLength": len(data)}]}
    a = G.load_gltf(make_glb(doc, data), no_fetch)
    assert a.triangle_count == 2  # fan (1,2,0), (2,3,0); the line primitive is skipped
    assert vertex(a.meshes[0][0].positions, 0) == [1, 0, 0] and vertex(a.meshes[0][0].positions, 2) == [0, 0, 0]
    m = a.materials[0]
    assert m.emission == (0.5, 0.6, 0.7) and m.albedo == (0, 0, 0) and m.metallic == 0
    assert "point and line primitives are skipped" in a.warnings


def test_errors_mirror_the_reference():
    with pytest.raises(G.GLTFError, match="no triangle meshes"):
        G.load_gltf(json.dumps({"asset": {"version": "2.0"}}).encode(), no_fetch)
    data, _ = pack(np.zeros(9, np.float32))
    doc = {"asset": {"version": "2.0"}, "nodes": [{"mesh": 0}],
           "meshes": [{"primitives": [{"attributes": {"POSITION": 0}}]}],
           "accessors": [{"bufferView": 0, "componentType": FLOAT, "count": 4, "type": "VEC3"}],
           "bufferViews": [{"buffer": 0, "byteLength": 36}], "buffers": [{"byteLength": len(data)}]}
    with pytest.raises(G.GLTFError, match="reads past its bufferView"):
        G.load_gltf(make_glb(doc, data), no_fetch)
    with pytest.raises(G.GLTFError, match="cycle"):
        G.load_gltf(triangle_glb({"children": [0]}), no_fetch)


# ------------------------------------------------------------------ packing (scene.test.ts:121-166)
def _quad(x0):
    return M.quad([x0, 0, 0], [x0 + 1, 0, 0], [x0 + 1, 1, 0], [x0, 1, 0])


def _fake_textures(n):
    return [S.Texture(np.zeros((1, 1, 4), np.uint8), "t%d" % i) for i in range(n)]


def test_texture_layers_per_usage():
    a = S.material(base_color_map=3, normal_map=1, metal_rough_map=1)
    b = S.material(base_color_map=0, emissive_map=3, metal_rough_map=2)
    sc = S.Scene(meshes=[S.MeshInstance(_quad(0), a), S.MeshInstance(_quad(2), b)], textures=_fake_textures(4))
    p = S.pack_scene(sc)
    assert p.color_layers == [3, 0] and p.data_layers == [1, 2]
    mt = p.materials.reshape(-1, 40)
    assert list(mt[0, 16:20]) == [0, 0, 0, -1]  # base colour, metal-rough, normal, emissive
    assert list(mt[1, 16:20]) == [1, 1, -1, 0]


def test_maps_past_the_scene_textures_are_rejected():
    sc = S.Scene(meshes=[S.MeshInstance(_quad(0), S.material(normal_map=0))])
    with pytest.raises(ValueError, match="texture 0"):
        S.pack_scene(sc)


def test_textured_alpha_mask_is_alpha_tested():
    m = _quad(0)
    uvs = np.array([0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.1, 0.2, 0.5, 0.6, 0.7, 0.8], np.float32)
    sc = S.Scene(meshes=[S.MeshInstance(M.Mesh(m.positions, m.normals, uvs),
                                        S.material(alpha_mode="mask", base_color_map=0)),
                         S.MeshInstance(_quad(2), S.matte((1, 1, 1)))], textures=_fake_textures(1))
    p = S.pack_scene(sc)
    assert list(p.tri_alpha) == [1, 1, 0, 0]
    assert np.allclose(p.uvs[:6], [0.1, 0.2, 0.3, 0.4, 0.5, 0.6]) and (p.uvs[12:] == 0).all()


# ------------------------------------------------------------------ PNG
def _chunk(kind, body):
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def _png(w, h, depth, ctype, raw_rows, plte=None, trns=None, interlace=0):
    out = I.PNG_SIGNATURE + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, interlace))
    if plte is not None:
        out += _chunk(b"PLTE", plte)
    if trns is not None:
        out += _chunk(b"tRNS", trns)
    return out + _chunk(b"IDAT", zlib.compress(raw_rows)) + _chunk(b"IEND", b"")


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def _filtered(rows, bpp):
    """Rows of bytes with filter type (row index mod 5) applied."""
    out, prev = b"", [0] * len(rows[0])
    for y, row in enumerate(rows):
        row = [int(v) for v in row]
        t = y % 5
        enc = []
        for i, x in enumerate(row):
            a = row[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            enc.append((x - [0, a, b, (a + b) // 2, _paeth(a, b, c)][t]) % 256)
        out += bytes([t]) + bytes(enc)
        prev = list(row)
    return out


def test_png_round_trip_and_filters():
    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, (37, 53, 4), dtype=np.uint8)
    assert np.array_equal(I.decode_png(I.encode_png(img)), img)
    rgb = rng.integers(0, 256, (11, 9, 3), dtype=np.uint8)
    d = I.decode_png(_png(9, 11, 8, 2, _filtered([list(r.reshape(-1)) for r in rgb], 3)))
    assert np.array_equal(d[:, :, :3], rgb) and (d[:, :, 3] == 255).all()
    g16 = rng.integers(0, 65536, (6, 5), dtype=np.uint16)
    rows = [list(r.astype(">u2").tobytes()) for r in g16]
    d = I.decode_png(_png(5, 6, 16, 0, _filtered(rows, 2)))
    want = ((g16.astype(np.uint32) * 255 + 32767) // 65535).astype(np.uint8)
    assert np.array_equal(d[:, :, 0], want) and np.array_equal(d[:, :, 2], want)


def test_png_palette_low_depth_and_interlace():
    pal = bytes([10, 20, 30, 40, 50, 60, 70, 80, 90, 200, 210, 220])
    idx = np.array([[0, 1, 2, 3, 3], [3, 2, 1, 0, 1]], np.uint8)
    raw = b"".join(b"\0" + np.packbits(np.unpackbits(r[:, None], axis=1)[:, 6:].reshape(-1)).tobytes() for r in idx)
    d = I.decode_png(_png(5, 2, 2, 3, raw, plte=pal, trns=bytes([0, 128])))
    assert list(d[0, 1]) == [40, 50, 60, 128] and list(d[1, 0]) == [200, 210, 220, 255] and d[0, 0, 3] == 0
    # Adam7: decode(interlaced) == image
    rng = np.random.default_rng(3)
    img = rng.integers(0, 256, (13, 10, 4), dtype=np.uint8)
    raw = b""
    for x0, y0, dx, dy in I.ADAM7:
        sub = img[y0::dy, x0::dx]
        if sub.size:
            raw += b"".join(b"\0" + r.tobytes() for r in sub)
    assert np.array_equal(I.decode_png(_png(10, 13, 8, 6, raw, interlace=1)), img)
    with pytest.raises(I.ImageDecodeError):
        I.decode_image(b"\xff\xd8\xff\xe0jpeg", "image/jpeg")


# ------------------------------------------------------------------ model.ts
def test_model_scene_and_undecodable_images(tmp_path):
    tex = np.zeros((4, 4, 4), np.uint8)
    tex[..., 0] = 255
    png = np.frombuffer(I.encode_png(tex), np.uint8)
    positions = np.array([0, 0, 0, 2, 0, 0, 0, 2, 0], np.float32)
    normals = np.array([0, 0, 1] * 3, np.float32)
    uvs = np.array([0, 0, 1, 0, 0, 1], np.float32)
    data, off = pack(positions, normals, uvs, np.array([0, 1, 2], np.uint16), png)
    doc = {
        "asset": {"version": "2.0"}, "nodes": [{"mesh": 0}],
        "meshes": [{"primitives": [{"attributes": {"POSITION": 0, "NORMAL": 1, "TEXCOORD_0": 2}, "indices": 3,
                                    "material": 0}, {"attributes": {"POSITION": 0}, "material": 1}]}],
        "materials": [{"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}},
                       "extensions": {"KHR_materials_volume": {"thicknessFactor": 1, "attenuationDistance": 4}}},
                      {"emissiveTexture": {"index": 1}}],
        "textures": [{"source": 0}, {"source": 1}],
        "images": [{"bufferView": 4, "mimeType": "image/png", "name": "red"}, {"uri": "glow.jpg"}],
        "accessors": [
            {"bufferView": 0, "componentType": FLOAT, "count": 3, "type": "VEC3"},
            {"bufferView": 1, "componentType": FLOAT, "count": 3, "type": "VEC3"},
            {"bufferView": 2, "componentType": FLOAT, "count": 3, "type": "VEC2"},
            {"bufferView": 3, "componentType": 5123, "count": 3, "type": "SCALAR"}],
        "bufferViews": [{"buffer": 0, "byteOffset": off[i], "byteLength": n}
                        for i, n in enumerate([36, 36, 24, 6, png.size])],
        "buffers": [{"byteLength": len(data)}],
    }
    (tmp_path / "m.glb").write_bytes(make_glb(doc, data))
    (tmp_path / "glow.jpg").write_bytes(b"\xff\xd8\xff\xe0not really")
    model = MD.load_model(str(tmp_path / "m.glb"))
    assert model.name == "m" and len(model.textures) == 2
    assert np.array_equal(model.textures[0].image, tex)
    assert 'could not decode image "glow.jpg"' in model.warnings
    assert model.asset.materials[1].emissive_map == -1 and model.asset.materials[0].base_color_map == 0
    sc = MD.scene_from_model(model, S.Environment())
    assert sc.ground.enabled and sc.textures is model.textures
    p = np.concatenate([mi.mesh.positions for mi in sc.meshes]).reshape(-1, 3)
    assert p[:, 1].min() == pytest.approx(0) and np.linalg.norm(p.max(0) - p.min(0)) == pytest.approx(2)
    assert sc.meshes[0].material.attenuation_distance == pytest.approx(4 / math.sqrt(2))
    packed = S.pack_scene(sc)
    assert packed.color_layers == [0] and packed.data_layers == []
