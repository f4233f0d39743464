"""Texture maps on the GPU (buildTextureArrays, surfaceAt's maps,
alphaOpaque's base-colour alpha) against the oracle.

* The texture arrays (resampling of every referenced image into its layer)
  equal the oracle's restatement bit for bit, for magnified images, for
  images whose size forces the mip chain (trilinear between two levels) and
  for sRGB and linear layers.
* Renders of a glTF model with base-colour, metal-rough, normal, emissive and
  alpha-masked maps follow the oracle per pixel (same random streams, same
  hits; shading differs by binary32 rounding) and converge to its binary64
  render.
"""
from dataclasses import replace

import numpy as np
import pytest

from oracle import render as OR
from lucent_gb300 import mesh as M
from lucent_gb300 import scene as S
from lucent_gb300 import workloads as W
from lucent_gb300._native import LucentError
from lucent_gb300.renderer import Batch, Renderer

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def textured():
    return W.textured_scene(0, 128)


def _renderer(scene, w, h, seed=0, max_bounces=6):
    r = Renderer(w, h)
    r.settings.max_bounces = max_bounces
    r.load_scene(scene)
    r.set_seed(seed)
    return r


def _close_frac(a, b, rel=1e-3):
    return (np.abs(a - b) <= rel * (np.abs(b) + 1e-3)).mean()


def test_texture_arrays_match_oracle(textured):
    r = _renderer(textured, 16, 16)
    col, dat = r.read_texture_arrays()
    r.dispose()
    prep = OR.prepare(textured)
    assert prep.tex_size == col.shape[1] == 128
    assert np.array_equal(col, prep.color_maps) and np.array_equal(dat, prep.data_maps)


def test_resampling_paths_match_oracle():
    # Sizes: 3000 x 40 (largest 3000 -> layer 2048, level of detail 0.55:
    # trilinear between levels 0 and 1), 1500 x 900 (minified too), 5 x 3
    # and 333 x 77 (magnified, odd sizes). sRGB and linear layers.
    rng = np.random.default_rng(4)
    shapes = [(40, 3000), (900, 1500), (3, 5), (77, 333)]
    texs = [S.Texture(rng.integers(0, 256, sh + (4,), dtype=np.uint8), "t%d" % i) for i, sh in enumerate(shapes)]
    meshes = []
    for i in range(4):
        q = M.quad([i, 0, 0], [i + 1, 0, 0], [i + 1, 1, 0], [i, 1, 0])
        q = M.Mesh(q.positions, q.normals, np.array([0, 0, 1, 0, 1, 1, 0, 0, 1, 1, 0, 1], np.float32))
        meshes.append(S.MeshInstance(q, S.material(base_color_map=i, metal_rough_map=(i + 1) % 4)))
    sc = S.Scene(meshes=meshes, textures=texs)
    sc.camera = S.Camera(position=(2.0, 0.5, 4.0), target=(2.0, 0.5, 0.0))
    r = _renderer(sc, 16, 16)
    col, dat = r.read_texture_arrays()
    r.dispose()
    prep = OR.prepare(sc)
    assert col.shape == (4, 2048, 2048, 4) and dat.shape == (4, 2048, 2048, 4)
    for k in range(4):
        assert np.array_equal(col[k], prep.color_maps[k]), ("colour", k, int((col[k] != prep.color_maps[k]).sum()))
        assert np.array_equal(dat[k], prep.data_maps[k]), ("data", k, int((dat[k] != prep.data_maps[k]).sum()))


def test_textured_render_matches_oracle_per_pixel(textured):
    w, h = 96, 64
    r = _renderer(textured, w, h, max_bounces=6)
    r.trace_samples(4)
    col, alb, nrm, hist = r.read()
    st = r.stats()
    r.dispose()
    prep = OR.prepare(textured)
    oc, oa, on, oh = OR.render(prep, w, h, 0, 4, max_bounces=6)
    assert np.array_equal(hist, oh) and not np.isnan(col).any()
    frac = _close_frac(col[..., :3], oc[..., :3])
    assert frac > 0.95, frac
    rmse = np.sqrt(np.mean((col[..., :3] - oc[..., :3]) ** 2)) / np.mean(oc[..., :3])
    assert rmse < 0.03, rmse
    assert _close_frac(alb, oa, 2e-3) > 0.95
    assert st["closest_rays"] > 0


def test_textured_render_converges_to_binary64(textured):
    w, h = 48, 32
    r = _renderer(textured, w, h, seed=3, max_bounces=6)
    for _ in range(4):
        r.trace_samples(64)
    col = r.read()[0]
    r.dispose()
    prep = OR.prepare(textured)
    ref, *_ = OR.render(prep, w, h, 3, 256, max_bounces=6, precision=64)
    rel = np.sqrt(np.mean((col[..., :3] - ref[..., :3]) ** 2)) / np.mean(ref[..., :3])
    assert rel < 0.02, rel


def test_maps_change_the_image(textured):
    # Dropping the maps (same geometry and factors) must change the render:
    # the maps are really sampled.
    plain = S.Scene(**{**textured.__dict__})
    plain.meshes = [S.MeshInstance(mi.mesh, replace(mi.material, base_color_map=-1, metal_rough_map=-1,
                                                      normal_map=-1, emissive_map=-1)) for mi in textured.meshes]
    plain.textures = []
    out = []
    for sc in (textured, plain):
        r = _renderer(sc, 48, 32)
        r.trace_samples(8)
        out.append(r.read()[0][..., :3])
        r.dispose()
    assert np.abs(out[0] - out[1]).mean() > 0.01 * out[1].mean()


def test_textured_batch_equals_single(textured):
    solo = []
    for sc in (textured, W.box_scene(1, 3)):
        r = _renderer(sc, 40, 32)
        r.trace_samples(3)
        solo.append(r.read())
        r.dispose()
    rs = [_renderer(sc, 40, 32) for sc in (textured, W.box_scene(1, 3))]
    b = Batch(rs)
    b.trace_samples(3)
    b.check()
    for r, want in zip(rs, solo):
        assert all(np.array_equal(x, y) for x, y in zip(r.read(), want))
        r.dispose()
    b.dispose()


def test_texture_errors(textured):
    r = _renderer(textured, 16, 16)
    from lucent_gb300 import adjoint as AD
    with pytest.raises(LucentError):  # the adjoint's parameters are factors: maps are not differentiated
        AD.backward(r, 1, 0, np.ones((16, 16, 3), np.float32))
    r.dispose()
    bad = S.Scene(meshes=[S.MeshInstance(M.quad([0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]),
                                         S.material(base_color_map=0))],
                  textures=[S.Texture(np.zeros((0, 4, 4), np.uint8))])
    r = Renderer(8, 8)
    with pytest.raises(LucentError):  # an empty image
        r.load_scene(bad)
    r.dispose()


def test_wide_traversal_changes_no_pixel_with_alpha_cutouts(textured):
    # The textured model has an alpha-mask cutout: deferred texture-alpha rays
    # go to the binary64 kernel from the wide traversal as from the binary one.
    out = []
    for wide in (True, False):
        r = Renderer(64, 64)
        r.settings.max_bounces = 6
        r.load_scene(textured)
        r.set_wide_bvh(wide)
        r.set_seed(3)
        r.trace_samples(4)
        out.append(r.read())
        r.dispose()
    assert all(np.array_equal(a, b) for a, b in zip(*out))
