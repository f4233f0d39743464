"""GPU path tracer vs the oracle's restatement of trace.frag.

Both sides draw each path's random numbers from the reference's per-pixel PCG
stream in the reference's order and take triangle hits from the reference's
binary64 intersector, so GPU and oracle follow the same paths; they differ
only by binary32 rounding in shading (FMA, libm), which occasionally flips a
Russian-roulette or lobe choice. The tests therefore bound (a) the share of
pixels that agree to 1e-3 relative and (b) the image RMSE, and compare a
converged image against the oracle's binary64 render.
"""
import numpy as np
import pytest

from oracle import render as OR
from lucent_gb300 import workloads as W
from lucent_gb300._native import LucentError
from lucent_gb300.renderer import Batch, Renderer

pytestmark = pytest.mark.gpu


def _gpu(scene, w, h, spp, seed=0, max_bounces=8, batches=1):
    r = Renderer(w, h)
    r.settings.max_bounces = max_bounces
    r.load_scene(scene)
    r.set_seed(seed)
    for _ in range(batches):
        r.trace_samples(spp // batches)
    col, alb, nrm, hist = r.read()
    st = r.stats()
    r.dispose()
    return col, alb, nrm, hist, st


def _close_frac(a, b, rel=1e-3):
    return (np.abs(a - b) <= rel * (np.abs(b) + 1e-3)).mean()


def test_box_scene_matches_oracle_per_pixel():
    sc = W.box_scene(0, 3)
    w = h = 64
    col, alb, nrm, hist, st = _gpu(sc, w, h, 4)
    prep = OR.prepare(sc)
    oc, oa, on, oh = OR.render(prep, w, h, 0, 4, max_bounces=8)
    assert np.all(hist == 4) and np.array_equal(hist, oh)
    assert not np.isnan(col).any()
    frac = _close_frac(col[..., :3], oc[..., :3])
    assert frac > 0.97, frac
    rmse = np.sqrt(np.mean((col[..., :3] - oc[..., :3]) ** 2)) / np.mean(oc[..., :3])
    assert rmse < 0.02, rmse
    assert _close_frac(alb, oa, 2e-3) > 0.97
    assert st["closest_rays"] > 0 and st["shadow_rays"] > 0


def test_converged_image_matches_fp64_render():
    sc = W.box_scene(1, 3)
    w = h = 32
    col, *_ = _gpu(sc, w, h, 256, seed=7, batches=4)
    prep = OR.prepare(sc)
    ref, *_ = OR.render(prep, w, h, 7, 256, max_bounces=8, precision=64)
    rel_rmse = np.sqrt(np.mean((col[..., :3] - ref[..., :3]) ** 2)) / np.mean(ref[..., :3])
    assert rel_rmse < 0.01, rel_rmse


def test_white_furnace():
    # A rough, IOR-1 sphere of albedo 1 under a uniform environment: the image
    # must match the binary64 oracle and stay within the model's energy bounds.
    sc = W.furnace_scene(albedo=1.0, roughness=1.0, ior=1.0, radiance=1.0)
    w = h = 32
    col, alb, *_ = _gpu(sc, w, h, 64, max_bounces=12)
    prep = OR.prepare(sc)
    ref, *_ = OR.render(prep, w, h, 0, 64, max_bounces=12, precision=64)
    cov = alb[..., 3] == 1.0  # every sample hit the sphere
    bg = alb[..., 3] == 0.0  # no sample did
    g = col[..., :3][cov].mean()
    o = ref[..., :3][cov].mean()
    assert abs(g - o) / o < 0.01, (g, o)
    assert 0.85 < g < 1.02, g
    assert bg.any() and np.allclose(col[..., :3][bg], 1.0, atol=1e-5)  # background sees the environment


@pytest.mark.parametrize("name,layers,lo,hi", [
    ("clearcoat", dict(roughness=0.6, clearcoat=1.0, clearcoat_roughness=0.2, ior=1.5), 0.5, 1.02),
    ("sheen", dict(roughness=0.8, sheen_color=(1.0, 1.0, 1.0), sheen_roughness=0.5), 0.5, 1.02),
    ("metal", dict(roughness=0.4, metallic=1.0), 0.5, 1.02),
    ("dielectric", dict(roughness=0.0, transmission=1.0, ior=1.5), 0.9, 1.02),
])
def test_white_furnace_layers(name, layers, lo, hi):
    """White furnace of each lobe of the layered BSDF (bsdf.glsl:114-248):
    clearcoat over GGX, Charlie sheen over Lambert, a rough conductor and a
    smooth dielectric sphere (no absorption: every path leaves with radiance
    1 unless the bounce limit cuts it). The image matches the binary64 oracle
    within 1 % and never gains energy."""
    sc = W.furnace_scene(albedo=1.0, radiance=1.0, **layers)
    w = h = 32
    col, alb, *_ = _gpu(sc, w, h, 64, max_bounces=12)
    prep = OR.prepare(sc)
    ref, *_ = OR.render(prep, w, h, 0, 64, max_bounces=12, precision=64)
    cov = alb[..., 3] == 1.0
    assert cov.mean() > 0.3
    g = col[..., :3][cov].mean()
    o = ref[..., :3][cov].mean()
    assert abs(g - o) / o < 0.01, (name, g, o)
    assert lo < g < hi, (name, g)


def test_converged_full_geometry_matches_fp64_render():
    """The bench scene itself (81,956 triangles, layered icosphere) converged:
    a 64x64 crop of the 512x512 frame at 1,024 spp against the binary64
    oracle render of the same samples. Same random streams on both sides, so
    the bar is on the image difference, not on Monte Carlo noise: relative
    RMSE below 1 % (a binary32 rounding that flips one sample's Russian
    roulette or lobe choice moves that sample alone)."""
    sc = W.box_scene(0, 6)
    col, *_ = _gpu(sc, 512, 512, 1024, seed=11, batches=4)
    prep = OR.prepare(sc)
    x0, y0 = 224, 208  # the icosphere, the short box and the floor
    ref, *_ = OR.render(prep, 512, 512, 11, 1024, max_bounces=8, precision=64, crop=(x0, y0, 64, 64))
    g = col[y0:y0 + 64, x0:x0 + 64, :3]
    r = ref[..., :3]
    rmse = np.sqrt(np.mean((g - r) ** 2)) / np.mean(r)
    assert rmse < 0.01, rmse


def test_full_size_box_scene_crop():
    # 512 x 512, 16 spp, depth 8 on the 81,956-triangle scene; a crop is
    # checked against the oracle (the whole frame would take the CPU minutes).
    sc = W.box_scene(0, 6)
    col, alb, nrm, hist, st = _gpu(sc, 512, 512, 16)
    assert np.all(hist == 16) and not np.isnan(col).any()
    prep = OR.prepare(sc)
    x0, y0 = 240, 200
    oc, *_ = OR.render(prep, 512, 512, 0, 16, max_bounces=8, crop=(x0, y0, 48, 48))
    g = col[y0:y0 + 48, x0:x0 + 48, :3]
    frac = _close_frac(g, oc[..., :3])
    assert frac > 0.9, frac
    rmse = np.sqrt(np.mean((g - oc[..., :3]) ** 2)) / np.mean(oc[..., :3])
    assert rmse < 0.05, rmse


@pytest.mark.parametrize("option", ["ray_sort", "top_levels", "wide_bvh"])
def test_traversal_options_change_no_pixel(option):
    # Sorting the rays changes the order paths are traced in, never a path;
    # the shared-memory copy of the top BVH levels changes where nodes are
    # read from, never a decision; the four-wide traversal skips box tests
    # whose outcome the grandchildren's own tests imply, and a hit's output
    # values depend on the ray and triangle alone: the images are identical
    # bit for bit.
    sc = W.box_scene(2, 3)
    out = []
    for on in (True, False):
        r = Renderer(64, 48)
        r.settings.max_bounces = 8
        r.load_scene(sc)
        getattr(r, "set_" + option)(on)
        r.set_seed(11)
        r.trace_samples(6)
        out.append(r.read())
        r.dispose()
    assert all(np.array_equal(a, b) for a, b in zip(*out))


def test_graph_replay_changes_no_pixel():
    # Full waves after a renderer's first replay a captured CUDA graph;
    # profiling mode launches every kernel directly. Same images either way,
    # including after an option change (a new graph).
    sc = W.box_scene(3, 3)
    out = []
    for profiling in (False, True):
        r = Renderer(48, 40)
        r.settings.max_bounces = 6
        r.load_scene(sc)
        r.set_profiling(profiling)
        r.set_seed(5)
        for i in range(4):
            if i == 2:
                r.set_ray_sort(False)
            r.trace_samples(2)
        out.append(r.read())
        r.dispose()
    assert all(np.array_equal(a, b) for a, b in zip(*out))


def test_pipelined_waves_change_no_pixel():
    # Pipelining alternates successive waves between two path buffers traced
    # on the renderer's own streams; only the accumulation runs on the
    # caller's stream, in call order. The images equal wave-by-wave tracing
    # bit for bit: across the waves of one trace (full waves and a last
    # partial one), across traces, through a camera move that reprojects the
    # history, a material change and an accumulation reset.
    import copy
    sc = W.box_scene(2, 3)
    cam2 = copy.deepcopy(sc.camera)
    cam2.position = (sc.camera.position[0] + 0.05, sc.camera.position[1], sc.camera.position[2])
    out = []
    for on in (True, False):
        r = Renderer(1024, 1024)  # 2^23 paths a wave: waves of 8 samples
        r.settings.max_bounces = 4
        r.load_scene(sc)
        r.set_pipelining(on)
        r.set_seed(3)
        r.trace_samples(20)  # 8 + 8 + 4
        r.trace_samples(3)
        r.trace_samples(5)
        r.upload_camera(cam2)  # temporal on: the next sample reprojects the history
        r.trace_samples(2)
        r.trace_samples(9)  # 8 + 1
        imgs = [a.copy() for a in r.read()]
        from lucent_gb300 import adjoint as AD
        m = np.array(r.packed.materials, np.float32).reshape(-1, 40)
        m[:, 0] *= 0.5  # albedo red
        AD.set_materials(r, m)
        r.trace_samples(4)
        r.reset()
        r.trace_samples(11)
        out.append(imgs + list(r.read()))
        r.dispose()
    assert all(np.array_equal(a, b) for a, b in zip(*out))


def test_kernel_launch_count():
    # lucent_render_stats.kernel_launches: a wave launches the camera kernel,
    # 7 kernels a bounce, a shade-counter reset for each bounce after the
    # first (the previous bounce's shadow rays run on the second stream), 3
    # per ray sort (after bounces 0 and 1 in waves under 2^21 paths), the
    # accumulation and the seed advance; a replayed graph counts as many;
    # reset launches one.
    r = Renderer(32, 32)
    r.settings.max_bounces = 3
    r.load_scene(W.box_scene(1, 3))
    wave = 1 + 7 * 4 + 3 + 3 * 2 + 2
    base = r.stats()["kernel_launches"]
    counts = []
    for _ in range(3):  # the first wave runs directly, the others replay its graph
        r.trace_samples(1)
        counts.append(r.stats()["kernel_launches"] - base)
    r.reset()
    after = r.stats()["kernel_launches"] - base
    r.dispose()
    assert counts == [wave, 2 * wave, 3 * wave]
    assert after == 3 * wave + 1


def test_views_share_the_scene_and_render_the_same_images():
    # A view renders its source's scene from its own camera with the scene's
    # device data shared: the image equals a renderer that loaded its own copy.
    from dataclasses import replace
    from lucent_gb300 import scene as S
    sc = W.adjoint_scene(1, 3)
    cams = W.adjoint_views(3)
    src = Renderer(48, 40)
    src.settings.max_bounces = 5
    src.load_scene(replace(sc, camera=cams[0]))
    views = [Renderer.view(src, 48, 40, camera=c) for c in cams[1:]]
    own = []
    for c in cams[1:]:
        r = Renderer(48, 40)
        r.settings.max_bounces = 5
        r.load_scene(replace(sc, camera=c))
        own.append(r)
    for r in views:
        r.settings.max_bounces = 5
        r.apply_settings()
    for r in [src] + views + own:
        r.set_seed(5)
        r.trace_samples(3)
    for v, o in zip(views, own):
        assert all(np.array_equal(a, b) for a, b in zip(v.read(), o.read()))
        assert v.stats()["triangles"] == o.stats()["triangles"]
    # a batch of the source and its views equals them traced alone
    alone = [r.read()[0].copy() for r in [src] + views]
    for r in [src] + views:
        r.reset()
        r.set_seed(5)
    b = Batch([src] + views)
    b.trace_samples(3)
    b.check()
    for r, a in zip([src] + views, alone):
        assert np.array_equal(r.read()[0], a)
    # materials are shared; the source cannot load another scene while views exist
    from lucent_gb300 import adjoint as AD
    m = np.array(src.packed.materials, np.float32).reshape(-1, 40)
    m[:, 0:3] *= 0.5
    AD.set_materials(views[0], m.reshape(-1))
    src.reset()
    src.set_seed(5)
    src.trace_samples(3)
    assert not np.array_equal(src.read()[0], alone[0])
    with pytest.raises(LucentError):
        src.load_scene(sc)
    for r in views + own + [src]:
        r.dispose()
