"""Analytic spheres, the sphere light, the ground, the procedural sky and the
analytic sun on the GPU against the oracle.

workloads.sky_scene has no environment map, so uploadLighting bakes the sky
(bakeSky, environment.ts:106-132) and turns the analytic sun on with
uSunPdf = 1 / solid angle (renderer.ts:359-367). Its spheres go through
hitSphere (scene.glsl:132-144) and win over triangles when closer (:200);
the emissive sphere is a sphere light sampled through the cone branch of
sampleLight and weighted by lightPdf (lights.glsl:99-158); next-event
estimation draws the sun with sampleSunDirection (lights.glsl:93). As in the
other render tests, both sides follow the same random streams, so the bars
are on per-pixel agreement at low spp and on the RMSE of a converged image
against the binary64 oracle render.
"""
import numpy as np
import pytest

from oracle import render as OR
from lucent_gb300 import workloads as W
from lucent_gb300.renderer import Renderer

pytestmark = pytest.mark.gpu


def _gpu(scene, w, h, spp, seed=0, max_bounces=8, batches=1):
    r = Renderer(w, h)
    r.settings.max_bounces = max_bounces
    r.load_scene(scene)
    r.set_seed(seed)
    for _ in range(batches):
        r.trace_samples(spp // batches)
    out = r.read()
    r.dispose()
    return out


def _close_frac(a, b, rel=1e-3):
    return (np.abs(a - b) <= rel * (np.abs(b) + 1e-3)).mean()


@pytest.fixture(scope="module")
def sky():
    sc = W.sky_scene(0)
    return sc, OR.prepare(sc)


def test_sky_scene_matches_oracle_per_pixel(sky):
    sc, prep = sky
    w, h = 96, 64
    col, alb, nrm, hist = _gpu(sc, w, h, 4)
    oc, oa, on, oh = OR.render(prep, w, h, 0, 4, max_bounces=8)
    assert np.array_equal(hist, oh) and not np.isnan(col).any()
    assert _close_frac(col[..., :3], oc[..., :3]) > 0.95
    assert _close_frac(alb, oa, 2e-3) > 0.97
    assert _close_frac(nrm, on, 2e-3) > 0.97
    # the frame holds sky, ground, spheres and the mesh
    assert (alb[..., 3] == 0).mean() > 0.05 and (alb[..., 3] > 0).mean() > 0.5


def test_sky_scene_converges_to_fp64(sky):
    sc, prep = sky
    w, h = 48, 32
    col, *_ = _gpu(sc, w, h, 256, seed=5, batches=2)
    ref, *_ = OR.render(prep, w, h, 5, 256, max_bounces=8, precision=64)
    rmse = np.sqrt(np.mean((col[..., :3] - ref[..., :3]) ** 2)) / np.mean(ref[..., :3])
    assert rmse < 0.01, rmse


def test_sphere_light_and_sun_carry_the_direct_light(sky):
    """The emissive sphere and the sun each contribute: switching either off
    changes the image, on the GPU as on the oracle, by the same amount."""
    import copy
    sc, _ = sky
    w, h = 48, 32
    base = _gpu(sc, w, h, 16)[0][..., :3].mean()
    no_sun = copy.deepcopy(sc)
    no_sun.sun.intensity = 0.0
    no_lamp = copy.deepcopy(sc)
    no_lamp.spheres = no_lamp.spheres[:3]
    for alt in (no_sun, no_lamp):
        g = _gpu(alt, w, h, 16)[0][..., :3].mean()
        o = OR.render(OR.prepare(alt), w, h, 0, 16, max_bounces=8)[0][..., :3].mean()
        ob = OR.render(OR.prepare(sc), w, h, 0, 16, max_bounces=8)[0][..., :3].mean()
        assert g < base and o < ob
        assert abs((base - g) - (ob - o)) < 0.02 * ob
