"""The large-mesh workload (torus knot with value-noise displacement,
dielectrics with Beer-Lambert absorption, alpha-blended triangles, a
lognormal HDRI with a baked sun disk, thin lens) on the GPU vs the oracle.

Small variants (6,400 triangles) are compared per pixel and converged; the
full workload (2,000,000 triangles, 1920x1080, 256 spp, depth 12, five
a-trous iterations) is rendered whole on the GPU and compared with the
oracle on crops. Paths follow the same random stream on both sides; a
binary32 rounding difference in shading can still flip a Russian-roulette,
lobe or Fresnel choice and send one sample elsewhere, so per-pixel bounds
are on the share of agreeing pixels at low spp and on relative RMSE at
high spp (where each pixel averages 256 samples).
"""
import numpy as np
import pytest

from oracle import render as OR
from lucent_gb300 import workloads as W
from lucent_gb300.renderer import Renderer

pytestmark = pytest.mark.gpu


def _gpu(scene, w, h, spp, seed=0, max_bounces=12):
    r = Renderer(w, h)
    r.settings.max_bounces = max_bounces
    r.load_scene(scene)
    r.set_seed(seed)
    r.trace_samples(spp)
    out = r.read()
    return r, out


def _close_frac(a, b, rel=1e-3):
    return (np.abs(a - b) <= rel * (np.abs(b) + 1e-3)).mean()


def _rel_rmse(a, b):
    return np.sqrt(np.mean((a - b) ** 2)) / np.mean(np.abs(b))


@pytest.fixture(scope="module")
def small_knot():
    sc = W.knot_scene(0, tubular=200, radial=16, env_width=256)
    return sc, OR.prepare(sc)


def test_small_knot_matches_oracle_per_pixel(small_knot):
    sc, prep = small_knot
    r, (col, alb, nrm, hist) = _gpu(sc, 96, 54, 2)
    oc, oa, on, oh = OR.render(prep, 96, 54, 0, 2, max_bounces=12)
    assert np.array_equal(hist, oh) and not np.isnan(col).any()
    assert 0.3 < (alb[..., 3] > 0.5).mean() < 0.9  # the knot fills part of the frame
    assert _close_frac(col[..., :3], oc[..., :3]) > 0.95
    assert _close_frac(alb, oa, 2e-3) > 0.97
    r.dispose()


def test_small_knot_converges_to_fp64(small_knot):
    sc, prep = small_knot
    r, (col, *_) = _gpu(sc, 48, 27, 512, seed=5)
    ref, *_ = OR.render(prep, 48, 27, 5, 512, max_bounces=12, precision=64)
    # The same 512 samples per pixel on both sides; residual differences are
    # the few samples whose path a rounding flip sent elsewhere. For scale:
    # two binary64 renders with different seeds differ by 3.5% relative RMSE
    # here, the oracle's binary32 and binary64 renders of one seed by 0.05%.
    assert _rel_rmse(col[..., :3], ref[..., :3]) < 0.01
    r.dispose()


def test_full_knot_workload():
    sc = W.knot_scene(0)
    r, (col, alb, nrm, hist) = _gpu(sc, 1920, 1080, 256)
    assert np.all(hist == 256) and not np.isnan(col).any()
    st = r.stats()
    assert st["triangles"] == 2_000_000
    prep = OR.prepare(sc)
    for x0, y0 in ((760, 600), (1150, 400)):
        oc, oa, *_ = OR.render(prep, 1920, 1080, 0, 256, max_bounces=12, crop=(x0, y0, 32, 32))
        g = col[y0:y0 + 32, x0:x0 + 32, :3]
        assert (oa[..., 3] > 0.5).mean() > 0.5  # mostly on the knot
        assert _close_frac(alb[y0:y0 + 32, x0:x0 + 32], oa, 2e-3) > 0.97
        assert _rel_rmse(g, oc[..., :3]) < 0.05
    # five a-trous iterations, then the display pass
    r.denoise(5)
    den = r.read_denoised()
    assert not np.isnan(den).any()
    img = r.display(1.0)
    assert img.shape == (1080, 1920, 4) and img[..., :3].std() > 5
    r.dispose()
