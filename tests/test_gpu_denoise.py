"""Denoiser (variance.frag + atrous.frag, run as runDenoiser) and display
pass (display.frag) on the GPU vs the oracle's restatement.

Both sides get the same inputs: the GPU renderer's own accumulation targets,
read back after tracing, go through the oracle's denoiser and display pass.
The kernels keep the shaders' unfused multiply-add order, so the only
differences left are expf/powf last-place rounding, carried through up to
five filter iterations: the tolerances below bound that (relative 1e-4 on
the filtered illumination, 1e-3 on the propagated variance, 2e-6 on the
display values before quantization, and at most one 8-bit step after it).
"""
import numpy as np
import pytest

from oracle import render as OR
from lucent_gb300 import workloads as W
from lucent_gb300.renderer import Renderer, atrous_levels, denoise_weight

pytestmark = pytest.mark.gpu


def _camera(r):
    c = OR.OrcCamera()
    s = r.camera_state
    c.pos[:], c.right[:], c.up[:], c.forward[:] = s.position, s.right, s.up, s.forward
    c.tan_half_fov, c.aperture, c.focus_dist = s.tan_half_fov, s.aperture, s.focus_distance
    return c


def _renderer(scene, w, h, spp, seed=0):
    r = Renderer(w, h)
    r.settings.max_bounces = 8
    r.load_scene(scene)
    r.set_seed(seed)
    if spp:
        r.trace_samples(spp)
    return r


def _rel_err(a, b, floor):
    return np.abs(a - b) / (np.abs(b) + floor)


def _check_denoised(g, o):
    assert not np.isnan(g).any()
    e_rgb = _rel_err(g[..., :3], o[..., :3], 1e-4)
    assert e_rgb.max() < 1e-4, e_rgb.max()
    e_var = _rel_err(g[..., 3], o[..., 3], 1e-7)
    assert e_var.max() < 1e-3, e_var.max()


@pytest.mark.parametrize("spp,size", [(1, (64, 64)), (4, (50, 37)), (16, (96, 64)), (64, (64, 48))])
def test_denoise_matches_oracle(spp, size):
    # spp < 4 takes the 7x7 spatial variance; spp >= 4 the second moment.
    # The level count follows atrousLevels(spp): 5, 5, 4, 3.
    w, h = size
    r = _renderer(W.box_scene(0, 3), w, h, spp, seed=3)
    levels = atrous_levels(spp)
    r.denoise(levels)
    g = r.read_denoised()
    col, alb, nrm, hist = r.read()
    o = OR.denoise(col, alb, nrm, hist, _camera(r), levels)
    _check_denoised(g, o)
    cov = alb[..., 3] >= 0.5
    assert cov.mean() > 0.3
    # uncovered pixels pass the raw colour through every pass
    assert np.array_equal(g[~cov][:, :3], col[~cov][:, :3])
    r.dispose()


@pytest.mark.parametrize("levels", [0, 1, 2, 5])
def test_denoise_level_counts(levels):
    r = _renderer(W.box_scene(2, 3), 40, 40, 2, seed=1)
    r.denoise(levels)
    g = r.read_denoised()
    col, alb, nrm, hist = r.read()
    _check_denoised(g, OR.denoise(col, alb, nrm, hist, _camera(r), levels))
    r.dispose()


def test_denoise_sigmas():
    r = _renderer(W.box_scene(1, 3), 48, 40, 8, seed=5)
    r.denoise(3, sigma_l=1.0, sigma_n=16.0, sigma_p=4.0)
    g = r.read_denoised()
    col, alb, nrm, hist = r.read()
    _check_denoised(g, OR.denoise(col, alb, nrm, hist, _camera(r), 3, 1.0, 16.0, 4.0))
    r.dispose()


@pytest.mark.parametrize("tonemap,tm", [("aces", 0), ("reinhard", 1), ("none", 2)])
@pytest.mark.parametrize("weight,exposure", [(0.0, 1.0), (1.0, 1.0), (0.4, 2.5)])
def test_display_matches_oracle(tonemap, tm, weight, exposure):
    r = _renderer(W.box_scene(0, 3), 64, 48, 8, seed=2)
    den = None
    if weight > 0:
        r.denoise(4)
        den = r.read_denoised()
    img, rgb = r.display(weight, exposure=exposure, tonemap=tonemap, want_float=True)
    col, alb, *_ = r.read()
    o = OR.display(col, alb, den, weight, exposure, tm)
    assert np.abs(rgb - o).max() < 2e-6, np.abs(rgb - o).max()
    q = np.rint(np.clip(o, 0, 1) * 255).astype(np.int32)
    d = np.abs(img[..., :3].astype(np.int32) - q)
    assert d.max() <= 1 and (d == 0).mean() > 0.999
    assert np.all(img[..., 3] == 255)
    r.dispose()


@pytest.mark.parametrize("view", [(100, 75), (128, 96), (50, 31), (64, 48)])
def test_display_view_matches_oracle(view):
    # display.frag's Catmull-Rom branch: the renderer's 64 x 48 targets as the
    # traced region shown in a view of another size (the reference's preview
    # while the camera moves); at equal sizes the plain display pass.
    r = _renderer(W.box_scene(0, 3), 64, 48, 8, seed=3)
    r.denoise(3)
    den = r.read_denoised()
    col, alb, *_ = r.read()
    for weight, tonemap, tm in ((0.0, "aces", 0), (0.6, "reinhard", 1), (0.3, "none", 2)):
        img, rgb = r.display(weight, exposure=1.5, tonemap=tonemap, want_float=True, view=view)
        assert img.shape == (view[1], view[0], 4) and rgb.shape == (view[1], view[0], 3)
        o = OR.display_view(col, alb, den, view[0], view[1], weight, 1.5, tm)
        assert np.abs(rgb - o).max() < 1e-4, np.abs(rgb - o).max()
        q = np.rint(np.clip(o, 0, 1) * 255).astype(np.int32)
        d = np.abs(img[..., :3].astype(np.int32) - q)
        assert d.max() <= 1 and (d == 0).mean() > 0.995
    if view == (64, 48):
        assert np.array_equal(r.display(0.3, exposure=1.5, tonemap="none"),
                              r.display(0.3, exposure=1.5, tonemap="none", view=view))
    r.dispose()


def test_render_loop_denoises_then_presents():
    # render() traces samples_per_frame, denoises with atrousLevels(frame)
    # and blends with denoiseWeight(frame), like the reference's render().
    r = _renderer(W.box_scene(0, 3), 48, 48, 0, seed=0)
    r.settings.samples_per_frame = 2
    for _ in range(3):
        img = r.render()
    assert r.samples() == 6
    col, alb, nrm, hist = r.read()
    den = OR.denoise(col, alb, nrm, hist, _camera(r), atrous_levels(6))
    o = OR.display(col, alb, den, denoise_weight(6), 1.0, 0)
    q = np.rint(np.clip(o, 0, 1) * 255).astype(np.int32)
    assert np.abs(img[..., :3].astype(np.int32) - q).max() <= 1
    r.settings.max_samples = 7
    r.render()
    r.render()  # nothing left to trace
    assert r.samples() == 7
    r.dispose()


def test_denoised_is_closer_to_converged():
    # SVGF's purpose: at 4 spp the filtered image is nearer the converged
    # render than the raw accumulation, both as displayed (tone-mapped sRGB)
    # and in linear radiance away from the directly seen light (whose pixels,
    # up to ~200x brighter, dominate a linear RMSE and are not filtered
    # differently from any other). Oracle calibration: display RMSE 0.102 ->
    # 0.056, off-light linear RMSE 0.139 -> 0.052.
    sc = W.box_scene(1, 3)
    r = _renderer(sc, 64, 64, 4, seed=11)
    r.denoise(atrous_levels(4))
    den = r.read_denoised()
    col, alb, *_ = r.read()
    shown_raw = r.display(0.0, want_float=True)[1]
    shown_den = r.display(1.0, want_float=True)[1]
    ref_r = _renderer(sc, 64, 64, 512, seed=1000)
    ref, *_ = ref_r.read()
    shown_ref = ref_r.display(0.0, want_float=True)[1]
    cov = alb[..., 3] >= 0.5
    remod = np.where(cov[..., None], den[..., :3] * np.maximum(alb[..., :3], 1e-3), col[..., :3])
    off_light = cov & (ref[..., :3].mean(-1) < 2)

    def rmse(x, m=None):
        return np.sqrt(np.mean(x ** 2 if m is None else x[m] ** 2))

    assert rmse(shown_den - shown_ref) < 0.7 * rmse(shown_raw - shown_ref)
    assert rmse(remod - ref[..., :3], off_light) < 0.5 * rmse(col[..., :3] - ref[..., :3], off_light)
    r.dispose()
    ref_r.dispose()


def test_denoise_and_display_errors():
    from lucent_gb300._native import LucentError
    r = _renderer(W.box_scene(0, 2), 16, 16, 1)
    with pytest.raises(LucentError):
        r.denoise(6)
    with pytest.raises(LucentError):
        r.display(0.5)  # no denoised image yet
    with pytest.raises(LucentError):
        r.read_denoised()
    r.denoise(1)
    r.display(0.5)
    r.reset()
    with pytest.raises(LucentError):
        r.display(0.5)  # reset drops the filtered image
    with pytest.raises(KeyError):
        r.display(0.0, tonemap="filmic")
    r.dispose()
