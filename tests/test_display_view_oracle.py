"""The oracle's display pass with a view size (display.frag:42-67): at equal
sizes it is the plain pass; when the view differs, the Catmull-Rom weights of
display.frag:51-54 sum to one, so a constant traced region shows as the same
constant (before the dither, which depends on the view pixel only), and the
upsampled image interpolates the region's texels at their centres."""
import numpy as np

from oracle import render as OR


def _images(h, w, seed):
    rng = np.random.default_rng(seed)
    col = rng.uniform(0, 2, (h, w, 4)).astype(np.float32)
    alb = rng.uniform(0, 1, (h, w, 4)).astype(np.float32)
    alb[..., 3] = (rng.random((h, w)) > 0.2).astype(np.float32)
    den = rng.uniform(0, 2, (h, w, 4)).astype(np.float32)
    return col, alb, den


def test_equal_sizes_are_the_plain_pass():
    col, alb, den = _images(30, 40, 0)
    for weight, exposure, tm in ((0.0, 1.0, 0), (0.5, 2.0, 1), (1.0, 0.7, 2)):
        assert np.array_equal(OR.display(col, alb, den, weight, exposure, tm),
                              OR.display_view(col, alb, den, 40, 30, weight, exposure, tm))


def test_constant_region_stays_constant():
    col, alb, den = _images(30, 40, 1)
    col[..., :3] = 0.3
    for vw, vh in ((64, 48), (100, 75), (41, 29), (20, 15)):
        up = OR.display_view(col, alb, den, vw, vh, 0.0, 1.0, 2)
        flat = OR.display_view(np.full((vh, vw, 4), 0.3, np.float32), np.ones((vh, vw, 4), np.float32), None,
                               vw, vh, 0.0, 1.0, 2)
        assert np.abs(up - flat).max() < 1e-6


def test_upsampling_reproduces_a_linear_ramp():
    # Catmull-Rom reproduces linear functions: a ramp across the region comes
    # out as the ramp sampled at each view pixel's texel coordinate
    # (x + 0.5) * w / vw - 0.5, away from the clamped border.
    h, w = 16, 20
    ramp = np.zeros((h, w, 4), np.float32)
    ramp[..., 0] = np.linspace(0.0, 0.5, w, dtype=np.float32)[None, :]
    alb = np.ones((h, w, 4), np.float32)
    vw, vh = 2 * w, 2 * h
    up = OR.display_view(ramp, alb, None, vw, vh, 0.0, 1.0, 2)
    dither = OR.display_view(np.zeros((vh, vw, 4), np.float32), alb[:1, :1].repeat(vh, 0).repeat(vw, 1), None,
                             vw, vh, 0.0, 1.0, 2)  # zero radiance: the dither alone

    def srgb(v):
        return np.where(v < 0.0031308, v * 12.92, 1.055 * np.power(v, 1 / 2.4) - 0.055)

    xs = np.arange(4, vw - 4)
    expect = srgb(np.interp((xs + 0.5) * w / vw - 0.5, np.arange(w), ramp[0, :, 0].astype(np.float64)))
    got = (up - dither)[vh // 2, xs, 0]
    assert np.abs(got - expect).max() < 1e-5
