"""Host precompute of the lighting, checked without a GPU: the product's
buildEnvSampler (lucent_env_sampler, the table upload_lighting sends to the
device) equals the oracle's restatement of environment.ts:52-85 and
alias.ts:17-65 on the large-mesh workload's HDRI (1024 x 512, lognormal
luminance with a baked sun disk), a baked procedural sky and edge cases; the
product's bakeSky equals the oracle's restatement of environment.ts:106-132
and passes the reference's own test (environment.test.ts:138-147)."""
import ctypes as C

import numpy as np
import pytest

import oracle
from lucent_gb300 import _native as N
from lucent_gb300 import _native_render as NR  # noqa: F401  (declares the renderer signatures)
from lucent_gb300 import scene as S
from lucent_gb300 import workloads as W


def _product_sampler(rgb, w, h, max_w=1024):
    L = N.lib()
    img = np.ascontiguousarray(rgb, np.float32).reshape(-1)
    gw, gh, total = C.c_uint32(), C.c_uint32(), C.c_double()
    N.check(L.lucent_env_sampler(N.ptr(img, C.c_float), w, h, max_w, C.byref(gw), C.byref(gh), None, None))
    table = np.zeros(gw.value * gh.value * 4, np.float32)
    N.check(L.lucent_env_sampler(N.ptr(img, C.c_float), w, h, max_w, C.byref(gw), C.byref(gh),
                                 N.ptr(table, C.c_float), C.byref(total)))
    return gw.value, gh.value, table, total.value


def _same(rgb, w, h, max_w=1024):
    a = _product_sampler(rgb, w, h, max_w)
    b = oracle.build_env_sampler(rgb, w, h, max_w)
    assert a[0] == b[0] and a[1] == b[1]
    assert np.array_equal(a[2].view(np.uint32), b[2].view(np.uint32))
    assert a[3] == b[3]
    return a


def test_env_sampler_on_the_large_mesh_hdri():
    sc = W.knot_scene(0, tubular=8, radial=4, env_width=1024)  # the workload's HDRI; a tiny knot
    img = sc.env.map
    gw, gh, table, total = _same(img.data, img.width, img.height)
    assert (gw, gh) == (1024, 512) and total > 0
    # the baked sun disk is the brightest cell by far
    pdf = table.reshape(-1, 4)[:, 2]
    assert pdf.max() > 100 * np.median(pdf)


def test_env_sampler_on_baked_sky_and_edge_cases():
    sc = W.sky_scene(0)
    sky = S.bake_sky(sc.sky, sc.sun)
    _same(sky.data, sky.width, sky.height)
    _same(sky.data, sky.width, sky.height, max_w=200)  # averaged cells, gh rounded
    rng = np.random.Generator(np.random.PCG64(3))
    odd = rng.uniform(0, 2, 37 * 19 * 3).astype(np.float32)
    _same(odd, 37, 19)
    _same(odd, 37, 19, max_w=8)
    black = np.zeros(16 * 8 * 3, np.float32)
    assert _same(black, 16, 8)[3] == 0
    single = np.zeros(64 * 32 * 3, np.float32)
    single[(10 * 64 + 20) * 3 + 1] = 5.0
    _same(single, 64, 32)


def test_env_sampler_rejects_bad_weights():
    bad = np.ones(8 * 4 * 3, np.float32)
    bad[3:6] = -1.0  # a pixel of negative luminance: a negative cell weight (alias.ts:24)
    with pytest.raises(N.LucentError):
        _product_sampler(bad, 8, 4)
    bad[3:6] = 1.0
    bad[5] = np.inf
    with pytest.raises(N.LucentError):
        _product_sampler(bad, 8, 4)
    _product_sampler(np.ones(8 * 4 * 3, np.float32), 8, 4)  # a good call clears the thread's error text


def test_bake_sky_equals_oracle_and_reference_test():
    sc = W.sky_scene(0)
    for width in (64, 256, 1024):
        a = S.bake_sky(sc.sky, sc.sun, width).data.reshape(width // 2, width, 3)
        b = oracle.bake_sky(sc.sky, sc.sun, width)
        d = np.abs(a.view(np.int32).astype(np.int64) - b.view(np.int32).astype(np.int64))
        assert d.max() <= 1, d.max()  # numpy's and libm's sin/cos/pow may differ in the last place
    # environment.test.ts:138-147
    sky = S.Sky(enabled=True, zenith=(0.2, 0.4, 0.9), horizon=(0.8, 0.85, 0.95), ground=(0.3, 0.25, 0.2),
                intensity=2.0)
    sun = S.Sun(elevation=40.0, azimuth=0.0, color=(1.0, 1.0, 1.0), intensity=0.0, angular_radius=1.0)
    for img in (S.bake_sky(sky, sun, 64).data.reshape(32, 64, 3), oracle.bake_sky(sky, sun, 64)):
        assert img[0, 10, 2] > img[0, 10, 0]
        assert abs(img[0, 10, 2] - 2 * 0.9) < 0.05
        assert img[31, 10, 0] > img[31, 10, 2]
    off = S.Sky(enabled=False, zenith=sky.zenith, horizon=sky.horizon, ground=sky.ground, intensity=2.0)
    assert not S.bake_sky(off, sun, 64).data.any() and not oracle.bake_sky(off, sun, 64).any()


def test_sun_uniforms():
    """uploadLighting's sun (renderer.ts:359-367): on only without an
    environment map, radiance = colour x intensity / solid angle, pdf =
    1 / solid angle."""
    import math
    sc = W.sky_scene(0)
    L = S.lighting(sc)
    solid = 2 * math.pi * (1 - math.cos(math.radians(sc.sun.angular_radius)))
    assert L.sun_enabled == 1
    assert abs(L.sun_pdf - 1 / solid) < 1e-12 * L.sun_pdf
    assert np.allclose(L.sun_radiance, np.array(sc.sun.color) * sc.sun.intensity / solid)
    sc.env.map = S.HDRImage(2, 1, np.ones(6, np.float32))
    assert S.lighting(sc).sun_enabled == 0  # renderer.ts:362
