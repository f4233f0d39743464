"""buildEnvSampler on the GPU (lucent_env_sampler_device) against the host's
(lucent_env_sampler, equal to the oracle's restatement of
environment.ts:52-85 and alias.ts:17-65 bit for bit).

The device build's cell weights are the reference's; its total and its
prefix sums are exact double-double scans where the reference sums left to
right in binary64, and its alias pairing is the closed form of Vose's stack
order over those sums. The tests hold it to the reference's own criteria
(alias.test: every cell drawn with its pmf to within 5e-7, zero-weight cells
never drawn) and to the host table: the same alias in every cell, the same
pdf columns, keep probabilities within 1e-7 (the reference's sequential sums
carry about 1e-9 of rounding that the exact scans do not). A renderer whose
map and sampler are set on the device renders what the oracle renders with
the same table."""
import ctypes as C

import numpy as np
import pytest

from oracle import render as OR
from lucent_gb300 import _native as N
from lucent_gb300 import _native_render as NR  # noqa: F401  (declares the signatures)
from lucent_gb300 import scene as S
from lucent_gb300 import workloads as W
from lucent_gb300.renderer import Renderer

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _host(rgb, w, h, max_w=1024):
    img = np.ascontiguousarray(rgb, np.float32).reshape(-1)
    gw, gh, total = C.c_uint32(), C.c_uint32(), C.c_double()
    N.check(N.lib().lucent_env_sampler(N.ptr(img, C.c_float), w, h, max_w, C.byref(gw), C.byref(gh), None, None))
    table = np.zeros(gw.value * gh.value * 4, np.float32)
    N.check(N.lib().lucent_env_sampler(N.ptr(img, C.c_float), w, h, max_w, C.byref(gw), C.byref(gh),
                                       N.ptr(table, C.c_float), C.byref(total)))
    return gw.value, gh.value, table.reshape(-1, 4), total.value


def _device(rgb, w, h, max_w=1024):
    d = torch.from_numpy(np.ascontiguousarray(rgb, np.float32).reshape(-1)).cuda()
    gw0 = max(1, min(w, max_w))
    gh0 = max(1, min(h, int(np.floor(h * gw0 / w + 0.5))))
    table = torch.zeros(gw0 * gh0 * 4, dtype=torch.float32, device="cuda")
    gw, gh, total = C.c_uint32(), C.c_uint32(), C.c_double()
    N.check(N.lib().lucent_env_sampler_device(d.data_ptr(), w, h, max_w, C.byref(gw), C.byref(gh),
                                              table.data_ptr(), C.byref(total), None))
    assert (gw.value, gh.value) == (gw0, gh0)
    return gw.value, gh.value, table.cpu().numpy().reshape(-1, 4), total.value


def _drawn(table):
    """Probability of drawing each cell: (prob_i + sum over j aliasing i of (1 - prob_j)) / n."""
    n = table.shape[0]
    prob = table[:, 0].astype(np.float64)
    alias = table[:, 1].astype(np.int64)
    p = prob / n
    np.add.at(p, alias, (1 - prob) / n)
    return p


def _check(rgb, w, h, max_w=1024):
    hg, hh, ht, htot = _host(rgb, w, h, max_w)
    dg, dh, dt, dtot = _device(rgb, w, h, max_w)
    assert (hg, hh) == (dg, dh)
    assert abs(dtot - htot) <= 1e-12 * max(htot, 1e-300)
    n = ht.shape[0]
    pmf = ht[:, 2].astype(np.float64) / n  # the host's pdfUV column: pmf * n rounded to binary32
    assert np.all(np.abs(_drawn(dt) - pmf) < 5e-7)
    zero = pmf == 0
    assert np.all(dt[zero, 0] == 0) and not np.isin(np.nonzero(zero)[0], dt[~zero, 1].astype(np.int64)).any()
    assert np.mean(dt[:, 1] == ht[:, 1]) >= 0.999
    assert np.mean(dt[:, 2] == ht[:, 2]) >= 0.9999
    assert np.all(np.abs(dt[:, 0].astype(np.float64) - ht[:, 0]) <= 1e-7)
    return np.all(dt == ht, axis=1).mean()


def test_device_sampler_on_the_large_mesh_hdri():
    sc = W.knot_scene(0, tubular=8, radial=4, env_width=1024)
    _check(sc.env.map.data, 1024, 512)


def test_device_sampler_on_sky_zero_rows_and_edge_cases():
    sc = W.sky_scene(0)
    sky = S.bake_sky(sc.sky, sc.sun, 256)
    _check(sky.data, sky.width, sky.height)
    _check(sky.data, sky.width, sky.height, max_w=100)
    rng = np.random.Generator(np.random.PCG64(3))
    img = rng.uniform(0, 2, (64, 128, 3)).astype(np.float32)
    img[20:30] = 0  # zero-weight rows: never drawn
    img[:, 5] = 0
    _check(img, 128, 64)
    _check(rng.uniform(0, 1, 37 * 19 * 3).astype(np.float32), 37, 19)
    _check(np.zeros(16 * 8 * 3, np.float32), 16, 8)  # black: uniform fallback
    single = np.zeros((32, 64, 3), np.float32)
    single[10, 20] = 5.0
    _check(single, 64, 32)


def test_device_sampler_reference_weights():
    """alias.test's weights [1, 0, 3, 6, 0.5, 9.5] as a 6 x 1 grey map
    (luminance = grey, sin(theta) = 1 on the single row)."""
    w = np.array([1, 0, 3, 6, 0.5, 9.5], np.float32)
    rgb = np.repeat(w[:, None], 3, 1)
    _, _, t, total = _device(rgb, 6, 1)
    p = _drawn(t)
    assert np.all(np.abs(p - w / w.sum()) < 5e-7)
    assert t[1, 0] == 0 and not (t[:, 1] == 1).any()


def test_rejects_bad_maps():
    bad = np.ones((4, 8, 3), np.float32)
    bad[1, 2] = -1
    with pytest.raises(N.LucentError):
        _device(bad, 8, 4)
    bad[1, 2] = np.inf
    with pytest.raises(N.LucentError):
        _device(bad, 8, 4)


def test_renderer_with_device_sampler_matches_oracle():
    sc = W.knot_scene(0, tubular=200, radial=16, env_width=256)
    w, h, spp = 96, 54, 2
    r = Renderer(w, h)
    r.settings.max_bounces = 12
    r.load_scene(sc)
    img = sc.env.map
    d = torch.from_numpy(np.ascontiguousarray(img.data, np.float32)).cuda()
    r.set_env_device(d.data_ptr(), img.width, img.height)
    r.trace_samples(spp)
    col, alb, nrm, hist = r.read()
    r.dispose()
    _, _, table, total = _device(img.data, img.width, img.height)
    prep = OR.prepare(sc)
    t = np.ascontiguousarray(table.reshape(-1), np.float32)
    prep.keep.append(t)
    prep.scene.env_alias = t.ctypes.data_as(C.POINTER(C.c_float))
    oc, oa, on, oh = OR.render(prep, w, h, 0, spp, max_bounces=12)
    assert np.array_equal(hist, oh)
    close = (np.abs(col[..., :3] - oc[..., :3]) <= 1e-3 * (np.abs(oc[..., :3]) + 1e-3)).mean()
    assert close > 0.95, close
