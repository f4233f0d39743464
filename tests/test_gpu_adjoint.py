"""Path replay backpropagation (lucent_renderer_backward) vs binary64 finite
differences of the oracle.

The reference of the gradient is the oracle's detached-sampling estimator
(orc_detached_dot): the same paths (seeds, directions, pdfs, MIS weights,
lobe and roulette choices, clamp scales) with BSDF values and environment
radiance taken from perturbed parameters, differenced centrally in binary64.
That is exactly the quantity path replay differentiates, so the two agree up
to binary32 rounding and the rare sample whose path a binary32 rounding
sends elsewhere; the bar is 1e-3 relative.
"""
import numpy as np
import pytest

from oracle import render as OR
from lucent_gb300 import adjoint as AD
from lucent_gb300 import workloads as W
from lucent_gb300._native import LucentError
from lucent_gb300.renderer import Renderer

pytestmark = pytest.mark.gpu

W_, H_, SPP, SEED, DEPTH = 64, 64, 4, 7, 6


@pytest.fixture(scope="module")
def setup():
    sc = W.adjoint_scene(0, 4)  # 5,156 triangles, 33 materials, 256 x 128 HDRI
    r = Renderer(W_, H_)
    r.settings.max_bounces = DEPTH
    r.load_scene(sc)
    prep = OR.prepare(sc)
    dl = np.zeros((H_, W_, 4), np.float32)
    dl[..., :3] = np.random.default_rng(0).uniform(0.5, 1.5, (H_, W_, 3))
    img = AD.forward(r, SPP, SEED)
    dm, de = AD.backward(r, SPP, SEED, dl[..., :3])
    yield sc, r, prep, dl, img, dm, de
    r.dispose()


def _dot(prep, dl, mats=None, env=None):
    return OR.detached_dot(prep, W_, H_, SEED, SPP, dl, materials_eval=mats, env_eval=env, max_bounces=DEPTH)


def test_forward_matches_oracle(setup):
    sc, r, prep, dl, img, dm, de = setup
    g = float((dl[..., :3].astype(np.float64) * img).sum())
    o = _dot(prep, dl)
    assert abs(g - o) / abs(o) < 1e-3


def test_material_gradients_match_finite_differences(setup):
    sc, r, prep, dl, img, dm, de = setup
    assert dm.shape == (33, 6) and np.isfinite(dm).all()
    m0 = prep.packed.materials.copy()
    th = AD.get_params(m0)
    h = 1e-4
    errs = []
    for idx in np.argsort(-np.abs(dm).reshape(-1))[:24]:  # the 24 largest gradients
        m, k = divmod(int(idx), 6)
        lo, hi = AD.PARAM_RANGES[k]
        tp, tm = th.copy(), th.copy()
        tp[m, k] = min(hi, th[m, k] + h)
        tm[m, k] = max(lo, th[m, k] - h)
        fd = (_dot(prep, dl, AD.set_params(m0, tp)) - _dot(prep, dl, AD.set_params(m0, tm))) / (tp[m, k] - tm[m, k])
        errs.append(abs(dm[m, k] - fd) / abs(fd))
    errs = np.array(errs)
    assert np.median(errs) < 2e-4 and errs.max() < 1e-3, errs


def test_environment_gradients_match_finite_differences(setup):
    sc, r, prep, dl, img, dm, de = setup
    assert de.shape == (128, 256, 3) and np.isfinite(de).all()
    env0 = prep.env_data.copy()
    flat = de.reshape(-1)
    errs = []
    for idx in np.argsort(-np.abs(flat))[:12]:
        step = 1e-3 * max(1.0, abs(float(env0[idx])))
        ep, em = env0.copy(), env0.copy()
        ep[idx] += step
        em[idx] -= step
        fd = (_dot(prep, dl, env=ep) - _dot(prep, dl, env=em)) / (float(ep[idx]) - float(em[idx]))
        errs.append(abs(flat[idx] - fd) / abs(fd))
    assert max(errs) < 1e-3, errs


def test_backward_leaves_the_image_alone_and_is_linear_in_dl(setup):
    sc, r, prep, dl, img, dm, de = setup
    before = r.read()[0].copy()
    dm2, de2 = AD.backward(r, SPP, SEED, 2.0 * dl[..., :3])
    assert np.array_equal(r.read()[0], before)
    np.testing.assert_allclose(dm2, 2.0 * dm, rtol=1e-4, atol=1e-6 * np.abs(dm).max())
    np.testing.assert_allclose(de2, 2.0 * de, rtol=1e-4, atol=1e-6 * np.abs(de).max())


def test_gradient_descent_reduces_the_image_loss():
    # Target from the scene's own parameters; start from perturbed parameters
    # and descend along the adjoint's gradient. Every render uses the same
    # samples (seed 0), so the loss is a smooth function of the parameters
    # that is zero at the target's.
    sc = W.adjoint_scene(1, 3)
    r = Renderer(48, 48)
    r.settings.max_bounces = 4
    r.load_scene(sc)
    gt = AD.get_params(r.packed.materials)
    target = AD.forward(r, 16, 0)
    rng = np.random.default_rng(5)
    theta = np.clip(gt + rng.normal(0, 0.1, gt.shape), 0, 1).astype(np.float32)
    losses = []
    m1, m2 = np.zeros_like(theta), np.zeros_like(theta)  # Adam, lr 0.02
    for it in range(1, 13):
        img = AD.forward(r, 16, 0, theta=theta)
        losses.append(float(((img - target) ** 2).sum()))
        dm, _ = AD.backward(r, 16, 0, 2.0 * (img - target), env_grad=False)
        m1 = 0.9 * m1 + 0.1 * dm
        m2 = 0.999 * m2 + 0.001 * dm * dm
        step = (m1 / (1 - 0.9 ** it)) / (np.sqrt(m2 / (1 - 0.999 ** it)) + 1e-8)
        theta = np.clip(theta - 0.02 * 0.85 ** it * step, 0, 1).astype(np.float32)
    assert min(losses[4:]) < 0.5 * losses[0], losses
    r.dispose()


def test_backward_errors(setup):
    sc, r, prep, dl, img, dm, de = setup
    with pytest.raises(LucentError):
        bad = np.full((H_, W_, 3), np.nan, np.float32)
        AD.backward(r, SPP, SEED, bad)
    with pytest.raises(LucentError):
        AD.set_materials(r, np.zeros(40 * 3, np.float32))  # wrong material count
