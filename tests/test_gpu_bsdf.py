"""The renderer's BSDF (bsdf.glsl evalOpaque, sampleOpaque, sampleDielectric
as compiled into the shade kernel) vs the oracle's binary64 evaluation of the
same formulas on 10^6 seeded tuples.

Error measure: for every output component, |gpu - f64| / max(|f64|, floor)
with floor = 1e-6 times the component's largest magnitude over all tuples
(values below that are noise around zero, e.g. a lobe's far tail).

- evalOpaque f and pdf: within 1e-5 relative.
- sampleOpaque: the sampled direction within 1e-5 (absolute, unit vectors)
  of the binary64 direction; its pdf and weight against the binary64
  evaluation AT THE DIRECTION THE GPU RETURNED (pdf = evalOpaque pdf there,
  weight = f cos / pdf), since the pdf of a sharp lobe changes by percents
  when its direction moves by one binary32 ulp.
- sampleDielectric: flags equal, direction within 1e-5, weight exact.
A discrete choice (lobe, reflect/refract, ok) compares a uniform with a
binary32 probability: where the two lie within 1e-5 the binary64 choice may
differ; such tuples are counted and must stay below 1 in 10^4.
"""
import numpy as np
import pytest

from oracle import render as OR
from lucent_gb300.renderer import bsdf_eval_tuples

pytestmark = pytest.mark.gpu

N_TUPLES = 1_000_000


def make_tuples(n, seed=0):
    """Materials in the layered model's ranges; unit n, clearcoat normal
    near n, wo in n's hemisphere, wi anywhere, six uniforms, front face."""
    g = np.random.default_rng(seed)
    t = np.zeros((n, 32), np.float32)
    t[:, 0:3] = g.uniform(0, 1, (n, 3))
    t[:, 3] = g.uniform(size=n) < 0.5
    t[:, 4] = g.uniform(0.0, 1, n)
    t[:, 5] = g.uniform(1.0, 2.5, n)
    t[:, 6] = np.where(g.uniform(size=n) < 0.3, 0, g.uniform(0, 1, n))
    t[:, 7] = g.uniform(0.0, 1, n)
    sheen = np.where(g.uniform(size=n) < 0.3, 0, g.uniform(0, 1, n))
    t[:, 8:11] = sheen[:, None] * g.uniform(0.5, 1, (n, 3))
    t[:, 11] = g.uniform(0, 1, n)
    t[:, 12] = g.uniform(size=n) < 0.2

    def unit(m):
        v = g.normal(size=(m, 3))
        return v / np.linalg.norm(v, axis=1, keepdims=True)

    nrm = unit(n).astype(np.float32)
    t[:, 13:16] = nrm
    nc = nrm + 0.2 * unit(n)
    t[:, 16:19] = nc / np.linalg.norm(nc, axis=1, keepdims=True)
    wo = unit(n)
    t[:, 19:22] = np.where((wo * nrm).sum(1, keepdims=True) < 0, -wo, wo)
    t[:, 22:25] = unit(n)
    t[:, 25:31] = g.uniform(0, 1, (n, 6))
    t[:, 31] = g.uniform(size=n) < 0.5
    return t


def rel_err(g, r):
    floor = 1e-6 * np.abs(r).max(axis=0, keepdims=True)
    return np.abs(g - r) / np.maximum(np.abs(r), np.maximum(floor, 1e-30))


@pytest.fixture(scope="module")
def evaluated():
    t = make_tuples(N_TUPLES)
    g = bsdf_eval_tuples(t).astype(np.float64)
    r = OR.bsdf_tuples(t, 64)
    return t, g, r


def _report(name, e):
    q = np.quantile(e, [0.5, 0.999, 0.99999]) if e.size else [0, 0, 0]
    print(f"{name}: n={e.size} median={q[0]:.2e} p99.9={q[1]:.2e} p99.999={q[2]:.2e} max={e.max() if e.size else 0:.2e}"
          f" frac>1e-5={(e > 1e-5).mean() if e.size else 0:.2e}")


def test_eval_opaque(evaluated):
    t, g, r = evaluated
    e = rel_err(g[:, 0:4], r[:, 0:4]).max(axis=1)
    _report("evalOpaque f,pdf", e)
    zero = (r[:, 0:4] == 0).all(axis=1)
    assert (g[zero, 0:4] == 0).mean() > 0.9999  # below-horizon gates agree
    assert (e > 1e-5).mean() < 1e-4, (e > 1e-5).mean()


def test_sample_opaque(evaluated):
    t, g, r = evaluated
    both = (g[:, 10] > 0) & (r[:, 10] > 0)
    flip = (g[:, 10] > 0) != (r[:, 10] > 0)
    dir_err = np.abs(g[:, 4:7] - r[:, 4:7]).max(axis=1)
    same_lobe = both & (dir_err < 1e-3)
    print(f"sampleOpaque: valid both {both.mean():.4f}, validity differs {flip.mean():.2e}, "
          f"lobe differs {(both & ~same_lobe).mean():.2e}")
    _report("sampleOpaque dir (abs)", dir_err[same_lobe])
    assert (flip | (both & ~same_lobe)).mean() < 1e-4
    assert (dir_err[same_lobe] > 1e-5).mean() < 1e-4
    # pdf and weight against binary64 at the GPU's own direction
    t2 = t[same_lobe].copy()
    t2[:, 22:25] = g[same_lobe, 4:7].astype(np.float32)
    r2 = OR.bsdf_tuples(t2, 64)
    n = t2[:, 13:16].astype(np.float64)
    cos = (n * t2[:, 22:25].astype(np.float64)).sum(1)
    pdf = r2[:, 3]
    ok = pdf > 0
    w_ref = r2[ok, 0:3] * (cos[ok] / pdf[ok])[:, None]
    e_pdf = rel_err(g[same_lobe, 10][ok], pdf[ok])
    e_w = rel_err(g[same_lobe, 7:10][ok], w_ref).max(axis=1)
    _report("sampleOpaque pdf at gpu dir", e_pdf)
    _report("sampleOpaque weight at gpu dir", e_w)
    assert ok.mean() > 0.9999
    assert (e_pdf > 1e-5).mean() < 1e-4 and (e_w > 1e-5).mean() < 1e-4


def test_sample_dielectric(evaluated):
    t, g, r = evaluated
    same = (g[:, 11] == r[:, 11]) & (g[:, 18] == r[:, 18])
    print(f"sampleDielectric: flags differ {(~same).mean():.2e}")
    assert (~same).mean() < 1e-4
    ok = same & (r[:, 11] == 1)
    d = np.abs(g[ok, 12:15] - r[ok, 12:15]).max(axis=1)
    _report("sampleDielectric dir (abs)", d)
    assert (d > 1e-5).mean() < 1e-4
    assert np.array_equal(g[ok, 15:18], r[ok, 15:18].astype(np.float32).astype(np.float64))


def test_eval_gradient_matches_fp64_finite_differences():
    """The adjoint's BSDF derivative (eval_opaque_grad) vs central
    differences of the oracle's binary64 evalOpaque, step 1e-4 (one-sided at
    a range end, e.g. clearcoat = 0 or metallic in {0, 1}, where the
    one-sided difference's own truncation error is ~1e-4); tuples within two
    steps of the roughness clamp (alpha = max(r^2, 1e-3)) are skipped. Bar:
    1e-3 relative (floor 1e-3 of the component's largest value) on all but
    1 in 10^3 tuples."""
    from lucent_gb300.renderer import bsdf_grad_tuples
    n = 100_000
    t = make_tuples(n, seed=3)
    g = bsdf_grad_tuples(t).astype(np.float64)
    h = 1e-4
    cols = {0: 0, 1: 1, 2: 2, 3: 4, 4: 3, 5: 6}  # adjoint parameter -> tuple column
    keep = np.abs(t[:, 4] - np.sqrt(1e-3)) > 2 * h
    for p, col in cols.items():
        up, dn = t.copy(), t.copy()
        lo_edge = t[:, col] - h < 0
        hi_edge = t[:, col] + h > 1
        up[:, col] = np.where(hi_edge, t[:, col], t[:, col] + h)
        dn[:, col] = np.where(lo_edge, t[:, col], t[:, col] - h)
        fp = OR.bsdf_tuples(up, 64)[:, 0:3]
        fm = OR.bsdf_tuples(dn, 64)[:, 0:3]
        fd = (fp - fm) / (up[:, col:col + 1] - dn[:, col:col + 1]).astype(np.float64)
        gd = g[:, 3 + 3 * p:6 + 3 * p]
        scale = np.abs(fd).max(axis=0, keepdims=True)  # channels a parameter does not touch have fd = gd = 0
        err = (np.abs(gd - fd) / np.maximum(np.abs(fd), np.maximum(1e-3 * scale, 1e-12))).max(axis=1)[keep]
        _report("d f / d %s" % ("r", "g", "b", "roughness", "metallic", "clearcoat")[p], err)
        assert (err > 1e-3).mean() < 1e-3, (p, (err > 1e-3).mean())
