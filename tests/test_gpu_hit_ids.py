"""Hit ids of the renderer's own traversal against the reference's CPU intersector.

The bench's path-tracing workload (box scene seed 0: 81,956 triangles,
512x512, 16 spp, depth 8) traces its closest-hit rays with the renderer's
policy: sorted ray streams, the four-wide view, the top BVH levels staged in
shared memory, tMin = EPS (1e-6, common.glsl:8) and tMax = 1e30. The renderer
captures every ray of chosen bounces with the hit it found
(lucent_renderer_capture_rays), and this test runs the same binary32 rays
through the oracle's binary64 intersectBVH (src/math/bvh.ts:265-320) with the
same tMin/tMax: every id must be equal (the renderer's slot mapped through
the BVH's triIndices), misses included (t = 1e30, the shaders' INF,
common.glsl). The renderer stores binary32 estimates of t, u, v like the
GLSL's own hitTriangle (the BVH API returns the binary64 values rounded);
each must lie within the error bound the traversal's binary32 test works
with (2^-19 x the absolute-value evaluations of the numerator and of det, so
2^-18 (xA + |x| dA) / |det| for a quotient) of the binary64 value.

Shadow rays (occluded, scene.glsl:336-377) are checked the same way against
the oracle's any-hit over the same tree, and the alpha-tested torus knot
exercises the alpha any-hit inside both traversals (the blend test draws from
the captured per-path key).
"""
import numpy as np
import pytest

import oracle
from oracle import render as OR
from lucent_gb300 import workloads as W
from lucent_gb300.renderer import Renderer

pytestmark = pytest.mark.gpu

T_MIN, T_MAX = 1e-6, 1e30
GLSL_INF = np.float32(1e30)


def _trace(scene, w, h, spp, bounces, max_bounces=8, sort=True, wide=True, top=True, seed=0):
    r = Renderer(w, h)
    r.settings.max_bounces = max_bounces
    r.load_scene(scene)
    r.set_ray_sort(sort)
    r.set_wide_bvh(wide)
    r.set_top_levels(top)
    r.set_seed(seed)
    r.capture_rays(bounces, max_rays=w * h * spp)
    r.trace_samples(spp)
    out = {b: (r.read_rays(b), r.read_rays(b, shadow=True)) for b in bounces}
    r.dispose()
    return out


def _check_closest(prep, rec, use_intersect_bvh=True):
    rays = np.ascontiguousarray(rec[:, [0, 1, 2, 4, 5, 6]])
    slot = rec[:, 11].view(np.int32)
    t32 = rec[:, 8]
    keys = rec[:, 12].view(np.uint32)
    assert rays.shape[0] > 0
    # The renderer's slot is the BVH leaf slot; the reference reports triIndices[slot].
    tri = prep.bvh.tri_indices.astype(np.int64)
    gpu_ids = np.where(slot >= 0, tri[np.maximum(slot, 0)], -1)
    u64 = v64 = None
    if use_intersect_bvh:  # the reference's CPU intersector itself (no alpha in this scene)
        ids, t64, u64, v64 = oracle.intersect_bvh(prep.bvh, prep.packed.positions, rays, T_MIN, T_MAX)
        ids = ids.astype(np.int64)
    else:  # alpha-tested scene: the same traversal with the alpha test before a hit counts
        oslot, t64 = OR.closest_slots(prep, rays, keys, T_MIN, T_MAX)
        ids = np.where(oslot >= 0, tri[np.maximum(oslot, 0)], -1)
    bad = np.nonzero(gpu_ids != ids)[0]
    assert bad.size == 0, "%d of %d ids differ, first at ray %d: gpu %d oracle %d" % (
        bad.size, ids.size, bad[0], gpu_ids[bad[0]], ids[bad[0]])
    hit = ids >= 0
    assert np.all(t32[~hit] == GLSL_INF)
    bt, bu, bv = _estimate_bounds(prep, rays[hit], slot[hit])
    err_t = np.abs(t32[hit].astype(np.float64) - t64[hit])
    assert np.all(err_t <= bt), float((err_t / bt).max())
    if u64 is not None:
        assert np.all(np.abs(rec[hit, 9].astype(np.float64) - u64[hit]) <= bu)
        assert np.all(np.abs(rec[hit, 10].astype(np.float64) - v64[hit]) <= bv)
    return int(hit.sum()), int(ids.size)


def _estimate_bounds(prep, rays, slots):
    """Error bounds of the binary32 estimates of t, u, v (mt_classify in
    closest_hit.cuh): numerators and det within 2^-19 of their absolute-value
    evaluations, so x = X / det within 2^-18 (xA + |x| dA) / |det|."""
    tri = prep.bvh.tri_indices.astype(np.int64)[slots]
    v = prep.packed.positions.reshape(-1, 3, 3)[tri].astype(np.float64)
    o, d = rays[:, :3].astype(np.float64), rays[:, 3:].astype(np.float64)
    e1, e2, s = v[:, 1] - v[:, 0], v[:, 2] - v[:, 0], o - v[:, 0]
    p, q = np.cross(d, e2), np.cross(s, e1)
    det = np.einsum("ij,ij->i", e1, p)
    ad, ae1, ae2, as_ = np.abs(d), np.abs(e1), np.abs(e2), np.abs(s)

    def across(a, b):
        return np.stack([a[:, 1] * b[:, 2] + a[:, 2] * b[:, 1], a[:, 2] * b[:, 0] + a[:, 0] * b[:, 2],
                         a[:, 0] * b[:, 1] + a[:, 1] * b[:, 0]], 1)

    ap, aq = across(ad, ae2), across(as_, ae1)
    dA = np.einsum("ij,ij->i", ae1, ap)
    uA, vA, tA = np.einsum("ij,ij->i", as_, ap), np.einsum("ij,ij->i", ad, aq), np.einsum("ij,ij->i", ae2, aq)
    t = np.einsum("ij,ij->i", e2, q) / det
    u = np.einsum("ij,ij->i", s, p) / det
    w = np.einsum("ij,ij->i", d, q) / det
    g = 2.0 ** -18 / np.abs(det)
    tiny = 1e-30
    return g * (tA + np.abs(t) * dA) + tiny, g * (uA + np.abs(u) * dA) + tiny, g * (vA + np.abs(w) * dA) + tiny


def _check_shadow(prep, rec):
    if rec.shape[0] == 0:
        return 0
    rays7 = np.ascontiguousarray(rec[:, [0, 1, 2, 4, 5, 6, 3]])
    keys = rec[:, 7].view(np.uint32)
    occ = rec[:, 8] > 0.5
    ref = OR.any_slots(prep, rays7, keys, T_MIN)
    bad = np.nonzero(occ != ref)[0]
    assert bad.size == 0, "%d of %d shadow answers differ" % (bad.size, occ.size)
    return int(occ.size)


@pytest.fixture(scope="module")
def box():
    sc = W.box_scene(0, 6)
    return sc, OR.prepare(sc)


def test_renderer_hit_ids_equal_intersect_bvh_full_frame(box):
    """The bench's frame itself: 512x512, 16 spp, bounces 0, 1, 2 (sorted
    streams) and 5 (a deep bounce)."""
    sc, prep = box
    caps = _trace(sc, 512, 512, 16, (0, 1, 2, 5))
    assert caps[0][0].shape[0] == 512 * 512 * 16
    total = 0
    for b, (closest, shadow) in caps.items():
        hits, n = _check_closest(prep, closest)
        total += n
        assert hits > 0.5 * n or b > 2
        _check_shadow(prep, shadow[:400_000])
    assert total > 8_000_000


@pytest.mark.parametrize("sort,wide,top", [(False, True, True), (True, False, True), (True, False, False),
                                           (False, False, False), (True, True, False)])
def test_renderer_hit_ids_in_every_traversal_mode(box, sort, wide, top):
    sc, prep = box
    caps = _trace(sc, 512, 512, 1, (0, 1, 2, 4), sort=sort, wide=wide, top=top, seed=3)
    for b, (closest, shadow) in caps.items():
        _check_closest(prep, closest)
        _check_shadow(prep, shadow)


def test_renderer_hit_ids_with_alpha_any_hit():
    """Alpha-blended triangles (10 % of the knot): the blend test draws from
    the path's key inside the traversal, on both sides."""
    sc = W.knot_scene(0, tubular=400, radial=40, env_width=256)
    prep = OR.prepare(sc)
    assert prep.packed.tri_alpha.mean() > 0.05
    caps = _trace(sc, 192, 108, 4, (0, 1, 3), max_bounces=12)
    for b, (closest, shadow) in caps.items():
        _check_closest(prep, closest, use_intersect_bvh=False)
        _check_shadow(prep, shadow)
