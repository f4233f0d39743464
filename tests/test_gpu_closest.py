"""GPU closest-hit parity: hit ids equal the oracle's restatement of the
reference's intersectBVH (src/math/bvh.ts:265-320) bit for bit; t, u, v equal
the oracle's binary64 values rounded to binary32 (0 ulp; the bar is 2 ulp)."""
import math

import numpy as np
import pytest

import oracle
from lucent_gb300 import DeviceBVH, mesh, workloads
from lucent_gb300.bvh import BVH, AABB, intersect_bvh
from refcases import LCG, bvh_vs_brute_rays, random_soup, torus_rays

pytestmark = pytest.mark.gpu


def _compare(dev, ob, pos, rays32, t_min=1e-5, t_max=math.inf):
    ids_o, t_o, u_o, v_o = oracle.intersect_bvh(ob, pos, rays32, t_min, t_max)
    # binary32 path with and without the shared-memory top levels, over the
    # four-wide view, then all binary64
    for exact, top, wide in ((False, True, False), (False, False, False), (False, False, True), (True, True, False)):
        dev.set_mode(exact, top_levels=top, wide=wide)
        prim, t, u, v = dev.intersect(rays32, t_min, t_max)
        bad = np.nonzero(prim != ids_o)[0]
        assert bad.size == 0, "exact=%s top=%s wide=%s: %d id mismatches, first ray %d: gpu %d oracle %d" % (
            exact, top, wide, bad.size, bad[:1], prim[bad[:1]], ids_o[bad[:1]])
        hit = ids_o >= 0
        assert np.array_equal(t[hit], t_o[hit].astype(np.float32))
        assert np.array_equal(u[hit], u_o[hit].astype(np.float32))
        assert np.array_equal(v[hit], v_o[hit].astype(np.float32))
        assert np.all(np.isinf(t[~hit]))
    dev.set_mode(False)  # the default: four-wide
    return ids_o


def _dev(pos):
    ob = oracle.build_bvh(pos)
    return ob, DeviceBVH(ob.nodes, ob.tri_indices, pos, ob.node_count)


def test_reference_soup_case():  # test/bvh.test.ts:90-110 inputs
    rand = LCG(42)
    soup = random_soup(2000, rand)
    ob, dev = _dev(soup)
    rays = bvh_vs_brute_rays(rand, 400)
    prim, t, u, v = dev.intersect_f64(rays)
    ids, to, uo, vo = oracle.intersect_bvh(ob, soup, rays)
    assert np.array_equal(prim, ids)
    hit = ids >= 0
    assert np.array_equal(t[hit], to[hit]) and np.array_equal(u[hit], uo[hit]) and np.array_equal(v[hit], vo[hit])
    _compare(dev, ob, soup, rays.astype(np.float32))


def test_reference_torus_case():  # test/bvh.test.ts:112-124 inputs
    m = mesh.torus_knot(tubular_segments=80, radial_segments=10)
    ob, dev = _dev(m.positions)
    rays = torus_rays(LCG(99), 200)
    prim, t, _, _ = dev.intersect_f64(rays)
    ids, to, _, _ = oracle.intersect_bvh(ob, m.positions, rays)
    assert np.array_equal(prim, ids) and np.array_equal(t[ids >= 0], to[ids >= 0])


def test_random_soup_subset():
    pos, rays = workloads.soup_and_rays(seed=0, n_tri=65536, n_rays=200_000)
    ob, dev = _dev(pos)
    ids = _compare(dev, ob, pos, rays)
    assert (ids >= 0).mean() > 0.3


def test_config1_all_rays():
    """Config 1 whole: 65,536-triangle soup, all 10^6 rays of seed 0, tMin
    1e-5, tMax inf, against the oracle's intersectBVH (ids, t, u, v)."""
    pos, rays = workloads.soup_and_rays(seed=0, n_tri=65536, n_rays=1_000_000)
    ob, dev = _dev(pos)
    ids = _compare(dev, ob, pos, rays)
    assert ids.size == 1_000_000 and (ids >= 0).mean() > 0.3


def test_adversarial_rays_mesh():
    m = mesh.merge_meshes([mesh.torus_knot(tubular_segments=120, radial_segments=16),
                           mesh.box([-2, -2, -2], [2, 2, 2], inward=True),
                           mesh.transform(mesh.box([-0.5, -0.5, -0.5], [0.5, 0.5, 0.5]), rotate_y=0.3)])
    ob, dev = _dev(m.positions)
    rng = np.random.Generator(np.random.PCG64(5))
    rays = workloads.adversarial_rays(m.positions, rng, 1500)
    for t_min, t_max in ((1e-5, math.inf), (0.0, math.inf), (1e-6, 2.5), (0.5, 3.0)):
        _compare(dev, ob, m.positions, rays, t_min, t_max)


def test_adversarial_rays_soup():
    pos, _ = workloads.soup_and_rays(seed=3, n_tri=4096, n_rays=1)
    ob, dev = _dev(pos)
    rays = workloads.adversarial_rays(pos, np.random.Generator(np.random.PCG64(9)), 2000)
    _compare(dev, ob, pos, rays)


def test_coincident_and_duplicate_triangles():  # bvh.test.ts:78-86 plus exact ties
    one = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32)
    soup = np.tile(one, 64)
    ob, dev = _dev(soup)
    rays = np.array([[0.2, 0.2, -1, 0, 0, 1], [0.25, 0.25, 1, 0, 0, -1], [0.5, 0.5, -1, 0, 0, 1],
                     [0.1, 0.1, -1, 0.01, 0.02, 1]], np.float32)
    ids = _compare(dev, ob, soup, rays)
    assert ids[0] >= 0


def test_coplanar_ties_and_flat_leaves():
    # Boxes standing on a floor (bottom faces in the floor's plane), a second
    # triangulation of the floor (the other diagonal) and a few coplanar
    # overlapping quads: rays from above and below meet two or more triangles
    # at one distance, and flat leaf boxes whose entry equals the running
    # closest. The kernels defer such ties and visit such leaves
    # conditionally; the hits must still be the reference's.
    floor_a = mesh.quad((-2, 0, 2), (2, 0, 2), (2, 0, -2), (-2, 0, -2))
    floor_b = mesh.quad((2, 0, 2), (2, 0, -2), (-2, 0, -2), (-2, 0, 2))
    parts = [floor_a, floor_b,
             mesh.transform(mesh.box((-0.3, 0.0, -0.3), (0.3, 1.2, 0.3)), translate=(-0.4, 0.0, -0.35), rotate_y=0.4),
             mesh.transform(mesh.box((-0.3, 0.0, -0.3), (0.3, 0.6, 0.3)), translate=(0.45, 0.0, 0.3), rotate_y=1.1),
             mesh.quad((-1, 0.6, 1), (1, 0.6, 1), (1, 0.6, -1), (-1, 0.6, -1)),
             mesh.quad((-0.5, 0.6, 0.5), (0.5, 0.6, 0.5), (0.5, 0.6, -0.5), (-0.5, 0.6, -0.5))]
    m = mesh.merge_meshes(parts)
    ob, dev = _dev(m.positions)
    rng = np.random.Generator(np.random.PCG64(11))
    n = 4000
    o = np.concatenate([rng.uniform(-2, 2, (n, 1)), rng.uniform(0.7, 3.0, (n, 1)), rng.uniform(-2, 2, (n, 1))], 1)
    d = np.concatenate([rng.normal(size=(n, 1)) * 0.5, -np.ones((n, 1)), rng.normal(size=(n, 1)) * 0.5], 1)
    below = o * np.array([1, -1, 1]) + np.array([0, 0.3, 0])
    up = d * np.array([1, -1, 1])
    rays = np.concatenate([np.concatenate([o, d], 1), np.concatenate([below, up], 1)]).astype(np.float64)
    rays[:, 3:] /= np.linalg.norm(rays[:, 3:], axis=1, keepdims=True)
    rays = np.concatenate([rays, workloads.adversarial_rays(m.positions, rng, 800)]).astype(np.float32)
    hits = [(_compare(dev, ob, m.positions, rays, t_min, t_max) >= 0).mean()
            for t_min, t_max in ((1e-6, 1e30), (1e-5, math.inf), (0.0, 2.0))]
    assert hits[0] > 0.5 and hits[2] > 0.2, hits


def test_empty_and_single():
    ob = oracle.build_bvh(np.zeros(0, np.float32))
    dev = DeviceBVH(ob.nodes, ob.tri_indices, np.zeros(0, np.float32), ob.node_count)
    prim, t, _, _ = dev.intersect(np.array([[0, 0, 0, 0, 0, 1]], np.float32))
    assert prim[0] == -1 and np.isinf(t[0])
    tri = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32)
    ob, dev = _dev(tri)
    _compare(dev, ob, tri, np.array([[0.2, 0.2, -1, 0, 0, 1], [2, 2, -1, 0, 0, 1]], np.float32))


def test_pick_api_mirrors_reference():
    soup = random_soup(300, LCG(3))
    ob = oracle.build_bvh(soup)
    bvh = BVH(ob.nodes, ob.node_count, ob.tri_indices, AABB(ob.bounds[:3], ob.bounds[3:]))
    ray = {"origin": [0.0, 0.0, -20.0], "dir": [0.0, 0.0, 1.0]}
    h = intersect_bvh(bvh, soup, ray)
    ids, t, u, v = oracle.intersect_bvh(ob, soup, np.array([[0, 0, -20, 0, 0, 1.0]]))
    if ids[0] < 0:
        assert h is None
    else:
        assert (h.tri_index, h.t, h.u, h.v) == (ids[0], t[0], u[0], v[0])


def test_invalid_bvh_rejected():
    from lucent_gb300 import LucentError
    ob = oracle.build_bvh(random_soup(50, LCG(1)))
    bad = ob.nodes.copy()
    bad[3] = 1e6  # root's children far outside the node array
    with pytest.raises(LucentError):
        DeviceBVH(bad, ob.tri_indices, random_soup(50, LCG(1)), ob.node_count)
