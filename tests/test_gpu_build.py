"""GPU BVH builder parity: node array, node count, triIndices and bounds equal
the oracle's restatement of buildBVH (src/math/bvh.ts:52-252) on the same
input. Node bounds compare as numbers (the sign of a zero is not pinned)."""
import math

import numpy as np
import pytest

import oracle
from lucent_gb300 import bvh as B
from lucent_gb300 import mesh, workloads
from refcases import LCG, random_soup

pytestmark = pytest.mark.gpu


def _check(pos, max_leaf=4, bins=12):
    ob = oracle.build_bvh(pos, max_leaf, bins)
    gb = B.build_bvh(pos, max_leaf, bins)
    assert gb.node_count == ob.node_count
    assert np.array_equal(gb.tri_indices, ob.tri_indices)
    assert np.array_equal(gb.nodes, ob.nodes)  # numeric equality (+0 == -0)
    assert np.array_equal(np.array(gb.bounds.min + gb.bounds.max), ob.bounds)
    # The device copy answers rays exactly like the oracle over its own BVH.
    return ob, gb


def test_reference_unit_cases():  # bvh.test.ts:31-86 inputs
    _check(np.zeros(0, np.float32))
    _check(np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32))
    _check(random_soup(500, LCG(7)))
    _check(random_soup(300, LCG(3)))
    _check(random_soup(2000, LCG(42)))
    _check(np.tile(np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32), 64))


def test_options():
    soup = random_soup(3000, LCG(11))
    for ml, bins in ((1, 12), (2, 4), (8, 16), (4, 32), (16, 2)):
        _check(soup, ml, bins)


def test_meshes_with_ties_and_flat_boxes():
    _check(mesh.torus_knot(tubular_segments=80, radial_segments=10).positions)
    _check(mesh.icosphere(4).positions)
    boxes = mesh.merge_meshes([mesh.box([-1, -1, -1], [1, 1, 1], inward=True)] +
                              [mesh.box([i, 0, j], [i + 0.5, 0.5, j + 0.5]) for i in range(8) for j in range(8)])
    _check(boxes.positions)
    # many identical triangles mixed with distinct ones: equal centroids everywhere
    grid = np.tile(np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32), 3000)
    _check(np.concatenate([grid, random_soup(2000, LCG(4))]))


def test_big_nodes_pipeline():
    # > 2048 triangles exercises the chunked big-node levels; > 4096 makes
    # multi-chunk tasks; the soup crosses several levels.
    pos, _ = workloads.soup_and_rays(seed=0, n_tri=65536, n_rays=1)
    ob, gb = _check(pos)
    assert oracle.bvh_depth(ob) < 64


def test_large_displaced_knot():
    m = mesh.displace(mesh.torus_knot(tubular_segments=1500, radial_segments=100), 0.05, 3, seed=1)
    _check(m.positions)


def test_config3_knot_two_million():
    """Config 3's mesh: the torus knot tessellated to 2,000,000 triangles with
    3-octave value-noise displacement (amplitude 0.05), node array and
    triIndices equal to the oracle's buildBVH."""
    from lucent_gb300 import workloads as W
    pos = W.knot_mesh(0).positions
    assert pos.size == 9 * 2_000_000
    _check(pos)


def test_largest_batch_scene():
    """The largest scene of the batched workload (config 5), built on the GPU
    exactly as the batch loads it, against the oracle's buildBVH."""
    from lucent_gb300 import workloads as W
    sizes = W.batch_sizes()
    big = int(np.argmax(sizes))
    sc, _ = W.batch_scene(big)
    from lucent_gb300 import scene as S
    p = S.pack_scene(sc)
    assert p.tri_count == sizes[big] > 1_000_000
    _check(p.positions)


def test_built_handle_intersects_like_oracle():
    pos, rays = workloads.soup_and_rays(seed=2, n_tri=20000, n_rays=50000)
    gb = B.build_bvh(pos)
    prim, t, _, _ = gb._device.intersect(rays)
    ob = oracle.build_bvh(pos)
    ids, to, _, _ = oracle.intersect_bvh(ob, pos, rays)
    assert np.array_equal(prim, ids)
    nodes, tri = B.download(gb._device)
    assert np.array_equal(nodes, ob.nodes) and np.array_equal(tri, ob.tri_indices)


def test_build_from_device_positions():
    torch = pytest.importorskip("torch")
    pos, _ = workloads.soup_and_rays(seed=5, n_tri=30000, n_rays=1)
    d = torch.from_numpy(pos).cuda()
    dev = B.build_device(d.data_ptr(), pos.size // 9)
    nodes, tri = B.download(dev)
    ob = oracle.build_bvh(pos)
    assert np.array_equal(nodes, ob.nodes) and np.array_equal(tri, ob.tri_indices)


def test_invalid_inputs():
    from lucent_gb300 import LucentError
    with pytest.raises(ValueError):
        B.build_bvh(np.zeros(10, np.float32))
    bad = random_soup(10, LCG(1))
    bad[4] = math.nan
    with pytest.raises(LucentError):
        B.build_bvh(bad)
    with pytest.raises(LucentError):
        B.build_bvh(random_soup(10, LCG(1)), bins=64)
