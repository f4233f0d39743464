"""The four-wide view of the BVH (lucent_gb300/csrc/traverse_wide.cuh) on the
CPU: its records restated in numpy, and a binary64 closest-hit traversal over
them that tests only the records (a node's grandchildren, never its inner
children) must give intersectBVH's hits on the reference test's own inputs
(test/bvh.test.ts soup and torus cases). This checks the argument the wide
kernels rest on, that skipping the inner children's box tests changes no
decision, with the reference's own binary64 tests (the oracle's
aabb_intersect and intersect_triangle)."""
import math

import numpy as np

import oracle
from lucent_gb300 import mesh
from refcases import LCG, bvh_vs_brute_rays, random_soup, torus_rays


def wide_view(nodes, node_count):
    """[node_count, 4] records (min, first, max, count) as the GPU builds them:
    node n's grandchildren in visiting order, a leaf child in place of its
    absent children; an inner record's `first` is its own index; count -1:
    unused."""
    nd = np.asarray(nodes, np.float64).reshape(-1, 8)[:node_count]
    empty = np.array([np.inf] * 3 + [0.0] + [-np.inf] * 3 + [-1.0])
    out = np.tile(empty, (node_count, 4, 1))

    def rec(c):
        r = nd[c].copy()
        if r[7] == 0:
            r[3] = c
        return r

    for n in range(node_count):
        if nd[n, 7] > 0:
            continue
        f = int(nd[n, 3])
        k = 0
        for c in (f, f + 1):
            if nd[c, 7] > 0:
                out[n, k] = nd[c]
                k += 1
            else:
                g = int(nd[c, 3])
                out[n, k], out[n, k + 1] = rec(g), rec(g + 1)
                k += 2
    return out


def closest_wide(nodes, node_count, wide, tri_indices, positions, o, d, t_min=1e-5, t_max=math.inf):
    """Closest hit over the wide view: each record's box tested when the
    reference would pop it (the first passing record of an expansion at once,
    the others when popped), triangles in leaf order."""
    inv = np.array([1.0 / x if x != 0 else math.copysign(math.inf, x) for x in d])
    pos = np.asarray(positions, np.float64).reshape(-1, 9)
    closest, best = t_max, -1

    def visit(r):
        nonlocal closest, best
        if oracle.aabb_intersect(r[0:3], r[4:7], o, inv, closest) == math.inf:
            return None
        if r[7] > 0:
            first = int(r[3])
            for i in range(int(r[7])):
                tri = int(tri_indices[first + i])
                p = pos[tri]
                h = oracle.intersect_triangle(o, d, p[0:3], p[3:6], p[6:9], t_min, closest)
                if h is not None:
                    closest, best = h[0], tri
            return None
        return int(r[3])  # an inner record that passed: expand it

    root = np.asarray(nodes, np.float64).reshape(-1, 8)[0].copy()
    if root[7] == 0:
        root[3] = 0
    stack = [root]
    while stack:
        n = visit(stack.pop())
        if n is not None:
            stack.extend(wide[n][::-1][wide[n][::-1, 7] >= 0])  # first record on top
    return best, closest


def _check(positions, rays):
    ob = oracle.build_bvh(positions)
    wide = wide_view(ob.nodes, ob.node_count)
    ids, t, _, _ = oracle.intersect_bvh(ob, positions, rays)
    for k, ray in enumerate(np.asarray(rays, np.float64)):
        best, tc = closest_wide(ob.nodes, ob.node_count, wide, ob.tri_indices, positions, ray[:3], ray[3:])
        assert best == ids[k], (k, best, ids[k])
        if best >= 0:
            assert tc == t[k]


def test_wide_view_records():
    m = mesh.torus_knot(tubular_segments=40, radial_segments=8)
    ob = oracle.build_bvh(m.positions)
    nd = np.asarray(ob.nodes, np.float64).reshape(-1, 8)[:ob.node_count]
    wide = wide_view(ob.nodes, ob.node_count)
    for n in range(ob.node_count):
        used = wide[n][wide[n][:, 7] >= 0]
        if nd[n, 7] > 0:
            assert used.size == 0
            continue
        assert 2 <= len(used) <= 4
        for r in used:  # every record lies inside its node's box (the nesting the wide kernels rely on)
            assert np.all(r[0:3] >= nd[n, 0:3]) and np.all(r[4:7] <= nd[n, 4:7])


def test_wide_traversal_matches_intersect_bvh_on_the_soup():  # test/bvh.test.ts:90-110 inputs
    rand = LCG(42)
    soup = random_soup(2000, rand)
    _check(soup, bvh_vs_brute_rays(rand, 120))


def test_wide_traversal_matches_intersect_bvh_on_the_torus():  # test/bvh.test.ts:112-124 inputs
    m = mesh.torus_knot(tubular_segments=80, radial_segments=10)
    _check(m.positions, torus_rays(LCG(99), 120))
