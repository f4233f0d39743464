"""Pins the oracle to the reference's own unit tests (CPU only).

Each test restates one assertion of the reference's Vitest suite on the
reference's exact inputs (same LCG, same generators) and checks that the C++
restatement gives the answer the reference's test demands.
"""
import math

import numpy as np
import pytest

import oracle
from lucent_gb300 import mesh
from refcases import LCG, bvh_vs_brute_rays, random_soup, torus_rays

NODE = 8


# ---------------------------------------------------------------- test/bvh.test.ts
def test_empty_soup():  # bvh.test.ts:31-35
    b = oracle.build_bvh(np.zeros(0, np.float32))
    assert b.node_count == 1
    ids, *_ = oracle.intersect_bvh(b, np.zeros(0, np.float32), np.array([[0, 0, 0, 0, 0, 1.0]]))
    assert ids[0] == -1


def test_single_leaf():  # bvh.test.ts:37-43
    b = oracle.build_bvh(np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32))
    assert b.node_count == 1
    assert b.nodes[7] == 1 and b.nodes[3] == 0


def _leaf_ranges(b):
    for n in range(b.node_count):
        cnt = int(b.nodes[n * NODE + 7])
        if cnt > 0:
            yield n, int(b.nodes[n * NODE + 3]), cnt


def test_every_triangle_once():  # bvh.test.ts:45-59
    soup = random_soup(500, LCG(7))
    b = oracle.build_bvh(soup)
    seen = np.zeros(500, np.int32)
    for _, first, cnt in _leaf_ranges(b):
        for i in range(cnt):
            t = b.tri_indices[first + i]
            assert seen[t] == 0
            seen[t] = 1
    assert seen.all()


def test_children_adjacent_bounds_nested():  # bvh.test.ts:61-76
    soup = random_soup(300, LCG(3))
    b = oracle.build_bvh(soup)
    nd = b.nodes.reshape(-1, 8)
    for n in range(b.node_count):
        if nd[n, 7] != 0:
            continue
        left = int(nd[n, 3])
        for c in (left, left + 1):
            assert (nd[c, 0:3] >= nd[n, 0:3] - 1e-6).all()
            assert (nd[c, 4:7] <= nd[n, 4:7] + 1e-6).all()


def test_coincident_centroids_terminate():  # bvh.test.ts:78-86
    soup = np.tile(np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32), 64)
    b = oracle.build_bvh(soup, max_leaf_size=4)
    assert b.node_count > 1
    ids, t, _, _ = oracle.intersect_bvh(b, soup, np.array([[0.2, 0.2, -1, 0, 0, 1.0]]))
    assert abs(t[0] - 1) < 0.5e-2  # toBeCloseTo(1)


def test_bvh_agrees_with_brute_force_soup():  # bvh.test.ts:90-110
    rand = LCG(42)
    soup = random_soup(2000, rand)
    b = oracle.build_bvh(soup)
    rays = bvh_vs_brute_rays(rand, 400)
    ia, ta, _, _ = oracle.intersect_bvh(b, soup, rays)
    ib, tb, _, _ = oracle.intersect_all(soup, rays)
    hits = ib >= 0
    assert hits.sum() > 50
    assert (ia[hits] >= 0).all()
    assert np.all(np.abs(ta[hits] - tb[hits]) < 0.5e-5)  # toBeCloseTo(b.t, 5)
    assert (ia[hits] == ib[hits]).all()
    assert (ia[~hits] == -1).all()


def test_bvh_agrees_with_brute_force_torus_knot():  # bvh.test.ts:112-124
    m = mesh.torus_knot(tubular_segments=80, radial_segments=10)
    assert mesh.triangle_count(m) == 1600
    b = oracle.build_bvh(m.positions)
    rays = torus_rays(LCG(99), 200)
    ia, ta, _, _ = oracle.intersect_bvh(b, m.positions, rays)
    ib, tb, _, _ = oracle.intersect_all(m.positions, rays)
    assert (ia == ib).all()
    assert np.array_equal(ta, tb)  # exact t equality (toBe)


def test_t_max_respected():  # bvh.test.ts:126-132
    soup = random_soup(100, LCG(5))
    b = oracle.build_bvh(soup)
    ray = np.array([[0, 0, -20, 0, 0, 1.0]])
    ib, tb, _, _ = oracle.intersect_all(soup, ray)
    if ib[0] < 0:
        pytest.skip("reference case has no hit")
    ia, *_ = oracle.intersect_bvh(b, soup, ray, 1e-5, tb[0] * 0.5)
    assert ia[0] == -1


def test_invalid_length_rejected():  # bvh.test.ts:55-57 (error path)
    with pytest.raises(oracle.OracleError):
        oracle.build_bvh(np.zeros(10, np.float32))


# ---------------------------------------------------------------- test/ray.test.ts
V0, V1, V2 = [-1, -1, 0], [1, -1, 0], [0, 1, 0]


def close(a, b, digits=2):
    return abs(a - b) < 0.5 * 10 ** -digits


def test_triangle_two_sided_barycentrics():  # ray.test.ts:9-20
    f = oracle.intersect_triangle([0, 0, -3], [0, 0, 1], V0, V1, V2)
    assert close(f[0], 3)
    bk = oracle.intersect_triangle([0, 0, 3], [0, 0, -1], V0, V1, V2)
    assert close(bk[0], 3)
    c = oracle.intersect_triangle([0, -1 / 3, -1], [0, 0, 1], V0, V1, V2)
    assert close(c[1], 1 / 3) and close(c[2], 1 / 3)


def test_triangle_misses():  # ray.test.ts:22-26
    assert oracle.intersect_triangle([2, 2, -1], [0, 0, 1], V0, V1, V2) is None
    assert oracle.intersect_triangle([0, 0, -1], [0, 0, -1], V0, V1, V2) is None
    assert oracle.intersect_triangle([0, 0, -3], [0, 0, 1], V0, V1, V2, 1e-5, 2) is None


def test_triangle_parallel():  # ray.test.ts:28-30
    assert oracle.intersect_triangle([0, 0, 0], [1, 0, 0], V0, V1, V2) is None


def test_sphere_roots():  # ray.test.ts:33-37
    assert close(oracle.intersect_sphere([0, 0, -5], [0, 0, 1], [0, 0, 0], 1), 4)
    assert close(oracle.intersect_sphere([0, 0, 0], [0, 0, 1], [0, 0, 0], 1), 1)
    assert oracle.intersect_sphere([0, 5, -5], [0, 0, 1], [0, 0, 0], 1) is None
    assert oracle.intersect_sphere([0, 0, 5], [0, 0, 1], [0, 0, 0], 1) is None


# ---------------------------------------------------------------- test/aabb.test.ts
def test_slab_known_answers():  # aabb.test.ts:21-33
    mn, mx = [-1, -1, -1], [1, 1, 1]

    def inv(d):
        return [1 / x if x != 0 else math.inf for x in d]

    assert close(oracle.aabb_intersect(mn, mx, [0, 0, -5], inv([0, 0, 1]), math.inf), 4)
    assert oracle.aabb_intersect(mn, mx, [0, 0, -5], inv([0, 0, -1]), math.inf) == math.inf
    assert oracle.aabb_intersect(mn, mx, [5, 5, -5], inv([0, 0, 1]), math.inf) == math.inf
    assert close(oracle.aabb_intersect(mn, mx, [0.5, 0.5, -5], inv([0, 0, 1]), math.inf), 4)
    assert oracle.aabb_intersect(mn, mx, [0, 0, -5], inv([0, 0, 1]), 2) == math.inf
    assert oracle.aabb_intersect(mn, mx, [0, 0, 0], inv([1, 0, 0]), math.inf) == 0


# ---------------------------------------------------------------- test/environment.test.ts
def test_alias_reproduces_distribution():  # environment.test.ts:16-29
    w = [1, 0, 3, 6, 0.5, 9.5]
    prob, alias, pmf, total = oracle.build_alias(w)
    n = len(w)
    p = np.zeros(n)
    for j in range(n):
        p[j] += prob[j] / n
        p[alias[j]] += (1 - prob[j]) / n
    assert np.all(np.abs(p - np.array(w) / sum(w)) < 0.5e-6)
    assert total == sum(w)


def test_alias_never_draws_zero_weight():  # environment.test.ts:31-35
    prob, alias, _, _ = oracle.build_alias([0, 5, 0, 1])
    rand = LCG(7)
    for _ in range(2000):
        u0, u1 = rand(), rand()
        i = min(3, math.floor(u0 * 4))  # sampleAlias, src/math/alias.ts:68-72
        k = i if u1 < prob[i] else alias[i]
        assert k in (1, 3)


def test_alias_uniform_fallback_and_errors():  # environment.test.ts:37-44
    _, _, pmf, total = oracle.build_alias([0, 0, 0, 0])
    assert list(pmf) == [0.25] * 4 and total == 0
    for bad in ([1, -1], [1, float("nan")], []):
        with pytest.raises(oracle.OracleError):
            oracle.build_alias(bad)


def test_env_pdf_integrates_to_one():  # environment.test.ts:112-136
    width, height = 64, 32
    data = np.full(width * height * 3, 0.1, np.float32)
    bright = (10 * width + 40) * 3
    data[bright:bright + 3] = 500
    gw, gh, table, _ = oracle.build_env_sampler(data, width, height, 32)
    assert (gw, gh) == (32, 16)
    t = table.reshape(-1, 4)
    integral = (t[:, 2].astype(np.float64) / (gw * gh)).sum()
    assert abs(integral - 1) < 0.5e-6
    assert int(np.argmax(t[:, 2])) == 5 * 32 + 20
    for i in range(20):
        a = int(t[i, 1])
        assert abs(t[i, 3] - t[a, 2]) < 0.5e-6


def test_sheen_lut_range_and_monotone():  # environment.test.ts:150-158
    lut = oracle.sheen_lut(8, 48)
    assert (lut >= 0).all() and (lut <= 1).all()
    assert oracle.sheen_albedo(0.7, 1, 96) > oracle.sheen_albedo(0.7, 0.2, 96)


def test_sheen_matches_monte_carlo():  # environment.test.ts:160-183
    cos_v, r = 0.5, 0.6
    alpha = r * r
    v = [math.sqrt(1 - cos_v * cos_v), 0, cos_v]
    rand = LCG(11)
    s = 0.0
    n = 200000
    inv = 1 / alpha
    for _ in range(n):
        z = rand()
        phi = 2 * math.pi * rand()
        sn = math.sqrt(1 - z * z)
        lx, ly = sn * math.cos(phi), sn * math.sin(phi)
        hx, hy, hz = lx + v[0], ly + v[1], z + v[2]
        ln = math.hypot(hx, hy, hz)
        ch = hz / ln
        d = (2 + inv) * max(0.0, 1 - ch * ch) ** (inv / 2) / (2 * math.pi)
        s += d * (1 / (4 * (z + cos_v - z * cos_v))) * z
    assert abs(oracle.sheen_albedo(cos_v, r, 256) - 2 * math.pi * s / n) < 0.5e-2


# ---------------------------------------------------------------- test/mesh.test.ts
def _closed(pos):
    key = lambda i: "%.5f,%.5f,%.5f" % (pos[i], pos[i + 1], pos[i + 2])
    edges = {}
    for t in range(0, pos.size, 9):
        v = [key(t), key(t + 3), key(t + 6)]
        for e in range(3):
            k = (v[e], v[(e + 1) % 3])
            edges[k] = edges.get(k, 0) + 1
    return all(n == 1 and edges.get((b, a)) == 1 for (a, b), n in edges.items())


def test_mesh_generators():  # mesh.test.ts:24-80
    q = mesh.quad([0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0])
    assert mesh.triangle_count(q) == 2 and list(q.normals[:3]) == [0, 0, 1]
    b = mesh.box([-1, -1, -1], [1, 1, 1])
    assert mesh.triangle_count(b) == 12 and _closed(b.positions)
    for t in range(0, b.positions.size, 9):
        assert np.dot(b.normals[t:t + 3], b.positions[t:t + 3]) > 0
    k = mesh.torus_knot(tubular_segments=40, radial_segments=8)
    assert mesh.triangle_count(k) == 640 and _closed(k.positions)
    assert np.all(np.abs(np.linalg.norm(k.normals.reshape(-1, 3), axis=1) - 1) < 0.5e-4)
    t = mesh.transform(q, scale=2, rotate_y=math.pi / 2, translate=[5, 0, 0])
    assert close(t.positions[3], 5) and close(t.positions[4], 0) and close(t.positions[5], -2)
    assert close(t.normals[0], 1) and close(t.normals[2], 0)
    ico = mesh.icosphere(2)
    assert mesh.triangle_count(ico) == 320 and _closed(ico.positions)
