"""Oracle: CPU restatement of the reference's BVH / ray / lighting arithmetic.

TEST INFRASTRUCTURE ONLY. Imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU-baseline leg, and only as the checker; the product package
`lucent_gb300` never imports it.

The C++ sources (lucent_oracle.cpp, oracle_render.cpp) restate the reference
file:line by file:line; this module is a thin numpy/ctypes wrapper.
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        _lib = C.CDLL(path)
        _declare(_lib)
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


_F, _D, _U32, _I32 = C.c_float, C.c_double, C.c_uint32, C.c_int32


def _declare(L):
    P = C.POINTER
    L.orc_build_bvh.argtypes = [P(_F), C.c_uint64, C.c_int, C.c_int, P(_F), P(_U32), P(_U32), P(_D)]
    L.orc_bvh_depth.argtypes = [P(_F), _U32]
    L.orc_intersect_bvh.argtypes = [P(_F), _U32, P(_U32), _U32, P(_F), P(_D), C.c_uint64, _D, _D,
                                    P(_I32), P(_D), P(_D), P(_D), C.c_int]
    L.orc_intersect_bvh_f32.argtypes = [P(_F), _U32, P(_U32), _U32, P(_F), P(_F), C.c_uint64, _D, _D,
                                        P(_I32), P(_D), P(_D), P(_D), C.c_int]
    L.orc_intersect_all.argtypes = [P(_F), _U32, P(_D), C.c_uint64, _D, _D, P(_I32), P(_D), P(_D), P(_D),
                                    C.c_int]
    L.orc_intersect_triangle.argtypes = [P(_D)] * 5 + [_D, _D, P(_D), P(_D), P(_D)]
    L.orc_intersect_sphere.argtypes = [P(_D), P(_D), P(_D), _D, _D, _D, P(_D)]
    L.orc_aabb_intersect.argtypes = [P(_D), P(_D), P(_D), P(_D), _D]
    L.orc_aabb_intersect.restype = _D
    L.orc_glsl_traversal_counts.argtypes = [P(_F), _U32, P(_F), _U32, P(_F), C.c_uint64, _F, P(_U32),
                                            P(_U32), P(_I32), C.c_int]
    L.orc_ts_traversal_counts.argtypes = [P(_F), P(_U32), _U32, P(_F), P(_F), C.c_uint64, _D, _D, P(_U32),
                                          P(_U32), C.c_int]
    L.orc_build_alias.argtypes = [P(_D), _U32, P(_F), P(_U32), P(_D), P(_D)]
    L.orc_build_env_sampler.argtypes = [P(_F), _U32, _U32, _U32, P(_U32), P(_U32), P(_F), P(_D)]
    L.orc_sheen_albedo.argtypes = [_D, _D, C.c_int]
    L.orc_sheen_albedo.restype = _D
    L.orc_sheen_lut.argtypes = [C.c_int, C.c_int, P(_F)]
    L.orc_bake_sky.argtypes = [_U32, P(_D), P(_D), P(_D), _D, C.c_int, _D, _D, P(_D), _D, _D, P(_F)]
    L.orc_bake_sky.restype = None
    try:
        from . import render as _render
        _render.declare(L)
    except ImportError:
        pass


class OracleError(RuntimeError):
    pass


class BVH:
    """Mirror of the reference's BVH interface (src/math/bvh.ts:18-24)."""

    def __init__(self, nodes, node_count, tri_indices, bounds):
        self.nodes = nodes
        self.node_count = node_count
        self.tri_indices = tri_indices
        self.bounds = bounds


def build_bvh(positions, max_leaf_size=4, bins=12):
    """buildBVH (src/math/bvh.ts:52). positions: float32 flat (9 per triangle)."""
    pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1)
    if pos.size % 9:
        raise OracleError("positions length %d is not a multiple of 9" % pos.size)
    n = pos.size // 9
    nodes = np.zeros(max(1, 2 * n - 1) * 8, np.float32)
    tri = np.zeros(max(n, 1), np.uint32)
    cnt = _U32(0)
    bounds = np.zeros(6, np.float64)
    st = lib().orc_build_bvh(_p(pos, _F), pos.size, max_leaf_size, bins, _p(nodes, _F), C.byref(cnt),
                             _p(tri, _U32), _p(bounds, _D))
    if st:
        raise OracleError("orc_build_bvh failed: %d" % st)
    return BVH(nodes[: cnt.value * 8].copy(), cnt.value, tri[:n].copy(), bounds)


def bvh_depth(bvh):
    return lib().orc_bvh_depth(_p(bvh.nodes, _F), bvh.node_count)


def _rays64(rays):
    return np.ascontiguousarray(rays, dtype=np.float64).reshape(-1, 6)


def intersect_bvh(bvh, positions, rays, t_min=1e-5, t_max=np.inf, threads=0):
    """intersectBVH (src/math/bvh.ts:265) over many rays; rays float64 or float32 [n,6].

    Returns (ids int32 with -1 on a miss, t, u, v) as float64 arrays.
    """
    pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1)
    n_tri = bvh.tri_indices.size
    f32 = np.asarray(rays).dtype == np.float32
    r = np.ascontiguousarray(rays, dtype=np.float32 if f32 else np.float64).reshape(-1, 6)
    n = r.shape[0]
    ids = np.empty(n, np.int32)
    t, u, v = (np.empty(n, np.float64) for _ in range(3))
    args = (_p(bvh.nodes, _F), bvh.node_count, _p(np.ascontiguousarray(bvh.tri_indices, np.uint32), _U32), n_tri,
            _p(pos, _F))
    if f32:
        st = lib().orc_intersect_bvh_f32(*args, _p(r, _F), n, t_min, t_max, _p(ids, _I32), _p(t, _D), _p(u, _D),
                                         _p(v, _D), threads)
    else:
        st = lib().orc_intersect_bvh(*args, _p(r, _D), n, t_min, t_max, _p(ids, _I32), _p(t, _D), _p(u, _D),
                                     _p(v, _D), threads)
    if st:
        raise OracleError("orc_intersect_bvh failed: %d" % st)
    return ids, t, u, v


def intersect_all(positions, rays, t_min=1e-5, t_max=np.inf, threads=0):
    """intersectAllTriangles (src/math/bvh.ts:323), brute force."""
    pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1)
    r = _rays64(rays)
    n = r.shape[0]
    ids = np.empty(n, np.int32)
    t, u, v = (np.empty(n, np.float64) for _ in range(3))
    lib().orc_intersect_all(_p(pos, _F), pos.size // 9, _p(r, _D), n, t_min, t_max, _p(ids, _I32), _p(t, _D),
                            _p(u, _D), _p(v, _D), threads)
    return ids, t, u, v


def intersect_triangle(origin, direction, v0, v1, v2, t_min=1e-5, t_max=np.inf):
    """intersectTriangle (src/math/ray.ts:22). Returns (t, u, v) or None."""
    a = [np.ascontiguousarray(x, np.float64) for x in (origin, direction, v0, v1, v2)]
    t, u, v = _D(), _D(), _D()
    if lib().orc_intersect_triangle(*[_p(x, _D) for x in a], t_min, t_max, C.byref(t), C.byref(u), C.byref(v)):
        return t.value, u.value, v.value
    return None


def intersect_sphere(origin, direction, center, radius, t_min=1e-5, t_max=np.inf):
    """intersectSphere (src/math/ray.ts:48)."""
    a = [np.ascontiguousarray(x, np.float64) for x in (origin, direction, center)]
    t = _D()
    if lib().orc_intersect_sphere(*[_p(x, _D) for x in a], radius, t_min, t_max, C.byref(t)):
        return t.value
    return None


def aabb_intersect(bmin, bmax, origin, inv_dir, t_max):
    """AABB.intersect (src/math/aabb.ts:84)."""
    a = [np.ascontiguousarray(x, np.float64) for x in (bmin, bmax, origin, inv_dir)]
    return lib().orc_aabb_intersect(*[_p(x, _D) for x in a], t_max)


def glsl_traversal_counts(nodes, node_count, geo, rays, t_min=1e-6, threads=0):
    """Inner nodes visited / triangles tested per ray in the GLSL traversal order."""
    r = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
    n = r.shape[0]
    inner = np.empty(n, np.uint32)
    tris = np.empty(n, np.uint32)
    slot = np.empty(n, np.int32)
    g = np.ascontiguousarray(geo, np.float32)
    lib().orc_glsl_traversal_counts(_p(np.ascontiguousarray(nodes, np.float32), _F), node_count, _p(g, _F),
                                    g.size // 12, _p(r, _F), n, t_min, _p(inner, _U32), _p(tris, _U32),
                                    _p(slot, _I32), threads)
    return inner, tris, slot


def ts_traversal_counts(bvh, positions, rays, t_min=1e-5, t_max=np.inf, threads=0):
    """Nodes popped / triangles tested per ray in intersectBVH's left-first order."""
    r = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
    n = r.shape[0]
    popped = np.empty(n, np.uint32)
    tests = np.empty(n, np.uint32)
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1)
    lib().orc_ts_traversal_counts(_p(bvh.nodes, _F), _p(np.ascontiguousarray(bvh.tri_indices, np.uint32), _U32),
                                  bvh.tri_indices.size, _p(pos, _F), _p(r, _F), n, t_min, t_max,
                                  _p(popped, _U32), _p(tests, _U32), threads)
    return popped, tests


def leaf_order_geometry(bvh, positions):
    """Triangles gathered into slot order, 12 floats each (the GLSL geo layout)."""
    tri = np.asarray(positions, np.float32).reshape(-1, 3, 3)[bvh.tri_indices]
    g = np.zeros((tri.shape[0], 3, 4), np.float32)
    g[:, :, :3] = tri
    return g.reshape(-1)


def build_alias(weights):
    """buildAliasTable (src/math/alias.ts:17) -> (prob f32, alias u32, pmf f64, total)."""
    w = np.ascontiguousarray(weights, np.float64)
    n = w.size
    prob = np.zeros(max(n, 1), np.float32)
    alias = np.zeros(max(n, 1), np.uint32)
    pmf = np.zeros(max(n, 1), np.float64)
    total = _D()
    if lib().orc_build_alias(_p(w, _D), n, _p(prob, _F), _p(alias, _U32), _p(pmf, _D), C.byref(total)):
        raise OracleError("alias table needs at least one finite weight >= 0")
    return prob[:n], alias[:n], pmf[:n], total.value


def build_env_sampler(rgb, width, height, max_width=1024):
    """buildEnvSampler (src/scene/environment.ts:52) -> (gw, gh, table f32[gw*gh*4], total)."""
    img = np.ascontiguousarray(rgb, np.float32).reshape(-1)
    gw = min(width, max_width)
    table = np.zeros(gw * height * 4 + 4, np.float32)
    a, b = _U32(), _U32()
    total = _D()
    if lib().orc_build_env_sampler(_p(img, _F), width, height, max_width, C.byref(a), C.byref(b), _p(table, _F),
                                   C.byref(total)):
        raise OracleError("env sampler failed")
    return a.value, b.value, table[: a.value * b.value * 4].copy(), total.value


def bake_sky(sky, sun, width=1024):
    """bakeSky (src/scene/environment.ts:106-132) -> float32 [width/2, width, 3]."""
    out = np.zeros(width * (width // 2) * 3, np.float32)
    z, h, g, c = (np.ascontiguousarray(v, np.float64) for v in (sky.zenith, sky.horizon, sky.ground, sun.color))
    lib().orc_bake_sky(width, _p(z, _D), _p(h, _D), _p(g, _D), float(sky.intensity), 1 if sky.enabled else 0,
                       float(sun.elevation), float(sun.azimuth), _p(c, _D), float(sun.intensity),
                       float(sun.angular_radius), _p(out, _F))
    return out.reshape(width // 2, width, 3)


def sheen_albedo(cos_v, roughness, steps=128):
    return lib().orc_sheen_albedo(cos_v, roughness, steps)


def sheen_lut(size=16, steps=96):
    out = np.zeros(size * size, np.float32)
    lib().orc_sheen_lut(size, steps, _p(out, _F))
    return out
