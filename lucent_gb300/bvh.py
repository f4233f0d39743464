"""BVH API mirroring the reference's src/math/bvh.ts on the GB300.

`build_bvh` / `build_bvh_async` (bvh.ts:52, bvh-async.ts:8) build on the GPU
and return the reference's BVH layout; `intersect_bvh` (bvh.ts:265) answers
one ray like the reference's CPU intersector; `DeviceBVH` is the device-
resident form that answers millions of rays per call.
"""
import ctypes as C
import math
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _native as N

NODE_STRIDE = 8  # bvh.ts:16


@dataclass
class BVHHit:
    """bvh.ts:254-259."""
    t: float
    tri_index: int
    u: float
    v: float


class AABB:
    def __init__(self, mn, mx):
        self.min = list(mn)
        self.max = list(mx)


@dataclass
class BVH:
    """bvh.ts:18-24: nodes (8 floats per node), node_count, tri_indices, bounds."""
    nodes: np.ndarray
    node_count: int
    tri_indices: np.ndarray
    bounds: AABB
    _device: Optional["DeviceBVH"] = None


class DeviceBVH:
    """A BVH and its triangles resident on the GPU (a lucent_bvh handle)."""

    def __init__(self, nodes, tri_indices, positions, node_count=None):
        nodes = np.ascontiguousarray(nodes, np.float32).reshape(-1)
        tri = np.ascontiguousarray(tri_indices, np.uint32).reshape(-1)
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1)
        if pos.size != tri.size * 9:
            raise ValueError("positions cover %d triangles; triIndices has %d" % (pos.size // 9, tri.size))
        self.node_count = int(node_count if node_count is not None else nodes.size // NODE_STRIDE)
        self.tri_count = int(tri.size)
        h = C.c_void_p()
        N.check(N.lib().lucent_bvh_create(N.ptr(nodes, C.c_float), self.node_count, N.ptr(tri, C.c_uint32),
                                          self.tri_count, N.ptr(pos, C.c_float), C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            N.lib().lucent_bvh_destroy(self._h)
            self._h = None

    __del__ = close

    def set_mode(self, exact, top_levels=True, wide=True):
        """lucent_bvh_set_mode: all-binary64 traversal (exact), else the
        binary32 path over the four-wide view of the tree (wide), or over the
        binary nodes with (top_levels) or without the shared-memory copy of
        the top BVH levels. Results are identical in every mode."""
        mode = 1 if exact else 3 if wide else 0 if top_levels else 2
        N.check(N.lib().lucent_bvh_set_mode(self._h, mode))

    def intersect(self, rays, t_min=1e-5, t_max=math.inf, stream=None):
        """Closest hits of float32 rays [n, 6] -> (prim int32 (-1 miss), t, u, v) float32."""
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        n = r.shape[0]
        prim = np.empty(n, np.int32)
        t, u, v = (np.empty(n, np.float32) for _ in range(3))
        N.check(N.lib().lucent_bvh_intersect(self._h, N.ptr(r, C.c_float), n, t_min, t_max, N.ptr(prim, C.c_int32),
                                             N.ptr(t, C.c_float), N.ptr(u, C.c_float), N.ptr(v, C.c_float),
                                             stream))
        return prim, t, u, v

    def intersect_device(self, rays_ptr, n, prim_ptr, t_ptr=None, u_ptr=None, v_ptr=None, t_min=1e-5,
                         t_max=math.inf, stream=None):
        """Asynchronous form on device pointers (ints); call check() to synchronise."""
        N.check(N.lib().lucent_bvh_intersect_device(self._h, rays_ptr, n, t_min, t_max, prim_ptr, t_ptr, u_ptr,
                                                    v_ptr, stream))

    def check(self, stream=None):
        N.check(N.lib().lucent_bvh_check(self._h, stream))

    def intersect_f64(self, rays, t_min=1e-5, t_max=math.inf):
        """Closest hits of binary64 rays [n, 6] -> (prim, t, u, v) in binary64."""
        r = np.ascontiguousarray(rays, np.float64).reshape(-1, 6)
        n = r.shape[0]
        prim = np.empty(n, np.int32)
        t, u, v = (np.empty(n, np.float64) for _ in range(3))
        N.check(N.lib().lucent_bvh_intersect_f64(self._h, N.ptr(r, C.c_double), n, t_min, t_max,
                                                 N.ptr(prim, C.c_int32), N.ptr(t, C.c_double),
                                                 N.ptr(u, C.c_double), N.ptr(v, C.c_double), None))
        return prim, t, u, v


def device_bvh(bvh: BVH, positions) -> DeviceBVH:
    """The device copy of a reference-layout BVH (cached on the BVH object)."""
    if bvh._device is None:
        bvh._device = DeviceBVH(bvh.nodes, bvh.tri_indices, positions, bvh.node_count)
    return bvh._device


def intersect_bvh(bvh: BVH, positions, ray, t_min=1e-5, t_max=math.inf) -> Optional[BVHHit]:
    """intersectBVH (bvh.ts:265-320) for one binary64 ray {origin, dir}; None on a miss."""
    if bvh.tri_indices.size == 0:  # bvh.ts:274
        return None
    o, d = (ray["origin"], ray["dir"]) if isinstance(ray, dict) else ray
    dev = device_bvh(bvh, positions)
    prim, t, u, v = dev.intersect_f64(np.array([list(o) + list(d)], np.float64), t_min, t_max)
    if prim[0] < 0:
        return None
    return BVHHit(float(t[0]), int(prim[0]), float(u[0]), float(v[0]))


def _wrap_handle(h, node_count, tri_count):
    dev = DeviceBVH.__new__(DeviceBVH)
    dev._h = h
    dev.node_count = node_count
    dev.tri_count = tri_count
    return dev


def build_bvh(positions, max_leaf_size=4, bins=12, stream=None) -> BVH:
    """buildBVH (bvh.ts:52-252) on the GPU: the reference's node array, triIndices and bounds.

    The returned BVH also keeps its device copy, so intersect calls need no upload.
    """
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1)
    if pos.size % 9:
        raise ValueError("positions length %d is not a multiple of 9" % pos.size)  # bvh.ts:55-57
    n = pos.size // 9
    nodes = np.zeros(max(1, 2 * n - 1) * NODE_STRIDE, np.float32)
    tri = np.zeros(max(n, 1), np.uint32)
    cnt = C.c_uint32()
    bounds = np.zeros(6, np.float64)
    opts = N.BvhOpts(max_leaf_size, bins)
    h = C.c_void_p()
    N.check(N.lib().lucent_bvh_build(N.ptr(pos, C.c_float), pos.size, C.byref(opts), N.ptr(nodes, C.c_float),
                                     C.byref(cnt), N.ptr(tri, C.c_uint32), N.ptr(bounds, C.c_double), C.byref(h),
                                     stream))
    nc = cnt.value
    b = BVH(nodes[: nc * NODE_STRIDE].copy(), nc, tri[:n].copy(), AABB(bounds[:3], bounds[3:]))
    b._device = _wrap_handle(h, nc, n)
    return b


def build_bvh_async(positions, max_leaf_size=4, bins=12):
    """buildBVHAsync (bvh-async.ts:8): a future resolving to the BVH.

    The GPU build does not occupy the page's thread in the reference's sense;
    the future runs it on a worker thread so callers keep their own loop going.
    """
    import concurrent.futures as cf
    ex = cf.ThreadPoolExecutor(max_workers=1)
    fut = ex.submit(build_bvh, positions, max_leaf_size, bins)
    ex.shutdown(wait=False)
    return fut


def build_device(positions_ptr, tri_count, max_leaf_size=4, bins=12, stream=None) -> DeviceBVH:
    """Builds from device-resident positions (an int pointer); returns only the device BVH."""
    opts = N.BvhOpts(max_leaf_size, bins)
    h = C.c_void_p()
    N.check(N.lib().lucent_bvh_build_device(positions_ptr, tri_count, C.byref(opts), C.byref(h), stream))
    nc = C.c_uint32()
    tc = C.c_uint32()
    N.check(N.lib().lucent_bvh_info(h, C.byref(nc), C.byref(tc)))
    return _wrap_handle(h, nc.value, tc.value)


def download(dev: DeviceBVH):
    """Reference-layout (nodes, triIndices) of a device BVH."""
    nodes = np.zeros(dev.node_count * NODE_STRIDE, np.float32)
    tri = np.zeros(max(dev.tri_count, 1), np.uint32)
    N.check(N.lib().lucent_bvh_download(dev.handle, N.ptr(nodes, C.c_float), N.ptr(tri, C.c_uint32)))
    return nodes, tri[: dev.tri_count]
