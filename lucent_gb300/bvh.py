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

    def set_mode(self, exact):
        N.check(N.lib().lucent_bvh_set_mode(self._h, 1 if exact else 0))

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
