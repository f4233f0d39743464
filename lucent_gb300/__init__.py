"""Lucent GB300: the path-tracing hot path of Lucent on one GB300 (sm_103a).

Host-side mirror of the reference's TypeScript interface over the C ABI in
include/lucent.h. Modules:
  bvh       buildBVH / intersectBVH (src/math/bvh.ts)
  mesh      triangle-soup generators (src/scene/mesh.ts)
  workloads seeded synthetic scenes and ray sets
"""
from ._native import LucentError, NativeMissing, lib  # noqa: F401
from .bvh import BVH, BVHHit, DeviceBVH, NODE_STRIDE, build_bvh, build_bvh_async, intersect_bvh  # noqa: F401

__all__ = ["BVH", "BVHHit", "DeviceBVH", "NODE_STRIDE", "build_bvh", "build_bvh_async", "intersect_bvh", "LucentError", "NativeMissing", "lib"]
