"""The no-allocation closest-hit entry point (lucent_bvh_intersect_noalloc).

Callers that may not allocate device memory (their own allocator owns the
GPU's memory, or they cannot take cudaMalloc's synchronisation) pass every
buffer themselves; the kernels' scratch is a file-scope device array inside
the library. This test builds the device layouts in buffers it owns, calls
the entry point through the C ABI twice in a row, and checks both results
against the allocating entry point (lucent_bvh_intersect) with the same
tolerance as the other closest-hit tests: equal ids, equal t, u, v.
Collected last so that a failure here never hides another test's result.
"""
import ctypes as C
import math

import numpy as np
import pytest

from lucent_gb300 import _native as N
from lucent_gb300 import bvh as B
from lucent_gb300 import workloads

pytestmark = pytest.mark.gpu


def _device_layouts(bvh, positions):
    """Node array with integer fields as int32 bits; triangles in slot order."""
    ref = bvh.nodes.reshape(-1, 8)
    nodes = ref.copy()
    ints = nodes.view(np.int32)
    ints[:, 3] = ref[:, 3].astype(np.int32)
    ints[:, 7] = ref[:, 7].astype(np.int32)
    src = bvh.tri_indices.astype(np.int64)
    tris = np.zeros((src.size, 3, 4), np.float32)
    tris[:, :, :3] = positions.reshape(-1, 3, 3)[src]
    tris.view(np.int32)[:, 0, 3] = src.astype(np.int32)
    return nodes.reshape(-1), tris.reshape(-1)


def test_no_alloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    pos, rays = workloads.soup_and_rays(seed=4, n_tri=20000, n_rays=200_000)
    bvh = B.build_bvh(pos)
    ref_prim, ref_t, ref_u, ref_v = bvh._device.intersect(rays, 1e-5, math.inf)

    nodes, tris = _device_layouts(bvh, pos)
    d_nodes = torch.from_numpy(nodes).cuda()
    d_tris = torch.from_numpy(tris).cuda()
    d_rays = torch.from_numpy(np.ascontiguousarray(rays)).cuda()
    n = rays.shape[0]
    L = N.lib()
    L.lucent_bvh_intersect_noalloc.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p,
                                               C.c_uint32, C.c_double, C.c_double, C.c_void_p, C.c_void_p,
                                               C.c_void_p, C.c_void_p, C.c_void_p]
    L.lucent_bvh_intersect_noalloc.restype = C.c_int32
    for _ in range(2):  # the shared scratch keeps the previous call's contents
        prim = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        t, u, v = (torch.zeros(n, dtype=torch.float32, device="cuda") for _ in range(3))
        N.check(L.lucent_bvh_intersect_noalloc(d_nodes.data_ptr(), bvh.node_count, d_tris.data_ptr(), pos.size // 9,
                                               d_rays.data_ptr(), n, 1e-5, math.inf, prim.data_ptr(), t.data_ptr(),
                                               u.data_ptr(), v.data_ptr(), None))
        p = prim.cpu().numpy()
        assert np.array_equal(p, ref_prim)
        hit = p >= 0
        assert hit.mean() > 0.3
        assert np.array_equal(t.cpu().numpy()[hit], ref_t[hit])
        assert np.array_equal(u.cpu().numpy()[hit], ref_u[hit])
        assert np.array_equal(v.cpu().numpy()[hit], ref_v[hit])
