"""The no-allocation closest-hit entry point (lucent_bvh_intersect_noalloc).

Callers that may not allocate device memory (their own allocator owns the
GPU's memory, or they cannot take cudaMalloc's synchronisation) pass every
buffer themselves; the kernels' scratch is a file-scope device array inside
the library. This test builds the device layouts in buffers it owns, calls
the entry point through the C ABI twice in a row, and checks both results
against the allocating entry point (lucent_bvh_intersect) with the same
tolerance as the other closest-hit tests: equal ids, equal t, u, v, and
t = +inf on misses. It also covers the call's limits: more rays than the
scratch holds, an empty tree, NULL t/u/v outputs, bad t ranges and trees
whose records point outside their arrays (refused before any traversal).
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

MAX_RAYS = 1 << 20  # the scratch array's ray capacity (include/lucent.h)


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


def _entry():
    L = N.lib()
    fn = L.lucent_bvh_intersect_noalloc
    fn.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_double, C.c_double,
                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int32
    return fn


def _ptr(x):
    return None if x is None else x.data_ptr()


@pytest.fixture(scope="module")
def case():
    torch = pytest.importorskip("torch")
    pos, rays = workloads.soup_and_rays(seed=4, n_tri=20000, n_rays=200_000)
    bvh = B.build_bvh(pos)
    ref = bvh._device.intersect(rays, 1e-5, math.inf)
    nodes, tris = _device_layouts(bvh, pos)
    return dict(torch=torch, pos=pos, rays=rays, bvh=bvh, ref=ref, nodes=nodes, tris=tris,
                d_nodes=torch.from_numpy(nodes).cuda(), d_tris=torch.from_numpy(tris).cuda(),
                d_rays=torch.from_numpy(np.ascontiguousarray(rays)).cuda())


def _outputs(torch, n):
    prim = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    t, u, v = (torch.full((n,), 5.0, dtype=torch.float32, device="cuda") for _ in range(3))
    return prim, t, u, v


def test_no_alloc_matches_allocating_entry_point(case):
    torch, fn = case["torch"], _entry()
    ref_prim, ref_t, ref_u, ref_v = case["ref"]
    n = case["rays"].shape[0]
    for _ in range(2):  # the shared scratch keeps the previous call's contents
        prim, t, u, v = _outputs(torch, n)
        N.check(fn(_ptr(case["d_nodes"]), case["bvh"].node_count, _ptr(case["d_tris"]), case["pos"].size // 9,
                   _ptr(case["d_rays"]), n, 1e-5, math.inf, _ptr(prim), _ptr(t), _ptr(u), _ptr(v), None))
        p = prim.cpu().numpy()
        assert np.array_equal(p, ref_prim)
        hit = p >= 0
        assert 0.3 < hit.mean() < 1.0
        tt, uu, vv = t.cpu().numpy(), u.cpu().numpy(), v.cpu().numpy()
        assert np.array_equal(tt[hit], ref_t[hit])
        assert np.array_equal(uu[hit], ref_u[hit])
        assert np.array_equal(vv[hit], ref_v[hit])
        assert np.all(np.isposinf(tt[~hit])) and np.all(uu[~hit] == 0) and np.all(vv[~hit] == 0)


def test_no_alloc_null_t_u_v_and_t_range(case):
    torch, fn = case["torch"], _entry()
    ref_prim = case["ref"][0]
    n = 50_000
    prim = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    N.check(fn(_ptr(case["d_nodes"]), case["bvh"].node_count, _ptr(case["d_tris"]), case["pos"].size // 9,
               _ptr(case["d_rays"]), n, 1e-5, math.inf, _ptr(prim), None, None, None, None))
    assert np.array_equal(prim.cpu().numpy(), ref_prim[:n])
    for t_min, t_max in [(-1.0, math.inf), (math.nan, 1.0), (0.0, math.nan)]:
        st = fn(_ptr(case["d_nodes"]), case["bvh"].node_count, _ptr(case["d_tris"]), case["pos"].size // 9,
                _ptr(case["d_rays"]), n, t_min, t_max, _ptr(prim), None, None, None, None)
        assert st == 1, (t_min, t_max)  # LUCENT_ERR_INVALID


def test_no_alloc_ray_limit(case):
    torch, fn = case["torch"], _entry()
    prim = torch.zeros(8, dtype=torch.int32, device="cuda")
    # Rejected on the host before any launch: the buffers are never touched.
    st = fn(_ptr(case["d_nodes"]), case["bvh"].node_count, _ptr(case["d_tris"]), case["pos"].size // 9,
            _ptr(case["d_rays"]), MAX_RAYS + 1, 1e-5, math.inf, _ptr(prim), None, None, None, None)
    assert st == 5  # LUCENT_ERR_UNSUPPORTED
    assert "1048576" in N.lib().lucent_last_error().decode()


def test_no_alloc_empty_tree(case):
    torch, fn = case["torch"], _entry()
    n = 1000
    empty = torch.zeros(8, dtype=torch.float32, device="cuda")  # the reference's single empty leaf
    prim, t, u, v = _outputs(torch, n)
    N.check(fn(_ptr(empty), 1, None, 0, _ptr(case["d_rays"]), n, 1e-5, math.inf, _ptr(prim), _ptr(t), _ptr(u),
               _ptr(v), None))
    assert np.all(prim.cpu().numpy() == -1)
    assert np.all(np.isposinf(t.cpu().numpy()))
    assert np.all(u.cpu().numpy() == 0) and np.all(v.cpu().numpy() == 0)


@pytest.mark.parametrize("flaw", ["child_past_end", "child_before_parent", "leaf_past_triangles",
                                  "negative_count", "source_index"])
def test_no_alloc_refuses_malformed_tree(case, flaw):
    """Each flaw would make a traversal read outside the caller's buffers; the
    device check refuses the tree before any traversal kernel runs. The check
    itself reads only node_count nodes and tri_count triangles."""
    torch, fn = case["torch"], _entry()
    nodes = case["nodes"].reshape(-1, 8).copy()
    tris = case["tris"].reshape(-1, 12).copy()
    ints = nodes.view(np.int32)
    inner = np.nonzero(ints[:, 7] == 0)[0]
    leaves = np.nonzero(ints[:, 7] > 0)[0]
    m = nodes.shape[0]
    if flaw == "child_past_end":
        bad = int(inner[len(inner) // 2])
        ints[bad, 3] = m - 1
    elif flaw == "child_before_parent":
        bad = int(inner[len(inner) // 2])
        ints[bad, 3] = bad
    elif flaw == "leaf_past_triangles":
        bad = int(leaves[-1])
        ints[bad, 3] = tris.shape[0] - 1
        ints[bad, 7] = 2
    elif flaw == "negative_count":
        bad = int(leaves[0])
        ints[bad, 7] = -3
    else:
        bad = m + 17
        tris.view(np.int32)[17, 3] = tris.shape[0]
    d_nodes = torch.from_numpy(nodes.reshape(-1)).cuda()
    d_tris = torch.from_numpy(tris.reshape(-1)).cuda()
    n = 10_000
    prim, t, u, v = _outputs(torch, n)
    st = fn(_ptr(d_nodes), m, _ptr(d_tris), tris.shape[0], _ptr(case["d_rays"]), n, 1e-5, math.inf, _ptr(prim),
            _ptr(t), _ptr(u), _ptr(v), None)
    assert st == 1  # LUCENT_ERR_INVALID
    msg = N.lib().lucent_last_error().decode()
    assert "malformed BVH" in msg
    if bad < m:
        assert "node %d" % bad in msg
    else:
        assert "slot %d" % (bad - m) in msg
    assert np.all(prim.cpu().numpy() == -7), "outputs written for a refused tree"
    # The scratch is left usable: a good call right after gives the right answer.
    N.check(fn(_ptr(case["d_nodes"]), case["bvh"].node_count, _ptr(case["d_tris"]), case["pos"].size // 9,
               _ptr(case["d_rays"]), n, 1e-5, math.inf, _ptr(prim), None, None, None, None))
    assert np.array_equal(prim.cpu().numpy(), case["ref"][0][:n])
