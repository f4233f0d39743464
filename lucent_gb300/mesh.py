"""Triangle-soup generators mirroring the reference's src/scene/mesh.ts.

A Mesh holds float32 `positions` and `normals` (9 floats per triangle) and
optional `uvs` (6 per triangle), exactly the reference's layout (mesh.ts:9-13).
Arithmetic is binary64 with a binary32 rounding at the store, as the
reference's Float32Array writes do.

Two generators are new (the workloads need them and the reference has none):
`icosphere` (recursive subdivision) and `displace` (value-noise displacement
along the vertex normal).
"""
from dataclasses import dataclass
from typing import Optional

import numpy as np


@dataclass
class Mesh:
    positions: np.ndarray
    normals: np.ndarray
    uvs: Optional[np.ndarray] = None

    @property
    def triangle_count(self):
        return self.positions.size // 9


def triangle_count(m):
    """triangleCount (mesh.ts:15)."""
    return m.positions.size // 9


def _normalize(v):
    """normalize (src/math/vec3.ts:29-33): scale by 1/length, zero stays zero."""
    v = np.asarray(v, np.float64)
    n = np.sqrt(v[..., 0:1] * v[..., 0:1] + v[..., 1:2] * v[..., 1:2] + v[..., 2:3] * v[..., 2:3])
    return np.where(n == 0, 0.0, v * (1.0 / np.where(n == 0, 1.0, n)))


def merge_meshes(meshes):
    """mergeMeshes (mesh.ts:18-31): concatenation; uvs zero-filled if any input has them."""
    pos = np.concatenate([m.positions for m in meshes]).astype(np.float32) if meshes else np.zeros(0, np.float32)
    nrm = np.concatenate([m.normals for m in meshes]).astype(np.float32) if meshes else np.zeros(0, np.float32)
    if any(m.uvs is not None for m in meshes):
        uvs = np.concatenate([m.uvs if m.uvs is not None else np.zeros(triangle_count(m) * 6, np.float32)
                              for m in meshes]).astype(np.float32)
        return Mesh(pos, nrm, uvs)
    return Mesh(pos, nrm)


def from_triangles(tris):
    """fromTriangles (mesh.ts:34-43): flat face normals."""
    t = np.asarray(tris, np.float64).reshape(-1, 3, 3)
    n = _normalize(np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0]))
    pos = t.reshape(-1).astype(np.float32)
    nrm = np.repeat(n[:, None, :], 3, axis=1).reshape(-1).astype(np.float32)
    return Mesh(pos, nrm)


def quad(a, b, c, d):
    """quad (mesh.ts:46-51): triangles (a, b, c) and (a, c, d)."""
    return from_triangles([[a, b, c], [a, c, d]])


def floor_quad(center, half):
    """floor (mesh.ts:54-62): horizontal square facing +Y."""
    x, y, z = center
    return quad([x - half, y, z + half], [x + half, y, z + half], [x + half, y, z - half], [x - half, y, z - half])


def box(mn, mx, inward=False):
    """box (mesh.ts:65-80): 12 triangles, faces in +Z, -Z, +X, -X, +Y, -Y order."""
    x0, y0, z0 = mn
    x1, y1, z1 = mx
    faces = [
        [(x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1)],
        [(x1, y0, z0), (x0, y0, z0), (x0, y1, z0), (x1, y1, z0)],
        [(x1, y0, z1), (x1, y0, z0), (x1, y1, z0), (x1, y1, z1)],
        [(x0, y0, z0), (x0, y0, z1), (x0, y1, z1), (x0, y1, z0)],
        [(x0, y1, z1), (x1, y1, z1), (x1, y1, z0), (x0, y1, z0)],
        [(x0, y0, z0), (x1, y0, z0), (x1, y0, z1), (x0, y0, z1)],
    ]
    return merge_meshes([quad(d, c, b, a) if inward else quad(a, b, c, d) for a, b, c, d in faces])


def torus_knot(p=2, q=3, radius=1.0, tube=0.32, tubular_segments=200, radial_segments=20):
    """torusKnot (mesh.ts:95-156): ring frame from two curve points 0.01 apart."""
    def curve(t):
        cu, su = np.cos(t), np.sin(t)
        quop = (q / p) * t
        cs = np.cos(quop)
        return np.stack([radius * (2 + cs) * 0.5 * cu, radius * (2 + cs) * su * 0.5,
                         radius * np.sin(quop) * 0.5], -1)

    i = np.arange(tubular_segments, dtype=np.float64)
    u = (i / tubular_segments) * p * np.pi * 2
    P1, P2 = curve(u), curve(u + 0.01)
    T = P2 - P1
    N0 = P2 + P1
    B = _normalize(np.cross(T, N0))
    N = _normalize(np.cross(B, T))
    j = np.arange(radial_segments, dtype=np.float64)
    v = (j / radial_segments) * np.pi * 2
    cx = -tube * np.cos(v)
    cy = tube * np.sin(v)
    offset = N[:, None, :] * cx[None, :, None] + B[:, None, :] * cy[None, :, None]
    ring = P1[:, None, :] + offset
    ring_n = _normalize(offset)
    ii = np.arange(tubular_segments)
    jj = np.arange(radial_segments)
    I, J = np.meshgrid(ii, jj, indexing="ij")
    I1 = (I + 1) % tubular_segments
    J1 = (J + 1) % radial_segments
    # emit(i,j, i1,j, i1,j1) then emit(i,j, i1,j1, i,j1) per (i, j) (mesh.ts:147-154)
    ta = np.stack([np.stack([I, J], -1), np.stack([I1, J], -1), np.stack([I1, J1], -1)], -2)
    tb = np.stack([np.stack([I, J], -1), np.stack([I1, J1], -1), np.stack([I, J1], -1)], -2)
    idx = np.stack([ta, tb], 2).reshape(-1, 3, 2)
    pos = ring[idx[..., 0], idx[..., 1]].reshape(-1).astype(np.float32)
    nrm = ring_n[idx[..., 0], idx[..., 1]].reshape(-1).astype(np.float32)
    return Mesh(pos, nrm)


def transform(mesh, translate=(0.0, 0.0, 0.0), scale=1.0, rotate_y=0.0):
    """transform (mesh.ts:159-182): scale, then rotate about Y, then translate."""
    c, s = np.cos(rotate_y), np.sin(rotate_y)
    p = mesh.positions.astype(np.float64).reshape(-1, 3) * scale
    n = mesh.normals.astype(np.float64).reshape(-1, 3)
    pos = np.stack([p[:, 0] * c + p[:, 2] * s + translate[0], p[:, 1] + translate[1],
                    -p[:, 0] * s + p[:, 2] * c + translate[2]], -1)
    nrm = np.stack([n[:, 0] * c + n[:, 2] * s, n[:, 1], -n[:, 0] * s + n[:, 2] * c], -1)
    return Mesh(pos.reshape(-1).astype(np.float32), nrm.reshape(-1).astype(np.float32), mesh.uvs)


def icosphere(subdivisions, radius=1.0, center=(0.0, 0.0, 0.0)):
    """Icosahedron subdivided `subdivisions` times: 20 * 4**s triangles, smooth normals."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t],
                      [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    faces = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                      [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                      [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    tri = _normalize(verts[faces])  # [F,3,3] on the unit sphere
    for _ in range(subdivisions):
        a, b, c = tri[:, 0], tri[:, 1], tri[:, 2]
        ab, bc, ca = _normalize(a + b), _normalize(b + c), _normalize(c + a)
        tri = np.stack([np.stack([a, ab, ca], 1), np.stack([ab, b, bc], 1), np.stack([ca, bc, c], 1),
                        np.stack([ab, bc, ca], 1)], 1).reshape(-1, 3, 3)
    pos = (tri * radius + np.asarray(center, np.float64)).reshape(-1).astype(np.float32)
    return Mesh(pos, tri.reshape(-1).astype(np.float32))


def _value_noise(p, seed, cells):
    """Trilinear value noise on an integer lattice hashed with a 32-bit mix."""
    p = p * cells
    i0 = np.floor(p).astype(np.int64)
    f = p - i0
    f = f * f * (3 - 2 * f)

    def h(ix, iy, iz):
        x = (ix * 73856093) ^ (iy * 19349663) ^ (iz * 83492791) ^ (seed * 2654435761)
        x = x & 0xFFFFFFFF
        x = ((x >> 16) ^ x) * 0x45D9F3B & 0xFFFFFFFF
        x = ((x >> 16) ^ x) * 0x45D9F3B & 0xFFFFFFFF
        x = (x >> 16) ^ x
        return (x & 0xFFFFFF) / float(0xFFFFFF) * 2.0 - 1.0

    out = 0.0
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                w = (np.where(dx, f[:, 0], 1 - f[:, 0]) * np.where(dy, f[:, 1], 1 - f[:, 1])
                     * np.where(dz, f[:, 2], 1 - f[:, 2]))
                out = out + w * h(i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz)
    return out


def displace(mesh, amplitude, octaves=3, seed=0, base_cells=4.0):
    """Moves every vertex along its normal by `amplitude` x octave-summed value noise.

    Shared vertices move identically (the noise is a function of position), so
    closed meshes stay closed.
    """
    p = mesh.positions.astype(np.float64).reshape(-1, 3)
    n = mesh.normals.astype(np.float64).reshape(-1, 3)
    # The noise depends on the position only: evaluate it once per distinct vertex.
    key = np.ascontiguousarray(mesh.positions.reshape(-1, 3)).view(np.dtype((np.void, 12))).reshape(-1)
    uniq, first, inverse = np.unique(key, return_index=True, return_inverse=True)
    pu = p[first]
    du = np.zeros(pu.shape[0])
    amp, norm = 1.0, 0.0
    for o in range(octaves):
        du += amp * _value_noise(pu, seed + o, base_cells * (2 ** o))
        norm += amp
        amp *= 0.5
    d = du[inverse.reshape(-1)] * (amplitude / norm)
    pos = (p + n * d[:, None]).reshape(-1).astype(np.float32)
    return Mesh(pos, mesh.normals.copy(), mesh.uvs)
