"""Seeded synthetic workloads (inputs shared byte for byte by the GPU path,
the oracle and the benchmarks).

Random soup + rays (65,536 triangles, 10^6 rays, seed 0), drawn from
numpy.random.Generator(PCG64(seed)) in this fixed order:
  1. triangle centres   uniform [-1, 1]^3          shape (T, 3)
  2. vertex offsets     normal(0, 0.01)            shape (T, 3, 3)
  3. ray origin dirs    standard normal            shape (R, 3)  -> radius-3 sphere
  4. ray targets        uniform [-1, 1]^3          shape (R, 3)
Directions are normalised in binary64 and every array is stored as float32.
"""
import numpy as np


def soup_and_rays(seed=0, n_tri=65536, n_rays=1_000_000):
    rng = np.random.Generator(np.random.PCG64(seed))
    centres = rng.uniform(-1.0, 1.0, size=(n_tri, 3))
    offs = rng.normal(0.0, 0.01, size=(n_tri, 3, 3))
    positions = (centres[:, None, :] + offs).reshape(-1).astype(np.float32)
    rays = sphere_rays(rng, n_rays)
    return positions, rays


def sphere_rays(rng, n, radius=3.0):
    g = rng.normal(size=(n, 3))
    o = radius * g / np.linalg.norm(g, axis=1, keepdims=True)
    tgt = rng.uniform(-1.0, 1.0, size=(n, 3))
    o32 = o.astype(np.float32).astype(np.float64)
    d = tgt - o32
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o32, d], axis=1).astype(np.float32)


def adversarial_rays(positions, rng, n_each=2000):
    """Rays aimed at vertices, edge midpoints and triangle interiors, grazing
    rays in triangle planes, axis-aligned rays and rays starting on triangles.
    These are the cases where binary32 and binary64 decisions can differ."""
    tri = positions.reshape(-1, 3, 3).astype(np.float64)
    T = tri.shape[0]
    out = []

    def add(o, tgt):
        d = tgt - o
        n = np.linalg.norm(d, axis=1, keepdims=True)
        keep = n[:, 0] > 0
        out.append(np.concatenate([o[keep], d[keep] / n[keep]], 1))

    pick = rng.integers(0, T, n_each)
    far = rng.normal(size=(n_each, 3))
    far = 4.0 * far / np.linalg.norm(far, axis=1, keepdims=True)
    add(far, tri[pick, rng.integers(0, 3, n_each)])  # exact vertices
    k = rng.integers(0, 3, n_each)
    add(far, 0.5 * (tri[pick, k] + tri[pick, (k + 1) % 3]))  # edge midpoints
    add(far, tri[pick].mean(1))  # centroids
    # grazing: origin in the triangle's plane, aimed across it
    e1 = tri[pick, 1] - tri[pick, 0]
    e2 = tri[pick, 2] - tri[pick, 0]
    c = tri[pick].mean(1)
    add(c - 3.0 * e1, c + e2 * 0.1)
    # axis-aligned rays through centroids (zero direction components)
    ax = rng.integers(0, 3, n_each)
    o = c.copy()
    o[np.arange(n_each), ax] -= 3.0
    out.append(np.concatenate([o, np.eye(3)[ax]], 1))
    # rays starting exactly on a triangle (at its centroid)
    dirs = rng.normal(size=(n_each, 3))
    out.append(np.concatenate([c, dirs / np.linalg.norm(dirs, axis=1, keepdims=True)], 1))
    return np.concatenate(out).astype(np.float32)
