"""Input generators of the reference's own unit tests, restated exactly.

The reference's randomised tests draw from one LCG
(test/bvh.test.ts:7-13, test/environment.test.ts:7-13):
    s = (s * 1664525 + 1013904223) >>> 0; return s / 2**32
which is exact in u32 arithmetic, so these reproduce the reference's inputs
bit for bit (binary64 values, binary32 at Float32Array stores).
"""
import numpy as np


class LCG:
    def __init__(self, seed):
        self.s = seed & 0xFFFFFFFF

    def __call__(self):
        self.s = (self.s * 1664525 + 1013904223) & 0xFFFFFFFF
        return self.s / 4294967296.0


def random_soup(count, rand):
    """randomSoup (test/bvh.test.ts:15-28)."""
    out = np.zeros(count * 9, np.float32)
    for i in range(count):
        cx = rand() * 10 - 5
        cy = rand() * 10 - 5
        cz = rand() * 10 - 5
        for k in range(3):
            out[i * 9 + k * 3] = cx + rand() - 0.5
            out[i * 9 + k * 3 + 1] = cy + rand() - 0.5
            out[i * 9 + k * 3 + 2] = cz + rand() - 0.5
    return out


def normalize(v):
    """normalize (src/math/vec3.ts:29-33) on one binary64 triple."""
    ln = (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) ** 0.5
    if ln == 0:
        return [0.0, 0.0, 0.0]
    s = 1 / ln
    return [v[0] * s, v[1] * s, v[2] * s]


def bvh_vs_brute_rays(rand, n=400):
    """Rays of test/bvh.test.ts:95-98 (origin in [-8,8]^3, direction normalised)."""
    rays = []
    for _ in range(n):
        o = [rand() * 16 - 8, rand() * 16 - 8, rand() * 16 - 8]
        d = normalize([rand() - 0.5, rand() - 0.5, rand() - 0.5])
        rays.append(o + d)
    return np.array(rays, np.float64)


def torus_rays(rand, n=200):
    """Rays of test/bvh.test.ts:117-119."""
    rays = []
    for _ in range(n):
        o = [rand() * 6 - 3, rand() * 6 - 3, 4.0]
        d = normalize([rand() * 0.4 - 0.2, rand() * 0.4 - 0.2, -1.0])
        rays.append(o + d)
    return np.array(rays, np.float64)
