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


# ----------------------------------------------------------------------------- path-tracing scenes
def box_scene(seed=0, subdivisions=6, width=512, height=512):
    """Closed box of 5 Lambert quads (albedo U[0.2,0.8]^3) lit by one ceiling quad
    light of radiance 15, two boxes rotated U[0, pi/2] about Y, and an
    icosphere (20 * 4**subdivisions triangles; 81,920 at 6) with random
    layered-BSDF parameters: roughness U[0.05,1], metallic Bernoulli(0.5),
    clearcoat U[0,1], sheen U[0,1] (-> sheen colour).

    Draw order from numpy.random.Generator(PCG64(seed)): 5 wall albedos (5x3),
    2 box albedos (2x3), 2 box rotations, sphere albedo (3), roughness,
    metallic, clearcoat, clearcoat roughness, sheen, sheen roughness.
    The environment is black (the open front side sees nothing), so the quad
    light is the only emitter; the analytic sun is off.
    """
    from . import mesh as M
    from . import scene as S
    rng = np.random.Generator(np.random.PCG64(seed))
    walls = rng.uniform(0.2, 0.8, size=(5, 3))
    box_alb = rng.uniform(0.2, 0.8, size=(2, 3))
    rot = rng.uniform(0.0, np.pi / 2, size=2)
    sph_alb = rng.uniform(0.2, 0.8, size=3)
    rough = rng.uniform(0.05, 1.0)
    metallic = float(rng.random() < 0.5)
    coat = rng.uniform(0.0, 1.0)
    coat_rough = rng.uniform(0.0, 0.5)
    sheen = rng.uniform(0.0, 1.0)
    sheen_rough = rng.uniform(0.2, 1.0)
    x0, x1, y0, y1, z0, z1 = -1.0, 1.0, 0.0, 2.0, -1.0, 1.0
    quads = [  # counter-clockwise seen from inside the box
        M.quad((x0, y0, z1), (x1, y0, z1), (x1, y0, z0), (x0, y0, z0)),  # floor, +Y
        M.quad((x0, y1, z0), (x1, y1, z0), (x1, y1, z1), (x0, y1, z1)),  # ceiling, -Y
        M.quad((x0, y0, z0), (x1, y0, z0), (x1, y1, z0), (x0, y1, z0)),  # back, +Z
        M.quad((x0, y0, z1), (x0, y0, z0), (x0, y1, z0), (x0, y1, z1)),  # left, +X
        M.quad((x1, y0, z0), (x1, y0, z1), (x1, y1, z1), (x1, y1, z0)),  # right, -X
    ]
    meshes = [S.MeshInstance(q, S.matte(tuple(walls[i]))) for i, q in enumerate(quads)]
    lamp = M.quad((-0.25, 1.98, -0.25), (0.25, 1.98, -0.25), (0.25, 1.98, 0.25), (-0.25, 1.98, 0.25))
    meshes.append(S.MeshInstance(lamp, S.light((1.0, 1.0, 1.0), 15.0)))
    tall = M.transform(M.box((-0.3, 0.0, -0.3), (0.3, 1.2, 0.3)), translate=(-0.4, 0.0, -0.35), rotate_y=rot[0])
    short = M.transform(M.box((-0.3, 0.0, -0.3), (0.3, 0.6, 0.3)), translate=(0.45, 0.0, 0.3), rotate_y=rot[1])
    meshes.append(S.MeshInstance(tall, S.matte(tuple(box_alb[0]))))
    meshes.append(S.MeshInstance(short, S.matte(tuple(box_alb[1]))))
    ball = M.icosphere(subdivisions, radius=0.3, center=(0.45, 0.9, 0.3))
    meshes.append(S.MeshInstance(ball, S.material(albedo=tuple(sph_alb), roughness=rough, metallic=metallic,
                                                  clearcoat=coat, clearcoat_roughness=coat_rough,
                                                  sheen_color=(sheen, sheen, sheen), sheen_roughness=sheen_rough)))
    cam = S.Camera(position=(0.0, 1.0, 3.4), target=(0.0, 1.0, 0.0), fov=40.0, aperture=0.0, focus_distance=3.4)
    black = S.HDRImage(2, 1, np.zeros(6, np.float32))
    env = S.Environment(map=black, name="black", background=True, backdrop=(0.0, 0.0, 0.0))
    sc = S.Scene(name="box", camera=cam, env=env, meshes=meshes)
    return sc


def furnace_scene(albedo=1.0, roughness=1.0, ior=1.0, radiance=1.0):
    """A sphere inside a uniform environment of the given radiance (white furnace)."""
    from . import mesh as M
    from . import scene as S
    w, h = 16, 8
    env = S.Environment(map=S.HDRImage(w, h, np.full(w * h * 3, radiance, np.float32)), background=True)
    ball = M.icosphere(4, radius=1.0)
    mat = S.material(albedo=(albedo, albedo, albedo), roughness=roughness, ior=ior)
    cam = S.Camera(position=(0.0, 0.0, 4.0), target=(0.0, 0.0, 0.0), fov=30.0, focus_distance=4.0)
    return S.Scene(name="furnace", camera=cam, env=env, meshes=[S.MeshInstance(ball, mat)])
