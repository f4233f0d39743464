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


def furnace_scene(albedo=1.0, roughness=1.0, ior=1.0, radiance=1.0, **layers):
    """A sphere inside a uniform environment of the given radiance (white
    furnace). Extra keyword arguments set further material fields (clearcoat,
    sheen_color, transmission, ...)."""
    from . import mesh as M
    from . import scene as S
    w, h = 16, 8
    env = S.Environment(map=S.HDRImage(w, h, np.full(w * h * 3, radiance, np.float32)), background=True)
    ball = M.icosphere(4, radius=1.0)
    mat = S.material(albedo=(albedo, albedo, albedo), roughness=roughness, ior=ior, **layers)
    cam = S.Camera(position=(0.0, 0.0, 4.0), target=(0.0, 0.0, 0.0), fov=30.0, focus_distance=4.0)
    return S.Scene(name="furnace", camera=cam, env=env, meshes=[S.MeshInstance(ball, mat)])


def sky_scene(seed=0, subdivisions=3):
    """Outdoor scene for the analytic parts of traceScene and the lights: the
    procedural sky baked by bakeSky (no environment map, so the analytic sun
    is on: renderer.ts:359-367), the ground plane, analytic spheres
    (scene.glsl:132-144) of layered, metallic and dielectric materials, one
    emissive sphere (a sphere light, lights.glsl:99-158), and an icosphere
    mesh beside them (BVH triangles in the same frame).

    Draw order from numpy.random.Generator(PCG64(seed)): sun elevation
    U[20, 60], azimuth U[0, 360), 3 sphere albedos (3 x 3), the mesh albedo (3).
    """
    from . import mesh as M
    from . import scene as S
    rng = np.random.Generator(np.random.PCG64(seed))
    elev, azim = rng.uniform(20.0, 60.0), rng.uniform(0.0, 360.0)
    alb = rng.uniform(0.2, 0.8, (3, 3))
    mesh_alb = rng.uniform(0.2, 0.8, 3)
    spheres = [
        S.Sphere((-1.1, 0.5, 0.0), 0.5, S.material(albedo=tuple(alb[0]), roughness=0.4, clearcoat=0.8,
                                                   clearcoat_roughness=0.1, sheen_color=(0.5, 0.5, 0.5),
                                                   sheen_roughness=0.4)),
        S.Sphere((0.0, 0.45, -0.6), 0.45, S.metal(tuple(alb[1]), roughness=0.25)),
        S.Sphere((1.05, 0.4, 0.2), 0.4, S.glass(ior=1.5, roughness=0.05)),
        S.Sphere((0.3, 1.6, 0.9), 0.15, S.light((1.0, 0.8, 0.6), 30.0)),
    ]
    ball = M.icosphere(subdivisions, radius=0.35, center=(0.2, 0.35, 0.8))
    meshes = [S.MeshInstance(ball, S.material(albedo=tuple(mesh_alb), roughness=0.6))]
    sun = S.Sun(elevation=float(elev), azimuth=float(azim), color=(1.0, 0.95, 0.9), intensity=3.0,
                angular_radius=2.0)
    sky = S.Sky(enabled=True, intensity=1.0)
    env = S.Environment(map=None, background=True)
    ground = S.Ground(enabled=True, height=0.0, material=S.matte((0.45, 0.45, 0.42)))
    cam = S.Camera(position=(0.0, 1.2, 4.0), target=(0.0, 0.45, 0.0), fov=45.0, focus_distance=4.0)
    return S.Scene(name="sky", camera=cam, sun=sun, sky=sky, env=env, ground=ground, spheres=spheres, meshes=meshes)


def knot_scene(seed=0, tubular=5000, radial=200, env_width=1024):
    """Large-mesh scene: torusKnot(p=2, q=3) tessellated to 2 * tubular *
    radial triangles (2,000,000 at 5000 x 200) and displaced along the normals
    by 3-octave value noise of amplitude 0.05; 16 layered materials (4
    dielectrics with IOR U[1.3,1.8] and Beer-Lambert sigma_a U[0,2]^3 as
    attenuationDistance 1, attenuationColor exp(-sigma_a); 12 opaque with the
    box scene's parameter ranges, two of them alpha-blended at alpha 0.5 and
    covering 10% of the triangles); an env_width x env_width/2 HDRI of
    lognormal(0, 1) luminance with a 0.5 degree sun disk of radiance 5e4 baked
    in (the analytic sun is off with a map); thin-lens camera, aperture 0.02.

    Materials follow bands of the tube: band b = (160 * i) // tubular for
    tubular index i, and b % 20 picks the material (18 -> 14, 19 -> 15, the
    alpha-blended ones; r < 18 -> [0..13, 4..7][r]).
    Draw order from numpy.random.Generator(PCG64(seed)): 4 IORs, 4 x 3
    sigma_a, 4 dielectric roughnesses, then per opaque material albedo (3),
    roughness, metallic, clearcoat, clearcoat roughness, sheen, sheen
    roughness; then the HDRI luminance (H x W) and tints (H x W x 3).
    """
    from . import mesh as M
    from . import scene as S
    rng = np.random.Generator(np.random.PCG64(seed))
    mats = []
    iors = rng.uniform(1.3, 1.8, 4)
    sig = rng.uniform(0.0, 2.0, (4, 3))
    drough = rng.uniform(0.0, 0.3, 4)
    for k in range(4):
        mats.append(S.material(albedo=(1.0, 1.0, 1.0), transmission=1.0, ior=float(iors[k]),
                               roughness=float(drough[k]), attenuation_distance=1.0,
                               attenuation_color=tuple(float(x) for x in np.exp(-sig[k]))))
    for k in range(12):
        alb = rng.uniform(0.2, 0.8, 3)
        rough = rng.uniform(0.05, 1.0)
        metallic = float(rng.random() < 0.5)
        coat, coat_rough = rng.uniform(0.0, 1.0), rng.uniform(0.0, 0.5)
        sheen, sheen_rough = rng.uniform(0.0, 1.0), rng.uniform(0.2, 1.0)
        extra = {"alpha": 0.5, "alpha_mode": "blend"} if k >= 10 else {}
        mats.append(S.material(albedo=tuple(float(x) for x in alb), roughness=float(rough), metallic=metallic,
                               clearcoat=float(coat), clearcoat_roughness=float(coat_rough),
                               sheen_color=(float(sheen),) * 3, sheen_roughness=float(sheen_rough), **extra))
    knot = knot_mesh(seed, tubular, radial)
    tube_index = np.arange(knot.triangle_count) // (2 * radial)
    r = ((160 * tube_index) // tubular) % 20
    pick = np.array([0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 4, 5, 6, 7, 14, 15])[r]
    pos = knot.positions.reshape(-1, 9)
    nrm = knot.normals.reshape(-1, 9)
    meshes = []
    for m in range(16):
        sel = pick == m
        if sel.any():
            meshes.append(S.MeshInstance(M.Mesh(pos[sel].reshape(-1).copy(), nrm[sel].reshape(-1).copy()), mats[m]))
    W, H = env_width, env_width // 2
    lum = np.exp(rng.normal(0.0, 1.0, (H, W)))
    tint = rng.uniform(0.8, 1.2, (H, W, 3))
    tint /= (tint @ np.array([0.2126, 0.7152, 0.0722]))[..., None]
    img = lum[..., None] * tint
    sun = np.array(S.from_spherical(np.radians(35.0), np.radians(40.0)))
    cos_r = np.cos(np.radians(0.25))
    x = (np.arange(W) + 0.5) / W
    y = (np.arange(H) + 0.5) / H
    X, Y = np.meshgrid(x, y)
    dx, dy, dz = S.direction_from_uv(X, Y)
    near = np.argwhere(dx * sun[0] + dy * sun[1] + dz * sun[2] > np.cos(np.radians(2.0)))
    sub = (np.arange(16) + 0.5) / 16
    for yy, xx in near:  # supersampled disk coverage
        su, sv = np.meshgrid((xx + sub) / W, (yy + sub) / H)
        ex, ey, ez = S.direction_from_uv(su, sv)
        cover = np.mean(ex * sun[0] + ey * sun[1] + ez * sun[2] >= cos_r)
        img[yy, xx] += 5e4 * cover
    env = S.Environment(map=S.HDRImage(W, H, img.astype(np.float32).reshape(-1)), name="lognormal + sun",
                        background=True)
    cam = S.Camera(position=(0.0, 0.4, 4.2), target=(0.0, 0.0, 0.0), fov=40.0, aperture=0.02,
                   focus_distance=4.22)
    return S.Scene(name="knot", camera=cam, env=env, meshes=meshes)


def env_lognormal(rng, width, height):
    """HDRI of lognormal(0, 1) luminance with per-texel tints U[0.8,1.2]^3
    normalised to that luminance; draws luminance (H x W) then tints."""
    from . import scene as S
    lum = np.exp(rng.normal(0.0, 1.0, (height, width)))
    tint = rng.uniform(0.8, 1.2, (height, width, 3))
    tint /= (tint @ np.array([0.2126, 0.7152, 0.0722]))[..., None]
    return S.HDRImage(width, height, (lum[..., None] * tint).astype(np.float32).reshape(-1))


BATCH_RESOLUTIONS = (256, 512, 768, 1024)


def _batch_shape(rng, tri_lo, tri_hi):
    """The first draws of batch_scene: (knot?, resolution, tubular, radial, icosphere subdivisions)."""
    target = float(np.exp(rng.uniform(np.log(tri_lo), np.log(tri_hi))))
    knot = rng.random() < 0.5
    res = BATCH_RESOLUTIONS[int(rng.integers(0, len(BATCH_RESOLUTIONS)))]
    radial = int(rng.integers(16, 64))
    tubular = max(8, int(round(target / (2 * radial))))
    sub = int(np.clip(np.round(np.log(target / 20.0) / np.log(4.0)), 0, 9))
    return knot, res, tubular, radial, sub


def batch_sizes(count=64, tri_lo=10_000, tri_hi=2_000_000):
    """Triangle counts of batch_scene(0 .. count - 1), without building them."""
    out = []
    for seed in range(count):
        knot, _, tubular, radial, sub = _batch_shape(np.random.Generator(np.random.PCG64(seed)), tri_lo, tri_hi)
        out.append(2 * tubular * radial if knot else 20 * 4 ** sub)
    return np.array(out, np.int64)


def knot_mesh(seed=0, tubular=5000, radial=200):
    """The displaced torus knot of knot_scene alone (2 * tubular * radial triangles)."""
    from . import mesh as M
    return M.displace(M.torus_knot(2, 3, radius=1.0, tube=0.32, tubular_segments=tubular, radial_segments=radial),
                      0.05, octaves=3, seed=seed)


def batch_scene(seed, tri_lo=10_000, tri_hi=2_000_000):
    """One scene of the batched workload: a displaced torus knot or
    icosphere with a triangle count log-uniform in [tri_lo, tri_hi], four
    layered materials, a 512 x 256 lognormal HDRI, a square resolution from
    BATCH_RESOLUTIONS. Returns (scene, resolution).

    Draw order from numpy.random.Generator(PCG64(seed)): log triangle count,
    shape (knot if < 0.5), resolution index, knot radial segments in
    [16, 64), then per material albedo (3), roughness, metallic, clearcoat,
    sheen; then the HDRI.
    """
    from . import mesh as M
    from . import scene as S
    rng = np.random.Generator(np.random.PCG64(seed))
    knot, res, tubular, radial, sub = _batch_shape(rng, tri_lo, tri_hi)
    if knot:
        mesh = M.torus_knot(2, 3, 1.0, 0.32, tubular, radial)
    else:
        mesh = M.icosphere(sub, radius=1.2)
    mesh = M.displace(mesh, 0.05, octaves=3, seed=seed)
    mats = []
    for _ in range(4):
        alb = rng.uniform(0.2, 0.8, 3)
        rough, metallic = rng.uniform(0.05, 1.0), float(rng.random() < 0.5)
        coat, sheen = rng.uniform(0.0, 1.0), rng.uniform(0.0, 1.0)
        mats.append(S.material(albedo=tuple(float(x) for x in alb), roughness=float(rough), metallic=metallic,
                               clearcoat=float(coat), clearcoat_roughness=0.1, sheen_color=(float(sheen),) * 3,
                               sheen_roughness=0.5))
    n = mesh.triangle_count
    band = (np.arange(n) * 4) // max(n, 1)
    pos, nrm = mesh.positions.reshape(-1, 9), mesh.normals.reshape(-1, 9)
    meshes = [S.MeshInstance(M.Mesh(pos[band == k].reshape(-1).copy(), nrm[band == k].reshape(-1).copy()), mats[k])
              for k in range(4) if (band == k).any()]
    env = S.Environment(map=env_lognormal(rng, 512, 256), name="lognormal", background=True)
    cam = S.Camera(position=(0.0, 0.3, 4.0), target=(0.0, 0.0, 0.0), fov=45.0, focus_distance=4.0)
    return S.Scene(name="batch%d" % seed, camera=cam, env=env, meshes=meshes), res


def adjoint_scene(seed=0, subdivisions=6, env_size=(256, 128)):
    """The inverse-rendering workload: the box scene's geometry with 32
    materials (5 walls, the lamp, 2 boxes and the icosphere split into 24
    bands of its triangles, each a layered material with the box scene's
    parameter ranges) under a lognormal env_size HDRI seen through the open
    front. Draw order from numpy.random.Generator(PCG64(seed + 1000)): 24
    band materials (albedo 3, roughness, metallic, clearcoat, sheen), then
    the HDRI."""
    from . import mesh as M
    from . import scene as S
    sc = box_scene(seed, subdivisions)
    rng = np.random.Generator(np.random.PCG64(seed + 1000))
    ball = sc.meshes[-1]
    n = ball.mesh.triangle_count
    band = (np.arange(n) * 24) // n
    pos, nrm = ball.mesh.positions.reshape(-1, 9), ball.mesh.normals.reshape(-1, 9)
    meshes = sc.meshes[:-1]
    for k in range(24):
        alb = rng.uniform(0.2, 0.8, 3)
        rough, metallic = rng.uniform(0.05, 1.0), float(rng.random() < 0.5)
        coat, sheen = rng.uniform(0.0, 1.0), rng.uniform(0.0, 1.0)
        mat = S.material(albedo=tuple(float(x) for x in alb), roughness=float(rough), metallic=metallic,
                         clearcoat=float(coat), clearcoat_roughness=0.2, sheen_color=(float(sheen),) * 3,
                         sheen_roughness=0.5)
        sel = band == k
        meshes.append(S.MeshInstance(M.Mesh(pos[sel].reshape(-1).copy(), nrm[sel].reshape(-1).copy()), mat))
    env = S.Environment(map=env_lognormal(rng, *env_size), name="lognormal", background=True)
    return S.Scene(name="adjoint", camera=sc.camera, env=env, meshes=meshes)


def adjoint_views(count=8):
    """Camera positions of the multi-view inverse-rendering workload: a 2 x 4
    grid in front of the box's open side, all aimed at the box centre."""
    from . import scene as S
    out = []
    for i in range(count):
        x = -0.6 + 1.2 * (i % 4) / 3.0
        y = 0.7 + 0.6 * (i // 4)
        out.append(S.Camera(position=(x, y, 3.4), target=(0.0, 1.0, 0.0), fov=40.0, focus_distance=3.4))
    return out


# ------------------------------------------------------------------ textured model
def _noise_rgb(rng, n, cells, lo, hi):
    """Smooth value noise (bilinear over a cells x cells grid, wrapping) in [lo, hi]^3, [n, n, 3] floats."""
    grid = rng.uniform(lo, hi, (cells, cells, 3))
    x = (np.arange(n) + 0.5) / n * cells - 0.5
    i0 = np.floor(x).astype(int)
    f = x - i0
    i0 %= cells
    i1 = (i0 + 1) % cells
    a = grid[i0][:, i0] * (1 - f)[None, :, None] + grid[i0][:, i1] * f[None, :, None]
    b = grid[i1][:, i0] * (1 - f)[None, :, None] + grid[i1][:, i1] * f[None, :, None]
    return a * (1 - f)[:, None, None] + b * f[:, None, None]


def textured_model_glb(seed=0, tex=256):
    """A GLB exercising every map of the layered material: a slab with tiled
    (texture-transformed) base colour, metal-rough and normal maps; an
    icosphere with spherical texture coordinates, base colour and normal maps
    and a clearcoat; an alpha-masked cut-out quad; an emissive panel with an
    emissive map. Textures are seeded value noise encoded as PNG."""
    from . import gltf as G
    from . import images as I
    from . import mesh as M
    rng = np.random.default_rng(seed)
    u8 = lambda x: np.clip(np.rint(x * 255), 0, 255).astype(np.uint8)

    def rgba(rgb, a=None):
        out = np.empty(rgb.shape[:2] + (4,), np.uint8)
        out[..., :3] = u8(rgb)
        out[..., 3] = 255 if a is None else u8(a)
        return out

    base = _noise_rgb(rng, tex, 8, 0.1, 0.9)
    checker = ((np.arange(tex)[:, None] // (tex // 8) + np.arange(tex)[None, :] // (tex // 8)) % 2)[..., None]
    base = base * (0.55 + 0.45 * checker)
    mr = _noise_rgb(rng, tex, 6, 0.0, 1.0)
    mr[..., 0] = 1.0
    mr[..., 1] = 0.15 + 0.85 * mr[..., 1]           # roughness in G
    mr[..., 2] = (mr[..., 2] > 0.55).astype(float)  # metal in B
    height = _noise_rgb(rng, tex, 16, 0.0, 1.0)[..., 0]
    gy, gx = np.gradient(height * 6.0)
    nrm = np.stack([-gx, -gy, np.ones_like(gx)], -1)
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    cut = _noise_rgb(rng, tex, 5, 0.0, 1.0)[..., 0]
    glow = _noise_rgb(rng, tex, 4, 0.2, 1.0)
    images = [rgba(base), rgba(np.clip(mr, 0, 1)), rgba(nrm * 0.5 + 0.5),
              rgba(_noise_rgb(rng, tex, 6, 0.3, 1.0), (cut > 0.45).astype(float)), rgba(glow)]

    def spherical_uv(m, center):
        p = m.positions.reshape(-1, 3).astype(np.float64) - np.array(center)
        p = p / np.linalg.norm(p, axis=1, keepdims=True)
        u = 0.5 + np.arctan2(p[:, 2], p[:, 0]) / (2 * np.pi)
        v = np.arccos(np.clip(p[:, 1], -1, 1)) / np.pi
        return np.stack([u, v], 1).astype(np.float32).reshape(-1)

    def quad_uv(m, reps):
        return (np.array([0, 0, 1, 0, 1, 1, 0, 0, 1, 1, 0, 1], np.float32) * reps)

    slab = M.quad([-2, 0, 2], [2, 0, 2], [2, 0, -2], [-2, 0, -2])
    sphere = M.icosphere(3, 0.7, (0.0, 0.7, 0.0))
    cutout = M.quad([-1.8, 0, -1.2], [-0.4, 0, -1.2], [-0.4, 1.4, -1.2], [-1.8, 1.4, -1.2])
    panel = M.quad([0.6, 0.1, -1.6], [1.8, 0.1, -1.6], [1.8, 1.1, -1.6], [0.6, 1.1, -1.6])
    meshes = [(slab, quad_uv(slab, 3.0), 0), (sphere, spherical_uv(sphere, (0.0, 0.7, 0.0)), 1), (cutout, quad_uv(cutout, 1.0), 2),
              (panel, quad_uv(panel, 1.0), 3)]
    blob = b""
    views, accessors, prims = [], [], []

    def add(data, **extra):
        nonlocal blob
        raw = np.ascontiguousarray(data).tobytes()
        views.append({"buffer": 0, "byteOffset": len(blob), "byteLength": len(raw), **extra})
        blob += raw + b"\0" * (-len(raw) % 4)
        return len(views) - 1

    for mesh, uv, mat in meshes:
        n = mesh.positions.size // 3
        pos = mesh.positions.reshape(-1, 3)
        ids = []
        for arr, typ in ((pos, "VEC3"), (mesh.normals.reshape(-1, 3), "VEC3"), (uv.reshape(-1, 2), "VEC2")):
            acc = {"bufferView": add(arr.astype(np.float32)), "componentType": 5126, "count": n, "type": typ}
            if typ == "VEC3" and len(ids) == 0:
                acc["min"], acc["max"] = pos.min(0).tolist(), pos.max(0).tolist()
            accessors.append(acc)
            ids.append(len(accessors) - 1)
        prims.append({"attributes": {"POSITION": ids[0], "NORMAL": ids[1], "TEXCOORD_0": ids[2]}, "material": mat})
    image_views = [add(np.frombuffer(I.encode_png(im), np.uint8)) for im in images]
    doc = {
        "asset": {"version": "2.0", "generator": "lucent_gb300.workloads"},
        "scene": 0, "scenes": [{"nodes": [0]}], "nodes": [{"mesh": 0}],
        "meshes": [{"primitives": prims}],
        "materials": [
            {"pbrMetallicRoughness": {"baseColorTexture": {"index": 0, "extensions": {"KHR_texture_transform": {
                "offset": [0.1, 0.2], "rotation": 0.3, "scale": [1.5, 1.5]}}},
                "metallicRoughnessTexture": {"index": 1}, "metallicFactor": 1.0, "roughnessFactor": 1.0},
             "normalTexture": {"index": 2, "scale": 0.8}},
            {"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}, "metallicFactor": 0.0,
                                      "roughnessFactor": 0.45},
             "normalTexture": {"index": 2}, "extensions": {"KHR_materials_clearcoat": {"clearcoatFactor": 0.6}}},
            {"pbrMetallicRoughness": {"baseColorTexture": {"index": 3}, "metallicFactor": 0.0,
                                      "roughnessFactor": 0.7},
             "alphaMode": "MASK", "alphaCutoff": 0.5, "doubleSided": True},
            {"pbrMetallicRoughness": {"baseColorFactor": [0.05, 0.05, 0.05, 1], "metallicFactor": 0.0},
             "emissiveTexture": {"index": 4}, "emissiveFactor": [1, 0.9, 0.8],
             "extensions": {"KHR_materials_emissive_strength": {"emissiveStrength": 6.0}}},
        ],
        "textures": [{"source": i} for i in range(len(images))],
        "images": [{"bufferView": v, "mimeType": "image/png", "name": "tex%d" % i} for i, v in enumerate(image_views)],
        "accessors": accessors, "bufferViews": views, "buffers": [{"byteLength": len(blob)}],
    }
    return G.write_glb(doc, blob)


def textured_scene(seed=0, tex=256, env_width=256):
    """textured_model_glb through the model path (load_gltf, decode_images,
    scene_from_model) under a lognormal HDRI."""
    from . import gltf as G
    from . import model as MD
    from . import scene as S
    rng = np.random.default_rng(seed + 1000)
    env = S.Environment(map=env_lognormal(rng, env_width, env_width // 2), name="lognormal")
    model = MD.model_from_asset("textured", G.load_gltf(textured_model_glb(seed, tex)))
    return MD.scene_from_model(model, env)
