"""Seeded synthetic scenes with the shapes of the benchmark workloads (no assets are shipped).

* cornell_box: the procedural Cornell-style box (5 wall quads + 2 boxes = 34 triangles, plus a separate
  2-triangle 0.25 x 0.25 emissive ceiling quad of radiance 15), built directly at the scene-proxy
  boundary rather than through glTF (the reference glTF loader drops untextured factors).
* terrain_spheres: the incoherent-ray stress scene, an fBm heightfield on an n x n grid (2 n^2
  triangles; n = 1024 gives 2,097,152) plus icospheres of 20 * 4^level triangles (level 5 = 20,480) at
  uniform random positions, with Lambertian / GGX metal (roughness U[0.05, 0.5]) / dielectric (IOR 1.5)
  materials drawn uniformly, lit by an environment cube with a baked sun disk.
* random_rays: origins uniform in a box, isotropic directions.
"""
from __future__ import annotations

import numpy as np

from .abi import (SPK_SKY_CUBE, Instance, Material, Mesh, Scene, Sky, camera_from_look)


def _quad(p0, p1, p2, p3, normal, tangent):
    pos = np.array([p0, p1, p2, p3], np.float32)
    nrm = np.tile(np.asarray(normal, np.float32), (4, 1))
    tan = np.tile(np.asarray(list(tangent) + [1.0], np.float32), (4, 1))
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    idx = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    return Mesh(pos, nrm, idx, tan, uv)


def unit_cube() -> Mesh:
    """Unit cube [-0.5, 0.5]^3 with 24 vertices (flat face normals pointing out) and 12 triangles."""
    pos, nrm, tan, uv, idx = [], [], [], [], []
    faces = [((1, 0, 0), (0, 1, 0)), ((-1, 0, 0), (0, -1, 0)), ((0, 1, 0), (-1, 0, 0)),
             ((0, -1, 0), (1, 0, 0)), ((0, 0, 1), (1, 0, 0)), ((0, 0, -1), (1, 0, 0))]
    for n, t in faces:
        n = np.array(n, np.float64)
        t = np.array(t, np.float64)
        b = np.cross(n, t)
        base = len(pos)
        for su, sv in ((-1, -1), (1, -1), (1, 1), (-1, 1)):
            pos.append(0.5 * n + 0.5 * su * t + 0.5 * sv * b)
            nrm.append(n)
            tan.append(list(t) + [1.0])
            uv.append([(su + 1) / 2, (sv + 1) / 2])
        idx += [[base, base + 1, base + 2], [base, base + 2, base + 3]]
    return Mesh(np.array(pos), np.array(nrm), np.array(idx), np.array(tan), np.array(uv))


def _rot_z(angle):
    c, s = np.cos(angle), np.sin(angle)
    return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])


def _affine(lin, t):
    return np.concatenate([np.asarray(lin, np.float64), np.asarray(t, np.float64)[:, None]], 1).astype(np.float32)


def cornell_box(seed: int = 0):
    """Returns (scene, camera_args). Room [0,1]^3 (Z up, Y front), open towards the camera at -Y."""
    rng = np.random.default_rng(seed)

    def gray():
        return (float(rng.uniform(0.1, 0.8)),) * 3

    red = (float(rng.uniform(0.5, 0.8)), float(rng.uniform(0.1, 0.2)), float(rng.uniform(0.1, 0.2)))
    green = (float(rng.uniform(0.1, 0.2)), float(rng.uniform(0.5, 0.8)), float(rng.uniform(0.1, 0.2)))
    materials = [Material.lambertian(gray()), Material.lambertian(gray()), Material.lambertian(gray()),
                 Material.lambertian(red), Material.lambertian(green), Material.lambertian(gray()),
                 Material.lambertian(gray()), Material.light((15.0, 15.0, 15.0))]
    meshes = [
        _quad((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 0)),      # floor
        _quad((0, 0, 1), (0, 1, 1), (1, 1, 1), (1, 0, 1), (0, 0, -1), (1, 0, 0)),     # ceiling
        _quad((0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1), (0, -1, 0), (1, 0, 0)),     # back wall
        _quad((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1), (1, 0, 0), (0, 1, 0)),      # left wall (red)
        _quad((1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0), (-1, 0, 0), (0, 1, 0)),     # right wall (green)
        unit_cube(),
        _quad((0.375, 0.375, 0.999), (0.375, 0.625, 0.999), (0.625, 0.625, 0.999), (0.625, 0.375, 0.999),
              (0, 0, -1), (1, 0, 0)),                                                # ceiling light
    ]
    eye = np.eye(3)
    instances = [Instance(k, k, _affine(eye, (0, 0, 0))) for k in range(5)]
    tall = _rot_z(0.30) @ np.diag([0.28, 0.28, 0.60])
    short = _rot_z(-0.29) @ np.diag([0.28, 0.28, 0.30])
    instances.append(Instance(5, 5, _affine(tall, (0.32, 0.62, 0.30))))
    instances.append(Instance(5, 6, _affine(short, (0.68, 0.36, 0.15))))
    instances.append(Instance(6, 7, _affine(eye, (0, 0, 0))))
    scene = Scene(meshes, instances, materials, Sky(), name="cornell")
    cam = dict(position=(0.5, -1.3, 0.5), target=(0.5, 0.5, 0.5), world_up=(0, 0, 1), vfov_rad=np.deg2rad(40.0),
               focus_distance=1.8, aperture_radius=0.035 / 22.0 / 2.0, exposure=1.0)
    return scene, cam


def _value_noise(n, cells, rng):
    """Bilinear value noise sampled on an (n+1)^2 grid, `cells` lattice cells across."""
    lattice = rng.uniform(-1.0, 1.0, size=(cells + 2, cells + 2))
    x = np.linspace(0.0, cells, n + 1)
    i = np.floor(x).astype(int)
    f = x - i
    f = f * f * (3 - 2 * f)
    a = lattice[np.ix_(i, i)]
    b = lattice[np.ix_(i + 1, i)]
    c = lattice[np.ix_(i, i + 1)]
    d = lattice[np.ix_(i + 1, i + 1)]
    fx = f[:, None]
    fy = f[None, :]
    return (a * (1 - fx) + b * fx) * (1 - fy) + (c * (1 - fx) + d * fx) * fy


def heightfield(n: int, size: float, amplitude: float, seed: int) -> Mesh:
    """fBm heightfield over [-size/2, size/2]^2: (n+1)^2 vertices, 2 n^2 triangles."""
    rng = np.random.default_rng(seed)
    h = np.zeros((n + 1, n + 1))
    amp, cells = 1.0, 4
    for _ in range(6):
        h += amp * _value_noise(n, cells, rng)
        amp *= 0.5
        cells *= 2
    h *= amplitude
    xs = np.linspace(-size / 2, size / 2, n + 1)
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    pos = np.stack([X, Y, h], -1).reshape(-1, 3)
    dx = size / n
    gx = np.gradient(h, dx, axis=0)
    gy = np.gradient(h, dx, axis=1)
    nrm = np.stack([-gx, -gy, np.ones_like(h)], -1)
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    tan = np.stack([np.ones_like(h), np.zeros_like(h), gx], -1)
    tan /= np.linalg.norm(tan, axis=-1, keepdims=True)
    tan = np.concatenate([tan, np.ones_like(h)[..., None]], -1).reshape(-1, 4)
    uv = np.stack([(X / size + 0.5), (Y / size + 0.5)], -1).reshape(-1, 2)
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    v00 = (ii * (n + 1) + jj).reshape(-1)
    v10 = v00 + (n + 1)
    v01 = v00 + 1
    v11 = v10 + 1
    idx = np.empty((2 * n * n, 3), np.int64)
    idx[0::2] = np.stack([v00, v10, v11], -1)
    idx[1::2] = np.stack([v00, v11, v01], -1)
    return Mesh(pos, nrm.reshape(-1, 3), idx, tan, uv)


def icosphere(level: int) -> Mesh:
    """Unit icosphere with 20 * 4^level triangles (outward normals = positions)."""
    t = (1.0 + 5 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, np.float64) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(level):
        cache = {}
        new_faces = []

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            new_faces += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = new_faces
    pos = np.array(verts)
    up = np.where(np.abs(pos[:, 2:3]) < 0.9, np.array([[0, 0, 1.0]]), np.array([[1.0, 0, 0]]))
    tan = np.cross(up, pos)
    tan /= np.linalg.norm(tan, axis=1, keepdims=True)
    tan = np.concatenate([tan, np.ones((len(pos), 1))], 1)
    return Mesh(pos, pos, np.array(faces), tan, None)


def sky_cube(size: int, sun_dir, sun_radiance: float, sun_cos: float = 0.9995) -> np.ndarray:
    """Environment cube (+X,-X,+Y,-Y,+Z,-Z) with a blue-white gradient and a baked sun disk, so a
    sky-only evaluator sees the sun (the reference's cpu path ignores the directional light)."""
    u = (np.arange(size) / max(1, size - 1)) * 2 - 1
    U, V = np.meshgrid(u, u, indexing="xy")  # rows are v, columns u
    faces = []
    for f in range(6):
        # inverse of Image2DCube::DirectionToTextureCoordinate per face
        if f == 0:
            d = np.stack([np.ones_like(U), -V, -U], -1)
        elif f == 1:
            d = np.stack([-np.ones_like(U), -V, U], -1)
        elif f == 2:
            d = np.stack([U, np.ones_like(U), V], -1)
        elif f == 3:
            d = np.stack([U, -np.ones_like(U), -V], -1)
        elif f == 4:
            d = np.stack([U, -V, np.ones_like(U)], -1)
        else:
            d = np.stack([-U, -V, -np.ones_like(U)], -1)
        d /= np.linalg.norm(d, axis=-1, keepdims=True)
        z = np.clip(d[..., 2], -1, 1)
        tz = np.clip(z * 0.5 + 0.5, 0, 1)[..., None]
        horizon = np.array([0.9, 0.9, 0.95])
        zenith = np.array([0.25, 0.45, 0.9])
        col = horizon * (1 - tz) + zenith * tz
        col = np.where(z[..., None] < 0, np.array([0.3, 0.28, 0.25]), col)
        s = np.asarray(sun_dir, np.float64)
        s = s / np.linalg.norm(s)
        cosang = d @ s
        col = col + (cosang > sun_cos)[..., None] * sun_radiance
        rgba = np.concatenate([col, np.ones(col.shape[:-1] + (1,))], -1)
        faces.append(rgba)
    return np.stack(faces).astype(np.float32)


def terrain_spheres(seed: int = 0, grid: int = 1024, num_spheres: int = 64, sphere_level: int = 5,
                    size: float = 100.0, cube_size: int = 64):
    """Returns (scene, camera_args) of the incoherent-ray stress scene."""
    rng = np.random.default_rng(seed)
    terrain = heightfield(grid, size, amplitude=6.0, seed=seed + 1)
    sphere = icosphere(sphere_level)
    materials = [Material.lambertian((0.45, 0.42, 0.35))]
    instances = [Instance(0, 0, _affine(np.eye(3), (0, 0, 0)))]
    hpos = terrain.positions.reshape(grid + 1, grid + 1, 3)
    for k in range(num_spheres):
        r = float(rng.uniform(0.8, 3.0))
        x, y = rng.uniform(-0.4 * size, 0.4 * size, 2)
        gi = int(np.clip((x / size + 0.5) * grid, 0, grid))
        gj = int(np.clip((y / size + 0.5) * grid, 0, grid))
        z = float(hpos[gi, gj, 2]) + r + float(rng.uniform(0.0, 4.0))
        kind = int(rng.integers(0, 3))
        if kind == 0:
            mat = Material.lambertian(tuple(rng.uniform(0.1, 0.9, 3)))
        elif kind == 1:
            mat = Material.metal(tuple(rng.uniform(0.5, 1.0, 3)), float(rng.uniform(0.05, 0.5)))
        else:
            mat = Material.glass((1.0, 1.0, 1.0), 1.5)
        materials.append(mat)
        lin = _rot_z(float(rng.uniform(0, 2 * np.pi))) * r
        instances.append(Instance(1, len(materials) - 1, _affine(lin, (x, y, z))))
    cube = sky_cube(cube_size, sun_dir=(0.4, 0.3, 0.85), sun_radiance=40.0)
    scene = Scene([terrain, sphere], instances, materials, Sky(SPK_SKY_CUBE, (0, 0, 0), cube), name="terrain")
    cam = dict(position=(0.0, -0.55 * size, 14.0), target=(0.0, 0.0, 0.0), world_up=(0, 0, 1),
               vfov_rad=np.deg2rad(50.0), focus_distance=50.0, aperture_radius=0.035 / 22.0 / 2.0, exposure=1.0)
    return scene, cam


def random_rays(lo, hi, n: int, seed: int = 0) -> np.ndarray:
    """(n, 6) float32 rays: origins uniform in [lo, hi], isotropic unit directions."""
    rng = np.random.default_rng(seed)
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    o = lo + (hi - lo) * rng.random((n, 3))
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    out = np.empty((n, 6), np.float32)
    out[:, :3] = o
    out[:, 3:] = d
    return out


def make_camera(cam_args: dict, width: int, height: int):
    return camera_from_look(width=width, height=height, **cam_args)


def _rotation(rng) -> np.ndarray:
    """Uniform random rotation (QR of a Gaussian matrix with a sign fix)."""
    q, r = np.linalg.qr(rng.standard_normal((3, 3)))
    q = q @ np.diag(np.sign(np.diag(r)))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def _random_material(rng):
    kind = rng.choice(3, p=[0.55, 0.3, 0.15])
    if kind == 0:
        return Material.lambertian(tuple(rng.uniform(0.05, 0.9, 3)))
    if kind == 1:
        return Material.metal(tuple(rng.uniform(0.4, 1.0, 3)), float(rng.uniform(0.05, 0.6)))
    return Material.glass((1.0, 1.0, 1.0), 1.5)


def random_training_scene(seed: int, sphere_level: int = 3, grid: int = 48):
    """A seeded procedural scene for denoiser training data: a heightfield floor, 3-12 random boxes and
    icospheres (random scale, rotation and material: Lambertian / GGX metal / glass), 1-3 emissive boxes
    of random colour and radiance, and either a sun-and-sky environment cube or a gradient sky.
    Returns (scene, camera_args) with a random look-at camera above the floor."""
    from .abi import SPK_SKY_GRADIENT
    rng = np.random.default_rng(seed)
    size = 20.0
    floor = heightfield(grid, size, amplitude=float(rng.uniform(0.0, 1.5)), seed=seed + 7)
    meshes = [floor, unit_cube(), icosphere(sphere_level)]
    materials = [Material.lambertian(tuple(rng.uniform(0.2, 0.8, 3)))]
    instances = [Instance(0, 0, _affine(np.eye(3), (0, 0, 0)))]
    for _ in range(int(rng.integers(3, 13))):
        mesh = int(rng.integers(1, 3))
        scale = rng.uniform(0.6, 3.0, 3) if mesh == 1 else np.full(3, rng.uniform(0.5, 2.0))
        lin = _rotation(rng) @ np.diag(scale)
        pos = (float(rng.uniform(-6, 6)), float(rng.uniform(-6, 6)), float(rng.uniform(0.5, 3.5)))
        materials.append(_random_material(rng))
        instances.append(Instance(mesh, len(materials) - 1, _affine(lin, pos)))
    for _ in range(int(rng.integers(1, 4))):
        col = rng.uniform(0.3, 1.0, 3)
        radiance = col / col.max() * float(rng.uniform(3.0, 20.0))
        materials.append(Material.light(tuple(radiance)))
        lin = _rotation(rng) @ np.diag(rng.uniform(0.3, 1.5, 3))
        pos = (float(rng.uniform(-7, 7)), float(rng.uniform(-7, 7)), float(rng.uniform(3.0, 8.0)))
        instances.append(Instance(1, len(materials) - 1, _affine(lin, pos)))
    if rng.random() < 0.6:
        sun = np.array([rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(0.2, 1.0)])
        sky = Sky(SPK_SKY_CUBE, (0, 0, 0), sky_cube(32, sun_dir=sun, sun_radiance=float(rng.uniform(10, 50)),
                                                     sun_cos=float(rng.uniform(0.995, 0.9995))))
    else:
        sky = Sky(SPK_SKY_GRADIENT, tuple(rng.uniform(0.1, 1.0, 3)), None)
    scene = Scene(meshes, instances, materials, sky, name=f"train{seed}")
    ang = rng.uniform(0, 2 * np.pi)
    dist = rng.uniform(10, 18)
    cam = dict(position=(float(dist * np.cos(ang)), float(dist * np.sin(ang)), float(rng.uniform(2.0, 9.0))),
               target=(float(rng.uniform(-2, 2)), float(rng.uniform(-2, 2)), float(rng.uniform(0.0, 2.0))),
               world_up=(0, 0, 1), vfov_rad=float(np.deg2rad(rng.uniform(35, 65))), focus_distance=10.0,
               aperture_radius=0.035 / 22.0 / 2.0, exposure=1.0)
    return scene, cam


def batch_scenes():
    """The three scenes of the batched workload, about 10k, 200k and 2.1M triangles, built like the stress
    scene (fBm heightfield + icospheres, Lambertian / GGX metal / glass, sun-and-sky cube)."""
    small = terrain_spheres(seed=11, grid=56, num_spheres=4, sphere_level=3, size=30.0, cube_size=32)
    mid = terrain_spheres(seed=12, grid=300, num_spheres=16, sphere_level=3, size=60.0, cube_size=32)
    big = terrain_spheres(seed=13, grid=1024, num_spheres=8, sphere_level=2, size=100.0, cube_size=64)
    return [small, mid, big]


def batch_requests(scene_cams, num: int = 32, seed: int = 0):
    """`num` render requests: scene uniform, pixel count log-uniform in [128^2, 1920 x 1080] with an aspect
    ratio in [1, 16/9], spp uniform in {1, 4, 16, 64}, depth 8 (Russian roulette after depth 3)."""
    rng = np.random.default_rng(seed)
    out = []
    lo, hi = np.log(128 * 128), np.log(1920 * 1080)
    for k in range(num):
        scene = int(rng.integers(0, len(scene_cams)))
        npix = float(np.exp(rng.uniform(lo, hi)))
        aspect = float(rng.uniform(1.0, 16.0 / 9.0))
        w = max(2, min(1920, int(round(np.sqrt(npix * aspect)))))
        h = max(2, min(1080, int(round(npix / w))))
        spp = int(rng.choice([1, 4, 16, 64]))
        out.append(dict(scene=scene, width=w, height=h, spp=spp, bounce=8, seed=k,
                        camera=make_camera(scene_cams[scene], w, h)))
    return out
