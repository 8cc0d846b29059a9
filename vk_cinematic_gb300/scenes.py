"""Seeded synthetic scenes for the benchmark configurations.

Everything here is host-side input generation: meshes in the reference's
``VertexPNT`` layout (position, normal, uv = 8 float32), object transforms,
materials, cameras and ray batches.  The same arrays are handed to the GPU
library and, in tests, to the CPU oracle, so both render identical inputs.

Meshes follow the reference's procedural generators:

* ``icosphere(level)`` - ``CreateIcosahedronMesh`` (src/mesh_generation.cpp:
  220-337): 12 unit vertices, 20 faces, each level splits every face in four,
  appending three new unit-length midpoint vertices per face (no vertex
  sharing), so level L has 12 + 60(4^L - 1)/3 vertices and 20*4^L faces.  The
  reference caps the arrays at 2048 vertices (level <= 3); this generator has
  no cap.
* ``plane()`` - ``CreatePlaneMesh`` (src/mesh_generation.cpp:1-21).

All arithmetic is float32 with one rounding per operation, in the
reference's operation order, so the level-3 sphere is bit-identical to the
reference's.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

NO_TEXTURE = 0xFFFFFFFF
SKY_TEXTURE = 0xFFFFFFFE

f32 = np.float32


def _normalize_rows(u: np.ndarray) -> np.ndarray:
    """math_lib.h:503-512: v * (1 / sqrt(x*x + y*y + z*z)) when length > FLT_EPSILON."""
    u = u.astype(np.float32)
    x, y, z = u[:, 0], u[:, 1], u[:, 2]
    ln = np.sqrt((x * x + y * y) + z * z)
    out = np.zeros_like(u)
    ok = ln > np.finfo(np.float32).eps
    inv = np.ones_like(ln)
    inv[ok] = f32(1.0) / ln[ok]
    out[ok] = u[ok] * inv[ok, None]
    return out


def _unit_vertices(p: np.ndarray) -> np.ndarray:
    """CreateUnitVertex (src/mesh_generation.cpp:206-213) for each row."""
    pos = _normalize_rows(p)
    v = np.zeros((len(pos), 8), np.float32)
    v[:, 0:3] = pos
    v[:, 3:6] = pos
    v[:, 6] = pos[:, 0]
    v[:, 7] = pos[:, 1]
    return v


def icosphere(level: int) -> tuple[np.ndarray, np.ndarray]:
    t = (f32(1.0) + np.sqrt(f32(5.0))) * f32(0.5)
    o = f32(1.0)
    z = f32(0.0)
    base = np.array(
        [[-o, t, z], [o, t, z], [-o, -t, z], [o, -t, z],
         [z, -o, t], [z, o, t], [z, -o, -t], [z, o, -t],
         [t, z, -o], [t, z, o], [-t, z, -o], [-t, z, o]], np.float32)
    verts = [_unit_vertices(base)]
    faces = np.array(
        [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
         [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
         [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
         [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    count = 12
    for _ in range(level):
        pos = np.concatenate(verts)[:, 0:3]
        n = len(faces)
        ea = faces[:, [0, 1, 2]]
        eb = faces[:, [1, 2, 0]]
        mid = (pos[ea.reshape(-1)] + pos[eb.reshape(-1)]).astype(np.float32)
        verts.append(_unit_vertices(mid))
        added = count + np.arange(3 * n, dtype=np.int64).reshape(n, 3)
        count += 3 * n
        nf = np.empty((n, 4, 3), np.int64)
        nf[:, 0] = np.stack([faces[:, 0], added[:, 0], added[:, 2]], 1)
        nf[:, 1] = np.stack([faces[:, 1], added[:, 1], added[:, 0]], 1)
        nf[:, 2] = np.stack([faces[:, 2], added[:, 2], added[:, 1]], 1)
        nf[:, 3] = added
        faces = nf.reshape(-1, 3)
    return np.ascontiguousarray(np.concatenate(verts)), faces.reshape(-1).astype(np.uint32)


def plane() -> tuple[np.ndarray, np.ndarray]:
    v = np.array(
        [[-0.5, -0.5, 0, 0, 0, 1, 0, 0],
         [0.5, -0.5, 0, 0, 0, 1, 1, 0],
         [0.5, 0.5, 0, 0, 0, 1, 1, 1],
         [-0.5, 0.5, 0, 0, 0, 1, 0, 1]], np.float32)
    return v, np.array([0, 1, 2, 2, 3, 0], np.uint32)


def quat_axis_angle(axis, angle: float) -> np.ndarray:
    """Quat(axis, angle) = (axis * sin(a/2), cos(a/2)) (math_lib.h:556-563),
    evaluated in double and rounded once so every host agrees on the bits."""
    ax = np.asarray(axis, np.float64)
    s, c = math.sin(angle * 0.5), math.cos(angle * 0.5)
    return np.array([ax[0] * s, ax[1] * s, ax[2] * s, c], np.float32)


IDENTITY_QUAT = np.array([0, 0, 0, 1], np.float32)


def material(albedo=(0, 0, 0), emission=(0, 0, 0), roughness=0.0,
             albedo_texture=NO_TEXTURE, emission_texture=NO_TEXTURE) -> dict:
    return dict(albedo=tuple(float(a) for a in albedo),
                emission=tuple(float(e) for e in emission),
                roughness=float(roughness),
                albedo_texture=int(albedo_texture),
                emission_texture=int(emission_texture))


@dataclass
class SceneObject:
    mesh: int
    material: int
    position: np.ndarray
    rotation: np.ndarray
    scale: np.ndarray


@dataclass
class Scene:
    """A renderable configuration: meshes, objects, materials, camera, options."""

    name: str
    meshes: list = field(default_factory=list)          # (vertices, indices, smooth)
    objects: list = field(default_factory=list)         # SceneObject
    materials: dict = field(default_factory=dict)       # id -> material dict
    textures: dict = field(default_factory=dict)        # id -> (H, W, 4) float32
    background: int = 0
    sky: np.ndarray | None = None                       # 13 floats or None
    width: int = 0
    height: int = 0
    camera_position: np.ndarray = None
    camera_rotation: np.ndarray = None
    film_distance: float = 0.5
    spp: int = 1
    max_bounces: int = 3
    seed: int = 0

    @property
    def triangle_count(self) -> int:
        return sum(len(self.meshes[o.mesh][1]) // 3 for o in self.objects)


def look_rotation_x(position, target) -> np.ndarray:
    """Rotation about +X that points the camera's -Z at the target (which must
    lie in the camera's YZ plane)."""
    d = np.asarray(target, np.float64) - np.asarray(position, np.float64)
    pitch = math.atan2(d[1], -d[2])
    return quat_axis_angle((1, 0, 0), pitch)


def config1_scene(width=128, height=128, spp=8, seed=1) -> Scene:
    """128x128, 8 spp, 3 bounces; icosphere level 3 (radius 1, centre (0,1,0))
    on a 20x20 ground quad at y=0; diffuse albedo 0.8 (roughness 0) under a
    constant environment of 1.0; camera (0,1,3) looking at the origin with a
    90 degree field of view (film distance 0.5)."""
    s = Scene("config1")
    sv, si = icosphere(3)
    pv, pi = plane()
    s.meshes = [(sv, si, False), (pv, pi, False)]
    s.objects = [
        SceneObject(0, 1, np.array([0, 1, 0], np.float32), IDENTITY_QUAT.copy(),
                    np.array([1, 1, 1], np.float32)),
        SceneObject(1, 1, np.array([0, 0, 0], np.float32),
                    quat_axis_angle((1, 0, 0), -math.pi * 0.5),
                    np.array([20, 20, 20], np.float32)),
    ]
    s.materials = {0: material(emission=(1, 1, 1)), 1: material(albedo=(0.8, 0.8, 0.8))}
    s.background = 0
    s.width, s.height, s.spp, s.max_bounces, s.seed = width, height, spp, 3, seed
    s.camera_position = np.array([0, 1, 3], np.float32)
    s.camera_rotation = quat_axis_angle((1, 0, 0), -math.atan(1.0 / 3.0))
    s.film_distance = 0.5
    return s


def soup(n_tris: int, seed: int = 2, half_extent: float = 0.01) -> tuple[np.ndarray, np.ndarray]:
    """Triangle soup: centres uniform in the unit cube, each vertex at the
    centre plus a uniform offset in [-h, h]^3 (random winding).  Returned in
    the VertexPNT layout with normal (0,0,1) and uv (0,0)."""
    rng = np.random.default_rng(seed)
    c = rng.random((n_tris, 1, 3), dtype=np.float32)
    off = (rng.random((n_tris, 3, 3), dtype=np.float32) * f32(2.0) - f32(1.0)) * f32(half_extent)
    p = (c + off).reshape(-1, 3).astype(np.float32)
    v = np.zeros((len(p), 8), np.float32)
    v[:, 0:3] = p
    v[:, 5] = 1.0
    return v, np.arange(len(p), dtype=np.uint32)


def soup_rays(n_rays: int, seed: int = 3, radius: float = 2.0) -> np.ndarray:
    """Rays with origins uniform on a sphere of the given radius around the
    cube centre (0.5, 0.5, 0.5), aimed at uniform points in the unit cube.
    Returns (n, 6) float32 origin + unit direction."""
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((n_rays, 3))
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    o = (0.5 + radius * g).astype(np.float32)
    tgt = rng.random((n_rays, 3)).astype(np.float32)
    d = (tgt.astype(np.float64) - o.astype(np.float64))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, d.astype(np.float32)], axis=1).astype(np.float32)


def config2_scene(n_tris=1 << 20, seed=2) -> Scene:
    """One soup object with the identity transform."""
    s = Scene("config2")
    v, i = soup(n_tris, seed)
    s.meshes = [(v, i, False)]
    s.objects = [SceneObject(0, 1, np.zeros(3, np.float32), IDENTITY_QUAT.copy(),
                             np.ones(3, np.float32))]
    s.materials = {0: material(emission=(1, 1, 1)), 1: material(albedo=(0.8, 0.8, 0.8))}
    return s


def default_sky() -> np.ndarray:
    """Vertical gradient 0.2 (straight down) to 1.0 (straight up) plus a sun
    disc of 0.5 degree radius and radiance 1e4.  Layout: bottom(3) top(3)
    sunDir(3) cosSunRadius sunRadiance(3)."""
    sd = np.array([0.35, 0.8, 0.45], np.float64)
    sd /= np.linalg.norm(sd)
    p = np.zeros(13, np.float32)
    p[0:3] = 0.2
    p[3:6] = 1.0
    p[6:9] = sd
    p[9] = math.cos(math.radians(0.5))
    p[10:13] = 1.0e4
    return p


def config3_scene(width=1920, height=1080, spp=64, max_bounces=5, n_spheres=256, level=5,
                  seed=3) -> Scene:
    """256 icospheres (level 5, 20,480 triangles each, one shared mesh) with
    log-uniform radius in [0.05, 1], centres uniform in the 20 x 5 x 20 box
    x, z in [-10, 10], y in [0, 5], over a 40 x 40 ground quad at y = 0.
    85% diffuse (albedo uniform 0.1-0.9 per channel, roughness 0), 15%
    emissive (grey radiance uniform in [1, 50], albedo 0); ground albedo 0.5.
    Sky: default_sky().  Camera at (0, 6, 18) looking at (0, 1, 0), 90 degree
    field of view across the image width."""
    rng = np.random.default_rng(seed)
    s = Scene("config3")
    sv, si = icosphere(level)
    pv, pi = plane()
    s.meshes = [(sv, si, False), (pv, pi, False)]
    s.materials = {0: material(emission_texture=SKY_TEXTURE),
                   1: material(albedo=(0.5, 0.5, 0.5))}
    s.objects = [SceneObject(1, 1, np.zeros(3, np.float32),
                             quat_axis_angle((1, 0, 0), -math.pi * 0.5),
                             np.array([40, 40, 40], np.float32))]
    radius = np.exp(rng.uniform(math.log(0.05), math.log(1.0), n_spheres))
    centre = np.stack([rng.uniform(-10, 10, n_spheres), rng.uniform(0, 5, n_spheres),
                       rng.uniform(-10, 10, n_spheres)], 1)
    emissive = rng.random(n_spheres) < 0.15
    next_id = 2
    for k in range(n_spheres):
        if emissive[k]:
            e = float(rng.uniform(1.0, 50.0))
            s.materials[next_id] = material(emission=(e, e, e))
        else:
            s.materials[next_id] = material(albedo=tuple(rng.uniform(0.1, 0.9, 3)))
        r = f32(radius[k])
        s.objects.append(SceneObject(0, next_id, centre[k].astype(np.float32),
                                     IDENTITY_QUAT.copy(), np.array([r, r, r], np.float32)))
        next_id += 1
    s.background = 0
    s.sky = default_sky()
    s.width, s.height, s.spp, s.max_bounces, s.seed = width, height, spp, max_bounces, seed
    s.camera_position = np.array([0, 6, 18], np.float32)
    s.camera_rotation = look_rotation_x(s.camera_position, (0, 1, 0))
    s.film_distance = 0.5
    return s


def config4_scenes(count=32, seed=4, max_triangles=2_000_000) -> list:
    """Config 4: `count` scenes generated like config 3 with per-scene triangle
    counts log-uniform in [1k, 2M] (sphere count and subdivision level vary),
    square images with side log-uniform in [64, 1024], spp log-uniform in
    [1, 256] and max bounces uniform in 1..8."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        tris = float(np.exp(rng.uniform(math.log(1000), math.log(max_triangles))))
        level = 5
        while level > 1 and 20 * 4 ** level > tris:
            level -= 1
        n_spheres = int(max(1, min(4096, round(tris / (20 * 4 ** level)))))
        side = int(round(math.exp(rng.uniform(math.log(64), math.log(1024)))))
        spp = int(round(math.exp(rng.uniform(math.log(1), math.log(256)))))
        bounces = int(rng.integers(1, 9))
        s = config3_scene(width=side, height=side, spp=spp, max_bounces=bounces,
                          n_spheres=n_spheres, level=level, seed=seed * 1000 + k)
        s.name = f"config4[{k}]"
        out.append(s)
    return out


# ---- compute-shader path tracer inputs ---------------------------------------------------

CPT_MATERIAL_RED, CPT_MATERIAL_BLUE, CPT_MATERIAL_CHECKERBOARD = 0, 1, 2
CPT_MATERIAL_WHITE_LIGHT = 5


def checkerboard_image(size: int = 256, grid: int = 16) -> np.ndarray:
    """CreateCheckerBoardImage (src/image.cpp:134-160): 0.18 grey with 0.04
    squares of 16 texels, RGBA32F."""
    y, x = np.mgrid[0:size, 0:size]
    odd = ((x // grid) + (y // grid)) % 2 == 1
    img = np.empty((size, size, 4), np.float32)
    img[...] = np.array([0.18, 0.18, 0.18, 1.0], np.float32)
    img[odd] = np.array([0.04, 0.04, 0.04, 1.0], np.float32)
    return img


def _trs(position, rotation_x: float, scale) -> tuple[np.ndarray, np.ndarray]:
    """Column-major model matrix T * Rx * S and its inverse, each computed in
    double and rounded once (16 floats each)."""
    c, s = math.cos(rotation_x), math.sin(rotation_x)
    t = np.eye(4)
    t[:3, 3] = position
    r = np.eye(4)
    r[1, 1], r[1, 2], r[2, 1], r[2, 2] = c, -s, s, c
    sc = np.diag([scale[0], scale[1], scale[2], 1.0])
    m = t @ r @ sc
    inv = np.linalg.inv(m)
    return (m.T.reshape(-1).astype(np.float32), inv.T.reshape(-1).astype(np.float32))


def compute_pt_scene(n_spheres: int = 16, level: int = 3, seed: int = 5,
                     light: bool = True) -> dict:
    """A scene for the compute-shader path tracer, laid out like the
    reference's disabled test geometry in src/shaders/test_compute.comp.glsl:
    a 50 x 50 checkerboard ground quad, unit red spheres on a 5-unit grid
    from (-8, 1, -8) (4 x 4 for 16 spheres; further spheres at seeded spots),
    a radius-5 white light sphere at (0, 10, 0) and one blue sphere (a
    material the shader treats as black).  Returns the buffers of
    ComputePTScene plus the camera transform."""
    rng = np.random.default_rng(seed)
    pv, pi = plane()
    sv, si = icosphere(level)
    sv8 = np.zeros((len(sv), 8), np.float32)
    sv8[:, 0:3] = sv[:, 0:3]
    sv8[:, 3:6] = sv[:, 0:3]
    sv8[:, 6:8] = sv[:, 6:8] if sv.shape[1] >= 8 else 0.0
    vertices = np.concatenate([pv, sv8]).astype(np.float32)
    indices = np.concatenate([pi, si]).astype(np.uint32)
    meshes = np.array([[len(pi), 0, 0], [len(si), len(pi), len(pv)]], np.uint32)
    models, invs, ents = [], [], []

    def add(mesh, material, position, rot_x=0.0, scale=(1.0, 1.0, 1.0)):
        m, inv = _trs(position, rot_x, scale)
        models.append(m)
        invs.append(inv)
        ents.append((mesh, material, len(models) - 1))

    add(0, CPT_MATERIAL_CHECKERBOARD, (0.0, 0.0, 0.0), -math.pi / 2, (50.0, 50.0, 50.0))
    for k in range(n_spheres):
        if k < 16:
            pos = (-8.0 + 5.0 * (k % 4), 1.0, -8.0 + 5.0 * (k // 4))
        else:
            pos = (float(rng.uniform(-20, 20)), float(rng.uniform(0.5, 4)),
                   float(rng.uniform(-20, 10)))
        add(1, CPT_MATERIAL_RED, pos)
    add(1, CPT_MATERIAL_BLUE, (6.0, 1.5, 6.0), 0.0, (1.5, 1.5, 1.5))
    if light:
        add(1, CPT_MATERIAL_WHITE_LIGHT, (0.0, 10.0, 0.0), 0.0, (5.0, 5.0, 5.0))
    # camera: position (0, 6, 22), pitched down 12 degrees; forward = R * (0, 0, -1)
    a = math.radians(-12.0)
    ca, sa = math.cos(a), math.sin(a)
    cam = np.zeros((4, 4))
    cam[0] = (1.0, 0.0, 0.0, 0.0)        # right
    cam[1] = (0.0, ca, sa, 0.0)          # up
    cam[2] = (0.0, sa, -ca, 0.0)         # forward
    cam[3] = (0.0, 6.0, 22.0, 0.0)       # position
    return dict(vertices=vertices, indices=indices, meshes=meshes,
                model=np.stack(models), inv_model=np.stack(invs),
                entities=np.array(ents, np.uint32), texture=checkerboard_image(),
                camera_transform=cam.reshape(-1).astype(np.float32))


def equirect_hdri(width: int = 2048, height: int = 1024, seed: int = 6) -> np.ndarray:
    """A seeded synthetic equirectangular HDR environment (RGBA32F, row 0 =
    top): sky gradient over a darker ground, a sun of radiance 50 (above the
    radiance clamp of 10), four bright panels and per-texel noise.  Stands in
    for the EXR HDRI the reference loads from disk (src/main.cpp:1298-1313)."""
    rng = np.random.default_rng(seed)
    v = (np.arange(height, dtype=np.float64) + 0.5) / height
    u = (np.arange(width, dtype=np.float64) + 0.5) / width
    uu, vv = np.meshgrid(u, v)
    elev = (0.5 - vv) * np.pi                      # +pi/2 at the top row
    img = np.zeros((height, width, 4), np.float64)
    sky = np.clip(elev / (np.pi / 2), 0, 1)[..., None]
    img[..., :3] = (np.array([0.9, 0.95, 1.0]) * (1 - sky) + np.array([0.25, 0.45, 0.9]) * sky)
    ground = (elev < 0)[..., None]
    img[..., :3] = np.where(ground, np.array([0.12, 0.1, 0.08]) * (1 + 0.5 * np.cos(8 * uu))[..., None],
                            img[..., :3])
    # sun at azimuth 0.3 turns, elevation 35 degrees, radius 2 degrees
    az0, el0 = 0.3 * 2 * np.pi, np.radians(35)
    az = uu * 2 * np.pi
    cosd = np.sin(elev) * np.sin(el0) + np.cos(elev) * np.cos(el0) * np.cos(az - az0)
    img[..., :3] += np.where((cosd > np.cos(np.radians(2.0)))[..., None], 50.0, 0.0)
    for k in range(4):
        u0, v0 = rng.uniform(0, 0.9), rng.uniform(0.2, 0.45)
        du, dv = rng.uniform(0.02, 0.08), rng.uniform(0.02, 0.06)
        m = (uu > u0) & (uu < u0 + du) & (vv > v0) & (vv < v0 + dv)
        img[m, :3] += rng.uniform(3, 15, 3)
    img[..., :3] *= 1.0 + 0.05 * rng.standard_normal((height, width, 1))
    img[..., 3] = 1.0
    return np.ascontiguousarray(img.astype(np.float32))
