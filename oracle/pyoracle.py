"""Python access to the CPU oracles.  TEST INFRASTRUCTURE ONLY.

Two backends expose the same interface:

* ``"port"`` - ``oracle/_build/liboracle.so``, our CPU restatement of the
  reference hot path (``oracle/sp_oracle.cpp``).  It builds on any host.
* ``"ref"``  - ``oracle/_ref/libspref.so``, the reference's own sources
  compiled in place by ``oracle/Makefile`` (x86-64 hosts where the reference
  tree is mounted).

Only tests, the smoke check and the CPU-baseline leg of ``bench.py`` may use
this module.  The product never imports it.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libspref.so")
# Where the reference checkout is looked for: $VK_CINEMATIC_REFERENCE, else
# the location it is mounted at in the build container.  Only the reference
# harness build reads it; nothing on a GPU host needs the reference.
REFERENCE_ENV = "VK_CINEMATIC_REFERENCE"
MOUNTED_REFERENCE = "/root/reference"


def reference_root() -> str:
    return os.environ.get(REFERENCE_ENV) or MOUNTED_REFERENCE

_f = ctypes.c_float
_u32 = ctypes.c_uint32
_i32 = ctypes.c_int
_vp = ctypes.c_void_p
_u64 = ctypes.c_uint64
_d = ctypes.c_double


def build_port() -> str:
    """Compile the oracle port (any host)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_LIB


def build_ref(reference: str | None = None) -> str | None:
    """Compile the reference harness when the reference tree is present on an
    x86-64 host; returns the library path or None."""
    import platform

    reference = reference or reference_root()
    if not os.path.isdir(os.path.join(reference, "src")):
        return None
    if platform.machine() not in ("x86_64", "AMD64"):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={reference}"], check=True)
    return REF_LIB


def _p(a: np.ndarray):
    return a.ctypes.data_as(_vp)


def _f32(x, n=None):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    if n is not None:
        assert a.size == n, (a.size, n)
    return a


MATERIAL_DTYPE = np.dtype(
    [
        ("albedo", np.float32, 3),
        ("albedoTexture", np.uint32),
        ("emission", np.float32, 3),
        ("emissionTexture", np.uint32),
        ("roughness", np.float32),
    ]
)
assert MATERIAL_DTYPE.itemsize == 36

PATH_VERTEX_DTYPE = np.dtype(
    [
        ("materialId", np.uint32),
        ("worldPosition", np.float32, 3),
        ("outgoingDir", np.float32, 3),
        ("incomingDir", np.float32, 3),
        ("normal", np.float32, 3),
        ("uv", np.float32, 2),
    ]
)
assert PATH_VERTEX_DTYPE.itemsize == 60

NO_TEXTURE = 0xFFFFFFFF
SKY_TEXTURE = 0xFFFFFFFE


def material(albedo=(0, 0, 0), emission=(0, 0, 0), roughness=0.0,
             albedo_texture=NO_TEXTURE, emission_texture=NO_TEXTURE):
    m = np.zeros((), dtype=MATERIAL_DTYPE)
    m["albedo"] = albedo
    m["emission"] = emission
    m["roughness"] = roughness
    m["albedoTexture"] = albedo_texture
    m["emissionTexture"] = emission_texture
    return m


class _Lib:
    _cache: dict = {}

    def __init__(self, kind: str):
        path = PORT_LIB if kind == "port" else REF_LIB
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.kind = kind
        self.prefix = "oracle_" if kind == "port" else "ref_"
        self.lib = ctypes.CDLL(path)
        for name, res in [
            ("random_unilateral", _f),
            ("random_bilateral", _f),
            ("xorshift32", _u32),
            ("aabb4", _u32),
            ("world_create", _vp),
            ("render_tiles_mt", _d),
        ]:
            fn = getattr(self.lib, self.prefix + name, None)
            if fn is not None:
                fn.restype = res
        for name in ("world_render_tiles_mt", "world_render_hashed_mt", "world_render_tile_list"):
            fn = getattr(self.lib, self.prefix + name, None)
            if fn is not None:
                fn.restype = _d
        if kind == "ref":
            self.lib.ref_world_create.argtypes = [_u64]
        self.lib.__getattr__(self.prefix + "world_create").restype = _vp
        self.lib.__getattr__(self.prefix + "world_destroy").argtypes = [_vp]

    def fn(self, name):
        return getattr(self.lib, self.prefix + name)

    @classmethod
    def get(cls, kind):
        if kind not in cls._cache:
            cls._cache[kind] = _Lib(kind)
        return cls._cache[kind]


def available(kind: str) -> bool:
    return os.path.exists(PORT_LIB if kind == "port" else REF_LIB)


class Oracle:
    """Primitive-level functions of one backend."""

    def __init__(self, kind: str = "port"):
        self.L = _Lib.get(kind)
        self.kind = kind

    # RNG -----------------------------------------------------------------
    def rng_sequence(self, seed: int, n: int, which: str):
        st = _u32(seed)
        fn = self.L.fn({"xorshift": "xorshift32", "uni": "random_unilateral",
                        "bi": "random_bilateral"}[which])
        dt = np.uint32 if which == "xorshift" else np.float32
        return np.array([fn(ctypes.byref(st)) for _ in range(n)], dtype=dt)

    def sample_seed(self, seed, x, y, s) -> int:
        name = "sample_seed_c" if self.kind == "port" else "sample_seed"
        f = self.L.fn(name)
        f.restype = _u32
        return int(f(_u32(seed), _u32(x), _u32(y), _u32(s)))

    # Camera ----------------------------------------------------------------
    def configure_camera(self, w, h, pos, rot, film):
        out = np.zeros(19, np.float32)
        self.L.fn("configure_camera")(_u32(w), _u32(h), _p(_f32(pos, 3)), _p(_f32(rot, 4)),
                                      _f(film), _p(out))
        return out

    def film_positions(self, w, h, pos, rot, film, pixels):
        px = _f32(pixels).reshape(-1, 2)
        out = np.zeros((len(px), 3), np.float32)
        self.L.fn("film_positions")(_u32(w), _u32(h), _p(_f32(pos, 3)), _p(_f32(rot, 4)),
                                    _f(film), _u32(len(px)), _p(px), _p(out))
        return out

    # Primitives ------------------------------------------------------------
    def ray_triangle(self, o, d, a, b, c):
        out = np.zeros(6, np.float32)
        self.L.fn("ray_triangle_mt")(*[_p(_f32(v, 3)) for v in (o, d, a, b, c)], _p(out))
        return out

    def aabb4(self, mins, maxs, o, invd):
        return int(self.L.fn("aabb4")(_p(_f32(mins, 12)), _p(_f32(maxs, 12)),
                                      _p(_f32(o, 3)), _p(_f32(invd, 3))))

    def hemisphere(self, state: int, normal):
        st = _u32(state)
        out = np.zeros(3, np.float32)
        self.L.fn("hemisphere")(ctypes.byref(st), _p(_f32(normal, 3)), _p(out))
        return out, st.value

    def transform_aabb(self, bmin, bmax, pos, rot, scale):
        out = np.zeros(6, np.float32)
        self.L.fn("transform_aabb")(_p(_f32(bmin, 3)), _p(_f32(bmax, 3)), _p(_f32(pos, 3)),
                                    _p(_f32(rot, 4)), _p(_f32(scale, 3)), _p(out))
        return out

    def object_matrices(self, pos, rot, scale):
        out = np.zeros(32, np.float32)
        self.L.fn("object_matrices")(_p(_f32(pos, 3)), _p(_f32(rot, 4)), _p(_f32(scale, 3)),
                                     _p(out))
        return out[:16], out[16:]

    # BVH -------------------------------------------------------------------
    def bvh_build_flat(self, mins, maxs):
        mins = _f32(mins).reshape(-1, 3)
        maxs = _f32(maxs).reshape(-1, 3)
        n = len(mins)
        cap = max(4 * n + 8, 16)
        out = np.zeros((cap, 11), np.float32)
        cnt = self.L.fn("bvh_build_flat")(_p(mins), _p(maxs), _u32(n), _p(out), _u32(cap))
        if cnt < 0:
            raise RuntimeError(f"bvh_build_flat failed: {cnt}")
        return out[:cnt].copy()

    def bvh_query(self, mins, maxs, rays, max_hits):
        mins = _f32(mins).reshape(-1, 3)
        maxs = _f32(maxs).reshape(-1, 3)
        rays = _f32(rays).reshape(-1, 6)
        out = np.zeros((len(rays), 3 + max_hits), np.uint32)
        rc = self.L.fn("bvh_query")(_p(mins), _p(maxs), _u32(len(mins)), _u32(len(rays)),
                                    _p(rays), _u32(max_hits), _p(out))
        if rc != 0:
            raise RuntimeError(f"bvh_query failed: {rc}")
        return out


class World:
    """A scene + material system held by one backend."""

    def __init__(self, kind: str = "port", arena_bytes: int = 1 << 30):
        self.L = _Lib.get(kind)
        self.kind = kind
        if kind == "ref":
            self.h = self.L.fn("world_create")(_u64(arena_bytes))
        else:
            self.h = self.L.fn("world_create")()
        self.h = _vp(self.h)
        self.spp = 1
        self.max_bounces = 3

    def close(self):
        if self.h:
            self.L.fn("world_destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_mesh(self, vertices, indices, smooth=False) -> int:
        v = _f32(vertices).reshape(-1, 8)
        i = np.ascontiguousarray(indices, dtype=np.uint32)
        rc = self.L.fn("world_add_mesh")(self.h, _p(v), _u32(len(v)), _p(i), _u32(len(i)),
                                         _i32(int(smooth)))
        if rc < 0:
            raise RuntimeError(f"add_mesh failed {rc}")
        return rc

    def add_object(self, mesh, material_id, pos, rot, scale):
        rc = self.L.fn("world_add_object")(self.h, _i32(mesh), _u32(material_id),
                                           _p(_f32(pos, 3)), _p(_f32(rot, 4)),
                                           _p(_f32(scale, 3)))
        if rc != 0:
            raise RuntimeError(f"add_object failed {rc}")

    def build(self):
        rc = self.L.fn("world_build")(self.h)
        if rc != 0:
            raise RuntimeError(f"build failed {rc}")

    def register_material(self, mat, mid: int) -> int:
        m = np.ascontiguousarray(np.asarray(mat, dtype=MATERIAL_DTYPE))
        return self.L.fn("world_register_material")(self.h, _p(m), _u32(mid))

    def register_texture(self, rgba, tid: int) -> int:
        a = _f32(rgba)
        h, w = a.shape[0], a.shape[1]
        return self.L.fn("world_register_texture")(self.h, _p(a), _u32(w), _u32(h), _u32(tid))

    def set_background(self, mid: int):
        self.L.fn("world_set_background")(self.h, _u32(mid))

    def set_sky(self, params):
        assert self.kind == "port", "the analytic sky is an extension of the port"
        self.L.fn("world_set_sky")(self.h, _p(_f32(params, 13)))

    def set_options(self, spp=1, max_bounces=3, radiance_clamp=10.0, max_broadphase=32,
                    max_midphase=128):
        self.spp = spp
        self.max_bounces = max_bounces
        if self.kind != "port":
            assert max_bounces == 3, "the reference has 3 bounces"
            return
        opt = (_u32 * 5)()
        buf = np.array([spp, max_bounces, 0, max_broadphase, max_midphase], np.uint32)
        buf[2] = np.float32(radiance_clamp).view(np.uint32)
        ctypes.memmove(opt, buf.ctypes.data, 20)
        self.L.fn("world_set_options")(self.h, ctypes.byref(opt))

    def intersect(self, rays):
        rays = _f32(rays).reshape(-1, 6)
        out = np.zeros((len(rays), 6), np.float32)
        mat = np.zeros(len(rays), np.uint32)
        metrics = np.zeros(12, np.uint64)
        rc = self.L.fn("world_intersect")(self.h, _u32(len(rays)), _p(rays), _p(out), _p(mat),
                                          _p(metrics))
        if rc != 0:
            raise RuntimeError(f"intersect failed {rc}")
        return out, mat, metrics

    def closest(self, rays, ties=False):
        """(t, object, triangle) per ray through the reference's scene query;
        with ties=True also a bool array flagging rays whose best t is an
        exact tie between two candidates."""
        assert self.kind == "port"
        rays = _f32(rays).reshape(-1, 6)
        t = np.zeros(len(rays), np.float32)
        obj = np.zeros(len(rays), np.int32)
        tri = np.zeros(len(rays), np.int32)
        tied = np.zeros(len(rays), np.int32)
        rc = self.L.fn("world_closest")(self.h, _u32(len(rays)), _p(rays), _p(t), _p(obj),
                                        _p(tri), _p(tied))
        if rc != 0:
            raise RuntimeError(f"closest failed {rc}")
        return (t, obj, tri, tied.astype(bool)) if ties else (t, obj, tri)

    def set_build_bvh(self, on: bool):
        assert self.kind == "port"
        self.L.fn("world_set_build_bvh")(self.h, _i32(int(on)))

    def set_watertight(self, on: bool):
        """Brute-force queries (closest_brute) use the watertight triangle test."""
        assert self.kind == "port"
        self.L.fn("world_set_watertight")(self.h, _i32(int(on)))

    def closest_brute(self, rays, threads=None, ties=False):
        """Brute-force closest hit over every triangle; ties as in closest()."""
        assert self.kind == "port"
        rays = _f32(rays).reshape(-1, 6)
        t = np.zeros(len(rays), np.float32)
        obj = np.zeros(len(rays), np.int32)
        tri = np.zeros(len(rays), np.int32)
        tied = np.zeros(len(rays), np.int32)
        threads = threads or os.cpu_count() or 1
        self.L.fn("world_closest_brute")(self.h, _u32(len(rays)), _p(rays), _u32(threads), _p(t),
                                         _p(obj), _p(tri), _p(tied))
        return (t, obj, tri, tied.astype(bool)) if ties else (t, obj, tri)

    def path_trace_tile(self, width, height, cam_pos, cam_rot, film, tile, rng_state, pixels=None):
        if pixels is None:
            pixels = np.zeros((height, width, 4), np.float32)
        st = _u32(rng_state)
        metrics = np.zeros(12, np.uint64)
        t = np.ascontiguousarray(tile, dtype=np.uint32)
        if self.kind == "ref":
            rc = self.L.fn("world_path_trace_tile")(
                self.h, _u32(width), _u32(height), _p(_f32(cam_pos, 3)), _p(_f32(cam_rot, 4)),
                _f(film), _p(t), ctypes.byref(st), _u32(self.spp), _p(pixels), _p(metrics))
        else:
            rc = self.L.fn("world_path_trace_tile")(
                self.h, _u32(width), _u32(height), _p(_f32(cam_pos, 3)), _p(_f32(cam_rot, 4)),
                _f(film), _p(t), ctypes.byref(st), _p(pixels), _p(metrics))
        if rc != 0:
            raise RuntimeError(f"path_trace_tile failed {rc}")
        return pixels, st.value, metrics

    def path_trace_hashed(self, width, height, cam_pos, cam_rot, film, seed, region=None,
                          nan_policy=0, per_sample=False):
        if region is None:
            region = (0, 0, width, height)
        reg = np.ascontiguousarray(region, dtype=np.uint32)
        out = np.zeros((height, width, 4), np.float32)
        npx = int((reg[2] - reg[0]) * (reg[3] - reg[1]))
        ps = np.zeros((npx, self.spp, 3), np.float32) if per_sample else None
        nans = _u32(0)
        metrics = np.zeros(12, np.uint64)
        args = [self.h, _u32(width), _u32(height), _p(_f32(cam_pos, 3)), _p(_f32(cam_rot, 4)),
                _f(film), _p(reg)]
        if self.kind == "ref":
            args += [_u32(self.spp)]
        args += [_u32(seed), _i32(nan_policy), _p(out), ctypes.byref(nans), _p(metrics),
                 _p(ps) if ps is not None else None]
        rc = self.L.fn("world_path_trace_hashed")(*args)
        if rc != 0:
            raise RuntimeError(f"path_trace_hashed failed {rc}")
        return out, nans.value, metrics, ps

    def radiance_for_path(self, vertices):
        v = np.ascontiguousarray(np.asarray(vertices, dtype=PATH_VERTEX_DTYPE))
        out = np.zeros(3, np.float32)
        self.L.fn("world_radiance_for_path")(self.h, _p(v), _u32(v.size), _p(out))
        return out

    def render_tiles_mt(self, width, height, cam_pos, cam_rot, film, tile_size, first_tile,
                        tile_count, threads, pixels=None):
        assert self.kind == "port"
        if pixels is None:
            pixels = np.zeros((height, width, 4), np.float32)
        metrics = np.zeros(12, np.uint64)
        dt = self.L.fn("world_render_tiles_mt")(
            self.h, _u32(width), _u32(height), _p(_f32(cam_pos, 3)), _p(_f32(cam_rot, 4)),
            _f(film), _u32(tile_size), _u32(first_tile), _u32(tile_count), _u32(threads),
            _p(pixels), _p(metrics))
        if dt < 0:
            raise RuntimeError("render_tiles_mt: a capacity of the reference overflowed")
        return dt, pixels, metrics

    def render_tile_list(self, width, height, cam_pos, cam_rot, film, tile_size, tile_ids,
                         threads, pixels=None):
        """The reference's tile mode over an explicit list of tile ids (row-major
        tile order), `threads` workers popping tiles from a shared counter."""
        assert self.kind == "port"
        if pixels is None:
            pixels = np.zeros((height, width, 4), np.float32)
        ids = np.ascontiguousarray(tile_ids, dtype=np.uint32)
        metrics = np.zeros(12, np.uint64)
        dt = self.L.fn("world_render_tile_list")(
            self.h, _u32(width), _u32(height), _p(_f32(cam_pos, 3)), _p(_f32(cam_rot, 4)),
            _f(film), _u32(tile_size), _p(ids), _u32(len(ids)), _u32(threads), _p(pixels),
            _p(metrics))
        if dt < 0:
            raise RuntimeError("render_tile_list: a capacity of the reference overflowed")
        return dt, pixels, metrics

    def render_hashed_mt(self, width, height, cam_pos, cam_rot, film, seed, row_begin, row_end,
                         threads, out=None):
        assert self.kind == "port"
        if out is None:
            out = np.zeros((height, width, 4), np.float32)
        metrics = np.zeros(12, np.uint64)
        dt = self.L.fn("world_render_hashed_mt")(
            self.h, _u32(width), _u32(height), _p(_f32(cam_pos, 3)), _p(_f32(cam_rot, 4)),
            _f(film), _u32(seed), _u32(row_begin), _u32(row_end), _u32(threads), _p(out),
            _p(metrics))
        if dt < 0:
            raise RuntimeError("render_hashed_mt: a capacity of the reference overflowed")
        return dt, out, metrics


def compute_pt_tiles(scene: dict, width: int, height: int, tile: int, film_distance: float,
                     tiles, image=None):
    """The compute-shader path tracer's restatement (oracle_compute_pt_tiles)
    over the listed tiles.  `scene` holds the arrays of
    vk_cinematic_gb300.scenes.compute_pt_scene.  Returns (image, counters)
    with counters = [rays, hits, triangle tests]."""
    L = _Lib.get("port").lib
    if image is None:
        image = np.zeros((height, width, 4), np.float32)
    v = np.ascontiguousarray(scene["vertices"], np.float32)
    i = np.ascontiguousarray(scene["indices"], np.uint32)
    m = np.ascontiguousarray(scene["meshes"], np.uint32)
    mm = np.ascontiguousarray(scene["model"], np.float32)
    im = np.ascontiguousarray(scene["inv_model"], np.float32)
    e = np.ascontiguousarray(scene["entities"], np.uint32)
    tex = scene.get("texture")
    tex = None if tex is None else np.ascontiguousarray(tex, np.float32)
    ct = np.ascontiguousarray(scene["camera_transform"], np.float32)
    tl = np.ascontiguousarray(tiles, np.uint32).reshape(-1)
    counters = np.zeros(3, np.uint64)
    L.oracle_compute_pt_tiles(
        _p(v), _p(i), _p(m), _p(mm), _p(im), _p(e), _u32(len(e)),
        _p(tex) if tex is not None else None, _u32(0 if tex is None else tex.shape[1]),
        _u32(0 if tex is None else tex.shape[0]), _p(ct), _u32(width), _u32(height), _u32(tile),
        _u32(tile), _f(film_distance), _p(tl), _u32(len(tl)), _p(image), _p(counters))
    return image, counters


def create_cube_map(equirect: np.ndarray, width: int, height: int, kind: str = "port"):
    """CreateCubeMap (src/cubemap.cpp:235-291): (6, height, width, 4) float32."""
    lib = _Lib.get(kind).lib
    eq = np.ascontiguousarray(equirect, np.float32)
    out = np.zeros((6, height, width, 4), np.float32)
    fn = lib.oracle_create_cube_map if kind == "port" else lib.ref_create_cube_map
    rc = fn(_p(eq), _u32(eq.shape[1]), _u32(eq.shape[0]), _u32(width), _u32(height), _p(out))
    if kind == "ref" and rc != 0:
        raise RuntimeError("the reference asserted in CreateCubeMap")
    return out


def create_irradiance_cube_map(equirect: np.ndarray, width: int, height: int, spp: int = 32,
                               mode: int = 0, kind: str = "port"):
    """CreateIrradianceCubeMap (src/cubemap.cpp:106-233); mode 0 = uniform
    (phi, theta) grid, 1 = random offsets."""
    lib = _Lib.get(kind).lib
    eq = np.ascontiguousarray(equirect, np.float32)
    out = np.zeros((6, height, width, 4), np.float32)
    if kind == "port":
        lib.oracle_create_irradiance_cube_map(_p(eq), _u32(eq.shape[1]), _u32(eq.shape[0]),
                                              _u32(width), _u32(height), _u32(spp), _u32(mode),
                                              _p(out))
    else:
        rc = lib.ref_create_irradiance_cube_map(_p(eq), _u32(eq.shape[1]), _u32(eq.shape[0]),
                                                _u32(width), _u32(height), _u32(spp),
                                                _u32(mode), _p(out))
        if rc != 0:
            raise RuntimeError("the reference asserted in CreateIrradianceCubeMap")
    return out


def ray_triangle_watertight(o, d, a, b, c):
    """Watertight test of the port: (t, u, v); t = -1 on a miss."""
    out = np.zeros(3, np.float32)
    _Lib.get("port").lib.oracle_ray_triangle_watertight(
        _p(_f32(o, 3)), _p(_f32(d, 3)), _p(_f32(a, 3)), _p(_f32(b, 3)), _p(_f32(c, 3)), _p(out))
    return out
