"""ctypes binding of libgbsp.so (include/gbsp.h) for tests and the benchmark.

The library is the product; this module only marshals arguments.  It never
falls back to anything: if the shared library is missing or the device
call fails, it raises.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_vp = ctypes.c_void_p
_u32 = ctypes.c_uint32
_i32 = ctypes.c_int32
_f32 = ctypes.c_float
_u64 = ctypes.c_uint64

GBSP_NO_TEXTURE = 0xFFFFFFFF
GBSP_SKY_TEXTURE = 0xFFFFFFFE
RNG_HASH_PER_SAMPLE = 0
RNG_TILE_SEQUENTIAL = 1
NAN_ZERO = 0
NAN_PROPAGATE = 1
METRIC_COUNT = 16
METRIC_NAMES = [
    "elapsed_ns", "paths_traced", "rays_traced", "ray_hit_count", "ray_miss_count",
    "intersect_scene_ns", "broadphase_node_visits", "shade_ns", "midphase_node_visits",
    "triangle_tests", "midphase_box_tests", "mesh_tests_performed", "nan_samples",
    "trace_launches", "kernel_launches",
]

# Every symbol include/gbsp.h declares.
EXPORTS = [
    "gbsp_runtime_create", "gbsp_runtime_destroy", "gbsp_runtime_synchronize",
    "gbsp_runtime_stream", "gbsp_last_error_string", "gbsp_version", "gbsp_options_default",
    "gbsp_configure_camera", "gbsp_calculate_film_positions", "gbsp_scene_create",
    "gbsp_scene_destroy", "gbsp_create_mesh", "gbsp_add_object_to_scene", "gbsp_clear_objects",
    "gbsp_build_scene_broadphase", "gbsp_scene_info", "gbsp_ray_intersect_scene",
    "gbsp_intersect_closest_device", "gbsp_material_system_create",
    "gbsp_material_system_destroy", "gbsp_register_material", "gbsp_register_texture",
    "gbsp_set_background_material", "gbsp_set_procedural_sky", "gbsp_path_trace_tile",
    "gbsp_path_trace_frame", "gbsp_frame_device_pointer", "gbsp_icosphere", "gbsp_plane_mesh",
    "gbsp_sample_seed", "gbsp_path_trace_tile_noalloc", "gbsp_batch_create",
    "gbsp_batch_destroy", "gbsp_batch_set_config", "gbsp_batch_get_config",
    "gbsp_batch_autotune", "gbsp_batch_launch", "gbsp_frame_aov_device_pointer",
    "gbsp_frame_copy_region", "gbsp_dn_features", "gbsp_dn_conv3x3_forward",
    "gbsp_dn_flip_transpose", "gbsp_dn_relu_backward", "gbsp_dn_conv3x3_weight_grad",
    "gbsp_dn_conv3x3_weight_grad_tc", "gbsp_dn_conv3x3_filter_tc",
    "gbsp_dn_tc_rate",
    "gbsp_dn_filter", "gbsp_dn_relmse_backward", "gbsp_dn_adam", "gbsp_tonemap",
    "gbsp_cpt_scene_create", "gbsp_cpt_scene_destroy", "gbsp_cpt_render_tiles",
    "gbsp_create_cube_map", "gbsp_create_irradiance_cube_map", "gbsp_xorshift32_jump",
    "gbsp_dn_conv3x3_forward_tc", "gbsp_dn_status", "gbsp_scene_set_intersection",
    "gbsp_dn_tile_fallback", "gbsp_scene_set_node_width", "gbsp_scene_node_width",
    "gbsp_batch_set_node_widths", "gbsp_batch_get_node_widths", "gbsp_path_trace_tile_list",
    "gbsp_dn_tile_check", "gbsp_dn_tile_merge", "gbsp_dn_conv3x3_weight_grad_tcgen05",
    "gbsp_path_trace_tile_list_spp", "gbsp_path_trace_tile_split",
]


class Options(ctypes.Structure):
    _fields_ = [("spp", _u32), ("max_bounces", _u32), ("seed", _u32), ("rng_mode", _u32),
                ("nan_policy", _u32), ("radiance_clamp", _f32), ("wave_paths", _u32),
                ("flags", _u32)]


FLAG_STAGE_TIMING = 1
FLAG_AOV = 2
FLAG_TRACE_PER_LANE = 4
FLAG_TRACE_PER_WARP = 8
FLAG_SORT_DIRECTIONS = 16
ISECT_REFERENCE_MT = 0
ISECT_WATERTIGHT = 1


class ImagePlane(ctypes.Structure):
    _fields_ = [("pixels", _vp), ("width", _u32), ("height", _u32)]


class Camera(ctypes.Structure):
    _fields_ = [("right", _f32 * 3), ("up", _f32 * 3), ("forward", _f32 * 3),
                ("position", _f32 * 3), ("filmCenter", _f32 * 3),
                ("imagePlane", ctypes.POINTER(ImagePlane)), ("halfPixelWidth", _f32),
                ("halfPixelHeight", _f32), ("halfFilmWidth", _f32), ("halfFilmHeight", _f32)]


class Context(ctypes.Structure):
    _fields_ = [("camera", ctypes.POINTER(Camera)), ("scene", _vp), ("materialSystem", _vp),
                ("runtime", _vp), ("options", ctypes.POINTER(Options))]


class Tile(ctypes.Structure):
    _fields_ = [("minX", _u32), ("minY", _u32), ("maxX", _u32), ("maxY", _u32)]


class Metrics(ctypes.Structure):
    _fields_ = [("values", _u64 * METRIC_COUNT)]

    def as_dict(self):
        return {n: int(self.values[i]) for i, n in enumerate(METRIC_NAMES)}


class Material(ctypes.Structure):
    _fields_ = [("albedo", _f32 * 3), ("albedoTexture", _u32), ("emission", _f32 * 3),
                ("emissionTexture", _u32), ("roughness", _f32)]


assert ctypes.sizeof(Material) == 36


class GbspError(RuntimeError):
    pass


_LIB = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libgbsp.so (building it in-tree if needed)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if build_if_missing:
        _build.build()
    if not os.path.exists(path):
        raise GbspError(f"{path} is missing: run vk_cinematic_gb300.build first")
    lib = ctypes.CDLL(path)
    lib.gbsp_last_error_string.restype = ctypes.c_char_p
    lib.gbsp_runtime_stream.restype = _vp
    lib.gbsp_frame_device_pointer.restype = _vp
    lib.gbsp_frame_aov_device_pointer.restype = _vp
    lib.gbsp_sample_seed.restype = _u32
    lib.gbsp_calculate_film_positions.restype = _u32
    lib.gbsp_xorshift32_jump.restype = _u32
    lib.gbsp_xorshift32_jump.argtypes = [_u32, ctypes.c_uint64]
    lib.gbsp_scene_node_width.restype = _u32
    for name in EXPORTS:
        getattr(lib, name)  # raises if a declared symbol is not exported
    _LIB = lib
    return lib


def _check(rc: int):
    if rc != 0:
        msg = _LIB.gbsp_last_error_string().decode(errors="replace")
        raise GbspError(f"gbsp status {rc}: {msg}")


def _p(a: np.ndarray):
    return a.ctypes.data_as(_vp)


def default_options(**kw) -> Options:
    o = Options()
    load().gbsp_options_default(ctypes.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class Runtime:
    def __init__(self, device: int = 0, stream: int | None = None):
        self.L = load()
        h = _vp()
        _check(self.L.gbsp_runtime_create(_i32(device), _vp(stream) if stream else None,
                                          ctypes.byref(h)))
        self.h = h

    @property
    def stream(self) -> int:
        return self.L.gbsp_runtime_stream(self.h)

    def synchronize(self):
        _check(self.L.gbsp_runtime_synchronize(self.h))

    def close(self):
        if self.h:
            self.L.gbsp_runtime_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MaterialSystem:
    def __init__(self, rt: Runtime):
        self.L, self.rt = rt.L, rt
        h = _vp()
        _check(self.L.gbsp_material_system_create(rt.h, ctypes.byref(h)))
        self.h = h

    def register(self, mid: int, albedo=(0, 0, 0), emission=(0, 0, 0), roughness=0.0,
                 albedo_texture=GBSP_NO_TEXTURE, emission_texture=GBSP_NO_TEXTURE):
        m = Material()
        m.albedo[:] = [float(a) for a in albedo]
        m.emission[:] = [float(e) for e in emission]
        m.roughness = float(roughness)
        m.albedoTexture = int(albedo_texture)
        m.emissionTexture = int(emission_texture)
        _check(self.L.gbsp_register_material(self.h, ctypes.byref(m), _u32(mid)))

    def register_texture(self, tid: int, rgba: np.ndarray):
        a = np.ascontiguousarray(rgba, dtype=np.float32)
        _check(self.L.gbsp_register_texture(self.h, _p(a), _u32(a.shape[1]), _u32(a.shape[0]),
                                            _u32(tid)))

    def set_background(self, mid: int):
        _check(self.L.gbsp_set_background_material(self.h, _u32(mid)))

    def set_sky(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        assert p.size == 13
        _check(self.L.gbsp_set_procedural_sky(self.h, _p(p)))

    def close(self):
        if self.h:
            self.L.gbsp_material_system_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Scene:
    def __init__(self, rt: Runtime):
        self.L, self.rt = rt.L, rt
        h = _vp()
        _check(self.L.gbsp_scene_create(rt.h, ctypes.byref(h)))
        self.h = h
        # add_object's transform (position 3, rotation 4, scale 3 floats) goes
        # through this buffer, whose three pointers are made once: converting
        # three arrays per call cost more than the call itself
        self._xf = np.empty(10, np.float32)
        base = self._xf.ctypes.data
        self._xf_ptrs = (_vp(base), _vp(base + 12), _vp(base + 28))

    def set_intersection(self, mode: int):
        """ISECT_REFERENCE_MT (default) or ISECT_WATERTIGHT."""
        _check(self.L.gbsp_scene_set_intersection(self.h, _u32(mode)))

    def set_node_width(self, width: int):
        """BVH node width of this scene's queries and renders: 8 (default) or 4."""
        _check(self.L.gbsp_scene_set_node_width(self.h, _u32(width)))

    @property
    def node_width(self) -> int:
        return int(self.L.gbsp_scene_node_width(self.h))

    def create_mesh(self, vertices: np.ndarray, indices: np.ndarray, smooth=False) -> int:
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 8)
        i = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1)
        out = _u32()
        _check(self.L.gbsp_create_mesh(self.h, _p(v), _u32(len(v)), _p(i), _u32(len(i)),
                                       _i32(int(smooth)), ctypes.byref(out)))
        return out.value

    def add_object(self, mesh, material, position, rotation, scale):
        """sp_AddObjectToScene.  The library copies the transform during the
        call; like the scene itself, one Scene takes one call at a time."""
        xf = self._xf
        xf[0:3] = position
        xf[3:7] = rotation
        xf[7:10] = scale
        _check(self.L.gbsp_add_object_to_scene(self.h, _u32(mesh), _u32(material),
                                               *self._xf_ptrs))

    def clear_objects(self):
        _check(self.L.gbsp_clear_objects(self.h))

    def build_broadphase(self):
        _check(self.L.gbsp_build_scene_broadphase(self.h))

    def info(self):
        o, t, n, d = _u32(), _u64(), _u32(), _u32()
        _check(self.L.gbsp_scene_info(self.h, ctypes.byref(o), ctypes.byref(t), ctypes.byref(n),
                                      ctypes.byref(d)))
        return dict(objects=o.value, triangles=t.value, mesh_nodes=n.value, max_depth=d.value)

    def intersect(self, rays: np.ndarray):
        """sp_RayIntersectScene on a host batch: returns (t,n,u,v) rows, material ids, metrics."""
        r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        out = np.zeros((len(r), 6), np.float32)
        mat = np.zeros(len(r), np.uint32)
        m = Metrics()
        _check(self.L.gbsp_ray_intersect_scene(self.h, _u32(len(r)), _p(r), _p(out), _p(mat),
                                               ctypes.byref(m)))
        return out, mat, m

    def intersect_closest_device(self, count: int, rays_ptr: int, t_ptr: int, tri_ptr: int,
                                 obj_ptr: int = 0):
        _check(self.L.gbsp_intersect_closest_device(self.h, _u32(count), _vp(rays_ptr),
                                                    _vp(t_ptr), _vp(tri_ptr),
                                                    _vp(obj_ptr) if obj_ptr else None))

    def close(self):
        if self.h:
            self.L.gbsp_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Renderer:
    """Camera + image plane + context for one scene and material system."""

    def __init__(self, rt: Runtime, scene: Scene, ms: MaterialSystem, width: int, height: int,
                 position, rotation, film_distance: float, options: Options | None = None):
        self.L, self.rt, self.scene, self.ms = rt.L, rt, scene, ms
        self.plane = ImagePlane(None, width, height)
        self.camera = Camera()
        p = np.ascontiguousarray(position, dtype=np.float32)
        r = np.ascontiguousarray(rotation, dtype=np.float32)
        _check(self.L.gbsp_configure_camera(ctypes.byref(self.camera), ctypes.byref(self.plane),
                                            _p(p), _p(r), _f32(film_distance)))
        self.options = options or default_options()
        self.ctx = Context(ctypes.pointer(self.camera), scene.h, ms.h, rt.h,
                           ctypes.pointer(self.options))
        self.width, self.height = width, height

    def set_host_pixels(self, array: np.ndarray | None):
        if array is None:
            self.plane.pixels = None
        else:
            assert array.dtype == np.float32 and array.flags["C_CONTIGUOUS"]
            assert array.size == self.width * self.height * 4
            self.plane.pixels = array.ctypes.data
        self._pixels = array

    def frame(self, metrics: bool = True, pixels: np.ndarray | None = None):
        out = pixels if pixels is not None else np.zeros((self.height, self.width, 4), np.float32)
        self.set_host_pixels(out)
        m = Metrics() if metrics else None
        _check(self.L.gbsp_path_trace_frame(ctypes.byref(self.ctx),
                                            ctypes.byref(m) if m is not None else None))
        self.set_host_pixels(None)
        return out, m

    def frame_async(self):
        """Device-only frame (no host copy, no metrics, no synchronisation)."""
        self.set_host_pixels(None)
        _check(self.L.gbsp_path_trace_frame(ctypes.byref(self.ctx), None))

    def frame_device(self, metrics: bool = True):
        """Device-only frame (the image stays in device memory); with metrics
        the call waits for the frame and returns its counters."""
        self.set_host_pixels(None)
        m = Metrics() if metrics else None
        _check(self.L.gbsp_path_trace_frame(ctypes.byref(self.ctx),
                                            ctypes.byref(m) if m is not None else None))
        return m

    def tile_device(self, tile, rng_state: int = 0):
        """Tile render kept in device memory (frame buffer of the runtime)."""
        self.set_host_pixels(None)
        rng = _u32(rng_state)
        m = Metrics()
        t = Tile(*[int(v) for v in tile])
        _check(self.L.gbsp_path_trace_tile(ctypes.byref(self.ctx), t, ctypes.byref(rng),
                                           ctypes.byref(m)))
        return m

    def tile_split_device(self, tile, first_spp: int, image2_ptr: int, metrics: bool = False):
        """gbsp_path_trace_tile_split: options.spp samples per pixel in one pass;
        the mean of the first `first_spp` lands in the runtime's frame buffer
        (and G-buffers), the mean of the rest in the device image at
        image2_ptr (width x height RGBA32F).  Returns the metrics when asked."""
        self.set_host_pixels(None)
        m = Metrics() if metrics else None
        t = Tile(*[int(v) for v in tile])
        _check(self.L.gbsp_path_trace_tile_split(ctypes.byref(self.ctx), t, _u32(first_spp),
                                                 _vp(image2_ptr),
                                                 ctypes.byref(m) if m is not None else None))
        return m

    def tile(self, tile, rng_state: int = 0, pixels: np.ndarray | None = None):
        out = pixels if pixels is not None else np.zeros((self.height, self.width, 4), np.float32)
        self.set_host_pixels(out)
        rng = _u32(rng_state)
        m = Metrics()
        t = Tile(*[int(v) for v in tile])
        _check(self.L.gbsp_path_trace_tile(ctypes.byref(self.ctx), t, ctypes.byref(rng),
                                           ctypes.byref(m)))
        self.set_host_pixels(None)
        return out, rng.value, m

    def tile_list_device(self, tiles, metrics: bool = False):
        """Renders the listed (minX, minY, maxX, maxY) tiles in one pass into the
        runtime's frame buffer (device); returns the metrics when asked."""
        self.set_host_pixels(None)
        # gbsp_tile is four uint32 (minX, minY, maxX, maxY): an (n, 4) array is its layout
        tl = np.ascontiguousarray(tiles, dtype=np.uint32).reshape(-1, 4)
        m = Metrics() if metrics else None
        _check(self.L.gbsp_path_trace_tile_list(ctypes.byref(self.ctx), _p(tl), _u32(len(tl)),
                                                ctypes.byref(m) if m is not None else None))
        return m

    def tile_list_spp_device(self, tiles, spp, metrics: bool = False):
        """gbsp_path_trace_tile_list_spp: the listed (minX, minY, maxX, maxY)
        tiles, tile i at spp[i] samples per pixel, in one pass into the
        runtime's frame buffer (device); returns the metrics when asked."""
        self.set_host_pixels(None)
        # gbsp_tile is four uint32 (minX, minY, maxX, maxY): an (n, 4) array is its layout
        tl = np.ascontiguousarray(tiles, dtype=np.uint32).reshape(-1, 4)
        sp = np.ascontiguousarray(spp, dtype=np.uint32).reshape(-1)
        if len(sp) != len(tl):
            raise ValueError("one spp per tile")
        m = Metrics() if metrics else None
        _check(self.L.gbsp_path_trace_tile_list_spp(ctypes.byref(self.ctx), _p(tl), _p(sp),
                                                    _u32(len(tl)),
                                                    ctypes.byref(m) if m is not None else None))
        return m

    def frame_device_pointer(self) -> int:
        return self.L.gbsp_frame_device_pointer(self.rt.h)

    def aov_device_pointer(self) -> int:
        return self.L.gbsp_frame_aov_device_pointer(self.rt.h)

    def copy_region(self, x0, y0, w, h, dst_radiance_ptr: int, dst_aov_ptr: int = 0):
        _check(self.L.gbsp_frame_copy_region(self.rt.h, _u32(x0), _u32(y0), _u32(w), _u32(h),
                                             _vp(dst_radiance_ptr),
                                             _vp(dst_aov_ptr) if dst_aov_ptr else None))


def film_positions(camera: Camera, pixels: np.ndarray) -> np.ndarray:
    px = np.ascontiguousarray(pixels, dtype=np.float32).reshape(-1, 2)
    out = np.zeros((len(px), 3), np.float32)
    load().gbsp_calculate_film_positions(ctypes.byref(camera), _p(out), _p(px), _u32(len(px)))
    return out


def sample_seed(seed, x, y, s) -> int:
    return int(load().gbsp_sample_seed(_u32(seed), _u32(x), _u32(y), _u32(s)))


def icosphere(level: int):
    L = load()
    nv, ni = _u32(), _u32()
    _check(L.gbsp_icosphere(_u32(level), None, None, ctypes.byref(nv), ctypes.byref(ni)))
    v = np.zeros((nv.value, 8), np.float32)
    i = np.zeros(ni.value, np.uint32)
    _check(L.gbsp_icosphere(_u32(level), _p(v), _p(i), ctypes.byref(nv), ctypes.byref(ni)))
    return v, i


def plane_mesh():
    v = np.zeros((4, 8), np.float32)
    i = np.zeros(6, np.uint32)
    _check(load().gbsp_plane_mesh(_p(v), _p(i)))
    return v, i


def upload_scene(rt: Runtime, s, options: Options | None = None):
    """Builds device objects for a vk_cinematic_gb300.scenes.Scene."""
    scene = Scene(rt)
    meshes = [scene.create_mesh(v, i, sm) for (v, i, sm) in s.meshes]
    for o in s.objects:
        scene.add_object(meshes[o.mesh], o.material, o.position, o.rotation, o.scale)
    scene.build_broadphase()
    ms = MaterialSystem(rt)
    for tid, tex in s.textures.items():
        ms.register_texture(tid, tex)
    for mid, m in s.materials.items():
        ms.register(mid, **m)
    ms.set_background(s.background)
    if s.sky is not None:
        ms.set_sky(s.sky)
    opt = options or default_options(spp=s.spp, max_bounces=s.max_bounces, seed=s.seed)
    rend = Renderer(rt, scene, ms, s.width, s.height, s.camera_position, s.camera_rotation,
                    s.film_distance, opt) if s.width else None
    return scene, ms, rend


class BatchItem(ctypes.Structure):
    _fields_ = [("scene", _vp), ("materialSystem", _vp), ("camera", ctypes.POINTER(Camera)),
                ("options", Options), ("deviceImage", _vp)]


BATCH_THREAD_PER_PIXEL = 0
BATCH_PATH_STATE = 1
BATCH_WAVEFRONT = 2
BATCH_KERNEL_NAMES = {BATCH_THREAD_PER_PIXEL: "thread_per_pixel", BATCH_PATH_STATE: "path_state",
                      BATCH_WAVEFRONT: "wavefront"}


class BatchConfig(ctypes.Structure):
    _fields_ = [("block", _u32), ("chunk", _u32), ("blocksPerSm", _u32), ("useGraph", _u32),
                ("kernel", _u32), ("wavePaths", _u32)]

    def as_dict(self):
        return dict(kernel=BATCH_KERNEL_NAMES[self.kernel], block=self.block, chunk=self.chunk,
                    blocks_per_sm=self.blocksPerSm, use_graph=self.useGraph,
                    wave_paths=self.wavePaths)


class Batch:
    """Many renderers' frames in one persistent launch (gbsp_batch_*).  Each
    item renders into a device image (a torch tensor's storage)."""

    def __init__(self, rt: Runtime, renderers, images):
        self.L, self.rt = rt.L, rt
        n = len(renderers)
        arr = (BatchItem * n)()
        for k, (r, img) in enumerate(zip(renderers, images)):
            arr[k].scene = r.scene.h
            arr[k].materialSystem = r.ms.h
            arr[k].camera = ctypes.pointer(r.camera)
            arr[k].options = r.options
            arr[k].deviceImage = img
        self._keep = (renderers, arr)
        h = _vp()
        _check(self.L.gbsp_batch_create(rt.h, arr, _u32(n), ctypes.byref(h)))
        self.h = h

    def config(self) -> BatchConfig:
        c = BatchConfig()
        _check(self.L.gbsp_batch_get_config(self.h, ctypes.byref(c)))
        return c

    def set_config(self, block=128, chunk=1, blocks_per_sm=8, use_graph=1,
                   kernel=BATCH_WAVEFRONT, wave_paths=0):
        c = BatchConfig(block, chunk, blocks_per_sm, use_graph, kernel, wave_paths)
        _check(self.L.gbsp_batch_set_config(self.h, ctypes.byref(c)))

    def autotune(self, trials=2) -> BatchConfig:
        c = BatchConfig()
        _check(self.L.gbsp_batch_autotune(self.h, _u32(trials), ctypes.byref(c)))
        return c

    def node_widths(self) -> list:
        n = len(self._keep[0])
        w = (_u32 * n)()
        _check(self.L.gbsp_batch_get_node_widths(self.h, w))
        return [int(v) for v in w]

    def set_node_widths(self, widths):
        n = len(self._keep[0])
        w = (_u32 * n)(*[int(v) for v in widths])
        _check(self.L.gbsp_batch_set_node_widths(self.h, w))

    def launch(self, metrics: bool = True):
        m = Metrics() if metrics else None
        _check(self.L.gbsp_batch_launch(self.h, ctypes.byref(m) if m is not None else None))
        return m

    def close(self):
        if self.h:
            self.L.gbsp_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- compute-shader path tracer (gbsp_cpt_*) ------------------------------------------

class CptMesh(ctypes.Structure):
    _fields_ = [("indexCount", _u32), ("indicesOffset", _u32), ("vertexDataOffset", _u32)]


class CptEntity(ctypes.Structure):
    _fields_ = [("meshIndex", _u32), ("materialId", _u32), ("modelMatrixIndex", _u32)]


class CptView(ctypes.Structure):
    _fields_ = [("width", _u32), ("height", _u32), ("tileWidth", _u32), ("tileHeight", _u32),
                ("filmDistance", _f32), ("cameraTransform", _f32 * 16)]


class ComputePTScene:
    """Scene buffers of the compute-shader path tracer on the device.

    vertices: (V, 8) float32 VertexPNT rows; indices: (I,) uint32; meshes:
    (M, 3) uint32 (indexCount, indicesOffset, vertexDataOffset); model /
    inv_model: (K, 16) float32 column-major; entities: (E, 3) uint32 (mesh,
    material, matrix); texture: (H, W, 4) float32 or None."""

    def __init__(self, rt: Runtime, vertices, indices, meshes, model, inv_model, entities,
                 texture=None):
        self.L, self.rt = rt.L, rt
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 8)
        i = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1)
        m = np.ascontiguousarray(meshes, dtype=np.uint32).reshape(-1, 3)
        mm = np.ascontiguousarray(model, dtype=np.float32).reshape(-1, 16)
        im = np.ascontiguousarray(inv_model, dtype=np.float32).reshape(-1, 16)
        e = np.ascontiguousarray(entities, dtype=np.uint32).reshape(-1, 3)
        if texture is not None:
            t = np.ascontiguousarray(texture, dtype=np.float32)
            th, tw = t.shape[:2]
        else:
            t, th, tw = None, 0, 0
        h = _vp()
        _check(self.L.gbsp_cpt_scene_create(
            rt.h, _p(v), _u32(len(v)), _p(i), _u32(len(i)), _p(m), _u32(len(m)), _p(mm), _p(im),
            _u32(len(mm)), _p(e), _u32(len(e)), _p(t) if t is not None else None, _u32(tw),
            _u32(th), ctypes.byref(h)))
        self.h = h

    def render_tiles(self, view: CptView, tiles, device_image: int, metrics: bool = True):
        tl = np.ascontiguousarray(tiles, dtype=np.uint32).reshape(-1)
        m = Metrics() if metrics else None
        _check(self.L.gbsp_cpt_render_tiles(self.h, ctypes.byref(view), _p(tl), _u32(len(tl)),
                                            _vp(device_image),
                                            ctypes.byref(m) if m is not None else None))
        return m

    def close(self):
        if self.h:
            self.L.gbsp_cpt_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def cpt_view(width=256, height=192, tile=16, film_distance=0.8, camera_transform=None) -> CptView:
    v = CptView()
    v.width, v.height, v.tileWidth, v.tileHeight = width, height, tile, tile
    v.filmDistance = film_distance
    ct = np.eye(4, dtype=np.float32).reshape(-1) if camera_transform is None else \
        np.asarray(camera_transform, dtype=np.float32).reshape(-1)
    for k in range(16):
        v.cameraTransform[k] = float(ct[k])
    return v


# ---- cube maps ----------------------------------------------------------------------------

IRRADIANCE_UNIFORM = 0
IRRADIANCE_RANDOM = 1


def create_cube_map(equirect, width: int, height: int, faces=None, stream: int = 0):
    """CreateCubeMap on the device: equirect is a (H, W, 4) float32 CUDA
    tensor; returns (6, height, width, 4)."""
    import torch

    L = load()
    if faces is None:
        faces = torch.empty((6, height, width, 4), dtype=torch.float32, device=equirect.device)
    _check(L.gbsp_create_cube_map(_vp(stream), _vp(equirect.data_ptr()),
                                  _u32(equirect.shape[1]), _u32(equirect.shape[0]), _u32(width),
                                  _u32(height), _vp(faces.data_ptr())))
    return faces


def create_irradiance_cube_map(equirect, width: int, height: int, spp: int = 32,
                               mode: int = IRRADIANCE_UNIFORM, faces=None, stream: int = 0):
    import torch

    L = load()
    if faces is None:
        faces = torch.empty((6, height, width, 4), dtype=torch.float32, device=equirect.device)
    _check(L.gbsp_create_irradiance_cube_map(
        _vp(stream), _vp(equirect.data_ptr()), _u32(equirect.shape[1]), _u32(equirect.shape[0]),
        _u32(width), _u32(height), _u32(spp), _u32(mode), _vp(faces.data_ptr())))
    return faces


def xorshift32_jump(state: int, steps: int) -> int:
    return int(load().gbsp_xorshift32_jump(_u32(state), ctypes.c_uint64(steps)))


def tonemap(frame, out=None, stream: int = 0):
    """gbsp_tonemap: (H, W, 4) float32 CUDA tensor -> (H, W) uint32 packed 8-bit RGBA."""
    import torch

    L = load()
    n = frame.shape[0] * frame.shape[1]
    if out is None:
        out = torch.empty(frame.shape[:2], dtype=torch.int32, device=frame.device)
    _check(L.gbsp_tonemap(_vp(stream), _vp(frame.data_ptr()), ctypes.c_uint64(n),
                          _vp(out.data_ptr())))
    return out
