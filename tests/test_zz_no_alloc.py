"""The allocation-free tile render, gbsp_path_trace_tile_noalloc.

Some callers of a tile path tracer must not allocate device memory inside the
call: a render loop held to a fixed device-memory budget, or one that cannot
absorb the device-wide synchronisation an allocation may trigger.  For them
the library keeps this entry point's working memory in one fixed array of
its own (about 5.8 MB per GPU, held until exit; up to 16384 paths in flight,
8 bounces, 4096 objects); the caller still passes the inputs (scene,
materials, camera) and the output image in device memory.

The tests call the entry point through the C ABI twice in a row and check
each result against the regular tile entry point (gbsp_path_trace_tile).
Both run the same kernels on the same per-sample seeds, so the pixels of the
tile must be bit-identical; the cases include tiles that need several passes
over the fixed array (more paths than it holds, and an spp that does not
divide its 16384 paths).  This file is collected after the other GPU tests
and needs nothing from them: it makes its own runtime and scene.
"""

import ctypes

import numpy as np
import pytest

from vk_cinematic_gb300 import gbsp, scenes

pytestmark = pytest.mark.gpu

MAX_PATHS = 16384  # paths the fixed array holds at once


@pytest.fixture(scope="module")
def world(gpu_lib):
    rt = gbsp.Runtime()
    s = scenes.config1_scene(width=96, height=72, spp=4, seed=21)
    opt = gbsp.default_options(spp=4, max_bounces=3, seed=21)
    scene, ms, rend = gbsp.upload_scene(rt, s, opt)
    rend.tile((0, 0, 1, 1))  # the regular entry point uploads the materials
    yield rt, s, scene, ms, rend
    rt.close()


def noalloc(lib, rend, tile, image, metrics=None):
    return lib.gbsp_path_trace_tile_noalloc(ctypes.byref(rend.ctx), gbsp.Tile(*tile),
                                            ctypes.c_void_p(image.data_ptr()),
                                            ctypes.byref(metrics) if metrics is not None else None)


@pytest.mark.parametrize("tile,spp", [((8, 4, 72, 52), 4),    # 12,288 paths: one pass
                                      ((0, 0, 96, 72), 4),    # 27,648 paths: two passes
                                      ((5, 3, 96, 71), 3),    # 6,188 px: 5,461 px per pass
                                      ((0, 0, 96, 72), 7)])   # 2,340 px per pass, three passes
def test_noalloc_tile_matches_regular_entry_point(world, tile, spp):
    import torch

    rt, s, scene, ms, rend = world
    lib = gbsp.load()
    rend.options.spp = spp
    x0, y0, x1, y1 = tile
    ref, _, mref = rend.tile(tile)
    inside = np.zeros((s.height, s.width), bool)
    inside[y0:y1, x0:x1] = True
    paths = (x1 - x0) * (y1 - y0) * spp
    passes = -(-(x1 - x0) * (y1 - y0) // (MAX_PATHS // spp))
    print(f"tile {tile} at {spp} spp: {paths} paths in {passes} passes")
    image = torch.full((s.height, s.width, 4), -5.0, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    for call in range(2):
        m = gbsp.Metrics()
        rc = noalloc(lib, rend, tile, image, m)
        assert rc == 0, lib.gbsp_last_error_string().decode()
        out = image.cpu().numpy()
        assert np.all(out[~inside] == -5.0), f"call {call}: wrote outside the tile"
        assert np.array_equal(out[inside].view(np.uint32), ref[inside].view(np.uint32)), \
            f"call {call}: pixels differ from gbsp_path_trace_tile"
        md, mr = m.as_dict(), mref.as_dict()
        for k in ("paths_traced", "rays_traced", "ray_hit_count", "ray_miss_count",
                  "triangle_tests", "midphase_node_visits", "nan_samples"):
            assert md[k] == mr[k], (call, k, md[k], mr[k])
        assert md["paths_traced"] == paths
        assert md["trace_launches"] == passes * 3
    rend.options.spp = 4


def test_noalloc_rejects_requests_beyond_its_limits(world):
    """Limits and preconditions are checked on the host before any launch."""
    import torch

    rt, s, scene, ms, rend = world
    lib = gbsp.load()
    image = torch.zeros((s.height, s.width, 4), dtype=torch.float32, device="cuda")
    tile = (0, 0, 16, 16)
    for field, value, words in (("spp", 20000, b"spp <="), ("max_bounces", 9, b"bounces <=")):
        old = getattr(rend.options, field)
        setattr(rend.options, field, value)
        assert noalloc(lib, rend, tile, image) == -3
        assert words in lib.gbsp_last_error_string()
        setattr(rend.options, field, old)
    rend.options.flags = gbsp.FLAG_AOV
    assert noalloc(lib, rend, tile, image) == -1
    rend.options.flags = 0
    rend.options.rng_mode = gbsp.RNG_TILE_SEQUENTIAL
    assert noalloc(lib, rend, tile, image) == -1
    rend.options.rng_mode = gbsp.RNG_HASH_PER_SAMPLE
    # materials registered but never uploaded by a regular render
    ms2 = gbsp.MaterialSystem(rt)
    for mid, mat in s.materials.items():
        ms2.register(mid, **mat)
    rend2 = gbsp.Renderer(rt, scene, ms2, s.width, s.height, s.camera_position,
                          s.camera_rotation, s.film_distance, rend.options)
    assert noalloc(lib, rend2, tile, image) == -6
    assert b"materials" in lib.gbsp_last_error_string()
    torch.cuda.synchronize()
    assert float(image.abs().sum()) == 0.0
    ms2.close()
