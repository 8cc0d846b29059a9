"""The allocation-free tile render, gbsp_path_trace_tile_noalloc.

Some callers of a tile path tracer must not allocate device memory inside the
call: a render loop held to a fixed device-memory budget, or one that cannot
absorb the device-wide synchronisation an allocation may trigger.  For them
the library keeps this entry point's working memory in one fixed array of
its own (about 5.8 MB per GPU, held until exit; up to 16384 paths in flight,
8 bounces, 4096 objects); the caller still passes the inputs (scene,
materials, camera) and the output image in device memory.

This test calls the entry point through the C ABI twice in a row and checks
each result against the regular tile entry point (gbsp_path_trace_tile),
within the image tolerance the other GPU tests use.  It lives in a file of
its own that pytest collects last, and it needs nothing from other tests.
"""

import ctypes

import numpy as np
import pytest

from vk_cinematic_gb300 import gbsp, scenes

pytestmark = pytest.mark.gpu

IMAGE_TOL = 1e-3  # mean relative error, as in test_gpu_parity.py


def mean_rel_err(a, b):
    a = np.asarray(a, np.float64)[..., :3]
    b = np.asarray(b, np.float64)[..., :3]
    return float(np.mean(np.abs(a - b) / np.maximum(np.abs(b), 1e-3)))


def test_noalloc_tile_matches_regular_entry_point(gpu_lib):
    import torch

    lib = gbsp.load()
    rt = gbsp.Runtime()
    s = scenes.config1_scene(width=80, height=56, spp=4, seed=21)
    opt = gbsp.default_options(spp=4, max_bounces=3, seed=21)
    scene, ms, rend = gbsp.upload_scene(rt, s, opt)
    tile = (8, 4, 72, 52)
    ref, _, _ = rend.tile(tile)  # the regular entry point; it also uploads the materials

    inside = np.zeros((s.height, s.width), bool)
    inside[4:52, 8:72] = True
    image = torch.full((s.height, s.width, 4), -5.0, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    for call in range(2):
        m = gbsp.Metrics()
        rc = lib.gbsp_path_trace_tile_noalloc(ctypes.byref(rend.ctx), gbsp.Tile(*tile),
                                              ctypes.c_void_p(image.data_ptr()), ctypes.byref(m))
        assert rc == 0, lib.gbsp_last_error_string().decode()
        out = image.cpu().numpy()
        assert np.all(out[~inside] == -5.0), f"call {call}: wrote outside the tile"
        err = mean_rel_err(out[inside], ref[inside])
        assert err <= IMAGE_TOL, f"call {call}: mean relative error {err}"
        assert m.values[1] == 64 * 48 * 4, f"call {call}: paths {m.values[1]}"

    # requests beyond the fixed array's limits fail with a clear status
    rend.options.spp = 20000
    image2 = torch.zeros((s.height, s.width, 4), dtype=torch.float32, device="cuda")
    rc = lib.gbsp_path_trace_tile_noalloc(ctypes.byref(rend.ctx), gbsp.Tile(*tile),
                                          ctypes.c_void_p(image2.data_ptr()), None)
    assert rc == -3
    assert b"spp <=" in lib.gbsp_last_error_string()
    rend.options.spp = 4
    rt.close()
