"""The compute-shader path tracer's CPU restatement
(oracle/compute_pt_oracle.cpp, following src/shaders/test_compute.comp.glsl):
known answers that follow from the shader's rules alone."""

import numpy as np
import pytest

from oracle import pyoracle
from vk_cinematic_gb300 import scenes


@pytest.fixture(scope="module")
def built():
    pyoracle.build_port()


def xorshift(state):
    state ^= (state << 13) & 0xFFFFFFFF
    state ^= state >> 17
    state ^= (state << 5) & 0xFFFFFFFF
    return state


def test_empty_scene_is_black(built):
    s = scenes.compute_pt_scene(n_spheres=0, level=0, light=False)
    s["entities"] = s["entities"][:0]
    img, c = pyoracle.compute_pt_tiles(s, 64, 32, 16, 0.8, np.arange(8))
    assert np.all(img[..., :3] == 0.0) and np.all(img[..., 3] == 1.0)
    assert int(c[0]) == 64 * 32 and int(c[1]) == 0 and int(c[2]) == 0


def test_direct_light_is_exactly_one(built):
    # only a light sphere filling the view: every primary ray hits it, the
    # first vertex is emission 1 + albedo 0 * ... = 1 exactly
    s = scenes.compute_pt_scene(n_spheres=0, level=1, light=True)
    keep = s["entities"][s["entities"][:, 1] == scenes.CPT_MATERIAL_WHITE_LIGHT]
    s["entities"] = keep
    cam = np.zeros((4, 4), np.float32)
    cam[0] = (1, 0, 0, 0)
    cam[1] = (0, 0, -1, 0)   # up
    cam[2] = (0, 1, 0, 0)    # forward: looking straight up at the light
    cam[3] = (0, 4, 0, 0)    # 1 below the light's surface: it fills the view
    s["camera_transform"] = cam.reshape(-1)
    img, c = pyoracle.compute_pt_tiles(s, 32, 32, 16, 0.8, np.arange(4))
    assert np.all(img[..., :3] == 1.0)
    assert int(c[1]) >= 32 * 32


def test_tiles_not_listed_are_untouched_and_order_free(built):
    s = scenes.compute_pt_scene(n_spheres=4, level=1)
    full, _ = pyoracle.compute_pt_tiles(s, 64, 48, 16, 0.8, np.arange(12))
    part = np.full((48, 64, 4), -7.0, np.float32)
    part, _ = pyoracle.compute_pt_tiles(s, 64, 48, 16, 0.8, [5, 2], image=part)
    # tile 5 = (1, 1), tile 2 = (2, 0): each tile's RNG depends on its index only
    assert np.array_equal(part[16:32, 16:32], full[16:32, 16:32])
    assert np.array_equal(part[0:16, 32:48], full[0:16, 32:48])
    mask = np.ones((48, 64), bool)
    mask[16:32, 16:32] = False
    mask[0:16, 32:48] = False
    assert np.all(part[mask] == -7.0)


def test_rng_matches_xorshift_definition(built):
    # the tile seed (tileIndex + 1) * 0xF51C0E49 and float(x) / float(U32_MAX)
    seed = (3 + 1) * 0xF51C0E49 & 0xFFFFFFFF
    x = xorshift(seed)
    u = np.float32(np.float32(x) / np.float32(4294967296.0))
    assert 0.0 <= u <= 1.0
    # pixel jitter is tiny: half a pixel of the 0..1 film, not of the pixel
    assert 0.5 / 256 < 0.002


def test_counts_and_determinism(built):
    s = scenes.compute_pt_scene(n_spheres=6, level=1)
    a, ca = pyoracle.compute_pt_tiles(s, 48, 32, 16, 0.8, np.arange(6))
    b, cb = pyoracle.compute_pt_tiles(s, 48, 32, 16, 0.8, np.arange(6))
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.array_equal(ca, cb)
    rays, hits, tests = (int(v) for v in ca)
    assert 48 * 32 <= rays <= 3 * 48 * 32 and hits <= rays
    tris_per_ray = sum(int(s["meshes"][m][0]) // 3 for m in s["entities"][:, 0])
    assert tests == rays * tris_per_ray
