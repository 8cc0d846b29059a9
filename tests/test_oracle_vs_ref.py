"""The oracle port against the reference's own code, live (x86-64 hosts with
the reference tree; skipped elsewhere).  Bit-exact on fresh random inputs,
complementing the stored golden vectors."""

import ctypes
import math

import numpy as np
import pytest

import pyoracle as po
from vk_cinematic_gb300 import scenes
from golden_scenes import build_world


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def test_icosphere_levels_match_reference(ref):
    lib = ctypes.CDLL(po.REF_LIB)
    for level in range(4):
        v = np.zeros((2048, 8), np.float32)
        i = np.zeros(4096, np.uint32)
        nv, ni = ctypes.c_uint32(), ctypes.c_uint32()
        assert lib.ref_icosphere(level, v.ctypes.data_as(ctypes.c_void_p),
                                 i.ctypes.data_as(ctypes.c_void_p), ctypes.byref(nv),
                                 ctypes.byref(ni)) == 0
        sv, si = scenes.icosphere(level)
        assert np.array_equal(bits(v[:nv.value]), bits(sv))
        assert np.array_equal(i[:ni.value], si)


def random_scene(seed):
    rng = np.random.default_rng(seed)
    s = scenes.config1_scene(width=24, height=20, spp=3, seed=seed)
    s.objects = []
    for k in range(int(rng.integers(3, 12))):
        ax = rng.normal(size=3)
        rot = scenes.quat_axis_angle(ax / np.linalg.norm(ax), float(rng.uniform(-3, 3)))
        sc = np.float32(rng.uniform(0.2, 1.2))
        mesh = int(rng.integers(0, 2))
        pos = rng.uniform([-2, 0, -3], [2, 2.5, 0]).astype(np.float32)
        s.objects.append(scenes.SceneObject(mesh, int(rng.integers(1, 3)), pos, rot,
                                            np.array([sc, sc, sc], np.float32)))
    s.objects.append(scenes.SceneObject(1, 1, np.zeros(3, np.float32),
                                        scenes.quat_axis_angle((1, 0, 0), -math.pi / 2),
                                        np.array([20, 20, 20], np.float32)))
    s.materials[2] = scenes.material(albedo=(0.2, 0.7, 0.4), emission=(0.5, 0.1, 0.0),
                                     roughness=0.5)
    return s


@pytest.mark.parametrize("seed", [11, 12, 13])
def test_random_scenes_match_reference(ref, seed):
    s = random_scene(seed)
    wr = build_world("ref", s)
    wp = build_world("port", s)
    rng = np.random.default_rng(seed)
    org = rng.uniform(-3, 3, (2000, 3)).astype(np.float32) + np.float32([0, 1.5, 2])
    d = rng.normal(size=(2000, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    rays = np.concatenate([org, d], 1).astype(np.float32)
    a = wr.intersect(rays)
    b = wp.intersect(rays)
    assert np.array_equal(bits(a[0]), bits(b[0]))
    img_r = wr.path_trace_hashed(s.width, s.height, s.camera_position, s.camera_rotation,
                                 s.film_distance, s.seed)[0]
    img_p = wp.path_trace_hashed(s.width, s.height, s.camera_position, s.camera_rotation,
                                 s.film_distance, s.seed)[0]
    assert np.array_equal(bits(img_r), bits(img_p))


def test_to_color_matches_reference(ref):
    """ToColor (src/math_lib.h:523-532), the last step of the display
    conversion: every level boundary k/255 with its neighbouring floats, the
    ends of [0, 1] and random values, bit for bit."""
    levels = np.arange(256, dtype=np.float32) / np.float32(255.0)
    vals = np.concatenate([
        levels, np.nextafter(levels, np.float32(0)), np.nextafter(levels, np.float32(1)),
        np.float32([0.0, -0.0, 1.0, 0.5, np.nextafter(np.float32(1), np.float32(0))]),
        np.random.default_rng(5).random(4000, dtype=np.float32),
    ]).astype(np.float32)
    vals = np.clip(vals, 0, 1)
    rgba = np.ascontiguousarray(np.stack(
        [vals, vals[::-1], np.roll(vals, 7), np.roll(vals, 101)], 1), dtype=np.float32)
    n = rgba.shape[0]
    got = np.zeros(n, np.uint32)
    want = np.zeros(n, np.uint32)
    ctypes.CDLL(po.PORT_LIB).oracle_to_color(rgba.ctypes.data_as(ctypes.c_void_p),
                                             ctypes.c_uint64(n),
                                             got.ctypes.data_as(ctypes.c_void_p))
    ctypes.CDLL(po.REF_LIB).ref_to_color(rgba.ctypes.data_as(ctypes.c_void_p),
                                         ctypes.c_uint64(n),
                                         want.ctypes.data_as(ctypes.c_void_p))
    assert np.array_equal(got, want)
    assert len(np.unique(want & 0xFF)) == 256
