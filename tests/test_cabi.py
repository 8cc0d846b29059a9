"""The C-ABI library on the CPU: it builds, loads, exports every symbol
include/gbsp.h declares, and its host-side entry points (camera, procedural
meshes, per-sample seeding) agree with the reference.  No device calls."""

import math
import os
import re

import numpy as np
import pytest

from vk_cinematic_gb300 import gbsp, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def test_header_declarations_are_exported():
    header = open(os.path.join(ROOT, "include", "gbsp.h")).read()
    declared = set(re.findall(r"\b(gbsp_[a-z0-9_]+)\s*\(", header))
    assert declared, "no declarations parsed"
    assert declared == set(gbsp.EXPORTS), declared ^ set(gbsp.EXPORTS)
    lib = gbsp.load()
    for name in declared:
        assert hasattr(lib, name), name


def test_icosphere_matches_reference_levels(golden):
    for level in range(6):
        v, i = gbsp.icosphere(level)
        sv, si = scenes.icosphere(level)
        assert np.array_equal(bits(v), bits(sv)) and np.array_equal(i, si)
        assert len(v) == 12 + 60 * ((4 ** level - 1) // 3) and len(i) == 60 * 4 ** level


def test_plane_mesh():
    v, i = gbsp.plane_mesh()
    pv, pi = scenes.plane()
    assert np.array_equal(v, pv) and np.array_equal(i, pi)


def test_sample_seed_matches_oracle(port):
    rng = np.random.default_rng(0)
    for _ in range(200):
        a = [int(x) for x in rng.integers(0, 2**32 - 1, 4)]
        assert gbsp.sample_seed(*a) == port.sample_seed(*a)
    # never the XorShift32 fixed point
    assert all(gbsp.sample_seed(s, 0, 0, 0) != 0 for s in range(1000))


def test_camera_matches_reference(golden):
    g = golden["primitives"]
    for k, row in enumerate(g["camera_in"]):
        w, h = int(row[0]), int(row[1])
        plane = gbsp.ImagePlane(None, w, h)
        cam = gbsp.Camera()
        pos = np.ascontiguousarray(row[2:5], np.float32)
        rot = np.ascontiguousarray(row[5:9], np.float32)
        rc = gbsp.load().gbsp_configure_camera(gbsp.ctypes.byref(cam), gbsp.ctypes.byref(plane),
                                                gbsp._p(pos), gbsp._p(rot),
                                                gbsp.ctypes.c_float(row[9]))
        assert rc == 0
        got = np.array(list(cam.right) + list(cam.up) + list(cam.forward) + list(cam.position) +
                       list(cam.filmCenter) + [cam.halfPixelWidth, cam.halfPixelHeight,
                                               cam.halfFilmWidth, cam.halfFilmHeight], np.float32)
        assert np.array_equal(bits(got), bits(g["camera_out"][k]))
        film = gbsp.film_positions(cam, g["film_pixels"] * np.float32(max(w, h) / 4))
        assert np.array_equal(bits(film), bits(g["film_out"][k]))


def test_runtime_without_device_fails_cleanly():
    """On a host with no usable GPU the runtime refuses with a status, never a
    crash or a CPU fallback."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(gbsp.GbspError, match="status -7"):
        gbsp.Runtime()


def test_invalid_arguments_return_status():
    lib = gbsp.load()
    assert lib.gbsp_configure_camera(None, None, None, None, gbsp.ctypes.c_float(0.5)) == -1
    assert b"NULL" in lib.gbsp_last_error_string()
    assert lib.gbsp_scene_create(None, None) == -1
    assert lib.gbsp_icosphere(11, None, None, None, None) == -3


def test_denoiser_planar_layout_round_trip():
    """The denoiser kernels take activations channel-group-planar,
    [B][H][C/8][W][8]; the host helpers convert NHWC to that layout and back,
    and element (b, y, x, c) lands at ((b H + y) C/8 + c/8) W + x) 8 + c % 8."""
    import torch

    from vk_cinematic_gb300.denoiser import from_planar, to_planar

    B, H, W, C = 2, 3, 5, 24
    t = torch.arange(B * H * W * C, dtype=torch.float32).reshape(B, H, W, C)
    p = to_planar(t)
    assert p.shape == (B, H, C // 8, W, 8) and p.is_contiguous()
    assert torch.equal(from_planar(p), t)
    flat = p.reshape(-1)
    for b, y, x, c in ((0, 0, 0, 0), (1, 2, 4, 23), (0, 1, 3, 9), (1, 0, 2, 16)):
        idx = (((b * H + y) * (C // 8) + c // 8) * W + x) * 8 + c % 8
        assert flat[idx].item() == t[b, y, x, c].item()


def test_add_object_passes_the_transform_it_was_given():
    """Scene.add_object hands gbsp_add_object_to_scene (sp_AddObjectToScene,
    src/sp_scene.cpp:77-117) pointers to the position, rotation and scale it
    was called with, rounded to float32 as the reference's f32 fields are,
    call after call; a vector of the wrong length is refused before the call."""
    import ctypes

    calls = []

    def read(ptr, n):
        return list(np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_float)),
                                          shape=(n,)).copy())

    class FakeLib:
        def gbsp_scene_create(self, rt, out):
            return 0

        def gbsp_add_object_to_scene(self, h, mesh, material, p, r, s):
            calls.append((mesh.value, material.value, read(p, 3), read(r, 4), read(s, 3)))
            return 0

    class FakeRuntime:
        L = FakeLib()
        h = None

    scene = gbsp.Scene(FakeRuntime())
    objs = scenes.config3_scene().objects[:20]
    for o in objs:
        scene.add_object(o.mesh, o.material, o.position, o.rotation, o.scale)
    scene.add_object(3, 7, (0.1, 2, -3), (0, 0, 0, 1), [1.5, 1.5, 1.5])
    assert len(calls) == len(objs) + 1
    for (mesh, mat, p, r, s), o in zip(calls, objs):
        assert (mesh, mat) == (o.mesh, o.material)
        assert np.array_equal(bits(p), bits(o.position))
        assert np.array_equal(bits(r), bits(o.rotation))
        assert np.array_equal(bits(s), bits(o.scale))
    mesh, mat, p, r, s = calls[-1]
    assert (mesh, mat) == (3, 7)
    assert np.array_equal(bits(p), bits(np.float32([0.1, 2, -3])))
    assert r == [0, 0, 0, 1] and s == [1.5, 1.5, 1.5]
    with pytest.raises(ValueError):
        scene.add_object(0, 0, (1, 2), (0, 0, 0, 1), (1, 1, 1))
    assert len(calls) == len(objs) + 1


def test_header_is_plain_c_and_links(tmp_path):
    """include/gbsp.h is a C header: a C99 program (-pedantic, warnings as
    errors) that takes the address of every function it declares compiles,
    links against libgbsp.so and runs (no device call), which is what a cgo,
    JNI or other FFI binding of the library does."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    gbsp.load()
    header = open(os.path.join(ROOT, "include", "gbsp.h")).read()
    names = sorted(set(re.findall(r"\b(gbsp_[a-z0-9_]+)\s*\(", header)))
    src = tmp_path / "abi.c"
    src.write_text(
        '#include <stdio.h>\n#include "gbsp.h"\n'
        "typedef void (*fn)(void);\n"
        "int main(void)\n{\n    fn table[] = {\n"
        + "".join(f"        (fn){n},\n" for n in names)
        + "    };\n    size_t n = 0, i;\n"
        "    for (i = 0; i < sizeof(table) / sizeof(table[0]); i++) n += table[i] != 0;\n"
        '    printf("%lu\\n", (unsigned long)n);\n    return 0;\n}\n')
    exe = tmp_path / "abi"
    build = os.path.dirname(gbsp._build.LIB)
    r = subprocess.run([cc, "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror",
                        "-I", os.path.join(ROOT, "include"), str(src), "-o",
                        str(exe), "-L", build, "-lgbsp", "-Wl,-rpath," + build],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    assert int(r.stdout.strip()) == len(names)
