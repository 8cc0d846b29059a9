"""The drop-in header against the reference's own headers and tests.

The reference's path-tracer unit tests (unit_tests/test_simd_path_tracer.cpp)
are compiled the way a vk_cinematic caller would switch to the GPU library:
the includes of sp_scene.h, sp_material_system.h, simd_path_tracer.h and
sp_metrics.h become one #include "sp_gpu.h", the unity-build includes of
sp_scene.cpp, sp_material_system.cpp and simd_path_tracer.cpp are dropped, and
everything else - platform.h, math_lib.h, tile.h, memory_pool.h, bvh.h,
image.h, mesh.h, simd.h, aabb.h, the unity framework - is the reference's
own.  The program links libgbsp.so.

Four of the file's tests call functions that are internal to the swapped
.cpp files rather than the sp_* API a caller uses (ComputeRadianceForPath,
sp_EvaluateMaterial, sp_RayIntersectMesh, sp_Mesh::midphaseTree); they are
cut from the generated copy, with their RUN_TEST lines.  The remaining
twelve tests compile unchanged against sp_gpu.h.

The generated file is written to pytest's temporary directory and never into
the repository.  The reference tree is only mounted in the x86-64 build
container, and its platform.h includes <x86intrin.h> (src/platform.h:10), so
this test compiles and links here (no GPU) and is skipped elsewhere; on a GPU
host the same tests run restated in tests/cpp/test_sp_gpu.cpp.
"""

import os
import platform
import re
import subprocess

import pytest

import pyoracle as po
from vk_cinematic_gb300 import build as gbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SWAPPED_HEADERS = ("sp_scene.h", "sp_material_system.h", "simd_path_tracer.h", "sp_metrics.h")
SWAPPED_SOURCES = ("sp_scene.cpp", "sp_material_system.cpp", "simd_path_tracer.cpp")
INTERNAL_TESTS = ("TestEvaluateLightPath", "TestMaterialAlbedoTexture", "TestRayIntersectMesh",
                  "TestCreateMeshBuildsBvhTreeSingleTriangle")


def swap_includes(text: str) -> str:
    """The reference test file with the sp_* includes swapped for sp_gpu.h and
    the tests of swapped-out internals removed."""
    out, placed = [], False
    for line in text.split("\n"):
        m = re.match(r'\s*#include\s+"([^"]+)"', line)
        if m and m.group(1) in SWAPPED_HEADERS:
            if not placed:
                out.append('#include "sp_gpu.h"')
                placed = True
            continue
        if m and m.group(1) in SWAPPED_SOURCES:
            continue
        if re.match(r"\s*RUN_TEST\((%s)\);" % "|".join(INTERNAL_TESTS), line):
            continue
        out.append(line)
    assert placed, "no sp_* include found"
    s = "\n".join(out)
    for name in INTERNAL_TESTS:
        i = s.index(f"void {name}()")
        k = s.index("{", i)
        depth = 0
        while True:
            depth += {"{": 1, "}": -1}.get(s[k], 0)
            if depth == 0:
                break
            k += 1
        s = s[:i] + s[k + 1:]
    return s


def cuda_lib_dir():
    for d in ("/usr/local/cuda/lib64", "/usr/local/cuda/targets/x86_64-linux/lib"):
        if os.path.exists(os.path.join(d, "libcudart.so")):
            return d
    return "/usr/local/cuda/lib64"


def test_reference_unit_tests_compile_against_sp_gpu_header(tmp_path):
    ref = po.reference_root()
    src = os.path.join(ref, "unit_tests", "test_simd_path_tracer.cpp")
    if not os.path.exists(src):
        pytest.skip("reference tree not mounted on this host")
    if platform.machine() not in ("x86_64", "AMD64"):
        pytest.skip("the reference's platform.h includes <x86intrin.h>")
    with open(src) as f:
        text = f.read()
    gen = swap_includes(text)
    assert gen.count("RUN_TEST(") == text.count("RUN_TEST(") - len(INTERNAL_TESTS)
    tu = tmp_path / "test_simd_path_tracer_sp_gpu.cpp"
    tu.write_text(gen)
    unity_dir = os.path.join(ref, "thirdparty", "unity")
    unity_o = tmp_path / "unity.o"
    r = subprocess.run(["gcc", "-c", "-O2", "-I", unity_dir, os.path.join(unity_dir, "unity.c"),
                        "-o", str(unity_o)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = gbuild.build()
    exe = tmp_path / "test_simd_path_tracer_sp_gpu"
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-DPLATFORM_LINUX",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ref, "src"), "-I", unity_dir,
           str(tu), str(unity_o), "-o", str(exe), "-L", os.path.dirname(lib), "-lgbsp",
           "-L", cuda_lib_dir(), "-lcudart", f"-Wl,-rpath,{os.path.dirname(lib)}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert exe.exists()
    # every sp_* entry point the remaining tests call resolves to libgbsp.so
    nm = subprocess.run(["nm", "-D", "--undefined-only", str(exe)], capture_output=True,
                        text=True).stdout
    for sym in ("gbsp_path_trace_tile", "gbsp_ray_intersect_scene", "gbsp_configure_camera",
                "gbsp_calculate_film_positions", "gbsp_build_scene_broadphase"):
        assert sym in nm, sym
