"""The drop-in C++ header: the reference's own unit tests restated against
include/sp_gpu.h (tests/cpp/test_sp_gpu.cpp), compiled with g++ and linked
to libgbsp.so.  The compile check runs on CPU; the program runs on a GPU."""

import os
import subprocess

import pytest

from vk_cinematic_gb300 import build as gbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_sp_gpu.cpp")
EXE = os.path.join(gbuild.BUILD, "test_sp_gpu")


def cuda_lib_dir():
    for d in ("/usr/local/cuda/lib64", "/usr/local/cuda/targets/sbsa-linux/lib",
              "/usr/local/cuda/targets/x86_64-linux/lib"):
        if os.path.exists(os.path.join(d, "libcudart.so")):
            return d
    return "/usr/local/cuda/lib64"


def compile_test():
    lib = gbuild.build()
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", EXE,
           "-L", os.path.dirname(lib), "-lgbsp", "-L", cuda_lib_dir(), "-lcudart",
           f"-Wl,-rpath,{os.path.dirname(lib)}", f"-Wl,-rpath,{cuda_lib_dir()}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return EXE


def test_sp_gpu_header_compiles_and_links():
    assert os.path.exists(compile_test())


@pytest.mark.gpu
def test_reference_unit_tests_through_sp_gpu_header(gpu_lib):
    exe = compile_test()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "7 tests, 0 failures" in r.stdout
