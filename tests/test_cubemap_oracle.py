"""The cube-map restatement (oracle/cubemap_oracle.cpp) against the
reference's own CreateCubeMap / CreateIrradianceCubeMap compiled from
src/cubemap.cpp (oracle/_ref), and the XorShift32 jump-ahead of the library
against the sequential stream."""

import numpy as np
import pytest

from oracle import pyoracle
from vk_cinematic_gb300 import gbsp, scenes


@pytest.fixture(scope="module")
def hdri():
    pyoracle.build_port()
    return scenes.equirect_hdri(256, 128)


def test_cube_map_bit_exact_vs_reference(ref, hdri):
    a = pyoracle.create_cube_map(hdri, 24, 16, "port")
    b = pyoracle.create_cube_map(hdri, 24, 16, "ref")
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("mode", [0, 1])
def test_irradiance_bit_exact_vs_reference(ref, hdri, mode):
    a = pyoracle.create_irradiance_cube_map(hdri, 6, 5, 16, mode, "port")
    b = pyoracle.create_irradiance_cube_map(hdri, 6, 5, 16, mode, "ref")
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert (a[..., :3] > 0).all()


def test_irradiance_of_constant_environment(hdri):
    # uniform grid: pi * sum(c * cos * sin) / N for a constant c; every
    # texel sees the same samples up to rotation, so all texels agree closely
    flat = np.full((64, 128, 4), 2.0, np.float32)
    out = pyoracle.create_irradiance_cube_map(flat, 4, 4, 0, 0)
    v = out[..., :3]
    assert np.allclose(v, v.flat[0], rtol=1e-5)
    assert 1.0 < v.flat[0] < 2.0  # pi * c * E[cos sin] on the grid (about 0.6 c)


def xorshift(x):
    x ^= (x << 13) & 0xFFFFFFFF
    x ^= x >> 17
    x ^= (x << 5) & 0xFFFFFFFF
    return x


def test_xorshift_jump_matches_sequential():
    seq = [0x45BA12F3]
    for _ in range(5000):
        seq.append(xorshift(seq[-1]))
    for n in (0, 1, 2, 3, 31, 32, 96, 1000, 4999, 5000):
        assert gbsp.xorshift32_jump(0x45BA12F3, n) == seq[n]
    # composition: jump(a + b) = jump(jump(a), b)
    s = gbsp.xorshift32_jump(0x1234567, 1 << 40)
    assert gbsp.xorshift32_jump(gbsp.xorshift32_jump(0x1234567, 1 << 39), 1 << 39) == s
