"""The compute-shader path tracer on the GPU (gbsp_cpt_*) against its CPU
restatement: every operation is a basic IEEE operation or sqrt, so images
and counters must agree bit for bit."""

import numpy as np
import pytest

from oracle import pyoracle
from vk_cinematic_gb300 import gbsp, scenes

pytestmark = pytest.mark.gpu


def render_gpu(s, width, height, tiles, fill=0.0):
    import torch

    rt = gbsp.Runtime()
    sc = gbsp.ComputePTScene(rt, s["vertices"], s["indices"], s["meshes"], s["model"],
                             s["inv_model"], s["entities"], s.get("texture"))
    img = torch.full((height, width, 4), fill, dtype=torch.float32, device="cuda")
    view = gbsp.cpt_view(width, height, 16, 0.8, s["camera_transform"])
    m = sc.render_tiles(view, tiles, img.data_ptr())
    out = img.cpu().numpy()
    sc.close()
    return out, m.as_dict()


@pytest.mark.parametrize("level,n_spheres", [(1, 16), (2, 24)])
def test_full_image_bit_exact(gpu_lib, level, n_spheres):
    pyoracle.build_port()
    s = scenes.compute_pt_scene(n_spheres=n_spheres, level=level)
    w, h = 256, 192
    tiles = np.arange((w // 16) * (h // 16))
    ref, c = pyoracle.compute_pt_tiles(s, w, h, 16, 0.8, tiles)
    got, m = render_gpu(s, w, h, tiles)
    same = got.view(np.uint32) == ref.view(np.uint32)
    assert same.all(), f"{(~same).sum()} words differ; first at {np.argwhere(~same)[:3]}"
    assert m["rays_traced"] == int(c[0])
    assert m["ray_hit_count"] == int(c[1])
    assert m["triangle_tests"] == int(c[2])
    assert (ref[..., :3] > 0).mean() > 0.05  # the light is seen


def test_tile_subset_and_ragged_image(gpu_lib):
    pyoracle.build_port()
    s = scenes.compute_pt_scene(n_spheres=5, level=3)
    w, h = 200, 120  # tiles clipped at the right and bottom edges
    tiles = np.array([0, 11, 12, 35, 40, 77, 3])  # 77 lies outside the image: no pixels
    ref = np.full((h, w, 4), -3.0, np.float32)
    ref, c = pyoracle.compute_pt_tiles(s, w, h, 16, 0.8, tiles, image=ref)
    got, m = render_gpu(s, w, h, tiles, fill=-3.0)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    assert m["rays_traced"] == int(c[0])


def test_rejects_bad_input(gpu_lib):
    s = scenes.compute_pt_scene(n_spheres=1, level=0)
    rt = gbsp.Runtime()
    bad = s["entities"].copy()
    bad[0, 0] = 9  # no mesh 9
    with pytest.raises(gbsp.GbspError, match="out of range"):
        gbsp.ComputePTScene(rt, s["vertices"], s["indices"], s["meshes"], s["model"],
                            s["inv_model"], bad, s["texture"])
    idx = s["indices"].copy()
    idx[0] = 10 ** 6
    with pytest.raises(gbsp.GbspError, match="vertex index"):
        gbsp.ComputePTScene(rt, s["vertices"], idx, s["meshes"], s["model"], s["inv_model"],
                            s["entities"], s["texture"])
