"""Batched rendering (config 4 pattern): many scenes of uneven size, spp and
bounce count in one persistent launch must give images bit-identical to
rendering each scene on its own, with and without CUDA-graph replay and
after autotuning."""

import numpy as np
import pytest

from vk_cinematic_gb300 import gbsp, scenes

pytestmark = pytest.mark.gpu


def small_batch_scenes():
    rng = np.random.default_rng(7)
    out = []
    for k in range(6):
        side = int(rng.integers(8, 40))
        s = scenes.config3_scene(width=side + int(rng.integers(0, 9)), height=side,
                                 spp=int(rng.integers(1, 9)), max_bounces=int(rng.integers(1, 9)),
                                 n_spheres=int(rng.integers(1, 40)), level=int(rng.integers(1, 4)),
                                 seed=100 + k)
        out.append(s)
    return out


def test_batch_matches_single_scene_renders(gpu_lib):
    import torch

    rt = gbsp.Runtime()
    ss = small_batch_scenes()
    rends, refs, imgs = [], [], []
    keep = []
    for s in ss:
        scene, ms, rend = gbsp.upload_scene(rt, s)
        keep.append((scene, ms))
        ref, m = rend.frame()
        refs.append(ref)
        rends.append(rend)
        imgs.append(torch.full((s.height, s.width, 4), -1.0, dtype=torch.float32, device="cuda"))
    torch.cuda.synchronize()
    batch = gbsp.Batch(rt, rends, [t.data_ptr() for t in imgs])
    total = sum(s.width * s.height * s.spp for s in ss)
    # wavefront: one wave, then waves of 1,000 paths (items split across waves)
    # (blocks per SM 0: the wavefront's kernels at the blocks the SMs hold)
    for kernel, use_graph, wave, bps in ((gbsp.BATCH_THREAD_PER_PIXEL, 0, 0, 4),
                                         (gbsp.BATCH_THREAD_PER_PIXEL, 1, 0, 4),
                                         (gbsp.BATCH_PATH_STATE, 0, 0, 4),
                                         (gbsp.BATCH_PATH_STATE, 1, 0, 4),
                                         (gbsp.BATCH_WAVEFRONT, 0, 0, 4),
                                         (gbsp.BATCH_WAVEFRONT, 1, 0, 4),
                                         (gbsp.BATCH_WAVEFRONT, 1, 1000, 4),
                                         (gbsp.BATCH_WAVEFRONT, 1, 0, 0)):
        batch.set_config(block=128, chunk=1, blocks_per_sm=bps, use_graph=use_graph,
                         kernel=kernel, wave_paths=wave)
        for _ in range(2):  # a replayed graph must reset its queue each time
            for t in imgs:
                t.fill_(-1.0)
            torch.cuda.synchronize()
            m = batch.launch()
            assert m.as_dict()["paths_traced"] == total
            for k, (t, ref) in enumerate(zip(imgs, refs)):
                got = t.cpu().numpy()
                assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), \
                    f"item {k} differs (kernel={kernel}, graph={use_graph}, wave={wave}, bps={bps})"
    # every item on 4-wide BVHs, then mixed widths: the same bits
    for widths in ([4] * len(ss), [4 if k % 2 else 8 for k in range(len(ss))]):
        batch.set_node_widths(widths)
        assert batch.node_widths() == widths
        for t in imgs:
            t.fill_(-1.0)
        torch.cuda.synchronize()
        batch.launch()
        for k, (t, ref) in enumerate(zip(imgs, refs)):
            assert np.array_equal(t.cpu().numpy().view(np.uint32), ref.view(np.uint32)), \
                f"item {k} differs at node widths {widths}"
    best = batch.autotune(trials=1)
    assert best.block in (64, 128, 256)
    assert best.kernel in (gbsp.BATCH_THREAD_PER_PIXEL, gbsp.BATCH_PATH_STATE,
                           gbsp.BATCH_WAVEFRONT)
    assert set(batch.node_widths()) <= {4, 8}
    print("autotuned node widths", batch.node_widths())
    for t in imgs:
        t.fill_(-1.0)
    torch.cuda.synchronize()
    batch.launch()
    for t, ref in zip(imgs, refs):
        assert np.array_equal(t.cpu().numpy().view(np.uint32), ref.view(np.uint32))
    batch.close()


def test_batch_rejects_tile_sequential(gpu_lib):
    import torch

    rt = gbsp.Runtime()
    s = small_batch_scenes()[0]
    o = gbsp.default_options(spp=1, rng_mode=gbsp.RNG_TILE_SEQUENTIAL)
    scene, ms, rend = gbsp.upload_scene(rt, s, o)
    img = torch.zeros((s.height, s.width, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(gbsp.GbspError, match="hash-per-sample"):
        gbsp.Batch(rt, [rend], [img.data_ptr()])
