"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Runs the reference harness (oracle/_ref/libspref.so, the unmodified
vk_cinematic sources compiled in place by oracle/Makefile) on seeded inputs
and stores inputs + outputs.  Needs an x86-64 host with the reference tree
mounted:

    python tests/golden/make_golden.py [--reference /path/to/vk_cinematic]

The fixtures pin the oracle port (tests/test_oracle_golden.py) and, through
it, the GPU path.  Values from the reference's own unit tests are included
as named cases next to the randomised ones.
"""

from __future__ import annotations

import argparse
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle as po  # noqa: E402
sys.path.insert(0, os.path.join(ROOT, "tests"))
from golden_scenes import build_world, textured_scene  # noqa: E402
from vk_cinematic_gb300 import scenes  # noqa: E402

RNG_SEEDS = [0xF51C0E49, 123456789, 0x1A34C249, 1, 0xFFFFFFFF, 0x80000000]


def gen_primitives(o: po.Oracle, rng: np.random.Generator) -> dict:
    out = {}
    # RNG streams (math_utils.h:184-214)
    for which in ("xorshift", "uni", "bi"):
        out[f"rng_{which}"] = np.stack([o.rng_sequence(s, 64, which) for s in RNG_SEEDS])
    out["rng_seeds"] = np.array(RNG_SEEDS, np.uint32)

    # Camera (unit_tests/test_simd_path_tracer.cpp:137-200 plus the config-1 camera)
    cams = [
        (4, 2, (0, 2, 0), (0, 0, 0, 1), 0.1),
        (4, 4, (0, 2, 0), (0, 0, 0, 1), 0.1),
        (128, 128, (0, 1, 3), tuple(scenes.quat_axis_angle((1, 0, 0), -math.atan(1 / 3))), 0.5),
        (1920, 1080, (0, 6, 18), tuple(scenes.look_rotation_x((0, 6, 18), (0, 1, 0))), 0.5),
        (77, 131, (1.5, -2, 7), tuple(scenes.quat_axis_angle((0.6, 0.8, 0), 0.7)), 0.3),
    ]
    cam_in = np.zeros((len(cams), 10), np.float32)
    cam_out = np.zeros((len(cams), 19), np.float32)
    pix = np.concatenate([np.array([[0.5, 0.5], [1.5, 0.5], [0.5, 1.5], [3.5, 3.5]], np.float32),
                          rng.uniform(0, 4, (28, 2)).astype(np.float32)])
    film = np.zeros((len(cams), len(pix), 3), np.float32)
    for k, (w, h, p, r, f) in enumerate(cams):
        cam_in[k] = [w, h, *p, *r, f]
        cam_out[k] = o.configure_camera(w, h, p, r, f)
        film[k] = o.film_positions(w, h, p, r, f, pix * np.float32(max(w, h) / 4))
    out.update(camera_in=cam_in, camera_out=cam_out, film_pixels=pix, film_out=film)

    # Moller-Trumbore (ray_intersection.cpp:156-190); unit_tests/unit_tests.cpp:348-426
    named = [
        ((0, 0, 1), (0, 0, -1), (-0.5, -0.5, -5), (0.5, -0.5, -5), (0, 0.5, -5)),
        ((0, 0, 1), (0, 0, -1), (4.5, -0.5, -5), (5.5, -0.5, -5), (5, 0.5, -5)),
        ((0, 0, 1), (0, 0, -1), (0, 0, -5), (1, 0, -5), (0.5, 1, -5)),
        ((0.5, 0.5, 1), (0, 0, -1), (-0.5, -0.5, -5), (0.5, -0.5, -5), (0, 0.5, -5)),
    ]
    n = 4000
    tri = rng.normal(size=(n, 3, 3)).astype(np.float32)
    org = rng.normal(size=(n, 3)).astype(np.float32) * np.float32(3)
    tgt = tri.mean(1) + rng.normal(size=(n, 3)).astype(np.float32) * np.float32(0.4)
    d = tgt - org
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    tri_in = np.zeros((len(named) + n, 15), np.float32)
    for k, c in enumerate(named):
        tri_in[k] = np.concatenate([np.asarray(x, np.float32) for x in c])
    tri_in[len(named):, 0:3] = org
    tri_in[len(named):, 3:6] = d
    tri_in[len(named):, 6:15] = tri.reshape(n, 9)
    tri_out = np.stack([o.ray_triangle(r[0:3], r[3:6], r[6:9], r[9:12], r[12:15]) for r in tri_in])
    out.update(tri_in=tri_in, tri_out=tri_out)

    # 4-box slab test (simd.h:198-271); test_simd_path_tracer.cpp:440-486
    box_cases = []
    mins = np.array([[-0.5, -0.5, -0.5], [-0.5, -0.5, 1.0], [-0.5, -0.5, 2.5], [-0.5, -0.5, 4.0]],
                    np.float32)
    maxs = np.array([[0.5, 0.5, 0.5], [0.5, 0.5, 2.0], [0.5, 0.5, 3.5], [0.5, 0.5, 5.0]], np.float32)
    for dd in [(0, 0, -1), (1, 0, 0), (0, 0, 1)]:
        box_cases.append((mins, maxs, np.array([0, 0, 10], np.float32), np.asarray(dd, np.float32)))
    bug_min = np.array([[-0.375038534, 0.843911469, 0.264082730], [0, 0, 0], [0, 0, 0], [0, 0, 0]],
                       np.float32)
    bug_max = np.array([[-0.238676921, 0.916244209, 0.386187375], [0, 0, 0], [0, 0, 0], [0, 0, 0]],
                       np.float32)
    box_cases.append((bug_min, bug_max, np.array([-2.68516445, -1.71131170, -1.71610022], np.float32),
                      np.array([0.576836348, 0.652352035, 0.491626590], np.float32)))
    for _ in range(4000):
        c = rng.normal(size=(4, 3)).astype(np.float32)
        e = np.abs(rng.normal(size=(4, 3))).astype(np.float32) * np.float32(0.5)
        if rng.random() < 0.2:
            e[:, rng.integers(0, 3)] = 0  # flat boxes, like the ground quad
        org = rng.normal(size=3).astype(np.float32) * np.float32(3)
        dd = rng.normal(size=3).astype(np.float32)
        if rng.random() < 0.05:
            dd[rng.integers(0, 3)] = 0  # axis-parallel directions (infinite inverse)
        box_cases.append(((c - e).astype(np.float32), (c + e).astype(np.float32), org, dd))
    box_in = np.zeros((len(box_cases), 30), np.float32)
    box_out = np.zeros(len(box_cases), np.uint32)
    with np.errstate(divide="ignore"):
        for k, (mn, mx, org, dd) in enumerate(box_cases):
            invd = (np.float32(1) / dd).astype(np.float32)
            box_in[k] = np.concatenate([mn.reshape(-1), mx.reshape(-1), org, invd])
            box_out[k] = o.aabb4(mn, mx, org, invd)
    out.update(aabb4_in=box_in, aabb4_out=box_out)

    # Hemisphere sampling chain (test_simd_path_tracer.cpp:530-544) + random normals
    st = 123456789
    nrm = np.array([0, -1, 0], np.float32)
    hemi_out = []
    for k in range(1000):
        v, st2 = o.hemisphere(st, nrm)
        hemi_out.append(v)
        nrm, st = v, st2
    hemi_states = np.zeros(2000, np.uint32)
    hemi_normals = np.zeros((2000, 3), np.float32)
    hemi_dirs = np.zeros((2000, 3), np.float32)
    hemi_next = np.zeros(2000, np.uint32)
    for k in range(2000):
        s0 = int(rng.integers(1, 2**32 - 1))
        nn = rng.normal(size=3)
        nn = (nn / np.linalg.norm(nn)).astype(np.float32)
        v, s1 = o.hemisphere(s0, nn)
        hemi_states[k], hemi_normals[k], hemi_dirs[k], hemi_next[k] = s0, nn, v, s1
    out.update(hemi_chain=np.stack(hemi_out), hemi_states=hemi_states, hemi_normals=hemi_normals,
               hemi_dirs=hemi_dirs, hemi_next=hemi_next)

    # Object transforms (sp_scene.cpp:77-117, aabb.h:29-58)
    xf_in = np.zeros((64, 16), np.float32)
    xf_out = np.zeros((64, 38), np.float32)
    for k in range(64):
        bmin = rng.normal(size=3).astype(np.float32)
        bmax = bmin + np.abs(rng.normal(size=3)).astype(np.float32)
        pos = rng.normal(size=3).astype(np.float32) * np.float32(5)
        ax = rng.normal(size=3)
        rot = scenes.quat_axis_angle(ax / np.linalg.norm(ax), float(rng.uniform(-3, 3)))
        sc = np.float32(np.exp(rng.uniform(-2, 2)))
        scale = np.array([sc, sc, sc], np.float32)
        xf_in[k] = np.concatenate([bmin, bmax, pos, rot, scale])
        m, inv = o.object_matrices(pos, rot, scale)
        xf_out[k] = np.concatenate([o.transform_aabb(bmin, bmax, pos, rot, scale), m, inv])
    out.update(xform_in=xf_in, xform_out=xf_out)
    return out


def gen_bvh(o: po.Oracle, rng: np.random.Generator) -> dict:
    """Agglomerative build + all-hits query (bvh.cpp:51-311); inputs from
    unit_tests/test_bvh.cpp:36-292 and random sets."""
    out = {}
    sets = {}
    sets["single"] = (np.full((1, 3), -0.5, np.float32), np.full((1, 3), 0.5, np.float32))
    sets["two"] = (np.array([[-0.5] * 3, [1] * 3], np.float32), np.array([[0.5] * 3, [2] * 3], np.float32))
    c = np.stack([np.arange(31, dtype=np.float32), np.zeros(31, np.float32), np.zeros(31, np.float32)], 1)
    sets["row31"] = (c - np.float32(0.25), c + np.float32(0.25))
    g = []
    for z in range(4):
        for x in range(4):
            g.append([-10 + 20 * (x / 3.0), 0, -10 + 20 * (z / 3.0)])
    g = np.array(g, np.float32)
    sets["grid16"] = (g - np.float32(0.5), g + np.float32(0.5))
    for n in (7, 64, 300):
        cc = rng.normal(size=(n, 3)).astype(np.float32) * np.float32(4)
        ee = np.abs(rng.normal(size=(n, 3))).astype(np.float32) * np.float32(0.3)
        sets[f"rand{n}"] = (cc - ee, cc + ee)
    for name, (mn, mx) in sets.items():
        out[f"bvh_{name}_min"] = mn
        out[f"bvh_{name}_max"] = mx
        out[f"bvh_{name}_tree"] = o.bvh_build_flat(mn, mx)
        lo = mn.min(0) - 2
        hi = mx.max(0) + 2
        org = rng.uniform(lo, hi, (256, 3)).astype(np.float32)
        tgt = rng.uniform(mn.min(0), mx.max(0), (256, 3)).astype(np.float32)
        d = tgt - org
        d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
        rays = np.concatenate([org, d], 1)
        if name == "grid16":
            rays[0] = [-20, 0, -10, 1, 0, 0]
        out[f"bvh_{name}_rays"] = rays
        out[f"bvh_{name}_hits"] = o.bvh_query(mn, mx, rays, 64)
    return out


def gen_scenes(rng: np.random.Generator) -> dict:
    out = {}
    s = scenes.config1_scene()
    w = build_world("ref", s)
    # scene query: camera-ish rays and random rays (sp_scene.cpp:229-339)
    org = np.concatenate([np.tile(s.camera_position, (1024, 1)),
                          rng.uniform(-3, 3, (3072, 3)).astype(np.float32) + np.float32([0, 1.5, 0])])
    tgt = np.concatenate([rng.uniform([-1.5, -0.5, -1.5], [1.5, 2.5, 1.5], (4096, 3))]).astype(np.float32)
    d = tgt - org
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    rays = np.concatenate([org, d], 1).astype(np.float32)
    res, mat, met = w.intersect(rays)
    out.update(c1_query_rays=rays, c1_query_out=res, c1_query_mat=mat, c1_query_metrics=met)
    # hash-per-sample image, full config 1
    img, nans, met, _ = w.path_trace_hashed(s.width, s.height, s.camera_position, s.camera_rotation,
                                            s.film_distance, s.seed)
    out.update(c1_hashed_image=img, c1_hashed_nans=np.uint32(nans), c1_hashed_metrics=met)
    # per-sample radiance in a 16x16 window
    reg = (56, 40, 72, 56)
    _, _, _, ps = w.path_trace_hashed(s.width, s.height, s.camera_position, s.camera_rotation,
                                      s.film_distance, s.seed, region=reg, per_sample=True)
    out.update(c1_sample_region=np.array(reg, np.uint32), c1_samples=ps)
    # the application's tile mode: 64x64 tiles, RNG reset per tile (main.cpp:731-844)
    tiles = np.zeros((s.height, s.width, 4), np.float32)
    mt = np.zeros(12, np.uint64)
    for ty in range(0, s.height, 64):
        for tx in range(0, s.width, 64):
            _, _, m = w.path_trace_tile(s.width, s.height, s.camera_position, s.camera_rotation,
                                        s.film_distance, (tx, ty, tx + 64, ty + 64), 0xF51C0E49,
                                        pixels=tiles)
            mt += m
    mt[0] = 0
    out.update(c1_tile_image=tiles, c1_tile_metrics=mt)
    w.close()

    # materials: textures, equirect background, smooth shading
    ts = textured_scene()
    w = build_world("ref", ts)
    img, nans, met, _ = w.path_trace_hashed(ts.width, ts.height, ts.camera_position,
                                            ts.camera_rotation, ts.film_distance, ts.seed)
    out.update(tex_image=img, tex_nans=np.uint32(nans), tex_metrics=met)
    # explicit paths (simd_path_tracer.cpp:107-175), incl. TestEvaluateLightPath
    # (test_simd_path_tracer.cpp:278-306), which is NaN at HEAD
    paths = np.zeros((256, 3), po.PATH_VERTEX_DTYPE)
    lens = np.zeros(256, np.uint32)
    paths[0, 0]["materialId"] = 1
    paths[0, 0]["normal"] = (0, 1, 0)
    paths[0, 0]["incomingDir"] = (0, 1, 0)
    paths[0, 1]["materialId"] = 0
    lens[0] = 2
    for k in range(1, 256):
        L = int(rng.integers(1, 4))
        lens[k] = L
        for v in range(L):
            nn = rng.normal(size=3)
            nn /= np.linalg.norm(nn)
            li = rng.normal(size=3)
            li /= np.linalg.norm(li)
            if li @ nn < 0:
                li = -li
            od = rng.normal(size=3)
            od /= np.linalg.norm(od)
            paths[k, v]["materialId"] = int(rng.choice([0, 1, 2, 77]))
            paths[k, v]["normal"] = nn
            paths[k, v]["incomingDir"] = li
            paths[k, v]["outgoingDir"] = od
            paths[k, v]["uv"] = rng.random(2)
    rad = np.stack([w.radiance_for_path(paths[k, :lens[k]]) for k in range(256)])
    out.update(path_vertices=paths, path_lengths=lens, path_radiance=rad)
    w.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=po.reference_root())
    args = ap.parse_args()
    if po.build_ref(args.reference) is None:
        sys.exit("the reference tree (x86-64 host) is needed to make golden vectors")
    o = po.Oracle("ref")
    rng = np.random.default_rng(20261203)
    prim = gen_primitives(o, rng)
    np.savez_compressed(os.path.join(HERE, "primitives.npz"), **prim)
    bvh = gen_bvh(o, rng)
    np.savez_compressed(os.path.join(HERE, "bvh.npz"), **bvh)
    sc = gen_scenes(rng)
    np.savez_compressed(os.path.join(HERE, "scenes.npz"), **sc)
    for f in ("primitives.npz", "bvh.npz", "scenes.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
