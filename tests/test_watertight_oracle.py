"""The watertight triangle test of the oracle port (Woop, Benthin and Wald,
JCGT 2013): same hits as Moller-Trumbore away from edges, and no ray aimed
at a shared edge or vertex of a closed mesh slips through."""

import numpy as np
import pytest

from oracle import pyoracle
from vk_cinematic_gb300 import scenes


@pytest.fixture(scope="module")
def port():
    pyoracle.build_port()
    return pyoracle.Oracle("port")


def test_interior_hits_agree_with_mt(port):
    rng = np.random.default_rng(11)
    agree = 0
    n = 2000
    for _ in range(n):
        a, b, c = rng.uniform(-1, 1, (3, 3)).astype(np.float32)
        bary = rng.dirichlet([1, 1, 1])
        bary = 0.05 + 0.85 * bary  # away from the edges
        bary /= bary.sum()
        target = (bary[0] * a + bary[1] * b + bary[2] * c).astype(np.float32)
        o = (target + rng.normal(0, 3, 3)).astype(np.float32)
        d = (target - o).astype(np.float32)
        d /= np.float32(np.linalg.norm(d))
        wt = pyoracle.ray_triangle_watertight(o, d, a, b, c)
        mt = port.ray_triangle(o, d, a, b, c)  # t, normal xyz, u, v
        mt = np.array([mt[0], mt[4], mt[5]], np.float32)
        assert (wt[0] >= 0) == (mt[0] >= 0)
        if mt[0] >= 0:
            # different rounding paths: t to 1e-4 relative, barycentrics to 1e-3 absolute
            assert np.isclose(wt[0], mt[0], rtol=1e-4)
            assert np.allclose(wt[1:], mt[1:], atol=1e-3)
            agree += 1
    assert agree > n // 3  # about half are back faces (culled by both)


def closest(world, rays):
    t, obj, tri = world.closest_brute(rays)
    return t, tri


def edge_rays(level=2, seed=3):
    """Rays from outside a unit icosphere aimed at its edge midpoints and
    vertices (points computed in float32 from the mesh itself)."""
    v, i = scenes.icosphere(level)
    pos = v[:, :3]
    tri = i.reshape(-1, 3)
    pts = []
    for f in tri:
        for k in range(3):
            p, q = pos[f[k]], pos[f[(k + 1) % 3]]
            pts.append(((p + q) * np.float32(0.5)).astype(np.float32))
            pts.append(p)
    pts = np.unique(np.array(pts, np.float32), axis=0)
    rng = np.random.default_rng(seed)
    origins = []
    for p in pts:
        n = p / np.linalg.norm(p)
        jitter = rng.normal(0, 0.3, 3)
        origins.append((p + 3.0 * (n + jitter)).astype(np.float32))
    origins = np.array(origins, np.float32)
    d = pts - origins
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    # keep rays that cross the surface: a ray grazing the silhouette may touch
    # only a back face there, which culling rightly rejects
    normal = pts / np.linalg.norm(pts, axis=1, keepdims=True)
    keep = -(d * normal).sum(axis=1) > 0.3
    return np.concatenate([origins, d], axis=1)[keep].astype(np.float32), v, i


def test_no_ray_slips_through_shared_edges(port):
    rays, v, i = edge_rays()
    res = {}
    for wt in (False, True):
        w = pyoracle.World("port")
        w.set_build_bvh(False)
        w.set_watertight(wt)
        w.add_mesh(v, i)
        w.add_object(0, 1, (0, 0, 0), (0, 0, 0, 1), (1, 1, 1))
        w.build()
        t, tri = closest(w, rays)
        res[wt] = int((tri < 0).sum())
    print(f"edge/vertex rays {len(rays)}: misses MT {res[False]}, watertight {res[True]}")
    assert res[True] == 0
