"""Scenes shared by the golden-vector script and the tests (host logic)."""

import numpy as np

import pyoracle as po
from vk_cinematic_gb300 import scenes


def build_world(kind: str, s: scenes.Scene) -> po.World:
    w = po.World(kind)
    for v, i, sm in s.meshes:
        w.add_mesh(v, i, sm)
    for ob in s.objects:
        w.add_object(ob.mesh, ob.material, ob.position, ob.rotation, ob.scale)
    w.build()
    for mid, m in s.materials.items():
        w.register_material(po.material(**m), mid)
    for tid, tex in s.textures.items():
        w.register_texture(tex, tid)
    w.set_background(s.background)
    w.set_options(spp=s.spp)
    return w


def textured_scene() -> scenes.Scene:
    """Config-1 geometry with a checkerboard albedo texture on the ground, an
    equirect environment texture as background emission and a smooth-shaded
    sphere (sp_material_system.cpp:59-105, image.h:3-18, sp_scene.cpp:206-214)."""
    s = scenes.config1_scene(width=48, height=40, spp=4, seed=7)
    s.meshes[0] = (s.meshes[0][0], s.meshes[0][1], True)
    chk = np.zeros((8, 8, 4), np.float32)
    yy, xx = np.mgrid[0:8, 0:8]
    chk[..., 0:3] = np.where(((xx + yy) % 2 == 0)[..., None], 0.9, 0.1)
    chk[..., 3] = 1
    env = np.zeros((16, 32, 4), np.float32)
    vv, uu = np.mgrid[0:16, 0:32]
    env[..., 0] = 0.2 + uu / 32.0
    env[..., 1] = 0.3 + vv / 16.0
    env[..., 2] = 0.5
    env[..., 3] = 1
    s.textures = {5: chk, 9: env}
    s.materials = {0: scenes.material(emission_texture=9),
                   1: scenes.material(albedo=(0.8, 0.8, 0.8)),
                   2: scenes.material(albedo_texture=5, roughness=0.3)}
    s.objects[1].material = 2
    return s
