"""Generates the golden fixtures of this directory from the oracle.

The reference has no tests or golden vectors for this path and cannot be
built or run here, so these fixtures pin the oracle restatement against
regressions (and the CUDA path against them): build_vectors.npz holds seeded
build_tl_bvh / build_bl_bvh inputs with their node arrays and prim orders;
frame_tiny.npz holds a 48x32 frame (2 chunks, 3 bounces, ReSTIR with spatial
reuse, 2 frames) with its camera stored explicitly.

Run: python tests/golden/gen_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "vulkan-voxel-restir-gi_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
import vrg  # noqa: E402
from helpers import random_aabbs, random_tris  # noqa: E402


def build_vectors():
    out = {}
    cases = [(1, 1, False), (2, 2, False), (3, 3, True), (4, 33, True), (5, 257, False), (6, 1000, True)]
    for k, (seed, n, grid) in enumerate(cases):
        rng = np.random.default_rng(seed)
        aabbs = random_aabbs(rng, n, grid=grid)
        power = rng.random(n).astype(np.float32)
        ids = rng.permutation(10 * n)[:n].astype(np.uint32)
        tr = (rng.integers(-3, 3, (n, 3)) * 32).astype(np.float32)
        nodes, order = oracle.build_tl_bvh(aabbs, power, ids, tr)
        out.update({f"tl{k}_aabbs": aabbs, f"tl{k}_power": power, f"tl{k}_ids": ids, f"tl{k}_tr": tr,
                    f"tl{k}_nodes": nodes, f"tl{k}_order": order})
    out["n_tl"] = np.array(len(cases))
    bl_cases = [(21, 1), (22, 2), (23, 17), (24, 300)]
    for k, (seed, n) in enumerate(bl_cases):
        rng = np.random.default_rng(seed)
        tris = random_tris(rng, n)
        lum = (rng.random(n) * 30).astype(np.float32)
        ids = rng.permutation(4 * n)[:n].astype(np.uint32)
        nodes, order, _, _ = oracle.build_bl_bvh(tris, lum, ids)
        out.update({f"bl{k}_tris": tris, f"bl{k}_lum": lum, f"bl{k}_ids": ids, f"bl{k}_nodes": nodes,
                    f"bl{k}_order": order})
    out["n_bl"] = np.array(len(bl_cases))
    np.savez_compressed(os.path.join(HERE, "build_vectors.npz"), **out)


TINY = dict(seed=77, nx=2, nz=1, emissive=0.03, W=48, H=32, nb=3)


def tiny_frame():
    t = TINY
    mats, n = vrg.terrain_materials(t["seed"])
    world = vrg.terrain_blocks(t["seed"], t["nx"], t["nz"], t["emissive"])
    W = oracle.build_world(mats, n, world)
    R = oracle.Renderer(t["W"], t["H"], t["nb"])
    out = {"blocks": world}
    for f in range(2):
        cam = vrg.orbit_camera(t["nx"], t["nz"], f, 16, t["W"], t["H"])
        camv = np.array(list(cam.eye) + list(cam.front) + list(cam.right) + list(cam.up), np.float32)
        p = vrg.RenderParams(1, 1, 4, t["nb"], vrg.MODE_PARITY, 0, 100 + f, 200 + f, 15.0, 0, 3, 0, 0)
        R.render(W, cam, p)
        img, view = R.image()
        out[f"f{f}_camera"] = camv
        out[f"f{f}_image"] = img
        out[f"f{f}_hit"] = R.readback(vrg.DBG_HIT, t["nb"])
        out[f"f{f}_radiance"] = R.readback(vrg.DBG_RADIANCE, t["nb"])
        out[f"f{f}_temporal"] = R.readback(vrg.DBG_TEMPORAL, t["nb"])
        out[f"f{f}_final"] = R.readback(vrg.DBG_FINAL, t["nb"])
    out["light_tl"] = W.read_tl(0)
    out["geo_tl"] = W.read_tl(1)
    np.savez_compressed(os.path.join(HERE, "frame_tiny.npz"), **out)
    R.close()
    W.close()


if __name__ == "__main__":
    build_vectors()
    tiny_frame()
    print("wrote", sorted(f for f in os.listdir(HERE) if f.endswith(".npz")))
