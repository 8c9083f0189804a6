"""Handle lifetimes: the context is shared by everything made from it (as the
reference's Arc-shared queues and allocators are), so handles may be
destroyed in any order.

* The context handle destroyed first: its scene, renderer and radiance cache
  keep the context alive, render the same frame bit for bit afterwards, and
  are then destroyed one by one.
* A Python process that leaves every handle to interpreter shutdown (where
  the cycle collector may finalize the context before its children) exits
  cleanly."""
import ctypes as C
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

import vrg
from helpers import params, terrain_world

pytestmark = pytest.mark.gpu

W, H = 48, 32


def test_context_destroyed_before_children():
    ctx = vrg.Context(0)
    lib = ctx.lib
    mats, n, blocks = terrain_world(52, 2, 1, 0.01)
    ctx.set_materials(mats, n)
    scene, objs = vrg.build_world(ctx, blocks)
    lt, gtl = scene.get_tlas()
    r = vrg.Renderer(ctx, W, H, 3)
    cache = vrg.RadianceCache(ctx, gtl[0]["min"], gtl[0]["max"], seed=5)
    cam = vrg.orbit_camera(2, 1, 3, 64, W, H)
    p = params(nee=1, view=1, spatial=2, nb=3, seeds=(1, 2, 3), flags=0)
    blob = r.save_state()
    img0, _ = r.render_params(scene, cam, p)
    q = cache.query(np.array([[1.0, 20.0, 1.0]], np.float32), np.array([[0.0, 1.0, 0.0]], np.float32),
                    np.array([[0.0, -1.0, 0.0]], np.float32))
    # the context handle goes first; the Python wrapper forgets it
    assert lib.vrg_context_destroy(ctx.h) == 0
    ctx.h = C.c_void_p()
    r.load_state(blob)  # the same frame again: same frame counter and reservoir history
    img1, _ = r.render_params(scene, cam, p)
    assert np.array_equal(img0, img1)
    q1 = cache.query(np.array([[1.0, 20.0, 1.0]], np.float32), np.array([[0.0, 1.0, 0.0]], np.float32),
                     np.array([[0.0, -1.0, 0.0]], np.float32))
    assert np.array_equal(q, q1)
    # children in an arbitrary order; the last one frees the context
    r.close()
    for o in objs:
        o.release()
    cache.close()
    scene.close()


def test_interpreter_shutdown_in_any_order():
    here = os.path.dirname(os.path.abspath(__file__))
    pkg = os.path.join(os.path.dirname(here), "vulkan-voxel-restir-gi_gb300")
    code = textwrap.dedent(f"""
        import sys
        sys.path[:0] = [{here!r}, {pkg!r}]
        import numpy as np
        import vrg
        from helpers import params, terrain_world
        ctx = vrg.Context(0)
        mats, n, blocks = terrain_world(53, 2, 2, 0.01)
        ctx.set_materials(mats, n)
        scene, objs = vrg.build_world(ctx, blocks)
        lt, gtl = scene.get_tlas()
        r = vrg.Renderer(ctx, {W}, {H}, 3)
        cache = vrg.RadianceCache(ctx, gtl[0]["min"], gtl[0]["max"], seed=5)
        r.set_cache(cache)
        cam = vrg.orbit_camera(2, 2, 1, 64, {W}, {H})
        for f in range(3):
            r.render_params(scene, cam, params(nee=1, view=1, spatial=2, nb=3, seeds=(f, 2, 3), flags=vrg.RENDER_CACHE))
        # a reference cycle through the cache: the cycle collector finalizes
        # these objects, and the context, in an order of its own at shutdown
        cache.cycle = [cache, r, scene, ctx]
        print("rendered", flush=True)
    """)
    res = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, (res.returncode, res.stdout[-500:], res.stderr[-2000:])
    assert "rendered" in res.stdout
