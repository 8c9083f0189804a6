"""Full-size parity: the headline workload itself, rendered by the CUDA path
and by the oracle.  The scene is the 4x4-chunk terrain of seed 20240601 with
0.5% emissive blocks; the frame is 1920x1080, 3 bounces, ReSTIR with 3
spatial neighbours in a 30 px box, M-cap 20 and a 1-slot history, on the orbit
camera.  Every captured per-bounce array (origin, direction, normal,
emissivity, reflectivity, mis weight, bsdf pdf, nee pdf, outgoing radiance,
q, hit), both reservoirs, the final target and the packed image are compared
bit for bit over two frames, the second reusing the first's reservoirs (any
NaN equal to any NaN: at this size a few reservoirs reach the reference's
0 / -0 weight, whose NaN encoding is the platform's)."""
import numpy as np
import pytest

import vrg
from helpers import compare_frame, params, terrain_world

pytestmark = pytest.mark.gpu

SEED, NX, NZ, EMISSIVE = 20240601, 4, 4, 0.005
W, H, NB = 1920, 1080, 3


def test_headline_workload_frames_bit_exact(gpu_ctx, orc):
    mats, n, world = terrain_world(SEED, NX, NZ, EMISSIVE)
    gpu_ctx.set_materials(mats, n)
    scene, objs = vrg.build_world(gpu_ctx, world)
    OW = orc.build_world(mats, n, world)
    gr = vrg.Renderer(gpu_ctx, W, H, NB)
    orr = orc.Renderer(W, H, NB)
    try:
        for f in range(2):
            cam = vrg.orbit_camera(NX, NZ, f, 64, W, H)
            p = params(nee=1, view=1, spatial=3, nb=NB, mode=vrg.MODE_CONFIG, seeds=(f, 1000 + f, 2000 + f),
                       radius=30.0, m_cap=20, slots=1)
            img, _ = gr.render_params(scene, cam, p)
            orr.render(OW, cam, p)
            oimg, _ = orr.image()
            diffs = compare_frame(gr, orr, NB)
            assert all(v == 0 for v in diffs.values()), (f, {k: v for k, v in diffs.items() if v})
            assert np.array_equal(img.reshape(-1), oimg.reshape(-1))
            assert gr.last_stats.error_flags == 0
            assert gr.last_stats.rays_closest > W * H
    finally:
        gr.close()
        OW.close()
        scene.close()
        for o in objs:
            o.release()
