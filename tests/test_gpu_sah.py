"""GPU binned-SAH builder vs the oracle restatement of bvh/build.rs:
node arrays (40-byte BvhNode) and primitive order bit-exact."""
import numpy as np
import pytest

from helpers import first_node_diff, gpu_build_bl, gpu_build_tl, nodes_equal, random_aabbs, random_tris

pytestmark = pytest.mark.gpu


def _check_tl(gpu_ctx, orc, sets):
    res = gpu_build_tl(gpu_ctx, sets)
    for (aabbs, power, ids, tr), (gn, go) in zip(sets, res):
        on, oo = orc.build_tl_bvh(aabbs, power, ids, tr)
        assert nodes_equal(gn, on), first_node_diff(gn, on)
        assert np.array_equal(go, oo)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 17, 100, 1000])
def test_tl_small_sizes(gpu_ctx, orc, n):
    rng = np.random.default_rng(n)
    aabbs = random_aabbs(rng, n)
    _check_tl(gpu_ctx, orc, [(aabbs, rng.random(n).astype(np.float32), np.arange(n), None)])


def test_tl_voxel_grid_ties(gpu_ctx, orc):
    # unit boxes on an integer grid: many equal centroids, equal costs, fallback splits
    rng = np.random.default_rng(7)
    sets = []
    for n in (3, 50, 700, 5000):
        aabbs = random_aabbs(rng, n, grid=True)
        sets.append((aabbs, np.zeros(n, np.float32), rng.integers(0, 32768, n).astype(np.uint32), None))
    _check_tl(gpu_ctx, orc, sets)


def test_tl_all_same_centroid(gpu_ctx, orc):
    # every centroid equal: scale = 32/0 -> bins NaN -> 0, half-split fallback
    n = 37
    aabbs = np.tile(np.array([[1, 2, 3, 2, 3, 4]], np.float32), (n, 1))
    _check_tl(gpu_ctx, orc, [(aabbs, np.ones(n, np.float32), np.arange(n), None)])


def test_tl_translated_batch(gpu_ctx, orc):
    rng = np.random.default_rng(3)
    sets = []
    for k in range(12):
        n = int(rng.integers(1, 400))
        tr = (rng.integers(-4, 4, (n, 3)) * 32).astype(np.float32)
        sets.append((random_aabbs(rng, n), rng.random(n).astype(np.float32) * 100, np.arange(n), tr))
    _check_tl(gpu_ctx, orc, sets)


def test_tl_large(gpu_ctx, orc):
    rng = np.random.default_rng(11)
    n = 60000
    aabbs = random_aabbs(rng, n, scale=1024.0)
    _check_tl(gpu_ctx, orc, [(aabbs, rng.random(n).astype(np.float32), np.arange(n), None)])


@pytest.mark.parametrize("n", [1, 2, 3, 9, 128, 3000])
def test_bl_triangles(gpu_ctx, orc, n):
    rng = np.random.default_rng(100 + n)
    tris = random_tris(rng, n)
    lum = (rng.random(n) * 50).astype(np.float32)
    ids = rng.permutation(n * 2)[:n].astype(np.uint32)
    (gn, go), = gpu_build_bl(gpu_ctx, [(tris, lum, ids)])
    on, oo, _, _ = orc.build_bl_bvh(tris, lum, ids)
    assert nodes_equal(gn, on), first_node_diff(gn, on)
    assert np.array_equal(go, oo)
