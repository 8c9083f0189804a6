"""Pins the C++ oracle's restatement of bvh/build.rs: against an independent
pure-Python restatement (bit-exact on small inputs), against the committed
golden vectors, and against the structural invariants the reference asserts
or relies on (1 prim per leaf, DFS child pairs, padding, power sums)."""
import os

import numpy as np
import pytest

import py_build_ref
from helpers import random_aabbs, random_tris

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("seed,n,grid", [(1, 1, False), (2, 2, False), (3, 3, False), (4, 7, True), (5, 40, False),
                                         (6, 120, True), (7, 200, False)])
def test_tl_matches_python_restatement(orc, seed, n, grid):
    rng = np.random.default_rng(seed)
    aabbs = random_aabbs(rng, n, grid=grid)
    power = rng.random(n).astype(np.float32)
    ids = np.arange(n, dtype=np.uint32)[::-1].copy()
    tr = (rng.integers(-2, 3, (n, 3)) * 32).astype(np.float32) if seed % 2 else None
    on, oo = orc.build_tl_bvh(aabbs, power, ids, tr)
    pn, po = py_build_ref.build_tl_bvh(aabbs, power, ids, tr)
    assert on.tobytes() == pn.tobytes()
    assert np.array_equal(oo, po)


@pytest.mark.parametrize("seed,n", [(11, 1), (12, 2), (13, 5), (14, 64), (15, 150)])
def test_bl_matches_python_restatement(orc, seed, n):
    rng = np.random.default_rng(seed)
    tris = random_tris(rng, n)
    lum = (rng.random(n) * 20).astype(np.float32)
    ids = rng.permutation(1000)[:n].astype(np.uint32)
    on, oo, root, rp = orc.build_bl_bvh(tris, lum, ids)
    pn, po = py_build_ref.build_bl_bvh(tris, lum, ids)
    assert on.tobytes() == pn.tobytes()
    assert np.array_equal(oo, po)


def test_equal_centroids_fallback_split(orc):
    # all centroids equal: scale = 32/0, bins NaN -> 0, partition empty -> split_at(n/2)
    n = 9
    aabbs = np.tile(np.array([[0, 0, 0, 1, 1, 1]], np.float32), (n, 1))
    nodes, order = orc.build_tl_bvh(aabbs, np.ones(n, np.float32), np.arange(n))
    assert np.array_equal(order, np.arange(n))  # no reordering
    # root splits 4 | 5, children appended as a pair
    assert nodes[0]["left"] == 1 and nodes[0]["right"] == 2
    pn, po = py_build_ref.build_tl_bvh(aabbs, np.ones(n, np.float32), np.arange(n))
    assert nodes.tobytes() == pn.tobytes()


def _check_invariants(nodes, order, aabbs, power):
    n = len(order)
    assert len(nodes) == 2 * n - 1
    assert sorted(order.tolist()) == list(range(n))
    leaves = nodes["left"] == 0xFFFFFFFF
    assert leaves.sum() == n
    assert nodes[0]["parent"] == 0xFFFFFFFF
    for i in np.nonzero(~leaves)[0]:
        l, r = int(nodes[i]["left"]), int(nodes[i]["right"])
        assert r == l + 1 and l > i
        assert nodes[l]["parent"] == i and nodes[r]["parent"] == i
        for c in (l, r):  # padded bounds contain the children
            assert np.all(nodes[i]["min"] <= nodes[c]["min"]) and np.all(nodes[i]["max"] >= nodes[c]["max"])
        assert nodes[i]["power"] == np.float32(np.float32(0) + nodes[l]["power"]) + nodes[r]["power"]


def test_invariants_large(orc):
    rng = np.random.default_rng(99)
    n = 5000
    aabbs = random_aabbs(rng, n, grid=True)
    power = rng.random(n).astype(np.float32)
    nodes, order = orc.build_tl_bvh(aabbs, power, np.arange(n))
    _check_invariants(nodes, order, aabbs, power)


def test_golden_build_vectors(orc):
    g = np.load(os.path.join(GOLDEN, "build_vectors.npz"))
    for k in range(int(g["n_tl"])):
        nodes, order = orc.build_tl_bvh(g[f"tl{k}_aabbs"], g[f"tl{k}_power"], g[f"tl{k}_ids"], g[f"tl{k}_tr"])
        assert nodes.tobytes() == g[f"tl{k}_nodes"].tobytes(), k
        assert np.array_equal(order, g[f"tl{k}_order"])
    for k in range(int(g["n_bl"])):
        nodes, order, _, _ = orc.build_bl_bvh(g[f"bl{k}_tris"], g[f"bl{k}_lum"], g[f"bl{k}_ids"])
        assert nodes.tobytes() == g[f"bl{k}_nodes"].tobytes(), k
        assert np.array_equal(order, g[f"bl{k}_order"])
