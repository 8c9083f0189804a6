"""Shared helpers of the parity tests: identical inputs for the CUDA library
(through the C ABI) and the oracle."""
import numpy as np

import oracle
import vrg


def random_aabbs(rng, n, scale=64.0, grid=False):
    if grid:
        lo = rng.integers(0, 32, size=(n, 3)).astype(np.float32)
        hi = lo + 1.0
    else:
        lo = (rng.random((n, 3)) * scale).astype(np.float32)
        hi = lo + (rng.random((n, 3)) * 4.0).astype(np.float32)
    return np.concatenate([lo, hi], axis=1).astype(np.float32)


def random_tris(rng, n, scale=32.0):
    base = (rng.random((n, 1, 3)) * scale).astype(np.float32)
    d = (rng.random((n, 3, 3)) * 2.0 - 1.0).astype(np.float32)
    return (base + d).reshape(n, 9).astype(np.float32)


def gpu_build_tl(ctx, sets):
    """sets: list of (aabbs (n,6), power (n,), ids (n,), translations (n,3) or None)."""
    lib = ctx.lib
    n = np.array([len(s[0]) for s in sets], np.uint32)
    poff = np.concatenate([[0], np.cumsum(n)[:-1]]).astype(np.uint32)
    nn = np.maximum(2 * n.astype(np.int64) - 1, 0)
    noff = np.concatenate([[0], np.cumsum(nn)[:-1]]).astype(np.uint32)
    aabbs = np.concatenate([s[0] for s in sets]).astype(np.float32)
    power = np.concatenate([s[1] for s in sets]).astype(np.float32)
    ids = np.concatenate([s[2] for s in sets]).astype(np.uint32)
    tr = np.concatenate([s[3] if s[3] is not None else np.zeros((len(s[0]), 3), np.float32)
                         for s in sets]).astype(np.float32)
    nodes = np.zeros(int(nn.sum()), dtype=vrg.NODE_DTYPE)
    order = np.zeros(int(n.sum()), np.uint32)
    P = vrg._ptr
    vrg.check(lib.vrg_build_tl_bvh_batched(ctx.h, len(sets), P(n), P(poff), P(noff), P(tr), P(aabbs), P(power),
                                           P(ids), P(nodes), P(order)), "tl batched")
    return [(nodes[noff[i]:noff[i] + nn[i]], order[poff[i]:poff[i] + n[i]]) for i in range(len(sets))]


def gpu_build_bl(ctx, sets):
    """sets: list of (tris (n,9), lum (n,), ids (n,))."""
    lib = ctx.lib
    n = np.array([len(s[0]) for s in sets], np.uint32)
    poff = np.concatenate([[0], np.cumsum(n)[:-1]]).astype(np.uint32)
    nn = np.maximum(2 * n.astype(np.int64) - 1, 0)
    noff = np.concatenate([[0], np.cumsum(nn)[:-1]]).astype(np.uint32)
    tris = np.concatenate([s[0] for s in sets]).astype(np.float32)
    lum = np.concatenate([s[1] for s in sets]).astype(np.float32)
    ids = np.concatenate([s[2] for s in sets]).astype(np.uint32)
    nodes = np.zeros(int(nn.sum()), dtype=vrg.NODE_DTYPE)
    order = np.zeros(int(n.sum()), np.uint32)
    P = vrg._ptr
    vrg.check(lib.vrg_build_bl_bvh_batched(ctx.h, len(sets), P(n), P(poff), P(noff), P(lum), P(tris), P(ids),
                                           P(nodes), P(order)), "bl batched")
    return [(nodes[noff[i]:noff[i] + nn[i]], order[poff[i]:poff[i] + n[i]]) for i in range(len(sets))]


def nodes_equal(a, b):
    """bit-exact comparison of two node arrays."""
    return a.shape == b.shape and a.tobytes() == b.tobytes()


def first_node_diff(a, b):
    ab = a.view(np.uint8).reshape(len(a), -1)
    bb = b.view(np.uint8).reshape(len(b), -1)
    d = np.nonzero((ab != bb).any(axis=1))[0]
    return None if len(d) == 0 else (int(d[0]), a[d[0]], b[d[0]])


def terrain_world(seed, nx, nz, emissive):
    mats, n = vrg.terrain_materials(seed)
    world = vrg.terrain_blocks(seed, nx, nz, emissive)
    return mats, n, world


def params(nee=1, view=0, spatial=0, nb=2, mode=vrg.MODE_PARITY, seeds=(11, 22, 33), radius=15.0, m_cap=0,
           slots=3, accumulate=0, flags=vrg.RENDER_CAPTURE):
    return vrg.RenderParams(nee, view, spatial, nb, mode, seeds[0], seeds[1], seeds[2], radius, m_cap, slots,
                            accumulate, flags)


SLICES = [(vrg.DBG_HIT, "hit"), (vrg.DBG_ORIGIN, "origin"), (vrg.DBG_DIRECTION, "direction"),
          (vrg.DBG_NORMAL, "normal"), (vrg.DBG_EMISSIVITY, "emissivity"), (vrg.DBG_REFLECTIVITY, "reflectivity"),
          (vrg.DBG_MIS, "mis"), (vrg.DBG_BSDF_PDF, "bsdf_pdf"), (vrg.DBG_NEE_PDF, "nee_pdf"),
          (vrg.DBG_RADIANCE, "radiance"), (vrg.DBG_Q, "q"), (vrg.DBG_TEMPORAL, "temporal"),
          (vrg.DBG_SPATIAL, "spatial"), (vrg.DBG_FINAL, "final")]


def compare_frame(gpu_r, orc_r, nb):
    """Returns {name: number of mismatching elements} over every captured slice:
    bit-exact, except that any NaN equals any NaN.  The reference's arithmetic
    makes a NaN in rare cases (a reservoir whose sample has negative luminance
    gets w_sum / (Z * p_hat) = 0 / -0), and the encoding of a NaN made by an
    invalid operation is the platform's: 0x7FFFFFFF on the GPU, 0x7FC00000 on
    an Arm host, 0xFFC00000 on an x86 host."""
    out = {}
    for what, name in SLICES:
        g = gpu_r.readback(what, nb)
        o = orc_r.readback(what, nb)
        diff = g.view(np.uint32) != o.view(np.uint32)
        if g.dtype == np.float32:
            diff &= ~(np.isnan(g) & np.isnan(o))
        out[name] = int(diff.sum())
    return out
