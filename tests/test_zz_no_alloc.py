"""The no-allocation build entry point, vrg_build_tl_bvh_noalloc.

Some callers cannot allocate device memory while they run (an engine that
owns the device-memory budget, a streaming worker next to a frame in flight),
so this entry point builds with scratch held in a fixed array inside the
library.  Checked through the C ABI against the allocating entry point,
vrg_build_tl_bvh_batched, and against the oracle's build_tl_bvh, on calls in
a row (each one runs on scratch left over by the one before): node arrays and
primitive order must match bit for bit (tolerance 0, the tolerance of every
BVH parity test here).  The sizes include roots of one, two and three prims
and the capacity edge, 32768 prims.  This file is collected last so that a
run stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(rng, n, grid):
    if grid:
        lo = rng.integers(0, 32, size=(n, 3)).astype(np.float32)
        hi = lo + 1.0
    else:
        lo = (rng.random((n, 3)) * 100.0).astype(np.float32)
        hi = lo + (rng.random((n, 3)) * 3.0).astype(np.float32)
    aabbs = np.concatenate([lo, hi], axis=1).astype(np.float32)
    power = (rng.random(n) * 10.0).astype(np.float32)
    ids = rng.permutation(1 << 20)[:n].astype(np.uint32)
    return aabbs, power, ids


def _reference_build(lib, vrg, ctx, aabbs, power, ids):
    n = len(aabbs)
    cnt = np.array([n], np.uint32)
    zero = np.zeros(1, np.uint32)
    tr = np.zeros((n, 3), np.float32)
    nodes = np.zeros(2 * n - 1, dtype=vrg.NODE_DTYPE)
    order = np.zeros(n, np.uint32)
    P = vrg._ptr
    vrg.check(lib.vrg_build_tl_bvh_batched(ctx.h, 1, P(cnt), P(zero), P(zero), P(tr), P(aabbs), P(power), P(ids),
                                           P(nodes), P(order)), "vrg_build_tl_bvh_batched")
    return nodes, order


def test_noalloc_matches_allocating_build_twice(vrglib, orc):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    vrg = vrglib
    lib = vrg.load_library()
    fn = lib.vrg_build_tl_bvh_noalloc
    fn.restype = C.c_int32
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]
    ctx = vrg.Context(0)
    try:
        rng = np.random.default_rng(2024)
        dev = torch.device("cuda:0")
        stream = torch.cuda.current_stream(dev)
        # calls in a row: a large grid-of-voxels set, then a smaller random set,
        # so the second call runs on scratch left over by the first; then the
        # small roots (1, 2 and 3 prims) and the capacity edge
        for n, grid in ((20000, True), (3001, False), (1, False), (2, True), (3, False), (32768, True),
                        (3, True)):
            aabbs, power, ids = _inputs(rng, n, grid)
            ref_nodes, ref_order = _reference_build(lib, vrg, ctx, aabbs, power, ids)
            d_aabbs = torch.from_numpy(aabbs).to(dev)
            d_power = torch.from_numpy(power).to(dev)
            d_ids = torch.from_numpy(ids.view(np.int32)).to(dev)
            d_nodes = torch.zeros((2 * n - 1) * 10, dtype=torch.int32, device=dev)
            d_order = torch.zeros(n, dtype=torch.int32, device=dev)
            torch.cuda.synchronize(dev)
            st = fn(d_aabbs.data_ptr(), d_power.data_ptr(), d_ids.data_ptr(), n, d_nodes.data_ptr(),
                    d_order.data_ptr(), stream.cuda_stream)
            assert st == 0, lib.vrg_last_error()
            torch.cuda.synchronize(dev)
            nodes = d_nodes.cpu().numpy().view(vrg.NODE_DTYPE)
            order = d_order.cpu().numpy().view(np.uint32)
            assert nodes.tobytes() == ref_nodes.tobytes(), f"node array differs (n={n})"
            assert np.array_equal(order, ref_order), f"prim order differs (n={n})"
            o_nodes, o_order = orc.build_tl_bvh(aabbs, power, ids)
            assert nodes.tobytes() == o_nodes.tobytes(), f"node array differs from the oracle (n={n})"
            assert np.array_equal(order, o_order), f"prim order differs from the oracle (n={n})"
    finally:
        ctx.close()


def test_noalloc_rejects_oversize(vrglib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = vrglib.load_library()
    fn = lib.vrg_build_tl_bvh_noalloc
    fn.restype = C.c_int32
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]
    dummy = torch.zeros(16, dtype=torch.float32, device="cuda:0")
    p = dummy.data_ptr()
    st = fn(p, p, p, 32769, p, p, None)
    assert st == vrglib.ERR_INVALID_ARGUMENT
    assert b"capacity" in lib.vrg_last_error()
