"""Neural radiance cache: the CUDA forward and gradients against the PyTorch
CPU oracle (tests/nrc_ref.py), and training convergence."""
import numpy as np
import pytest

import vrg
from nrc_ref import Model, corners

pytestmark = pytest.mark.gpu

LO, HI = (0.0, 0.0, 0.0), (64.0, 32.0, 64.0)


def _samples(rng, n):
    pos = (rng.random((n, 3)) * np.array(HI)).astype(np.float32)
    face = rng.integers(0, 6, n)
    nrm = np.zeros((n, 3), np.float32)
    nrm[np.arange(n), face // 2] = np.where(face % 2, 1.0, -1.0)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    target = (np.abs(np.sin(pos[:, :1] * 0.2)) * np.array([[2.0, 1.0, 0.5]]) + 0.1).astype(np.float32)
    return pos, nrm, d.astype(np.float32), target


# the two training kernels: tcgen05 (128-sample tiles, tensor-memory
# accumulators; the default) and the warp-level mma.sync kernel
TRAIN = {"tcgen05": 0, "mma_sync": vrg.NRC_TRAIN_WARP_MMA}


def _cache(gpu_ctx, levels=8, log2_t=12, seed=3, flags=0):
    return vrg.RadianceCache(gpu_ctx, LO, HI, levels=levels, log2_table=log2_t, base_resolution=4,
                             max_resolution=128, batch=4096, learning_rate=1e-2, seed=seed, flags=flags)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_forward_matches_oracle(gpu_ctx):
    rng = np.random.default_rng(1)
    c = _cache(gpu_ctx)
    pos, nrm, d, _ = _samples(rng, 777)
    # non-trivial table values
    tab = (rng.normal(size=c.levels * (1 << c.log2_table) * 2) * 0.5).astype(np.float32)
    c.write(vrg.NRC_TABLE, tab)
    y = c.query(pos, nrm, d)
    sc, dn, r1 = c.layout()
    m = Model(c.read(vrg.NRC_WEIGHTS), c.read(vrg.NRC_TABLE), c.levels, c.log2_table)
    yr = m.forward(corners(pos, LO, HI, sc, dn, r1, c.log2_table), nrm, d).detach().numpy()
    assert _rel(y, yr) < 2e-2
    c.close()


@pytest.mark.parametrize("train", list(TRAIN))
def test_gradients_match_oracle(gpu_ctx, train):
    rng = np.random.default_rng(2)
    c = _cache(gpu_ctx, flags=TRAIN[train])
    tab = (rng.normal(size=c.levels * (1 << c.log2_table) * 2) * 0.5).astype(np.float32)
    c.write(vrg.NRC_TABLE, tab)
    pos, nrm, d, target = _samples(rng, 1500)
    c.write(vrg.NRC_ZERO_GRADS)
    loss = c.train(pos, nrm, d, target, update=False)
    gw = c.read(vrg.NRC_WEIGHT_GRADS)
    gt = c.read(vrg.NRC_TABLE_GRADS)
    sc, dn, r1 = c.layout()
    m = Model(c.read(vrg.NRC_WEIGHTS), c.read(vrg.NRC_TABLE), c.levels, c.log2_table)
    y = m.forward(corners(pos, LO, HI, sc, dn, r1, c.log2_table), nrm, d)
    L = m.loss(y, target)
    L.backward()
    assert abs(loss - float(L.detach())) / float(L.detach()) < 2e-2
    for l in range(5):
        ref = m.Ws[l].grad.numpy().reshape(-1)
        got = gw[l * 4096:(l + 1) * 4096]
        assert _rel(got, ref) < 5e-2, (l, _rel(got, ref))
    ref5 = m.W5.grad.numpy().reshape(-1)
    assert _rel(gw[5 * 4096:5 * 4096 + 192], ref5) < 5e-2
    assert np.all(gw[5 * 4096 + 192:] == 0)
    reft = m.table.grad.numpy().reshape(-1)
    assert _rel(gt, reft) < 5e-2
    c.close()


@pytest.mark.parametrize("train", list(TRAIN))
def test_gradients_after_a_larger_batch(gpu_ctx, train):
    """The activation buffers grow to the largest batch seen; a smaller batch
    afterwards must write and read them with the same row pitch."""
    rng = np.random.default_rng(6)
    c = _cache(gpu_ctx, flags=TRAIN[train])
    tab = (rng.normal(size=c.levels * (1 << c.log2_table) * 2) * 0.5).astype(np.float32)
    c.write(vrg.NRC_TABLE, tab)
    big = _samples(rng, 4000)
    c.train(*big, update=False)  # grows the buffers to 4000 rows per layer
    pos, nrm, d, target = _samples(rng, 700)
    c.write(vrg.NRC_ZERO_GRADS)
    c.train(pos, nrm, d, target, update=False)
    gw = c.read(vrg.NRC_WEIGHT_GRADS)
    sc, dn, r1 = c.layout()
    m = Model(c.read(vrg.NRC_WEIGHTS), c.read(vrg.NRC_TABLE), c.levels, c.log2_table)
    m.loss(m.forward(corners(pos, LO, HI, sc, dn, r1, c.log2_table), nrm, d), target).backward()
    for l in range(5):
        ref = m.Ws[l].grad.numpy().reshape(-1)
        assert _rel(gw[l * 4096:(l + 1) * 4096], ref) < 5e-2, (l, _rel(gw[l * 4096:(l + 1) * 4096], ref))
    assert _rel(gw[5 * 4096:5 * 4096 + 192], m.W5.grad.numpy().reshape(-1)) < 5e-2
    c.close()


@pytest.mark.parametrize("train", list(TRAIN))
def test_training_converges(gpu_ctx, train):
    rng = np.random.default_rng(4)
    c = _cache(gpu_ctx, levels=12, log2_t=14, flags=TRAIN[train])
    pos, nrm, d, target = _samples(rng, 8192)
    first = c.train(pos, nrm, d, target)
    for _ in range(200):
        last = c.train(pos, nrm, d, target)
    assert last < 0.1 * first, (first, last)
    y = c.query(pos, nrm, d)
    assert np.mean(np.abs(y - target) / (np.abs(target) + 0.1)) < 0.2
    c.close()


# The learned-cache workload's own configuration: 16 levels x 2^19 entries x
# 2 FP16 features, resolutions 16 -> 2048 over the 8x8-chunk scene's box, and
# a 65,536-sample batch (the hash-collision regime of the fine levels, the
# scatter's atomics contention and the tensor-core tile count at full size).
C3 = dict(levels=16, log2_table=19, base_resolution=16, max_resolution=2048, batch=65536)
HI_C3 = (256.0, 32.0, 256.0)
N_C3 = 65536


def _c3(gpu_ctx, rng, seed, flags=0):
    c = vrg.RadianceCache(gpu_ctx, LO, HI_C3, learning_rate=1e-2, seed=seed, flags=flags, **C3)
    tab = (rng.normal(size=c.levels * (1 << c.log2_table) * 2) * 0.5).astype(np.float32)
    c.write(vrg.NRC_TABLE, tab)
    pos, nrm, d, target = _samples(rng, N_C3)
    pos = (rng.random((N_C3, 3)) * np.array(HI_C3)).astype(np.float32)
    return c, pos, nrm, d, target


@pytest.mark.parametrize("train", list(TRAIN))
def test_c3_forward_and_gradients_match_oracle(gpu_ctx, train):
    """At the workload's size: the inference output (encoding pass + the
    tcgen05 MLP), the training loss, every layer's weight gradient and the
    hash-table gradient against the float64 oracle, same tolerances as above."""
    rng = np.random.default_rng(31)
    c, pos, nrm, d, target = _c3(gpu_ctx, rng, 9, TRAIN[train])
    try:
        y = c.query(pos, nrm, d)
        c.write(vrg.NRC_ZERO_GRADS)
        loss = c.train(pos, nrm, d, target, update=False)
        gw = c.read(vrg.NRC_WEIGHT_GRADS)
        gt = c.read(vrg.NRC_TABLE_GRADS)
        sc, dn, r1 = c.layout()
        m = Model(c.read(vrg.NRC_WEIGHTS), c.read(vrg.NRC_TABLE), c.levels, c.log2_table)
        yr = m.forward(corners(pos, LO, HI_C3, sc, dn, r1, c.log2_table), nrm, d)
        assert _rel(y, yr.detach().numpy()) < 2e-2
        L = m.loss(yr, target)
        L.backward()
        assert abs(loss - float(L.detach())) / float(L.detach()) < 2e-2
        for l in range(5):
            ref = m.Ws[l].grad.numpy().reshape(-1)
            assert _rel(gw[l * 4096:(l + 1) * 4096], ref) < 5e-2, (l, _rel(gw[l * 4096:(l + 1) * 4096], ref))
        assert _rel(gw[5 * 4096:5 * 4096 + 192], m.W5.grad.numpy().reshape(-1)) < 5e-2
        reft = m.table.grad.numpy().reshape(-1)
        assert _rel(gt, reft) < 5e-2, _rel(gt, reft)
        assert np.count_nonzero(reft) > 1_000_000  # the batch touches the fine levels' hashed entries
    finally:
        c.close()


@pytest.mark.parametrize("train", list(TRAIN))
def test_c3_tensor_core_inference_equals_training_forward(gpu_ctx, train):
    """The inference MLP on tcgen05 and each training kernel's forward pass
    (tcgen05, and the warp-level mma.sync kernel) accumulate each K = 16 step in
    the same order: the same 65,536 samples give bit-identical outputs."""
    rng = np.random.default_rng(32)
    c, pos, nrm, d, target = _c3(gpu_ctx, rng, 10, TRAIN[train])
    try:
        y_tc = c.query(pos, nrm, d)
        c.train(pos, nrm, d, target, update=False)
        y_train = c.train_predictions()
        assert y_tc.shape == y_train.shape == (N_C3, 3)
        assert np.array_equal(y_tc.view(np.uint32), y_train.view(np.uint32)), \
            int((y_tc.view(np.uint32) != y_train.view(np.uint32)).sum())
    finally:
        c.close()


def test_training_kernels_agree(gpu_ctx):
    """The two training kernels on the same batch: the same loss and
    gradients up to the order of the FP32 atomic sums."""
    rng = np.random.default_rng(33)
    out = {}
    for name, fl in TRAIN.items():
        c, pos, nrm, d, target = _c3(gpu_ctx, np.random.default_rng(33), 11, fl)
        c.write(vrg.NRC_ZERO_GRADS)
        loss = c.train(pos, nrm, d, target, update=False)
        out[name] = (loss, c.read(vrg.NRC_WEIGHT_GRADS), c.read(vrg.NRC_TABLE_GRADS))
        c.close()
    a, b = out["tcgen05"], out["mma_sync"]
    assert abs(a[0] - b[0]) <= 1e-5 * abs(b[0])
    assert _rel(a[1], b[1]) < 1e-3
    assert _rel(a[2], b[2]) < 1e-3
