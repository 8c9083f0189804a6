"""Gradient oracle of the neural radiance cache: the same hash-grid encoding
and 5x64 ReLU MLP in PyTorch (CPU, float64), with the CUDA path's roundings
emulated (fp16 table reads, bf16 weights, bf16 activations between layers,
straight-through for the gradients) and the same relative L2 loss."""
import numpy as np
import torch

F64 = torch.float64


def bf16(x):
    return x + (x.to(torch.bfloat16).to(F64) - x).detach()


def oct_encode(v):
    v = np.asarray(v, np.float32)
    s = np.abs(v).sum(axis=1)
    px, py = v[:, 0] / s, v[:, 1] / s
    neg = v[:, 2] < 0
    tx = (1 - np.abs(py)) * np.where(px >= 0, 1.0, -1.0)
    ty = (1 - np.abs(px)) * np.where(py >= 0, 1.0, -1.0)
    px = np.where(neg, tx, px).astype(np.float32)
    py = np.where(neg, ty, py).astype(np.float32)
    return np.stack([px * np.float32(0.5) + np.float32(0.5), py * np.float32(0.5) + np.float32(0.5)], 1)


def corners(pos, lo, hi, scales, dense, res1, log2_t):
    """float32 corner indices and trilinear weights per level, as the kernel computes them."""
    lo = np.asarray(lo, np.float32)
    ext = np.asarray(hi, np.float32) - lo
    inv = np.where(ext > 0, np.float32(1) / np.where(ext > 0, ext, 1), np.float32(1)).astype(np.float32)
    p = np.clip((np.asarray(pos, np.float32) - lo) * inv, 0, 1).astype(np.float32)
    mask = (1 << log2_t) - 1
    out = []
    for l, s in enumerate(scales):
        g = (p * np.float32(s)).astype(np.float32)
        f = np.floor(g).astype(np.float32)
        i = f.astype(np.int64)
        t = (g - f).astype(np.float32)
        idx, w = [], []
        for k in range(8):
            d = [(k >> 2) & 1, (k >> 1) & 1, k & 1]
            c = i + np.array(d)
            c = c.astype(np.uint64)
            if dense[l]:
                r = np.uint64(res1[l])
                ix = (c[:, 0] + c[:, 1] * r + c[:, 2] * r * r) & np.uint64(mask)
            else:
                ix = (c[:, 0] ^ ((c[:, 1] * np.uint64(2654435761)) & np.uint64(0xFFFFFFFF)) ^
                      ((c[:, 2] * np.uint64(805459861)) & np.uint64(0xFFFFFFFF))) & np.uint64(mask)
            wk = np.ones(len(p), np.float32)
            for a in range(3):
                wk = (wk * (t[:, a] if d[a] else np.float32(1) - t[:, a])).astype(np.float32)
            idx.append(ix.astype(np.int64))
            w.append(wk)
        out.append((np.stack(idx, 1), np.stack(w, 1)))
    return out


class Model:
    def __init__(self, weights, table, levels, log2_t):
        self.levels, self.log2_t = levels, log2_t
        W = torch.tensor(weights, dtype=F64)
        self.Ws = [W[l * 4096:(l + 1) * 4096].reshape(64, 64).clone().requires_grad_(True) for l in range(5)]
        self.W5 = W[5 * 4096:5 * 4096 + 3 * 64].reshape(3, 64).clone().requires_grad_(True)
        self.table = torch.tensor(table, dtype=F64).reshape(levels, 1 << log2_t, 2).requires_grad_(True)

    def forward(self, cs, nrm, vdir):
        n = len(nrm)
        tab16 = self.table + (self.table.to(torch.float16).to(F64) - self.table).detach()
        feats = []
        for l, (idx, w) in enumerate(cs):
            v = tab16[l][torch.tensor(idx)]  # n x 8 x 2
            f = (torch.tensor(w, dtype=F64)[:, :, None] * v).sum(1)
            feats.append(f)
        x = torch.zeros(n, 64, dtype=F64)
        x[:, :2 * self.levels] = torch.cat(feats, 1)
        x[:, 2 * self.levels:2 * self.levels + 2] = torch.tensor(oct_encode(nrm), dtype=F64)
        x[:, 2 * self.levels + 2:2 * self.levels + 4] = torch.tensor(oct_encode(-np.asarray(vdir)), dtype=F64)
        h = bf16(x)
        for W in self.Ws:
            h = bf16(torch.relu(h @ bf16(W).T))
        return h @ bf16(self.W5).T

    def loss(self, y, target):
        t = torch.tensor(target, dtype=F64)
        m = (y.detach().sum(1) / 3.0)
        den = m * m + 0.01
        return (((y - t) ** 2).sum(1) / den).mean()
