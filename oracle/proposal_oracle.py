"""ORACLE — test infrastructure, not product code.

FP64 numpy restatement of the learned insertion proposal, the checker for the
GPU kernels in aleator_gb300/csrc/proposal.cu and the biased Widom estimator.
The reference has no learned proposal (its insertions are uniform,
monte_carlo_engine.cc:572-574, 882-884); what is restated here is the
definition the kernels implement:

* features phi(s) = [sin(2 pi k_j . s), cos(2 pi k_j . s)] for integer k_j;
* layers h_l = SiLU(W_l h_{l-1} + b_l), output f = W_L h_{L-1} + b_L, with the
  weights W rounded to BF16 (round to nearest even) and the biases in FP32;
* loss L = -sum_i softmax(tau l - lq)_i f_i + log mean_i exp(f_i - lq_i) and its
  gradient (lq: log density of the proposal a row was drawn from, 0 if uniform);
* the tabulated density P_c = (1 - u) softmax(f(centre_c)) + u / N.

Only tests/ may import this module.
"""
from __future__ import annotations

import numpy as np


def bf16_round(w: np.ndarray) -> np.ndarray:
    """FP32 -> BF16 (round to nearest even) -> FP32, as __float2bfloat16_rn."""
    u = np.ascontiguousarray(w, dtype=np.float32).view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


class MLP:
    """The network with the layout of the GPU parameter vector: per layer
    W [out x in] row-major, then b [out]."""

    def __init__(self, kvec, params, width=128, depth=3, round_bf16=True):
        self.k = np.asarray(kvec, dtype=np.float64).reshape(-1, 3)
        self.nf = len(self.k)
        self.width, self.depth = width, depth
        p = np.asarray(params, dtype=np.float32 if round_bf16 else np.float64)
        self.shapes = []
        n_in = 2 * self.nf
        off = 0
        self.W, self.b = [], []
        for layer in range(depth + 1):
            n_out = width if layer < depth else 1
            w = p[off:off + n_in * n_out].reshape(n_out, n_in)
            off += n_in * n_out
            b = p[off:off + n_out]
            off += n_out
            self.W.append((bf16_round(w) if round_bf16 else w).astype(np.float64))
            self.b.append(b.astype(np.float64))
            self.shapes.append((n_out, n_in))
            n_in = n_out
        assert off == p.size, "parameter count"
        self.n_params = off

    def features(self, s):
        s = np.asarray(s, dtype=np.float64).reshape(-1, 3)
        t = s @ self.k.T
        t = t - np.floor(t)
        return np.concatenate([np.sin(2 * np.pi * t), np.cos(2 * np.pi * t)], axis=1)

    def forward(self, s, keep=False):
        h = self.features(s)
        zs, hs = [], [h]
        for layer in range(self.depth):
            z = h @ self.W[layer].T + self.b[layer]
            h = z / (1.0 + np.exp(-z))
            zs.append(z)
            hs.append(h)
        f = (h @ self.W[-1].T + self.b[-1])[:, 0]
        return (f, zs, hs) if keep else f

    def loss_grad(self, samples, tau=1.0):
        """Loss and gradient (flat, in the GPU parameter order) for one batch
        of rows {s0, s1, s2, l} or {s0, s1, s2, l, lq} (lq: log density of the
        proposal the row was drawn from; 0 when absent)."""
        samples = np.asarray(samples, dtype=np.float64)
        lq = samples[:, 4] if samples.shape[1] > 4 else np.zeros(len(samples))
        f, zs, hs = self.forward(samples[:, :3], keep=True)
        tl = tau * samples[:, 3] - lq
        a = f - lq
        pf = np.exp(a - a.max())
        pf /= pf.sum()
        pl = np.exp(tl - tl.max())
        pl /= pl.sum()
        loss = -(pl * f).sum() + (a.max() + np.log(np.exp(a - a.max()).mean()))
        g = pf - pl
        grads = [None] * (self.depth + 1)
        dz = g[:, None]
        for layer in range(self.depth, -1, -1):
            grads[layer] = (dz.T @ hs[layer], dz.sum(axis=0))
            if layer > 0:
                dh = dz @ self.W[layer]
                z = zs[layer - 1]
                sg = 1.0 / (1.0 + np.exp(-z))
                dz = dh * sg * (1.0 + z * (1.0 - sg))
        flat = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
        return loss, flat


def tabulate(f_centres: np.ndarray, uniform_share: float) -> np.ndarray:
    """Cell probabilities P_c from the network at the cell centres."""
    f = np.asarray(f_centres, dtype=np.float64)
    p = np.exp(f - f.max())
    p /= p.sum()
    n = f.size
    p = (1.0 - uniform_share) * p + uniform_share / n
    return p / p.sum()


def cell_centres(cells: int) -> np.ndarray:
    """Cell centres in the table's order (x fastest)."""
    i = np.arange(cells ** 3)
    ix, iy, iz = i % cells, (i // cells) % cells, i // (cells * cells)
    return (np.stack([ix, iy, iz], axis=1) + 0.5) / cells


def biased_henry(du: np.ndarray, log_p: np.ndarray, temperature: float):
    """Importance-sampling Henry coefficient from per-trial dU and log p(s):
    K_H = mean(exp(-dU/T) / p) / T, and its relative standard error."""
    lw = -np.asarray(du) / temperature - np.asarray(log_p)
    m = lw.max()
    w = np.exp(lw - m)
    mean = w.mean()
    rel = w.std() / np.sqrt(len(w)) / mean
    return np.exp(m) * mean / temperature, rel
