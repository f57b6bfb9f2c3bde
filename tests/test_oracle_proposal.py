"""The learned-proposal oracle (oracle/proposal_oracle.py) on its own: its
gradient against central finite differences (FP64, 1e-6 relative), the
tabulated density's normalisation and uniform floor, the BF16 rounding
against hand-made cases, and the biased Henry estimator's uniform limit."""
import numpy as np

from oracle import proposal_oracle as PO


def _small(rng, nf=4, width=8, depth=2):
    k = rng.integers(-3, 4, size=(nf, 3))
    k[np.all(k == 0, axis=1)] = (1, 0, 0)
    n = 0
    n_in = 2 * nf
    for layer in range(depth + 1):
        n_out = width if layer < depth else 1
        n += n_in * n_out + n_out
        n_in = n_out
    return k, rng.normal(0, 0.7, n)


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    k, w = _small(rng)
    samples = np.concatenate([rng.random((64, 3)), rng.normal(0, 3, (64, 1)),
                              rng.normal(0, 1, (64, 1))], axis=1)
    for tau, rows in ((1.0, samples[:, :4]), (0.5, samples[:, :4]), (1.0, samples)):
        loss, g = PO.MLP(k, w, width=8, depth=2, round_bf16=False).loss_grad(rows, tau)
        for i in rng.choice(len(w), 25, replace=False):
            h = 1e-6
            wp, wm = w.copy(), w.copy()
            wp[i] += h
            wm[i] -= h
            lp, _ = PO.MLP(k, wp, width=8, depth=2, round_bf16=False).loss_grad(rows, tau)
            lm, _ = PO.MLP(k, wm, width=8, depth=2, round_bf16=False).loss_grad(rows, tau)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[i]) <= 1e-6 * max(1e-3, abs(fd)), (i, fd, g[i])


def test_tabulate_normalised_with_floor():
    rng = np.random.default_rng(1)
    f = rng.normal(0, 4, 8 ** 3)
    p = PO.tabulate(f, 0.1)
    assert abs(p.sum() - 1) <= 1e-12
    assert p.min() >= 0.1 / p.size * (1 - 1e-12)
    assert np.argmax(p) == np.argmax(f)
    c = PO.cell_centres(8)
    assert np.allclose(c[1], (1.5 / 8, 0.5 / 8, 0.5 / 8)) and np.allclose(c[8], (0.5 / 8, 1.5 / 8, 0.5 / 8))


def test_bf16_round_to_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, 1.0078125 + 2 ** -9, -3.14159], np.float32)
    r = PO.bf16_round(x)
    assert r[0] == 1.0
    assert r[1] == 1.0            # exactly half an ulp above 1.0: ties to even
    assert r[2] == np.float32(1.0078125)  # above the midpoint: rounds up
    assert abs(r[4] + 3.140625) < 1e-7


def test_biased_estimator_uniform_limit():
    rng = np.random.default_rng(2)
    du = rng.normal(-500, 800, 10000)
    k0, r0 = PO.biased_henry(du, np.zeros_like(du), 298.0)
    w = np.exp(-du / 298.0)
    assert abs(k0 / (w.mean() / 298.0) - 1) <= 1e-12
    assert abs(r0 / (w.std() / np.sqrt(len(w)) / w.mean()) - 1) <= 1e-12
