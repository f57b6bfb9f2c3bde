"""The learned insertion proposal on the GPU against its FP64 oracle
(oracle/proposal_oracle.py), and the biased Widom estimator against the
plain (uniform) method.

Tolerances: the network output within 2e-4 x max(1, |f|) (the hidden layers'
products on the tensor cores from BF16 hi + lo parts of the FP32 activations,
~16 significant bits, accumulated in FP32, against FP64 with the same
BF16-rounded weights); the batch loss
within 1e-5 relative and the gradient within 2e-3 relative (L2) of the
oracle's; the tabulated density exactly normalised (1e-9) and within 1e-5
relative of the oracle's table built from the same network outputs; biased
per-trial energies within 1e-10 relative of the oracle's LJ energies at the
same positions; the biased K_H within 3 of its standard errors (combined with
the reference run's) of a long uniform FP64 run."""
import numpy as np
import pytest

import oracle as O
from conftest import golden, rel_err
from oracle import proposal_oracle as PO

pytestmark = pytest.mark.gpu

T = 298.0


def _random_params(P, rng, scale=1.0):
    w = P.get_params().astype(np.float64)
    w = rng.normal(0, scale, w.size) * np.abs(w).mean() * 3 + 0.05 * rng.normal(0, 1, w.size)
    return w.astype(np.float32)


def test_forward_matches_oracle(lib):
    A, _ = lib
    P = A.Proposal(seed=5)
    rng = np.random.default_rng(0)
    P.set_params(_random_params(P, rng))
    s = rng.random((2000, 3)).astype(np.float32)
    f = P.forward(s)
    fo = PO.MLP(P.wave_vectors(), P.get_params()).forward(s)
    assert np.abs(fo).max() > 1.0  # a non-trivial network
    err = np.abs(f - fo) / np.maximum(1.0, np.abs(fo))
    assert err.max() <= 2e-4, (err.max(), err.mean())


def test_loss_and_gradient_match_oracle(lib):
    A, _ = lib
    P = A.Proposal(seed=9)
    rng = np.random.default_rng(1)
    P.set_params(_random_params(P, rng, 0.5))
    samples = np.concatenate([rng.random((700, 3)), rng.normal(0, 4, (700, 1))], axis=1)
    samples = samples.astype(np.float32)
    mlp = PO.MLP(P.wave_vectors(), P.get_params())
    # rows drawn from an earlier proposal carry its log density lq
    with_lq = np.concatenate([samples, rng.normal(0, 1, (700, 1)).astype(np.float32)], axis=1)
    for tau, rows in ((1.0, samples), (0.6, samples), (1.0, with_lq)):
        loss, g = P.loss_grad(rows, tau)
        lo, go = mlp.loss_grad(rows, tau)
        assert abs(loss - lo) <= 1e-5 * max(1.0, abs(lo))
        assert np.linalg.norm(g - go) <= 2e-3 * np.linalg.norm(go)
        # every layer's block is right, not just the norm
        assert np.corrcoef(g, go)[0, 1] >= 0.99999


def test_tabulated_density_normalised_and_matches_oracle(lib):
    A, _ = lib
    P = A.Proposal(seed=3)
    rng = np.random.default_rng(2)
    P.set_params(_random_params(P, rng))
    cells, u = 16, 0.2
    P.tabulate(cells, u)
    c = PO.cell_centres(cells)
    lp = P.log_density(c)
    assert abs(np.exp(lp).mean() - 1.0) <= 1e-9  # integrates to 1 over the cell
    ptab = PO.tabulate(P.forward(c.astype(np.float32)), u)
    assert rel_err(np.exp(lp) / cells ** 3, ptab, floor=0.0).max() <= 1e-5
    assert np.exp(lp).min() >= u * (1 - 1e-9)  # the uniform share is a floor
    # periodic: positions one cell length apart share the density
    s = rng.random((100, 3))
    assert np.array_equal(P.log_density(s), P.log_density(s + 1.0))


def test_training_fits_a_known_density(lib):
    """Samples with log-weights l(s) = 3 cos(2 pi s0) + 2 cos(2 pi (s1 + s2)):
    training lowers the loss and the trained log-density follows l."""
    A, _ = lib
    import torch

    rng = np.random.default_rng(4)
    n = 1 << 16
    s = rng.random((n, 3))
    l = 3 * np.cos(2 * np.pi * s[:, 0]) + 2 * np.cos(2 * np.pi * (s[:, 1] + s[:, 2]))
    rows = np.concatenate([s, l[:, None], np.zeros((n, 1))], axis=1).astype(np.float32)
    d = torch.tensor(rows, device="cuda")
    P = A.Proposal(seed=1)
    before, _ = P.loss_grad(rows[:8192])
    P.train(d.data_ptr(), n, epochs=40, batch=4096, lr=3e-3)
    after, _ = P.loss_grad(rows[:8192])
    assert after < before - 0.5
    c = PO.cell_centres(12)
    f = P.forward(c.astype(np.float32))
    lc = 3 * np.cos(2 * np.pi * c[:, 0]) + 2 * np.cos(2 * np.pi * (c[:, 1] + c[:, 2]))
    assert np.corrcoef(f, lc)[0, 1] >= 0.95


def _c1(A):
    from aleator_gb300 import workloads as W

    class _FW:
        guest_species = {"CH4": 4, "CO2_C": 5, "CO2_O": 6}

    g = golden("grid_cubic")
    ff = A.LennardJones(g["eps"], g["sigma"], 12.8, A.SHIFTED)
    p = A.ParticleData(g["x"], g["y"], g["z"], g["charge"], g["species"])
    return g, ff, p, W.ch4_guest(_FW)


def _trained(A, widom, n=1 << 18, cells=32, uniform_share=0.05):
    import torch

    d = torch.empty((n, A.SAMPLE_ROW), dtype=torch.float32, device="cuda")
    widom.samples(1234, 7, n, d.data_ptr())
    P = A.Proposal(seed=2)
    P.train(d.data_ptr(), n, epochs=30, batch=16384, lr=2e-3)
    P.tabulate(cells, uniform_share)
    return P, d


def test_biased_widom_per_trial_and_estimator(lib, orc):
    A, _ = lib
    g, ff, p, guest = _c1(A)
    widom = A.Widom(ff, p, g["lattice"], guest, T)
    P, _ = _trained(A, widom, n=1 << 16)
    r, du, fr = widom.run_biased(P, 42, 0, 20000, per_trial=True)
    # positions inside the cell, energies as the oracle's LJ scan at those positions
    assert fr.min() >= 0.0 and fr.max() <= 1.0
    m = np.asarray(g["lattice"]).reshape(3, 3)
    pos = fr @ m
    n_fw = len(g["x"])
    probe_lj = int(guest["lj_species"][0])
    for i in range(0, 20000, 997):
        x = np.append(g["x"], pos[i, 0])
        y = np.append(g["y"], pos[i, 1])
        z = np.append(g["z"], pos[i, 2])
        sp = np.append(g["species"], probe_lj).astype(np.uint32)
        ffd = {"eps": g["eps"], "sigma": g["sigma"], "cutoff": 12.8, "truncation": O.SHIFTED}
        e = orc.lj_particle_energy(ffd, m, x, y, z, sp, n_fw)
        assert abs(du[i] - e) <= 1e-10 * max(1.0, abs(e))
    # the kernel's estimator is importance sampling with the tabulated density
    kh, rel = PO.biased_henry(du, P.log_density(fr), T)
    assert abs(r["henry"] / kh - 1) <= 1e-9
    assert abs(r["rel_std_error"] / rel - 1) <= 1e-6


def test_biased_henry_agrees_with_uniform_and_gains(lib):
    A, _ = lib
    g, ff, p, guest = _c1(A)
    widom = A.Widom(ff, p, g["lattice"], guest, T)
    ref = widom.run(99, 3, 1 << 22)  # long uniform FP64 run
    P, _ = _trained(A, widom)
    n = 1 << 18
    b = widom.run_biased(P, 42, 0, n)
    u = widom.run(42, 0, n)
    se = np.hypot(b["rel_std_error"] * b["henry"], ref["rel_std_error"] * ref["henry"])
    assert abs(b["henry"] - ref["henry"]) <= 3 * se
    assert abs(u["henry"] - ref["henry"]) <= 3 * np.hypot(u["rel_std_error"] * u["henry"],
                                                          ref["rel_std_error"] * ref["henry"])
    # what the trained proposal gains: the same trials give a smaller error
    assert b["rel_std_error"] <= 0.5 * u["rel_std_error"], (b, u)
