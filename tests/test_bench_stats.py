"""Host-side statistics of the benchmark: chunks of one Widom trial stream
combine into the whole stream's K_H and relative standard error (the chunked
runs to a 1 % target use this)."""
import numpy as np

import bench


def _stats(lw, temperature):
    """What one Widom call reports for log-weights lw: the log mean weight
    and the relative standard error of the mean weight."""
    m = lw.max()
    s1 = np.exp(lw - m).sum()
    s2 = np.exp(2 * (lw - m)).sum()
    n = len(lw)
    mean = s1 / n
    var = s2 / n - mean * mean
    return {"n_trials": n, "log_mean_weight": m + np.log(mean),
            "rel_std_error": np.sqrt(max(var, 0.0) / n) / mean}


def test_chunks_combine_to_the_whole_stream():
    rng = np.random.default_rng(3)
    # heavy-tailed log-weights reaching e^60, as on the charged framework
    lw = np.concatenate([rng.normal(0.0, 3.0, 70_000), rng.normal(55.0, 2.0, 12)])
    rng.shuffle(lw)
    whole = _stats(lw, 298.0)
    cuts = [0, 1000, 3000, 7000, 15_000, 31_000, 70_012]
    chunks = [_stats(lw[a:b], 298.0) for a, b in zip(cuts[:-1], cuts[1:])]
    comb = bench.combine_widom(chunks, 298.0)
    assert comb["trials"] == len(lw)
    assert abs(comb["log_mean_weight"] - whole["log_mean_weight"]) <= 1e-12 * abs(whole["log_mean_weight"])
    assert abs(comb["henry"] / (np.exp(whole["log_mean_weight"]) / 298.0) - 1.0) <= 1e-12
    assert abs(comb["rel_std_error"] / whole["rel_std_error"] - 1.0) <= 1e-9


def test_loading_time_to_one_percent():
    """The running estimate (second half of the blocks so far) first within
    1 % of the reference with a 1 % standard error: a chain set that fills
    up over 10 blocks, then fluctuates about 100 molecules."""
    rng = np.random.default_rng(0)
    n = 64
    traj = []
    for b in range(60):
        level = 100.0 * min(1.0, (b + 1) / 10.0)
        traj.append((0.5 * (b + 1), level + rng.normal(0.0, 3.0, n)))
    t_hit, est = bench.loading_metrics(traj, 100.0, n)
    # 18 blocks: the second half (blocks 9-17) is all filled; 17 blocks still
    # hold the 90 % block 8
    assert t_hit == 9.0
    assert abs(est - 100.0) <= 0.5
    # never within 1 % of a wrong reference
    assert bench.loading_metrics(traj, 120.0, n)[0] is None


def test_loading_comparison_reports_a_lower_bound_when_uniform_never_gets_there(monkeypatch):
    """The comparison's bookkeeping on stand-in trajectories (no GPU): arms
    that reach a 1 % loading get their time; the uniform arm that does not
    makes each speed-up a lower bound, its wall time over the arm's time."""
    import types
    import bench

    def fake_run(A, torch, ff, p, fw, guest, ew, T, P, learned, seconds, n=152, proposal=None,
                 orient=1):
        rng = np.random.default_rng(orient + 10 * learned)
        tau = 0.3 if (orient > 1 and not learned) else (0.5 if learned else 3.0)
        traj = [(1.25 * (b + 1), 100.0 * (1 - np.exp(-1.25 * (b + 1) / tau)) + rng.normal(0, 0.3, n))
                for b in range(12)]
        return {"fit_seconds": 0.0, "traj": traj, "moves_per_chain": 1}

    monkeypatch.setattr(bench, "loading_run", fake_run)
    monkeypatch.setattr(bench, "henry_setup",
                        lambda A: (types.SimpleNamespace(lattice=None), None, None, None, None,
                                   298.0, 0.3, 10))
    monkeypatch.setattr(bench, "fit_proposal", lambda A, w: None)
    A = types.SimpleNamespace(Widom=lambda *a, **k: None, FP32=1)
    torch = types.SimpleNamespace(cuda=types.SimpleNamespace(synchronize=lambda: None))
    row = bench.loading_comparison(A, torch, pressures_bar=(10.0,), seconds=15.0, n=32,
                                   arms=("uniform", "uniform_orient", "learned"))["10 bar"]
    assert row["uniform"]["time_to_1pct_s"] is None and row["uniform"]["wall_s"] == 15.0
    assert row["uniform_orient"]["time_to_1pct_s"] == 2.5
    assert row["speedup"] is None and row["speedup_lower_bound"] == 15.0 / 2.5
    assert row["speedup_orientation_trials_lower_bound"] == 15.0 / 2.5
