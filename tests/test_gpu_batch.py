"""Batched energy grids and Widom runs (uneven triclinic frameworks, each with
its own force field, in one persistent launch per kernel behind a captured
CUDA graph): every grid equals the single-grid FP32 build of its framework bit
for bit, graph replays reproduce it, the autotuner records its choice, and
every framework's batched Widom result equals its own Widom run exactly."""
import numpy as np
import pytest

from aleator_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _frameworks(n, seed=2028):
    fws = W.random_triclinic_frameworks(n, seed=seed, max_atoms=600)
    return fws


def test_batch_equals_single_grids(lib):
    A, _ = lib
    fws = _frameworks(6)
    ffs = [A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED) for fw in fws]
    ps = [A.ParticleData.from_framework(fw) for fw in fws]
    guests = [[fw.guest_species["CH4"]] for fw in fws]
    spacing = 0.6
    batch = A.GridBatch(ffs, ps, [fw.lattice for fw in fws], guests, spacing)
    batch.build()
    st = batch.stats()
    assert st["grids"] == 6 and st["variant"] in (0, 1) and st["graph_launches"] == 1
    assert min(st["tune_ms"]) > 0
    counts = [batch.point_counts(i) for i in range(6)]
    assert len(set(counts)) > 1  # uneven grids
    first = [batch.table(i, guests[i][0]) for i in range(6)]
    for i, fw in enumerate(fws):
        single = A.FrameworkEnergyGrid(ffs[i], ps[i], fw.lattice, guests[i], spacing, A.FP32)
        assert single.point_counts() == counts[i]
        t = single.table(guests[i][0])
        assert np.array_equal(first[i], t), i
    # graph replays write the same tables
    batch.build()
    batch.build()
    assert batch.stats()["graph_launches"] == 3
    for i in range(6):
        assert np.array_equal(batch.table(i, guests[i][0]), first[i])


def test_batch_rejects_mixed_guest_counts(lib):
    A, _ = lib
    fws = _frameworks(2)
    ffs = [A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED) for fw in fws]
    ps = [A.ParticleData.from_framework(fw) for fw in fws]
    g = fws[0].guest_species["CH4"]
    with pytest.raises(ValueError):
        A.GridBatch(ffs, ps, [fw.lattice for fw in fws], [[g, g], [g, 0]], 0.6)


def test_widom_batch_equals_single_runs(lib):
    A, _ = lib
    fws = _frameworks(5, seed=7)
    ffs = [A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED) for fw in fws]
    ps = [A.ParticleData.from_framework(fw) for fw in fws]
    guests = [W.ch4_guest(fw) for fw in fws]
    seeds, streams = [11 + i for i in range(5)], [i for i in range(5)]
    for prec in (A.FP64, A.FP32):
        batch = A.WidomBatch(ffs, ps, [fw.lattice for fw in fws], guests, 298.0, precision=prec)
        for n in (3000, 5000):  # a second size re-captures the graph
            res = batch.run(seeds, streams, n, first_trial=17)
            for i, fw in enumerate(fws):
                w = A.Widom(ffs[i], ps[i], fw.lattice, guests[i], 298.0, precision=prec)
                r = w.run(seeds[i], streams[i], n, first_trial=17)
                assert res[i]["henry"] == r["henry"], (prec, n, i)
                assert res[i]["rel_std_error"] == r["rel_std_error"], (prec, n, i)
                assert res[i]["n_trials"] == n
