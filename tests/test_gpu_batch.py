"""Batched patterns (dbx_patterns): many models of different sizes, species
counts and bin counts in one histogram launch and one tensor-core
contraction, replayed as a CUDA graph. Each model's pattern must match the
FP64 oracle (max rel <= 1e-6) and its histograms the oracle bit for bit,
exactly as if it ran alone."""
import numpy as np
import pytest

import cudebye_gb300 as cd
from cudebye_gb300 import lattice

pytestmark = pytest.mark.gpu


def small_batch(seed, n=6, nmin=300, nmax=3000):
    rng = np.random.default_rng(seed)
    return [lattice.random_model(rng, nmin, nmax, lattice.GRID_CU, "b%d" % i, seed)
            for i in range(n)]


def species_of(models):
    return [s for m in models for s in m.species]


def check_against_oracle(engine, orc, mods, handles, I, K):
    for m, h, row in zip(mods, handles, I):
        hist = engine.histogram(h, m.rstep, m.nbins)  # resident after the pass
        want_h, bad = orc.model_histograms(m.xyz, m.counts, m.rstep, m.nbins)
        assert bad == 0
        np.testing.assert_array_equal(hist, want_h)
        want = orc.intensity(K, want_h, m.species, m.rstep)
        rel = np.abs(row - want) / np.abs(want)
        assert rel.max() <= 1e-6, (m.counts, rel.max())


def test_batch_tc_matches_oracle_and_replays(engine, orc):
    mods = small_batch(41)
    tt, K = mods[0].k_grid()
    K = K[::5]
    handles = [engine.upload(m.xyz, m.counts) for m in mods]
    try:
        nb = [m.nbins for m in mods]
        I1 = engine.patterns(handles, 1e-3, nb, species_of(mods), K)
        check_against_oracle(engine, orc, mods, handles, I1, K)
        # second pass: graph replay; new B factors (a re-scoring request)
        for m in mods:
            for s in m.species:
                s.beq = s.beq * 0.5 + 0.1
        I2 = engine.patterns(handles, 1e-3, nb, species_of(mods), K)
        check_against_oracle(engine, orc, mods, handles, I2, K)
        assert not np.array_equal(I1, I2)
        # graphs off: the same numbers (fixed reduction order)
        engine.set_graphs(False)
        I3 = engine.patterns(handles, 1e-3, nb, species_of(mods), K)
        engine.set_graphs(True)
        np.testing.assert_array_equal(I2, I3)
    finally:
        for h in handles:
            h.free()


def test_pattern_errors_report(engine, orc):
    """dbx_pattern_errors: each pattern's max relative error against the FP64
    direct sum at every 3rd q equals the error computed here against the
    CPU FP64 oracle (to the oracle's agreement with the device FP64 sum),
    and stays within 1e-6; a corrupted pattern is reported."""
    mods = small_batch(47, n=4)
    tt, K = mods[0].k_grid()
    K = K[::7]
    handles = [engine.upload(m.xyz, m.counts) for m in mods]
    try:
        nb = [m.nbins for m in mods]
        sp = species_of(mods)
        I = engine.patterns(handles, 1e-3, nb, sp, K)
        err = engine.pattern_errors(handles, 1e-3, nb, sp, K, I, q_stride=3)
        assert err.shape == (4,) and np.all(err <= 1e-6)
        for m, h, row, e in zip(mods, handles, I, err):
            want = orc.intensity(K[::3], engine.histogram(h, m.rstep, m.nbins),
                                 m.species, m.rstep)
            mine = float(np.max(np.abs(row[::3] - want) / np.abs(want)))
            assert abs(mine - e) <= 1e-10, (mine, e)
        bad = I.copy()
        bad[2, 3] *= 1.001
        err2 = engine.pattern_errors(handles, 1e-3, nb, sp, K, bad, q_stride=3)
        assert err2[2] >= 9e-4 and np.allclose(err2[[0, 1, 3]], err[[0, 1, 3]])
    finally:
        for h in handles:
            h.free()


def test_batch_result_independent_of_batch_mates(engine):
    """A model's pattern is the same alone and inside a batch."""
    mods = small_batch(42, n=5)
    tt, K = mods[0].k_grid()
    K = K[::7]
    handles = [engine.upload(m.xyz, m.counts) for m in mods]
    try:
        nb = [m.nbins for m in mods]
        I_all = engine.patterns(handles, 1e-3, nb, species_of(mods), K)
        for i in (0, 3):
            I_one = engine.patterns([handles[i]], 1e-3, [nb[i]], mods[i].species, K)
            np.testing.assert_allclose(I_one[0], I_all[i], rtol=1e-12)
    finally:
        for h in handles:
            h.free()


def test_plain_form(engine, orc):
    mods = small_batch(43, n=3, nmax=1500)
    tt, K = mods[0].k_grid()
    K = K[::25]
    handles = [engine.upload(m.xyz, m.counts) for m in mods]
    try:
        nb = [m.nbins for m in mods]
        I = engine.patterns(handles, 1e-3, nb, species_of(mods), K, mode="plain")
        for m, h, row in zip(mods, handles, I):
            hist = engine.histogram(h, m.rstep, m.nbins)
            want_h, _ = orc.model_histograms(m.xyz, m.counts, m.rstep, m.nbins)
            np.testing.assert_array_equal(hist, want_h)
            want = orc.intensity(K, want_h, m.species, m.rstep)
            assert np.abs(row - want).max() / np.abs(want).max() < 0.05
        I64 = engine.patterns(handles, 1e-3, nb, species_of(mods), K, mode="fp64")
        for m, h, row in zip(mods, handles, I64):
            want_h, _ = orc.model_histograms(m.xyz, m.counts, m.rstep, m.nbins)
            want = orc.intensity(K, want_h, m.species, m.rstep)
            np.testing.assert_allclose(row, want, rtol=1e-11)
    finally:
        for h in handles:
            h.free()


def test_batch_replay_after_single_pattern_calls(engine):
    """A single-pattern tensor-core call (dbx_pattern, also in the TF32 and
    BF16x3 comparison forms) between two dbx_patterns calls on the same
    models prepares the shared contraction state for another shape; the
    second batch call must prepare again instead of replaying the stale
    graph, and give the first call's numbers."""
    mods = small_batch(48, n=4)
    tt, K = mods[0].k_grid()
    K = K[::9]
    other = lattice.spinel(radius=11.0, target=1200, seed=49)
    _, K2 = other.k_grid()
    handles = [engine.upload(m.xyz, m.counts) for m in mods]
    h2 = engine.upload(other.xyz, other.counts)
    try:
        nb = [m.nbins for m in mods]
        I1 = engine.patterns(handles, 1e-3, nb, species_of(mods), K)
        for mode in ("tc", "tf32", "tc3"):
            engine.pattern(h2, other.rstep, other.nbins, other.species, K2[::3],
                           mode=mode)
            I2 = engine.patterns(handles, 1e-3, nb, species_of(mods), K)
            np.testing.assert_array_equal(I1, I2)
    finally:
        for h in handles:
            h.free()
        h2.free()


def test_autotuner_picks_shape_on_fine_bins(engine, orc):
    """A batch binned at 1e-4 A splits every histogram into several
    shared-memory windows: the batch autotuner times three tile-shape /
    window-geometry candidates and three task counts (dbx_batch_tuning),
    and the histograms of the plan it keeps equal the oracle's bin for bin.
    A single-window batch times the task counts only."""
    rng = np.random.default_rng(50)
    mods = []
    for i in range(3):
        m = lattice.random_model(rng, 800, 2500, lattice.GRID_CU, "f%d" % i, 50)
        m.rstep = 1e-4
        mods.append(m)
    tt, K = mods[0].k_grid()
    K = K[::30]
    handles = [engine.upload(m.xyz, m.counts) for m in mods]
    try:
        nb = [m.nbins for m in mods]
        assert min(nb) > 114688
        engine.patterns(handles, 1e-4, nb, species_of(mods), K)
        t = engine.batch_tuning()
        assert t["multi_window"] and t["shapes_timed"] == 3
        assert t["task_counts_timed"] == 3 and t["tasks"] > 0 and t["hist_ms"] > 0
        assert t["geometry"] in ("sampled", "disjoint") and t["rowq"] >= 0
        for m, h in zip(mods, handles):
            got = engine.histogram(h, 1e-4, m.nbins)  # resident after the pass
            want, bad = orc.model_histograms(m.xyz, m.counts, 1e-4, m.nbins)
            assert bad == 0
            np.testing.assert_array_equal(got, want)
        one = small_batch(51, n=2)
        h1 = [engine.upload(m.xyz, m.counts) for m in one]
        try:
            engine.patterns(h1, 1e-3, [m.nbins for m in one], species_of(one), K)
            t1 = engine.batch_tuning()
            assert not t1["multi_window"] and t1["shapes_timed"] == 0
            assert t1["task_counts_timed"] == 3
        finally:
            for h in h1:
                h.free()
    finally:
        for h in handles:
            h.free()
