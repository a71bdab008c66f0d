"""Parity at the benchmark's own workloads, against the CPU oracle.

The other GPU tests use models of up to ~40k atoms. These run the exact
workloads the benchmark times and compare them with the oracle, which
restates cuDebye-v15.cu:88-146 (histogram) and :493-538 (Debye sum):

* spinel_10nm (117,945 atoms, 6 pair types, 104,002 bins, 6,001 q): all six
  histograms bin for bin, from the tile kernel and from the plain
  one-thread-per-pair kernel, and the tensor-core intensities at every q
  within 1e-6 relative;
* plain_small (5,000 atoms, 3 pair types): the same, through dbx_pattern;
* the 256-model mix (seed 3, 4.4 M atoms): every model's histograms after
  one batched pass bin for bin, and every pattern within 1e-6 of the FP64
  oracle at every 10th q.

Histograms are integers: the tolerance is exact equality.
"""
import numpy as np
import pytest

from cudebye_gb300 import lattice

pytestmark = pytest.mark.gpu

TOL = 1e-6  # max relative intensity error of the tensor-core form vs FP64


def max_rel(got, want):
    return float(np.max(np.abs(got - want) / np.abs(want)))


def check_model(engine, orc, m, K, with_plain=True):
    mod = engine.upload(m.xyz, m.counts)
    try:
        want_h, bad = orc.model_histograms(m.xyz, m.counts, m.rstep, m.nbins)
        assert bad == 0
        I = engine.pattern(mod, m.rstep, m.nbins, m.species, K, mode="tc")
        h = engine.histogram(mod, m.rstep, m.nbins)  # resident from the pattern
        np.testing.assert_array_equal(h, want_h)
        assert int(h.sum()) == m.pairs
        if with_plain:
            p = 0
            for r in range(len(m.counts)):
                for c in range(r, len(m.counts)):
                    hp = engine.split_calc_dist_plain(mod, r, c, m.rstep, m.nbins)
                    np.testing.assert_array_equal(hp, want_h[p])
                    p += 1
        want_I = orc.intensity(K, want_h, m.species, m.rstep)
        err = max_rel(I, want_I)
        assert err <= TOL, err
        return err
    finally:
        mod.free()


def test_spinel_10nm_matches_oracle(engine, orc):
    m = lattice.spinel_10nm()
    assert (m.natoms, m.nbins, len(m.counts)) == (117945, 104002, 3)
    tt, K = m.k_grid()
    assert len(K) == 6001
    check_model(engine, orc, m, K)


def test_plain_small_matches_oracle(engine, orc):
    m = lattice.plain_small()
    assert m.natoms == 5000 and len(m.counts) == 2
    tt, K = m.k_grid()
    check_model(engine, orc, m, K)


def test_batch256_matches_oracle(engine, orc):
    mods = lattice.batch256(seed=3)
    assert len(mods) == 256
    tt, K = mods[0].k_grid()
    sp = [s for m in mods for s in m.species]
    nb = [m.nbins for m in mods]
    hs = [engine.upload(m.xyz, m.counts) for m in mods]
    try:
        I = engine.patterns(hs, 1e-3, nb, sp, K)
        worst = 0.0
        for m, h, row in zip(mods, hs, I):
            want_h, bad = orc.model_histograms(m.xyz, m.counts, m.rstep, m.nbins)
            assert bad == 0
            got = engine.histogram(h, m.rstep, m.nbins)  # resident after the pass
            np.testing.assert_array_equal(got, want_h)
            want_I = orc.intensity(K, want_h, m.species, m.rstep, q_stride=10)
            sel = np.arange(0, len(K), 10)
            worst = max(worst, max_rel(row[sel], want_I[sel]))
        assert worst <= TOL, worst
    finally:
        for h in hs:
            h.free()
