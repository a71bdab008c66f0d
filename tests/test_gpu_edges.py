"""Edge cases of the whole path against the oracle: species with no atoms,
coincident atoms (zero distances off the diagonal), a tiny bin count,
many species (55 pair types in one contraction), a model of one atom, and a
bin count at the limit of one shared-memory window and one bin past it.
Histograms must be bit-exact and intensities within 1e-6 of FP64."""
import numpy as np
import pytest

import cudebye_gb300 as cd
from cudebye_gb300 import lattice

pytestmark = pytest.mark.gpu


def check(engine, orc, xyz, counts, rstep, nbins, species, K, rtol=1e-6):
    m = engine.upload(xyz, counts)
    try:
        h = engine.histogram(m, rstep, nbins)
        want_h, bad = orc.model_histograms(xyz, counts, rstep, nbins)
        assert bad == 0
        np.testing.assert_array_equal(h, want_h)
        I = engine.pattern(m, rstep, nbins, species, K)
        want = orc.intensity(K, want_h, species, rstep)
        np.testing.assert_allclose(I, want, rtol=rtol, atol=0)
        return h
    finally:
        m.free()


def sp(names):
    return [lattice.species(n, 1.0, 0.3 + 0.1 * i) for i, n in enumerate(names)]


def test_empty_species(engine, orc):
    rng = np.random.default_rng(1)
    xyz = rng.uniform(-6, 6, (300, 3)).astype(np.float32)
    K = cd.k_grid(1.5406, 10, 130, 0.5)[1]
    h = check(engine, orc, xyz, [100, 0, 200], 1e-3, cd.channels(25, 1e-3),
              sp(["O", "Al", "Mg"]), K)
    assert h[1].sum() == 0 and h[3].sum() == 0 and h[4].sum() == 0  # 01, 11, 12


def test_empty_species_many_windows(engine, orc):
    """Empty species in a histogram of several windows (the planner samples
    tile pairs of every non-empty species pair to choose the windows)."""
    rng = np.random.default_rng(11)
    xyz = rng.uniform(-6, 6, (500, 3)).astype(np.float32)
    K = cd.k_grid(1.5406, 10, 130, 2.0)[1]
    h = check(engine, orc, xyz, [0, 200, 0, 300, 0], 5e-5,
              cd.channels(25, 5e-5), sp(["O", "Al", "Mg", "Fe", "O"]), K)
    assert h.shape[0] == 15 and h[0].sum() == 0


def test_coincident_atoms(engine, orc):
    rng = np.random.default_rng(2)
    base = rng.uniform(-5, 5, (150, 3)).astype(np.float32)
    xyz = np.concatenate([base, base[:70], base[10:90]])  # exact duplicates
    K = cd.k_grid(1.5406, 10, 130, 0.25)[1]
    h = check(engine, orc, xyz, [150, 70, 80], 1e-3, cd.channels(20, 1e-3),
              sp(["O", "Al", "Fe"]), K)
    assert h[1][0] == 70  # 0-1 pairs at distance 0 off the diagonal block


def test_tiny_bin_count(engine, orc):
    xyz = np.array([[0, 0, 0], [0.4, 0, 0], [0, 0.9, 0], [1.2, 0, 0]], np.float32)
    K = cd.k_grid(1.5406, 10, 130, 1.0)[1]
    check(engine, orc, xyz, [4], 1.0, 3, sp(["O"]), K)
    check(engine, orc, xyz, [1, 3], 1.0, 3, sp(["O", "Al"]), K)


def test_one_atom(engine, orc):
    xyz = np.zeros((1, 3), np.float32)
    K = cd.k_grid(1.5406, 10, 130, 1.0)[1]
    h = check(engine, orc, xyz, [1], 1e-3, 10, sp(["O"]), K)
    assert h[0][0] == 1


def test_many_species(engine, orc):
    rng = np.random.default_rng(3)
    counts = [int(c) for c in rng.integers(20, 200, 10)]
    xyz = rng.uniform(-8, 8, (sum(counts), 3)).astype(np.float32)
    names = ["O", "Al", "Mg", "Fe", "O", "Al", "Mg", "Fe", "O", "Al"]
    K = cd.k_grid(1.5406, 10, 130, 0.1)[1]
    h = check(engine, orc, xyz, counts, 1e-3, cd.channels(30, 1e-3), sp(names), K)
    assert h.shape[0] == 55


@pytest.mark.parametrize("nbins", [114688, 114689])
def test_window_capacity_edge(engine, orc, nbins):
    """Exactly one full shared-memory window, and one bin more (two
    windows, the second holding a single bin)."""
    rng = np.random.default_rng(4)
    xyz = (rng.uniform(-1, 1, (900, 3)) * [40, 1, 1]).astype(np.float32)
    rstep = 90.0 / nbins
    K = cd.k_grid(1.5406, 10, 130, 2.0)[1]
    check(engine, orc, xyz, [400, 500], rstep, nbins, sp(["O", "Al"]), K)
