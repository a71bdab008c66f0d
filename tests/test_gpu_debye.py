"""GPU Debye-sum parity against the FP64 CPU oracle (cuDebye-v15.cu:447-577).

Tolerances, written here as the contract:
 * prefactor (atomicScatter): FP64 on both sides, rel <= 1e-13
 * DBX_DEBYE_FP64 direct sum: rel <= 1e-11 per q
 * DBX_DEBYE_TC (tensor-core split contraction): max rel <= 1e-6 per q
 * DBX_DEBYE_FP32 (plain FP32 baseline form): reported, loose bound only
"""
import numpy as np
import pytest

import cudebye_gb300 as cd
from cudebye_gb300 import lattice

pytestmark = pytest.mark.gpu


def test_atomic_prop(engine, orc):
    tt, K = cd.k_grid(1.5406, 0.0, 180.0, 0.05)
    for a, b in [("O2-", "Al3+"), ("Al", "Al"), ("Fe", "O")]:
        sa, sb = lattice.species(a, 0.8333, 2.0), lattice.species(b, 1.0, 0.5)
        got = engine.atomic_prop(sa, sb, K)
        want = orc.prefactor(K, sa, sb)
        np.testing.assert_allclose(got, want, rtol=1e-13)


def _model_case(engine, orc, m, K, mode):
    mod = engine.upload(m.xyz, m.counts)
    try:
        got = engine.intensity(mod, m.rstep, m.nbins, m.species, K, mode=mode)
        h = engine.histogram(mod, m.rstep, m.nbins)
    finally:
        mod.free()
    want = orc.intensity(K, h, m.species, m.rstep)
    return got, want


def test_fp64_direct(engine, orc):
    m = lattice.plain_small()
    tt, K = m.k_grid()
    got, want = _model_case(engine, orc, m, K, "fp64")
    rel = np.abs(got - want) / np.abs(want)
    assert rel.max() <= 1e-11, rel.max()


def test_fp64_multi_species(engine, orc):
    m = lattice.spinel(radius=16.0, target=4000, seed=21)
    tt, K = m.k_grid()
    got, want = _model_case(engine, orc, m, K[::7], "fp64")
    rel = np.abs(got - want) / np.abs(want)
    assert rel.max() <= 1e-11, rel.max()


def test_tc_precision(engine, orc):
    m = lattice.spinel(radius=16.0, target=4000, seed=22)
    tt, K = m.k_grid()
    got, want = _model_case(engine, orc, m, K, "tc")
    rel = np.abs(got - want) / np.abs(want)
    assert rel.max() <= 1e-6, rel.max()


def test_tc_multi_tile_and_ragged_q(engine, orc):
    """nq not a multiple of 128, columns spanning several 64-chunk tiles
    (>16,384 bins), and a second call on the cached basis."""
    m = lattice.spinel(radius=20.0, target=6000, seed=23)
    tt, K = m.k_grid()
    for Kq in (K[::3], K[5::3]):
        got, want = _model_case(engine, orc, m, Kq, "tc")
        rel = np.abs(got - want) / np.abs(want)
        assert rel.max() <= 1e-6, rel.max()


def test_tc_precision_grid(engine, orc):
    """The 20,000-point q grid (2theta 5-150 deg at 0.7107 A, K up to 17)."""
    m = lattice.spinel(radius=20.0, target=6000, seed=24,
                       grid=lattice.GRID_PRECISION)
    tt, K = m.k_grid()
    assert len(K) == 20000
    got, want = _model_case(engine, orc, m, K[::4], "tc")
    rel = np.abs(got - want) / np.abs(want)
    assert rel.max() <= 1e-6, rel.max()


def test_tc_self_only_and_zero_q(engine, orc):
    """Single-atom species have only the self bin; K = 0 gives the
    reference's NaN only where a non-self bin exists."""
    xyz = np.array([[0, 0, 0], [1.5, 0, 0]], np.float32)
    sp = [lattice.species("O", 1.0, 0.5), lattice.species("Al", 1.0, 0.5)]
    K = np.array([0.0, 0.5, 3.0])
    mod = engine.upload(xyz, [1, 1])
    try:
        got = engine.intensity(mod, 1e-3, cd.channels(4, 1e-3), sp, K, mode="tc")
        h = engine.histogram(mod, 1e-3, cd.channels(4, 1e-3))
    finally:
        mod.free()
    want = orc.intensity(K, h, sp, 1e-3)
    assert np.isnan(want[0]) and np.isnan(got[0])
    np.testing.assert_allclose(got[1:], want[1:], rtol=1e-6)
    mod = engine.upload(xyz[:1], [1])
    try:
        got = engine.intensity(mod, 1e-3, 10, sp[:1], K, mode="tc")
    finally:
        mod.free()
    want = orc.prefactor(K, sp[0], sp[0]) * 1.0
    np.testing.assert_allclose(got, want, rtol=1e-12)


def test_fp32_plain_form_runs(engine, orc):
    m = lattice.plain_small()
    tt, K = m.k_grid()
    got, want = _model_case(engine, orc, m, K[::10], "fp32")
    assert np.all(np.isfinite(got))
    rel = np.abs(got - want) / np.abs(want)
    assert rel.max() < 0.5, rel.max()  # FP32 form: a speed baseline only


def test_zero_q_matches_reference_nan(engine, orc):
    """K = 0 (2theta = 0): the reference evaluates sin(0)/0 = NaN for every
    non-self bin (cuDebye-v15.cu:509); the engine reproduces that."""
    m = lattice.plain_small(natoms=50)
    K = np.array([0.0, 1.0])
    got, want = _model_case(engine, orc, m, K, "fp64")
    assert np.isnan(want[0]) and np.isnan(got[0])
    assert abs(got[1] - want[1]) <= 1e-11 * abs(want[1])


def test_tc3_form_is_the_less_precise_study_form(engine, orc):
    """DBX_DEBYE_TC3 (two digits, three products: BF16x3) runs through the
    same contraction; its error is reported, not bounded by 1e-6, and it is
    never more precise than the exact split on the same histograms."""
    m = lattice.spinel(radius=16.0, target=4000, seed=22,
                       grid=lattice.GRID_PRECISION)
    tt, K = m.k_grid()
    K = K[::8]
    got3, want = _model_case(engine, orc, m, K, "tc3")
    got, _ = _model_case(engine, orc, m, K, "tc")
    rel3 = np.abs(got3 - want) / np.abs(want)
    rel = np.abs(got - want) / np.abs(want)
    assert np.all(np.isfinite(got3))
    assert rel.max() <= 1e-6
    assert rel3.max() >= rel.max()
    assert rel3.max() < 1e-2, rel3.max()


def test_tf32_split_form(engine, orc):
    """DBX_DEBYE_TF32 (each operand split into tf32 hi/lo parts, three
    products with FP32 accumulation per 256-bin chunk, FP64 chunk and q
    sums) against the FP64 oracle on the precision grid (2theta 5-150 deg,
    0.7107 A): its max relative error is bounded by 1e-4 here (4.9e-5
    measured on a GB300: FP32 sums of 256 products per chunk round at
    2^-24 of their magnitude, and the chunk sums cancel), below the BF16x3
    form's (22 significant bits per operand against 16) and above the exact
    split's (whose FP32 sums are exact integers)."""
    m = lattice.spinel(radius=16.0, target=4000, seed=22,
                       grid=lattice.GRID_PRECISION)
    tt, K = m.k_grid()
    K = K[::8]
    got32, want = _model_case(engine, orc, m, K, "tf32")
    got3, _ = _model_case(engine, orc, m, K, "tc3")
    got, _ = _model_case(engine, orc, m, K, "tc")
    rel32 = np.abs(got32 - want) / np.abs(want)
    rel3 = np.abs(got3 - want) / np.abs(want)
    rel = np.abs(got - want) / np.abs(want)
    assert np.all(np.isfinite(got32))
    assert rel32.max() <= 1e-4, (rel32.max(), rel3.max(), rel.max())
    assert rel32.max() < rel3.max(), (rel32.max(), rel3.max())
    assert rel.max() <= rel32.max()


def test_patterns_on_a_caller_stream(engine, orc):
    """dbx_set_stream: patterns launched on a caller's stream equal those on
    the context's own stream bit for bit and the FP64 oracle within 1e-6,
    for a small model (whose prefactors run on the context's second stream,
    joined back into the caller's) and a larger one (in stream order)."""
    torch = pytest.importorskip("torch")
    small = lattice.plain_small()
    large = lattice.spinel(radius=20.0, target=25000, seed=23)
    tt, K = small.k_grid()
    K = K[::15]
    s = torch.cuda.Stream(device=torch.device("cuda", 0))
    for m in (small, large):
        mod = engine.upload(m.xyz, m.counts)
        try:
            own = engine.pattern(mod, m.rstep, m.nbins, m.species, K)
            engine.set_stream(s.cuda_stream)
            try:
                mine = [engine.pattern(mod, m.rstep, m.nbins, m.species, K).copy()
                        for _ in range(3)]
            finally:
                engine.set_stream(None)
            for I in mine:
                np.testing.assert_array_equal(I, own)
            h, bad = orc.model_histograms(m.xyz, m.counts, m.rstep, m.nbins)
            assert bad == 0
            want = orc.intensity(K, h, m.species, m.rstep)
            assert float(np.max(np.abs(own - want) / np.abs(want))) <= 1e-6
        finally:
            mod.free()
