"""Pin the CPU oracle against the reference's shipped outputs.

The reference's example run (Data/GammaAl2O3_10nm.deb, hist=2) shipped six
.debx histograms and a .debI; Data/UH3_7nm.deb shipped a .debI. The oracle
must reproduce every histogram file byte for byte (bit-exact bins and
counts) and the intensity files byte for byte at their 6-digit print
precision. Digests of the shipped files live in tests/golden/golden.json
(made by tests/golden/make_golden.py), so this runs without the reference.
"""
import hashlib
import os

import numpy as np
import pytest

REF_DATA = "/root/reference/Data"


def sha(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


@pytest.fixture(scope="module")
def gamma_run(orc, golden_deb, tmp_path_factory):
    prefix = str(tmp_path_factory.mktemp("orc") / "Gamma.deb")
    orc.run_deb(golden_deb["Gamma"], prefix)
    return prefix


@pytest.mark.parametrize("pair", ["0x0", "0x1", "0x2", "1x1", "1x2", "2x2"])
def test_gamma_debx_bit_exact(gamma_run, golden, pair):
    g = golden["Gamma"]["debx" + pair]
    path = gamma_run + "x" + pair
    assert sha(path) == g["sha256"], "histogram file differs from the reference"
    with open(path) as f:
        lines = f.read().splitlines()
    assert len(lines) == g["lines"]


def test_gamma_debI_exact(gamma_run, golden):
    assert sha(gamma_run + "I") == golden["Gamma"]["debI"]["sha256"]


def test_gamma_block_totals(gamma_run, golden):
    """Sum of each .debx equals the reference log's 'Distances Observed'."""
    totals = []
    for pair in ["0x0", "0x1", "0x2", "1x1", "1x2", "2x2"]:
        a = np.loadtxt(gamma_run + "x" + pair)
        totals.append(int(a[:, 1].sum()))
    assert totals == golden["Gamma"]["block_totals"]


def test_uh3_debI_exact(orc, golden_deb, golden, tmp_path):
    prefix = str(tmp_path / "UH3.deb")
    orc.run_deb(golden_deb["UH3"], prefix)
    assert sha(prefix + "I") == golden["UH3"]["debI"]["sha256"]
    assert not os.path.exists(prefix + "x0x0")  # hist = 0: no .debx


@pytest.mark.skipif(not os.path.isdir(REF_DATA),
                    reason="reference checkout not present")
def test_fixtures_match_reference_files(golden):
    """The committed digests are those of the reference's shipped files."""
    for pair in ["0x0", "0x1", "0x2", "1x1", "1x2", "2x2"]:
        with open(os.path.join(REF_DATA, "GammaAl2O3_10nm.debx" + pair), "rb") as f:
            b = f.read().replace(b"\r\n", b"\n")
        assert hashlib.sha256(b).hexdigest() == golden["Gamma"]["debx" + pair]["sha256"]


def test_pair_bin_formula(orc):
    """Unfused FP32: (dx*dx + dy*dy) + dz*dz, IEEE sqrtf, roundf."""
    f = np.float32
    for (a, b, rstep) in [((0, 0, 0), (1, 0, 0), 1e-4),
                          ((0.0, 0.0, 0.0), (2.7869, 0.0, 0.0), 1e-4),
                          ((1.5, -2.25, 3.0), (-1.0, 0.5, 0.125), 1e-3)]:
        inv = f(1.0 / rstep)
        d = [f(b[i]) - f(a[i]) for i in range(3)]
        s = f(f(d[0] * d[0]) + f(d[1] * d[1]))
        s = f(s + f(d[2] * d[2]))
        p = f(np.sqrt(s) * inv)
        want = int(np.floor(p + f(0.5))) if p - np.floor(p) != 0.5 else int(np.floor(p)) + 1
        assert orc.pair_bin(a, b, rstep) == want
