"""The whole-file drop-in on the GPU against the reference's own shipped
outputs: `cudebye GammaAl2O3_10nm.deb` must write the six .debx files byte
for byte as the reference did (digests in tests/golden/golden.json), and a
.debI that agrees with the shipped one to its print precision."""
import hashlib
import os
import subprocess

import numpy as np
import pytest

import cudebye_gb300 as cd

pytestmark = pytest.mark.gpu
PAIRS = ["0x0", "0x1", "0x2", "1x1", "1x2", "2x2"]


def sha(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def check_debI(path, g, rtol):
    with open(path) as f:
        lines = f.read().splitlines()
    assert len(lines) == g["lines"]
    for i, want in g["sample"].items():
        a = [float(v) for v in lines[int(i)].split("\t")]
        b = [float(v) for v in want.split("\t")]
        assert a[0] == b[0]
        # both sides are printed to 6 significant digits: allow one unit
        # of the last digit
        assert abs(a[1] - b[1]) <= rtol * abs(b[1]), (i, a, b)


@pytest.fixture(scope="module")
def gamma_gpu(engine, golden_deb, tmp_path_factory):
    prefix = str(tmp_path_factory.mktemp("gpu") / "Gamma.deb")
    engine.run_deb(golden_deb["Gamma"], prefix)
    return prefix


@pytest.mark.parametrize("pair", PAIRS)
def test_gamma_debx_bit_exact(gamma_gpu, golden, pair):
    assert sha(gamma_gpu + "x" + pair) == golden["Gamma"]["debx" + pair]["sha256"]


def test_gamma_debI(gamma_gpu, golden):
    check_debI(gamma_gpu + "I", golden["Gamma"]["debI"], 1.1e-5)


def test_uh3_cli(golden_deb, golden, tmp_path):
    """The command-line drop-in, as the reference is called
    (Matlab/multisim.m:56): cudebye <file.deb>."""
    import __graft_entry__
    __graft_entry__.build()
    prefix = str(tmp_path / "UH3.deb")
    r = subprocess.run([cd.CLI_PATH, golden_deb["UH3"], "--out", prefix],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    check_debI(prefix + "I", golden["UH3"]["debI"], 1.1e-5)
    assert not os.path.exists(prefix + "x0x0")


def test_cli_missing_file(tmp_path):
    r = subprocess.run([cd.CLI_PATH, str(tmp_path / "nope.deb")],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "does not exist" in r.stdout
