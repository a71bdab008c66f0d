"""The reference program itself on the GPU (cuDebye-v15.cu, compiled by
`make -C oracle ref` from an edited copy: CUDA 13 / gcc fixes only) as a
second parity point beside the CPU oracle:

* on the shipped Gamma-Al2O3 input it must write the six .debx files byte
  for byte as shipped (the same digests the engine is held to), on the
  shipped UH3 input the shipped .debI and the engine's to 6 digits, and
* on seeded synthetic models the engine's command line must write the same
  .debx files as the reference program, byte for byte, and a .debI that
  agrees to the format's print precision.

Skipped where the reference program was not built (its source is needed
once, to make the edited copy)."""
import hashlib
import os
import shutil
import subprocess

import numpy as np
import pytest

import cudebye_gb300 as cd
from cudebye_gb300 import lattice
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def sha(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


@pytest.fixture(scope="module")
def refprog():
    import __graft_entry__
    __graft_entry__.build()
    if not os.path.exists(pyoracle.REF_BIN):
        pytest.skip("reference program not built (its source was never here)")
    return pyoracle.REF_BIN


def run_ref(refprog, deb, timeout=600):
    """Run the reference program on `deb` (outputs land beside it)."""
    # its banner is not UTF-8 (cuDebye-v15.cu:610)
    r = subprocess.run([refprog, deb], capture_output=True,
                       encoding="latin-1", timeout=timeout)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    # its own consistency checks (cuDebye-v15.cu:371-410) must stay quiet
    assert "WARNING" not in r.stdout, r.stdout[-4000:]
    return r.stdout


def read_debI(path):
    a = np.loadtxt(path)
    return a[:, 0], a[:, 1]


def test_reference_program_gamma_golden(refprog, golden_deb, golden, tmp_path):
    deb = str(tmp_path / "Gamma.deb")
    shutil.copy(golden_deb["Gamma"], deb)
    run_ref(refprog, deb)
    for pair in ("0x0", "0x1", "0x2", "1x1", "1x2", "2x2"):
        assert sha(deb + "x" + pair) == golden["Gamma"]["debx" + pair]["sha256"], pair
    tt, ref_I = read_debI(deb + "I")
    g = golden["Gamma"]["debI"]
    assert len(tt) == g["lines"]
    for i, want in g["sample"].items():
        b = [float(v) for v in want.split("\t")]
        assert tt[int(i)] == b[0]
        # 6 significant digits on both sides: one unit of the last digit
        assert abs(ref_I[int(i)] - b[1]) <= 1.1e-5 * abs(b[1]), (i, ref_I[int(i)], b)


def test_reference_program_uh3(refprog, golden_deb, golden, tmp_path):
    """The other shipped input (UH3_7nm.deb, intensities only): the
    reference program's .debI on this GPU, the shipped one and the
    engine's command line agree to the format's 6 digits."""
    ref_dir, eng_dir = tmp_path / "ref", tmp_path / "eng"
    ref_dir.mkdir()
    eng_dir.mkdir()
    shutil.copy(golden_deb["UH3"], str(ref_dir / "UH3.deb"))
    shutil.copy(golden_deb["UH3"], str(eng_dir / "UH3.deb"))
    run_ref(refprog, str(ref_dir / "UH3.deb"))
    r = subprocess.run([cd.CLI_PATH, str(eng_dir / "UH3.deb"), "--quiet"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    tt_r, I_r = read_debI(str(ref_dir / "UH3.debI"))
    tt_e, I_e = read_debI(str(eng_dir / "UH3.debI"))
    assert np.array_equal(tt_r, tt_e)
    assert (np.abs(I_e - I_r) / np.abs(I_r)).max() <= 1.1e-5
    g = golden["UH3"]["debI"]
    assert len(tt_r) == g["lines"]
    for i, want in g["sample"].items():
        b = [float(v) for v in want.split("\t")]
        assert abs(I_r[int(i)] - b[1]) <= 1.1e-5 * abs(b[1]), (i, I_r[int(i)], b)


@pytest.mark.parametrize("case", ["spinel", "random3", "random1"])
def test_engine_cli_matches_reference_program(refprog, case, tmp_path):
    if case == "spinel":
        m = lattice.spinel(radius=22.0, target=9000, seed=11)
    else:
        rng = np.random.default_rng(17 if case == "random3" else 5)
        m = lattice.random_model(rng, 3000, 12000, lattice.GRID_CU, case, 17)
        if case == "random1":  # one species: only the diagonal kernel
            m = lattice.SynthModel(m.xyz, [m.natoms], m.names[:1],
                                   m.species[:1], m.rstep, m.rmax, m.lam,
                                   m.tt_min, m.tt_max, m.tt_step, m.seed,
                                   m.label)
    ref_dir, eng_dir = tmp_path / "ref", tmp_path / "eng"
    ref_dir.mkdir()
    eng_dir.mkdir()
    # small launch grid so the reference splits each block into several
    # launches, partial ones included (cuDebye-v15.cu:152-272)
    m.write_deb(str(ref_dir / "m.deb"), block=8, grid=96, hist=2)
    shutil.copy(str(ref_dir / "m.deb"), str(eng_dir / "m.deb"))
    run_ref(refprog, str(ref_dir / "m.deb"))
    r = subprocess.run([cd.CLI_PATH, str(eng_dir / "m.deb"), "--quiet"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    ns = len(m.counts)
    for i in range(ns):
        for j in range(i, ns):
            name = "m.debx%dx%d" % (i, j)
            assert sha(str(eng_dir / name)) == sha(str(ref_dir / name)), name
    tt_r, I_r = read_debI(str(ref_dir / "m.debI"))
    tt_e, I_e = read_debI(str(eng_dir / "m.debI"))
    assert np.array_equal(tt_r, tt_e)
    rel = np.abs(I_e - I_r) / np.abs(I_r)
    assert rel.max() <= 1.1e-5, float(rel.max())
