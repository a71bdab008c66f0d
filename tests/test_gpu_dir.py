"""The directory driver (dbx_run_dir / `cudebye --dir`, the reference's
multisim) and the binary .deb form on the GPU: every output equals what the
single-file drop-in writes for the same file (.debx byte for byte, .debI
values within 1e-9), files that already have a .debI are left alone, .xyz
files without a .deb are converted first, and a binary .deb gives the same
outputs as its text form."""
import hashlib
import lzma
import os
import shutil
import subprocess

import numpy as np
import pytest

import cudebye_gb300 as cd
from cudebye_gb300 import lattice

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sha(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def debI(path):
    return np.loadtxt(path, delimiter="\t")


def same_outputs(a_prefix, b_prefix, nspecies, hist):
    if hist in (1, 2):
        for r in range(nspecies):
            for c in range(r, nspecies):
                assert sha(a_prefix + "x%dx%d" % (r, c)) == sha(b_prefix + "x%dx%d" % (r, c))
    if hist != 1:
        A, B = debI(a_prefix + "I"), debI(b_prefix + "I")
        np.testing.assert_array_equal(A[:, 0], B[:, 0])
        np.testing.assert_allclose(A[:, 1], B[:, 1], rtol=1e-9)
    else:
        assert not os.path.exists(a_prefix + "I")


def make_dir(tmp_path):
    d = tmp_path / "runs"
    d.mkdir()
    rng = np.random.default_rng(61)
    files = []
    for i, hist in enumerate([2, 0, 1, 2]):
        m = lattice.random_model(rng, 500, 3000, lattice.GRID_CU, "m%d" % i, 61)
        name = "m%d.deb" % i
        m.write_deb(str(d / name), hist=hist)
        files.append((name, len(m.counts), hist))
    # another rstep: a group of its own
    m = lattice.spinel(radius=10.0, target=800, seed=5, rstep=2e-3)
    m.write_deb(str(d / "s.deb"), hist=2)
    files.append(("s.deb", len(m.counts), 2))
    # already computed: must be left alone
    shutil.copy(str(d / "m1.deb"), str(d / "done.deb"))
    (d / "done.debI").write_text("untouched\n")
    # an .xyz without .deb: converted with the table, then computed
    with open(os.path.join(GOLDEN, "UH3_7nm.xyz.xz"), "rb") as f:
        (d / "uh3.xyz").write_bytes(lzma.decompress(f.read()))
    with open(os.path.join(GOLDEN, "UH3_7nm.deb.xz"), "rb") as f:
        uh3 = lzma.decompress(f.read()).decode().split("\n")
    rows = []
    for l in uh3[4:6]:
        t = l.split()
        rows.append(" ".join([t[1]] + t[4:9] + [t[14]] + t[9:14]))
    table = tmp_path / "table.txt"
    table.write_text("# test excerpt\nElement a1 a2 a3 a4 a5 c b1 b2 b3 b4 b5\n"
                     + "\n".join(rows) + "\n")
    files.append(("uh3.deb", 2, 0))
    return d, str(table), files


def test_dir_driver_matches_single_runs(engine, tmp_path):
    d, table, files = make_dir(tmp_path)
    engine.run_dir(str(d), table)
    assert (d / "done.debI").read_text() == "untouched\n"
    assert not os.path.exists(str(d / "done.debx0x0"))
    with open(os.path.join(GOLDEN, "UH3_7nm.deb.xz"), "rb") as f:
        assert (d / "uh3.deb").read_bytes() == lzma.decompress(f.read())
    ref = tmp_path / "single"
    ref.mkdir()
    for name, P, hist in files:
        engine.run_deb(str(d / name), str(ref / name))
        same_outputs(str(d / name), str(ref / name), P, hist)
    # a second run finds nothing left to do (hist 1 files have no .debI and
    # are computed again, as multisim does)
    before = {f: sha(str(d / f)) for f in os.listdir(str(d))}
    engine.run_dir(str(d), table)
    after = {f: sha(str(d / f)) for f in os.listdir(str(d))}
    assert before == after


def test_dir_cli_and_errors(tmp_path):
    import __graft_entry__
    __graft_entry__.build()
    d = tmp_path / "cli"
    d.mkdir()
    m = lattice.plain_small()
    m.write_deb(str(d / "a.deb"), hist=0)
    (d / "bad.deb").write_text("0 8 1024\n1.5 10 20 0.1\n10 0.01 0\n1\n"
                               "2 O 1 0 1 1 1 1 1 1 1 1 1 1 0\n1 2 3\n")
    r = subprocess.run([cd.CLI_PATH, "--dir", str(d), "--quiet"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 1  # bad.deb: atom count mismatch
    assert "doesn't match" in r.stderr
    assert os.path.exists(str(d / "a.debI"))  # the good file was still done
    assert not os.path.exists(str(d / "bad.debI"))


def test_binary_deb_gives_the_same_outputs(engine, golden_deb, tmp_path):
    src = golden_deb["UH3"]
    b = cd.deb_pack(src, str(tmp_path / "uh3.debb"))
    engine.run_deb(src, str(tmp_path / "t.deb"))
    engine.run_deb(b, str(tmp_path / "b.deb"))
    assert sha(str(tmp_path / "t.debI")) == sha(str(tmp_path / "b.debI"))
    r = subprocess.run([cd.CLI_PATH, b, "--out", str(tmp_path / "c.deb"), "--quiet"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert sha(str(tmp_path / "t.debI")) == sha(str(tmp_path / "c.debI"))
