"""The .xyz -> .deb converter (dbx_xyz2deb, the reference's Matlab
xyz2deb): pinned to the reference's shipped pair Data/UH3_7nm.xyz ->
Data/UH3_7nm.deb, byte for byte, from both the six-column and the
four-column .xyz. Host only, no GPU."""
import lzma
import os

import pytest

import cudebye_gb300 as cd

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def unpack(name, dst):
    with open(os.path.join(GOLDEN, name + ".xz"), "rb") as f:
        raw = lzma.decompress(f.read())
    with open(dst, "wb") as f:
        f.write(raw)
    return raw


def table_from_deb(deb_bytes, path):
    """A RIETAN-layout table (element a1..a5 c b1..b5) holding the
    coefficients of the .deb's species lines (n name occ Beq a1..a5 b1..b5
    c), behind a comment block and a column header as in the real file."""
    lines = deb_bytes.decode().split("\n")
    nsp = int(lines[3])
    rows = []
    for l in lines[4:4 + nsp]:
        t = l.split()
        a, b, c = t[4:9], t[9:14], t[14]
        rows.append(" ".join([t[1].lower() if t[1] == "U" else t[1]] + a + [c] + b))
    with open(path, "w") as f:
        f.write("#  Waasmaier & Kirfel coefficients (test excerpt)\n#\n")
        f.write("Element a1 a2 a3 a4 a5 c b1 b2 b3 b4 b5\n")
        f.write("\n".join(rows) + "\n")


@pytest.mark.parametrize("xyz", ["UH3_7nm.xyz", "UH3_7nm_reduced.xyz"])
def test_uh3_xyz_gives_the_shipped_deb(tmp_path, xyz):
    want = unpack("UH3_7nm.deb", str(tmp_path / "want.deb"))
    src = str(tmp_path / xyz)
    unpack(xyz, src)
    table = str(tmp_path / "table.txt")
    table_from_deb(want, table)  # element names matched without case
    out = cd.xyz2deb(src, table)  # the script's defaults
    assert out == src[:-3] + "deb"
    with open(out, "rb") as f:
        got = f.read()
    assert got == want


def test_header_options_and_errors(tmp_path):
    src = tmp_path / "two.xyz"
    src.write_text("O 0 0 0 0.5 1.25\nAl 3 0 0 1 0.5\nO 0 4 0 0.5 1.25\n")
    table = tmp_path / "t.txt"
    table.write_text("# c\nElement a1 a2 a3 a4 a5 c b1 b2 b3 b4 b5\n"
                     "O 1 2 3 4 5 6 7 8 9 10 11\nAl 11 12 13 14 15 16 17 18 19 20 21\n")
    out = cd.xyz2deb(str(src), str(table), str(tmp_path / "x.deb"),
                     lam=0.7107, tt_min=5, tt_max=150, tt_step=0.05, rstep=0.001,
                     intensity=1, distances=1, device=1, block=8, grid=1024)
    lines = open(out).read().split("\n")
    assert lines[0] == "1 8 1024"
    assert lines[1] == "0.710700 5.00 150.00 0.05"
    # centred: x in [0, 3] -> [-1.5, 1.5], y in [0, 4] -> [-2, 2]; max r 2.5
    assert lines[2] == "6 0.0010 2"  # 2 ceil(1.025 * 2.5)
    assert lines[3] == "2"
    assert lines[4].startswith("1 Al 1.0000 0.5000 11.000000")
    assert lines[4].endswith(" 17.000000 18.000000 19.000000 20.000000 21.000000 16.000000")
    assert lines[5].startswith("2 O 0.5000 1.2500 1.000000")
    assert lines[6:9] == ["1.5\t-2\t0", "-1.5\t-2\t0", "-1.5\t2\t0"]
    d = cd.read_deb(out)  # the engine's reader takes it
    assert d.counts == [1, 2] and d.hist == 2
    with pytest.raises(cd.DebyeError) as e:
        cd.xyz2deb(str(tmp_path / "missing.xyz"), str(table))
    assert e.value.code == -4
    src.write_text("Fe 0 0 0\n")
    with pytest.raises(cd.DebyeError) as e:  # not in the table
        cd.xyz2deb(str(src), str(table))
    assert e.value.code == -5
