"""Generate the golden fixtures from the reference's shipped example data.

Reads the reference checkout (path given as the first argument, default
/root/reference) and writes, next to this script:

* ``GammaAl2O3_10nm.deb.xz`` and ``UH3_7nm.deb.xz`` — the shipped example
  inputs, xz-compressed byte for byte (Data/GammaAl2O3_10nm.deb,
  Data/UH3_7nm.deb).
* ``UH3_7nm.xyz.xz`` and ``UH3_7nm_reduced.xyz.xz`` — the shipped .xyz
  sources of UH3_7nm.deb (six and four columns), from which the reference's
  Matlab converter wrote that .deb (Data/UH3_7nm{,_reduced}.xyz).
* ``golden.json`` — for every shipped output (the six
  Data/GammaAl2O3_10nm.debx<i>x<j> histograms and the .debI intensities of
  Gamma and UH3): the SHA-256 and line count of the file with its CRLF line
  ends turned into LF, plus sampled lines, so a test can check a whole
  output file without the reference present. Also the per-block pair totals
  printed by the reference's run log (Data/cmd-logfile.txt: "Distances
  Expected ... Observed").

The reference wrote these files on Windows (CRLF); the engine and the oracle
write LF, which is what the reference writes on a POSIX host.
"""
import hashlib
import json
import lzma
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def lf_bytes(path):
    with open(path, "rb") as f:
        return f.read().replace(b"\r\n", b"\n")


def describe(path, every):
    b = lf_bytes(path)
    lines = b.decode().splitlines()
    return {
        "sha256": hashlib.sha256(b).hexdigest(),
        "lines": len(lines),
        "sample_every": every,
        "sample": {str(i): lines[i] for i in range(0, len(lines), every)},
        "head": lines[:10],
        "tail": lines[-10:],
    }


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    data = os.path.join(ref, "Data")
    for name in ("GammaAl2O3_10nm.deb", "UH3_7nm.deb", "UH3_7nm.xyz",
                 "UH3_7nm_reduced.xyz"):
        with open(os.path.join(data, name), "rb") as f:
            raw = f.read()
        with open(os.path.join(HERE, name + ".xz"), "wb") as f:
            f.write(lzma.compress(raw, preset=9 | lzma.PRESET_EXTREME))
    out = {"Gamma": {}, "UH3": {}}
    for p in ("0x0", "0x1", "0x2", "1x1", "1x2", "2x2"):
        out["Gamma"]["debx" + p] = describe(
            os.path.join(data, "GammaAl2O3_10nm.debx" + p), 997)
    out["Gamma"]["debI"] = describe(os.path.join(data, "GammaAl2O3_10nm.debI"), 97)
    out["UH3"]["debI"] = describe(os.path.join(data, "UH3_7nm.debI"), 97)
    # Per-block totals from the reference's console log.
    log = open(os.path.join(data, "cmd-logfile.txt"), encoding="latin-1").read()
    totals = [int(m.group(1)) for m in re.finditer(
        r"Distances Expected: (\d+) - Distances Observed: \d+", log)]
    out["Gamma"]["block_totals"] = totals
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote", HERE)


if __name__ == "__main__":
    main()
