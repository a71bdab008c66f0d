"""CPU tests: host logic, file formats, the C-ABI library's exports, and a
bit-level model of the device histogram's arithmetic. No GPU needed."""
import ctypes
import os
import re

import numpy as np
import pytest

import cudebye_gb300 as cd
from cudebye_gb300 import lattice

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "cudebye.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(dbx_\w+)\s*\(", txt)))


@pytest.fixture(scope="module")
def built_lib():
    from cudebye_gb300 import build
    return build.build()


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)  # loads without a GPU
    syms = declared_symbols()
    assert syms, "no declarations parsed"
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert set(syms) == set(cd.EXPORTS), "python binding list out of date"


def test_host_entry_points_without_gpu(built_lib):
    """The pure host entry points run without a device."""
    lib = cd.load_library(built_lib)
    assert lib.dbx_channels(356.0, 0.0001) == int(356 / 0.0001) + 2
    n = lib.dbx_k_grid(1.5418, 10.0, 140.0, 0.02, None, None)
    assert n == 6501
    tt = np.zeros(n)
    K = np.zeros(n)
    dp = ctypes.POINTER(ctypes.c_double)
    lib.dbx_k_grid(1.5418, 10.0, 140.0, 0.02, tt.ctypes.data_as(dp),
                   K.ctypes.data_as(dp))
    tt2, K2 = cd.k_grid(1.5418, 10.0, 140.0, 0.02)
    np.testing.assert_array_equal(tt, tt2)
    np.testing.assert_allclose(K, K2, rtol=1e-15)
    assert lib.dbx_strerror(-7) == b"distance beyond rmax"
    # no device: creating a context fails cleanly, with a status, no exit
    ctx = ctypes.c_void_p()
    rc = lib.dbx_create(ctypes.byref(ctx), 0, 0)
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        assert rc == -2 and not ctx


def test_noalloc_argument_checks_without_gpu(built_lib):
    """dbx_pair_histogram_noalloc refuses bad requests before any CUDA call:
    counts whose sum would overflow int64, a single count above the limit,
    equal starts with different counts, negative sizes. Run only where there
    is no GPU, so that the placeholder pointers can never reach a device."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("placeholder pointers: CPU-only check")
    except ImportError:
        pass
    lib = cd.load_library(built_lib)
    f = lib.dbx_pair_histogram_noalloc
    p = ctypes.c_void_p(16)
    big = (1 << 62) + 1  # a_count + b_count overflows int64
    assert f(p, p, p, 0, big, 1, big, 1e-3, 10, p, None) == -11
    assert f(p, p, p, 0, 1834993, 2000000, 1, 1e-3, 10, p, None) == -11
    assert f(p, p, p, 0, 1, 2000000, 1834992, 1e-3, 10, p, None) == -11
    assert f(p, p, p, 5, 10, 5, 11, 1e-3, 10, p, None) == -1
    assert f(p, p, p, 0, -1, 10, 1, 1e-3, 10, p, None) == -1
    assert f(p, p, p, 0, 1, 10, 1, 0.0, 10, p, None) == -1
    assert f(p, p, p, 0, 1, 10, 1, 1e-3, 0, p, None) == -1


def test_tile_order_is_a_hilbert_curve(built_lib):
    """The curve that orders atoms into tiles visits every cell of the
    2^bits cube once, each step to a face neighbour (so runs of it, the
    tiles, are connected and compact)."""
    cd.load_library(built_lib)
    for bits in (1, 2, 3, 4):
        n = 1 << bits
        cells = {}
        for x in range(n):
            for y in range(n):
                for z in range(n):
                    cells[cd.curve_index(x, y, z, bits)] = (x, y, z)
        assert sorted(cells) == list(range(n ** 3)), bits
        for k in range(n ** 3 - 1):
            step = sum(abs(a - b) for a, b in zip(cells[k], cells[k + 1]))
            assert step == 1, (bits, k, cells[k], cells[k + 1])
    # the largest grid the sort uses: corners and a sample stay in range
    top = (1 << 10) - 1
    for c in [(0, 0, 0), (top, top, top), (top, 0, 517), (3, 900, 12)]:
        assert 0 <= cd.curve_index(*c, 10) < 1 << 30
    assert cd.curve_index(1 << 10, 0, 0, 10) == -1
    assert cd.curve_index(0, 0, 0, 11) == -1


def test_k_grid_matches_oracle(orc):
    for grid in [(1.5418, 10.0, 140.0, 0.02), (1.5406, 10.0, 130.0, 0.02),
                 (0.7107, 5.0, 150.0, 145.0 / 19999)]:
        tt, K = cd.k_grid(*grid)
        tt2, K2 = orc.k_grid(*grid)
        assert len(tt) == len(tt2)
        np.testing.assert_array_equal(tt, tt2)
        np.testing.assert_allclose(K, K2, rtol=1e-15)


def test_channels():
    assert cd.channels(356, 0.0001) == 3560002  # Data/cmd-logfile.txt
    assert cd.channels(122, 0.0001) == int(122 / 0.0001) + 2


def test_reduce_check():
    h = np.zeros(100, np.int64)
    h[0] = 10
    h[30] = 45
    r = cd.reduce_check(h, 0.1, 10, 10, True)
    assert r["expected"] == 55 and r["observed"] == 55 and r["bin0"] == 10
    assert r["collisions"] == 0
    h[1] = 2  # two pairs at 0.1 A: below the 0.25 A "collision" limit
    r = cd.reduce_check(h, 0.1, 10, 10, True)
    assert r["collisions"] == 2


def test_read_deb_fixture(golden_deb):
    d = cd.read_deb(golden_deb["UH3"])
    assert d.counts == [27972, 8931] and d.names == ["H", "U"]
    assert d.hist == 0 and d.rmax == 122 and d.rstep == 0.0001
    assert d.xyz.shape == (36903, 3) and d.xyz.dtype == np.float32
    assert d.xyz[0].tolist() == [np.float32(-33.215), np.float32(-32.18533),
                                 np.float32(-31.20217)]
    assert abs(d.species[1].a[0] - 15.679275) < 1e-12


def test_read_deb_errors(tmp_path):
    with pytest.raises(cd.DebyeError) as e:
        cd.read_deb(str(tmp_path / "missing.deb"))
    assert e.value.code == -4
    p = tmp_path / "bad.deb"
    p.write_text("0 8 1024\n1.5 10 20 0.1\n10 0.01 0\n1\n"
                 "2 O 1 0 1 1 1 1 1 1 1 1 1 1 0\n0 0 0\n")
    with pytest.raises(cd.DebyeError) as e:
        cd.read_deb(str(p))
    assert e.value.code == -6


def test_synthetic_workloads():
    m = lattice.plain_small()
    assert m.natoms == 5000 and m.counts == [2000, 3000]
    assert m.pairs == 12502500  # 5000*5001/2
    tt, K = m.k_grid()
    assert len(tt) == 6001
    m2 = lattice.plain_small()
    np.testing.assert_array_equal(m.xyz, m2.xyz)  # seeded
    s = lattice.spinel_10nm()
    assert abs(s.natoms - 118000) < 300 and len(s.counts) == 3
    assert 100000 <= s.nbins <= 110000
    p = lattice.precision()
    assert len(p.k_grid()[0]) == 20000


def test_xyz2deb_rmax_rule():
    xyz = np.array([[0, 0, 0], [10, 0, 0]], np.float32)
    # centred half-extent 5 -> 2*ceil(5*1.025) = 12 (Matlab/xyz2deb.m:204)
    assert lattice.xyz2deb_rmax(xyz) == 12


def _f32_directed(x64, toward):
    """float64 value (exact) rounded to float32 toward zero ('z') or
    toward -inf ('d')."""
    r = x64.astype(np.float32)
    if toward == "z":
        over = np.abs(r.astype(np.float64)) > np.abs(x64)
        r[over] = np.nextafter(r[over], np.float32(0))
    else:
        over = r.astype(np.float64) > x64
        r[over] = np.nextafter(r[over], np.float32(-np.inf))
    return r


def _kernel_round_model(p):
    """The scalar kernel's roundf (bin_rel): floor(RZ(p + 0.5)) read from
    the bits of RD(a + 2^23) (float32 operations emulated exactly in
    float64)."""
    p = np.asarray(p, np.float32)
    a = _f32_directed(p.astype(np.float64) + 0.5, "z")
    t = _f32_directed(a.astype(np.float64) + 8388608.0, "d")
    return t.view(np.int32).astype(np.int64) - 0x4B000000


def _kernel_round2_model(p):
    """The tile kernels' roundf (bins2): q = 2p (exact), t = RD(q +
    8388609), bin = (bits(t) >> 1) + 0x25800000 - bits(2^23)."""
    p = np.asarray(p, np.float32)
    q = (p.astype(np.float64) * 2.0).astype(np.float32)  # exact doubling
    t = _f32_directed(q.astype(np.float64) + 8388609.0, "d")
    bits = t.view(np.int32).astype(np.int64)
    return (bits >> 1) + 0x25800000 - 0x4B000000


def test_exact_roundf_without_conversion():
    rng = np.random.default_rng(0)
    p = np.concatenate([
        rng.uniform(0, 4.2e6, 200000).astype(np.float32),
        rng.uniform(0, 3, 100000).astype(np.float32),
        (np.arange(0, 100000, dtype=np.float32) + np.float32(0.5)),  # ties
        np.nextafter(np.arange(1, 50000, dtype=np.float32) + np.float32(0.5),
                     np.float32(0)),
        np.nextafter(np.float32(0.5), np.float32(0)).reshape(1),
        np.array([0, 0.5, 1.5, 2.5, 4194303.5], np.float32)])
    # roundf for p >= 0: half away from zero = floor(p + 0.5), exact in f64
    want = np.floor(p.astype(np.float64) + 0.5).astype(np.int64)
    np.testing.assert_array_equal(_kernel_round_model(p), want)
    ok = p < np.float32(2 ** 22)  # beyond, every form lands out of range
    np.testing.assert_array_equal(_kernel_round2_model(p)[ok], want[ok])


def test_packed_roundf_every_float():
    """The tile kernels' one-add roundf equals floor(p + 0.5) for every
    float p in [0, 2^22), the bins any histogram can have; larger p give
    bins of at least 2^22 (out of range for every histogram)."""
    lo = int(np.float32(0).view(np.uint32))
    hi = int(np.float32(2.0 ** 22).view(np.uint32))
    step = 1 << 24
    for start in range(lo, hi, step):
        u = np.arange(start, min(start + step, hi), dtype=np.uint32)
        p = u.view(np.float32).astype(np.float64)
        q = 2.0 * p                       # exact
        t = np.floor(q + 8388609.0)       # RD in [2^23, 2^24): the integers
        t = np.where(q + 8388609.0 >= 2.0 ** 24,
                     2.0 * np.floor((q + 8388609.0) / 2.0), t)  # spacing 2
        got = np.floor((t - 8388608.0) / 2.0)
        np.testing.assert_array_equal(got, np.floor(p + 0.5))
    big = np.array([2.0 ** 22, 2.0 ** 23, 3e38], np.float32)
    assert np.all(_kernel_round2_model(big) >= 2 ** 22)


def _u32(x):
    return np.asarray(x).astype(np.uint64) & np.uint64(0xFFFFFFFF)


def _pair_add_bin(u, valid, mode, base, sadj, wl, kb, nbins, uo, ui):
    """The bin form of the tile kernel's pair add (hist.cu pair_add_bin):
    word address, increment and virtual bin, in uint32 arithmetic."""
    lk = _u32(u - base)
    if mode == "safe":
        u2, ign = np.where(valid, u, ui), ~valid
    elif mode == "full":
        u2, ign = np.where(valid, np.minimum(u, uo), ui), ~valid
    else:  # a middle window
        hit = valid & (lk < wl)
        u2, ign = np.where(hit, u, ui), ~hit
    inc = np.where(ign, 0, np.left_shift(np.uint64(1),
                                         _u32(u2 << np.uint64(4)) & np.uint64(31)))
    addr = _u32(sadj + ((u2 >> np.uint64(1)) << np.uint64(2)))
    return addr, inc, _u32(u2 - base)


def _pair_add_raw(w, valid, mode, base, sadj, wl, vo, vi):
    """The raw-bit form (hist.cu pair_add_raw): w = bits(RD(2p + 8388609))."""
    wbase = _u32(2 * base - 0x4B000000)
    sadjw, wl2 = _u32(sadj + 0x4B000000), _u32(2 * wl)
    wo, wi = _u32(wbase + 2 * vo), _u32(wbase + 2 * vi)
    if mode == "safe":
        w2, ign = np.where(valid, w, wi), ~valid
    elif mode == "full":
        w2, ign = np.where(valid, np.minimum(w, wo), wi), ~valid
    else:
        hit = valid & (_u32(w - wbase) < wl2)
        w2, ign = np.where(hit, w, wi), ~hit
    inc = np.where(ign, 0, np.left_shift(np.uint64(1),
                                         (w2 & np.uint64(2)) << np.uint64(3)))
    addr = _u32(sadjw + (w2 & np.uint64(0xFFFFFFFC)))
    return addr, inc, _u32(w2 - wbase) >> np.uint64(1)


def test_raw_bit_pair_add_matches_bin_form():
    """The tile kernel adds a pair either from its bin u = bits(2^23) + bin
    or from the raw rounding bits w = bits(2^23) + 2 bin + r; both must hit
    the same counter word and half (and, for the wrap compensation, the
    same virtual bin) in every mode that uses the raw form, for bins around
    every window edge and for the bits of NaN and infinite distances."""
    rng = np.random.default_rng(5)
    for trial in range(240):
        mode = ("safe", "full", "mid")[trial % 3]
        wl = int(rng.integers(1, 114689))
        nw = (wl + 1) // 2
        if mode == "mid":
            kb = int(rng.integers(0, 3_000_000)) & ~1
            olo = int(rng.integers(0, min(wl, 2000))) & ~1
        else:
            kb, olo = 0, 0
        lane = int(rng.integers(0, 32))
        vo = 2 * (nw + lane)
        vi = vo + 64
        sadj = (int(rng.integers(0, 1 << 14)) * 4
                - ((0x4B000000 + kb) >> 1) * 4) % (1 << 32)
        base = 0x4B000000 + kb + olo
        pkb, pwl = kb + olo, wl - olo
        pvo, pvi = (vo - olo) % (1 << 32), (vi - olo) % (1 << 32)
        edges = np.concatenate([pkb + np.arange(-4, 5), pkb + pwl + np.arange(-4, 5),
                                pkb + pvo + np.arange(-4, 5)])
        absb = np.concatenate([rng.integers(0, 1 << 22, 2000), edges])
        absb = absb[(absb >= 0) & (absb < (1 << 22))].astype(np.uint64)
        r = rng.integers(0, 2, absb.size).astype(np.uint64)
        w = np.concatenate([np.uint64(0x4B000000) + np.uint64(2) * absb + r,
                            np.array([0x7FC00000, 0xFFC00000, 0x7F800000,
                                      0x7F7FFFFF, 0x4B7FFFFF], np.uint64)])
        u = _u32((w >> np.uint64(1)) + np.uint64(0x25800000))
        valid = rng.random(w.size) < 0.8
        a = _pair_add_bin(u, valid, mode, base, sadj, pwl, pkb, None,
                          _u32(pvo + base), _u32(pvi + base))
        b = _pair_add_raw(w, valid, mode, base, sadj, pwl, pvo, pvi)
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)


def test_packed_counter_bookkeeping():
    """Serial model of add16: two 16-bit bins per 32-bit word, wraps and the
    low->high carry compensated in an int64 side array; true counts are
    recovered exactly for adversarial orders."""
    rng = np.random.default_rng(1)
    for trial in range(20):
        nadd = 300000
        bins = rng.choice(2, size=nadd, p=[0.5, 0.5])
        if trial % 3 == 0:
            bins[:] = 0
        if trial % 3 == 1:
            bins[:] = 1
        word = 0
        glob = [0, 0, 0]
        for b in bins:
            sh = 16 * b
            old = word
            word = (word + (1 << sh)) & 0xFFFFFFFF
            if ((old >> sh) & 0xFFFF) == 0xFFFF:
                glob[b] += 65536
                if sh == 0:
                    glob[1] -= 1
                    if (old >> 16) == 0xFFFF:
                        glob[1] += 65536
        got = [(word & 0xFFFF) + glob[0], (word >> 16) + glob[1]]
        assert got == [int((bins == 0).sum()), int((bins == 1).sum())]


def test_text_parser_matches_the_oracle_and_binary_form(golden_deb, tmp_path):
    """The engine's .deb parser (whole-file scan, from_chars) gives the
    oracle's values bit for bit; its binary form (dbx_deb_pack) round-trips
    them, and packing the binary form again gives the same bytes."""
    from oracle import pyoracle as orc
    for key in ("Gamma", "UH3"):
        src = golden_deb[key]
        hdr, sp, xyz = orc.read_deb(src)
        b1 = cd.deb_pack(src, str(tmp_path / (key + ".debb")))
        d = cd.read_debb(b1)
        assert (d.device, d.block, d.grid, d.hist) == (
            hdr["device"], hdr["block"], hdr["grid"], hdr["hist"])
        assert (d.lam, d.tt_min, d.tt_max, d.tt_step, d.rmax, d.rstep) == (
            hdr["lam"], hdr["tt_min"], hdr["tt_max"], hdr["tt_step"],
            hdr["rmax"], hdr["rstep"])
        assert d.counts == [s["n"] for s in sp]
        assert d.names == [s["name"] for s in sp]
        for got, want in zip(d.species, sp):
            assert got.occ == want["occ"] and got.beq == want["beq"]
            assert list(got.a) == want["a"] and list(got.b) == want["b"]
            assert got.c == want["c"]
        assert d.xyz.dtype == np.float32
        np.testing.assert_array_equal(d.xyz.view(np.uint32), xyz.view(np.uint32))
        b2 = cd.deb_pack(b1, str(tmp_path / (key + "2.debb")))
        assert open(b1, "rb").read() == open(b2, "rb").read()


def test_parser_edge_cases(tmp_path):
    p = tmp_path / "e.deb"
    p.write_text("0 8 1024\n1.5 10 20 0.1\n10 0.01 2\n2\n"
                 "1 O 1 0 1 1 1 1 1 1 1 1 1 1 0\n2 Al 1 0 1 1 1 1 1 1 1 1 1 1 0\n"
                 "\n  \r\n+1.5 -0 1e-3\r\n\t0.1 0.2 0.3\n\n7 8 9   \n")
    d = cd.read_debb(cd.deb_pack(str(p), str(tmp_path / "e.debb")))
    assert d.counts == [1, 2]
    np.testing.assert_array_equal(
        d.xyz, np.array([[1.5, -0.0, 1e-3], [0.1, 0.2, 0.3], [7, 8, 9]], np.float32))
    assert np.signbit(d.xyz[0, 1])
    p.write_text("0 8 1024\n1.5 10 20 0.1\n10 0.01 0\n1\n"
                 "2 O 1 0 1 1 1 1 1 1 1 1 1 1 0\n1 2 3\n")
    with pytest.raises(cd.DebyeError) as e:
        cd.deb_pack(str(p), str(tmp_path / "f.debb"))
    assert e.value.code == -6  # count mismatch
    p.write_text("0 8 1024\n1.5 10 20 0.1\n10 0.01 0\n1\n"
                 "1 O 1 0 1 1 1 1 1 1 1 1 1 1 0\n1 x 3\n")
    with pytest.raises(cd.DebyeError) as e:
        cd.deb_pack(str(p), str(tmp_path / "g.debb"))
    assert e.value.code == -5
