"""GPU histogram parity: the engine's int64 pair histograms must equal the
CPU oracle's bin for bin (the reference's FP32 formula, cuDebye-v15.cu:
88-146), through the C ABI, on seeded inputs and the reference's edge
cases: diagonal blocks with i == j, ragged tiles, one-atom species,
windows split across shared-memory capacity, 16-bit counter wraps, and
distances beyond rmax."""
import os
import subprocess

import numpy as np
import pytest

import cudebye_gb300 as cd
from cudebye_gb300 import lattice

pytestmark = pytest.mark.gpu


def gpu_vs_oracle(engine, orc, xyz, counts, rstep, nbins):
    m = engine.upload(xyz, counts)
    try:
        got = engine.histogram(m, rstep, nbins)
    finally:
        m.free()
    want, bad = orc.model_histograms(xyz, counts, rstep, nbins)
    assert bad == 0
    np.testing.assert_array_equal(got, want)
    return got


@pytest.mark.parametrize("counts,seed", [
    ([1], 0), ([2], 1), ([127], 2), ([128], 3), ([129], 4),
    ([300, 1], 5), ([1, 1, 1], 6), ([513, 77, 250], 7), ([1000, 3000], 8)])
def test_random_clusters(engine, orc, counts, seed):
    rng = np.random.default_rng(seed)
    n = sum(counts)
    xyz = rng.uniform(-12, 12, size=(n, 3)).astype(np.float32)
    nbins = cd.channels(45.0, 1e-3)
    gpu_vs_oracle(engine, orc, xyz, counts, 1e-3, nbins)


def test_plain_small_workload(engine, orc):
    m = lattice.plain_small()
    h = gpu_vs_oracle(engine, orc, m.xyz, m.counts, m.rstep, m.nbins)
    assert int(h.sum()) == m.pairs


def test_multi_window(engine, orc):
    """Fine bins: 400,002 bins exceed one shared-memory window, so tile
    pairs are grouped into several windows by their bounding boxes."""
    m = lattice.spinel(radius=14.0, target=1500, seed=11, rstep=1e-4)
    nbins = cd.channels(40.0, 1e-4)
    gpu_vs_oracle(engine, orc, m.xyz, m.counts, 1e-4, nbins)


@pytest.mark.parametrize("rstep", [4e-4, 1.5e-4, 4e-5])
def test_fine_bins_many_windows(engine, orc, rstep):
    """A 25,000-atom spinel-like particle binned finer than one window
    holds: 155,002 bins (2 windows), 413,335 (4) and 1,550,001 (14); tile
    pairs are listed per window from their bounding boxes, and every bin
    equals the oracle's."""
    m = lattice.spinel(radius=30.0, target=25000, seed=13, rstep=rstep)
    nbins = cd.channels(m.rmax, rstep)
    h = gpu_vs_oracle(engine, orc, m.xyz, m.counts, rstep, nbins)
    assert int(h.sum()) == m.pairs


ROWQ = r"""
import numpy as np, sys
sys.path.insert(0, %r)
import cudebye_gb300 as cd
from cudebye_gb300 import lattice
from oracle import pyoracle as orc
for radius, target, seed, rstep in ((30.0, 25000, 13, 1.5e-4), (14.0, 1500, 11, 1e-4)):
    m = lattice.spinel(radius=radius, target=target, seed=seed, rstep=rstep)
    nbins = cd.channels(m.rmax, rstep)
    with cd.Engine(0) as e:
        mod = e.upload(m.xyz, m.counts)
        got = e.histogram(mod, rstep, nbins)
        one = e.split_calc_dist(mod, 1, 1, rstep, nbins)
    want, bad = orc.model_histograms(m.xyz, m.counts, rstep, nbins)
    assert bad == 0
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(one, want[len(m.counts)])
print("OK")
"""


@pytest.mark.parametrize("factor", ["0", "0.01"])
def test_row_quarter_items(orc, factor):
    """Multi-window histograms with the 32-row item shape never used
    (DBX_HIST_ROWQ=0: 128-row items over column quarters only) and used
    wherever it lists fewer pairs (0.01), in child processes: every bin
    equals the oracle's, including diagonal and ragged tiles."""
    code = ROWQ % os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, DBX_HIST_ROWQ=factor)
    r = subprocess.run(["python", "-c", code], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr


def test_single_pair_entry_point(engine, orc):
    m = lattice.spinel(radius=12.0, target=1200, seed=12)
    mod = engine.upload(m.xyz, m.counts)
    starts = np.concatenate([[0], np.cumsum(m.counts)[:-1]])
    try:
        for (r, c) in cd.pair_list(len(m.counts)):
            got = engine.split_calc_dist(mod, r, c, m.rstep, m.nbins)
            want, _ = orc.block_histogram(m.xyz, starts[r], m.counts[r],
                                          starts[c], m.counts[c], r == c,
                                          m.rstep, m.nbins)
            np.testing.assert_array_equal(got, want)
    finally:
        mod.free()


def test_exact_lattice_ties(engine, orc):
    """Unjittered lattice: many exactly equal distances and x.5 bin ties."""
    g = np.arange(12, dtype=np.float32) * np.float32(0.5)
    xyz = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    gpu_vs_oracle(engine, orc, xyz, [len(xyz)], 0.25, cd.channels(12, 0.25))
    gpu_vs_oracle(engine, orc, xyz, [900, len(xyz) - 900], 1e-3,
                  cd.channels(12, 1e-3))


def test_counter_wraps(orc, tmp_path):
    """Millions of pairs in one bin per CTA task: the packed 16-bit shared
    counters wrap many times (low half into high half and out of the word)
    and must still give exact counts. Runs in a child process with few
    tasks so each task sees >65535 counts in a bin."""
    code = r"""
import numpy as np, sys
sys.path.insert(0, %r)
import cudebye_gb300 as cd
from oracle import pyoracle as orc
n0, n1 = 7000, 5000
xyz = np.zeros((n0 + n1 + 3, 3), np.float32)
xyz[n0:n0 + n1, 0] = 1.0          # species 1 at x = 1: all 0-1 pairs in bin 1
xyz[-3:] = [[0.5, 0, 0], [0, 0.5, 0], [0, 0, 3]]
counts = [n0, n1, 3]
with cd.Engine(0) as e:
    m = e.upload(xyz, counts)
    got = e.histogram(m, 1.0, 8)
want, bad = orc.model_histograms(xyz, counts, 1.0, 8)
assert bad == 0
np.testing.assert_array_equal(got, want)
assert got[0, 0] == n0 * (n0 + 1) // 2 and got[1, 1] == n0 * n1
print("OK")
""" % os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, DBX_HIST_TASKS="3")
    r = subprocess.run(["python", "-c", code], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr


WRAP_EDGE = r"""
import numpy as np, re, sys
sys.path.insert(0, %r)
import cudebye_gb300 as cd
from oracle import pyoracle as orc
n0, n1, n2 = 6000, 6000, 3000
xyz = np.zeros((n0 + n1 + n2, 3), np.float32)
xyz[n0:n0 + n1, 0] = 6.0
xyz[n0 + n1:, 0] = 8.0
counts = [n0, n1, n2]
with cd.Engine(0) as e:
    m = e.upload(xyz, counts)
    # 7 bins (odd): the 36M pairs 0-1 all bin at 6, the last bin, whose low
    # half carries into the window's spare half (bin 7) on every wrap;
    # none of that is out of range. 0-2 pairs bin at 8: out of range.
    try:
        e.histogram(m, 1.0, 7)
        raise SystemExit("no range error")
    except cd.DebyeError as err:
        assert err.code == -7, err
        got_bad = int(re.search(r"(\d+) distances", str(err)).group(1))
    _, bad = orc.model_histograms(xyz, counts, 1.0, 7)
    assert got_bad == bad == n0 * n2, (got_bad, bad)
    # 9 bins: everything in range, exact
    got = e.histogram(m, 1.0, 9)
    want, bad = orc.model_histograms(xyz, counts, 1.0, 9)
    assert bad == 0
    np.testing.assert_array_equal(got, want)
    # 6 bins: the 36M pairs at 6 are out of range; every lane's clamp lands
    # on the same spare word, which wraps many times: the count stays exact
    try:
        e.histogram(m, 1.0, 6)
        raise SystemExit("no range error")
    except cd.DebyeError as err:
        got_bad = int(re.search(r"(\d+) distances", str(err)).group(1))
    _, bad = orc.model_histograms(xyz, counts, 1.0, 6)
    assert got_bad == bad == n0 * n1 + n0 * n2, (got_bad, bad)
print("OK")
"""


def test_wraps_at_the_window_edge(orc):
    """Counter wraps in the last bin of an odd-sized window (its carry goes
    to the spare half past the window and must not count as a range error),
    and exact range-error counts when tens of millions of pairs fall beyond
    rmax into the same spare counter. Few tasks, so each wraps often."""
    code = WRAP_EDGE % os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, DBX_HIST_TASKS="3")
    r = subprocess.run(["python", "-c", code], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr


def test_kernel_sqrt_is_ieee_for_every_float(engine):
    """The histogram kernels' branch-free square root equals the IEEE
    sqrtf bit for bit on every non-negative float (2^31 - 2^23 + 1
    inputs)."""
    checked, bad, first = engine.check_sqrt()
    assert checked == 0x7F800001
    assert bad == 0, "first mismatch at bits 0x%08x" % first
    with pytest.raises(cd.DebyeError) as e:
        engine.check_sqrt(0x80000000, 0x80000001)  # negative floats: refused
    assert e.value.code == -1


def test_out_of_range_is_an_error(engine):
    """A distance beyond rmax: the reference writes out of bounds
    (README.md, "Third Line"); the engine returns DBX_ERR_RANGE."""
    xyz = np.array([[0, 0, 0], [0, 0, 10]], np.float32)
    m = engine.upload(xyz, [2])
    try:
        with pytest.raises(cd.DebyeError) as e:
            engine.histogram(m, 0.1, cd.channels(5.0, 0.1))
        assert e.value.code == -7
        h = engine.histogram(m, 0.1, cd.channels(10.0, 0.1))  # context still usable
        assert h[0, 0] == 2 and h[0, 100] == 1
    finally:
        m.free()


def test_out_of_range_count_many_windows(orc):
    """A fine-binned histogram of several windows whose rmax is half the
    particle's extent: the range error reports exactly the oracle's count
    of distances beyond rmax (each counted once, although their tile pairs
    reach several windows)."""
    code = r"""
import numpy as np, re, sys
sys.path.insert(0, %r)
import cudebye_gb300 as cd
from cudebye_gb300 import lattice
from oracle import pyoracle as orc
m = lattice.spinel(radius=12.0, target=900, seed=17, rstep=3e-5)
nbins = cd.channels(m.rmax / 2, 3e-5)
assert nbins > 3 * 114688
with cd.Engine(0) as e:
    mod = e.upload(m.xyz, m.counts)
    try:
        e.histogram(mod, 3e-5, nbins)
        raise SystemExit("no range error")
    except cd.DebyeError as err:
        assert err.code == -7, err
        got = int(re.search(r"(\d+) distances", str(err)).group(1))
    _, bad = orc.model_histograms(m.xyz, m.counts, 3e-5, nbins)
    assert got == bad > 0, (got, bad)
    h = e.histogram(mod, 3e-5, cd.channels(m.rmax, 3e-5))
    want, bad = orc.model_histograms(m.xyz, m.counts, 3e-5, cd.channels(m.rmax, 3e-5))
    assert bad == 0
    np.testing.assert_array_equal(h, want)
print("OK")
""" % os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run(["python", "-c", code], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr


def test_pattern_range_error_then_pattern(engine, orc):
    """A full pattern whose rmax is below the particle's extent: dbx_pattern
    reads back the histograms' out-of-range count with the intensities and
    returns DBX_ERR_RANGE with the oracle's count; the model's histograms are
    not kept, and a pattern with enough bins that follows on the same
    context and model equals the FP64 oracle's within 1e-6."""
    import re
    m = lattice.spinel(radius=12.0, target=1200, seed=19)
    tt, K = m.k_grid()
    K = K[::20]
    nbins = cd.channels(m.rmax / 2, m.rstep)
    mod = engine.upload(m.xyz, m.counts)
    try:
        with pytest.raises(cd.DebyeError) as e:
            engine.pattern(mod, m.rstep, nbins, m.species, K)
        assert e.value.code == -7
        got = int(re.search(r"(\d+) distances", str(e.value)).group(1))
        _, bad = orc.model_histograms(m.xyz, m.counts, m.rstep, nbins)
        assert got == bad > 0, (got, bad)
        I = engine.pattern(mod, m.rstep, m.nbins, m.species, K)
        want_h, bad = orc.model_histograms(m.xyz, m.counts, m.rstep, m.nbins)
        assert bad == 0
        want = orc.intensity(K, want_h, m.species, m.rstep)
        assert float(np.max(np.abs(I - want) / np.abs(want))) <= 1e-6
    finally:
        mod.free()


def test_out_of_range_count_one_window(engine, orc):
    """One window (rmax half the particle's extent, 1e-3 A bins): the pairs
    beyond rmax go to the lanes' out-of-range counters by the clamp of the
    one-window pair loop; the range error reports exactly the oracle's
    count of them, and the full-range histogram that follows on the same
    context equals the oracle's bin for bin."""
    import re
    m = lattice.spinel(radius=14.0, target=1500, seed=18)
    nbins = cd.channels(m.rmax / 2, m.rstep)
    assert nbins < 114688
    mod = engine.upload(m.xyz, m.counts)
    try:
        with pytest.raises(cd.DebyeError) as e:
            engine.histogram(mod, m.rstep, nbins)
        assert e.value.code == -7
        got = int(re.search(r"(\d+) distances", str(e.value)).group(1))
        _, bad = orc.model_histograms(m.xyz, m.counts, m.rstep, nbins)
        assert got == bad > 0, (got, bad)
        h = engine.histogram(mod, m.rstep, m.nbins)
        want, bad = orc.model_histograms(m.xyz, m.counts, m.rstep, m.nbins)
        assert bad == 0
        np.testing.assert_array_equal(h, want)
    finally:
        mod.free()


def test_bad_arguments(engine):
    m = engine.upload(np.zeros((2, 3), np.float32), [2])
    stale = cd.Model(engine, m.id, m.counts)
    try:
        with pytest.raises(cd.DebyeError) as e:
            engine.split_calc_dist(m, 1, 0, 0.1, 10)
        assert e.value.code == -1
    finally:
        m.free()
    with pytest.raises(cd.DebyeError) as e:
        engine.histogram(stale, 0.1, 10)
    assert e.value.code == -8


@pytest.mark.parametrize("rstep", [1e-3, 4e-4])
def test_device_sort_large_model(engine, orc, rstep):
    """Models of 32,768 atoms or more are sorted on the device; their
    histograms (one window, and several windows, whose plan copies the tile
    boxes back to the host) equal the oracle's."""
    m = lattice.spinel(radius=34.0, target=40000, seed=19, rstep=rstep)
    assert m.natoms >= 32768
    nbins = cd.channels(m.rmax, rstep)
    h = gpu_vs_oracle(engine, orc, m.xyz, m.counts, rstep, nbins)
    assert int(h.sum()) == m.pairs


DEVICE_SORT_EDGES = r"""
import numpy as np, re, sys
sys.path.insert(0, %r)
import cudebye_gb300 as cd
from cudebye_gb300 import lattice
from oracle import pyoracle as orc
rng = np.random.default_rng(5)
def check(e, xyz, counts, rstep, nbins):
    xyz = np.ascontiguousarray(xyz, np.float32)
    m = e.upload(xyz, counts)
    try:
        got = e.histogram(m, rstep, nbins)
    finally:
        m.free()
    want, bad = orc.model_histograms(xyz, counts, rstep, nbins)
    assert bad == 0
    np.testing.assert_array_equal(got, want)
with cd.Engine(0) as e:
    # empty and one-atom species among others, many species
    counts = [0, 1, 300, 0, 129, 128, 7, 1000, 2, 0, 55]
    check(e, rng.uniform(-9, 9, (sum(counts), 3)), counts, 1e-3, cd.channels(32, 1e-3))
    # every atom at one point (no extent), and a flat layer (one axis flat)
    check(e, np.zeros((300, 3)), [200, 100], 0.01, 10)
    flat = rng.uniform(-5, 5, (400, 3)); flat[:, 2] = 1.5
    check(e, flat, [400], 1e-3, cd.channels(15, 1e-3))
    # a lattice with exact ties, several windows
    g = np.arange(10, dtype=np.float32) * np.float32(0.5)
    lat = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    check(e, lat, [600, 400], 2e-5, cd.channels(8, 2e-5))
    # a NaN coordinate: the engine bins its 50 pairs (49 others and itself)
    # out of range, a deliberate difference from the reference, whose
    # (int)roundf(NaN) depends on the platform's conversion
    xyz = rng.uniform(-3, 3, (50, 3)).astype(np.float32); xyz[7, 1] = np.nan
    m = e.upload(xyz, [50])
    try:
        e.histogram(m, 1e-3, cd.channels(12, 1e-3))
        raise SystemExit("no range error")
    except cd.DebyeError as err:
        got = int(re.search(r"(\d+) distances", str(err)).group(1))
    finally:
        m.free()
    assert got == 50, got
    # the same over several windows: each of the 50 counted once
    m = e.upload(xyz, [50])
    try:
        e.histogram(m, 1e-5, cd.channels(12, 1e-5))
        raise SystemExit("no range error")
    except cd.DebyeError as err:
        got = int(re.search(r"(\d+) distances", str(err)).group(1))
    finally:
        m.free()
    assert got == 50, got
print("OK")
"""


def test_device_sort_edge_cases():
    """The device sort forced for every model size: empty, one-atom and
    many species, coincident atoms, a flat layer and exact lattice ties over
    several windows give the oracle's histograms; a NaN coordinate gives an
    exact range-error count."""
    code = DEVICE_SORT_EDGES % os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, DBX_DEVICE_SORT_MIN="1")
    r = subprocess.run(["python", "-c", code], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr


def test_interleaved_and_planar_uploads_agree(engine, orc):
    """dbx_model_upload_xyz (interleaved [n][3], de-interleaved on the host
    for small models and on the device before the device sort for large
    ones) and dbx_model_upload (x, y, z planes) give the same histograms,
    and the oracle's."""
    for m in (lattice.spinel(radius=14.0, target=2500, seed=61),
              lattice.spinel(radius=34.0, target=60000, seed=62)):  # 42,735 atoms: device sort
        h1 = engine.upload(m.xyz, m.counts)
        h2 = engine.upload_planes(m.xyz[:, 0], m.xyz[:, 1], m.xyz[:, 2], m.counts)
        try:
            a = engine.histogram(h1, m.rstep, m.nbins)
            b = engine.histogram(h2, m.rstep, m.nbins)
        finally:
            h1.free()
            h2.free()
        np.testing.assert_array_equal(a, b)
        want, bad = orc.model_histograms(m.xyz, m.counts, m.rstep, m.nbins)
        assert bad == 0
        np.testing.assert_array_equal(a, want)
