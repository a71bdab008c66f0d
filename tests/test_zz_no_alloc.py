"""The no-allocation pair histogram against the regular entry point.

dbx_pair_histogram_noalloc exists for callers that may not allocate device
memory (code living in another framework's memory pool or a fixed arena,
plugins whose host process owns every device allocation, services that
forbid device allocation after start-up): its scratch is one fixed
__device__ array. This test drives it through the C ABI with device
buffers the test itself owns (allocated here by torch, as such a caller's
host framework would) and checks, on two calls in a row that reuse the
shared scratch, that its histograms equal dbx_pair_histogram's bin for bin
(the histogram is integer: the tolerance is exact equality), then the CPU
oracle's on ragged and edge cases, and the size limit with device buffers
as large as the request claims. Collected last so that a failure here
cannot stop the other tests of a run that stops at the first failure.
"""
import ctypes

import numpy as np
import pytest

import cudebye_gb300 as cd
from cudebye_gb300 import lattice

pytestmark = pytest.mark.gpu

DBX_NOALLOC_MAX_ATOMS = 1834992  # include/cudebye.h


def device_xyz(torch, xyz):
    dev = torch.device("cuda", 0)
    return [torch.tensor(np.ascontiguousarray(xyz[:, c]), device=dev)
            for c in range(3)]


def call(engine, torch, xyzd, a0, na, b0, nb, rstep, nbins):
    dev = torch.device("cuda", 0)
    x, y, z = xyzd
    out = torch.full((nbins,), -7, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = engine.lib.dbx_pair_histogram_noalloc(
        ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
        ctypes.c_void_p(z.data_ptr()), a0, na, b0, nb, rstep, nbins,
        ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    return rc, out.cpu().numpy()


def noalloc(engine, torch, xyz, a0, na, b0, nb, rstep, nbins):
    return call(engine, torch, device_xyz(torch, xyz), a0, na, b0, nb, rstep,
                nbins)


def reference_entry(engine, xyz, counts, row, col, rstep, nbins):
    m = engine.upload(xyz, counts)
    try:
        return engine.split_calc_dist(m, row, col, rstep, nbins)
    finally:
        m.free()


def starts(c):
    return np.concatenate([[0], np.cumsum(c)[:-1]]).astype(int)


def test_noalloc_equals_pair_histogram_twice(engine):
    torch = pytest.importorskip("torch")
    # call 1: an off-diagonal species block, one shared-memory window
    m1 = lattice.spinel(radius=14.0, target=2500, seed=31)
    s1 = starts(m1.counts)
    rc, got = noalloc(engine, torch, m1.xyz, s1[0], m1.counts[0], s1[2],
                      m1.counts[2], m1.rstep, m1.nbins)
    assert rc == 0, cd.ERRORS.get(rc, rc)
    want = reference_entry(engine, m1.xyz, m1.counts, 0, 2, m1.rstep, m1.nbins)
    np.testing.assert_array_equal(got, want)
    # call 2, right after: a block with itself (i <= j incl. i == j), finer
    # bins spread over three windows, on scratch left by call 1
    m2 = lattice.spinel(radius=12.0, target=1800, seed=32, rstep=1e-4)
    s2 = starts(m2.counts)
    nbins2 = cd.channels(30.0, 1e-4)
    rc, got = noalloc(engine, torch, m2.xyz, s2[1], m2.counts[1], s2[1],
                      m2.counts[1], 1e-4, nbins2)
    assert rc == 0, cd.ERRORS.get(rc, rc)
    want = reference_entry(engine, m2.xyz, m2.counts, 1, 1, 1e-4, nbins2)
    np.testing.assert_array_equal(got, want)
    assert int(got.sum()) == m2.counts[1] * (m2.counts[1] + 1) // 2


def test_noalloc_edge_cases_match_oracle(engine, orc):
    """Ragged blocks against the CPU oracle: an odd bin count whose last
    window ends in a half-used counter word, an empty range, and a range
    error spread over several windows (the in-range bins still counted)."""
    torch = pytest.importorskip("torch")
    m = lattice.spinel(radius=13.0, target=2100, seed=33, rstep=1e-4)
    s = starts(m.counts)
    xyzd = device_xyz(torch, m.xyz)
    # odd nbins over three windows (the last one ends on a low half), past
    # the model's largest distance
    nb_odd = m.nbins | 1
    assert nb_odd % 2 == 1 and 2 * 114688 < nb_odd <= 3 * 114688
    rc, got = call(engine, torch, xyzd, s[0], m.counts[0], s[2], m.counts[2],
                   1e-4, nb_odd)
    want, bad = orc.block_histogram(m.xyz, s[0], m.counts[0], s[2],
                                    m.counts[2], False, 1e-4, nb_odd)
    assert bad == 0 and rc == 0, cd.ERRORS.get(rc, rc)
    np.testing.assert_array_equal(got, want)
    # an empty range: all zeros, no error
    rc, got = call(engine, torch, xyzd, s[1], 0, s[2], m.counts[2], 1e-4, 999)
    assert rc == 0 and not got.any()
    # a range error over several windows: bins end below the largest
    # distance; the pairs below nbins are still counted, bin for bin
    nb_short = 2 * 114688 + 500
    rc, got = call(engine, torch, xyzd, s[0], m.counts[0], s[0], m.counts[0],
                   1e-4, nb_short)
    want, bad = orc.block_histogram(m.xyz, s[0], m.counts[0], s[0],
                                    m.counts[0], True, 1e-4, nb_short)
    assert bad > 0
    assert cd.ERRORS.get(rc) == "DBX_ERR_RANGE"
    np.testing.assert_array_equal(got, want)


def test_noalloc_rejects_oversized_request(engine):
    torch = pytest.importorskip("torch")
    # device coordinates as long as the request claims, so that no access
    # could leave them even if the size check failed
    n = DBX_NOALLOC_MAX_ATOMS + 1
    xyzd = device_xyz(torch, np.zeros((n, 3), np.float32))
    # more atoms than the fixed scratch holds: refused before any GPU work
    rc, _ = call(engine, torch, xyzd, 0, DBX_NOALLOC_MAX_ATOMS, DBX_NOALLOC_MAX_ATOMS,
                 1, 1e-3, 100)
    assert cd.ERRORS.get(rc) == "DBX_ERR_LIMIT"
    rc, _ = call(engine, torch, xyzd, 0, n, 0, n, 1e-3, 100)
    assert cd.ERRORS.get(rc) == "DBX_ERR_LIMIT"
    # equal starts with different counts name no species block
    rc, _ = call(engine, torch, xyzd, 0, 10, 0, 11, 1e-3, 100)
    assert cd.ERRORS.get(rc) == "DBX_ERR_ARG"
