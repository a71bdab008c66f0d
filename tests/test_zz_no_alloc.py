"""The no-allocation pair histogram against the regular entry point.

dbx_pair_histogram_noalloc exists for callers that may not allocate device
memory (code living in another framework's memory pool or a fixed arena,
plugins whose host process owns every device allocation, services that
forbid device allocation after start-up): its scratch is one fixed
__device__ array. This test drives it through the C ABI with device
buffers the test itself owns (allocated here by torch, as such a caller's
host framework would) and checks, on two calls in a row that reuse the
shared scratch, that its histograms equal dbx_pair_histogram's bin for bin
(the histogram is integer: the tolerance is exact equality). It also
checks the size limit. Collected last so that a failure here cannot stop
the other tests of a run that stops at the first failure.
"""
import ctypes

import numpy as np
import pytest

import cudebye_gb300 as cd
from cudebye_gb300 import lattice

pytestmark = pytest.mark.gpu

DBX_NOALLOC_MAX_ATOMS = 1834992  # include/cudebye.h


def noalloc(engine, torch, xyz, a0, na, b0, nb, rstep, nbins):
    dev = torch.device("cuda", 0)
    x = torch.tensor(np.ascontiguousarray(xyz[:, 0]), device=dev)
    y = torch.tensor(np.ascontiguousarray(xyz[:, 1]), device=dev)
    z = torch.tensor(np.ascontiguousarray(xyz[:, 2]), device=dev)
    out = torch.full((nbins,), -7, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = engine.lib.dbx_pair_histogram_noalloc(
        ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
        ctypes.c_void_p(z.data_ptr()), a0, na, b0, nb, rstep, nbins,
        ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    return rc, out.cpu().numpy()


def reference_entry(engine, xyz, counts, row, col, rstep, nbins):
    m = engine.upload(xyz, counts)
    try:
        return engine.split_calc_dist(m, row, col, rstep, nbins)
    finally:
        m.free()


def test_noalloc_equals_pair_histogram_twice(engine):
    torch = pytest.importorskip("torch")
    starts = lambda c: np.concatenate([[0], np.cumsum(c)[:-1]]).astype(int)
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


def test_noalloc_rejects_oversized_request(engine):
    torch = pytest.importorskip("torch")
    xyz = np.zeros((4, 3), np.float32)
    # more atoms than the fixed scratch holds: refused before any GPU work
    rc, _ = noalloc(engine, torch, xyz, 0, DBX_NOALLOC_MAX_ATOMS, 0,
                    DBX_NOALLOC_MAX_ATOMS + 1, 1e-3, 100)
    assert cd.ERRORS.get(rc) == "DBX_ERR_LIMIT"
