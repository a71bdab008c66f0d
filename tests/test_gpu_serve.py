"""The pattern server (dbx_server_*): continuous batching with admission by
HBM footprint. Every result must match the FP64 oracle (max rel <= 1e-6)
and be the same whether the request ran alone or inside a mix of
concurrent requests of other sizes and q grids."""
import threading

import numpy as np
import pytest

import cudebye_gb300 as cd
from cudebye_gb300 import lattice

pytestmark = pytest.mark.gpu


def make_requests(seed, n, nmin=300, nmax=4000):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        npts = int(rng.integers(300, 2000))
        grid = (1.5406, 10.0, 130.0, 120.0 / (npts - 1))
        out.append(lattice.random_model(rng, nmin, nmax, grid, "r%d" % i, seed))
    return out


def oracle_I(orc, m, K, species=None):
    h, bad = orc.model_histograms(m.xyz, m.counts, m.rstep, m.nbins)
    assert bad == 0
    return orc.intensity(K, h, species or m.species, m.rstep)


def test_concurrent_requests_match_oracle(orc):
    reqs = make_requests(51, 8)
    with cd.Server(0) as srv:
        tickets = [srv.submit(m.species, m.rstep, m.nbins, m.k_grid()[1],
                              xyz=m.xyz, counts=m.counts) for m in reqs]
        results = [srv.wait(t, len(m.k_grid()[1])) for t, m in zip(tickets, reqs)]
        for m, (I, mid, lat) in zip(reqs, results):
            want = oracle_I(orc, m, m.k_grid()[1])
            assert np.max(np.abs(I - want) / np.abs(want)) <= 1e-6
            assert mid > 0 and lat > 0
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["resident_models"] == len(reqs)


def test_rescoring_resident_models(orc):
    m = make_requests(52, 1)[0]
    tt, K = m.k_grid()
    with cd.Server(0) as srv:
        I0, mid, _ = srv.wait(srv.submit(m.species, m.rstep, m.nbins, K,
                                         xyz=m.xyz, counts=m.counts), len(K))
        # new B factors, same q grid: weighted sum of the resident row sums
        sp2 = [lattice.species(n, s.occ, s.beq * 0.3 + 0.05)
               for n, s in zip(m.names, m.species)]
        I1, mid1, _ = srv.wait(srv.submit(sp2, m.rstep, m.nbins, K, model=mid),
                               len(K))
        assert mid1 == mid
        want = oracle_I(orc, m, K, sp2)
        assert np.max(np.abs(I1 - want) / np.abs(want)) <= 1e-6
        # a new q grid: contraction of the resident histograms
        K2 = cd.k_grid(0.7107, 5.0, 150.0, 0.05)[1]
        I2, _, _ = srv.wait(srv.submit(sp2, m.rstep, m.nbins, K2, model=mid),
                            len(K2))
        want2 = oracle_I(orc, m, K2, sp2)
        assert np.max(np.abs(I2 - want2) / np.abs(want2)) <= 1e-6
        with pytest.raises(cd.DebyeError) as e:  # unknown model
            srv.wait(srv.submit(sp2, m.rstep, m.nbins, K, model=99999), len(K))
        assert e.value.code == -8


def test_same_result_alone_and_in_the_mix():
    mix = make_requests(53, 10)
    probe = mix[4]
    K = probe.k_grid()[1]
    with cd.Server(0) as srv:
        alone, _, _ = srv.wait(srv.submit(probe.species, probe.rstep, probe.nbins,
                                          K, xyz=probe.xyz, counts=probe.counts),
                               len(K))
    with cd.Server(0) as srv:
        results = {}

        def client(i):
            m = mix[i]
            t = srv.submit(m.species, m.rstep, m.nbins, m.k_grid()[1],
                           xyz=m.xyz, counts=m.counts)
            results[i] = srv.wait(t, len(m.k_grid()[1]))[0]

        threads = [threading.Thread(target=client, args=(i,)) for i in range(len(mix))]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        assert srv.stats()["completed"] == len(mix)
    np.testing.assert_array_equal(results[4], alone)


def test_admission_by_hbm_budget(orc):
    """Under a budget that holds the lanes and about 1.5 models, sequential
    new models evict the least recently used idle one; a re-score of an
    evicted model reports DBX_ERR_MODEL; a request that can never fit
    reports DBX_ERR_NOMEM; results stay exact."""
    m = make_requests(54, 1, nmin=3000, nmax=4000)[0]
    K = m.k_grid()[1]

    def run(srv):
        I, mid, _ = srv.wait(srv.submit(m.species, m.rstep, m.nbins, K,
                                        xyz=m.xyz, counts=m.counts), len(K))
        return I, mid

    with cd.Server(0) as cal:  # calibrate: rounds alternate two lanes
        run(cal)
        u1 = cal.stats()["device_bytes"]   # lane 0 workspace + 1 model
        run(cal)
        u2 = cal.stats()["device_bytes"]   # + lane 1 workspace + 1 model
        run(cal)
        st = cal.stats()                   # + 1 model
        per_model, reserve = st["device_bytes"] - u2, st["lane_reserve"]
    assert per_model > 0
    budget = u2 + reserve + int(0.5 * per_model)  # room for two models
    with cd.Server(0, hbm_budget=budget) as srv:
        ids = []
        for _ in range(4):
            I, mid = run(srv)
            ids.append(mid)
        st = srv.stats()
        assert st["completed"] == 4 and st["evictions"] >= 2
        assert st["resident_models"] <= 2 and st["device_bytes"] <= budget
        want = oracle_I(orc, m, K)
        assert np.max(np.abs(I - want) / np.abs(want)) <= 1e-6
        with pytest.raises(cd.DebyeError) as e:  # the first model was evicted
            srv.wait(srv.submit(m.species, m.rstep, m.nbins, K, model=ids[0]),
                     len(K))
        assert e.value.code == -8
    with cd.Server(0, hbm_budget=u1 // 4) as srv:  # can never fit
        with pytest.raises(cd.DebyeError) as e:
            run(srv)
        assert e.value.code == -3


def test_a_failing_request_does_not_fail_its_round(orc):
    """A request whose model has a distance beyond its rmax fails only
    itself: the round it shared is redone request by request, and the
    others' results are exact."""
    good = make_requests(55, 5, nmin=500, nmax=1500)
    bad = make_requests(56, 1, nmin=500, nmax=1500)[0]
    with cd.Server(0) as srv:
        tickets = []
        for i, m in enumerate(good):
            if i == 2:  # too few bins: distances beyond rmax
                K = bad.k_grid()[1]
                tickets.append((srv.submit(bad.species, bad.rstep, bad.nbins // 4,
                                           K, xyz=bad.xyz, counts=bad.counts),
                                len(K)))
            K = m.k_grid()[1]
            tickets.append((srv.submit(m.species, m.rstep, m.nbins, K,
                                       xyz=m.xyz, counts=m.counts), len(K)))
        results = []
        for t, nq in tickets:
            try:
                results.append(srv.wait(t, nq))
            except cd.DebyeError as e:
                results.append(e)
        assert isinstance(results[2], cd.DebyeError) and results[2].code == -7
        ok = [r for i, r in enumerate(results) if i != 2]
        for m, (I, mid, _) in zip(good, ok):
            want = oracle_I(orc, m, m.k_grid()[1])
            assert np.max(np.abs(I - want) / np.abs(want)) <= 1e-6
        assert srv.stats()["completed"] == len(tickets)
