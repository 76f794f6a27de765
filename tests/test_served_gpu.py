"""Parity and bookkeeping of the served path (host queue -> launch slots -> mapped flags)."""
import threading

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _requests(rng, n, lo=1, hi=5000, kinds=(0, 1, 2), alphabet=4):
    k = rng.choice(kinds, n)
    la = np.exp(rng.uniform(np.log(lo), np.log(hi), n)).astype(int)
    lb = np.exp(rng.uniform(np.log(lo), np.log(hi), n)).astype(int)
    sa = [rng.integers(0, alphabet, x) for x in la]
    sb = [rng.integers(0, alphabet, x) for x in lb]
    return k, sa, sb


def _collect(srv, tickets, timeout_s=300):
    assert srv.drain(timeout_s)
    got = {}
    while True:
        t, r, lat = srv.poll_many(4096)
        if len(t) == 0:
            break
        for i in range(len(t)):
            got[int(t[i])] = (r[i], int(lat[i]))
    assert set(got) == set(tickets)
    return [got[t] for t in tickets]


def _check(results, kinds, sa, sb, sc, rule):
    o = O.align_batch(kinds, sa, sb, rule=rule, match=sc.match, mismatch=sc.mismatch, gap=sc.gap)
    res = np.array([r for r, _ in results], dtype=results[0][0].dtype)
    np.testing.assert_array_equal(res["status"], 0)
    np.testing.assert_array_equal(res["score"], o["score"])
    sw = np.asarray(kinds) == 2
    np.testing.assert_array_equal(res["sw_max"][sw], o["sw_max"][sw])
    np.testing.assert_array_equal(res["sw_max_y"][sw], o["sw_y"][sw])
    np.testing.assert_array_equal(res["sw_max_x"][sw], o["sw_x"][sw])
    assert all(lat > 0 for _, lat in results)


@pytest.mark.parametrize("rule", [0, 1])
def test_served_mixed(rule):
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(40 + rule)
    kinds, sa, sb = _requests(rng, 400)
    # wide pairs (global wrap rows), one for the plain path, empty ones
    for n1, n2 in [(16384, 900), (9000, 3000), (17000, 200), (0, 5), (7, 0)]:
        kinds = np.append(kinds, rng.integers(0, 3))
        sa.append(rng.integers(0, 4, n1))
        sb.append(rng.integers(0, 4, n2))
    sc = g.scoring(ed_boundary=rule)
    with g.Server(0, sc=sc) as srv:
        tickets = [srv.submit(int(k), a, b) for k, a, b in zip(kinds, sa, sb)]
        results = _collect(srv, tickets)
        st = srv.stats()
    _check(results, kinds, sa, sb, sc, rule)
    assert st["completed"] == st["submitted"] == len(kinds)
    assert st["queued"] == 0 and st["running"] == 0
    assert st["waves_launched"] >= 1 and st["kernels_launched"] >= 2
    assert 0 < st["hbm_bytes_peak"] <= st["hbm_budget_bytes"]


def test_served_small_budget_many_waves():
    """A tight budget and a small cell cap force many admissions; results stay exact."""
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(7)
    kinds, sa, sb = _requests(rng, 300, hi=3000)
    budget = 1 << 30
    sc = g.scoring(5, -4, -7)
    with g.Server(0, sc=sc, hbm_budget_bytes=budget, wave_max_cells=2_000_000, waves=2) as srv:
        tickets = [srv.submit(int(k), a, b) for k, a, b in zip(kinds, sa, sb)]
        results = _collect(srv, tickets)
        st = srv.stats()
        # a request that alone needs more than a slot's share of the budget is refused
        with pytest.raises(g.GmeError) as e:
            srv.submit(1, np.zeros(16384, np.int32), np.zeros(1 << 24, np.int32))
        assert e.value.status == 6
    _check(results, kinds, sa, sb, sc, 0)
    assert st["waves_launched"] > 5
    assert st["hbm_bytes_peak"] <= budget


def test_served_queue_full_takes_prefix():
    """A full queue takes a prefix of a submit_many call (its tickets are returned);
    the rest submitted again later completes exactly like the rest."""
    import time
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(13)
    kinds, sa, sb = _requests(rng, 500, hi=2000)
    symbols, pairs = g.pack_batch(kinds, sa, sb)
    sc = g.scoring()
    with g.Server(0, sc=sc, queue_max=64) as srv:
        first = srv.submit_many(symbols, pairs)
        assert 0 < len(first) <= 64
        tickets = list(first)
        rest = pairs[len(first):]
        while len(rest):
            t = srv.submit_many(symbols, rest)
            tickets += list(t)
            rest = rest[len(t):]
            if len(rest):
                time.sleep(0.001)
        results = _collect(srv, tickets)
    _check(results, kinds, sa, sb, sc, 0)


def test_served_poll_single_and_threads():
    """gme_poll per ticket, two submitting threads, unknown tickets rejected."""
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(11)
    kinds, sa, sb = _requests(rng, 200, hi=2500)
    sc = g.scoring()
    with g.Server(0, sc=sc, warps_per_block=8) as srv:
        tickets = [None] * len(kinds)

        def submit(part):
            for i in part:
                tickets[i] = srv.submit(int(kinds[i]), sa[i], sb[i])

        th = [threading.Thread(target=submit, args=(range(j, len(kinds), 2),)) for j in range(2)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        assert len(set(tickets)) == len(kinds)
        assert srv.drain(300)
        results = []
        for t in tickets:
            r = srv.poll(t)
            assert r is not None
            res = np.zeros(1, g.RESULT_DTYPE)
            for f in ("score", "sw_max", "sw_max_y", "sw_max_x", "status", "kind"):
                res[f] = r[0][f]
            results.append((res[0], r[1]))
        with pytest.raises(g.GmeError):
            srv.poll(tickets[0])  # already taken
        with pytest.raises(g.GmeError):
            srv.poll(10 ** 12)  # never issued
    _check(results, kinds, sa, sb, sc, 0)


def test_served_close_with_queue():
    """Closing a server with work queued and running neither hangs nor loses the GPU."""
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(3)
    kinds, sa, sb = _requests(rng, 500, lo=500, hi=4000)
    srv = g.Server(0, waves=1, wave_max_cells=2_000_000)
    for k, a, b in zip(kinds, sa, sb):
        srv.submit(int(k), a, b)
    srv.close()
    # the device is still usable afterwards
    with g.Server(0) as srv2:
        t = srv2.submit(0, np.arange(10) % 4, np.arange(12) % 4)
        assert srv2.drain(60)
        r, _ = srv2.poll(t)
        assert r["status"] == 0
        assert r["score"] == O.align(0, np.arange(10) % 4, np.arange(12) % 4)["score"]
