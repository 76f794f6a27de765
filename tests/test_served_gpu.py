"""Parity and bookkeeping of the served path, in both modes: ring (host queue ->
device-resident job rings -> one persistent kernel -> mapped flags) and waves (host
queue -> launch slots of the batched kernel -> mapped flags)."""
import threading
import time

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


MODES = [0, 1]  # SERVE_RING, SERVE_WAVES


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("rule", [0, 1])
def test_served_mixed(rule, mode):
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(40 + rule)
    kinds, sa, sb = _requests(rng, 400)
    # wide pairs (global wrap rows), one for the plain path, empty ones
    for n1, n2 in [(16384, 900), (9000, 3000), (17000, 200), (0, 5), (7, 0)]:
        kinds = np.append(kinds, rng.integers(0, 3))
        sa.append(rng.integers(0, 4, n1))
        sb.append(rng.integers(0, 4, n2))
    sc = g.scoring(ed_boundary=rule)
    with g.Server(0, sc=sc, mode=mode) as srv:
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
    with g.Server(0, sc=sc, hbm_budget_bytes=budget, wave_max_cells=2_000_000, waves=2,
                  mode=g.SERVE_WAVES) as srv:
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


@pytest.mark.parametrize("mode", MODES)
def test_served_queue_full_takes_prefix(mode):
    """A full queue takes a prefix of a submit_many call (its tickets are returned);
    the rest submitted again later completes exactly like the rest."""
    import time
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(13)
    kinds, sa, sb = _requests(rng, 500, hi=2000)
    symbols, pairs = g.pack_batch(kinds, sa, sb)
    sc = g.scoring()
    with g.Server(0, sc=sc, queue_max=64, mode=mode) as srv:
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


@pytest.mark.parametrize("mode", MODES)
def test_served_poll_single_and_threads(mode):
    """gme_poll per ticket, two submitting threads, unknown tickets rejected."""
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(11)
    kinds, sa, sb = _requests(rng, 200, hi=2500)
    sc = g.scoring()
    with g.Server(0, sc=sc, warps_per_block=8, mode=mode) as srv:
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


@pytest.mark.parametrize("mode", MODES)
def test_served_close_with_queue(mode):
    """Closing a server with work queued and running neither hangs nor loses the GPU."""
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(3)
    kinds, sa, sb = _requests(rng, 500, lo=500, hi=4000)
    srv = g.Server(0, waves=1, wave_max_cells=2_000_000, mode=mode)
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


def test_ring_tight_budget_recycles_the_arena():
    """Ring mode under a budget whose symbol arena is smaller than the stream: jobs are
    admitted as earlier ones complete and free their space; the server never holds
    more than the budget, refuses a request the arena could never hold, and every
    result is exact."""
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(21)
    kinds, sa, sb = _requests(rng, 4000, lo=1000, hi=8000)
    # about 250 MB of per-CTA rows, the rest split between the symbol arena (about
    # 85 MB) and launches of wide pairs: the stream's symbols (about 120 MB) cycle
    budget = 400 << 20
    sc = g.scoring(4, -3, -5)
    with g.Server(0, sc=sc, hbm_budget_bytes=budget) as srv:
        with pytest.raises(g.GmeError) as e:
            srv.submit(2, np.zeros(16384, np.int32), np.zeros(1 << 25, np.int32))
        assert e.value.status == 6
        tickets = [srv.submit(int(k), a, b) for k, a, b in zip(kinds, sa, sb)]
        results = _collect(srv, tickets)
        st = srv.stats()
    _check(results, kinds, sa, sb, sc, 0)
    assert st["hbm_bytes_peak"] <= budget


def test_ring_kernel_leaves_when_idle_and_comes_back():
    """The persistent kernel leaves after a short idle time; work submitted later
    launches it again and completes exactly."""
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(22)
    sc = g.scoring()
    with g.Server(0, sc=sc) as srv:
        allk, alla, allb, tickets = [], [], [], []
        for round_ in range(3):
            kinds, sa, sb = _requests(rng, 60, hi=3000)
            tickets += [srv.submit(int(k), a, b) for k, a, b in zip(kinds, sa, sb)]
            allk += list(kinds); alla += sa; allb += sb
            assert srv.drain(120)
            time.sleep(0.2)  # longer than the kernel's idle limit
        results = _collect(srv, tickets)
        st = srv.stats()
    _check(results, np.array(allk), alla, allb, sc, 0)
    assert st["waves_launched"] >= 3  # one launch of the persistent kernel per round


def test_ring_teams_share_the_largest_pairs():
    """Pairs of 2^26 cells and more are shared by a team of CTAs (band groups claimed
    one at a time); more such pairs at once than there are teams run alone.  Every
    result is exact, SW best cells included."""
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(23)
    shapes = [(8192, 8192), (16384, 5000), (3000, 30000), (2048, 40000), (16384, 4096), (12000, 9000)]
    kinds, sa, sb = [], [], []
    for i, (n1, n2) in enumerate(shapes * 3):
        kinds.append(i % 3)
        sa.append(rng.integers(0, 4, n1))
        sb.append(rng.integers(0, 4, n2))
    # more team-sized pairs than teams, then small ones behind them
    for i in range(70):
        kinds.append(i % 3)
        sa.append(rng.integers(0, 4, 4096))
        sb.append(rng.integers(0, 4, 16384))
    k2, a2, b2 = _requests(rng, 200, hi=3000)
    kinds = np.array(kinds + list(k2))
    sa += a2
    sb += b2
    sc = g.scoring(3, -2, -4)
    with g.Server(0, sc=sc) as srv:
        tickets = [srv.submit(int(k), a, b) for k, a, b in zip(kinds, sa, sb)]
        results = _collect(srv, tickets, timeout_s=600)
        st = srv.stats()
    _check(results, kinds, sa, sb, sc, 0)
    assert st["completed"] == len(kinds)


def test_ring_wide_pairs_while_traffic_flows():
    """A pair wider than the persistent kernel's rows, submitted while small requests
    keep arriving, completes while they still arrive (the kernel steps aside for its
    launch and comes back), and every result is exact."""
    import gpumemefficient_gb300 as g
    rng = np.random.default_rng(24)
    sc = g.scoring()
    wide = [(0, rng.integers(0, 4, 20000), rng.integers(0, 4, 3000)),
            (2, rng.integers(0, 4, 40000), rng.integers(0, 4, 500))]
    with g.Server(0, sc=sc) as srv:
        stop = threading.Event()
        small = []

        def feed():
            r2 = np.random.default_rng(25)
            while not stop.is_set():
                k, a, b = _requests(r2, 20, hi=2000)
                for x in zip(k, a, b):
                    small.append((int(x[0]), x[1], x[2], srv.submit(int(x[0]), x[1], x[2])))
                time.sleep(0.002)

        th = threading.Thread(target=feed)
        th.start()
        time.sleep(0.2)
        wt = [srv.submit(k, a, b) for k, a, b in wide]
        t0 = time.time()
        got = {}
        while len(got) < len(wt) and time.time() - t0 < 30:
            for t in wt:
                if t not in got:
                    r = srv.poll(t)
                    if r is not None:
                        got[t] = r
            time.sleep(0.005)
        waited = time.time() - t0
        stop.set()
        th.join()
        assert len(got) == len(wt), "wide pairs starved by the persistent kernel"
        assert waited < 10
        results = _collect(srv, [t for *_, t in small])
    _check(results, np.array([k for k, *_ in small]), [a for _, a, _, _ in small], [b for _, _, b, _ in small], sc, 0)
    o = O.align_batch([k for k, _, _ in wide], [a for _, a, _ in wide], [b for _, _, b in wide], rule=0)
    for i, t in enumerate(wt):
        r = got[t][0]
        assert r["status"] == 0 and r["score"] == o["score"][i]
