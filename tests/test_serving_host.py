"""Host-side pieces of the serving loop (CPU only): the request stream and the statistics."""
import math

import numpy as np

from iron_gb300.serving import Request, estimate_bytes, make_inputs, request_stream, summarize


def test_request_stream_matches_the_specification():
    reqs = request_stream(2000, rate=200.0, seed=0)
    t = np.array([r.arrival for r in reqs])
    assert t[0] == 0.0 and np.all(np.diff(t) >= 0)
    # Poisson at 200/s: mean inter-arrival 5 ms within sampling error
    assert abs(np.diff(t).mean() - 0.005) < 0.0005
    frac = np.mean([r.kind == "laplace" for r in reqs])
    assert abs(frac - 0.7) < 0.04
    ns = np.array([r.n for r in reqs])
    assert ns.min() >= 4 and ns.max() <= 64
    # log-uniform: the median side is near sqrt(4 * 64) = 16
    assert 14 <= np.median(ns) <= 18
    again = request_stream(2000, rate=200.0, seed=0)
    assert [(r.kind, r.n, r.seed) for r in reqs] == [(r.kind, r.n, r.seed) for r in again]


def test_inputs_are_deterministic_per_request():
    r1 = Request(0, "laplace", 5, 1234)
    r2 = Request(1, "laplace", 5, 1234)
    make_inputs(r1, pin=False)
    make_inputs(r2, pin=False)
    assert np.array_equal(r1.inputs["coords"].numpy(), r2.inputs["coords"].numpy())
    kap = r1.inputs["kappa"].numpy()
    assert kap.shape == (125,) and kap.min() >= 0.1 and kap.max() <= 10.0
    m = Request(2, "mr", 3, 77)
    make_inputs(m, pin=False)
    assert m.inputs["coords"].shape == (3, 7 ** 3)
    c = m.inputs["c"].numpy()
    assert c.shape == (2,) and c.min() >= 0.5 and c.max() <= 10.0
    assert 1.0 <= m.inputs["lam"] <= 1.1


def test_memory_estimates_grow_with_size():
    for kind in ("laplace", "mr"):
        prev = (0, 0)
        for n in (4, 8, 16, 32, 64):
            cur = estimate_bytes(kind, n)
            assert cur[0] > prev[0] and cur[1] > prev[1]
            prev = cur
    # the largest Mooney-Rivlin request fits a GB300 several times over
    res, work = estimate_bytes("mr", 64)
    assert 10e9 < res + work < 60e9


def test_summary_percentiles():
    reqs = [Request(i, "laplace", 4, i, arrival=0.01 * i) for i in range(100)]
    for i, r in enumerate(reqs):
        r.t_done = r.arrival + 0.001 * (i + 1)
    s = summarize(reqs)
    assert math.isclose(s["p50_ms"], np.percentile(np.arange(1, 101), 50), rel_tol=1e-9)
    assert math.isclose(s["p99_ms"], np.percentile(np.arange(1, 101), 99), rel_tol=1e-9)
    assert s["requests"] == 100


def test_ledger_charges_and_releases_exactly():
    from iron_gb300.serving import HbmLedger

    rng = np.random.default_rng(0)
    big = sum(estimate_bytes("mr", 40))
    L = HbmLedger(3 * big)
    running = []
    for step in range(3000):
        if running and (rng.random() < 0.5 or len(running) >= 6):
            rid, kind, n = running.pop(int(rng.integers(len(running))))
            L.finish(rid, kind, n)
        else:
            kind = "laplace" if rng.random() < 0.7 else "mr"
            n = int(rng.integers(4, 41))
            ok, evicted, dropped = L.admit(step, kind, n, int(rng.integers(8)))
            if ok:
                running.append((step, kind, n))
            assert all(L.users.get(k, 0) == 0 for k in evicted)
        L.check()
        assert L.in_use <= L.budget
    for rid, kind, n in running:
        L.finish(rid, kind, n)
    L.check()
    # nothing held: the largest request fits again after eviction, and nothing leaked
    ok, _, _ = L.admit(10 ** 6, "mr", 40, 0)
    assert ok
    assert L.evictions > 0


def test_ledger_refuses_what_cannot_fit_and_keeps_held_sizes():
    from iron_gb300.serving import BATCH_MAX_N, HbmLedger

    a, b = BATCH_MAX_N + 4, BATCH_MAX_N + 8  # sides with one request per slot
    L = HbmLedger(sum(estimate_bytes("laplace", b)))
    assert L.admit(1, "laplace", a, 0)[0]
    # a second size cannot evict the first while request 1 holds it
    assert not L.admit(2, "laplace", b, 1)[0]
    L.finish(1, "laplace", a)
    ok, evicted, dropped = L.admit(2, "laplace", b, 1)
    assert ok and evicted == [("laplace", a)] and dropped == [(0, "laplace", a)]
    L.check()
    # the same worker and size again costs nothing more
    before = L.in_use
    L.finish(2, "laplace", b)
    assert L.admit(3, "laplace", b, 1)[0] and L.in_use == before


def test_batched_slots_are_charged_for_their_capacity():
    from iron_gb300.serving import BATCH_MAX_N, LAPLACE_BATCH, HbmLedger, laplace_batch_capacity, slot_bytes

    assert laplace_batch_capacity(4) == laplace_batch_capacity(BATCH_MAX_N) == LAPLACE_BATCH
    assert laplace_batch_capacity(BATCH_MAX_N + 1) == 1
    n = 8
    res, work = estimate_bytes("laplace", n)
    assert slot_bytes("laplace", n) == LAPLACE_BATCH * work and slot_bytes("mr", n) == estimate_bytes("mr", n)[1]
    L = HbmLedger(10 * (res + LAPLACE_BATCH * work))
    # the first request of a batch charges the size and the whole slot, the others nothing
    for rid in range(LAPLACE_BATCH):
        assert L.admit(rid, "laplace", n, 0)[0]
        assert L.in_use == res + LAPLACE_BATCH * work
    for rid in range(LAPLACE_BATCH):
        L.finish(rid, "laplace", n)
    L.check()
    assert L.users[("laplace", n)] == 0


def test_mooney_rivlin_side_cap():
    full = request_stream(2000, rate=200.0, seed=0)
    capped = request_stream(2000, rate=200.0, seed=0, mr_n_hi=16)
    assert [(r.kind, r.seed, r.arrival) for r in full] == [(r.kind, r.seed, r.arrival) for r in capped]
    for a, b in zip(full, capped):
        if a.kind == "laplace":
            assert a.n == b.n
        else:
            assert 4 <= b.n <= 16 and b.n <= a.n
    assert max(r.n for r in capped if r.kind == "laplace") > 16
