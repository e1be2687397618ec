"""The serving loop on the GPU: every request's result is the same alone, in the mix and in a
batch (bit-identical: the kernels are deterministic and requests share no mutable state), matches
the plain FP64 path (Laplace solutions within 1e-8 of the unit boundary data, both solves stopping
at a relative residual of 1e-10; Mooney-Rivlin load steps both converged to Iron's tolerances,
geometry within 1e-7 and pressure within 1e-5 relative), a budget that holds one request at a time
still serves the stream, and a request that runs out of device memory is retried after the engine
drains.
"""
import numpy as np
import pytest

from iron_gb300.serving import (Request, ServingEngine, estimate_bytes, make_inputs, plain_fp64, request_stream,
                                slot_bytes)

pytestmark = pytest.mark.gpu


def _stream(n, seed, n_hi=7):
    reqs = request_stream(n, rate=1000.0, laplace_fraction=0.6, n_lo=3, n_hi=n_hi, seed=seed)
    for r in reqs:
        make_inputs(r)
    return reqs


@pytest.mark.parametrize("use_graphs", [True, False])
def test_results_same_alone_and_in_the_mix(gfe_cuda, use_graphs):
    reqs = _stream(12, 5)
    eng = ServingEngine(gfe_cuda, workers=4, use_graphs=use_graphs)
    stats = eng.serve(reqs, realtime=False)
    assert stats["requests"] == 12 and eng.stats["max_concurrent"] >= 2
    mixed = {r.rid: r.result.copy() for r in reqs}
    for r in reqs:
        r.result = None
        eng.serve([r], realtime=False)
        assert np.array_equal(r.result, mixed[r.rid]), (r.rid, r.kind, r.n)
    # a fresh engine with one worker (no overlap at all) gives the same results too
    eng1 = ServingEngine(gfe_cuda, workers=1, use_graphs=use_graphs)
    eng1.serve(reqs, realtime=False)
    for r in reqs:
        assert np.array_equal(r.result, mixed[r.rid]), (r.rid, r.kind, r.n)


def test_graphs_and_eager_agree_and_match_plain_fp64(gfe_cuda):
    reqs = _stream(8, 11)
    ServingEngine(gfe_cuda, workers=3, use_graphs=True).serve(reqs, realtime=False)
    g = {r.rid: r.result.copy() for r in reqs}
    ServingEngine(gfe_cuda, workers=3, use_graphs=False).serve(reqs, realtime=False)
    for r in reqs:
        assert np.array_equal(r.result, g[r.rid])
    mr_eng = {r.rid: r.info for r in reqs if r.kind == "mr"}
    assert all(i["reason"] in ("absolute residual", "relative residual", "relative step") for i in mr_eng.values())
    plain_fp64(reqs, realtime=False)
    for r in reqs:
        if r.kind == "laplace":
            assert np.abs(r.result - g[r.rid]).max() <= 1e-8, r.rid
        else:
            # the same load step solved to Iron's tolerances with FP32 contraction and Krylov
            # iterations in the engine and FP64 in the plain path
            assert r.info["newton_iterations"] >= 1 and r.info["reason"] != ""
            assert r.info["residual_norm"] <= max(1e-10, 1e-5 * r.info["initial_residual_norm"])
            nx = 3 * (2 * r.n + 1) ** 3
            assert np.abs(r.result[:nx] - g[r.rid][:nx]).max() <= 1e-7, r.rid
            p_ref = np.abs(r.result[nx:]).max()
            assert np.abs(r.result[nx:] - g[r.rid][nx:]).max() <= 1e-5 * p_ref, r.rid


def test_small_laplace_requests_are_batched(gfe_cuda):
    """Eleven queued Laplace requests of side 4 and three of side 5 on two workers run in batches
    (widths 1, 2, 4 and 8 with padding entries); each result equals the request's result alone."""
    reqs = [Request(i, "laplace", 4 if i < 11 else 5, 1000 + i) for i in range(14)]
    for r in reqs:
        make_inputs(r)
    eng = ServingEngine(gfe_cuda, workers=2)
    eng.serve(reqs, realtime=False)
    assert eng.stats["batches"] >= 2 and eng.stats["batched_requests"] >= 8
    assert max(r.info["batch"] for r in reqs) > 4
    together = {r.rid: r.result.copy() for r in reqs}
    for r in reqs:
        r.result = None
        eng.serve([r], realtime=False)
        assert r.info["batch"] == 1
        assert np.array_equal(r.result, together[r.rid]), r.rid
    # a batch of three (width 4: one padding entry) and the eager path give the same results too
    trio = reqs[:3]
    for use_graphs in (True, False):
        e = ServingEngine(gfe_cuda, workers=1, use_graphs=use_graphs)
        e.serve(trio, realtime=False)
        assert [r.info["batch"] for r in trio] == [3, 3, 3]
        for r in trio:
            assert np.array_equal(r.result, together[r.rid]), (use_graphs, r.rid)
        e.close()
    eng.close()


def test_tight_budget_serialises_and_evicts(gfe_cuda):
    reqs = _stream(10, 3, n_hi=6)
    biggest = max(estimate_bytes(r.kind, r.n)[0] + slot_bytes(r.kind, r.n) for r in reqs)
    eng = ServingEngine(gfe_cuda, workers=4, hbm_budget=int(1.05 * biggest))
    eng.serve(reqs, realtime=False)
    assert all(r.result is not None for r in reqs)
    assert eng.stats["evictions"] > 0
    assert eng.in_use <= eng.budget


def test_larger_meshes_many_workers(gfe_cuda):
    """Sixteen requests with sides up to 24 on eight workers (graphs on): every result equals the
    one-worker run of the same request."""
    reqs = _stream(16, 21, n_hi=24)
    eng = ServingEngine(gfe_cuda, workers=8)
    eng.serve(reqs, realtime=False)
    mixed = {r.rid: r.result.copy() for r in reqs}
    eng.close()
    eng1 = ServingEngine(gfe_cuda, workers=1)
    eng1.serve(reqs, realtime=False)
    for r in reqs:
        assert np.array_equal(r.result, mixed[r.rid]), (r.rid, r.kind, r.n)
    eng1.close()


@pytest.mark.parametrize("error", ["torch", "library"])
def test_out_of_memory_request_is_retried_after_drain(gfe_cuda, monkeypatch, error):
    """A request whose first attempt runs out of device memory (raised here on the host by a fake
    of the failing allocation, before any of its work is queued) goes back to the head of the
    queue; the engine drains, releases the allocator's cache, and the retry gives the request's
    usual result."""
    import torch

    from iron_gb300 import serving as S
    from iron_gb300._lib import GfeError

    reqs = _stream(8, 21)
    eng = ServingEngine(gfe_cuda, workers=3)
    eng.serve(reqs, realtime=False)
    ref = {r.rid: r.result.copy() for r in reqs}
    victims = {reqs[2].rid, reqs[5].rid}
    failed = set()
    real_prepare = S.ServingEngine._prepare

    def flaky_prepare(self, req, worker):
        if req.rid in victims and req.rid not in failed:
            failed.add(req.rid)
            if error == "torch":
                raise torch.cuda.OutOfMemoryError("fake out of memory")
            raise GfeError(-7, "fake device scratch allocation failure")
        return real_prepare(self, req, worker)

    monkeypatch.setattr(S.ServingEngine, "_prepare", flaky_prepare)
    for r in reqs:
        r.result = None
    eng.serve(reqs, realtime=False)
    assert failed == victims and eng.stats["oom_retries"] == 2
    for r in reqs:
        assert np.array_equal(r.result, ref[r.rid]), (r.rid, r.kind, r.n)


def test_repeated_out_of_memory_is_an_error(gfe_cuda, monkeypatch):
    from iron_gb300 import serving as S
    from iron_gb300._lib import GfeError

    reqs = _stream(4, 22)
    eng = ServingEngine(gfe_cuda, workers=2)
    real_prepare = S.ServingEngine._prepare

    def always_oom(self, req, worker):
        if req.rid == reqs[1].rid:
            raise GfeError(-7, "fake device scratch allocation failure")
        return real_prepare(self, req, worker)

    monkeypatch.setattr(S.ServingEngine, "_prepare", always_oom)
    with pytest.raises(GfeError, match="1 request"):
        eng.serve(reqs, realtime=False)
    assert eng.stats["oom_retries"] == S.OOM_RETRIES
