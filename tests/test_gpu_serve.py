"""Serving loop: continuous batching over a small seeded request mix.

Every request completes; each result (iterations and fields) is the same when the request
is served alone as when it is served in the mix (bitwise: each case's kernels and cluster
reductions do not depend on the other cases of its bucket, and the bucket's cluster size
is fixed by its bound).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib_ready():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from warpcfd_gb300.build import build_library
    build_library()


def test_served_alone_equals_in_mix():
    from warpcfd_gb300.serve import Server, make_request_mix

    reqs = make_request_mix(10, seed=7, rate=400.0, lo=32 * 32, hi=64 * 64)
    kw = dict(tol=1e-4, check_every=10, max_outer=300, buckets=(1024, 4096), keep_fields=True, atol=1e-7)
    mix = Server(**kw).run(reqs)
    assert len(mix.results) == len(reqs)
    s = mix.summary()
    assert s["max_active"] > 1 and s["p99_s"] >= s["p50_s"] > 0
    by_id = {r.rid: r for r in mix.results}
    for req in reqs[:4]:
        alone = Server(**kw).run([req]).results[0]
        got = by_id[req.rid]
        assert alone.iterations == got.iterations
        assert torch.equal(alone.fields.view(torch.int32), got.fields.view(torch.int32))  # bitwise, NaN too


def test_server_rejects_what_it_can_never_serve():
    """Requests no state of the server can admit -- too many cells for the largest bucket,
    an unknown kind, Re = 0, more bytes than the whole HBM budget -- come back as
    'rejected' while the rest are served; before, an over-budget head of the queue held
    the admission loop for ever."""
    from warpcfd_gb300.serve import Request, Server

    reqs = [Request(0, "cavity", 32 * 32, 100.0, 1.0, 0.0), Request(1, "cavity", 70_000, 100.0, 1.0, 0.0),
            Request(2, "bogus", 1024, 100.0, 1.0, 0.0), Request(3, "channel", 2048, 0.0, 1.0, 0.0),
            Request(4, "cavity", 40 * 40, 200.0, 1.0, 0.0)]
    rep = Server(max_outer=20, autotune=False).run(reqs)
    st = {r.rid: r.status for r in rep.results}
    assert len(st) == 5
    assert st[1] == st[2] == st[3] == "rejected"
    assert st[0] != "rejected" and st[4] != "rejected"
    summary = rep.summary()
    assert summary["rejected"] == 3 and summary["requests"] == 5
    small = Server(hbm_budget=1 << 20, max_outer=20, autotune=False).run([Request(0, "cavity", 32 * 32, 100.0, 1.0, 0.0)])
    assert [r.status for r in small.results] == ["rejected"]
    assert "budget" in small.results[0].rejected


def test_admission_order_does_not_change_results():
    """Longest-first admission (admission='largest') changes when a request runs, not what it
    computes: every result equals the first-come-first-served run's, bit for bit, and the
    diverged-request policy (a restart at half relaxation) is counted in the summary."""
    from warpcfd_gb300.serve import Server, make_request_mix

    reqs = make_request_mix(10, seed=11, rate=5000.0, lo=32 * 32, hi=64 * 64)
    kw = dict(tol=1e-4, check_every=10, max_outer=200, buckets=(1024, 4096), keep_fields=True, atol=1e-7,
              max_active=4)
    fifo = {r.rid: r for r in Server(**kw).run(reqs).results}
    rep = Server(admission="largest", **kw).run(reqs)
    largest = {r.rid: r for r in rep.results}
    assert set(fifo) == set(largest) == {r.rid for r in reqs}
    for rid, a in fifo.items():
        b = largest[rid]
        assert (a.iterations, a.status, a.retries) == (b.iterations, b.status, b.retries)
        assert torch.equal(a.fields.view(torch.int32), b.fields.view(torch.int32))
    s = rep.summary()
    assert "retried" in s and "converged_after_retry" in s
