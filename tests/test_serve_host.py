"""Host-side logic of the serving loop (no GPU): request mix, mesh-size ladder, result
status, admission estimate, rejection of requests no state of the server can admit."""
import math

import numpy as np

from warpcfd_gb300.serve import (CHANNEL_ASPECT, RELAXATION, MeshCache, Request, Result, Server, ServeReport,
                                 estimate_bytes, make_request_mix, side_ladder)


def test_request_mix_is_seeded_and_within_bounds():
    a = make_request_mix(200, seed=3, rate=100.0)
    b = make_request_mix(200, seed=3, rate=100.0)
    assert [(r.kind, r.cells, r.re, r.speed, r.arrival) for r in a] == \
           [(r.kind, r.cells, r.re, r.speed, r.arrival) for r in b]
    cells = np.array([r.cells for r in a])
    assert cells.min() >= 32 * 32 - 1 and cells.max() <= 256 * 256
    assert all(50.0 <= r.re <= 1000.0 and 0.5 <= r.speed <= 2.0 for r in a)
    arr = np.array([r.arrival for r in a])
    assert np.all(np.diff(arr) > 0)
    # Poisson arrivals at 100/s: mean gap about 10 ms
    assert 0.005 < np.diff(arr).mean() < 0.02
    kinds = {r.kind for r in a}
    assert kinds == {"cavity", "channel"}


def test_mesh_ladder_quantises_sizes():
    lad = side_ladder()
    assert lad[0] == 32 and lad[-1] == 256 and lad == sorted(set(lad))
    ratios = np.array(lad[1:]) / np.array(lad[:-1])
    assert ratios.max() < 1.12
    mc = MeshCache()
    nx, ny = mc.shape("cavity", 5000)
    assert nx == ny and abs(math.log(nx * ny / 5000)) < 0.12
    nx, ny = mc.shape("channel", 20000)
    assert nx == CHANNEL_ASPECT * ny and abs(math.log(nx * ny / 20000)) < 0.12


def test_result_status_and_relaxation_table():
    r = Result(1, "cavity", 100, 50, True, 1e-7, 0.0, 0.0, 1.0)
    assert r.status == "converged" and r.latency == 1.0
    assert Result(1, "cavity", 100, 50, False, float("nan"), 0.0, 0.0, 1.0).status == "diverged"
    assert Result(1, "cavity", 100, 4000, False, 1e-4, 0.0, 0.0, 1.0).status == "exhausted"
    # the relaxation of the reference's own examples per kind
    assert RELAXATION["cavity"] == (0.7, 0.3) and RELAXATION["channel"] == (0.3, 0.3)


def test_admission_estimate_grows_with_size():
    a, b = estimate_bytes(1024), estimate_bytes(65536)
    assert 0 < a < b and b > 1000 * 65536


def test_never_admissible_names_the_reason():
    """The check that keeps the admission loop from waiting for ever on a request that no
    state of the server can hold.  Only the bounds, budget and charged geometry bytes are
    read, so the server's device state (streams) is not built here."""
    srv = Server.__new__(Server)
    srv.bounds = (4096, 16384, 65536)
    srv.budget = 1 << 30
    srv._geometry_bytes = 0
    ok = Request(0, "cavity", 4096, 100.0, 1.0, 0.0)
    assert srv._never_admissible(ok) == ""
    assert "largest bucket" in srv._never_admissible(Request(1, "cavity", 70_000, 100.0, 1.0, 0.0))
    assert "unknown kind" in srv._never_admissible(Request(2, "pipe", 1024, 100.0, 1.0, 0.0))
    assert "positive" in srv._never_admissible(Request(3, "channel", 1024, 0.0, 1.0, 0.0))
    assert "positive" in srv._never_admissible(Request(4, "channel", 1024, 100.0, math.nan, 0.0))
    assert "no cells" in srv._never_admissible(Request(5, "cavity", 0, 100.0, 1.0, 0.0))
    srv.budget = estimate_bytes(4096) - 1
    assert "budget" in srv._never_admissible(ok)
    # geometry already on the device is never released, so it counts against the budget
    srv.budget, srv._geometry_bytes = estimate_bytes(4096) + 10, 11
    assert "budget" in srv._never_admissible(ok)
    srv._geometry_bytes = 10
    assert srv._never_admissible(ok) == ""


def test_rejected_results_are_counted_and_kept_out_of_latency():
    rep = ServeReport()
    rep.results = [Result(0, "cavity", 100, 50, True, 1e-7, 0.0, 0.0, 2.0),
                   Result(1, "cavity", 70_000, 0, False, math.nan, 0.0, 0.0, 0.0, None, "too many cells")]
    assert rep.results[1].status == "rejected"
    summary = rep.summary()
    assert summary["requests"] == 2 and summary["rejected"] == 1 and summary["converged"] == 1
    assert summary["p50_s"] == summary["p99_s"] == 2.0
