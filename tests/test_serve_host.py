"""Host-side logic of the serving loop (no GPU): request mix, mesh-size ladder, result
status, admission estimate, rejection of requests no state of the server can admit."""
import math

import numpy as np

from warpcfd_gb300.serve import (CHANNEL_ASPECT, RELAXATION, MeshCache, Request, Result, Server, ServeReport,
                                 StopRule, estimate_bytes, estimate_geometry_bytes, make_request_mix, side_ladder)


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
    srv = _host_server((4096, 16384, 65536), 1 << 30)
    ok = Request(0, "cavity", 4096, 100.0, 1.0, 0.0)
    assert srv._never_admissible(ok) == ""
    assert "largest bucket" in srv._never_admissible(Request(1, "cavity", 70_000, 100.0, 1.0, 0.0))
    assert "unknown kind" in srv._never_admissible(Request(2, "pipe", 1024, 100.0, 1.0, 0.0))
    assert "positive" in srv._never_admissible(Request(3, "channel", 1024, 0.0, 1.0, 0.0))
    assert "positive" in srv._never_admissible(Request(4, "channel", 1024, 100.0, math.nan, 0.0))
    assert "no cells" in srv._never_admissible(Request(5, "cavity", 0, 100.0, 1.0, 0.0))
    srv._geometry_charged.add(srv._mesh_key(ok))      # its mesh is on the device already
    srv.budget = estimate_bytes(4096) - 1
    assert "budget" in srv._never_admissible(ok)
    # geometry already on the device is never released, so it counts against the budget
    srv.budget, srv._geometry_bytes = estimate_bytes(4096) + 10, 11
    assert "budget" in srv._never_admissible(ok)
    srv._geometry_bytes = 10
    assert srv._never_admissible(ok) == ""


def _host_server(bounds, budget):
    """A Server with only the state its admission checks read (no device state)."""
    srv = Server.__new__(Server)
    srv.bounds = bounds
    srv.budget = budget
    srv.meshes = MeshCache()
    srv._geometry_charged = set()
    srv._geometry_bytes = 0
    return srv


def test_new_mesh_geometry_counts_against_the_budget():
    """A request whose mesh is not on the device yet must fit together with that mesh's
    geometry: the case alone would fit, the case plus its new geometry does not."""
    req = Request(0, "channel", 16384, 200.0, 1.0, 0.0)
    nx, ny = MeshCache().shape("channel", 16384)
    geo = estimate_geometry_bytes(nx * ny)
    assert geo > 0.3 * estimate_bytes(16384)
    srv = _host_server((4096, 16384, 65536), estimate_bytes(16384) + geo - 1)
    assert srv._new_geometry_bytes(req) == geo
    assert not srv._fits(req, 0)
    assert "budget" in srv._never_admissible(req)
    # one more byte and it fits, with nothing else admitted
    srv.budget += 1
    assert srv._fits(req, 0) and srv._never_admissible(req) == ""
    assert not srv._fits(req, 1)
    # once that mesh's geometry is charged (on the device), only its measured bytes count
    srv._geometry_charged.add(srv._mesh_key(req))
    srv._geometry_bytes = geo // 2
    assert srv._new_geometry_bytes(req) == 0
    assert srv._fits(req, geo // 2)
    # a request of another size has its own mesh and pays for its geometry again
    other = Request(1, "channel", 8000, 200.0, 1.0, 0.0)
    assert srv._new_geometry_bytes(other) > 0


def test_geometry_estimate_bounds_the_built_geometry():
    """estimate_geometry_bytes stays above the host-built geometry arrays the device
    copies, on cavity and channel meshes of the mix."""
    from warpcfd_gb300.FV.geometry import build_geometry

    mc = MeshCache()
    for kind, cells in (("cavity", 1024), ("channel", 6000), ("cavity", 20000)):
        m = mc.get(kind, cells)
        nb = sum(v.nbytes for v in build_geometry(m).values() if isinstance(v, np.ndarray))
        C = m.cell_properties.faces.shape[0]
        assert nb <= estimate_geometry_bytes(C) < 1.3 * nb


def test_rejected_results_are_counted_and_kept_out_of_latency():
    rep = ServeReport()
    rep.results = [Result(0, "cavity", 100, 50, True, 1e-7, 0.0, 0.0, 2.0),
                   Result(1, "cavity", 70_000, 0, False, math.nan, 0.0, 0.0, 0.0, None, "too many cells")]
    assert rep.results[1].status == "rejected"
    summary = rep.summary()
    assert summary["requests"] == 2 and summary["rejected"] == 1 and summary["converged"] == 1
    assert summary["p50_s"] == summary["p99_s"] == 2.0


def test_stop_rule_waits_for_the_residual_floor():
    """Converged = below tol and no new residual minimum for `patience` checks."""
    rule = StopRule(1e-6, patience=3)
    st = [float("inf"), 0]
    seq = [1e-3, 1e-5, 9e-7, 5e-7, 3e-7, 2e-7, 2.1e-7, 1.9999e-7, 2.05e-7]
    out = [rule.update(st, r) for r in seq]
    # falling below tol is not enough; three checks without a new minimum (0.1% better) are
    assert out == [False] * 8 + [True]
    assert StopRule(1e-6, patience=0).update([float("inf"), 0], 5e-7)
    assert not StopRule(1e-6, patience=0).update([float("inf"), 0], 2e-6)
    # a restart (new state) starts counting afresh
    st2 = [float("inf"), 0]
    assert not rule.update(st2, 2e-7)


def test_boundary_template_times_speed_equals_the_api_table():
    """build_solver forms a kind's boundary table once per mesh at unit speed and scales it:
    the same table, bit for bit, as the boundary helpers called at the request's speed."""
    from warpcfd_gb300.FV.boundary.boundary import Boundary
    from warpcfd_gb300.FV.field import Field

    fields = {k: Field(k, i) for i, k in enumerate("uvwp")}
    mc = MeshCache()

    def table(m, kind, speed):
        b = Boundary(fields, m.groups, m.face_properties.boundary_face_ids)
        if kind == "cavity":
            b.no_slip_wall("-X"), b.no_slip_wall("+X"), b.no_slip_wall("-Y")
            b.velocity_BC("+Y", u=speed, v=0.0, w=0.0)
        else:
            b.velocity_BC("-X", u=speed, v=0.0, w=0.0), b.pressure_BC("+X", p=0.0)
            b.no_slip_wall("-Y"), b.no_slip_wall("+Y")
        b.slip_wall("-Z"), b.slip_wall("+Z")
        return b.boundary_type, b.boundary_values

    for kind, speed in (("cavity", 1.37), ("channel", 0.61), ("cavity", 2.0)):
        m = mc.get(kind, 3000)
        t1, v1 = table(m, kind, 1.0)
        ts, vs = table(m, kind, speed)
        assert np.array_equal(t1, ts)
        assert np.array_equal((v1 * speed).view(np.int64), vs.view(np.int64))


def test_server_and_drop_in_share_the_stop_and_solver_policy():
    """The drop-in baseline runs the server's own stop rule, Krylov stops and refinement
    sweeps (only the batched pressure CG's arrangement differs), so the two are compared
    at the same convergence criterion."""
    import inspect

    from warpcfd_gb300 import serve

    srv = inspect.signature(Server.__init__).parameters
    drop = inspect.signature(serve.run_drop_in).parameters
    for name in ("tol", "check_every", "max_outer", "atol", "rtol", "max_retries", "retry_relax", "p_refine",
                 "patience"):
        assert srv[name].default == drop[name].default, name
    assert srv["patience"].default == serve.SERVE_PATIENCE == 10
    assert srv["cg_variant"].default == serve.SERVE_CG_VARIANT == 1
    assert inspect.signature(StopRule.__init__).parameters["patience"].default == serve.SERVE_PATIENCE
