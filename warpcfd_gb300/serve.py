"""Continuous-batching server for steady incompressible cases.

Requests arrive over time (seeded Poisson arrivals).  Each is a lid-driven cavity or a
channel of its own size, Reynolds number and lid/inlet speed.  The server

* admits a waiting request when its arrival time has passed, a batch slot is free and the
  HBM budget (the measured device bytes of the admitted cases) has room for its estimate;
* keeps every admitted case's fields, geometry and systems resident on the device;
* advances all admitted cases together with the batched form (``CaseBatch``): one launch
  sequence per outer iteration per size bucket, buckets on separate streams so their work
  overlaps on the device;
* every ``check_every`` iterations reads all cases' residuals with one copy per bucket,
  retires the converged ones (relative momentum residual below ``tol``) and admits new
  requests into the freed slots;
* records time-to-converged-solution (completion - arrival) per request and the
  cell-iterations done.

Mesh sizes are quantised to a log-spaced ladder of side lengths (about 8% apart) so
preprocessed meshes are cached and reused across requests.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from .batch import CaseBatch
from .FV import FVM
from .FV.implicit_Solvers import IncompressibleSolver
from .preprocess import Mesh, create_2D_grid, define_boundary_walls

CHANNEL_ASPECT = 4  # channel cases: (4 n) x n cells on a 4 x 1 domain


@dataclass
class Request:
    rid: int
    kind: str          # "cavity" or "channel"
    cells: int         # requested cell count
    re: float
    speed: float
    arrival: float     # seconds after the start of the run


@dataclass
class Result:
    rid: int
    kind: str
    cells: int
    iterations: int
    converged: bool
    residual: float
    arrival: float
    admitted: float
    finished: float
    fields: object = None
    rejected: str = ""   # why the request was never admitted ("" when it was)
    retries: int = 0     # restarts at reduced relaxation after a divergence

    @property
    def latency(self):
        return self.finished - self.arrival

    @property
    def status(self):
        """converged, diverged (non-finite residual), exhausted (max_outer reached) or
        rejected (never admitted: too large for the batched solver or the HBM budget, or
        a case that cannot be built)."""
        if self.rejected:
            return "rejected"
        if self.converged:
            return "converged"
        return "exhausted" if math.isfinite(self.residual) else "diverged"


def side_ladder(lo=32, hi=256, steps=28):
    """Log-spaced cavity side lengths (cells) from lo to hi."""
    return sorted({int(round(lo * (hi / lo) ** (i / (steps - 1)))) for i in range(steps)})


def make_request_mix(n_requests=1024, seed=0, rate=200.0, lo=32 * 32, hi=256 * 256):
    """Seeded mix: cells log-uniform in [lo, hi], Re ~ U[50, 1000], speed ~ U[0.5, 2],
    cavity or channel with a fair coin, Poisson arrivals at ``rate`` per second."""
    rng = np.random.default_rng(seed)
    cells = np.exp(rng.uniform(np.log(lo), np.log(hi), n_requests)).astype(np.int64)
    re = rng.uniform(50.0, 1000.0, n_requests)
    speed = rng.uniform(0.5, 2.0, n_requests)
    kind = np.where(rng.random(n_requests) < 0.5, "cavity", "channel")
    arrival = np.cumsum(rng.exponential(1.0 / rate, n_requests))
    return [Request(i, str(kind[i]), int(cells[i]), float(re[i]), float(speed[i]), float(arrival[i]))
            for i in range(n_requests)]


class MeshCache:
    """Meshes of the size ladder, built on first use and kept.  With a CUDA ``device`` a
    mesh is preprocessed by the GPU mesh pass (topology and fp64 geometry bit-identical to
    the host pass; a 65,536-cell mesh in milliseconds instead of ~0.5 s of host time, which
    would otherwise stall the serving loop that launches every bucket's rounds)."""

    def __init__(self, device=None):
        self.ladder = side_ladder()
        self.meshes = {}
        self.device = device

    def shape(self, kind, cells):
        if kind == "cavity":
            n = min(self.ladder, key=lambda s: abs(math.log(s * s / cells)))
            return (n, n)
        ny = min(self.ladder, key=lambda s: abs(math.log(CHANNEL_ASPECT * s * s / cells)))
        return (CHANNEL_ASPECT * ny, ny)

    def get(self, kind, cells):
        nx, ny = self.shape(kind, cells)
        key = (kind, nx, ny)
        if key not in self.meshes:
            lx = 1.0 if kind == "cavity" else float(CHANNEL_ASPECT)
            m = Mesh(create_2D_grid((0, 0, 0), nx, ny, lx, 1.0, 0.1), device=self.device)
            define_boundary_walls(m)
            self.meshes[key] = m
        return self.meshes[key]


RELAXATION = {
    # (u, p): the relaxation of the reference's own examples for each kind
    # (examples/LDC/LDC.py:48 and examples/Channel Flow/Channel Flow.py:51); the reference
    # method diverges on channels at the cavity's 0.7 / 0.3
    "cavity": (0.7, 0.3),
    "channel": (0.3, 0.3),
}


# Krylov stops of the served cases: each solve ends when its residual has dropped tenfold
# (or below 1e-12), so solve accuracy follows the outer residual down to the 1e-6 target;
# a fixed atol either stalls the outer iteration at its own level (1e-8: ~2e-6) or costs
# 3-4x the Krylov iterations (1e-10) for the same outer convergence.
SERVE_ATOL = 1e-12
SERVE_RTOL = (0.1, 0.1)
# one fp64 refinement sweep of the pressure solve per outer iteration (its correction to the
# same tenfold drop): the pressure of a converged case is accumulated in fp64
SERVE_P_REFINE = 1
# stop rule of a served case: no new residual minimum over this many checks of 10 outer
# iterations (see StopRule).  Where an fp32 iteration stops along its noise floor sets how
# close the served fields come to the fp64 fixed point: with 10 checks every field of the
# accuracy test's requests is within 1e-5 of it (single-reduction CG), with 5 the channel's
# p stops 8e-5 to 1.2e-4 away.
SERVE_PATIENCE = 10
# the batched pressure CG of the server: 1 = single-reduction (wcfd_batch_dims.cg_variant),
# one cluster all-reduce per iteration instead of two (+11% on the serving mix)
SERVE_CG_VARIANT = 1


def build_solver(req: Request, mesh, atol=1e-8, maxiter=500, device=None, rtol=(0.0, 0.0), relax_scale=1.0,
                 p_refine=0):
    """FVM + SIMPLE solver of one request (relaxation by kind times ``relax_scale``,
    nu = speed * L / Re).  ``rtol`` = (momentum, pressure) relative Krylov stops on top of
    ``atol``.  ``p_refine`` > 0: the pressure solve by that many fp64 refinement sweeps per
    outer iteration, each correction solved to the pressure rtol (the precision form: p is
    accumulated in fp64, so the converged pressure is not held at the fp32 CG's floor)."""
    nu = req.speed * 1.0 / req.re
    model = FVM(mesh, device=device)
    model.material.create_incompressible_newtonian_fluid(viscosity=nu, density=1.0)
    if req.kind == "cavity":
        model.set_reference_pressure(0, 0.0)
    # The boundary table of a kind depends on its mesh alone, its values on the lid/inlet
    # speed alone (every other value is 0): formed once per (mesh, kind) through the
    # boundary API at unit speed, then scaled -- the same table the API gives at this
    # speed, bit for bit, without the helpers' per-call work on every admission.
    cache = mesh.__dict__.setdefault("_serve_bc_templates", {})
    if req.kind not in cache:
        b = model.boundary
        if req.kind == "cavity":
            b.no_slip_wall("-X")
            b.no_slip_wall("+X")
            b.no_slip_wall("-Y")
            b.velocity_BC("+Y", u=1.0, v=0.0, w=0.0)
        else:
            b.velocity_BC("-X", u=1.0, v=0.0, w=0.0)
            b.pressure_BC("+X", p=0.0)
            b.no_slip_wall("-Y")
            b.no_slip_wall("+Y")
        b.slip_wall("-Z")
        b.slip_wall("+Z")
        cache[req.kind] = (b.boundary_type.copy(), b.boundary_values.copy())
    btype, bunit = cache[req.kind]
    model.boundary.boundary_type[...] = btype
    model.boundary.boundary_values[...] = bunit * float(req.speed)
    model.finalize()
    ur, pr = RELAXATION[req.kind]
    solver = IncompressibleSolver(model, ur * relax_scale, pr * relax_scale)
    solver.verbose = False
    solver.vel_equation.tol = atol
    solver.p_corr_equation.tol = atol
    solver.vel_equation.rtol, solver.p_corr_equation.rtol = rtol
    solver.vel_equation.max_iter = maxiter
    solver.p_corr_equation.max_iter = maxiter
    if p_refine > 0:
        solver.p_refine = int(p_refine)
        solver.p_refine_rtol = float(rtol[1]) if rtol[1] > 0 else 1e-3
    solver.case_struct()   # allocates the refinement arrays now, so case_bytes counts them
    return model, solver


def geometry_bytes(model) -> int:
    """Device bytes of a model's geometry (shared by every model of the same mesh)."""
    return int(sum(v.numel() * v.element_size() for v in model._geo.values() if isinstance(v, torch.Tensor)))


def case_bytes(model, solver, include_geometry=True) -> int:
    """Device bytes held by one admitted case (fields, systems, workspaces and, unless
    include_geometry is False, the mesh geometry it shares with other cases of its mesh)."""
    ts = [model.cell_values, model.cell_gradients, model.face_values, model.face_gradients, model.mass_fluxes,
          model.boundary_type, model.boundary_value, solver.rUA, solver.rUA_faces, solver.div_u,
          solver.vel_correction, solver.stats]
    if include_geometry:
        ts += [v for v in model._geo.values() if isinstance(v, torch.Tensor)]
    ts += [t for t in (solver.p_x64, solver.p_work) if t is not None]
    for e in (solver.vel_equation, solver.p_corr_equation):
        ts += [e.diag, e.off, e.rhs, e.x, e.ws_vec, e.ws_partials, e.ws_results, e.ws_barrier, e.stats]
    return int(sum(t.numel() * t.element_size() for t in ts))


def estimate_bytes(cells: int) -> int:
    """Admission estimate before building: about 1.1 kB per cell for a 2D-extruded hex case
    (16 B of it the fp64 pressure and refinement work arrays) plus fixed workspaces
    (measured with case_bytes on the mix's meshes)."""
    return int(1120 * cells + 2 * 8 * 2048 * 8 + 64 * 1024)


def estimate_geometry_bytes(cells: int) -> int:
    """Admission estimate of a mesh's device geometry before it is built: a 2D-extruded hex
    mesh has about four faces per cell (68 B of face records each), six 16-byte cell slots,
    four 4-byte off-diagonal columns and their four 2-byte offsets per cell, about 400 B per
    cell; 420 B per cell plus 64 KiB stays above geometry_bytes() on the mix's meshes."""
    return int(420 * cells + 64 * 1024)


class StopRule:
    """When a steady case counts as converged: its relative momentum residual (the initial
    residual of the outer iteration's momentum solve over ||b||) is below ``tol`` AND has
    stopped falling -- no new minimum (by more than 0.1%) over the last ``patience`` checks.
    The residual of an fp32 solve floors at ~1e-7 (~6e-8 on channels); a case stopped at
    1e-6 alone is still 3e-5 to 2e-4 from the fp64 fixed point, one run to its floor is
    within ~1e-6 on the velocities and ~1e-5 on p.  patience = 0 stops at ``tol``."""

    def __init__(self, tol=1e-6, patience=SERVE_PATIENCE):
        self.tol = float(tol)
        self.patience = int(patience)

    def update(self, state, r) -> bool:
        """``state`` is the case's [best residual, checks since it]; True when converged."""
        if r < state[0] * (1.0 - 1e-3):
            state[0], state[1] = r, 0
        else:
            state[1] += 1
        return bool(r < self.tol) and (self.patience == 0 or state[1] >= self.patience)


@dataclass
class _Slot:
    req: Request
    model: object
    solver: object
    bytes: int
    admitted: float
    iterations: int = 0
    retries: int = 0
    stop_state: list = field(default_factory=lambda: [float("inf"), 0])


@dataclass
class ServeReport:
    results: list = field(default_factory=list)
    wall: float = 0.0
    cell_iterations: int = 0
    max_active: int = 0
    peak_bytes: int = 0
    bucket_busy_s: list = field(default_factory=list)
    admit_s: float = 0.0

    def summary(self):
        served = [r for r in self.results if not r.rejected]
        lat = np.array([r.latency for r in served]) if served else np.zeros(1)
        conv = [r for r in self.results if r.converged]
        lat_c = np.array([r.latency for r in conv]) if conv else np.full(1, np.nan)
        return {
            "requests": len(self.results),
            "converged": len(conv),
            "diverged": int(sum(r.status == "diverged" for r in self.results)),
            "exhausted": int(sum(r.status == "exhausted" for r in self.results)),
            "rejected": int(sum(r.status == "rejected" for r in self.results)),
            "retried": int(sum(r.retries > 0 for r in self.results)),
            "converged_after_retry": int(sum(r.retries > 0 and r.converged for r in self.results)),
            "p50_converged_s": float(np.percentile(lat_c, 50)),
            "p99_converged_s": float(np.percentile(lat_c, 99)),
            "p50_s": float(np.percentile(lat, 50)),
            "p99_s": float(np.percentile(lat, 99)),
            "cell_iterations_per_s": self.cell_iterations / max(self.wall, 1e-9),
            "wall_s": self.wall,
            "max_active": self.max_active,
            "peak_case_bytes": self.peak_bytes,
            "bucket_gpu_busy_s": [round(x, 3) for x in self.bucket_busy_s],
            "host_admission_s": round(self.admit_s, 3),
        }


class Server:
    """Continuous batching over size buckets (bucket = cell count up to its bound)."""

    def __init__(self, hbm_budget=16 << 30, max_active=256, tol=1e-6, check_every=10, max_outer=4000,
                 patience=SERVE_PATIENCE,
                 buckets=(4096, 8192, 16384, 32768, 65536), atol=SERVE_ATOL, rtol=SERVE_RTOL, device=None,
                 clock=time.perf_counter, keep_fields=False, autotune=True, use_graphs=True, max_retries=1,
                 retry_relax=0.5, p_refine=SERVE_P_REFINE, admission="fifo", admit_slice_s=0.002,
                 cg_variant=SERVE_CG_VARIANT):
        self.budget = int(hbm_budget)
        # the batched pressure CG: 0 textbook, 1 single-reduction (wcfd_batch_dims.cg_variant)
        self.cg_variant = int(cg_variant)
        self.max_active = int(max_active)
        self.tol = float(tol)
        self.stop = StopRule(tol, patience)
        self.check_every = int(check_every)
        self.max_outer = int(max_outer)
        self.bounds = tuple(sorted(buckets))
        self.atol = atol
        self.rtol = tuple(rtol)
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        self.clock = clock
        self.meshes = MeshCache(device=self.device)
        self.autotune = autotune
        self.use_graphs = use_graphs
        # divergence policy: a case whose residual turns non-finite starts again from zero
        # fields with its relaxation factors scaled by retry_relax (per retry), at most
        # max_retries times; the iterations before the restart stay counted
        self.max_retries = int(max_retries)
        self.retry_relax = float(retry_relax)
        self.p_refine = int(p_refine)
        # order in which arrived requests are admitted: "fifo" (arrival order) or "largest"
        # (most cells first, arrival order among equals)
        if admission not in ("fifo", "largest"):
            raise ValueError("admission must be 'fifo' or 'largest'")
        self.admission = admission
        # admission yields to the bucket loop after this much host time, so a burst of
        # arrivals does not hold back the next rounds of the buckets already running
        self.admit_slice_s = float(admit_slice_s)
        self._geometry_charged = set()
        self._geometry_bytes = 0
        self.keep_fields = keep_fields
        self.streams = [torch.cuda.Stream(device=self.device) for _ in self.bounds]
        # cases are built (allocations, fills, uploads) on a side stream of their own, so
        # admission does not queue behind or beside the default stream; a bucket's stream
        # waits for it before its next round
        self.admit_stream = torch.cuda.Stream(device=self.device)
        # one cluster size per bucket, from its bound, so a case's arithmetic never depends
        # on which other cases share its batch: the fewest CTAs whose shared memory holds
        # the bucket's largest case (2D-extruded hex meshes: off-diagonal width 4), which
        # puts the most cases in flight at once
        from . import _lib
        rows = int(_lib.load().wcfd_batch_max_rows(4))
        if rows <= 0:
            raise RuntimeError("the cluster-resident solver does not fit this device")
        self.cluster_sizes = []
        for b in self.bounds:
            cs = 1
            while cs * rows < b:
                cs *= 2
            if cs > 16:
                raise ValueError(f"bucket bound {b} exceeds what 16 CTAs hold ({16 * rows} cells)")
            self.cluster_sizes.append(cs)

    def _bucket(self, cells):
        for i, b in enumerate(self.bounds):
            if cells <= b:
                return i
        return len(self.bounds) - 1

    def _never_admissible(self, req) -> str:
        """Why ``req`` can never be admitted, or "": an unknown kind, a non-positive or
        non-finite Re or speed, more cells than the largest bucket's cluster solver holds,
        or more device bytes than the whole budget."""
        if req.kind not in RELAXATION:
            return f"unknown kind {req.kind!r}"
        if not (math.isfinite(req.re) and req.re > 0 and math.isfinite(req.speed) and req.speed > 0):
            return "Re and speed must be positive and finite"
        if req.cells < 1:
            return "no cells"
        if req.cells > self.bounds[-1]:
            return f"{req.cells} cells exceed the largest bucket ({self.bounds[-1]})"
        # geometry on the device is never released: the case must fit beside all of it,
        # and beside its own mesh's geometry when that is not on the device yet
        need = estimate_bytes(req.cells) + self._new_geometry_bytes(req)
        if need + self._geometry_bytes > self.budget:
            return f"needs about {need} device bytes, more than the budget ({self.budget}) leaves"
        return ""

    def _mesh_key(self, req):
        return (req.kind,) + self.meshes.shape(req.kind, req.cells)

    def _new_geometry_bytes(self, req) -> int:
        """Estimated device bytes of ``req``'s mesh geometry if it is not on the device yet,
        else 0 (it is then already charged)."""
        key = self._mesh_key(req)
        if key in self._geometry_charged:
            return 0
        return estimate_geometry_bytes(key[1] * key[2])

    def _fits(self, req, used) -> bool:
        """Whether ``req`` fits the budget now, beside the admitted cases' ``used`` bytes,
        the geometry on the device and its own mesh's geometry if that is new."""
        return (used + self._geometry_bytes + self._new_geometry_bytes(req) + estimate_bytes(req.cells)
                <= self.budget)

    def _admit(self, req, t0):
        """Build the case (the mesh and its device geometry come from caches) and charge its
        device bytes; a mesh's geometry is charged once, when it first reaches the device."""
        mesh = self.meshes.get(req.kind, req.cells)
        model, solver = build_solver(req, mesh, atol=self.atol, device=self.device, rtol=self.rtol,
                                     p_refine=self.p_refine)
        nb = case_bytes(model, solver, include_geometry=False)
        key = self._mesh_key(req)
        if key not in self._geometry_charged:
            self._geometry_charged.add(key)
            self._geometry_bytes += geometry_bytes(model)
        return _Slot(req, model, solver, nb, self.clock() - t0)

    def _restart(self, slot, t0):
        """A fresh case for ``slot``'s request (zero fields) at its relaxation times
        retry_relax ** (retries + 1); admission time and iterations carry over."""
        mesh = self.meshes.get(slot.req.kind, slot.req.cells)
        retries = slot.retries + 1
        model, solver = build_solver(slot.req, mesh, atol=self.atol, device=self.device, rtol=self.rtol,
                                     relax_scale=self.retry_relax ** retries, p_refine=self.p_refine)
        nb = case_bytes(model, solver, include_geometry=False)
        return _Slot(slot.req, model, solver, nb, slot.admitted, slot.iterations, retries)

    def run(self, requests) -> ServeReport:
        """Serve ``requests`` (arrival times relative to the start of the call).

        Each size bucket runs its own rounds of ``check_every`` batched iterations on its own
        stream, so a bucket of small cases is never held back by a bucket of large ones.  A
        round ends with an asynchronous copy of the bucket's solver outcomes to pinned host
        memory; the host polls the round's event, retires converged, diverged and exhausted
        cases, adds the requests admitted meanwhile and starts the bucket's next round.
        Admission (mesh lookup, case build and upload) runs on the host while rounds are in
        flight."""
        from . import _lib

        pending = sorted(requests, key=lambda r: r.arrival)
        nb = len(self.bounds)
        active = [[] for _ in range(nb)]     # cases of the bucket's current batch
        incoming = [[] for _ in range(nb)]   # admitted, joining at the bucket's next round
        batches = [None] * nb
        inflight = [None] * nb               # (start event, end event, pinned stats) of the round in flight
        busy = [0.0] * nb
        used = 0
        report = ServeReport()
        cur = torch.cuda.current_stream(self.device)
        t0 = self.clock()
        qi = 0
        waiting = []                         # arrived, not yet admitted, in admission order
        while qi < len(pending) or waiting or any(active) or any(incoming):
            # admission: arrived requests while slots and memory allow
            now = self.clock() - t0
            arrived = False
            while qi < len(pending) and pending[qi].arrival <= now:
                waiting.append(pending[qi])
                qi += 1
                arrived = True
            if arrived and self.admission == "largest":
                # longest first: the large cases start early and small ones fill the tail
                waiting.sort(key=lambda r: (-r.cells, r.arrival))
            t_slice = self.clock()
            while waiting:
                if self.clock() - t_slice > self.admit_slice_s and (any(active) or any(incoming)):
                    break
                req = waiting[0]
                # a request that no state of the server can admit is rejected, not queued
                # (it would hold the head of the queue for ever)
                why = self._never_admissible(req)
                if why:
                    report.results.append(Result(req.rid, req.kind, req.cells, 0, False, float("nan"), req.arrival,
                                                 now, now, None, why))
                    waiting.pop(0)
                    continue
                n_live = sum(len(a) for a in active) + sum(len(a) for a in incoming)
                if n_live >= self.max_active or not self._fits(req, used):
                    break
                ta = self.clock()
                try:
                    with torch.cuda.stream(self.admit_stream):
                        slot = self._admit(req, t0)
                except (ValueError, KeyError, AssertionError, NotImplementedError, _lib.WcfdError) as e:
                    report.admit_s += self.clock() - ta
                    report.results.append(Result(req.rid, req.kind, req.cells, 0, False, float("nan"), req.arrival,
                                                 now, self.clock() - t0, None, f"cannot build the case: {e}"))
                    waiting.pop(0)
                    continue
                report.admit_s += self.clock() - ta
                if used + slot.bytes + self._geometry_bytes > self.budget:
                    # the measured bytes (or the mesh's measured geometry) exceed the
                    # estimates: release the case; with nothing else admitted it can never
                    # fit, otherwise it waits for cases to retire
                    del slot
                    if n_live == 0:
                        report.results.append(Result(req.rid, req.kind, req.cells, 0, False, float("nan"),
                                                     req.arrival, now, self.clock() - t0, None,
                                                     "measured device bytes exceed the budget"))
                        waiting.pop(0)
                        continue
                    break
                used += slot.bytes
                report.peak_bytes = max(report.peak_bytes, used + self._geometry_bytes)
                incoming[self._bucket(slot.model.num_cells)].append(slot)
                waiting.pop(0)
            report.max_active = max(report.max_active, sum(len(a) for a in active) + sum(len(a) for a in incoming))
            progressed = False
            for bi in range(nb):
                if inflight[bi] is not None:
                    e0, e1, host = inflight[bi]
                    if not e1.query():
                        continue
                    inflight[bi] = None
                    busy[bi] += e0.elapsed_time(e1) * 1e-3
                    st = np.frombuffer(host.numpy().tobytes(), dtype=_lib.STATS_DTYPE).reshape(-1, 2)
                    res = st[:, 0]["initial_residual"] / np.maximum(st[:, 0]["rhs_norm"], 1e-300)
                    keep = []
                    for s, r in zip(active[bi], res):
                        s.iterations += self.check_every
                        report.cell_iterations += s.model.num_cells * self.check_every
                        done = self.stop.update(s.stop_state, r)
                        if (not math.isfinite(r) and s.retries < self.max_retries
                                and s.iterations < self.max_outer):
                            # diverged: restart from zero fields at reduced relaxation
                            with torch.cuda.stream(self.admit_stream):
                                s2 = self._restart(s, t0)
                            used += s2.bytes - s.bytes
                            incoming[bi].append(s2)
                            continue
                        if done or not math.isfinite(r) or s.iterations >= self.max_outer:
                            report.results.append(Result(s.req.rid, s.req.kind, s.model.num_cells, s.iterations,
                                                         done, float(r), s.req.arrival, s.admitted,
                                                         self.clock() - t0,
                                                         s.model.cell_values.clone() if self.keep_fields else None,
                                                         retries=s.retries))
                            used -= s.bytes
                        else:
                            keep.append(s)
                    if len(keep) != len(active[bi]):
                        active[bi] = keep
                        batches[bi] = None
                    progressed = True
                if incoming[bi]:
                    active[bi].extend(incoming[bi])
                    incoming[bi] = []
                    batches[bi] = None
                if not active[bi]:
                    continue
                stream = self.streams[bi]
                fresh = batches[bi] is None
                if fresh:
                    # the case table is uploaded on the current stream
                    batches[bi] = CaseBatch([s.solver for s in active[bi]], cluster_size=self.cluster_sizes[bi],
                                            cg_variant=self.cg_variant)
                # the bucket's stream runs after the uploads of admitted cases and the table
                stream.wait_stream(cur)
                stream.wait_stream(self.admit_stream)
                if fresh and self.autotune:
                    from .autotune import tune_field_block
                    with torch.cuda.stream(stream):
                        tune_field_block(batches[bi], key=("serve", self.bounds[bi], self.cluster_sizes[bi]))
                host = torch.empty(batches[bi].stats.numel(), dtype=torch.uint8, pin_memory=True)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                with torch.cuda.stream(stream):
                    e0.record(stream)
                    if self.use_graphs:
                        batches[bi].steps(self.check_every)
                    else:
                        for _ in range(self.check_every):
                            batches[bi].step()
                    host.copy_(batches[bi].stats, non_blocking=True)
                    e1.record(stream)
                inflight[bi] = (e0, e1, host)
                progressed = True
            if not progressed:
                if not any(active) and not any(incoming) and not waiting and qi < len(pending):
                    time.sleep(max(0.0, min(pending[qi].arrival - (self.clock() - t0), 0.01)))
                else:
                    time.sleep(20e-6)
        torch.cuda.synchronize(self.device)
        report.wall = self.clock() - t0
        report.bucket_busy_s = busy
        return report


def run_drop_in(requests, tol=1e-6, check_every=10, max_outer=4000, atol=SERVE_ATOL, rtol=SERVE_RTOL, device=None,
                max_retries=1, retry_relax=0.5, p_refine=SERVE_P_REFINE, patience=SERVE_PATIENCE):
    """The same requests through the plain drop-in path, one case at a time in arrival
    order, with the server's stop and divergence policy (a diverged case restarts from
    zero fields at reduced relaxation, at most ``max_retries`` times): the baseline the
    batched server is compared with."""
    meshes = MeshCache(device=device if device is not None else torch.device("cuda", torch.cuda.current_device()))
    stop = StopRule(tol, patience)
    cell_iters = 0
    t0 = time.perf_counter()
    results = []
    for req in sorted(requests, key=lambda r: r.arrival):
        mesh = meshes.get(req.kind, req.cells)
        model, solver = build_solver(req, mesh, atol=atol, device=device, rtol=rtol, p_refine=p_refine)
        total = 0
        retries = 0
        r = float("inf")
        state = [float("inf"), 0]
        while total < max_outer:
            for _ in range(check_every):
                solver.step()
            total += check_every
            cell_iters += model.num_cells * check_every
            st = solver.solve_stats()[0]
            r = st["initial_residual"] / max(st["rhs_norm"], 1e-300)
            if not math.isfinite(r):
                if retries < max_retries and total < max_outer:
                    retries += 1
                    model, solver = build_solver(req, mesh, atol=atol, device=device, rtol=rtol,
                                                 relax_scale=retry_relax ** retries, p_refine=p_refine)
                    state = [float("inf"), 0]
                    continue
                break
            if stop.update(state, r):
                break
        converged = bool(math.isfinite(r) and r < tol and (patience == 0 or state[1] >= patience))
        results.append((req.rid, total, r, retries, converged))
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    return {"cell_iterations_per_s": cell_iters / wall, "wall_s": wall, "results": results}
