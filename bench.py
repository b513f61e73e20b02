"""Benchmark of the SIMPLE outer iteration (cell-iterations/s) on GB300.

Default workload: the 3D lid-driven cavity, 128^3 hexes (2,097,152 cells) in a unit box,
lid u = 1, Re = 400, relaxation 0.7 / 0.3, fp32 fields and matrices with float-float
(fp64-class) Krylov reductions -- the single large case the roofline is measured on.
One step = one SIMPLE outer iteration (momentum BiCGSTAB + pressure CG, up to 500
iterations each, atol 1e-5).  Synthetic seeded mesh (built by the GPU mesh pass), zero
initial fields.  The same JSON line carries a ``serving`` block: the serving mix (1,024
steady cavity/channel requests, seeded Poisson arrivals) through the continuous-batching
server, with the drop-in path run one case at a time on a stratified sample of the same
mix for ``batched_over_drop_in`` (``--no-serving`` leaves it out).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload cavity3d|channel|cavity|cylinder|serve]
  python bench.py --impl reference ...   # the CPU restatement of the reference algorithm

Timing: W untimed steps, then K steps, each bracketed by CUDA events on the solver
stream; between steps a 256 MiB buffer is written to flush L2 (the flush is outside the
events).  A barrier and torch.cuda.synchronize() bracket the timed region; the time is
the max over ranks.  Under torchrun every rank runs its own case (replicas: the path
does not shard), so scaling is weak.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (description, builder args)
    "channel": "steady channel 400x80x1 hex on 10x1, u_in=1, p_out=0, Re=200, SIMPLE 0.3/0.3, fp32 (fp64 reductions)",
    "cavity": "lid-driven cavity 64x64x1 hex, lid u=1, Re=100, SIMPLE 0.7/0.3, fp32 (fp64 reductions)",
    "cavity3d": "3D lid-driven cavity 128^3 hex, lid u=1, Re=400, SIMPLE 0.7/0.3, fp32 (fp64 reductions)",
    "cylinder": "cylinder D=0.1 in a 2.2x0.41 channel, 247k prism/hex cells (hex O-grid, prism far field, "
                "interior nodes jittered up to 10%, seed 0), parabolic inlet U_max=1.5, Re=100, PISO dt=5e-4 with "
                "2 correctors and non-orthogonal correction, fp32 with fp64 iterative refinement of the pressure "
                "solve (3 sweeps, inner relative stop 1e-3); one step = one time step",
    "serve": "serving mix: steady cavity/channel requests, cells log-uniform in [32^2, 256^2], Re ~ U[50, 1000], "
             "speed ~ U[0.5, 2], seeded Poisson arrivals, converged: relative momentum residual below 1e-6 and "
             "no longer falling (no new minimum over 10 checks of 10 iterations); "
             "continuous batching (batched form; its pressure CG in the single-reduction arrangement) vs the "
             "drop-in path one case at a time (textbook CG)",
}
METRIC = "cell-iterations/s"

# DRAM bytes (read + written) of the dominant kernel measured with ncu
# (`dram__bytes_read.sum + dram__bytes_write.sum`, one capture per workload):
#   channel   cg_cluster_kernel: 1.47 MB per launch whatever the iteration count (the
#             system is read once into shared memory)
#   cavity3d  cg_kernel (int16 column offsets): 15.40 GB for a 174-iteration launch =
#             88.5 MB per iteration (the vectors stay in L2; the matrix streams)
MEASURED_TRAFFIC = {
    "channel": {"per_launch": 1.473e6, "per_iteration": 0.0},
    "cavity3d": {"per_launch": 0.0, "per_iteration": 15.403e9 / 174},
}


def build_mesh(workload):
    from warpcfd_gb300.preprocess import (Mesh, create_2D_grid, create_3D_grid, create_cylinder_channel_grid,
                                          define_boundary_walls, define_cylinder_group)

    import torch
    # the large meshes go through the GPU mesh pass (bit-identical topology to the host pass)
    dev = "cuda" if torch.cuda.is_available() else None
    if workload == "cylinder":
        g, info = create_cylinder_channel_grid(scale=1.15, jitter=0.1, seed=0, prisms=True)
        m = Mesh(g, device=dev)
        define_boundary_walls(m)
        define_cylinder_group(m, info["cylinder"])
        return m
    if workload == "channel":
        m = Mesh(create_2D_grid((0, 0, 0), 400, 80, 10.0, 1.0, 0.1))
    elif workload == "cavity":
        m = Mesh(create_2D_grid((0, 0, 0), 64, 64, 1.0, 1.0, 0.1))
    elif workload == "cavity3d":
        m = Mesh(create_3D_grid((0, 0, 0), 128, 128, 128, 1.0, 1.0, 1.0), device=dev)
    else:
        raise ValueError(workload)
    define_boundary_walls(m)
    return m


def solver_setup(workload):
    """(steady, u_relax, p_relax, dt, correctors, non-orthogonal correction) of a workload.

    The channel uses the relaxation of the reference's own channel example (0.3 / 0.3,
    examples/Channel Flow/Channel Flow.py:51): with the cavity's 0.7 / 0.3
    (examples/LDC/LDC.py:48) the reference method diverges on this channel within a few
    dozen iterations (no Rhie-Chow face flux, velocity inlet, pressure outlet)."""
    if workload == "cylinder":
        return False, None, None, 5e-4, 2, True
    if workload == "channel":
        return True, 0.3, 0.3, 1.0, 1, False
    return True, 0.7, 0.3, 1.0, 1, False


def inlet_profile(mesh, u_max=1.5, height=0.41):
    """Parabolic inlet u(y) = 4 u_max y (H - y) / H^2 on the '-X' faces, in group order."""
    ids = mesh.groups["-X"].ids
    y = mesh._geometry64["face_centroid"][ids, 1]
    return 4.0 * u_max * y * (height - y) / height ** 2


def case_setup(workload, mesh=None):
    """(nu, rho, reference cell, bc function) of a workload."""
    if workload == "cylinder":
        u_in = inlet_profile(mesh)

        def bc(b):
            b.velocity_BC("-X", u=u_in, v=0.0, w=0.0)
            b.pressure_BC("+X", p=0.0)
            b.no_slip_wall("-Y")
            b.no_slip_wall("+Y")
            b.no_slip_wall("cylinder")
            b.slip_wall("-Z")
            b.slip_wall("+Z")
        return 1e-3, 1.0, None, bc
    if workload == "channel":
        def bc(b):
            b.velocity_BC("-X", u=1.0, v=0.0, w=0.0)
            b.pressure_BC("+X", p=0.0)
            b.no_slip_wall("-Y")
            b.no_slip_wall("+Y")
            b.slip_wall("-Z")
            b.slip_wall("+Z")
        return 1.0 / 200.0, 1.0, None, bc
    if workload == "cavity":
        def bc(b):
            b.no_slip_wall("-X")
            b.no_slip_wall("+X")
            b.no_slip_wall("-Y")
            b.velocity_BC("+Y", u=1.0, v=0.0, w=0.0)
            b.slip_wall("+Z")
            b.slip_wall("-Z")
        return 0.01, 1.0, 0, bc
    if workload == "cavity3d":
        def bc(b):
            for w in ("-X", "+X", "-Y", "-Z", "+Z"):
                b.no_slip_wall(w)
            b.velocity_BC("+Y", u=1.0, v=0.0, w=0.0)
        return 1.0 / 400.0, 1.0, 0, bc
    raise ValueError(workload)


def build_gpu_case(workload, mesh, p_refine=None):
    from warpcfd_gb300.FV import FVM
    from warpcfd_gb300.FV.implicit_Solvers import IncompressibleSolver

    nu, rho, ref, bc = case_setup(workload, mesh)
    steady, ur, pr, dt, ncorr, corr = solver_setup(workload)
    model = FVM(mesh)
    model.material.create_incompressible_newtonian_fluid(viscosity=nu * rho, density=rho)
    if ref is not None:
        model.set_reference_pressure(ref, 0.0)
    bc(model.boundary)
    model.finalize()
    solver = IncompressibleSolver(model, ur, pr, correction=corr, steady_state=steady)
    solver.set_iterations(1, ncorr, 1)
    if not steady:
        solver.set_time_stepping(1, dt)
    if p_refine is None:
        # the precision form of the pressure solve for the cylinder (its configuration asks for it)
        p_refine = 3 if workload == "cylinder" else 0
    if p_refine > 0:
        solver.p_refine, solver.p_refine_rtol = int(p_refine), 1e-3
    solver.verbose = False
    return model, solver


def build_oracle_case(workload, mesh, T=np.float32, **solve):
    from oracle.simple_ref import OracleCase, geometry_from_mesh
    from warpcfd_gb300.FV.boundary import Boundary
    from warpcfd_gb300.FV.field import Field

    nu, rho, ref, bc = case_setup(workload, mesh)
    fields = {k: Field(k, i) for i, k in enumerate("uvwp")}
    b = Boundary(fields, mesh.groups, mesh.face_properties.boundary_face_ids)
    bc(b)
    b.check()
    corr = solver_setup(workload)[5]
    return OracleCase(geometry_from_mesh(mesh), b.boundary_type, b.boundary_values, nu * rho, rho, T=T,
                      reference_cell=ref, correction=corr, **solve)


def oracle_step(oc, workload, n=1):
    steady, ur, pr, dt, ncorr, _ = solver_setup(workload)
    if steady:
        oc.run(ur, pr, n_outer=n, n_inner=ncorr)
    else:
        oc.run(None, None, n_outer=1, n_inner=ncorr, steady=False, n_time=n, dt=dt)


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index, enabled=True):
        self.index = index
        self.enabled = enabled
        self.p = None

    def __enter__(self):
        if not self.enabled:
            return self
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "50"], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.p = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.p is not None:
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
                self.out = ""

    def summary(self):
        rows = []
        for ln in (self.out or "").strip().splitlines():
            f = [x.strip() for x in ln.split(",")]
            if len(f) >= 9:
                rows.append(f)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        reasons = set()
        for r in rows:
            for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"),
                               r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(rows[0][2]) if rows[0][2].replace(".", "").isdigit() else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def cpu_warmup_steps(mesh, requested=3):
    """Untimed oracle steps before a CPU timing: none on meshes of a million cells or more
    (one outer iteration of the 128^3 cavity is ~30 s of numpy; a CPU has no warm-up
    beyond the first step's allocations, which the timed sample then includes)."""
    return 0 if mesh.num_cells >= 1_000_000 else requested


def cpu_baseline(workload, mesh, seconds=15.0, warm=3):
    """The oracle (fp32, the same algorithm) on this host: ``warm`` untimed outer
    iterations from zero fields, then as many timed ones as fit in ~``seconds`` (at least
    one)."""
    warm = cpu_warmup_steps(mesh, warm)
    oc = build_oracle_case(workload, mesh)
    oracle_step(oc, workload, warm)
    t0 = time.perf_counter()
    n = 0
    while True:
        oracle_step(oc, workload, 1)
        n += 1
        if time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": mesh.num_cells * n / dt, "unit": METRIC, "cores": 1, "nproc": os.cpu_count(), "kind": "port",
            "sample": f"{n} SIMPLE outer iterations (after {warm} untimed) of the same {workload} case, numpy/scipy "
                      f"fp32 restatement (oracle/simple_ref.py), single thread ({os.cpu_count()} host cores)"}


def fp64_field_error(workload, mesh, steps=20):
    """Every field of a fresh GPU run (fp32, the drop-in path) against the fp64 oracle run
    of the same method, both ``steps`` outer iterations from zero fields: relative L2
    (u, v, w against ||U||, p against ||p||).  Part of the CPU leg: the oracle is the
    checker here, not the thing measured."""
    import torch

    note = None
    if workload == "cavity3d":
        # the numpy oracle does not run 2.1M cells within the bench's time: the same case
        # (lid u = 1, Re 400, SIMPLE 0.7 / 0.3) on a 32^3 mesh
        from warpcfd_gb300.preprocess import Mesh, create_3D_grid, define_boundary_walls

        n = 32
        mesh = Mesh(create_3D_grid((0, 0, 0), n, n, n, 1.0, 1.0, 1.0), device="cuda")
        define_boundary_walls(mesh)
        note = "the 128^3 case's configuration on a 32^3 mesh (32,768 cells): the numpy oracle does not run " \
               "2.1M cells within the bench's time"
    elif workload not in ("channel", "cavity"):
        return {"unavailable": f"the fp64 numpy oracle does not run {workload} within the bench's time"}
    # the Krylov solves as the drop-in runs them (the reference's stops), then tightened on
    # both sides -- momentum to atol 1e-9, pressure by 4 fp64 refinement sweeps of 1e-3 --
    # so that the second comparison measures the method and not where a loose stop ended
    tight = dict(atol=1e-9, maxiter=5000, p_refine=4, p_refine_rtol=1e-3)
    out = {"steps": steps, "oracle": "fp64 and fp32 numpy restatements of the same method"}
    t0 = time.perf_counter()
    for label, solve in (("reference_stops", {}), ("tightened", tight)):
        model, solver = build_gpu_case(workload, mesh)
        if solve:
            for eq in (solver.vel_equation, solver.p_corr_equation):
                eq.tol, eq.max_iter = solve["atol"], solve["maxiter"]
            solver.p_refine, solver.p_refine_rtol = solve["p_refine"], solve["p_refine_rtol"]
        for _ in range(steps):
            solver.step()
        torch.cuda.synchronize()
        g = model.cell_values.double().cpu().numpy()
        oc = build_oracle_case(workload, mesh, T=np.float64, **solve)
        oracle_step(oc, workload, steps)
        o = np.asarray(oc.cell_values, dtype=np.float64)
        o32 = build_oracle_case(workload, mesh, T=np.float32, **solve)
        oracle_step(o32, workload, steps)
        f32 = np.asarray(o32.cell_values, dtype=np.float64)
        un = max(float(np.linalg.norm(o[:, 0:3])), 1e-300)
        pn = max(float(np.linalg.norm(o[:, 3])), 1e-300)

        def rel(a):
            e = {f: float(np.linalg.norm(a[:, i] - o[:, i]) / un) for i, f in enumerate("uvw")}
            e["p"] = float(np.linalg.norm(a[:, 3] - o[:, 3]) / pn)
            return e
        # the fp32 oracle's own distance from the fp64 run is the method's rounding floor
        out[label] = {"rel_l2": rel(g), "fp32_oracle_rel_l2": rel(f32), "gpu_vs_fp32_oracle": {
            f: float(np.linalg.norm(g[:, i] - f32[:, i]) / max(float(np.linalg.norm(f32[:, i if f == "p" else slice(0, 3)])), 1e-300))
            for i, f in enumerate("uvwp")}}
        del model, solver
    out["oracle_seconds"] = round(time.perf_counter() - t0, 2)
    if note:
        out["case"] = note
    # the drop-in's own figures stay at the top level
    out.update({k: out["reference_stops"][k] for k in ("rel_l2", "fp32_oracle_rel_l2", "gpu_vs_fp32_oracle")})
    return out


def warp_probe():
    """Whether warp-lang (the reference's runtime, not vendored) can be imported here."""
    import importlib.util

    if importlib.util.find_spec("warp") is None:
        return {"warp_available": False, "why": "importlib.util.find_spec('warp') is None"}
    try:
        import warp
        return {"warp_available": True, "version": getattr(warp, "__version__", "?")}
    except Exception as e:  # noqa: BLE001 - any import failure is the answer
        return {"warp_available": False, "why": f"import warp failed: {e!r}"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    mesh = build_mesh(args.workload)
    oc = build_oracle_case(args.workload, mesh)
    warm = cpu_warmup_steps(mesh, args.warmup)
    oracle_step(oc, args.workload, warm)
    # each step is one full outer iteration of the workload; stop early (and say so) if
    # the K steps would not end within --ref-seconds
    t0 = time.perf_counter()
    done = 0
    while done < args.steps:
        oracle_step(oc, args.workload, 1)
        done += 1
        if time.perf_counter() - t0 > args.ref_seconds:
            break
    dt = time.perf_counter() - t0
    v = mesh.num_cells * done / dt
    probe = warp_probe()
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": args.gpus,
            "steps": done, "steps_requested": args.steps, "warmup": args.warmup, "warmup_run": warm,
            "ms_per_step": 1e3 * dt / done,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOADS[args.workload], "cells": mesh.num_cells},
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": 1, "nproc": os.cpu_count(), "kind": "port",
                             "sample": f"{done} SIMPLE outer iterations after {warm} untimed, numpy/"
                                       "scipy fp32 restatement of the reference algorithm, single thread "
                                       f"({os.cpu_count()} host cores); the reference itself needs warp-lang: "
                                       f"{probe}"},
            "reference_runtime": probe,
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def stratified_sample(reqs, n):
    """``n`` requests spread evenly over the mix sorted by (kind, cells): each kind keeps
    its share and each kind's sizes their spread (evenly spaced quantiles)."""
    order = sorted(reqs, key=lambda r: (r.kind, r.cells, r.rid))
    if n >= len(order):
        return order
    idx = np.unique(np.linspace(0, len(order) - 1, n).round().astype(np.int64))
    return [order[i] for i in idx]


def serve_mix(args, local, rank=0, world=1, dist=None):
    """The serving mix through the continuous-batching server (this rank's round-robin
    share), then the drop-in path one case at a time on a stratified sample of the same
    share with the same stop settings.  Returns the whole-job figures."""
    import torch

    from warpcfd_gb300.replicas import max_over_ranks, shard, sum_over_ranks
    from warpcfd_gb300.serve import Server, make_request_mix, run_drop_in

    reqs_all = make_request_mix(args.requests, seed=0, rate=args.rate)
    reqs = shard(reqs_all, rank, world)
    # warm-up: a few small requests touch every kernel and the caches
    Server(max_outer=30, cg_variant=args.serve_cg).run(make_request_mix(4, seed=1, rate=1e6, lo=32 * 32, hi=48 * 48))
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    with ClockSampler(local, enabled=not args.no_clocks) as clocks:
        rep = Server(max_outer=args.max_outer, max_active=args.max_active, use_graphs=args.serve_graphs,
                     admission=args.admission, cg_variant=args.serve_cg).run(reqs)
    summ = rep.summary()
    wall = max_over_ranks(summ["wall_s"])
    cell_its = sum_over_ranks(rep.cell_iterations)
    value = cell_its / wall
    sample = stratified_sample(reqs, min(args.drop_in_sample, len(reqs)))
    drop = run_drop_in(sample, max_outer=args.max_outer)
    drop_rate = sum_over_ranks(drop["cell_iterations_per_s"]) / world
    by_kind = {k: sum(r.kind == k for r in sample) for k in ("cavity", "channel")}
    mix_kind = {k: sum(r.kind == k for r in reqs) for k in ("cavity", "channel")}
    drop_status = {}
    for res in drop["results"]:
        r = res[2]
        st = "converged" if res[4] else ("diverged" if not np.isfinite(r) else "exhausted")
        drop_status[st] = drop_status.get(st, 0) + 1
    drop_status["retried"] = int(sum(res[3] > 0 for res in drop["results"]))
    return {
        "value": value, "wall": wall, "requests": len(reqs_all), "serving": summ, "clocks": clocks.summary(),
        "batched_pressure_cg": "single-reduction" if args.serve_cg == 1 else "textbook",
        "drop_in": {"requests_per_rank": len(sample), "sample": "stratified: evenly spaced over the mix sorted by "
                    "(kind, cells)", "sample_kinds": by_kind, "mix_kinds": mix_kind,
                    "sample_cells_median": float(np.median([r.cells for r in sample])),
                    "mix_cells_median": float(np.median([r.cells for r in reqs])),
                    "cell_iterations_per_s": drop_rate, "wall_s": drop["wall_s"], "status": drop_status},
        "batched_over_drop_in": value / world / max(drop_rate, 1e-9),
    }


def run_serve(args):
    """Serving mix through the continuous-batching server; the drop-in path (one case at a
    time, same settings) runs a stratified sample of the same mix for the comparison.
    Under torchrun each rank serves its round-robin share of the mix on its own GPU
    (replicas, no collective on the data path); rank 0 prints the whole-job figures."""
    import torch

    from warpcfd_gb300.build import build_library

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    build_library()
    out = serve_mix(args, local, rank, world, dist)
    if dist is not None:
        dist.destroy_process_group()
    if rank != 0:
        return 0
    line = {
        "metric": METRIC, "value": out["value"], "unit": METRIC, "n_gpus": world, "steps": out["requests"],
        "warmup": 4, "ms_per_step": 1e3 * out["wall"] / max(out["requests"], 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOADS["serve"], "requests": out["requests"], "arrival_rate_per_s": args.rate,
                   "max_outer": args.max_outer, "step": "one request served to completion",
                   "parallelism": f"request shards x{world}"},
        "serving": out["serving"], "drop_in": out["drop_in"], "batched_over_drop_in": out["batched_over_drop_in"],
        "clocks": out["clocks"],
    }
    print(json.dumps(line))
    return 0


def run_ours(args):
    import torch

    from warpcfd_gb300 import perfmodel
    from warpcfd_gb300.build import build_library

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    build_library()
    mesh = build_mesh(args.workload)
    model, solver = build_gpu_case(args.workload, mesh, args.p_refine)
    C = mesh.num_cells
    g = model._geo_host
    K, B, F, W = g["n_faces"], g["n_bfaces"], g["faces_per_cell"], g["ell_width"]
    Ki = K - B
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    for _ in range(args.warmup):
        solver.step()
    torch.cuda.synchronize()
    snap = solver.snapshot()  # the end-to-end pass below replays the same K steps from here

    K_ = args.steps
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * K_)]
    kev = [torch.cuda.Event(enable_timing=True) for _ in range(4 * K_)]
    for e in kev:
        e.record(stream)          # materialise the CUDA events before handing them to the C side
    stats_hist = torch.zeros((K_, solver.stats.numel()), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local, enabled=not args.no_clocks) as clocks:
        for i in range(K_):
            flush.zero_()
            solver.set_timing_events(kev[4 * i: 4 * i + 4])
            ev[2 * i].record(stream)
            solver.step()
            ev[2 * i + 1].record(stream)
            stats_hist[i].copy_(solver.stats)
        torch.cuda.synchronize()
    solver.set_timing_events(None)
    if dist is not None:
        dist.barrier()
    step_ms = np.array([ev[2 * i].elapsed_time(ev[2 * i + 1]) for i in range(K_)])
    bicg_ms = np.array([kev[4 * i].elapsed_time(kev[4 * i + 1]) for i in range(K_)])
    cg_ms = np.array([kev[4 * i + 2].elapsed_time(kev[4 * i + 3]) for i in range(K_)])
    from warpcfd_gb300.FV.implicit_Solvers.incompressible import STATS_DTYPE
    hist = np.frombuffer(stats_hist.cpu().numpy().tobytes(), dtype=STATS_DTYPE).reshape(K_, 2)
    k_u = hist[:, 0]["iterations"].astype(np.int64)
    k_p = hist[:, 1]["iterations"].astype(np.int64)
    finite = bool(torch.isfinite(model.cell_values).all().item())
    if not finite:
        raise SystemExit("bench: the fields went non-finite during the timed steps; no valid measurement")
    rel_res = hist[:, 0]["initial_residual"] / np.maximum(hist[:, 0]["rhs_norm"], 1e-300)
    from warpcfd_gb300.replicas import job_throughput, max_over_ranks
    total_ms = max_over_ranks(float(step_ms.sum()))
    value = job_throughput(C * K_, world, total_ms * 1e-3)

    # end to end through the public API with host buffers (H2D inputs, D2H result per step):
    # the same K steps again from the post-warm-up snapshot (the path is bitwise
    # reproducible, so the Krylov counts match the timed steps one for one)
    solver.restore(snap)
    host_in = torch.empty((C, 4), dtype=torch.float32).pin_memory()
    host_out = torch.empty((C, 4), dtype=torch.float32).pin_memory()
    host_in.copy_(model.cell_values.cpu())
    e2e_stats = torch.zeros_like(stats_hist)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(K_):
        model.cell_values.copy_(host_in, non_blocking=True)
        solver.step()
        e2e_stats[i].copy_(solver.stats)
        host_out.copy_(model.cell_values, non_blocking=True)
        torch.cuda.synchronize()
        host_in, host_out = host_out, host_in
    e2e_s = time.perf_counter() - t0
    same = bool(torch.equal(e2e_stats, stats_hist))
    e2e = {"value": world * C * K_ / e2e_s, "unit": METRIC, "h2d_bytes_per_step": C * 16,
           "d2h_bytes_per_step": C * 16, "same_steps_as_timed": same}

    # roofline of the dominant kernel (algorithmic bytes / event time)
    from warpcfd_gb300 import _lib
    rows = int(_lib.load().wcfd_batch_max_rows(W))  # rows per CTA of the cluster-resident CG
    grid_cg = C > 16 * rows
    # the grid CG streams int16 column offsets when the mesh has them (wcfd_mesh.ell_dcol)
    col_bytes = 2 if grid_cg and g.get("ell_dcol") is not None else 4
    cg_bytes = sum(perfmodel.cg_bytes(C, W, int(k), col_bytes) for k in k_p)
    bi_bytes = sum(perfmodel.bicgstab_bytes(C, W, int(k)) for k in k_u)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    if cg_ms.sum() >= bicg_ms.sum():
        kname = "cg_kernel" if grid_cg else "cg_cluster_kernel"
        kbytes, kms, nl = cg_bytes, cg_ms.sum(), K_
    else:
        kname, kbytes, kms, nl = "bicgstab_kernel", bi_bytes, bicg_ms.sum(), K_
    achieved = kbytes / (kms * 1e-3) / 1e9
    traffic = None
    mt = MEASURED_TRAFFIC.get(args.workload)
    if mt is not None and kname.startswith("cg"):
        traffic = mt["per_launch"] + mt["per_iteration"] * float(k_p.mean())
    step_bytes = [perfmodel.simple_step_bytes(C, K, Ki, B, F, W, int(a), int(b), col_bytes=col_bytes)["total"]
                  for a, b in zip(k_u, k_p)]
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": K_, "warmup": args.warmup,
        "ms_per_step": total_ms / K_, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload], "cells": C, "faces": K, "l2": "flushed between steps "
                   "(256 MiB write outside the step events)", "parallelism": f"replicas x{world}",
                   "krylov_iters_mean": {"bicgstab": float(k_u.mean()), "cg": float(k_p.mean())},
                   "relaxation": [solver.u_relaxation_factor, solver.p_relaxation_factor],
                   "p_refine_sweeps": int(solver.p_refine),
                   "fields_finite": finite,
                   "momentum_rel_residual": {"first": float(rel_res[0]), "last": float(rel_res[-1])}},
        "e2e": e2e,
        "gpu_launches": (6 + 7 * solver.NUM_INNER_LOOPS) * K_,
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peaks
                     else "fallback", "traffic": traffic,
                     "traffic_note": "ncu DRAM bytes per launch of this kernel on this workload (one capture, "
                                     "scaled by the mean iteration count)" if traffic is not None else None,
                     "bytes_per_launch": kbytes / nl, "ms_per_launch": kms / nl,
                     "step_bytes_per_s_GBs": float(np.sum(step_bytes) / (total_ms * 1e-3) / 1e9)},
        "kernel_ms": {"bicgstab": float(bicg_ms.mean()), "cg": float(cg_ms.mean()), "step": float(step_ms.mean())},
    }
    if traffic is not None:
        # the same launch judged by the DRAM bytes ncu measured for it instead of the
        # algorithmic bytes (below 1 x algorithmic: the vectors hit L2)
        line["roofline"]["achieved_dram"] = traffic / (kms / nl * 1e-3) / 1e9
        line["roofline"]["frac_dram"] = line["roofline"]["achieved_dram"] / peak
    if rank == 0:
        line["clocks"] = clocks.summary()
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(args.workload, mesh, seconds=args.cpu_seconds)
            line["fp64_oracle"] = fp64_field_error(args.workload, mesh)
    if world == 1 and args.workload == "cavity3d" and not args.no_serving:
        # the serving half of the metric (p50/p99 time to a converged solution, batched
        # over drop-in), on the same GPU after the 128^3 case is released
        del model, solver, snap, flush
        torch.cuda.empty_cache()
        line["serving"] = serve_mix(args, local)
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cavity3d", choices=sorted(WORKLOADS))
    ap.add_argument("--p-refine", type=int, default=None,
                    help="fp64 refinement sweeps of the pressure solve (default: 3 for cylinder, else 0)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-seconds", type=float, default=90.0)
    ap.add_argument("--no-serving", action="store_true", help="leave the serving block out of the default line")
    ap.add_argument("--no-clocks", action="store_true", help="do not sample nvidia-smi during the timed region")
    ap.add_argument("--requests", type=int, default=1024, help="serve workload: requests in the mix")
    ap.add_argument("--max-active", type=int, default=256, help="serve workload: cases in flight at most")
    ap.add_argument("--rate", type=float, default=2000.0, help="serve workload: Poisson arrival rate (1/s)")
    ap.add_argument("--max-outer", type=int, default=4000, help="serve workload: outer-iteration cap per request")
    ap.add_argument("--drop-in-sample", type=int, default=48, help="serve workload: requests run through the drop-in")
    ap.add_argument("--admission", default="fifo", choices=["fifo", "largest"],
                    help="serve workload: admission order of arrived requests")
    ap.add_argument("--serve-cg", type=int, default=1, help="serving: the batched pressure CG, 0 textbook, "
                    "1 single-reduction (one cluster all-reduce per iteration; the server's default)")
    ap.add_argument("--serve-graphs", type=int, default=1, help="serve workload: replay each bucket round as a "
                    "captured CUDA graph (1) or launch it eagerly (0)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "serve":
        return run_serve(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
