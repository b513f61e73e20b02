"""Generates the golden fixtures of tests/golden/ from the oracle (oracle/simple_ref.py).

  python tests/golden/make_golden.py [name ...]

ldc64_fp64_converged.npz : 64x64x1 cavity, Re 100, SIMPLE 0.7/0.3, fp64 fields and
                           reductions, Krylov atol 1e-10, 1500 outer iterations
                           (steady state reached; changes < 1e-9 per 100 iterations).
ldc64_fp32_converged.npz : the same converged run in fp32 fields (fp64 reductions),
                           atol 1e-7: with the fp64 run it measures the fp32 floor.
ldc64_fp32_500.npz       : the same case at the reference's own settings (fp32,
                           atol 1e-5, maxiter 500, 500 outer iterations) -- the numbers
                           the reference's configuration produces with this algorithm.
ldc64_fp64_500.npz       : the same at fp64 with the reference's fp64 atol (1e-6).

Fixed-iteration parity runs (the drop-in's parity bar: 500 iterations of the 64x64
cavity, 100 of the 400x80 channel at Re 200 and 0.3 / 0.3, from zero fields), with the
Krylov solves tightened so that the two sides compare the method, not where a loose
stop happened to end a solve: momentum BiCGSTAB atol 1e-9 and the pressure solve by
fp64 iterative refinement (4 sweeps, each a CG correction to a 1e-3 relative drop),
maxiter 5000 (never reached):
ldc64_fp32_500_refined.npz, channel400_fp32_100_refined.npz : fp32 fields (the method
                           as the drop-in computes it);
ldc64_fp64_500_refined.npz, channel400_fp64_100_refined.npz : fp64 fields, momentum atol
                           1e-12, the same refinement in fp64 (the fp64 oracle of the
                           same method).
The channel fixtures store cell_values as float32 to keep the files small (the rounding,
6e-8 relative, is far below the distances they are compared at).
Each file stores cell_values (C,4) and the per-iteration Krylov counts.

serve_fp64_converged.npz : three requests of the serving mix's mesh ladder (a 32 x 32 cavity
                           at Re 100 and speed 1, a 51 x 51 cavity at Re 400 and speed 1.5, a
                           128 x 32 channel on 4 x 1 at Re 100 and speed 1), each run by the
                           fp64 oracle at the server's relaxation (0.7 / 0.3 cavity, 0.3 / 0.3
                           channel), momentum atol 1e-13 and the pressure solved by 4 fp64
                           refinement sweeps per iteration (an absolute stop alone leaves the
                           pinned pressure system's solution moving at ~1e-6), until no field
                           moves by more than 1e-10 of its scale over an iteration (five orders
                           below the 1e-5 the served results are held to): the fixed point a
                           served result is compared with.  r{i}_fp32 holds the fp32 oracle's run
                           of the same request (momentum atol 1e-9, the same pressure refinement)
                           for as many iterations as the fp64 run took plus half: the fp32 floor
                           of the method against that fixed point.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.simple_ref import OracleCase, geometry_from_mesh  # noqa: E402
from tests.cases import cavity_bc, cavity_mesh, channel_bc, channel_mesh, host_boundary  # noqa: E402

TIGHT = dict(maxiter=5000, p_refine=4, p_refine_rtol=1e-3)
SPECS = {
    "ldc64_fp64_converged": dict(T=np.float64, atol=1e-10, iters=1500),
    "ldc64_fp32_converged": dict(T=np.float32, atol=1e-7, iters=1500),
    "ldc64_fp32_500": dict(T=np.float32, atol=1e-5, iters=500),
    "ldc64_fp64_500": dict(T=np.float64, atol=1e-6, iters=500),
    "ldc64_fp32_500_refined": dict(T=np.float32, atol=1e-9, iters=500, **TIGHT),
    "ldc64_fp64_500_refined": dict(T=np.float64, atol=1e-12, iters=500, **TIGHT),
    "channel400_fp32_100_refined": dict(case="channel", T=np.float32, atol=1e-9, iters=100, store=np.float32,
                                        **TIGHT),
    "channel400_fp64_100_refined": dict(case="channel", T=np.float64, atol=1e-12, iters=100, store=np.float32,
                                        **TIGHT),
}


def case_for(spec):
    """(mesh, boundary, nu, reference cell, (u_relax, p_relax)) of a fixture's case."""
    if spec.get("case", "cavity") == "cavity":
        m = cavity_mesh(64)
        return m, host_boundary(m, cavity_bc), 0.01, 0, (0.7, 0.3)
    m = channel_mesh(400, 80)
    return m, host_boundary(m, channel_bc), 1.0 / 200.0, None, (0.3, 0.3)


SERVE_REQUESTS = [  # (rid, kind, cells, Re, speed)
    (0, "cavity", 1024, 100.0, 1.0),
    (1, "cavity", 2500, 400.0, 1.5),
    (2, "channel", 4096, 100.0, 1.0),
]


def make_serve_converged(max_iters=8000):
    from warpcfd_gb300.serve import RELAXATION, MeshCache

    mc = MeshCache()
    out = {}
    for rid, kind, cells, re, speed in SERVE_REQUESTS:
        m = mc.get(kind, cells)
        nu = speed / re
        if kind == "cavity":
            b = host_boundary(m, cavity_bc, lid=speed)
            ref = 0
        else:
            b = host_boundary(m, channel_bc, u_in=speed)
            ref = None
        oc = OracleCase(geometry_from_mesh(m), b.boundary_type, b.boundary_values, nu, 1.0, T=np.float64,
                        reference_cell=ref, atol=1e-13, maxiter=20000, p_refine=4, p_refine_rtol=1e-3)
        ur, pr = RELAXATION[kind]
        t = time.time()
        for it in range(max_iters):
            prev = oc.cell_values.copy()
            oc.run(ur, pr, n_outer=1)
            scale = np.abs(oc.cell_values).max(axis=0) + 1e-300
            if np.all(np.abs(oc.cell_values - prev).max(axis=0) <= 1e-10 * scale):
                break
        else:
            raise RuntimeError(f"request {rid} did not reach its fixed point in {max_iters} iterations")
        print(f"serve request {rid} ({kind}, {m.num_cells} cells): {it + 1} iterations, {time.time() - t:.1f}s",
              flush=True)
        out[f"r{rid}"] = oc.cell_values.copy()
        out[f"r{rid}_spec"] = np.array([rid, cells, re, speed, 1.0 if kind == "cavity" else 0.0])
        out[f"r{rid}_iterations"] = it + 1
        o32 = OracleCase(geometry_from_mesh(m), b.boundary_type, b.boundary_values, nu, 1.0, T=np.float32,
                         reference_cell=ref, atol=1e-9, maxiter=20000, p_refine=4, p_refine_rtol=1e-3)
        o32.run(ur, pr, n_outer=(3 * (it + 1)) // 2)
        out[f"r{rid}_fp32"] = o32.cell_values.astype(np.float64)
    np.savez_compressed(os.path.join(HERE, "serve_fp64_converged.npz"), **out)


def make(name):
    if name == "serve_fp64_converged":
        return make_serve_converged()
    spec = SPECS[name]
    m, b, nu, ref, relax = case_for(spec)
    oc = OracleCase(geometry_from_mesh(m), b.boundary_type, b.boundary_values, nu, 1.0, T=spec["T"],
                    reference_cell=ref, atol=spec["atol"], maxiter=spec.get("maxiter", 500),
                    p_refine=spec.get("p_refine", 0), p_refine_rtol=spec.get("p_refine_rtol", 1e-3))
    t = time.time()
    oc.run(*relax, n_outer=spec["iters"], log=True)
    krylov = np.array([(a, c) for a, _, c in oc.log], dtype=np.int32)
    np.savez_compressed(os.path.join(HERE, name + ".npz"),
                        cell_values=oc.cell_values.astype(spec.get("store", np.float64)),
                        krylov=krylov, atol=spec["atol"], iters=spec["iters"])
    print(name, f"{time.time() - t:.1f}s", "krylov max", krylov.max(0))


if __name__ == "__main__":
    names = sys.argv[1:] or (list(SPECS) + ["serve_fp64_converged"])
    if len(names) > 1:
        import multiprocessing as mp

        with mp.get_context("spawn").Pool(min(len(names), os.cpu_count() or 1)) as pool:
            pool.map(make, names)
    else:
        make(names[0])
