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
Each file stores cell_values (C,4) and the per-iteration Krylov counts.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.simple_ref import OracleCase, geometry_from_mesh  # noqa: E402
from tests.cases import cavity_bc, cavity_mesh, host_boundary  # noqa: E402

SPECS = {
    "ldc64_fp64_converged": dict(T=np.float64, atol=1e-10, iters=1500),
    "ldc64_fp32_converged": dict(T=np.float32, atol=1e-7, iters=1500),
    "ldc64_fp32_500": dict(T=np.float32, atol=1e-5, iters=500),
    "ldc64_fp64_500": dict(T=np.float64, atol=1e-6, iters=500),
}


def make(name):
    spec = SPECS[name]
    m = cavity_mesh(64)
    b = host_boundary(m, cavity_bc)
    oc = OracleCase(geometry_from_mesh(m), b.boundary_type, b.boundary_values, 0.01, 1.0, T=spec["T"],
                    reference_cell=0, atol=spec["atol"])
    t = time.time()
    oc.run(0.7, 0.3, n_outer=spec["iters"], log=True)
    krylov = np.array([(a, c) for a, _, c in oc.log], dtype=np.int32)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), cell_values=oc.cell_values.astype(np.float64),
                        krylov=krylov, atol=spec["atol"], iters=spec["iters"])
    print(name, f"{time.time() - t:.1f}s")


if __name__ == "__main__":
    for n in (sys.argv[1:] or list(SPECS)):
        make(n)
