"""The GPU drop-in against the reference's own code.

tests/golden/ref_*.npz hold the fields the unmodified warp_cfd solver computed on the
numpy Warp stand-in (tests/golden/make_reference_golden.py; float64, Krylov solves
tightened to 1e-13): a 16 x 16 cavity and an 80 x 16 channel (30 SIMPLE iterations), a
jittered 12 x 12 cavity with skew correction and with non-orthogonal correction (20
iterations), and a 12 x 12 PISO run (8 time steps, 2 correctors).  The GPU runs the same
case through the C ABI in float32 with its solves tightened (momentum BiCGSTAB to atol
1e-9, the pressure solve by fp64 iterative refinement).

The bar per field (u, v, w on the velocity scale, p relative): within 1e-5 of the
reference, or, where float32 arithmetic cannot get that close, within three times the
distance of the oracle's own float32 run of the same method (same tightened solves, the
reference's mesh arrays) from the reference.  Measured: on the cavities every field is
within 2e-6; on the channel the float32 method itself is 1.4e-5 (u) and 8e-5 (p) away
and the GPU the same; PISO p is 6e-5 (float32 oracle 3e-5).
"""
import glob
import os

import numpy as np
import pytest
import torch

from tests.cases import cavity_bc, channel_bc
from tests.gpu_helpers import fields, make_pair
from tests.test_reference_pin import NAMES, _grid_for, field_errors, load, oracle_run

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib_ready():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from warpcfd_gb300.build import build_library
    build_library()


@pytest.mark.parametrize("name", NAMES)
def test_gpu_matches_the_reference(name):
    from warpcfd_gb300.preprocess import Mesh, define_boundary_walls

    d = load(name)
    m = Mesh(_grid_for(name))
    define_boundary_walls(m)
    channel = int(d["reference_cell"]) < 0
    piso = bool(d["piso"])
    relax = d["relax"]
    model, solver, _ = make_pair(m, channel_bc if channel else cavity_bc, nu=float(d["viscosity"]),
                                 ref_cell=None if channel else 0, u_relax=float(relax[0]), p_relax=float(relax[1]),
                                 steady=not piso, dt=float(d["dt"]), atol=1e-9, correction=bool(d["correction"]),
                                 inner=int(d["correctors"]) if piso else 1)
    solver.vel_equation.max_iter = 5000
    solver.p_corr_equation.max_iter = 5000
    solver.p_refine = 4
    solver.p_refine_rtol = 1e-3
    for _ in range(int(d["steps"])):
        solver.step()
    g = fields(model)
    st = solver.solve_stats()
    assert st[0]["status"] == "ok" and st[1]["status"] == "ok", st
    e = field_errors(g, d["cell_values"])
    # the float32 floor of the method: the oracle's float32 run with the same tightened
    # solves (pressure refined the same way), from the reference's own mesh arrays
    f32 = field_errors(oracle_run(d, T=np.float32, atol=1e-9, maxiter=5000, p_refine=4), d["cell_values"])
    fmt = lambda x: " ".join(f"{k} {v:.2e}" for k, v in x.items())  # noqa: E731
    print(f"\n{name}: GPU (fp32) vs the reference (fp64 on the Warp stand-in): {fmt(e)}"
          f"\n{name}: fp32 oracle vs the reference: {fmt(f32)}")
    for f in "uvwp":
        assert e[f] <= max(1e-5, 3.0 * f32[f]), (f, e, f32)
