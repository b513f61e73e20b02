"""Runs the unmodified warp_cfd solver (from the reference sources) on the numpy Warp
stand-in (oracle/warp_stand_in) and writes its outputs as fixtures tests/golden/ref_*.npz.

  python tests/golden/make_reference_golden.py [name ...]     (needs the warp_cfd sources:
                                                              $WCFD_REFERENCE, default
                                                              /root/reference)

warp-lang (the reference's runtime) is not installed on these machines, so the stand-in
executes the reference's own Warp kernels as Python, one call per thread index, and
restates the third-party pieces it calls (warp.sparse for 1x1 blocks, warp.optim.linear
cg / bicgstab / Jacobi preconditioner).  The imports that are case-broken on Linux
(FV/model.py:12 ``warp_cfd.FV.convergence``, FV/terms/convection.py:6 and
diffusion.py:5 ``warp_cfd.FV.implicit_Schemes``) are aliased to the files that exist.
Meshes come from this package's structured generators, handed to the reference's own
``Mesh`` through the pyvista stand-in.

Every case runs in float64 (``FVM(..., float_dtype=wp.float64)``) with the Krylov
tolerance tightened to 1e-13 and maxiter 20000, so the solves end at the solution and
not at a rounding-dependent stopping point: the fixtures pin the method.  Each file
stores the reference mesh pass's arrays (before ``finalize``), the boundary table, the
settings and the final ``model.cell_values``.

Cases (small meshes: the stand-in runs a kernel thread per Python call):
  ref_ldc16            64^2-style cavity at 16 x 16, Re 100, SIMPLE 0.7 / 0.3, 30 iterations
                       (examples/LDC/LDC.py:38-49)
  ref_channel80x16     channel 80 x 16 on 10 x 1, velocity inlet u = 1, pressure outlet,
                       Re 200, SIMPLE 0.3 / 0.3, 30 iterations (examples/Channel Flow/
                       Channel Flow.py:41-51 with a velocity inlet; at 40 x 8 the method
                       diverges at Re 200, in the reference as in the oracle)
  ref_ldc12_skew       12 x 12 cavity, interior nodes jittered by 20% (seed 1): skew
                       correction of the face values, 20 iterations
  ref_ldc12_corrected  the same mesh with non-orthogonal correction (correction=True)
  ref_piso_ldc12       12 x 12 cavity, PISO (steady_state=False), dt 0.05, 2 correctors,
                       8 time steps
"""
from __future__ import annotations

import contextlib
import importlib.abc
import importlib.util
import io
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
STAND_IN = os.path.join(ROOT, "oracle", "warp_stand_in")
REFERENCE = os.environ.get("WCFD_REFERENCE", "/root/reference")

CASES = {
    "ref_ldc16": dict(kind="cavity", n=16, iters=30),
    "ref_channel80x16": dict(kind="channel", nx=80, ny=16, iters=30),
    "ref_ldc12_skew": dict(kind="cavity", n=12, jitter=0.2, seed=1, iters=20),
    "ref_ldc12_corrected": dict(kind="cavity", n=12, jitter=0.2, seed=1, iters=20, correction=True),
    "ref_piso_ldc12": dict(kind="cavity", n=12, piso=True, dt=0.05, steps=8, correctors=2),
}
TOL = 1e-13
MAXITER = 20000

# (case-broken name used by the reference's imports) -> (the module that exists)
_ALIASES = {"warp_cfd.FV.convergence": "warp_cfd.FV.Convergence",
            "warp_cfd.FV.implicit_Schemes": "warp_cfd.FV.Implicit_Schemes"}


class _CaseAliasFinder(importlib.abc.MetaPathFinder):
    def find_spec(self, fullname, path, target=None):
        for alias, real in _ALIASES.items():
            if fullname == alias or fullname.startswith(alias + "."):
                rel = (real + fullname[len(alias):]).replace(".", os.sep)
                base = os.path.join(REFERENCE, rel)
                if os.path.isdir(base):
                    return importlib.util.spec_from_file_location(fullname, os.path.join(base, "__init__.py"),
                                                                  submodule_search_locations=[base])
                return importlib.util.spec_from_file_location(fullname, base + ".py")
        return None


def _setup_imports():
    if STAND_IN not in sys.path:
        sys.path.insert(0, STAND_IN)
    if REFERENCE not in sys.path:
        sys.path.insert(1, REFERENCE)
    if not any(isinstance(f, _CaseAliasFinder) for f in sys.meta_path):
        sys.meta_path.insert(0, _CaseAliasFinder())


def _grid(spec):
    """This package's structured generator -> the pyvista stand-in grid."""
    import pyvista as pv

    from warpcfd_gb300.preprocess.grid import create_2D_grid

    if spec["kind"] == "cavity":
        g = create_2D_grid((0, 0, 0), spec["n"], spec["n"], 1.0, 1.0, 0.1, jitter=spec.get("jitter", 0.0),
                           seed=spec.get("seed", 0))
    else:
        g = create_2D_grid((0, 0, 0), spec["nx"], spec["ny"], 10.0, 1.0, 0.1)
    return pv.UnstructuredGrid(g.cells, g.celltypes, g.points)


def _mesh_arrays(m):
    """The reference mesh pass's arrays (numpy, before finalize converts them)."""
    cp, fp = m.cell_properties, m.face_properties
    out = {}
    for pre, obj in (("cell_", cp), ("face_", fp)):
        for k, v in obj.__dict__.items():
            if isinstance(v, np.ndarray):
                out[pre + k] = v.copy()
    out["nodes"] = m.nodes.copy()
    out["cells"] = m.cells.copy()
    return out


def run_case(name):
    _setup_imports()
    import warp as wp
    from warp_cfd.FV.implicit_Solvers import IncompressibleSolver
    from warp_cfd.FV.model import FVM
    from warp_cfd.preprocess import Mesh, define_boundary_walls

    spec = CASES[name]
    m = Mesh(_grid(spec))
    define_boundary_walls(m)
    arrays = _mesh_arrays(m)
    model = FVM(m, output_variables=["u", "v", "w", "p"], float_dtype=wp.float64)
    b = model.boundary
    if spec["kind"] == "cavity":
        nu = 0.01
        model.material.create_incompressible_newtonian_fluid(viscosity=nu, density=1.0)
        model.set_reference_pressure(0, 0.0)
        b.no_slip_wall("-X")
        b.no_slip_wall("+X")
        b.no_slip_wall("-Y")
        b.velocity_BC("+Y", u=1, v=0, w=0)
        b.slip_wall("+Z")
        b.slip_wall("-Z")
        relax = (0.7, 0.3)
    else:
        nu = 1.0 / 200.0
        model.material.create_incompressible_newtonian_fluid(viscosity=nu, density=1.0)
        b.velocity_BC("-X", u=1, v=0, w=0)
        b.pressure_BC("+X", p=0.0)
        b.no_slip_wall("-Y")
        b.no_slip_wall("+Y")
        b.slip_wall("-Z")
        b.slip_wall("+Z")
        relax = (0.3, 0.3)
    bc_type = b.boundary_type.copy()
    bc_value = b.boundary_values.copy()
    t0 = time.time()
    with contextlib.redirect_stdout(io.StringIO()):
        model.finalize()
        if spec.get("piso"):
            solver = IncompressibleSolver(model, correction=spec.get("correction", False), steady_state=False)
            solver.set_time_stepping(spec["steps"], spec["dt"])
            solver.set_iterations(1, spec["correctors"], 1)
            n = spec["steps"]
        else:
            solver = IncompressibleSolver(model, *relax, correction=spec.get("correction", False))
            solver.set_iterations(spec["iters"], 1, 1)
            n = spec["iters"]
        for eq in (solver.vel_equation, solver.p_corr_equation):
            eq.tol = TOL
            eq.max_iter = MAXITER
        solver.run(n + 1)       # convergence report at step 0 and at the end only
    cell_values = model.cell_values.numpy().copy()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), cell_values=cell_values, bc_type=bc_type,
                        bc_value=bc_value, viscosity=nu, density=1.0, relax=np.array(relax),
                        reference_cell=0 if spec["kind"] == "cavity" else -1,
                        correction=bool(spec.get("correction", False)), piso=bool(spec.get("piso", False)),
                        dt=spec.get("dt", 1.0), steps=n, correctors=spec.get("correctors", 1), tol=TOL,
                        maxiter=MAXITER, **{"mesh_" + k: v for k, v in arrays.items()})
    print(name, f"{time.time() - t0:.1f}s", "C =", cell_values.shape[0], flush=True)


if __name__ == "__main__":
    sys.path.insert(0, ROOT)
    names = sys.argv[1:] or list(CASES)
    if len(names) > 1:
        import multiprocessing as mp

        with mp.get_context("spawn").Pool(min(len(names), os.cpu_count() or 1)) as pool:
            pool.map(run_case, names)
    else:
        run_case(names[0])
