"""Properties of the step on the 128^3 lid-driven cavity (2,097,152 cells, Re = 400, the
bandwidth workload), a size the oracle cannot step in test time:

* the fields stay finite and bounded by the lid speed after three outer iterations;
* the pressure solve (grid-cooperative CG over 152 blocks) reports ||b|| and its final
  ||b - A x|| as float64 recomputes them from the assembled matrix and right-hand side;
* a step replayed from a snapshot repeats the fields and fluxes bit for bit: the grid
  Krylov kernels merge the blocks' partial sums in one fixed order.
"""
import pytest
import torch

from tests.cases import cavity3d_bc

pytestmark = pytest.mark.gpu

N = 128


@pytest.fixture(scope="module")
def cavity128():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from warpcfd_gb300.build import build_library
    from warpcfd_gb300.FV import FVM
    from warpcfd_gb300.FV.implicit_Solvers import IncompressibleSolver
    from warpcfd_gb300.preprocess import Mesh, create_3D_grid, define_boundary_walls

    build_library()
    m = Mesh(create_3D_grid((0, 0, 0), N, N, N, 1.0, 1.0, 1.0), device="cuda")
    define_boundary_walls(m)
    model = FVM(m)
    model.material.create_incompressible_newtonian_fluid(viscosity=1.0 / 400.0, density=1.0)
    model.set_reference_pressure(0, 0.0)
    cavity3d_bc(model.boundary)
    model.finalize()
    solver = IncompressibleSolver(model, 0.7, 0.3)
    solver.verbose = False
    solver.set_iterations(1, 1, 1)
    for _ in range(3):
        solver.step()
    torch.cuda.synchronize()
    return model, solver


def test_fields_finite_and_bounded(cavity128):
    model, _ = cavity128
    v = model.cell_values
    assert v.shape[0] == N ** 3
    assert bool(torch.isfinite(v).all())
    speed = v[:, :3].abs().max().item()
    assert 0.0 < speed <= 1.5, speed


def test_pressure_solve_norms_match_float64_recomputation(cavity128):
    model, solver = cavity128
    pe = solver.p_corr_equation
    x = torch.zeros_like(pe.x)
    st, _ = pe.solve_Axb(x)
    torch.cuda.synchronize()
    A = pe.matrix
    A64 = torch.sparse_csr_tensor(A.crow_indices(), A.col_indices(), A.values().double(), A.shape)
    b = pe.rhs.double()
    r = b - (A64 @ x.double().reshape(-1, 1)).reshape(-1)
    bn, rn = b.norm().item(), r.norm().item()
    info = (st, bn, rn, pe.tol)
    assert st["status"] == "ok" and st["iterations"] > 10, info
    # x0 = 0: the kernel's float-float norm of b against float64 over the same float32 array
    assert abs(st["rhs_norm"] - bn) <= 1e-6 * bn, info
    assert abs(st["initial_residual"] - bn) <= 1e-6 * bn, info
    assert st["residual"] <= pe.tol * (1 + 1e-6), info
    # the recurrence residual against the true one: float32 vectors over ~170 iterations
    assert rn <= max(2.0 * pe.tol, st["residual"] + 1e-3 * bn), info


def test_step_replays_bit_for_bit(cavity128):
    model, solver = cavity128
    snap = solver.snapshot()
    solver.step()
    torch.cuda.synchronize()
    a, fa = model.cell_values.clone(), model.mass_fluxes.clone()
    solver.restore(snap)
    solver.step()
    torch.cuda.synchronize()
    assert torch.equal(a, model.cell_values)
    assert torch.equal(fa, model.mass_fluxes)
