"""Shared set-up of the GPU parity tests: the same case on the GPU (through the C ABI)
and in the oracle."""
import numpy as np
import torch

from oracle.simple_ref import OracleCase, geometry_from_mesh
from warpcfd_gb300.FV import FVM
from warpcfd_gb300.FV.implicit_Solvers import IncompressibleSolver


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def vel_err(g, o, comp):
    """||g_o - o_o|| / ||U|| for velocity component ``comp`` (U = all three components),
    so a near-zero transverse component is judged on the velocity scale."""
    return float(np.linalg.norm(g[:, comp] - o[:, comp]) / max(np.linalg.norm(o[:, 0:3]), 1e-300))


def make_pair(mesh, bc_fn, nu=0.01, rho=1.0, ref_cell=0, u_relax=0.7, p_relax=0.3, steady=True, dt=1.0,
              atol=None, correction=False, inner=1):
    model = FVM(mesh)
    model.material.create_incompressible_newtonian_fluid(viscosity=nu * rho, density=rho)
    if ref_cell is not None:
        model.set_reference_pressure(ref_cell, 0.0)
    bc_fn(model.boundary)
    model.finalize()
    solver = IncompressibleSolver(model, u_relax if steady else None, p_relax if steady else None,
                                  correction=correction, steady_state=steady)
    solver.verbose = False
    solver.set_iterations(1, inner, 1)
    if not steady:
        solver.set_time_stepping(1, dt)
    if atol is not None:
        solver.vel_equation.tol = atol
        solver.p_corr_equation.tol = atol
    b = model.boundary
    oc = OracleCase(geometry_from_mesh(mesh), b.boundary_type, b.boundary_values, nu * rho, rho, T=np.float32,
                    reference_cell=ref_cell, correction=correction, atol=atol)
    return model, solver, oc


def oracle_step(oc, u_relax=0.7, p_relax=0.3, steady=True, dt=1.0, inner=1):
    oc.run(u_relax, p_relax, n_outer=1, n_inner=inner, steady=steady, dt=dt, log=True)


def fields(model):
    torch.cuda.synchronize()
    return model.cell_values.cpu().numpy().astype(np.float64)
