"""Pins of the oracle (the checker): analytic known answers for its operators, its
Krylov solvers against scipy, and the converged cavity against the Ghia et al.
centre-line tables that the reference ships (examples/LDC/*; read at test time)."""
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from oracle.simple_ref import OracleCase, bicgstab, cg, geometry_from_mesh, jacobi_inverse
from tests.cases import cavity3d_mesh, cavity_bc, cavity_mesh, channel_bc, channel_mesh, host_boundary
from tests.conftest import REFERENCE


def _case(m, bc_fn, T=np.float64, nu=0.01, **kw):
    b = host_boundary(m, bc_fn)
    return OracleCase(geometry_from_mesh(m), b.boundary_type, b.boundary_values, nu, 1.0, T=T, **kw)


def test_green_gauss_exact_for_linear_field():
    m = cavity3d_mesh(5)            # orthogonal hexes
    c = _case(m, lambda b: [b.no_slip_wall(w) for w in ("-X", "+X", "-Y", "+Y", "-Z", "+Z")])
    a = np.array([0.3, -1.2, 2.0])
    c.face_values[:, 0] = c.g.face_centroid @ a + 0.5
    c.calculate_gradients((0,))
    np.testing.assert_allclose(c.cell_gradients[:, 0], np.tile(a, (m.num_cells, 1)), atol=1e-12)
    assert np.abs(c.cell_gradients[:, 1:]).max() == 0.0


def test_skew_corrected_interpolation_exact_for_linear_field():
    m = cavity_mesh(7, jitter=0.15, seed=4)
    c = _case(m, cavity_bc)
    a = np.array([1.5, -0.7, 0.0])
    c.cell_values[:, 3] = c.g.centroid @ a + 2.0
    c.cell_gradients[:, 3] = a
    c.face_interpolation((3,))
    ii = c.g.internal_ids
    np.testing.assert_allclose(c.face_values[ii, 3], c.g.face_centroid[ii] @ a + 2.0, atol=1e-12)
    c.skew = False
    c.face_interpolation((3,))
    assert np.abs(c.face_values[ii, 3] - (c.g.face_centroid[ii] @ a + 2.0)).max() > 1e-4


def test_uniform_flow_is_divergence_free():
    m = cavity3d_mesh(4, jitter=0.1, seed=9)
    c = _case(m, lambda b: [b.no_slip_wall(w) for w in ("-X", "+X", "-Y", "+Y", "-Z", "+Z")])
    U = np.array([0.4, -0.2, 0.9])
    c.face_values[:, 0:3] = U
    c.calculate_mass_flux()
    np.testing.assert_allclose(c.mass_fluxes, (c.g.n_owner @ U) * c.g.area, rtol=1e-12)
    assert np.abs(c.div_flux()).max() < 1e-13


@pytest.mark.parametrize("solver", ["cg", "bicgstab"])
def test_krylov_matches_direct_solve(solver):
    rng = np.random.default_rng(0)
    n = 400
    A = sp.random(n, n, density=0.01, random_state=1, format="csr")
    A = A + A.T if solver == "cg" else A
    A = A + sp.diags(np.abs(A).sum(axis=1).A1 + 1.0)
    A = A.tocsr()
    b = rng.standard_normal(n)
    x = np.zeros(n)
    fn = cg if solver == "cg" else bicgstab
    k, r = fn(A, b, x, jacobi_inverse(A.diagonal().copy()), 1e-12, 500)
    assert r <= 1e-12 and 0 < k < 500
    np.testing.assert_allclose(x, spla.spsolve(A.tocsc(), b), rtol=1e-9, atol=1e-11)


def test_channel_develops_poiseuille_profile():
    m = channel_mesh(40, 12, lx=8.0, ly=1.0)
    c = _case(m, channel_bc, nu=0.1)
    c.run(0.7, 0.3, n_outer=300)
    cent = c.g.centroid
    outlet = np.abs(cent[:, 0] - cent[:, 0].max()) < 1e-9
    y = cent[outlet, 1]
    u = c.cell_values[outlet, 0]
    order = np.argsort(y)
    y, u = y[order], u[order]
    exact = 6.0 * y * (1.0 - y)           # mean 1, max 1.5
    assert np.abs(u - exact).max() < 0.03
    # global mass balance of the corrected velocity field: inflow = outflow
    c.apply_bc()
    c.face_interpolation()
    c.calculate_mass_flux()
    bmf = c.mass_fluxes[c.g.boundary_ids]
    assert abs(bmf.sum()) < 1e-4 * np.abs(bmf).sum()


GHIA_U = os.path.join(REFERENCE, "examples", "LDC", "u_velocity_results.txt")
GHIA_V = os.path.join(REFERENCE, "examples", "LDC", "v_velocity_results.csv")


def _read_table(path, sep):
    with open(path) as f:
        head = f.readline().strip().split(sep)
        rows = [list(map(float, ln.strip().split(sep))) for ln in f if ln.strip()]
    return head, np.array(rows)


@pytest.mark.skipif(not os.path.exists(GHIA_U), reason="reference data files not mounted")
def test_cavity_matches_ghia_centrelines():
    n = 32
    m = cavity_mesh(n)
    c = _case(m, cavity_bc, nu=0.01)
    c.run(0.7, 0.3, n_outer=400)
    cent = c.g.centroid
    hu, tu = _read_table(GHIA_U, "\t")
    hv, tv = _read_table(GHIA_V, ",")
    col_u = hu.index("100")
    col_v = hv.index("100")
    # vertical centre line x = 0.5 lies on a face: average the two cell columns
    xs = np.unique(np.round(cent[:, 0], 12))
    left, right = xs[n // 2 - 1], xs[n // 2]
    ys = np.unique(np.round(cent[:, 1], 12))
    uc = np.array([0.5 * (c.cell_values[(np.abs(cent[:, 0] - left) < 1e-9) & (np.abs(cent[:, 1] - y) < 1e-9), 0][0] +
                          c.cell_values[(np.abs(cent[:, 0] - right) < 1e-9) & (np.abs(cent[:, 1] - y) < 1e-9), 0][0])
                   for y in ys])
    u_at = np.interp(tu[:, 0], np.concatenate([[0.0], ys, [1.0]]), np.concatenate([[0.0], uc, [1.0]]))
    assert np.abs(u_at - tu[:, col_u]).max() < 0.06
    bot, top = ys[n // 2 - 1], ys[n // 2]
    vc = np.array([0.5 * (c.cell_values[(np.abs(cent[:, 1] - bot) < 1e-9) & (np.abs(cent[:, 0] - x) < 1e-9), 1][0] +
                          c.cell_values[(np.abs(cent[:, 1] - top) < 1e-9) & (np.abs(cent[:, 0] - x) < 1e-9), 1][0])
                   for x in xs])
    v_at = np.interp(tv[:, 0], np.concatenate([[0.0], xs, [1.0]]), np.concatenate([[0.0], vc, [0.0]]))
    assert np.abs(v_at - tv[:, col_v]).max() < 0.06
