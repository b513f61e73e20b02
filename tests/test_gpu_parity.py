"""Parity of the CUDA path (through the C ABI) with the oracle on the same seeded inputs.

Tolerances (relative L2; a velocity component is measured against the norm of the whole
velocity field, p against its own norm; fp32 arithmetic on both sides, so the only
differences are summation order and fma contraction):
  single operators ............... 1e-5 (faces/gradients), 1e-5 (assembled matrices)
  one SIMPLE/PISO step ........... 1e-5 (u, v, w), 1e-4 (p)
  5-step trajectory .............. 1e-4 (u, v, w), 1e-3 (p)
The fixed-iteration-count comparison at the reference's own Krylov tolerance is
path-dependent (see test_gpu_converged.py for the converged comparison).
"""
import numpy as np
import pytest
import torch

from tests.cases import (cavity3d_bc, cavity3d_mesh, cavity_bc, cavity_mesh, channel_bc, channel_mesh,
                         mixed_cavity3d_mesh, prism_cavity_mesh, prism_channel_mesh, tet_cavity3d_mesh)
from tests.gpu_helpers import fields, make_pair, oracle_step, rel_l2, vel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib_ready():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from warpcfd_gb300.build import build_library
    build_library()


def _seed_state(model, oc, seed):
    rng = np.random.default_rng(seed)
    C = model.num_cells
    cv = rng.uniform(-1, 1, size=(C, 4)).astype(np.float32)
    cg = rng.uniform(-1, 1, size=(C, 4, 3)).astype(np.float32)
    model.cell_values.copy_(torch.from_numpy(cv))
    model.cell_gradients.copy_(torch.from_numpy(cg))
    oc.cell_values[:] = cv
    oc.cell_gradients[:] = cg


@pytest.mark.parametrize("jitter", [0.0, 0.15])
def test_face_pass_gradients_flux_div(jitter):
    m = cavity_mesh(12, jitter=jitter, seed=5)
    model, solver, oc = make_pair(m, cavity_bc)
    _seed_state(model, oc, 1)
    model.set_boundary_conditions()
    model.face_interpolation()
    oc.apply_bc()
    oc.face_interpolation()
    fv = model.face_values.cpu().numpy()
    for o in range(4):
        assert rel_l2(fv[:, o], oc.face_values[:, o]) < 1e-6
    model.calculate_gradients()
    oc.calculate_gradients()
    g = model.cell_gradients.cpu().numpy()
    assert rel_l2(g, oc.cell_gradients) < 1e-5
    model.calculate_mass_flux()
    oc.calculate_mass_flux()
    assert rel_l2(model.mass_fluxes.cpu().numpy(), oc.mass_fluxes) < 1e-6
    d = model.divFlux().cpu().numpy()
    assert np.abs(d - oc.div_flux()).max() <= 1e-5 * np.abs(oc.mass_fluxes).max()
    # p-only gradient zeroes every other field (model.py:237)
    model.calculate_gradients("p")
    g = model.cell_gradients.cpu().numpy()
    assert np.abs(g[:, :3]).max() == 0.0 and np.abs(g[:, 3]).max() > 0


def test_upwind_face_interpolation():
    m = cavity_mesh(8, jitter=0.1, seed=2)
    model, solver, oc = make_pair(m, cavity_bc)
    _seed_state(model, oc, 2)
    mf = np.random.default_rng(3).standard_normal(m.num_faces).astype(np.float32)
    model.mass_fluxes.copy_(torch.from_numpy(mf))
    model.face_interpolation(upwind=True)
    fv = model.face_values.cpu().numpy()
    fp = m.face_properties
    ii = fp.internal_face_ids
    P, N = fp.adjacent_cells[ii, 0], fp.adjacent_cells[ii, 1]
    up = np.where(mf[ii] > 0, P, N)
    oc.face_interpolation()  # skew term of the linear scheme = same skew correction
    lin = oc.cell_values[P] * oc.g.psi[ii, None] + oc.g.psi2[ii, None] * oc.cell_values[N]
    skew = oc.face_values[ii] - lin
    np.testing.assert_allclose(fv[ii], oc.cell_values[up] + skew, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("case", ["cavity", "channel", "cavity3d", "prism_channel", "mixed_cavity3d"])
def test_assembly_matches_oracle(case):
    mk = {"cavity": (lambda: cavity_mesh(10, jitter=0.1, seed=1), cavity_bc, 0),
          "channel": (lambda: channel_mesh(20, 5), channel_bc, None),
          "cavity3d": (lambda: cavity3d_mesh(5), cavity3d_bc, 0),
          "prism_channel": (lambda: prism_channel_mesh(20, 5), channel_bc, None),
          "mixed_cavity3d": (lambda: mixed_cavity3d_mesh(5, 0.5, seed=1), cavity3d_bc, 0)}[case]
    m = mk[0]()
    model, solver, oc = make_pair(m, mk[1], ref_cell=mk[2])
    _seed_state(model, oc, 4)
    # the face pass of an outer iteration, on both sides
    model.set_boundary_conditions()
    model.face_interpolation()
    model.calculate_gradients()
    model.calculate_mass_flux()
    oc.apply_bc()
    oc.face_interpolation()
    oc.calculate_gradients()
    oc.calculate_mass_flux()
    solver.assemble_momentum()
    wc = oc.convection_weights()
    wd = oc.diffusion_weights((0, 1, 2), 0.01)
    vals, rhs = oc.assemble(3, [(wc, 1.0), (wd, -1.0)], (), [(oc.grad_term(), -1.0)])
    oc.relax(vals, rhs, 0.7, (0, 1, 2))
    A_ref = oc.momentum_matrix(vals).toarray()
    A_gpu = solver.vel_equation.dense.cpu().numpy()
    assert rel_l2(A_gpu, A_ref) < 1e-5
    assert rel_l2(solver.vel_equation.rhs.cpu().numpy(), rhs.reshape(-1)) < 1e-5
    rua_ref = oc.g.volume / (vals[0, oc.diag_pos] * np.float32(1.0))
    assert rel_l2(solver.rUA.cpu().numpy(), rua_ref) < 1e-5
    # pressure system with rUA_f and div from the same state
    rua_f = np.random.default_rng(5).uniform(0.1, 1.0, size=m.num_faces).astype(np.float32)
    solver.rUA_faces.copy_(torch.from_numpy(rua_f))
    div = oc.div_flux()
    solver.div_u.copy_(torch.from_numpy(div))
    solver.assemble_pressure()
    wpd = oc.diffusion_weights((3,), rua_f)
    pv, prhs = oc.assemble(1, [(wpd, 1.0)])
    prhs[:, 0] += div
    if mk[2] is not None:
        rc = mk[2]
        s, e = oc.indptr[rc], oc.indptr[rc + 1]
        pv[0, s:e] = np.where(oc.pat_cols[s:e] == rc, 1.0, 0.0)
        prhs[rc, 0] = 0.0
    assert rel_l2(solver.p_corr_equation.dense.cpu().numpy(), oc.matrix(pv[0]).toarray()) < 1e-5
    assert rel_l2(solver.p_corr_equation.rhs.cpu().numpy(), prhs[:, 0]) < 1e-5


@pytest.mark.parametrize("case", ["cavity", "cavity_skew", "channel", "cavity3d"])
def test_simple_steps_track_oracle(case):
    mk = {"cavity": (lambda: cavity_mesh(24), cavity_bc, 0, 0.01),
          "cavity_skew": (lambda: cavity_mesh(16, jitter=0.15, seed=11), cavity_bc, 0, 0.01),
          "channel": (lambda: channel_mesh(40, 8), channel_bc, None, 0.05),
          "cavity3d": (lambda: cavity3d_mesh(8), cavity3d_bc, 0, 0.01)}[case]
    m = mk[0]()
    model, solver, oc = make_pair(m, mk[1], ref_cell=mk[2], nu=mk[3])
    for it in range(5):
        solver.step()
        oracle_step(oc)
        g = fields(model)
        st = solver.solve_stats()
        tol_u = 1e-5 if it == 0 else 1e-4
        tol_p = 1e-4 if it == 0 else 1e-3
        for o in range(3):
            assert vel_err(g, oc.cell_values, o) < tol_u, (it, o)
        assert rel_l2(g[:, 3], oc.cell_values[:, 3]) < tol_p, it
        assert st[0]["status"] in ("ok", "not converged") and st[1]["status"] in ("ok", "not converged")
        # the GPU needs the same number of Krylov iterations (+-2 near the stop boundary)
        assert abs(st[0]["iterations"] - oc.log[-1][0]) <= 2
        assert abs(st[1]["iterations"] - oc.log[-1][2]) <= 2


def test_piso_steps_track_oracle():
    m = cavity_mesh(20, jitter=0.1, seed=3)
    model, solver, oc = make_pair(m, cavity_bc, steady=False, dt=0.01, inner=2)
    for it in range(4):
        solver.step()
        oracle_step(oc, None, None, steady=False, dt=0.01, inner=2)
        g = fields(model)
        for o in (0, 1):
            assert vel_err(g, oc.cell_values, o) < 1e-4, (it, o)
        assert rel_l2(g[:, 3], oc.cell_values[:, 3]) < 1e-3, it


def test_snapshot_restore_replays_steps_bitwise():
    """Checkpoint/resume of a case: the steps after restore() repeat those after snapshot()."""
    m = cavity_mesh(24, jitter=0.1, seed=4)
    model, solver, _ = make_pair(m, cavity_bc, atol=1e-7)
    for _ in range(3):
        solver.step()
    snap = solver.snapshot()
    for _ in range(4):
        solver.step()
    torch.cuda.synchronize()
    first = model.cell_values.clone()
    k_first = solver.solve_stats()
    solver.restore(snap)
    for _ in range(4):
        solver.step()
    torch.cuda.synchronize()
    assert torch.equal(model.cell_values, first)
    assert solver.solve_stats() == k_first


def test_cuda_graph_replay_is_bitwise_identical():
    m = cavity_mesh(16)
    model_a, solver_a, _ = make_pair(m, cavity_bc)
    model_b, solver_b, _ = make_pair(m, cavity_bc)
    for _ in range(4):
        solver_a.step()
    solver_b.run(steps_per_check=0, use_cuda_graph=True)   # 1 outer loop: eager first step
    for _ in range(3):
        solver_b._graph_step_counted()
    torch.cuda.synchronize()
    assert torch.equal(model_a.cell_values, model_b.cell_values)


def test_runs_are_bitwise_reproducible():
    m = cavity_mesh(20, jitter=0.1, seed=1)
    outs = []
    for _ in range(2):
        model, solver, _ = make_pair(m, cavity_bc)
        for _ in range(3):
            solver.step()
        outs.append(fields(model))
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("case", ["cavity", "channel", "cavity3d"])
def test_cg_paths_agree_with_oracle(case):
    """The cluster-resident CGs (shared memory of one thread-block cluster: textbook, path
    2, and the single-reduction arrangement, path 3) and the grid-cooperative CG (path 1)
    solve the same assembled pressure system like the oracle's CG.  The single-reduction
    iterates equal the textbook ones up to rounding, which on the ill-conditioned channel
    system moves the solution at the absolute stop by up to ~1e-4: held to 3e-4."""
    import ctypes as ct

    from oracle.simple_ref import cg as oracle_cg, jacobi_inverse
    from warpcfd_gb300 import _lib

    mk = {"cavity": (lambda: cavity_mesh(40, jitter=0.1, seed=1), cavity_bc, 0),
          "channel": (lambda: channel_mesh(200, 40), channel_bc, None),
          "cavity3d": (lambda: cavity3d_mesh(16), cavity3d_bc, 0)}[case]
    m = mk[0]()
    model, solver, oc = make_pair(m, mk[1], ref_cell=mk[2])
    for _ in range(2):
        solver.step()
    torch.cuda.synchronize()
    pe = solver.p_corr_equation
    A = pe.matrix.to_dense().cpu().numpy().astype(np.float32)
    import scipy.sparse as sp
    As = sp.csr_matrix(A)
    b = pe.rhs.cpu().numpy()
    xo = np.zeros_like(b)
    ko, _ = oracle_cg(As, b, xo, jacobi_inverse(np.diag(A).copy()), 1e-6, 300)
    lib = _lib.load()
    out = {}
    try:
        for path in (1, 2, 3):
            assert lib.wcfd_set_krylov_path(path) == 0
            x = torch.zeros_like(pe.x)
            pe.tol, pe.max_iter = 1e-6, 300
            st, _ = pe.solve_Axb(x)
            out[path] = (x.cpu().numpy(), st)
    finally:
        lib.wcfd_set_krylov_path(0)
    for path, (x, st) in out.items():
        assert abs(st["iterations"] - ko) <= max(2, ko // 50), (path, st, ko)
        assert rel_l2(x, xo) < (1e-4 if path < 3 else 3e-4), path
    assert rel_l2(out[1][0], out[2][0]) < 1e-4
    assert rel_l2(out[1][0], out[3][0]) < 3e-4


@pytest.mark.parametrize("prisms", [False, True])
def test_cylinder_piso_with_correction_tracks_oracle(prisms):
    """The cylinder-in-channel PISO case, small: jittered O-grid of hexes around a cylinder and
    a far field of hexes or of prisms (the prism/hex mesh of the benchmark case), parabolic
    inlet, PISO with 2 correctors and the non-orthogonal Laplacian correction."""
    from warpcfd_gb300.preprocess import (Mesh, create_cylinder_channel_grid, define_boundary_walls,
                                          define_cylinder_group)

    g, info = create_cylinder_channel_grid(scale=0.18 if prisms else 0.25, jitter=0.1, seed=5, prisms=prisms)
    m = Mesh(g)
    define_boundary_walls(m)
    define_cylinder_group(m, info["cylinder"])
    ids = m.groups["-X"].ids
    y = m._geometry64["face_centroid"][ids, 1]
    u_in = 4.0 * 1.5 * y * (0.41 - y) / 0.41 ** 2

    def bc(b):
        b.velocity_BC("-X", u=u_in, v=0.0, w=0.0)
        b.pressure_BC("+X", p=0.0)
        b.no_slip_wall("-Y")
        b.no_slip_wall("+Y")
        b.no_slip_wall("cylinder")
        b.slip_wall("-Z")
        b.slip_wall("+Z")

    # This pressure system is poorly conditioned (Neumann walls and cylinder, a weak outlet
    # Dirichlet row, coefficients scaled by dt): the rounding of an fp32 assembly alone
    # moves p by a few percent, while u, v are fixed to ~1e-5.  The GPU runs the precision
    # form (fp64 iterative refinement of the pressure solve, so the solve adds no error of
    # its own) and is held against an fp64 oracle solved to atol 1e-12: u, v to 1e-4 and p
    # within 3x the spread between the fp32 oracle (atol 1e-7) and the fp64 oracle.
    model, solver, oc = make_pair(m, bc, nu=1e-3, ref_cell=None, steady=False, dt=5e-4, correction=True,
                                  inner=2, atol=1e-7)
    solver.p_refine, solver.p_refine_rtol = 3, 1e-3
    from oracle.simple_ref import OracleCase, geometry_from_mesh
    b = model.boundary
    oc64 = OracleCase(geometry_from_mesh(m), b.boundary_type, b.boundary_values, 1e-3, 1.0, T=np.float64,
                      correction=True, atol=1e-12, maxiter=3000)
    for it in range(3):
        solver.step()
        oracle_step(oc, None, None, steady=False, dt=5e-4, inner=2)
        oracle_step(oc64, None, None, steady=False, dt=5e-4, inner=2)
        gv = fields(model)
        for o in (0, 1):
            assert vel_err(gv, oc64.cell_values, o) < 1e-4, (it, o)
        err_gpu = rel_l2(gv[:, 3], oc64.cell_values[:, 3])
        err_o32 = rel_l2(oc.cell_values[:, 3], oc64.cell_values[:, 3])
        assert err_gpu < 3 * err_o32 + 1e-4, (it, err_gpu, err_o32, solver.solve_stats())


def test_fp64_refined_pressure_solve_is_fp64_accurate():
    """Precision form: wcfd_cg_refine solves the fp32-assembled pressure system to fp64
    accuracy (checked against an fp64 direct solve of the same matrix)."""
    import ctypes as ct

    import scipy.sparse.linalg as spla

    from warpcfd_gb300 import _lib

    m = cavity_mesh(24, jitter=0.1, seed=4)
    model, solver, _ = make_pair(m, cavity_bc)
    for _ in range(2):
        solver.step()
    torch.cuda.synchronize()
    pe = solver.p_corr_equation
    A = pe.matrix.to_dense().cpu().numpy().astype(np.float64)
    b = pe.rhs.cpu().numpy().astype(np.float64)
    x_exact = spla.spsolve(__import__("scipy.sparse", fromlist=["csr_matrix"]).csr_matrix(A), b)
    C = model.num_cells
    x64 = torch.zeros(C, dtype=torch.float64, device="cuda")
    x32 = torch.zeros(C, dtype=torch.float32, device="cuda")
    work = torch.zeros(2 * C + 4, dtype=torch.float32, device="cuda")
    st = torch.zeros(_lib.STATS_BYTES, dtype=torch.uint8, device="cuda")
    _lib.call("wcfd_cg_refine", ct.byref(model.mesh_struct()), pe.system_struct(), ct.c_void_p(x64.data_ptr()),
              ct.c_void_p(x32.data_ptr()), ct.c_void_p(work.data_ptr()), pe.workspace_struct(), 4, 1e-3, 500,
              ct.c_void_p(st.data_ptr()), ct.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    err64 = rel_l2(x64.cpu().numpy(), x_exact)
    it4 = int(np.frombuffer(st.cpu().numpy().tobytes(), dtype=_lib.STATS_DTYPE)[0]["iterations"])
    # the statistics count the correction solves of every sweep: more than one sweep's
    x1 = torch.zeros(C, dtype=torch.float64, device="cuda")
    _lib.call("wcfd_cg_refine", ct.byref(model.mesh_struct()), pe.system_struct(), ct.c_void_p(x1.data_ptr()),
              ct.c_void_p(x32.data_ptr()), ct.c_void_p(work.data_ptr()), pe.workspace_struct(), 1, 1e-3, 500,
              ct.c_void_p(st.data_ptr()), ct.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    it1 = int(np.frombuffer(st.cpu().numpy().tobytes(), dtype=_lib.STATS_DTYPE)[0]["iterations"])
    assert it4 > it1 > 0, (it4, it1)
    # one fp32 CG to its floor, for comparison
    x_plain = torch.zeros(C, dtype=torch.float32, device="cuda")
    pe.tol, pe.max_iter = 0.0, 500
    pe.solve_Axb(x_plain)
    err32 = rel_l2(x_plain.cpu().numpy(), x_exact)
    assert err64 < 1e-9, (err64, err32)
    assert err64 < 1e-3 * err32


@pytest.mark.parametrize("path", [1, 2, 3])
def test_relative_krylov_stop(path):
    """wcfd_krylov_solve: the solve ends at ||r|| <= rtol ||r_0|| (both methods, both CG
    paths), after fewer iterations than an absolute stop far below it; rtol 0 reproduces
    wcfd_cg bit for bit."""
    from warpcfd_gb300 import _lib

    m = cavity_mesh(24, jitter=0.1, seed=4)
    model, solver, _ = make_pair(m, cavity_bc)
    for _ in range(2):
        solver.step()
    torch.cuda.synchronize()
    lib = _lib.load()
    lib.wcfd_set_krylov_path(path)
    try:
        for eq in (solver.p_corr_equation, solver.vel_equation):
            x0 = eq.x.clone()
            eq.tol, eq.max_iter, eq.rtol = 1e-14, 500, 1e-2
            x = x0.clone()
            st, _ = eq.solve_Axb(x)
            assert st["residual"] <= 1e-2 * st["initial_residual"] * (1 + 1e-6), st
            eq.rtol = 1e-6
            x_deep = x0.clone()
            deep, _ = eq.solve_Axb(x_deep)
            assert st["iterations"] < deep["iterations"], (st, deep)
            # rtol = 0 is the reference's absolute stop: the same bits as wcfd_cg / wcfd_bicgstab
            eq.rtol, eq.tol = 0.0, 1e-6
            xa, xb = x0.clone(), x0.clone()
            sa, _ = eq.solve_Axb(xa)
            fn = "wcfd_bicgstab" if eq.linear_solver == "bicgstab" else "wcfd_cg"
            import ctypes as ct
            _lib.call(fn, ct.byref(model.mesh_struct()), eq.system_struct(), ct.c_void_p(xb.data_ptr()),
                      eq.workspace_struct(), 1e-6, 500, ct.c_void_p(eq.stats.data_ptr()),
                      ct.c_void_p(torch.cuda.current_stream().cuda_stream))
            torch.cuda.synchronize()
            assert torch.equal(xa, xb)
    finally:
        lib.wcfd_set_krylov_path(0)


def test_device_convergence_monitor_matches_reference_norms():
    """wcfd_convergence_norms (one fused pass) gives the norms of model.py:278-316 computed
    the reference's way (torch fp64 over the same arrays)."""
    m = cavity_mesh(24, jitter=0.1, seed=4)
    model, solver, _ = make_pair(m, cavity_bc)
    for _ in range(3):
        solver.step()
    torch.cuda.synchronize()
    ve = solver.vel_equation
    norms = model.convergence_norms(ve.system_struct(), solver.HbyA, solver.div_u, solver.rUA,
                                    solver.p_corr_equation.x)
    Ax = ve.apply(solver.HbyA).reshape(-1, 3).double()
    b = ve.rhs.reshape(-1, 3).double()
    ref = [float(torch.linalg.vector_norm(Ax[:, o] - b[:, o])) for o in range(3)]
    ref += [float(torch.linalg.vector_norm(b[:, o])) for o in range(3)]
    div = model.divFlux(solver.div_u).double()
    ref.append(float(div.abs().sum()))
    vc = model.cell_gradients[:, 3, :].double() * solver.rUA.double()[:, None]
    ref.append(float(vc.abs().max()))
    ref.append(float(solver.p_corr_equation.x.double().abs().max()))
    for k, (got, want) in enumerate(zip(norms, ref)):
        # the residual is a difference of fp32 SpMV results: both sides round A x in fp32
        tol = 1e-4 if k < 3 else 1e-6
        assert abs(got - want) <= tol * max(abs(want), 1e-30) + 1e-12, (k, got, want)
    conv, _ = model.check_convergence_norms(norms)
    assert set(conv) >= {"momentum_x", "continuity", "velocity_correction", "pressure_correction"}


@pytest.mark.parametrize("case", ["cavity_skew", "channel"])
def test_rhie_chow_option_tracks_oracle(case):
    """Opt-in Rhie-Chow convecting flux (IncompressibleSolver.rhie_chow): the GPU follows the
    oracle's restatement of the same option step by step."""
    mk = {"cavity_skew": (lambda: cavity_mesh(16, jitter=0.15, seed=11), cavity_bc, 0, 0.01),
          "channel": (lambda: channel_mesh(40, 8), channel_bc, None, 0.05)}[case]
    model, solver, oc = make_pair(mk[0](), mk[1], ref_cell=mk[2], nu=mk[3])
    solver.rhie_chow = True
    oc.rhie_chow = True
    for it in range(5):
        solver.step()
        oracle_step(oc)
        g = fields(model)
        tol_u = 1e-5 if it == 0 else 1e-4
        tol_p = 1e-4 if it == 0 else 1e-3
        for o in range(3):
            assert vel_err(g, oc.cell_values, o) < tol_u, (it, o)
        assert rel_l2(g[:, 3], oc.cell_values[:, 3]) < tol_p, it
    # the option changes the flux from the second iteration on (rUA_f is zero before)
    m2, s2, _ = make_pair(mk[0](), mk[1], ref_cell=mk[2], nu=mk[3])
    for _ in range(5):
        s2.step()
    assert not torch.equal(model.cell_values, m2.cell_values)


def test_cluster_cg_at_its_size_limit():
    """The cluster-resident CG at the largest system its 16 CTAs hold (65,536 rows of width
    4, 4,096 rows per CTA, 4 rows per thread) and one row past it (the solve falls back to
    the grid-cooperative kernel) agree with the grid kernel on the same systems."""
    from warpcfd_gb300 import _lib

    lib = _lib.load()
    rows = int(lib.wcfd_batch_max_rows(4))
    assert rows == 4096
    for n, m_ in ((256, 256), (257, 256)):
        mesh = cavity_mesh(n) if n == m_ else channel_mesh(n, m_, lx=float(n) / m_)
        bc = cavity_bc if n == m_ else channel_bc
        model, solver, _ = make_pair(mesh, bc, ref_cell=0 if n == m_ else None)
        solver.step()
        torch.cuda.synchronize()
        pe = solver.p_corr_equation
        out = {}
        try:
            for path in (1, 2):
                assert lib.wcfd_set_krylov_path(path) == 0
                x = torch.zeros_like(pe.x)
                pe.tol, pe.max_iter = 1e-7, 400
                st, _ = pe.solve_Axb(x)
                out[path] = (x.cpu().numpy(), st)
        finally:
            lib.wcfd_set_krylov_path(0)
        assert abs(out[1][1]["iterations"] - out[2][1]["iterations"]) <= max(2, out[1][1]["iterations"] // 50), (n, out)
        assert rel_l2(out[1][0], out[2][0]) < 1e-4, n


@pytest.mark.parametrize("steady", [True, False])
def test_term_equation_api_matches_fused_assembly(steady):
    """The reference's Term/Equation API (terms forming their weights, form_system, relax,
    add_RHS, replace_row) builds the same momentum and pressure systems as the fused solver
    assembly, to rounding (the generic assembly adds the terms' weights in another order)."""
    m = cavity_mesh(12, jitter=0.1, seed=6)
    model, solver, oc = make_pair(m, cavity_bc, steady=steady, dt=0.01)
    _seed_state(model, oc, 7)
    model.set_boundary_conditions()
    model.face_interpolation()
    model.calculate_gradients()
    model.calculate_mass_flux()
    solver.assemble_momentum()                 # fused: terms, relaxation (steady) and rUA
    ve = solver.vel_equation
    fused = [t.clone() for t in (ve.diag, ve.off, ve.rhs)]
    ve.diag.zero_(), ve.off.zero_(), ve.rhs.zero_()
    nu = float(model.material.viscosity) / float(model.material.density)
    solver.convection(model)
    solver.diffusion(model, viscosity=nu)
    solver.grad_P(model)
    inv_density = 1.0 / float(model.material.density)
    if steady:
        ve.form_system([solver.convection, -solver.diffusion], explicit_terms=-inv_density * solver.grad_P, fvm=model)
        ve.relax(solver.u_relaxation_factor, model)
    else:
        solver.ddt(model, dt=0.01)
        ve.form_system([solver.ddt, solver.convection, -solver.diffusion],
                       explicit_terms=-inv_density * solver.grad_P, fvm=model)
    torch.cuda.synchronize()
    for a, b in zip(fused, (ve.diag, ve.off, ve.rhs)):
        assert rel_l2(b.cpu().numpy(), a.cpu().numpy()) < 1e-6
    # pressure: form_system + add_RHS(div) + replace_row, against the fused pressure assembly
    rua_f = torch.rand(m.num_faces, device="cuda") + 0.1
    solver.rUA_faces.copy_(rua_f)
    div = torch.randn(m.num_cells, device="cuda")
    solver.div_u.copy_(div)
    solver.assemble_pressure()
    pe = solver.p_corr_equation
    fused = [t.clone() for t in (pe.diag, pe.off, pe.rhs)]
    pe.diag.zero_(), pe.off.zero_(), pe.rhs.zero_()
    solver.p_correction_diffusion(model, viscosity=rua_f)
    pe.form_system(solver.p_correction_diffusion, fvm=model)
    pe.add_RHS(div)
    pe.replace_row(model.reference_pressure_cell_id, float(model.reference_pressure))
    torch.cuda.synchronize()
    for a, b in zip(fused, (pe.diag, pe.off, pe.rhs)):
        assert rel_l2(b.cpu().numpy(), a.cpu().numpy()) < 1e-6


def _reference_style_iteration(model, solver):
    """One outer iteration written as IncompressibleSolver.run writes it
    (warp_cfd/FV/implicit_Solvers/incompressible.py:95-156), on this package's API."""
    from warpcfd_gb300.FV.kernels import calculate_rUA, get_HbyA, interpolate_cell_value_to_face

    density = float(model.material.density)
    nu = float(model.material.viscosity) / density
    inv_density = 1.0 / density
    ve, pe = solver.vel_equation, solver.p_corr_equation
    model.set_boundary_conditions()
    model.face_interpolation()
    model.calculate_gradients()
    model.calculate_mass_flux()
    solver.convection(model)
    solver.diffusion(model, viscosity=nu)
    solver.grad_P(model)
    ve.form_system([solver.convection, -solver.diffusion], explicit_terms=-inv_density * solver.grad_P, fvm=model)
    ve.relax(solver.u_relaxation_factor, model)
    Ap = ve.diagonal
    _, HbyA = ve.solve_Axb(solver.HbyA)
    p_grad = model.get_gradient("p").flatten()
    rUA = calculate_rUA(Ap, density, model, solver.rUA)
    HbyA = get_HbyA(HbyA, rUA, p_grad)
    interpolate_cell_value_to_face(solver.rUA_faces, rUA, model)
    model.replace_cell_values(["u", "v", "w"], HbyA)
    model.face_interpolation()
    model.calculate_gradients()
    model.calculate_mass_flux()
    div_u = model.divFlux()
    solver.p_correction_diffusion(model, viscosity=solver.rUA_faces)
    pe.form_system(solver.p_correction_diffusion, fvm=model)
    pe.add_RHS(div_u)
    if model.reference_pressure_cell_id is not None:
        pe.replace_row(model.reference_pressure_cell_id, float(model.reference_pressure))
    _, p_new = pe.solve_Axb()
    model.relax(p_new, alpha=solver.p_relaxation_factor, output_index=3)
    model.face_interpolation("p")
    model.calculate_gradients("p")
    vel_correction = model.get_gradient("p", coeff=rUA).flatten()
    HbyA -= vel_correction
    model.replace_cell_values(["u", "v", "w"], HbyA)


def test_reference_style_loop_matches_fused_step():
    """A SIMPLE loop written against the reference's API (terms, form_system, relax,
    solve_Axb, calculate_rUA, get_HbyA, ...) follows the fused step: the same solves on
    the same systems, differing only where a separate kernel rounds an expression the fused
    kernel contracts into one FMA."""
    m = cavity_mesh(20, jitter=0.1, seed=8)
    model_a, solver_a, _ = make_pair(m, cavity_bc)
    model_b, solver_b, _ = make_pair(m, cavity_bc)
    for it in range(3):
        solver_a.step()
        _reference_style_iteration(model_b, solver_b)
        ga, gb = fields(model_a), fields(model_b)
        for o in range(3):
            assert vel_err(gb, ga, o) < 1e-5, (it, o)
        assert rel_l2(gb[:, 3], ga[:, 3]) < 1e-4, it


@pytest.mark.parametrize("variant", ["skew", "corrected", "upwind_linear"])
def test_explicit_internal_terms_option_tracks_oracle(variant):
    """Opt-in internal-face explicit weights (IncompressibleSolver.explicit_internal_terms):
    the convection skew term, the upwindLinear term and the non-orthogonal diffusion part
    reach the RHS on the GPU as in the oracle's restatement of the same option."""
    m = cavity_mesh(16, jitter=0.15, seed=11)
    corr = variant == "corrected"
    model, solver, oc = make_pair(m, cavity_bc, correction=corr)
    solver.explicit_internal_terms = True
    oc.explicit_internal = True
    if variant == "upwind_linear":
        solver.convection.interpolation = "upwindLinear"
        oc.conv_scheme = "upwindLinear"
    for it in range(4):
        solver.step()
        oracle_step(oc)
        g = fields(model)
        tol_u = 1e-5 if it == 0 else 1e-4
        tol_p = 1e-4 if it == 0 else 1e-3
        for o in range(3):
            assert vel_err(g, oc.cell_values, o) < tol_u, (it, o)
        assert rel_l2(g[:, 3], oc.cell_values[:, 3]) < tol_p, it
    m2, s2, _ = make_pair(m, cavity_bc, correction=corr)
    for _ in range(4):
        s2.step()
    assert not torch.equal(model.cell_values, m2.cell_values)


@pytest.mark.parametrize("case", ["prism_cavity", "mixed_cavity_skew", "prism_channel", "mixed_cavity3d",
                                  "tet_cavity3d", "tet_cavity3d_skew"])
def test_prism_and_mixed_meshes_track_oracle(case):
    """Wedge, tetrahedral and mixed hex/prism meshes (null slots past a wedge's five
    faces): the GPU step follows the oracle on the same mesh, corrected and uncorrected.  The
    prism channel is 5 long: on a 10-long one the oracle's own results move by 1.1e-5
    when only the summation order of its SpMV changes, above the 1e-5 bound."""
    mk = {"prism_cavity": (lambda: prism_cavity_mesh(12, "wedge"), cavity_bc, 0, 0.01, False),
          "mixed_cavity_skew": (lambda: prism_cavity_mesh(16, "mixed", jitter=0.1, seed=5), cavity_bc, 0, 0.01, True),
          "prism_channel": (lambda: prism_channel_mesh(20, 5, lx=5.0), channel_bc, None, 0.05, False),
          "mixed_cavity3d": (lambda: mixed_cavity3d_mesh(8, 0.5, seed=2), cavity3d_bc, 0, 0.01, True),
          "tet_cavity3d": (lambda: tet_cavity3d_mesh(5), cavity3d_bc, 0, 0.01, False),
          "tet_cavity3d_skew": (lambda: tet_cavity3d_mesh(5, jitter=0.15, seed=6), cavity3d_bc, 0, 0.01, True)}[case]
    m = mk[0]()
    model, solver, oc = make_pair(m, mk[1], ref_cell=mk[2], nu=mk[3], correction=mk[4])
    for it in range(5):
        solver.step()
        oracle_step(oc)
        g = fields(model)
        tol_u = 1e-5 if it == 0 else 1e-4
        tol_p = 1e-4 if it == 0 else 1e-3
        for o in range(3):
            assert vel_err(g, oc.cell_values, o) < tol_u, (it, o)
        assert rel_l2(g[:, 3], oc.cell_values[:, 3]) < tol_p, it
        st = solver.solve_stats()
        assert abs(st[1]["iterations"] - oc.log[-1][2]) <= 2


@pytest.mark.parametrize("case", ["cavity_skew", "cavity3d"])
def test_central_difference_convection_tracks_oracle(case):
    """ConvectionTerm interpolation 'central difference' (convection.py:43-91): the fused
    momentum assembly takes the (psi, 1 - psi) weights, as the oracle does; an unsupported
    scheme raises instead of running upwind."""
    mk = {"cavity_skew": (lambda: cavity_mesh(16, jitter=0.15, seed=11), cavity_bc, 0, 0.02),
          "cavity3d": (lambda: cavity3d_mesh(8), cavity3d_bc, 0, 0.02)}[case]
    model, solver, oc = make_pair(mk[0](), mk[1], ref_cell=mk[2], nu=mk[3])
    solver.convection.interpolation = "central difference"
    oc.conv_scheme = "central difference"
    for it in range(4):
        solver.step()
        oracle_step(oc)
        g = fields(model)
        tol_u = 1e-5 if it == 0 else 1e-4
        tol_p = 1e-4 if it == 0 else 1e-3
        for o in range(3):
            assert vel_err(g, oc.cell_values, o) < tol_u, (it, o)
        assert rel_l2(g[:, 3], oc.cell_values[:, 3]) < tol_p, it
    m2, s2, _ = make_pair(mk[0](), mk[1], ref_cell=mk[2], nu=mk[3])
    for _ in range(4):
        s2.step()
    assert not torch.equal(model.cell_values, m2.cell_values)
    solver.convection.interpolation = "custom"
    with pytest.raises(NotImplementedError):
        solver.step()


@pytest.mark.parametrize("shape", [(1, 1), (2, 1), (3, 2), (33, 1), (7, 5)])
def test_tiny_and_odd_meshes_track_oracle(shape):
    """Edge cases of the mesh size: a single cell (every face a boundary face, no
    off-diagonals: W = 0), one-row meshes (W = 1, 2), and sizes that fill no warp or block
    evenly; the step follows the oracle.  The velocities of a one-cell-tall strip are ~4e-4,
    so at the reference's absolute Krylov stop (1e-5) both runs stop anywhere within a few
    percent of the solution; both solve to 1e-9 here, so the comparison measures the
    arithmetic, not the stopping point."""
    from warpcfd_gb300.preprocess import Mesh, create_2D_grid, define_boundary_walls

    nx, ny = shape
    m = Mesh(create_2D_grid((0, 0, 0), nx, ny, 1.0, 1.0, 0.1))
    define_boundary_walls(m)
    model, solver, oc = make_pair(m, cavity_bc, ref_cell=0, nu=0.05, atol=1e-9)
    assert model._geo["ell_width"] == min(4, (nx > 1) * (1 + (nx > 2)) + (ny > 1) * (1 + (ny > 2)))
    for it in range(3):
        solver.step()
        oracle_step(oc)
        g = fields(model)
        un = np.linalg.norm(oc.cell_values[:, 0:3])
        if un > 0:
            for o in range(3):
                assert vel_err(g, oc.cell_values, o) < 1e-4, (it, o)
        pn = np.linalg.norm(oc.cell_values[:, 3])
        assert np.linalg.norm(g[:, 3] - oc.cell_values[:, 3]) <= 1e-3 * pn + 1e-6, it
        assert np.isfinite(g).all()


@pytest.mark.parametrize("case", ["tet_cavity3d", "mixed_cavity3d"])
def test_piso_on_tetra_and_mixed_meshes_tracks_oracle(case):
    """Transient PISO (2 correctors, non-orthogonal correction) on a jittered tetrahedral
    cavity and on a mixed hex/prism cavity follows the oracle."""
    mk = {"tet_cavity3d": lambda: tet_cavity3d_mesh(5, jitter=0.1, seed=3),
          "mixed_cavity3d": lambda: mixed_cavity3d_mesh(7, 0.5, seed=4)}[case]
    model, solver, oc = make_pair(mk(), cavity3d_bc, steady=False, dt=0.01, inner=2, correction=True)
    for it in range(4):
        solver.step()
        oracle_step(oc, None, None, steady=False, dt=0.01, inner=2)
        g = fields(model)
        for o in range(3):
            assert vel_err(g, oc.cell_values, o) < 1e-4, (it, o)
        assert rel_l2(g[:, 3], oc.cell_values[:, 3]) < 1e-3, it
