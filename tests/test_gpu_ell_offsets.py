"""The grid CG reading int16 column offsets (wcfd_mesh.ell_dcol) gives the same bits as the
grid CG reading the int32 columns: the same columns, the same order of operations; the
momentum BiCGSTAB reads the int32 columns either way and is unchanged by the table.  Both
replace warp.optim.linear.cg / bicgstab as called by Equation.solve_Axb
(warp_cfd/FV/terms/equation.py:195-200)."""
import ctypes as ct

import pytest
import torch

from tests.cases import cavity3d_bc, cavity3d_mesh, channel_bc, channel_mesh
from tests.gpu_helpers import make_pair

pytestmark = pytest.mark.gpu


def _solve(eq, mesh_struct, x):
    from warpcfd_gb300 import _lib

    fn = "wcfd_bicgstab" if eq.linear_solver == "bicgstab" else "wcfd_cg"
    stream = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call(fn, ct.byref(mesh_struct), eq.system_struct(), ct.c_void_p(x.data_ptr()), eq.workspace_struct(),
              float(eq.tol), int(eq.max_iter), ct.c_void_p(eq.stats.data_ptr()), stream)
    torch.cuda.synchronize()
    return eq.stats.clone()


@pytest.mark.parametrize("case", ["cavity3d", "channel"])
def test_offsets_same_bits_as_columns(case):
    from warpcfd_gb300 import _lib

    mk = {"cavity3d": (lambda: cavity3d_mesh(24), cavity3d_bc, 0),
          "channel": (lambda: channel_mesh(200, 40), channel_bc, None)}[case]
    model, solver, _ = make_pair(mk[0](), mk[1], ref_cell=mk[2])
    assert model._geo["ell_dcol"] is not None
    for _ in range(2):
        solver.step()
    lib = _lib.load()
    assert lib.wcfd_set_krylov_path(1) == 0  # the grid-cooperative kernels
    try:
        for eq in (solver.p_corr_equation, solver.vel_equation):
            eq.tol, eq.max_iter = 1e-7, 300
            out = []
            for use_offsets in (True, False):
                m = model.mesh_struct()
                if not use_offsets:
                    m.ell_dcol = None
                assert (m.ell_dcol is not None) == use_offsets
                x = torch.zeros_like(eq.x)
                st = _solve(eq, m, x)
                out.append((x, st))
            assert torch.equal(out[0][1], out[1][1]), eq.linear_solver
            assert torch.equal(out[0][0], out[1][0]), eq.linear_solver
    finally:
        lib.wcfd_set_krylov_path(0)


def test_mesh_check_catches_a_wrong_offset():
    from warpcfd_gb300 import _lib

    model, _, _ = make_pair(cavity3d_mesh(6), cavity3d_bc)
    d = model._geo["ell_dcol"].clone()
    d[2, 17] += 1
    m = model.mesh_struct()
    m.ell_dcol = d.data_ptr()
    counts = (ct.c_int32 * 5)()
    lib = _lib.load()
    rc = lib.wcfd_check_mesh(ct.byref(m), counts, ct.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == _lib.WCFD_ERR_ARGUMENT
    assert list(counts) == [0, 0, 0, 0, 1]
    assert model.check_mesh() == [0, 0, 0, 0, 0]
