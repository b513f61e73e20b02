"""GPU test of wcfd_cg_noalloc, the allocation-free pressure solve.

Some callers hold their own input and output device arrays but cannot allocate device
workspace (device memory fixed at start-up, plugins that may not allocate).  For them
the library keeps the CG workspace in a fixed array of its own.  This test calls that
entry point through the C ABI, twice in a row on the same system, and checks each
result against wcfd_cg run with a caller-provided workspace on the same grid-cooperative
kernel: the same grid and the same fixed reduction order, so x, the iteration count, the
status and the residuals must agree to the last bit.  It does so on a small jittered
cavity and on a cavity just under the size limit (the top of the workspace's vector
region and the partial-sum and barrier words right after it are then in use), and
checks that a system above the limit is refused.
The file name makes pytest collect it after every other test.
"""
import ctypes as ct

import numpy as np
import pytest
import torch

from tests.cases import cavity_bc, cavity_mesh

pytestmark = pytest.mark.gpu

MAX_CELLS = 131072   # WCFD_NOALLOC_MAX_CELLS in include/wcfd.h


def _stats(t):
    from warpcfd_gb300 import _lib

    raw = np.frombuffer(t.cpu().numpy().tobytes(), dtype=_lib.STATS_DTYPE)[0]
    return (int(raw["iterations"]), int(raw["status"]), float(raw["residual"]), float(raw["initial_residual"]),
            float(raw["rhs_norm"]))


def _pressure_system(n, jitter, seed):
    """A GPU cavity case stepped once, which leaves an assembled pressure system behind."""
    from warpcfd_gb300.FV import FVM
    from warpcfd_gb300.FV.implicit_Solvers import IncompressibleSolver

    m = cavity_mesh(n, jitter=jitter, seed=seed)
    model = FVM(m)
    model.material.create_incompressible_newtonian_fluid(viscosity=0.01, density=1.0)
    model.set_reference_pressure(0, 0.0)
    cavity_bc(model.boundary)
    model.finalize()
    solver = IncompressibleSolver(model, 0.7, 0.3)
    solver.verbose = False
    solver.step()
    torch.cuda.synchronize()
    return model, solver


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from warpcfd_gb300 import _lib
    from warpcfd_gb300.build import build_library

    build_library()
    lib = _lib.load()
    fn = lib.wcfd_cg_noalloc
    fn.restype = ct.c_int
    fn.argtypes = [ct.POINTER(_lib.Mesh_t), _lib.System_t, ct.c_void_p, ct.c_double, ct.c_int32, ct.c_void_p,
                   ct.c_void_p]
    return lib


@pytest.mark.parametrize("n,jitter", [(48, 0.1), (362, 0.0)])
def test_noalloc_cg_matches_workspace_cg(lib, n, jitter):
    from warpcfd_gb300 import _lib

    model, solver = _pressure_system(n, jitter, 3)
    C = model.num_cells
    assert C <= MAX_CELLS
    if n == 362:
        assert C > MAX_CELLS - 64      # just under the limit
    pe = solver.p_corr_equation
    mesh_t = model.mesh_struct()
    stream = ct.c_void_p(torch.cuda.current_stream().cuda_stream)

    x_ref = torch.zeros(C, dtype=torch.float32, device="cuda")
    st_ref = torch.zeros(_lib.STATS_BYTES, dtype=torch.uint8, device="cuda")
    # the reference result comes from wcfd_cg on its grid-cooperative kernel, the one the
    # allocation-free entry point runs
    assert lib.wcfd_set_krylov_path(1) == 0
    try:
        rc = lib.wcfd_cg(ct.byref(mesh_t), pe.system_struct(), ct.c_void_p(x_ref.data_ptr()),
                         pe.workspace_struct(), 1e-6, 500, ct.c_void_p(st_ref.data_ptr()), stream)
    finally:
        lib.wcfd_set_krylov_path(0)
    assert rc == 0, lib.wcfd_last_error()
    torch.cuda.synchronize()
    ref = _stats(st_ref)
    assert ref[1] in (0, 4) and ref[0] > 0

    for _ in range(2):
        x = torch.zeros(C, dtype=torch.float32, device="cuda")
        st = torch.zeros(_lib.STATS_BYTES, dtype=torch.uint8, device="cuda")
        rc = lib.wcfd_cg_noalloc(ct.byref(mesh_t), pe.system_struct(), ct.c_void_p(x.data_ptr()), 1e-6, 500,
                                 ct.c_void_p(st.data_ptr()), stream)
        assert rc == 0, lib.wcfd_last_error()
        torch.cuda.synchronize()
        # iterations, status, final and initial residual and |b|: all bit for bit
        assert _stats(st) == ref
        assert torch.equal(x, x_ref)


def test_noalloc_cg_refuses_more_than_the_limit(lib):
    from warpcfd_gb300 import _lib

    model, solver = _pressure_system(16, 0.0, 0)
    pe = solver.p_corr_equation
    big = _lib.Mesh_t.from_buffer_copy(model.mesh_struct())
    big.n_cells = MAX_CELLS + 1
    x = torch.zeros(model.num_cells, dtype=torch.float32, device="cuda")
    st = torch.zeros(_lib.STATS_BYTES, dtype=torch.uint8, device="cuda")
    stream = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.wcfd_cg_noalloc(ct.byref(big), pe.system_struct(), ct.c_void_p(x.data_ptr()), 1e-6, 500,
                             ct.c_void_p(st.data_ptr()), stream)
    assert rc == _lib.WCFD_ERR_TOO_LARGE
    assert b"WCFD_NOALLOC_MAX_CELLS" in lib.wcfd_last_error()
