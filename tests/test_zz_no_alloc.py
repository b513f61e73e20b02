"""GPU test of wcfd_cg_noalloc, the allocation-free pressure solve.

Some callers hold their own input and output device arrays but cannot allocate device
workspace (device memory fixed at start-up, plugins that may not allocate).  For them
the library keeps the CG workspace in a fixed array of its own.  This test calls that
entry point through the C ABI, twice in a row on the same system, and checks each
result against wcfd_cg run with a caller-provided workspace (relative L2 <= 1e-6, same
iteration count), then checks that a system above the size limit is refused.
The file name makes pytest collect it after every other test.
"""
import ctypes as ct

import numpy as np
import pytest
import torch

from tests.cases import cavity_bc, cavity_mesh
from tests.gpu_helpers import make_pair, rel_l2

pytestmark = pytest.mark.gpu

MAX_CELLS = 131072   # WCFD_NOALLOC_MAX_CELLS in include/wcfd.h


def _stats(t):
    from warpcfd_gb300 import _lib

    raw = np.frombuffer(t.cpu().numpy().tobytes(), dtype=_lib.STATS_DTYPE)
    return int(raw["iterations"][0]), int(raw["status"][0]), float(raw["residual"][0])


def test_noalloc_cg_matches_workspace_cg():
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

    m = cavity_mesh(48, jitter=0.1, seed=3)
    model, solver, _ = make_pair(m, cavity_bc)
    solver.step()                       # leaves an assembled pressure system behind
    torch.cuda.synchronize()
    pe = solver.p_corr_equation
    mesh_t = model.mesh_struct()
    stream = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    C = model.num_cells

    x_ref = torch.zeros(C, dtype=torch.float32, device="cuda")
    st_ref = torch.zeros(_lib.STATS_BYTES, dtype=torch.uint8, device="cuda")
    # the reference result comes from wcfd_cg on its grid-cooperative kernel, the one the
    # allocation-free entry point runs, so the two must agree to the last bit
    assert lib.wcfd_set_krylov_path(1) == 0
    try:
        rc = lib.wcfd_cg(ct.byref(mesh_t), pe.system_struct(), ct.c_void_p(x_ref.data_ptr()),
                         pe.workspace_struct(), 1e-6, 500, ct.c_void_p(st_ref.data_ptr()), stream)
    finally:
        lib.wcfd_set_krylov_path(0)
    assert rc == 0, lib.wcfd_last_error()
    torch.cuda.synchronize()
    it_ref, status_ref, _ = _stats(st_ref)
    assert status_ref in (0, 4) and it_ref > 0

    for _ in range(2):
        x = torch.zeros(C, dtype=torch.float32, device="cuda")
        st = torch.zeros(_lib.STATS_BYTES, dtype=torch.uint8, device="cuda")
        rc = fn(ct.byref(mesh_t), pe.system_struct(), ct.c_void_p(x.data_ptr()), 1e-6, 500,
                ct.c_void_p(st.data_ptr()), stream)
        assert rc == 0, lib.wcfd_last_error()
        torch.cuda.synchronize()
        it, status, _ = _stats(st)
        assert (it, status) == (it_ref, status_ref)
        assert rel_l2(x.cpu().numpy(), x_ref.cpu().numpy()) <= 1e-6

    big = _lib.Mesh_t.from_buffer_copy(mesh_t)
    big.n_cells = MAX_CELLS + 1
    rc = fn(ct.byref(big), pe.system_struct(), ct.c_void_p(x_ref.data_ptr()), 1e-6, 500,
            ct.c_void_p(st_ref.data_ptr()), stream)
    assert rc == _lib.WCFD_ERR_TOO_LARGE
    assert b"WCFD_NOALLOC_MAX_CELLS" in lib.wcfd_last_error()
