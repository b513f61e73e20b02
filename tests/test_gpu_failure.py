"""Failure detection on the GPU without a fault: the grid barrier of the cooperative Krylov
kernels is checked for correct sums, and a wait that nothing satisfies (one block never
arrives) runs out after its bounded limit and comes back as WCFD_BARRIER_TIMEOUT with the
context still usable."""
import ctypes as ct
import time

import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib_ready():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from warpcfd_gb300.build import build_library
    build_library()


def _check(skip, phases):
    from warpcfd_gb300 import _lib
    res = (ct.c_int32 * 3)()
    _lib.check(_lib.load().wcfd_grid_barrier_check(skip, phases, res, None))
    return list(res)


def test_grid_barrier_sums_are_exact():
    status, bad, blocks = _check(-1, 2000)
    assert (status, bad) == (0, 0)
    assert blocks >= torch.cuda.get_device_properties(0).multi_processor_count


def test_grid_barrier_wait_runs_out_and_context_survives():
    from warpcfd_gb300 import _lib
    _, _, blocks = _check(-1, 1)
    t0 = time.perf_counter()
    status, bad, _ = _check(blocks - 1, 5)
    elapsed = time.perf_counter() - t0
    assert status == _lib.WCFD_BARRIER_TIMEOUT and bad == 0
    assert 1.0 < elapsed < 30.0
    # the context is still usable: a clean check and a device computation afterwards
    assert _check(-1, 10)[:2] == [0, 0]
    x = torch.arange(1000, device="cuda", dtype=torch.float32)
    assert float(x.sum()) == 499500.0
