"""Batched form: many cases advanced together, one launch sequence per outer iteration.

A :class:`CaseBatch` holds finalized ``IncompressibleSolver`` cases whose meshes share the
cell type (faces per cell) and off-diagonal width.  Their C case structs are copied into a
device case table; ``wcfd_batch_simple_iteration`` then runs every field, assembly and
solve kernel once for the whole table (each case's Krylov solves on one thread-block
cluster), so the number of launches per iteration does not grow with the number of
cases.  All cases' solver outcomes land in one device buffer, read with one copy.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np
import torch

from . import _lib


class CaseBatch:
    """``cluster_size``: CTAs per case for the Krylov solves (0 = the library's pick);
    ``field_block``: threads per block of the field and assembly kernels (0 = 256; see
    warpcfd_gb300.autotune).  The device case table is uploaded on the stream current at
    construction (and at refresh()); a caller that steps the batch on another stream must
    first make that stream wait for this one."""

    def __init__(self, solvers, cluster_size: int = 0, device=None, field_block: int = 0, cg_variant: int = 0):
        if not solvers:
            raise ValueError("a batch needs at least one case")
        self.solvers = list(solvers)
        g0 = self.solvers[0].model._geo
        self.faces_per_cell = g0["faces_per_cell"]
        self.ell_width = g0["ell_width"]
        for s in self.solvers:
            g = s.model._geo
            if g["faces_per_cell"] != self.faces_per_cell or g["ell_width"] != self.ell_width:
                raise ValueError("every case of a batch must have the same cell type and off-diagonal width")
            if (s.NUM_INNER_LOOPS, s.NUM_ORTHOGONAL_CORRECTORS) != (self.solvers[0].NUM_INNER_LOOPS,
                                                                      self.solvers[0].NUM_ORTHOGONAL_CORRECTORS):
                raise ValueError("every case of a batch must use the same corrector counts")
            if int(s.p_refine) != int(self.solvers[0].p_refine):
                raise ValueError("every case of a batch must use the same number of pressure refinement sweeps")
        self.device = self.solvers[0].model.device
        n = len(self.solvers)
        self.stats = torch.zeros(n * 2 * _lib.STATS_BYTES, dtype=torch.uint8, device=self.device)
        self.dims = _lib.BatchDims_t(
            max(s.model.num_cells for s in self.solvers), max(s.model.num_faces for s in self.solvers),
            self.faces_per_cell, self.ell_width, self.solvers[0].NUM_INNER_LOOPS,
            self.solvers[0].NUM_ORTHOGONAL_CORRECTORS, int(cluster_size), int(field_block), 0,
            int(self.solvers[0].p_refine), int(cg_variant))
        self._graph = None
        self._graph_steps = 0
        self.table = torch.empty(n * ct.sizeof(_lib.Case_t), dtype=torch.uint8, device=self.device)
        self.refresh()

    def __len__(self):
        return len(self.solvers)

    @property
    def field_block(self) -> int:
        return self.dims.field_block or 256

    @property
    def cluster_size(self) -> int:
        d = _lib.BatchDims_t.from_buffer_copy(self.dims)
        return d.cluster_size or int(_lib.load().wcfd_batch_cluster_size(ct.byref(d)))

    def refresh(self):
        """(Re)build the device case table from the solvers' current parameters."""
        n = len(self.solvers)
        arr = (_lib.Case_t * n)()
        xt = 0
        for i, s in enumerate(self.solvers):
            c = _lib.Case_t.from_buffer_copy(s.case_struct())
            c.stats = self.stats.data_ptr() + i * 2 * _lib.STATS_BYTES
            c.events = None
            arr[i] = c
            xt |= int(c.prm.explicit_terms)
        if xt != self.dims.explicit_terms:
            # the assembly kernels the step launches depend on it: a captured graph is stale
            self.dims.explicit_terms = xt
            self._graph = None
            self._graph_steps = 0
        host = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8)
        self.table.copy_(host.to(self.device))

    def step(self):
        """One SIMPLE outer iteration (or PISO step) of every case, on the current stream."""
        lib = _lib.load()
        rc = lib.wcfd_batch_simple_iteration(ct.c_void_p(self.table.data_ptr()), len(self.solvers),
                                             ct.byref(self.dims),
                                             ct.c_void_p(torch.cuda.current_stream().cuda_stream))
        if rc != 0:
            raise _lib.WcfdError(rc, lib.wcfd_batch_last_error().decode(errors="replace"))

    def steps(self, n: int):
        """n outer iterations of every case as one CUDA graph replay on the current stream
        (the graph of n batched steps is captured on first use, without running them, and
        kept while the batch lives: the launch sequence depends only on the dims).  The
        current stream must not be the legacy default stream."""
        if self._graph is None or self._graph_steps != n:
            _lib.check(_lib.load().wcfd_batch_prepare(ct.byref(self.dims)))
            g = torch.cuda.CUDAGraph()
            g.capture_begin(capture_error_mode="thread_local")
            try:
                for _ in range(n):
                    self.step()
            finally:
                g.capture_end()
            self._graph, self._graph_steps = g, n
        self._graph.replay()

    def solve_stats(self):
        """Per case: [(momentum stats), (pressure stats)] as numpy records."""
        raw = np.frombuffer(self.stats.cpu().numpy().tobytes(), dtype=_lib.STATS_DTYPE)
        return raw.reshape(len(self.solvers), 2)

    def relative_residuals(self) -> np.ndarray:
        """Per case: initial momentum residual / ||b|| of the last outer iteration (the
        nonlinear residual of the momentum equations at the start of that iteration)."""
        st = self.solve_stats()
        return st[:, 0]["initial_residual"] / np.maximum(st[:, 0]["rhs_norm"], 1e-300)
