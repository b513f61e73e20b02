"""Equation: the fixed-pattern linear system of one or three fields
(warp_cfd/FV/terms/equation.py:10-204).

Storage (per mesh, fixed for the run): ``diag`` (C*n, interleaved rows n*c + o as the
reference's BSR rows D*i+o), ``off`` (W x C, slot-major; shared by the n components
because the momentum off-diagonals do not depend on the component), ``rhs`` (C*n),
solution ``x`` (C*n).  ``matrix`` / ``dense`` export the same operator in CSR form.
``solve_Axb`` runs the persistent Krylov kernel: BiCGSTAB for n = 3 (the reference's
default solver, equation.py:11) and CG for n = 1 when ``solver='cg'``
(incompressible.py:32), Jacobi-preconditioned, atol 1e-5 (fp32), maxiter 500
(equation.py:35-39).
"""
from __future__ import annotations

import ctypes as ct

import numpy as np
import torch

from ... import _lib
from ..field import Field


class Equation:
    def __init__(self, fvm, fields, solver="bicgstab") -> None:
        if isinstance(fields, str):
            fields = [fields]
        if all(f in fvm.output_variables for f in fields):
            self.fields = [fvm.fields[f] for f in fields]
            self.global_output_indices = [f.index for f in self.fields]
        else:
            self.fields = [Field(f) for f in fields]
            self.global_output_indices = None
        self.num_outputs = len(fields)
        if self.num_outputs not in (1, 3):
            raise NotImplementedError("systems of 1 field (scalar) or 3 fields (velocity) are supported")
        solver = getattr(solver, "__name__", solver)
        if solver not in ("cg", "bicgstab"):
            raise ValueError("solver must be 'cg' or 'bicgstab'")
        if solver == "cg" and self.num_outputs != 1:
            raise NotImplementedError("cg is provided for scalar systems")
        if solver == "bicgstab" and self.num_outputs != 3:
            solver = "cg"
        self.linear_solver = solver
        self.fvm = fvm
        self.max_iter = 500
        self.tol = 1.0e-5
        # relative stop ||r|| <= rtol ||r_0|| on top of tol; 0 = tol alone, as in the reference
        self.rtol = 0.0
        C = fvm.num_cells
        n = self.num_outputs
        W = fvm._geo["ell_width"]
        dev = fvm.device
        f32 = dict(dtype=torch.float32, device=dev)
        self.sparse_rows = C * n
        self.diag = torch.zeros(C * n, **f32)
        self.off = torch.zeros(max(W, 1) * C, **f32)
        self.rhs = torch.zeros(C * n, **f32)
        self._x = torch.zeros(C * n, **f32)
        lib = _lib.load()
        nws = int(lib.wcfd_krylov_workspace_floats(C, n))
        self.ws_vec = torch.zeros(nws, **f32)
        self.ws_partials = torch.zeros(8 * _lib.MAX_BLOCKS, dtype=torch.float64, device=dev)
        self.ws_results = torch.zeros(8, dtype=torch.float64, device=dev)
        self.ws_barrier = torch.zeros(_lib.BARRIER_WORDS, dtype=torch.int32, device=dev)
        self.stats = torch.zeros(_lib.STATS_BYTES, dtype=torch.uint8, device=dev)

    @property
    def x(self):
        return self._x

    @property
    def diagonal(self):
        """Diagonal of the assembled system (equation.py:80-83)."""
        return self.diag

    def system_struct(self) -> _lib.System_t:
        return _lib.System_t(self.diag.data_ptr(), self.off.data_ptr(), self.rhs.data_ptr(), self.num_outputs, 0)

    def workspace_struct(self) -> _lib.KrylovWS_t:
        return _lib.KrylovWS_t(self.ws_vec.data_ptr(), self.ws_partials.data_ptr(), self.ws_results.data_ptr(),
                               self.ws_barrier.data_ptr())

    def apply(self, x: torch.Tensor) -> torch.Tensor:
        """y = A x (warp.sparse.bsr_mv)."""
        x = x.contiguous()
        y = torch.empty_like(x)
        m = self.fvm.mesh_struct()
        _lib.call("wcfd_spmv", ct.byref(m), self.system_struct(), ct.c_void_p(x.data_ptr()),
                  ct.c_void_p(y.data_ptr()), ct.c_void_p(torch.cuda.current_stream().cuda_stream))
        return y

    @property
    def matrix(self):
        """The system as a torch sparse CSR tensor (C*n x C*n), built on demand."""
        g = self.fvm._geo
        C, W, n = g["n_cells"], g["ell_width"], self.num_outputs
        col = g["ell_col"][:W].long()                   # (W, C)
        off = self.off[: W * C].reshape(W, C)
        own = torch.arange(C, device=col.device).expand(W, C)
        valid = col != own
        rows, cols, vals = [], [], []
        for o in range(n):
            rows.append(n * torch.arange(C, device=col.device) + o)
            cols.append(n * torch.arange(C, device=col.device) + o)
            vals.append(self.diag.reshape(C, n)[:, o])
            rows.append((n * own + o)[valid])
            cols.append((n * col + o)[valid])
            vals.append(off[valid])
        r = torch.cat(rows)
        c = torch.cat(cols)
        v = torch.cat(vals)
        coo = torch.sparse_coo_tensor(torch.stack([r, c]), v, (C * n, C * n)).coalesce()
        return coo.to_sparse_csr()

    @property
    def dense(self):
        return self.matrix.to_dense()

    # ------------------------------------------------------------------ assembly (equation.py:99-194)
    def form_system(self, implicit_terms=None, explicit_terms=None, *, fvm=None):
        """Assemble the system from terms (equation.py:99-125): any list of implicit terms,
        face-based (convection, diffusion) or cell-based (ddt), each with its assigned scale,
        added by one cell-parallel, atomic-free kernel (wcfd_assemble_terms), then every
        explicit term's weights times its scale added to the right-hand side.  Each term must
        have been called (``term(model, ...)``) so that its weights are current.  The
        system is overwritten (the reference resets it first, equation.py:202-204)."""
        fvm = self.fvm if fvm is None else fvm
        terms = [] if implicit_terms is None else (list(implicit_terms) if isinstance(implicit_terms, (list, tuple))
                                                   else [implicit_terms])
        if len(terms) > _lib.MAX_TERMS:
            raise ValueError(f"at most {_lib.MAX_TERMS} implicit terms")
        arr = (_lib.Term_t * max(len(terms), 1))()
        for i, t in enumerate(terms):
            if not t.implicit:
                raise AssertionError("form_system's implicit_terms must be implicit terms")
            if t.num_outputs != self.num_outputs:
                raise ValueError(f"a term of {t.num_outputs} fields in a system of {self.num_outputs}")
            if t.weights is None:
                raise ValueError("call the term first (term(model, ...)) so that its weights exist")
            arr[i] = _lib.Term_t(t.weights.data_ptr(), float(t.scale), int(bool(t.cell_based)))
        stream = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
        _lib.call("wcfd_assemble_terms", ct.byref(fvm.mesh_struct()), self.system_struct(), arr, len(terms), stream)
        ex = [] if explicit_terms is None else (list(explicit_terms) if isinstance(explicit_terms, (list, tuple))
                                                else [explicit_terms])
        for t in ex:
            if t.implicit:
                raise AssertionError("explicit_terms must be explicit terms")
            if t.weights is None:
                raise ValueError("call the term first (term(model, ...)) so that its weights exist")
            self.add_RHS(t.weights, t.scale)

    def relax(self, relaxation_factor, fvm=None):
        """Implicit relaxation on the diagonal (equation.py:173-182)."""
        fvm = self.fvm if fvm is None else fvm
        assert self.global_output_indices is not None, "Relaxation is only available for fields defined in fvm"
        f0 = self.global_output_indices[0]
        assert list(self.global_output_indices) == list(range(f0, f0 + self.num_outputs)), \
            "relaxation of non-contiguous fields"
        _lib.call("wcfd_relax", ct.byref(fvm.mesh_struct()), self.system_struct(),
                  ct.c_void_p(fvm.cell_values.data_ptr()), int(f0), float(relaxation_factor),
                  ct.c_void_p(torch.cuda.current_stream().cuda_stream))

    def replace_row(self, row_id, rhs_value):
        """Rows become the identity with the given right-hand side (equation.py:185-194)."""
        rows = [row_id] if isinstance(row_id, int) else [int(r) for r in row_id]
        vals = [rhs_value] * len(rows) if isinstance(rhs_value, (int, float)) else [float(v) for v in rhs_value]
        assert len(rows) == len(vals)
        m = self.fvm.mesh_struct()
        stream = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
        for r, v in zip(rows, vals):
            _lib.call("wcfd_replace_row", ct.byref(m), self.system_struct(), int(r), float(v), stream)

    def add_RHS(self, arr, scale=1.0):
        """rhs += scale arr (equation.py:167-168), on the device (wcfd_add_rhs)."""
        a = arr.reshape(-1)
        if a.numel() != self.rhs.numel():
            raise ValueError(f"add_RHS: {a.numel()} values for a right-hand side of {self.rhs.numel()}")
        if a.dtype != torch.float32 or not a.is_contiguous() or a.device != self.rhs.device:
            a = a.to(device=self.rhs.device, dtype=torch.float32).contiguous()
        _lib.call("wcfd_add_rhs", ct.c_void_p(self.rhs.data_ptr()), ct.c_void_p(a.data_ptr()), float(scale),
                  int(a.numel()), ct.c_void_p(torch.cuda.current_stream().cuda_stream))

    def reset(self):
        self.rhs.zero_()
        self.diag.zero_()
        self.off.zero_()

    def solve_Axb(self, x=None):
        """Krylov solve from x (warm start, in place).  Returns (stats dict, x)."""
        if x is None:
            x = self.x
        m = self.fvm.mesh_struct()
        stream = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
        if self.rtol > 0.0:
            _lib.call("wcfd_krylov_solve", ct.byref(m), self.system_struct(), ct.c_void_p(x.data_ptr()),
                      self.workspace_struct(), int(self.linear_solver == "bicgstab"), float(self.tol),
                      float(self.rtol), int(self.max_iter), ct.c_void_p(self.stats.data_ptr()), stream)
        else:
            fn = "wcfd_bicgstab" if self.linear_solver == "bicgstab" else "wcfd_cg"
            _lib.call(fn, ct.byref(m), self.system_struct(), ct.c_void_p(x.data_ptr()), self.workspace_struct(),
                      float(self.tol), int(self.max_iter), ct.c_void_p(self.stats.data_ptr()), stream)
        raw = np.frombuffer(self.stats.cpu().numpy().tobytes(), dtype=_lib.STATS_DTYPE)[0]
        return dict(iterations=int(raw["iterations"]), status=_lib.STATUS_NAMES.get(int(raw["status"]), "?"),
                    residual=float(raw["residual"]), initial_residual=float(raw["initial_residual"]),
                    rhs_norm=float(raw["rhs_norm"])), x
