"""IncompressibleSolver: SIMPLE / PISO driver with the API of
warp_cfd/FV/implicit_Solvers/incompressible.py:10-172.

One outer iteration (or PISO time step) is one call of ``wcfd_simple_iteration``, a fixed
sequence of fused kernels and two persistent Krylov launches on the current stream; with
``use_cuda_graph`` the sequence is captured once and replayed.  Solver outcomes stay on
the device until a convergence check reads them.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np
import torch

from ... import _lib
from ..model import FVM, _stream
from ..terms import ConvectionTerm, DdtTerm, DiffusionTerm, Equation, GradTerm

STATS_DTYPE = _lib.STATS_DTYPE


class IncompressibleSolver:
    def __init__(self, model: FVM, u_relaxation_factor=None, p_relaxation_factor=None, correction=False,
                 steady_state=True) -> None:
        if not model.finalized:
            raise ValueError("Please call method model.finalize() before passing model in to solver")
        self.model = model
        self.float_dtype = model.float_dtype
        velocity_vars = ["u", "v", "w"]
        self.steady_state = steady_state
        self.correction = correction
        if not steady_state:
            self.ddt = DdtTerm(model, velocity_vars)
        self.convection = ConvectionTerm(model, velocity_vars, "upwind")
        self.diffusion = DiffusionTerm(model, velocity_vars, correction=correction)
        self.grad_P = GradTerm(model, "p")
        self.vel_equation = Equation(model, fields=velocity_vars)
        self.p_correction_diffusion = DiffusionTerm(model, "p", correction=correction)
        self.p_corr_equation = Equation(model, fields="p", solver="cg")
        self.p_relaxation_factor = p_relaxation_factor
        self.u_relaxation_factor = u_relaxation_factor
        self.material = model.material
        C, K, dev = model.num_cells, model.num_faces, model.device
        f32 = dict(dtype=torch.float32, device=dev)
        self.HbyA = self.vel_equation.x          # (3C) interleaved, the momentum x0/out
        self.rUA = torch.zeros(C, **f32)
        self.rUA_faces = torch.zeros(K, **f32)
        self.div_u = torch.zeros(C, **f32)
        self.vel_correction = torch.zeros(C * 3, **f32)
        self.stats = torch.zeros(2 * STATS_DTYPE.itemsize, dtype=torch.uint8, device=dev)
        self.set_time_stepping(1, 1.0)
        self.NUM_ORTHOGONAL_CORRECTORS = 1
        self.NUM_OUTER_LOOPS = 1
        self.NUM_INNER_LOOPS = 1
        self.steps_done = 0
        self.verbose = True
        # precision form: fp64 iterative refinement of the pressure solve (0 = off)
        self.p_refine = 0
        self.p_refine_rtol = 1e-3
        # opt-in Rhie-Chow convecting flux (the reference re-interpolates the flux from the
        # corrected cell velocities, incompressible.py:97-99)
        self.rhie_chow = False
        # opt-in: internal-face explicit weights (skew correction of the convection, the
        # upwindLinear term when convection.interpolation == 'upwindLinear', the
        # non-orthogonal diffusion part) reach the RHS; the reference drops them
        self.explicit_internal_terms = False
        self.p_x64 = None
        self.p_work = None
        self._graph = None
        self._graph_key = None
        self._mesh_t = model.mesh_struct(correction=correction)
        self._events = None
        self._events_ptr = None

    def set_timing_events(self, events):
        """Record 4 torch.cuda.Events (already recorded once, so they exist) around the
        momentum solve and the last pressure solve of every step; None to stop."""
        if events is None:
            self._events, self._events_ptr = None, None
            return
        arr = (ct.c_void_p * 4)(*[ct.c_void_p(e.cuda_event) for e in events])
        self._events = (events, arr)
        self._events_ptr = ct.cast(arr, ct.c_void_p)

    def set_time_stepping(self, MAX_TIME_STEPS, dt, automatic=False, CFL_Max=1.0):
        if automatic is not False:
            raise NotImplementedError("automatic time stepping not yet implemented")
        self.MAX_TIME_STEPS = MAX_TIME_STEPS
        self.dt = dt

    def set_iterations(self, NUM_OUTER_LOOPS, NUM_INNER_LOOPS, NUM_ORTHOGONAL_CORRECTORS):
        self.NUM_OUTER_LOOPS = NUM_OUTER_LOOPS
        self.NUM_INNER_LOOPS = NUM_INNER_LOOPS
        self.NUM_ORTHOGONAL_CORRECTORS = NUM_ORTHOGONAL_CORRECTORS

    # ------------------------------------------------------------------ case struct
    def params(self) -> _lib.Params_t:
        m = self.model
        rho = float(self.material.density)
        nu = float(self.material.viscosity) / rho
        steady = bool(self.steady_state)
        ur = self.u_relaxation_factor if (steady and self.u_relaxation_factor is not None) else 0.0
        pr = self.p_relaxation_factor if (steady and self.p_relaxation_factor is not None) else 0.0
        ref = m.reference_pressure_cell_id
        return _lib.Params_t(nu, rho, float(ur), float(pr), float(self.dt), float(m.reference_pressure),
                             -1 if ref is None else int(ref), int(steady), int(self.NUM_INNER_LOOPS),
                             int(self.NUM_ORTHOGONAL_CORRECTORS), int(self.vel_equation.max_iter),
                             int(bool(m.skew_correction)), float(self.vel_equation.tol),
                             float(self.p_corr_equation.tol), int(self.p_refine), int(bool(self.rhie_chow)),
                             float(self.p_refine_rtol),
                             float(self.vel_equation.rtol), float(self.p_corr_equation.rtol), self._explicit_bits(),
                             self._convection_code())

    def _convection_code(self) -> int:
        scheme = self.convection.interpolation
        if scheme not in _lib.CONVECTION:
            raise NotImplementedError(f"convection interpolation {scheme!r} is not available on this path "
                                      "(upwind, upwindLinear, central difference)")
        return _lib.CONVECTION[scheme]

    def _explicit_bits(self) -> int:
        if not self.explicit_internal_terms:
            return 0
        bits = (1 if self.model.skew_correction else 0) | (4 if self.correction else 0)
        if self.convection.interpolation == "upwindLinear":
            bits |= 2
        return bits

    def _param_key(self):
        m = self.model
        return (self.material.density, self.material.viscosity, self.steady_state, self.u_relaxation_factor,
                self.p_relaxation_factor, self.dt, m.reference_pressure_cell_id, m.reference_pressure,
                self.NUM_INNER_LOOPS, self.NUM_ORTHOGONAL_CORRECTORS, self.vel_equation.max_iter,
                m.skew_correction, self.vel_equation.tol, self.p_corr_equation.tol, self._events_ptr,
                self.p_refine, self.p_refine_rtol, self.vel_equation.rtol, self.p_corr_equation.rtol, self.rhie_chow,
                self._explicit_bits(), self.convection.interpolation)

    def case_struct(self) -> _lib.Case_t:
        """The C struct of this case; rebuilt only when a parameter changed (the device
        arrays never move)."""
        key = self._param_key()
        if getattr(self, "_case_key", None) != key:
            self._case = self._build_case_struct()
            self._case_key = key
        return self._case

    def _build_case_struct(self) -> _lib.Case_t:
        m = self.model
        ve, pe = self.vel_equation, self.p_corr_equation
        if self.p_refine > 0 and self.p_x64 is None:
            self.p_x64 = pe.x.to(torch.float64)
            self.p_work = torch.zeros(2 * m.num_cells + 4, dtype=torch.float32, device=m.device)
        return _lib.Case_t(self._mesh_t, m.bc_struct(), m.state_struct(), ve.system_struct(), pe.system_struct(),
                           self.HbyA.data_ptr(), pe.x.data_ptr(), self.rUA.data_ptr(), self.rUA_faces.data_ptr(),
                           self.div_u.data_ptr(),
                           self.p_x64.data_ptr() if self.p_x64 is not None else None,
                           self.p_work.data_ptr() if self.p_work is not None else None,
                           ve.workspace_struct(), pe.workspace_struct(),
                           self.stats.data_ptr(), self.params(), self._events_ptr)

    # ------------------------------------------------------------------ checkpoint
    def state_tensors(self):
        """The device arrays that carry a case from one step to the next: the model's
        fields and mass fluxes, HbyA (momentum warm start), the pressure solution (warm
        start), rUA, rUA_f, the divergence and the fp64 pressure of the precision form.
        Everything else a step touches is rewritten before it is read."""
        m = self.model
        ts = [m.cell_values, m.cell_gradients, m.face_values, m.face_gradients, m.mass_fluxes, self.HbyA,
              self.p_corr_equation.x, self.rUA, self.rUA_faces, self.div_u]
        if self.p_x64 is not None:
            ts.append(self.p_x64)
        return ts

    def snapshot(self):
        """Device copies of the case state (resume with restore())."""
        return [t.clone() for t in self.state_tensors()]

    def restore(self, snap):
        """Put a snapshot() back; the next steps repeat the ones that followed it bit for bit."""
        ts = self.state_tensors()
        if len(ts) != len(snap):
            raise ValueError("snapshot does not match this case")
        for t, v in zip(ts, snap):
            t.copy_(v)

    # ------------------------------------------------------------------ stepping
    def step(self):
        """One SIMPLE outer iteration or one PISO time step on the current stream."""
        _lib.call("wcfd_simple_iteration", ct.byref(self.case_struct()), _stream())

    def assemble_momentum(self):
        """Momentum system from the current fields (incompressible.py:102-113) into
        vel_equation.diag/off/rhs, and rUA."""
        _lib.call("wcfd_assemble_momentum", ct.byref(self.case_struct()), _stream())

    def assemble_pressure(self):
        """Pressure system from rUA_faces and div_u (incompressible.py:134-140) into
        p_corr_equation.diag/off/rhs."""
        _lib.call("wcfd_assemble_pressure", ct.byref(self.case_struct()), _stream())

    def solve_stats(self):
        """(momentum, pressure) Krylov outcomes of the last step: iterations, status, residual."""
        raw = np.frombuffer(self.stats.cpu().numpy().tobytes(), dtype=STATS_DTYPE)
        return [dict(iterations=int(r["iterations"]), status=_lib.STATUS_NAMES.get(int(r["status"]), "?"),
                     residual=float(r["residual"]), initial_residual=float(r["initial_residual"]),
                     rhs_norm=float(r["rhs_norm"])) for r in raw]

    def momentum_residual_operator(self):
        return self.vel_equation.apply

    def run(self, steps_per_check=10, use_cuda_graph=False):
        """incompressible.py:72-172 (the convergence check never stops the loop, as there)."""
        nsteps = self.NUM_OUTER_LOOPS if self.steady_state else self.MAX_TIME_STEPS
        for nt in range(self.MAX_TIME_STEPS if not self.steady_state else 1):
            for n_outer in range(self.NUM_OUTER_LOOPS if self.steady_state else 1):
                if use_cuda_graph:
                    self._graph_step_counted()
                else:
                    self.step()
                steps = n_outer if self.steady_state else nt
                if steps_per_check and steps % steps_per_check == 0:
                    self.report(steps)
        if self.verbose:
            print(f"MAX ITERATIONS OF {nsteps} REACHED. Terminating")
        return self.report(nsteps)

    def _graph_step_counted(self):
        if self._graph is None or self._param_key() != self._graph_key:
            # first call captures; the capture itself does not execute, so run one eager step
            key = self._param_key()
            self.step()
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self.step()
            self._graph, self._graph_key = g, key
        else:
            self._graph.replay()

    def report(self, steps):
        ve = self.vel_equation
        st = self.solve_stats()
        # the norms of model.py:278-316 from the device convergence monitor (one fused pass)
        norms = self.model.convergence_norms(ve.system_struct(), self.HbyA, self.div_u, self.rUA,
                                             self.p_corr_equation.x)
        conv, converged = self.model.check_convergence_norms(norms)
        if self.verbose:
            print(f"step iter: {steps}")
            print(f"Outer loop Linear Solve {st[0]} Inner loop solve {st[1]}:")
            print({k: (v if isinstance(v, float) else (round(v[0], 9), v[1])) for k, v in conv.items()})
        return conv, converged
