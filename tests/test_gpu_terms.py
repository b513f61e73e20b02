"""The Term / Equation API forms the reference's weight arrays on the device.

ConvectionTerm (upwind, central difference, upwindLinear), DiffusionTerm (plain and
non-orthogonally corrected, scalar and per-face viscosity), DdtTerm and GradTerm are called
as the reference calls them (term(model, ...)) and their weights are compared entry by entry
with the oracle's restatement of warp_cfd/FV/terms/{convection,diffusion,ddt,grad}.py (the
(C, F, n, 3), (C, n, 2) and (3C,) layouts); Equation.form_system on any list of those terms
is compared with the oracle's assembly (equation.py:99-125) as matrices and right-hand sides.
"""
import numpy as np
import pytest
import torch

from tests.cases import (cavity3d_bc, cavity3d_mesh, cavity_bc, cavity_mesh, channel_bc, channel_mesh,
                         prism_cavity_mesh)
from tests.gpu_helpers import make_pair, rel_l2
from tests.test_gpu_parity import _seed_state

pytestmark = pytest.mark.gpu

CASES = {
    "cavity_skew": (lambda: cavity_mesh(10, jitter=0.15, seed=3), cavity_bc, 0, False),
    "cavity_corrected": (lambda: cavity_mesh(10, jitter=0.15, seed=3), cavity_bc, 0, True),
    "channel": (lambda: channel_mesh(20, 5), channel_bc, None, False),
    "prism_cavity": (lambda: prism_cavity_mesh(8, "mixed", jitter=0.1, seed=2), cavity_bc, 0, True),
    "cavity3d": (lambda: cavity3d_mesh(5, jitter=0.1, seed=4), cavity3d_bc, 0, False),
}


@pytest.fixture(scope="module", autouse=True)
def _lib_ready():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from warpcfd_gb300.build import build_library
    build_library()


def _prepared(case):
    mk, bc, ref, corr = CASES[case]
    m = mk()
    model, solver, oc = make_pair(m, bc, ref_cell=ref, correction=corr)
    _seed_state(model, oc, 11)
    model.set_boundary_conditions()
    model.face_interpolation()
    model.calculate_gradients()
    model.calculate_mass_flux()
    oc.apply_bc()
    oc.face_interpolation()
    oc.calculate_gradients()
    oc.calculate_mass_flux()
    return m, model, solver, oc, corr


def _close(got, ref, tol=1e-6):
    got = got.detach().cpu().numpy().astype(np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    assert got.shape == ref.shape
    # zero where the reference is zero, to rounding (no weight leaks into another slot or
    # field; a skew vector the oracle rounds to exactly 0 can be ~1e-8 on the device)
    assert np.all(np.abs(got[ref == 0]) <= 1e-6 * np.abs(ref).max())
    assert rel_l2(got, ref) <= tol, rel_l2(got, ref)


@pytest.mark.parametrize("case", list(CASES))
def test_term_weights_match_oracle(case):
    from warpcfd_gb300.FV.terms import ConvectionTerm, DdtTerm, DiffusionTerm, GradTerm

    m, model, solver, oc, corr = _prepared(case)
    vel = ["u", "v", "w"]
    for scheme in ("upwind", "central difference", "upwindLinear"):
        t = ConvectionTerm(model, vel, scheme)
        t(model)
        _close(t.weights, oc.convection_weights(scheme=scheme))
    d = DiffusionTerm(model, vel, correction=corr)
    d(model, viscosity=0.01)
    _close(d.weights, oc.diffusion_weights((0, 1, 2), 0.01))
    rua_f = np.random.default_rng(5).uniform(0.1, 1.0, size=m.num_faces).astype(np.float32)
    dp = DiffusionTerm(model, "p", correction=corr)
    dp(model, viscosity=torch.from_numpy(rua_f).cuda())
    _close(dp.weights, oc.diffusion_weights((3,), rua_f))
    t = DdtTerm(model, vel)
    t(model, dt=0.01)
    _close(t.weights, oc.ddt_weights(0.01))
    g = GradTerm(model, "p")
    g(model)
    _close(g.weights, oc.grad_term())


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("steady", [True, False])
def test_form_system_from_terms_matches_oracle_assembly(case, steady):
    from warpcfd_gb300.FV.terms import ConvectionTerm, DdtTerm, DiffusionTerm, Equation, GradTerm

    m, model, solver, oc, corr = _prepared(case)
    vel = ["u", "v", "w"]
    conv = ConvectionTerm(model, vel, "upwind")
    diff = DiffusionTerm(model, vel, correction=corr)
    grad = GradTerm(model, "p")
    conv(model)
    diff(model, viscosity=0.01)
    grad(model)
    eq = Equation(model, vel)
    wc = oc.convection_weights()
    wd = oc.diffusion_weights((0, 1, 2), 0.01)
    if steady:
        eq.form_system([conv, -diff], explicit_terms=-1.0 * grad)
        vals, rhs = oc.assemble(3, [(wc, 1.0), (wd, -1.0)], (), [(oc.grad_term(), -1.0)])
    else:
        ddt = DdtTerm(model, vel)
        ddt(model, dt=0.02)
        eq.form_system([ddt, conv, -diff], explicit_terms=-1.0 * grad)
        vals, rhs = oc.assemble(3, [(wc, 1.0), (wd, -1.0)], [(oc.ddt_weights(0.02), 1.0)], [(oc.grad_term(), -1.0)])
    assert rel_l2(eq.dense.cpu().numpy(), oc.momentum_matrix(vals).toarray()) < 1e-6
    assert rel_l2(eq.rhs.cpu().numpy(), rhs.reshape(-1)) < 1e-6
    # a scalar system: diffusion with a per-face coefficient, add_RHS, then form_system again
    # overwrites it (the reference resets the system first)
    rua_f = np.random.default_rng(6).uniform(0.1, 1.0, size=m.num_faces).astype(np.float32)
    pd = DiffusionTerm(model, "p", correction=corr)
    pd(model, viscosity=torch.from_numpy(rua_f).cuda())
    pe = Equation(model, "p", solver="cg")
    div = np.random.default_rng(7).standard_normal(m.num_cells).astype(np.float32)
    for _ in range(2):
        pe.form_system(pd)
        pe.add_RHS(torch.from_numpy(div).cuda())
    pv, prhs = oc.assemble(1, [(oc.diffusion_weights((3,), rua_f), 1.0)])
    prhs[:, 0] += div
    assert rel_l2(pe.dense.cpu().numpy(), oc.matrix(pv[0]).toarray()) < 1e-6
    assert rel_l2(pe.rhs.cpu().numpy(), prhs[:, 0]) < 1e-6


def test_form_system_requires_called_terms():
    from warpcfd_gb300.FV.terms import ConvectionTerm, Equation

    m, model, solver, oc, corr = _prepared("channel")
    eq = Equation(model, ["u", "v", "w"])
    with pytest.raises(ValueError, match="call the term"):
        eq.form_system([ConvectionTerm(model, ["u", "v", "w"])])
