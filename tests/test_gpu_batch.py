"""Batched form: each case gives the same result alone and in the mix.

* in the mix vs alone in a batch of one with the same cluster size: bitwise equal (every
  case's kernels and its cluster's reductions do not depend on the other cases);
* in the mix vs the single-case drop-in path (grid/cluster Krylov kernels with their own
  partition): within the step-parity tolerances of test_gpu_parity.py, with the same
  Krylov iteration counts (+-2).
"""
import numpy as np
import pytest
import torch

from tests.cases import cavity3d_bc, cavity3d_mesh, cavity_bc, cavity_mesh, channel_bc, channel_mesh
from tests.gpu_helpers import fields, make_pair, rel_l2, vel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib_ready():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from warpcfd_gb300.build import build_library
    build_library()


def _cases():
    specs = [(lambda: cavity_mesh(16), cavity_bc, 0, 0.01),
             (lambda: cavity_mesh(24, jitter=0.1, seed=2), cavity_bc, 0, 0.005),
             (lambda: channel_mesh(40, 8), channel_bc, None, 0.05),
             (lambda: cavity_mesh(32), cavity_bc, 0, 0.002)]
    out = []
    for mk, bc, ref, nu in specs:
        model, solver, _ = make_pair(mk(), bc, ref_cell=ref, nu=nu)
        out.append((model, solver))
    return out


def test_mix_equals_alone_and_drop_in():
    from warpcfd_gb300.batch import CaseBatch

    steps = 5
    mix = _cases()
    batch = CaseBatch([s for _, s in mix])
    cs = batch.cluster_size
    assert cs >= 1
    for _ in range(steps):
        batch.step()
    got = [fields(m) for m, _ in mix]
    st_mix = batch.solve_stats()
    for i, (mk_model, mk_solver) in enumerate(_cases()):
        alone = CaseBatch([mk_solver], cluster_size=cs)
        for _ in range(steps):
            alone.step()
        assert np.array_equal(fields(mk_model), got[i]), i
    for i, (model, solver) in enumerate(_cases()):
        for _ in range(steps):
            solver.step()
        ref = fields(model)
        for o in range(3):
            assert vel_err(got[i], ref, o) < 1e-4, (i, o)
        assert rel_l2(got[i][:, 3], ref[:, 3]) < 1e-3, i
        st = solver.solve_stats()
        assert abs(st[1]["iterations"] - int(st_mix[i, 1]["iterations"])) <= 2, i
    res = batch.relative_residuals()
    assert np.all(np.isfinite(res)) and np.all(res > 0)


def test_batch_rejects_mixed_widths():
    from warpcfd_gb300.batch import CaseBatch

    m2, s2, _ = make_pair(cavity_mesh(8), cavity_bc)
    m3, s3, _ = make_pair(cavity3d_mesh(4), cavity3d_bc)
    with pytest.raises(ValueError):
        CaseBatch([s2, s3])


def test_graph_replay_field_block_and_autotune_keep_results():
    """CaseBatch.steps (a captured CUDA graph of n batched steps), any field block size and
    the autotuner's timed trial steps leave every case's result bit for bit as eager
    steps at the default block size give it."""
    from warpcfd_gb300.autotune import tune_field_block
    from warpcfd_gb300.batch import CaseBatch

    ref = _cases()
    b_ref = CaseBatch([s for _, s in ref])
    for _ in range(6):
        b_ref.step()
    want = [fields(m) for m, _ in ref]

    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        graphed = _cases()
        b = CaseBatch([s for _, s in graphed], field_block=128)
        b.steps(3)
        b.steps(3)  # replays the graph captured by the first call
    torch.cuda.current_stream().wait_stream(side)
    for i, (m, _) in enumerate(graphed):
        assert np.array_equal(fields(m), want[i]), i

    tuned = _cases()
    b2 = CaseBatch([s for _, s in tuned])
    fb = tune_field_block(b2, key=("test", 1))
    assert fb in (128, 256, 512) and b2.field_block == fb
    for _ in range(6):
        b2.step()
    for i, (m, _) in enumerate(tuned):
        assert np.array_equal(fields(m), want[i]), i


def test_batch_with_explicit_terms_matches_alone():
    """A batch whose cases use the opt-in explicit internal terms (the assembly kernels with
    those terms compiled in): each case equals itself alone in a batch of one, bit for bit,
    and differs from the same case without the option."""
    from warpcfd_gb300.batch import CaseBatch

    def make(xt):
        m1, s1, _ = make_pair(cavity_mesh(16, jitter=0.15, seed=11), cavity_bc, correction=True)
        m2, s2, _ = make_pair(cavity_mesh(12, jitter=0.1, seed=3), cavity_bc, correction=True)
        for s in (s1, s2):
            s.explicit_internal_terms = xt
        return [(m1, s1), (m2, s2)]

    mix = make(True)
    batch = CaseBatch([s for _, s in mix])
    assert batch.dims.explicit_terms == 5
    for _ in range(4):
        batch.step()
    got = [fields(m) for m, _ in mix]
    for i, (m, s) in enumerate(make(True)):
        alone = CaseBatch([s], cluster_size=batch.cluster_size)
        for _ in range(4):
            alone.step()
        assert np.array_equal(fields(m), got[i]), i
    plain = make(False)
    pb = CaseBatch([s for _, s in plain], cluster_size=batch.cluster_size)
    assert pb.dims.explicit_terms == 0
    for _ in range(4):
        pb.step()
    assert not np.array_equal(fields(plain[0][0]), got[0])


def test_batched_refined_pressure_equals_alone_and_tracks_drop_in():
    """The batched form's fp64-refined pressure solve (two sweeps per corrector): a case in
    the mix equals the same case alone (bitwise, same cluster size), and follows the
    drop-in's refined solve (wcfd_cg_refine, the drop-in's own Krylov partition) within the
    step tolerances."""
    from warpcfd_gb300.batch import CaseBatch

    def cases():
        out = []
        for mk, bc, ref, nu in ((lambda: cavity_mesh(16), cavity_bc, 0, 0.01),
                                (lambda: channel_mesh(40, 8), channel_bc, None, 0.05),
                                (lambda: cavity_mesh(24, jitter=0.1, seed=2), cavity_bc, 0, 0.005)):
            model, solver, _ = make_pair(mk(), bc, ref_cell=ref, nu=nu, atol=1e-7)
            solver.p_refine = 2
            solver.p_refine_rtol = 1e-2
            out.append((model, solver))
        return out

    steps = 4
    mix = cases()
    batch = CaseBatch([s for _, s in mix])
    assert batch.dims.p_refine == 2
    cs = batch.cluster_size
    for _ in range(steps):
        batch.step()
    got = [fields(m) for m, _ in mix]
    assert all(np.isfinite(g).all() for g in got)
    for i, (model, solver) in enumerate(cases()):
        alone = CaseBatch([solver], cluster_size=cs)
        for _ in range(steps):
            alone.step()
        assert np.array_equal(fields(model), got[i]), i
    for i, (model, solver) in enumerate(cases()):
        for _ in range(steps):
            solver.step()
        ref = fields(model)
        for o in range(3):
            assert vel_err(got[i], ref, o) < 1e-4, (i, o)
        assert rel_l2(got[i][:, 3], ref[:, 3]) < 1e-3, i


def test_batch_rejects_mixed_refinement_counts():
    from warpcfd_gb300.batch import CaseBatch

    (m0, s0), (m1, s1) = [make_pair(cavity_mesh(8), cavity_bc)[:2] for _ in range(2)]
    s1.p_refine = 1
    with pytest.raises(ValueError, match="refinement"):
        CaseBatch([s0, s1])


@pytest.mark.parametrize("cluster_size", [1, 4])
def test_single_reduction_cg_tracks_textbook(cluster_size):
    """The batched single-reduction CG (wcfd_batch_dims.cg_variant = 1: one cluster
    all-reduce and one cluster barrier per iteration) follows the textbook batched CG
    within the step tolerances, with 1, 2 and 4 rows per thread (a 64^2 cavity on one CTA
    holds 4,096 rows) and, on 4-CTA clusters, neighbours in other CTAs; a case in the mix
    equals the same case alone bitwise."""
    from warpcfd_gb300.batch import CaseBatch

    def cases():
        out = []
        for mk, bc, ref, nu in ((lambda: cavity_mesh(16), cavity_bc, 0, 0.01),
                                (lambda: channel_mesh(80, 16), channel_bc, None, 0.05),
                                (lambda: cavity_mesh(64), cavity_bc, 0, 0.01)):
            model, solver, _ = make_pair(mk(), bc, ref_cell=ref, nu=nu, atol=1e-7)
            out.append((model, solver))
        return out

    steps = 4
    runs = {}
    for variant in (0, 1):
        mix = cases()
        batch = CaseBatch([s for _, s in mix], cluster_size=cluster_size, cg_variant=variant)
        assert batch.dims.cg_variant == variant
        for _ in range(steps):
            batch.step()
        runs[variant] = ([fields(m) for m, _ in mix], batch.solve_stats())
    got, st1 = runs[1]
    ref, st0 = runs[0]
    for i in range(3):
        assert np.isfinite(got[i]).all(), i
        for o in range(3):
            assert vel_err(got[i], ref[i], o) < 1e-4, (i, o)
        assert rel_l2(got[i][:, 3], ref[i][:, 3]) < 1e-3, i
        k0, k1 = int(st0[i, 1]["iterations"]), int(st1[i, 1]["iterations"])
        assert abs(k1 - k0) <= max(2, k0 // 20), (i, k0, k1)
    model, solver = cases()[2]
    alone = CaseBatch([solver], cluster_size=cluster_size, cg_variant=1)
    for _ in range(steps):
        alone.step()
    assert np.array_equal(fields(model), got[2])
