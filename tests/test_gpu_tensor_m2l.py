"""The dense tensor-core passes (tcgen05, split TF32) of the mixed path: the M2L with one operator
per class of directions with equal polar angle and distance (azimuthal phases applied per row),
and the M2M / L2L with one operator per octant, forced on (FMMBEM_TENSOR_M2L=1,
FMMBEM_TENSOR_M2M=1), against the FP64 matvec, the SIMT tiles and the oracle,
for even and odd orders, one and several right-hand sides, and the Burton-Miller operator."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
K1 = 2 * np.pi * 1000 / 343.0
K2 = 2 * np.pi * 8000 / 343.0


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def make_plan(fm, mode, *args, **kw):
    """The dense tensor-core passes (M2L, M2M and L2L) forced off ("0") or on ("1"), the
    three-stage form off."""
    env = {"FMMBEM_TENSOR_M2L": mode, "FMMBEM_TENSOR_M2M": mode, "FMMBEM_TC3": "0"}
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        return fm.Plan(*args, **kw)
    finally:
        for k, v in old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v


# (p = 16 at 1 kHz would leave the FP32 range in the coaxial tables: no mixed path there)
@pytest.mark.parametrize("p,k", [(8, K1), (9, K1), (13, K1), (16, K2)])
def test_tensor_m2l_matches_fp64_and_oracle(fm, oracle, p, k):
    V, F = fm.icosphere(3, 0.1)
    kw = dict(k=k, depth=3, p_levels={2: p, 3: p}, rule=1, a=0.5, b=0.0, c=-1.0)
    plan = make_plan(fm, "1", V, F, **kw)
    assert all(plan.info.m2l_tensor[l] == 1 for l in (2, 3))
    assert [plan.info.pass_dense[l] for l in (2, 3)] == [2, 7]
    simt = make_plan(fm, "0", V, F, **kw)
    assert not any(simt.info.m2l_tensor[l] for l in range(13))
    assert not any(simt.info.pass_dense[l] for l in range(13))
    rng = np.random.default_rng(p)
    x = rng.standard_normal(plan.nf) + 1j * rng.standard_normal(plan.nf)
    y64 = plan.matvec(x, fm.FMM_FP64)
    ym = plan.matvec(x, fm.FMM_MIXED)
    assert rel(ym, y64) < 1e-5
    assert rel(ym, simt.matvec(x, fm.FMM_MIXED)) < 1e-5
    T = oracle.tree_for_fmm(V, F, depth=3)
    assert rel(ym, oracle.FMM(V, F, k, T, [p, p], a=0.5, b=0.0, c=-1.0, rule=1).apply(x)) < 1e-5
    # several right-hand sides in one pass, and the captured graph on the repeat
    X = np.stack([x, 1j * x, rng.standard_normal(plan.nf) + 0j])
    for _ in range(3):
        Y = plan.matvec(X.reshape(-1), fm.FMM_MIXED).reshape(3, -1)
        for r in range(3):
            assert rel(Y[r], plan.matvec(X[r], fm.FMM_FP64)) < 1e-5
    plan.close()
    simt.close()


def test_tensor_m2l_on_the_81920_triangle_workload(fm):
    """Orders 40/30/20/14/10: the levels with p <= 16 (14 and 10) on the tensor cores."""
    V, F = fm.icosphere(6, 0.3)
    P2 = {2: 40, 3: 30, 4: 20, 5: 14, 6: 10}
    plan = make_plan(fm, "1", V, F, k=K2, depth=6, p_levels=P2, rule=0, a=0.5, b=0.0, c=-1.0)
    assert [plan.info.m2l_tensor[l] for l in range(2, 7)] == [0, 0, 0, 1, 1]
    # M2M out of / L2L into level 6 (orders 10 and 14) run dense too; level 5's parent has p = 20
    assert [plan.info.pass_dense[l] for l in range(2, 7)] == [0, 0, 0, 2, 7]
    rng = np.random.default_rng(0)
    x = rng.standard_normal(plan.nf) + 1j * rng.standard_normal(plan.nf)
    y64 = plan.matvec(x, fm.FMM_FP64)
    assert rel(plan.matvec(x, fm.FMM_MIXED), y64) < 1e-6
    xs, it, rr, ok = plan.gmres(plan.plane_wave(), tol=1e-6, maxit=500, restart=60, precision=fm.FMM_MIXED)
    assert ok
    plan.close()


def test_tensor_m2l_with_burton_miller(fm, oracle):
    V, F = fm.icosphere(3, 0.1)
    alpha = 1j / K1
    kw = dict(k=K1, depth=3, p_levels={2: 10, 3: 10}, rule=1, a=0.5, b=0.0, c=-1.0, alpha=alpha)
    plan = make_plan(fm, "1", V, F, **kw)
    rng = np.random.default_rng(5)
    x = rng.standard_normal(plan.nf) + 1j * rng.standard_normal(plan.nf)
    T = oracle.tree_for_fmm(V, F, depth=3)
    yo = oracle.FMM(V, F, K1, T, [10, 10], a=0.5, b=0.0, c=-1.0, rule=1, alpha=alpha).apply(x)
    assert rel(plan.matvec(x, fm.FMM_MIXED), yo) < 1e-5
    plan.close()


def test_tensor_m2l_in_the_transposed_operator(fm, oracle):
    """The transposed matvec reuses the M2L lists and operators, so its mixed path runs on the
    tensor cores too."""
    V, F = fm.icosphere(3, 0.1)
    kw = dict(k=K1, depth=3, p_levels={2: 10, 3: 10}, rule=0, a=0.3, b=0.7 + 0.2j, c=-1.0)
    plan = make_plan(fm, "1", V, F, **kw)
    rng = np.random.default_rng(9)
    y = rng.standard_normal(plan.nf) + 1j * rng.standard_normal(plan.nf)
    at64 = plan.matvec_adjoint(y, fm.FMM_FP64)
    assert rel(plan.matvec_adjoint(y, fm.FMM_MIXED), at64) < 1e-5
    assert rel(plan.matvec_adjoint(y, fm.FMM_MIXED, conjugate=True), plan.matvec_adjoint(y, fm.FMM_FP64, conjugate=True)) < 1e-5
    T = oracle.tree_for_fmm(V, F, depth=3)
    orc = oracle.FMM(V, F, K1, T, [10, 10], a=0.3, b=0.7 + 0.2j, c=-1.0, rule=0)
    assert rel(at64, orc.apply(y, transpose=True)) < 1e-10
    plan.close()


def test_many_columns_with_morton_ranges_and_resident_operator(fm):
    """16 columns on the 81,920-triangle sphere with p = 8 at the leaves: the expansions of the
    deep levels exceed the L2 budget, so the items run in Morton ranges of the destinations, and
    the p = 8 tensor-core level keeps its operator resident.  Every column against its own
    single-column matvec and two against FP64."""
    V, F = fm.icosphere(6, 0.3)
    P2 = {2: 30, 3: 20, 4: 14, 5: 10, 6: 8}
    plan = make_plan(fm, "1", V, F, k=K2, depth=6, p_levels=P2, rule=0, a=0.5, b=0.0, c=-1.0)
    assert plan.info.m2l_tensor[6] == 1
    rng = np.random.default_rng(16)
    X = rng.standard_normal((16, plan.nf)) + 1j * rng.standard_normal((16, plan.nf))
    Y = plan.matvec(X.reshape(-1), fm.FMM_MIXED).reshape(16, -1)
    for r in range(16):
        assert rel(Y[r], plan.matvec(X[r], fm.FMM_MIXED)) < 1e-6, r
    for r in (0, 15):
        assert rel(Y[r], plan.matvec(X[r], fm.FMM_FP64)) < 1e-5, r
    plan.close()


def test_bounded_wait_gives_up_and_leaves_the_context_usable(fm):
    """Failure detection without a fault: the barrier wait the tensor-core M2L uses gives up
    after its limit on a barrier nothing completes, reports it, and the GPU goes on working."""
    gave_up, completed = fm.selftest_bounded_wait(0)
    assert gave_up and completed
    V, F = fm.icosphere(3, 0.1)
    plan = make_plan(fm, "1", V, F, k=K1, depth=3, p_levels={2: 8, 3: 8}, rule=1, a=0.5, b=0.0, c=-1.0)
    x = np.random.default_rng(3).standard_normal(plan.nf) + 0j
    assert rel(plan.matvec(x, fm.FMM_MIXED), plan.matvec(x, fm.FMM_FP64)) < 1e-5
    plan.close()
