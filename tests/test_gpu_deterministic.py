"""Deterministic mixed path (fmm_options.deterministic): the FP32 translations owner-computed
(each destination box accumulates its translations in one CTA, no atomics), so mixed results
repeat bit for bit, on plain and degree-scaled (low-frequency) plans, for several right-hand
sides and through a refined solve."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
K1 = 2 * np.pi * 1000 / 343.0
K2 = 2 * np.pi * 8000 / 343.0


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("k,p", [(K2, {2: 16, 3: 12}), (K1, {2: 16, 3: 16})])
def test_deterministic_mixed_repeats_bit_for_bit(fm, oracle, k, p):
    V, F = fm.icosphere(3, 0.1)
    kw = dict(k=k, depth=3, p_levels=p, rule=1, a=0.5, b=0.3 + 0.1j, c=-1.0)
    plan = fm.Plan(V, F, deterministic=True, **kw)
    rng = np.random.default_rng(31)
    x = rng.standard_normal(plan.nf) + 1j * rng.standard_normal(plan.nf)
    y1 = plan.matvec(x, fm.FMM_MIXED)
    y2 = plan.matvec(x, fm.FMM_MIXED)
    assert np.array_equal(y1, y2)
    y64 = plan.matvec(x, fm.FMM_FP64)
    assert rel(y1, y64) < 1e-5
    T = oracle.tree_for_fmm(V, F, depth=3)
    yo = oracle.FMM(V, F, k, T, [p[2], p[3]], a=0.5, b=0.3 + 0.1j, c=-1.0, rule=1).apply(x)
    assert rel(y1, yo) < 1e-5
    # columns of one call equal their single-column results bit for bit
    X = np.stack([x, 1j * x, rng.standard_normal(plan.nf) + 0j])
    Y = plan.matvec(X.reshape(-1), fm.FMM_MIXED).reshape(3, -1)
    assert np.array_equal(Y[0], y1)
    for r in range(3):
        assert np.array_equal(Y[r], plan.matvec(X[r], fm.FMM_MIXED))
    # the transposed operator too
    assert np.array_equal(plan.matvec_adjoint(x, fm.FMM_MIXED), plan.matvec_adjoint(x, fm.FMM_MIXED))
    plan.close()


def test_deterministic_refined_solve_repeats(fm):
    V, F = fm.icosphere(4, 0.1)
    plan = fm.Plan(V, F, k=K2, depth=4, p_levels={2: 16, 3: 14, 4: 10}, rule=1, a=0.5, b=0.0, c=-1.0, deterministic=True)
    b = plan.plane_wave()
    x1, it1, rr1, ok1 = plan.gmres(b, tol=1e-8, maxit=800, restart=60, precision=fm.FMM_MIXED)
    x2, it2, rr2, ok2 = plan.gmres(b, tol=1e-8, maxit=800, restart=60, precision=fm.FMM_MIXED)
    assert ok1 and ok2 and it1 == it2 and rr1 == rr2
    assert np.array_equal(x1, x2)
    x64, _, _, ok64 = plan.gmres(b, tol=1e-8, maxit=800, restart=60, precision=fm.FMM_FP64)
    assert ok64 and rel(x1, x64) < 1e-6
    plan.close()
