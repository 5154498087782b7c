"""FMM_FLOAT2: the FP64 matvec with its M2L (and the L2L fused into it) in float-float
arithmetic on the FP32 pipes, which the mixed solvers use for their residuals.  Against the
plain FP64 matvec and the FP64 oracle, the transposed operator, Burton-Miller, a low-frequency
plan (degree-scaled tables and expansions) and the refined solve."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
K1 = 2 * np.pi * 1000 / 343.0
K2 = 2 * np.pi * 8000 / 343.0


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_float2_matches_fp64_and_oracle(fm, oracle):
    V, F = fm.icosphere(3, 0.1)
    kw = dict(k=K2, depth=3, p_levels={2: 16, 3: 12}, rule=1, a=0.5, b=0.3 + 0.1j, c=-1.0)
    plan = fm.Plan(V, F, **kw)
    rng = np.random.default_rng(21)
    x = rng.standard_normal(plan.nf) + 1j * rng.standard_normal(plan.nf)
    y64 = plan.matvec(x, fm.FMM_FP64)
    yff = plan.matvec(x, fm.FMM_FLOAT2)
    assert rel(yff, y64) < 1e-11
    T = oracle.tree_for_fmm(V, F, depth=3)
    yo = oracle.FMM(V, F, K2, T, [16, 12], a=0.5, b=0.3 + 0.1j, c=-1.0, rule=1).apply(x)
    assert rel(yff, yo) < 1e-10
    # the transposed operator runs the same translations
    assert rel(plan.matvec_adjoint(x, fm.FMM_FLOAT2), plan.matvec_adjoint(x, fm.FMM_FP64)) < 1e-11
    plan.close()


def test_float2_on_the_81920_triangle_workload(fm):
    """Every level, including the split FP64 M2L of the 56-box level 2 (partial sums added in
    float-float too)."""
    V, F = fm.icosphere(6, 0.3)
    plan = fm.Plan(V, F, k=K2, depth=6, p_levels={2: 40, 3: 30, 4: 20, 5: 14, 6: 10}, rule=0, a=0.5, b=0.0, c=-1.0)
    rng = np.random.default_rng(22)
    x = rng.standard_normal(plan.nf) + 1j * rng.standard_normal(plan.nf)
    assert rel(plan.matvec(x, fm.FMM_FLOAT2), plan.matvec(x, fm.FMM_FP64)) < 1e-11
    plan.close()


def test_float2_with_burton_miller(fm):
    V, F = fm.icosphere(3, 0.1)
    plan = fm.Plan(V, F, k=K2, depth=3, p_levels={2: 14, 3: 10}, rule=1, a=0.5, b=0.0, c=-1.0, alpha=1j / K2)
    x = np.random.default_rng(23).standard_normal(plan.nf) + 0j
    assert rel(plan.matvec(x, fm.FMM_FLOAT2), plan.matvec(x, fm.FMM_FP64)) < 1e-11
    plan.close()


def test_float2_at_low_frequency_with_scaled_expansions(fm, oracle):
    """p = 16 at 1 kHz: the coaxial (S|R) entries leave the FP32 range, so the float-float
    translations run on degree-scaled tables and expansions, as the mixed path does."""
    V, F = fm.icosphere(3, 0.1)
    plan = fm.Plan(V, F, k=K1, depth=3, p_levels={2: 16, 3: 16}, rule=1, a=0.5, b=0.0, c=-1.0)
    assert plan.info.expansions_scaled == 1
    x = np.random.default_rng(24).standard_normal(plan.nf) + 1j * np.random.default_rng(25).standard_normal(plan.nf)
    yff = plan.matvec(x, fm.FMM_FLOAT2)
    assert np.isfinite(yff).all()
    assert rel(yff, plan.matvec(x, fm.FMM_FP64)) < 1e-11
    assert rel(plan.matvec_adjoint(x, fm.FMM_FLOAT2), plan.matvec_adjoint(x, fm.FMM_FP64)) < 1e-11
    T = oracle.tree_for_fmm(V, F, depth=3)
    assert rel(yff, oracle.FMM(V, F, K1, T, [16, 16], a=0.5, b=0.0, c=-1.0, rule=1).apply(x)) < 1e-10
    plan.close()


def test_refined_solve_with_float_float_residuals(fm):
    """The mixed solve (float-float residuals by default) reaches the same solution as with
    plain FP64 residuals (FMMBEM_FF_RESIDUAL=0) and as plain FP64 GMRES."""
    V, F = fm.icosphere(4, 0.1)
    plan = fm.Plan(V, F, k=K2, depth=4, p_levels={2: 16, 3: 14, 4: 10}, rule=1, a=0.5, b=0.0, c=-1.0)
    b = plan.plane_wave()
    x_ff, it, rr, ok = plan.gmres(b, tol=1e-9, maxit=800, restart=60, precision=fm.FMM_MIXED)
    assert ok and rr < 1e-9
    old = os.environ.get("FMMBEM_FF_RESIDUAL")
    os.environ["FMMBEM_FF_RESIDUAL"] = "0"
    try:
        x_64, it64, rr64, ok64 = plan.gmres(b, tol=1e-9, maxit=800, restart=60, precision=fm.FMM_MIXED)
    finally:
        if old is None:
            del os.environ["FMMBEM_FF_RESIDUAL"]
        else:
            os.environ["FMMBEM_FF_RESIDUAL"] = old
    assert ok64
    x_p, _, _, okp = plan.gmres(b, tol=1e-9, maxit=800, restart=60, precision=fm.FMM_FP64)
    assert okp
    assert rel(x_ff, x_p) < 1e-8 and rel(x_64, x_p) < 1e-8
    # the residual it reports is the FP64 one
    r = b - plan.matvec(x_ff, fm.FMM_FP64)
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1.01e-9
    plan.close()


def test_plain_gmres_on_the_float_float_matvec(fm):
    """fmm_gmres with FMM_FLOAT2: plain GMRES on the FP64-quality matvec reaches the plain FP64
    solution, and its reported residual is the true one."""
    V, F = fm.icosphere(4, 0.1)
    plan = fm.Plan(V, F, k=K2, depth=4, p_levels={2: 16, 3: 14, 4: 10}, rule=1, a=0.5, b=0.0, c=-1.0)
    b = plan.plane_wave()
    x2, it2, rr2, ok2 = plan.gmres(b, tol=1e-10, maxit=800, restart=60, precision=fm.FMM_FLOAT2)
    x64, it64, rr64, ok64 = plan.gmres(b, tol=1e-10, maxit=800, restart=60, precision=fm.FMM_FP64)
    assert ok2 and ok64
    assert abs(it2 - it64) <= 2
    assert rel(x2, x64) < 1e-9
    r = b - plan.matvec(x2, fm.FMM_FP64)
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1.01e-10
    plan.close()
