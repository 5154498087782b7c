"""GMRES (plain FP64 and mixed-precision iterative refinement) and the scattered field of a
rigid sphere against the Mie series."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
K1 = 2 * np.pi * 1000 / 343.0


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_rigid_sphere_solve_and_mie(fm, oracle):
    """Plane wave exp(ikz) on the 1280-triangle sphere (r = 0.1 m, 1 kHz, 7-point rule)."""
    V, F = fm.icosphere(3, 0.1)
    plan = fm.Plan(V, F, k=K1, depth=3, p_levels={2: 8, 3: 8}, rule=fm.RULE_DUNAVANT7, a=0.5, b=0.0, c=-1.0)
    b = plan.plane_wave((0.0, 0.0, 1.0))
    C = np.array([V[f[0]] + (2.0 / 3.0) * (0.5 * (V[f[1]] + V[f[2]]) - V[f[0]]) for f in F])
    assert rel(b, np.exp(1j * K1 * C[:, 2])) < 1e-14
    x64, it64, rr64, ok64 = plan.gmres(b, tol=1e-6, restart=40, precision=fm.FMM_FP64)
    assert ok64 and rr64 <= 1e-6
    xm, itm, rrm, okm = plan.gmres(b, tol=1e-6, restart=40, precision=fm.FMM_MIXED)
    assert okm and rrm <= 1e-6
    assert rel(xm, x64) < 1e-5
    # residual of the FP64 solution through the oracle operator
    T = oracle.tree_for_fmm(V, F, depth=3)
    A = oracle.FMM(V, F, K1, T, [8, 8], a=0.5, b=0.0, c=-1.0, rule=1)
    assert rel(A.apply(x64), b) < 2e-6
    pts = fm.fibonacci_sphere(100, 1.0)
    ff = plan.far_field(x64, pts)
    assert rel(ff, oracle.far_field(V, F, K1, x64, pts, rule=1)) < 1e-12
    assert rel(ff, oracle.mie_rigid(K1, 0.1, pts)) < 0.02
    assert rel(plan.far_field(xm, pts), ff) < 1e-5
    plan.close()


def test_gmres_reports_non_convergence(fm):
    V, F = fm.icosphere(2, 0.1)
    plan = fm.Plan(V, F, k=K1, depth=2, p_levels={2: 6}, rule=1, a=0.5, b=0.0, c=-1.0)
    b = plan.plane_wave((1.0, 0.0, 0.0))
    x, it, rr, ok = plan.gmres(b, tol=1e-14, maxit=2, restart=2, precision=fm.FMM_FP64)
    assert not ok and it == 2 and rr > 1e-14
    plan.close()


def test_batched_solve_matches_single_solves(fm, oracle):
    """Four plane-wave directions solved at once (lockstep GMRES, batched matvecs) against one
    solve per direction; the z-direction far field against the Mie series."""
    V, F = fm.icosphere(3, 0.1)
    plan = fm.Plan(V, F, k=K1, depth=3, p_levels={2: 8, 3: 8}, rule=fm.RULE_DUNAVANT7, a=0.5, b=0.0, c=-1.0)
    dirs = [(0.0, 0.0, 1.0), (1.0, 0.0, 0.0), (0.0, 0.6, 0.8), (-0.48, 0.6, 0.64)]
    B = np.stack([plan.plane_wave(d) for d in dirs])
    pts = fm.fibonacci_sphere(100, 1.0)
    for prec in (fm.FMM_FP64, fm.FMM_MIXED):
        X, it, rr, ok = plan.solve_batched(B, tol=1e-6, restart=40, precision=prec)
        assert ok and (rr <= 1e-6).all() and (it > 0).all()
        for r in range(len(dirs)):
            xs, _, rrs, oks = plan.gmres(B[r], tol=1e-6, restart=40, precision=prec)
            assert oks and rel(X[r], xs) < 2e-5
        assert rel(plan.far_field(X[0], pts), oracle.mie_rigid(K1, 0.1, pts)) < 0.02
    # a column that starts at its solution stops at once while the others iterate
    X0 = np.zeros_like(B)
    X0[2] = X[2]
    X, it, rr, ok = plan.solve_batched(B, X0=X0, tol=1e-5, restart=40, precision=fm.FMM_FP64)
    assert ok and it[2] == 0 and (it[[0, 1, 3]] > 0).all()
    plan.close()
