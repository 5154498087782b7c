"""Transposed and adjoint matvecs (fmm_matvec_adjoint) against the oracle's transposed FMM,
the dense transpose, and the bilinear identity y^T (A x) = x^T (A^T y)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
K1 = 2 * np.pi * 1000 / 343.0
K2 = 2 * np.pi * 8000 / 343.0
P2 = {2: 40, 3: 30, 4: 20, 5: 14, 6: 10}


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("abc,rule", [((0.5, 0.0, -1.0), 0), ((0.3, 0.7 + 0.2j, -1.0), 1)])
def test_transpose_matches_oracle_and_dense(fm, oracle, abc, rule):
    V, F = fm.icosphere(3, 0.1)
    a, b, c = abc
    plan = fm.Plan(V, F, k=K1, depth=3, p_levels={2: 8, 3: 8}, rule=rule, a=a, b=b, c=c)
    rng = np.random.default_rng(3)
    n = plan.nf
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    y = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    T = oracle.tree_for_fmm(V, F, depth=3)
    orc = oracle.FMM(V, F, K1, T, [8, 8], a=a, b=b, c=c, rule=rule)
    aty = plan.matvec_adjoint(y, fm.FMM_FP64)
    assert rel(aty, orc.apply(y, transpose=True)) < 1e-10
    # against the dense operator, to the accuracy of the forward FMM at the same orders
    A = oracle.dense_matrix(V, F, K1, a=a, b=b, c=c, rule=rule)
    fwd = rel(plan.matvec(x, fm.FMM_FP64), A @ x)
    assert rel(aty, A.T @ y) < max(3 * fwd, 1e-8)
    ahy = plan.matvec_adjoint(y, fm.FMM_FP64, conjugate=True)
    assert rel(ahy, A.conj().T @ y) < max(3 * fwd, 1e-8)
    # bilinear identity of the two FMM operators
    ax = plan.matvec(x, fm.FMM_FP64)
    scale = np.linalg.norm(x) * np.linalg.norm(y) * np.linalg.norm(A, 2)
    assert abs(y @ ax - x @ aty) < 1e-9 * scale
    # mixed precision
    assert rel(plan.matvec_adjoint(y, fm.FMM_MIXED), aty) < 1e-5
    assert rel(plan.matvec_adjoint(y, fm.FMM_MIXED, conjugate=True), ahy) < 1e-5
    plan.close()


def test_adjoint_full_size_device_buffers_and_nrhs(fm):
    """The 81,920-triangle workload: device and host buffers, two right-hand sides at once,
    the bilinear identity, and A^H x = conj(A^T conj(x))."""
    import torch

    V, F = fm.icosphere(6, 0.3)
    plan = fm.Plan(V, F, k=K2, depth=6, p_levels=P2, rule=0, a=0.5, b=0.0, c=-1.0)
    n = plan.nf
    rng = np.random.default_rng(4)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    y2 = rng.standard_normal(2 * n) + 1j * rng.standard_normal(2 * n)
    at2 = plan.matvec_adjoint(torch.from_numpy(y2).cuda(), fm.FMM_FP64).cpu().numpy()
    at_host = plan.matvec_adjoint(y2[:n], fm.FMM_FP64)
    assert np.array_equal(at2[:n], at_host)
    assert rel(at2[n:], plan.matvec_adjoint(y2[n:], fm.FMM_FP64)) < 1e-14
    ax = plan.matvec(x, fm.FMM_FP64)
    lhs, r = y2[:n] @ ax, x @ at_host
    assert abs(lhs - r) < 1e-7 * np.linalg.norm(x) * np.linalg.norm(y2[:n])
    ah = plan.matvec_adjoint(y2[:n], fm.FMM_FP64, conjugate=True)
    assert rel(ah, np.conj(plan.matvec_adjoint(np.conj(y2[:n]), fm.FMM_FP64))) < 1e-14
    assert rel(plan.matvec_adjoint(y2[:n], fm.FMM_MIXED), at_host) < 1e-5
    plan.close()
