"""The mixed path where plain FP32 tables would not do: low k t, where the coaxial (S|R)
entries leave the float range and the FP32 expansions are kept scaled by degree, and
truncation orders above 42, where the translation tiles take 4 columns."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
K1 = 2 * np.pi * 1000 / 343.0


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


@pytest.mark.parametrize("tensor", ["0", "1"])
def test_low_frequency_scaled_expansions(fm, oracle, tensor):
    """p = 16 at 1 kHz on the 1,280-triangle sphere: (S|R) entries near 1e40 at level 3."""
    V, F = fm.icosphere(3, 0.1)
    kw = dict(k=K1, depth=3, p_levels={2: 16, 3: 16}, rule=1, a=0.3, b=0.7 + 0.2j, c=-1.0)
    plan = make_plan(fm, tensor, V, F, **kw)
    info = plan.info
    assert info.expansions_scaled == 1
    assert info.m2l_columns[2] > 0 and info.m2l_columns[3] > 0
    assert [info.m2l_tensor[l] for l in (2, 3)] == ([1, 1] if tensor == "1" else [0, 0])
    rng = np.random.default_rng(11)
    x = rng.standard_normal(plan.nf) + 1j * rng.standard_normal(plan.nf)
    y64 = plan.matvec(x, fm.FMM_FP64)
    ym = plan.matvec(x, fm.FMM_MIXED)
    assert np.isfinite(ym).all()
    assert rel(ym, y64) < 1e-5
    T = oracle.tree_for_fmm(V, F, depth=3)
    assert rel(ym, oracle.FMM(V, F, K1, T, [16, 16], a=0.3, b=0.7 + 0.2j, c=-1.0, rule=1).apply(x)) < 1e-5
    # several columns, and the transposed operator (same scaled tables)
    X = np.stack([x, 1j * x, rng.standard_normal(plan.nf) + 0j])
    Y = plan.matvec(X.reshape(-1), fm.FMM_MIXED).reshape(3, -1)
    for r in range(3):
        assert rel(Y[r], plan.matvec(X[r], fm.FMM_FP64)) < 1e-5
    assert rel(plan.matvec_adjoint(x, fm.FMM_MIXED), plan.matvec_adjoint(x, fm.FMM_FP64)) < 1e-5
    # the refined solve reaches the FP64 solution
    b = plan.plane_wave()
    xm, it, rr, ok = plan.gmres(b, tol=1e-8, maxit=500, restart=60, precision=fm.FMM_MIXED)
    assert ok
    x64, _, _, ok64 = plan.gmres(b, tol=1e-8, maxit=500, restart=60, precision=fm.FMM_FP64)
    assert ok64 and rel(xm, x64) < 1e-6
    plan.close()


def test_high_frequency_plans_keep_plain_tables(fm):
    """The 20,480-triangle sphere at 8 kHz needs no scaling: its FP32 tables are the plain ones."""
    V, F = fm.icosphere(5, 0.3)
    k = 2 * np.pi * 8000 / 343.0
    plan = fm.Plan(V, F, k=k, depth=5, p_levels={2: 40, 3: 30, 4: 20, 5: 14}, rule=0, a=0.5, b=0.0, c=-1.0)
    assert plan.info.expansions_scaled == 0
    plan.close()


def test_orders_above_42_use_four_column_tiles(fm):
    """p = 50 at level 2 (ka = 14.7 on a 0.1 m sphere): two p^2 x 8 tiles would not fit in
    shared memory; 4-column tiles do (up to p = 60)."""
    V, F = fm.icosphere(3, 0.1)
    k = 2 * np.pi * 8000 / 343.0
    kw = dict(k=k, depth=3, p_levels={2: 50, 3: 36}, rule=1, a=0.5, b=0.0, c=-1.0, alpha=1j / k)
    plan = fm.Plan(V, F, **kw)
    info = plan.info
    assert info.m2l_columns[2] == 4
    rng = np.random.default_rng(12)
    x = rng.standard_normal(plan.nf) + 1j * rng.standard_normal(plan.nf)
    y64 = plan.matvec(x, fm.FMM_FP64)
    assert rel(plan.matvec(x, fm.FMM_MIXED), y64) < 1e-5
    X = np.stack([x, rng.standard_normal(plan.nf) + 0j])
    Y = plan.matvec(X.reshape(-1), fm.FMM_MIXED).reshape(2, -1)
    assert rel(Y[1], plan.matvec(X[1], fm.FMM_FP64)) < 1e-5
    plan.close()
    # orders above 60 still build without the mixed tables, and a mixed call says why
    plan = fm.Plan(V, F, k=k, depth=3, p_levels={2: 61, 3: 36}, rule=1, a=0.5, b=0.0, c=-1.0)
    assert plan.info.m2l_columns[2] == 0
    with pytest.raises(fm.FmmError, match="orders <= 60"):
        plan.matvec(x, fm.FMM_MIXED)
    plan.close()
