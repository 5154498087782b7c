"""The three-stage tensor-core translation passes (tc_rcr3.cu: rotation, coaxial and rotation
GEMMs on tcgen05, split TF32) against the FP64 path, the oracle and the SIMT tiles: plans built
with FMMBEM_TC3=1 run every batched pass in that form."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def make_plan(fm, tc3, *args, **kw):
    old = os.environ.get("FMMBEM_TC3")
    os.environ["FMMBEM_TC3"] = "1" if tc3 else "0"
    try:
        return fm.Plan(*args, **kw)
    finally:
        if old is None:
            del os.environ["FMMBEM_TC3"]
        else:
            os.environ["FMMBEM_TC3"] = old


def x_of(n, seed=0):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


@pytest.mark.parametrize("p_levels", [{2: 8, 3: 8}, {2: 16, 3: 12}])
def test_tc3_matches_oracle_small_sphere(fm, oracle, p_levels):
    V, F = fm.icosphere(3, 0.1)
    k = 2 * np.pi * 1000 / 343.0
    plan = make_plan(fm, True, V, F, k=k, depth=3, p_levels=p_levels, rule=1, a=0.5, b=0.0, c=-1.0)
    info = plan.info
    assert info.pass_tc3[2] & 2 and info.pass_tc3[3] == 7  # every batched pass in the three-stage form
    x = x_of(len(F))
    T = oracle.tree_for_fmm(V, F, depth=3)
    yo = oracle.FMM(V, F, k, T, [p_levels[2], p_levels[3]], a=0.5, b=0.0, c=-1.0, rule=1).apply(x)
    y64 = plan.matvec(x, fm.FMM_FP64)
    ym = plan.matvec(x, fm.FMM_MIXED)
    assert rel(y64, yo) < 1e-10
    assert rel(ym, yo) < 2e-6
    # columns and the transposed operator through the same passes
    X = np.concatenate([x, x_of(len(F), 1), x_of(len(F), 2)])
    Ym = plan.matvec(X, fm.FMM_MIXED)
    for r in range(3):
        xr = X[r * len(F):(r + 1) * len(F)]
        assert rel(Ym[r * len(F):(r + 1) * len(F)], plan.matvec(xr, fm.FMM_FP64)) < 2e-6
    yt = plan.matvec_adjoint(x, fm.FMM_MIXED)
    assert rel(yt, plan.matvec_adjoint(x, fm.FMM_FP64)) < 2e-6
    plan.close()


def test_tc3_orders_differ_between_levels(fm):
    """M2M and L2L between levels of different order (source order below the RCR order, and
    destination order below it), depth 4."""
    V, F = fm.icosphere(4, 0.3)
    k = 2 * np.pi * 4000 / 343.0
    pl = {2: 20, 3: 14, 4: 9}
    plan = make_plan(fm, True, V, F, k=k, depth=4, p_levels=pl, rule=0, a=0.5, b=0.0, c=-1.0)
    assert all(plan.info.pass_tc3[l] == 7 for l in (3, 4))
    ref = make_plan(fm, False, V, F, k=k, depth=4, p_levels=pl, rule=0, a=0.5, b=0.0, c=-1.0)
    x = x_of(len(F), 4)
    y64 = plan.matvec(x, fm.FMM_FP64)
    ym = plan.matvec(x, fm.FMM_MIXED)
    ys = ref.matvec(x, fm.FMM_MIXED)
    assert rel(ym, y64) < 2e-6
    assert rel(ym, ys) < 2e-6
    plan.close()
    ref.close()


def test_tc3_scaled_expansions(fm):
    """Low frequency, high order: FP32 expansions kept scaled by degree (coaxial entries near
    1e40 unscaled); the three-stage passes read the same scaled tables as the SIMT tiles."""
    V, F = fm.icosphere(3, 0.1)
    k = 2 * np.pi * 1000 / 343.0
    plan = make_plan(fm, True, V, F, k=k, depth=3, p_levels={2: 16, 3: 16}, rule=1, a=0.5, b=0.0, c=-1.0)
    assert plan.info.expansions_scaled == 1
    x = x_of(len(F), 5)
    assert rel(plan.matvec(x, fm.FMM_MIXED), plan.matvec(x, fm.FMM_FP64)) < 1e-5
    plan.close()


def test_tc3_full_size_workload(fm):
    """The 81,920-triangle sphere at 8 kHz, p = 40/30/20/14/10: every pass three-stage, mixed
    against FP64 at the tolerance of the SIMT path, repeated calls (the second captures the
    CUDA graph) equal to FP32 rounding."""
    V, F = fm.icosphere(6, 0.3)
    k = 2 * np.pi * 8000 / 343.0
    P2 = {2: 40, 3: 30, 4: 20, 5: 14, 6: 10}
    plan = make_plan(fm, True, V, F, k=k, depth=6, p_levels=P2, rule=0, a=0.5, b=0.0, c=-1.0)
    x = x_of(len(F), 6)
    y64 = plan.matvec(x, fm.FMM_FP64)
    for _ in range(3):
        ym = plan.matvec(x, fm.FMM_MIXED)
        assert rel(ym, y64) < 1e-6
    plan.close()
