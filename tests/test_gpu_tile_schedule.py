"""The SIMT translation tiles of the mixed path with each unit schedule forced on every pass
(FMMBEM_TILE_BAL=0: the default round-robin schedule, 1: the balanced schedule with narrow column
groups, 2: the balanced schedule with the default groups; the tensor-core forms off), against
the FP64 matvec, against each other, for one and several right-hand sides and through a scene's
work-queue kernels.  The orders cover every tile width of the plan path: p = 48 (4 columns per
CTA), 30 (8), 20 (16), 14 (32) and 10 (64)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
K = 2 * np.pi * 8000 / 343.0


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def make_plan(fm, bal, *args, **kw):
    env = {"FMMBEM_TILE_BAL": bal, "FMMBEM_TENSOR_M2L": "0", "FMMBEM_TENSOR_M2M": "0", "FMMBEM_TC3": "0"}
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


def plans_for(fm, bal):
    V, F = fm.icosphere(5, 0.3)
    a = make_plan(fm, bal, V, F, k=K, depth=5, p_levels={2: 48, 3: 30, 4: 20, 5: 14}, rule=0, a=0.5, b=0.0, c=-1.0)
    V, F = fm.icosphere(4, 0.15)
    b = make_plan(fm, bal, V, F, k=K, depth=4, p_levels={2: 20, 3: 14, 4: 10}, rule=1, a=0.5, b=0.0, c=-1.0,
                  alpha=1j / K)
    return [a, b]


@pytest.fixture(scope="module")
def results(fm):
    out = {}
    for bal in ("0", "1", "2"):
        plans = plans_for(fm, bal)
        try:
            info = [p.info for p in plans]
            assert all(i.m2l_tensor[l] == 0 and i.pass_tc3[l] == 0 for i in info for l in range(2, 6))
            rng = np.random.default_rng(7)
            xs = [rng.standard_normal(p.nf) + 1j * rng.standard_normal(p.nf) for p in plans]
            Xs = [rng.standard_normal((3, p.nf)) + 1j * rng.standard_normal((3, p.nf)) for p in plans]
            r = {"bal": [[i.pass_balanced[l] for l in range(2, 6)] for i in info]}
            r["mixed"] = [p.matvec(x, fm.FMM_MIXED) for p, x in zip(plans, xs)]
            r["fp64"] = [p.matvec(x, fm.FMM_FP64) for p, x in zip(plans, xs)]
            r["batched"] = [p.matvec(X, fm.FMM_MIXED) for p, X in zip(plans, Xs)]
            r["batched64"] = [np.stack([p.matvec(X[j], fm.FMM_FP64) for j in range(3)]) for p, X in zip(plans, Xs)]
            sc = fm.Scene(plans)
            y = sc.split(sc.matvec(sc.join(xs), fm.FMM_MIXED))
            r["scene"] = y
            sc.close()
            out[bal] = r
        finally:
            for p in plans:
                p.close()
    return out


@pytest.mark.parametrize("bal", ["0", "1", "2"])
def test_each_schedule_matches_fp64(results, bal):
    r = results[bal]
    if bal != "0":
        # every SIMT pass of both plans runs the forced schedule where its tile has one
        assert any(any(b) for b in r["bal"])
    for ym, y64 in zip(r["mixed"], r["fp64"]):
        assert rel(ym, y64) < 1e-5
    for Ym, Y64 in zip(r["batched"], r["batched64"]):
        for j in range(3):
            assert rel(Ym[j], Y64[j]) < 1e-5
    for ys, y64 in zip(r["scene"], r["fp64"]):
        assert rel(ys, y64) < 1e-5


def test_schedules_agree(results):
    # the schedules sum every output in the same order; only the order of the FP32 atomic
    # additions into the destinations differs
    for bal in ("1", "2"):
        for a, b in zip(results[bal]["mixed"], results["0"]["mixed"]):
            assert rel(a, b) < 1e-6
        for a, b in zip(results[bal]["batched"], results["0"]["batched"]):
            assert rel(a, b) < 1e-6
